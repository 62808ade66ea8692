/*
 * ref_cuda_prelude.h -- force-included when the reference's own CUDA sources are
 * compiled for sm_103a (BASELINE TIMING ONLY: builds baseline/_ref/libref_cuda.so,
 * never part of libpms).
 *
 * CUDA 12 removed texture references.  The reference reads its four
 * marching-cubes tables through them (MarchingCube_kernel.cuh:14-17, bound in
 * MarchingCube.cu:199-210).  Here a texture reference becomes a device-global
 * pointer: "texture<T, 1, mode> name;" declares that pointer, cudaBindTexture
 * copies the device address into it, and tex1Dfetch reads through it.
 */
#pragma once
#include <cuda_runtime.h>
#include <cstddef>
// standard headers the reference's sources reach only through includes that
// older toolchains made
#include <algorithm>
#include <fstream>
#include <iomanip>
#include <iostream>
#include <string>
#include <vector>
// thrust (Thrust.cuh) and what it pulls in, before the reference defines its
// "numThreads" macro (CudaUtils.h), a name these headers now use themselves
#include <cooperative_groups.h>
#include <thrust/count.h>
#include <thrust/device_ptr.h>
#include <thrust/device_vector.h>
#include <thrust/execution_policy.h>
#include <thrust/for_each.h>
#include <thrust/iterator/zip_iterator.h>
#include <thrust/scan.h>
#include <thrust/sort.h>
#include <thrust/tuple.h>
// the reference writes these unqualified
using std::ios;
using std::setiosflags;
using std::setprecision;
using std::setw;

template <class T, int Dim = 1, int Mode = 0>
struct RefTexture {
    const T* ptr;
};

#define texture __device__ RefTexture

template <class T, int Dim, int Mode>
__device__ __forceinline__ T tex1Dfetch(const RefTexture<T, Dim, Mode>& t, int i) {
    return t.ptr[i];
}

template <class T, int Dim, int Mode>
inline cudaError_t cudaBindTexture(size_t* offset, const RefTexture<T, Dim, Mode>& tex, const void* dev,
                                   const cudaChannelFormatDesc&, size_t = 0) {
    if (offset) *offset = 0;
    return cudaMemcpyToSymbol(tex, &dev, sizeof(dev));
}
