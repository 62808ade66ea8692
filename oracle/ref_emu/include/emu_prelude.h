/*
 * emu_prelude.h -- force-included before the reference's CUDA sources when they
 * are compiled for the CPU (TEST INFRASTRUCTURE, builds oracle/_ref only).
 *
 * It turns the CUDA C++ dialect used by the reference kernels into plain C++:
 * execution-space qualifiers vanish, built-in thread coordinates become
 * thread-local globals set by the launcher in harness.cpp, and the few device
 * intrinsics the kernels call are given their mathematical definitions
 * (correctly rounded add/sub, reciprocal square root from float64).
 */
#pragma once
#include <cmath>
#include <cstdint>
#include <cstring>
#include <cstdlib>
#include <algorithm>
#include <vector>
#include <string>
#include <iostream>

#define __host__
#define __device__
#define __global__
#define __constant__
#define __shared__
#define __forceinline__ inline
#define __align__(n)

typedef unsigned int uint;

#include "vector_types.h"

extern thread_local dim3 threadIdx;
extern thread_local dim3 blockIdx;
extern thread_local dim3 blockDim;
extern thread_local dim3 gridDim;

inline void __syncthreads() {}

/* round-to-nearest float32 add / subtract: what IEEE float32 + and - give */
inline float __fadd_rn(float a, float b) { volatile float r = a + b; return r; }
inline float __fsub_rn(float a, float b) { volatile float r = a - b; return r; }
inline float __fmul_rn(float a, float b) { volatile float r = a * b; return r; }
/* reciprocal square root from the float64 quotient 1/sqrt(x), rounded once to float32 */
inline float __frsqrt_rn(float x) { return (float)(1.0 / std::sqrt((double)x)); }
inline float rsqrtf(float x) { return 1.0f / std::sqrt(x); }

/* 1-D texture reference stand-in: tex1Dfetch reads the bound array */
enum cudaTextureReadMode { cudaReadModeElementType = 0 };
template <class T, int dim = 1, int mode = 0>
struct texture { const T* ptr = nullptr; };
template <class T, int dim, int mode>
inline T tex1Dfetch(const texture<T, dim, mode>& t, int i) { return t.ptr[i]; }

using std::min;
using std::max;
