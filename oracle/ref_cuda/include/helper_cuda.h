/* Error checks the reference's CUDA sources call (stand-in for the CUDA samples
 * header of that name; baseline timing build only): report and abort, as the
 * reference does on a failed call. */
#pragma once
#include <cstdio>
#include <cstdlib>
#include <cuda_runtime.h>

inline void ref_check_cuda(cudaError_t e, const char* what, const char* file, int line) {
    if (e != cudaSuccess) {
        std::fprintf(stderr, "reference CUDA build: %s failed at %s:%d: %s\n", what, file, line, cudaGetErrorString(e));
        std::exit(3);
    }
}
#define checkCudaErrors(val) ref_check_cuda((val), #val, __FILE__, __LINE__)
#define getLastCudaError(msg) ref_check_cuda(cudaGetLastError(), (msg), __FILE__, __LINE__)
