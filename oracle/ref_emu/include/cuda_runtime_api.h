/* Host-memory stand-ins for the few CUDA runtime calls that the reference's
 * inline helpers mention (CPU emulation; test infrastructure). */
#pragma once
#include <cstdlib>
#include <cstring>
#include <cstddef>
typedef int cudaError_t;
enum { cudaSuccess = 0 };
enum cudaMemcpyKind { cudaMemcpyHostToHost = 0, cudaMemcpyHostToDevice = 1, cudaMemcpyDeviceToHost = 2, cudaMemcpyDeviceToDevice = 3 };
typedef void* cudaStream_t;
inline cudaError_t cudaMalloc(void** p, size_t n) { *p = std::calloc(n ? n : 1, 1); return *p ? 0 : 2; }
inline cudaError_t cudaFree(void* p) { std::free(p); return 0; }
inline cudaError_t cudaMemset(void* p, int v, size_t n) { std::memset(p, v, n); return 0; }
inline cudaError_t cudaMemcpy(void* d, const void* s, size_t n, cudaMemcpyKind) { std::memmove(d, s, n); return 0; }
inline cudaError_t cudaGetLastError() { return 0; }
inline const char* cudaGetErrorString(cudaError_t) { return "emulated"; }
inline cudaError_t cudaMemGetInfo(size_t* a, size_t* t) { *a = 0; *t = 0; return 0; }
inline cudaError_t cudaDeviceSynchronize() { return 0; }
inline cudaError_t cudaSetDevice(int) { return 0; }
inline cudaError_t cudaGetDevice(int* d) { *d = 0; return 0; }
struct cudaDeviceProp { char name[256]; size_t totalGlobalMem; };
inline cudaError_t cudaGetDeviceProperties(cudaDeviceProp* p, int) { std::strcpy(p->name, "cpu-emulation"); p->totalGlobalMem = 0; return 0; }
