// scan_noalloc.cu -- an exclusive prefix sum that allocates nothing.
//
// Who needs it: host programs that embed this library but cannot let it call
// cudaMalloc -- a simulation or rendering host that owns all device memory
// through its own pool, or a frame loop that must not pay cudaMalloc's
// implicit device synchronisation in the middle of a frame.  They pass device
// input and output arrays; the only other memory used is the file-scope
// scratch array below, which every GPU that loads the library holds until the
// process exits.
//
// Limits and sharing: at most kNoAllocMaxElements (33,554,432) elements per
// call (4096 tiles of 8192; one partial sum per tile in the scratch array,
// 16 KiB).  Every call uses the same scratch array, which keeps the last
// call's partial sums; each call writes every partial it later reads, so
// nothing needs clearing.  Two calls that overlap on the GPU (different
// streams, or different host threads) race on the scratch array.
#include "pms_internal.h"

#include <mutex>

namespace pms {
namespace {

constexpr int kThreads = 256;
constexpr int kItems = 32;                          // per thread
constexpr uint64_t kTile = (uint64_t)kThreads * kItems;   // 8192 elements per block
constexpr int kMaxTiles = 4096;
constexpr uint64_t kNoAllocMaxElements = kTile * kMaxTiles;

// the only scratch: one partial sum per tile
static __device__ __align__(256) uint32_t g_noalloc_partials[kMaxTiles];

__device__ __forceinline__ uint32_t warp_incl(uint32_t v) {
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t t = __shfl_up_sync(0xffffffffu, v, o);
        if ((threadIdx.x & 31) >= o) v += t;
    }
    return v;
}

// block-wide exclusive scan of one value per thread; returns the block total in *total
__device__ __forceinline__ uint32_t block_excl(uint32_t v, uint32_t* warp_sums, uint32_t* total) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    uint32_t inc = warp_incl(v);
    if (lane == 31) warp_sums[wid] = inc;
    __syncthreads();
    if (wid == 0) {
        uint32_t s = lane < kThreads / 32 ? warp_sums[lane] : 0u;
        s = warp_incl(s);
        if (lane < kThreads / 32) warp_sums[lane] = s;
    }
    __syncthreads();
    uint32_t base = wid ? warp_sums[wid - 1] : 0u;
    *total = warp_sums[kThreads / 32 - 1];
    __syncthreads();
    return base + inc - v;
}

__global__ void __launch_bounds__(kThreads) k_tile_sums(const uint32_t* __restrict__ in, uint64_t n,
                                                        uint32_t* __restrict__ partials) {
    __shared__ uint32_t warp_sums[kThreads / 32];
    const uint64_t t0 = (uint64_t)blockIdx.x * kTile;
    uint32_t acc = 0;
    for (uint64_t i = t0 + threadIdx.x; i < t0 + kTile && i < n; i += kThreads) acc += in[i];
    uint32_t total;
    block_excl(acc, warp_sums, &total);
    if (threadIdx.x == 0) partials[blockIdx.x] = total;
}

// one block of 1024 threads scans up to 4096 partials (4 per thread)
__global__ void __launch_bounds__(1024) k_tile_offsets(uint32_t* __restrict__ partials, int ntiles,
                                                       uint32_t* __restrict__ total_out) {
    __shared__ uint32_t warp_sums[32];
    uint32_t v[4], s = 0;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        int i = threadIdx.x * 4 + k;
        v[k] = i < ntiles ? partials[i] : 0u;
        s += v[k];
    }
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    uint32_t inc = warp_incl(s);
    if (lane == 31) warp_sums[wid] = inc;
    __syncthreads();
    if (wid == 0) warp_sums[lane] = warp_incl(warp_sums[lane]);
    __syncthreads();
    uint32_t run = (wid ? warp_sums[wid - 1] : 0u) + inc - s;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        int i = threadIdx.x * 4 + k;
        if (i < ntiles) partials[i] = run;
        run += v[k];
    }
    if (threadIdx.x == 1023 && total_out) *total_out = run;
}

__global__ void __launch_bounds__(kThreads) k_tile_scan(const uint32_t* __restrict__ in, uint32_t* __restrict__ out,
                                                        uint64_t n, const uint32_t* __restrict__ partials) {
    __shared__ uint32_t tile[kThreads * 8];
    __shared__ uint32_t warp_sums[kThreads / 32];
    const uint64_t t0 = (uint64_t)blockIdx.x * kTile;
    uint32_t carry = partials[blockIdx.x];
    for (uint64_t s0 = t0; s0 < t0 + kTile && s0 < n; s0 += kThreads * 8) {
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            uint64_t i = s0 + k * kThreads + threadIdx.x;
            tile[k * kThreads + threadIdx.x] = i < n ? in[i] : 0u;
        }
        __syncthreads();
        uint32_t loc[8], sum = 0;
#pragma unroll
        for (int k = 0; k < 8; ++k) { loc[k] = tile[threadIdx.x * 8 + k]; sum += loc[k]; }
        uint32_t total;
        uint32_t run = block_excl(sum, warp_sums, &total) + carry;
#pragma unroll
        for (int k = 0; k < 8; ++k) { tile[threadIdx.x * 8 + k] = run; run += loc[k]; }
        __syncthreads();
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            uint64_t i = s0 + k * kThreads + threadIdx.x;
            if (i < n) out[i] = tile[k * kThreads + threadIdx.x];
        }
        carry += total;
        __syncthreads();
    }
}

// Device address of the scratch array, looked up once per device with that
// device current (host code cannot use the symbol itself as a device pointer).
std::mutex g_setup_mutex;
constexpr int kMaxDevices = 64;
uint32_t* g_partials_ptr[kMaxDevices] = {};

cudaError_t scratch_for_current_device(uint32_t** out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (!g_partials_ptr[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_partials);
        if (e != cudaSuccess) return e;
        g_partials_ptr[dev] = static_cast<uint32_t*>(p);
    }
    *out = g_partials_ptr[dev];
    return cudaSuccess;
}

}  // namespace
}  // namespace pms

extern "C" pms_status pms_exclusive_scan_u32_noalloc(const uint32_t* d_in, uint32_t* d_out, uint64_t n,
                                                     uint32_t* d_total, void* cuda_stream) {
    using namespace pms;
    if (n > kNoAllocMaxElements) return PMS_ERR_CAPACITY;
    if (n > 0 && (!d_in || !d_out)) return PMS_ERR_INVALID_ARGUMENT;
    cudaStream_t s = static_cast<cudaStream_t>(cuda_stream);
    uint32_t* partials = nullptr;
    if (scratch_for_current_device(&partials) != cudaSuccess) return PMS_ERR_CUDA;
    if (n == 0) {
        if (d_total && cudaMemsetAsync(d_total, 0, sizeof(uint32_t), s) != cudaSuccess) return PMS_ERR_CUDA;
        return PMS_OK;
    }
    const int ntiles = (int)((n + kTile - 1) / kTile);
    k_tile_sums<<<ntiles, kThreads, 0, s>>>(d_in, n, partials);
    if (cudaGetLastError() != cudaSuccess) return PMS_ERR_CUDA;
    k_tile_offsets<<<1, 1024, 0, s>>>(partials, ntiles, d_total);
    if (cudaGetLastError() != cudaSuccess) return PMS_ERR_CUDA;
    k_tile_scan<<<ntiles, kThreads, 0, s>>>(d_in, d_out, n, partials);
    if (cudaGetLastError() != cudaSuccess) return PMS_ERR_CUDA;
    return PMS_OK;
}
