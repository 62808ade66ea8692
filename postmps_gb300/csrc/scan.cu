// scan.cu -- device-wide exclusive prefix sums (replaces the reference's
// thrust::exclusive_scan wrapper, Thrust.cuh:17-38, which also copied the
// total back to the host; here the total stays on the device).
//
// Reduce-then-scan over a fixed number of blocks: each block owns one
// contiguous chunk, (1) reduces it, (2) one block scans the chunk sums,
// (3) each block rescans its chunk from its offset.  Tiles are staged through
// shared memory so that global loads and stores stay coalesced.
#include "pms_internal.h"
#include "k_common.cuh"

namespace pms {

static constexpr int kScanThreads = 256;
static constexpr int kScanItems = 8;
static constexpr int kScanTile = kScanThreads * kScanItems;   // 2048
static constexpr int kScanMaxBlocks = 1024;

template <class T>
__device__ __forceinline__ T warp_incl_scan(T v) {
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        T t = __shfl_up_sync(0xffffffffu, v, o);
        if ((threadIdx.x & 31) >= o) v += t;
    }
    return v;
}

// exclusive scan of one value per thread across the block; returns block total
template <class T>
__device__ __forceinline__ T block_excl_scan(T v, T* smem_warp, T& total) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    T inc = warp_incl_scan(v);
    if (lane == 31) smem_warp[wid] = inc;
    __syncthreads();
    if (wid == 0) {
        T s = (lane < kScanThreads / 32) ? smem_warp[lane] : T(0);
        s = warp_incl_scan(s);
        if (lane < kScanThreads / 32) smem_warp[lane] = s;
    }
    __syncthreads();
    T base = wid ? smem_warp[wid - 1] : T(0);
    total = smem_warp[kScanThreads / 32 - 1];
    __syncthreads();
    return base + inc - v;
}

template <class T>
__global__ void __launch_bounds__(kScanThreads) k_scan_reduce(const T* __restrict__ in, uint64_t n, uint64_t chunk,
                                                              T* __restrict__ partial, const uint32_t* __restrict__ n_dev) {
    __shared__ T warp_sums[kScanThreads / 32];
    uint64_t b0 = (uint64_t)blockIdx.x * chunk;
    uint64_t b1 = b0 + chunk < n ? b0 + chunk : n;
    const uint64_t nn = n_dev && (uint64_t)*n_dev < n ? (uint64_t)*n_dev : n;   // elements past nn count as 0
    T acc = 0;
    for (uint64_t i = b0 + threadIdx.x; i < b1; i += kScanThreads) acc += i < nn ? in[i] : T(0);
    T total;
    block_excl_scan<T>(acc, warp_sums, total);
    if (threadIdx.x == 0) partial[blockIdx.x] = total;
}

template <class T>
__global__ void __launch_bounds__(1024) k_scan_partials(T* __restrict__ partial, int nb, T* __restrict__ total_out) {
    __shared__ T warp_sums[32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    T v = threadIdx.x < nb ? partial[threadIdx.x] : T(0);
    T inc = warp_incl_scan(v);
    if (lane == 31) warp_sums[wid] = inc;
    __syncthreads();
    if (wid == 0) warp_sums[lane] = warp_incl_scan(warp_sums[lane]);
    __syncthreads();
    T base = wid ? warp_sums[wid - 1] : T(0);
    if (threadIdx.x < nb) partial[threadIdx.x] = base + inc - v;
    if (threadIdx.x == 1023 && total_out) *total_out = base + inc;
}

template <class T>
__global__ void __launch_bounds__(kScanThreads) k_scan_down(const T* __restrict__ in, T* __restrict__ out, uint64_t n,
                                                             uint64_t chunk, const T* __restrict__ partial,
                                                             const uint32_t* __restrict__ n_dev) {
    __shared__ T tile[kScanTile];
    __shared__ T warp_sums[kScanThreads / 32];
    uint64_t b0 = (uint64_t)blockIdx.x * chunk;
    uint64_t b1 = b0 + chunk < n ? b0 + chunk : n;
    const uint64_t nn = n_dev && (uint64_t)*n_dev < n ? (uint64_t)*n_dev : n;
    T carry = partial[blockIdx.x];
    for (uint64_t t0 = b0; t0 < b1; t0 += kScanTile) {
#pragma unroll
        for (int k = 0; k < kScanItems; ++k) {
            uint64_t i = t0 + k * kScanThreads + threadIdx.x;
            tile[k * kScanThreads + threadIdx.x] = i < nn && i < b1 ? in[i] : T(0);
        }
        __syncthreads();
        T loc[kScanItems];
        T sum = 0;
#pragma unroll
        for (int k = 0; k < kScanItems; ++k) { loc[k] = tile[threadIdx.x * kScanItems + k]; sum += loc[k]; }
        T total;
        T run = block_excl_scan<T>(sum, warp_sums, total) + carry;
#pragma unroll
        for (int k = 0; k < kScanItems; ++k) { T v = loc[k]; tile[threadIdx.x * kScanItems + k] = run; run += v; }
        __syncthreads();
#pragma unroll
        for (int k = 0; k < kScanItems; ++k) {
            uint64_t i = t0 + k * kScanThreads + threadIdx.x;
            if (i < b1) out[i] = tile[k * kScanThreads + threadIdx.x];
        }
        carry += total;
        __syncthreads();
    }
}

template <class T>
static pms_status scan_impl(pms_ctx* ctx, const T* in, T* out, uint64_t n, T* total_dev, const uint32_t* n_dev) {
    if (n == 0) {
        if (total_dev) PMS_CUDA(ctx, cudaMemsetAsync(total_dev, 0, sizeof(T), ctx->stream));
        return PMS_OK;
    }
    uint64_t tiles = (n + kScanTile - 1) / kScanTile;
    int nb = (int)(tiles < (uint64_t)kScanMaxBlocks ? tiles : (uint64_t)kScanMaxBlocks);
    uint64_t chunk = ((tiles + nb - 1) / nb) * kScanTile;
    nb = (int)((n + chunk - 1) / chunk);
    PMS_CUDA(ctx, ctx->scan.partial.ensure(sizeof(unsigned long long) * kScanMaxBlocks));
    T* partial = ctx->scan.partial.as<T>();
    k_scan_reduce<T><<<nb, kScanThreads, 0, ctx->stream>>>(in, n, chunk, partial, n_dev);
    PMS_LAUNCHED(ctx);
    k_scan_partials<T><<<1, 1024, 0, ctx->stream>>>(partial, nb, total_dev);
    PMS_LAUNCHED(ctx);
    k_scan_down<T><<<nb, kScanThreads, 0, ctx->stream>>>(in, out, n, chunk, partial, n_dev);
    PMS_LAUNCHED(ctx);
    return PMS_OK;
}

pms_status scan_u32(pms_ctx* ctx, const uint32_t* in, uint32_t* out, uint64_t n, uint32_t* total_dev,
                    const uint32_t* n_dev) {
    return scan_impl<uint32_t>(ctx, in, out, n, total_dev, n_dev);
}
pms_status scan_u64(pms_ctx* ctx, const unsigned long long* in, unsigned long long* out, uint64_t n,
                    unsigned long long* total_dev, const uint32_t* n_dev) {
    return scan_impl<unsigned long long>(ctx, in, out, n, total_dev, n_dev);
}

}  // namespace pms
