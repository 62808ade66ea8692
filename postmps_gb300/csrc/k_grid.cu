// k_grid.cu -- spatial hashing: bounding box, cell keys, stable counting sort
// of the particles by key, cell ranges, surface cells and the surface list.
//
// Reference: NeighborSearch_kernel.cuh:129-186 (calculateHash, calCellRange),
// Thrust.cuh:40-50 (thrust::sort_by_key, a stable radix sort of the 44-byte
// particle AoS), Anisotropic_kernel.cuh:15-155 (estimationOfSurfaceParticles,
// compactationOfParticles), FileData.cpp:240-257 (bounding box on the host).
//
// GB300 design: keys are cell indices < sp_size, so the stable sort is a
// counting sort -- one atomic histogram (which doubles as the cell-count
// array), one scan (which doubles as the cell-start array), one scatter, and a
// per-cell ordering fix that restores the input order inside each cell (the
// order a stable sort produces).  Only a uint32 permutation moves; the
// payload is gathered once into SoA float4 arrays (x, y, z, m/rho) that the
// neighbour loops read with one 16-byte load per particle.
#include "pms_internal.h"
#include "k_common.cuh"

namespace pms {

static constexpr int kThreads = 256;
static constexpr uint32_t kSmallCell = 64;     // per-thread insertion sort limit
static constexpr uint32_t kBigCell = 4096;     // per-block bitonic sort limit

// ---------------------------------------------------------------------------
// bounding box (FileData.cpp:240-257); non-finite positions are flagged
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kThreads) k_bbox(const float* __restrict__ pos, uint32_t n, Counters* __restrict__ cnt) {
    uint32_t mn[3] = {0xffffffffu, 0xffffffffu, 0xffffffffu}, mx[3] = {0u, 0u, 0u};
    bool bad = false;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            float v = pos[3 * (size_t)i + k];
            bad |= !isfinite(v);
            uint32_t o = ordered_bits(v);
            mn[k] = min(mn[k], o);
            mx[k] = max(mx[k], o);
        }
    }
#pragma unroll
    for (int k = 0; k < 3; ++k) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            mn[k] = min(mn[k], __shfl_xor_sync(0xffffffffu, mn[k], o));
            mx[k] = max(mx[k], __shfl_xor_sync(0xffffffffu, mx[k], o));
        }
    }
    if ((threadIdx.x & 31) == 0) {
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            atomicMin(&cnt->bbox_min[k], mn[k]);
            atomicMax(&cnt->bbox_max[k], mx[k]);
        }
    }
    if (__any_sync(0xffffffffu, bad) && (threadIdx.x & 31) == 0) atomicOr(&cnt->err, kErrNonFinite);
}

__global__ void k_counters_init(Counters* cnt, uint32_t n) {
    Counters c;
    memset(&c, 0, sizeof(c));
    c.n = n;
    for (int k = 0; k < 3; ++k) { c.bbox_min[k] = 0xffffffffu; c.bbox_max[k] = 0u; }
    *cnt = c;
}

// The counters into the context's mapped pinned mirror, stored by a kernel: a
// copy-engine transfer would queue behind a streamed mesh or diffuse copy.
__global__ void k_publish_counters(const uint32_t* __restrict__ src, uint32_t* __restrict__ dst, uint32_t words) {
    for (uint32_t i = threadIdx.x; i < words; i += blockDim.x) dst[i] = src[i];
}

pms_status launch_publish_counters(pms_ctx* ctx) {
    static_assert(sizeof(Counters) % 4 == 0, "counters are copied in 32-bit words");
    k_publish_counters<<<1, 128, 0, ctx->stream>>>(ctx->counters.as<uint32_t>(), ctx->h_counters_dev,
                                                   (uint32_t)(sizeof(Counters) / 4));
    PMS_LAUNCHED(ctx);
    return PMS_OK;
}

pms_status launch_bbox(pms_ctx* ctx) {
    Counters* cnt = ctx->counters.as<Counters>();
    k_counters_init<<<1, 1, 0, ctx->stream>>>(cnt, ctx->n);
    PMS_LAUNCHED(ctx);
    k_bbox<<<grid_for(ctx->n, kThreads, 152 * 8), kThreads, 0, ctx->stream>>>(ctx->in_pos.as<float>(), ctx->n, cnt);
    PMS_LAUNCHED(ctx);
    return PMS_OK;
}

// ---------------------------------------------------------------------------
// keys + histogram (calculateHash, NeighborSearch_kernel.cuh:129-152)
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kThreads) k_hash_count(KGrid g, const float* __restrict__ pos, uint32_t n,
                                                         uint32_t* __restrict__ keys, uint32_t* __restrict__ slot,
                                                         uint32_t* __restrict__ cell_count, Counters* __restrict__ cnt) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        uint3 c = sp_cell(g, pos[3 * (size_t)i], pos[3 * (size_t)i + 1], pos[3 * (size_t)i + 2]);
        uint32_t key = lin3(c.x, c.y, c.z, g.spres);
        if (key >= g.sp_size) { atomicOr(&cnt->err, kErrKeyRange); key = g.sp_size - 1; }
        keys[i] = key;
        slot[i] = atomicAdd(&cell_count[key], 1u);
    }
}

__global__ void __launch_bounds__(kThreads) k_scatter(const uint32_t* __restrict__ keys, const uint32_t* __restrict__ slot,
                                                      const uint32_t* __restrict__ cell_start, uint32_t n,
                                                      uint32_t* __restrict__ order) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        order[cell_start[keys[i]] + slot[i]] = i;
}

// Restores ascending input order inside every cell: what a stable sort by key
// yields.  Cells up to kSmallCell are sorted by one thread; larger ones are
// queued for k_cell_sort_big.
__global__ void __launch_bounds__(kThreads) k_cell_sort(const uint32_t* __restrict__ cell_count,
                                                        const uint32_t* __restrict__ cell_start, uint32_t ncells,
                                                        uint32_t* __restrict__ order, uint32_t* __restrict__ big,
                                                        Counters* __restrict__ cnt) {
    for (uint32_t c = blockIdx.x * blockDim.x + threadIdx.x; c < ncells; c += gridDim.x * blockDim.x) {
        uint32_t m = cell_count[c];
        if (m < 2) continue;
        if (m > kSmallCell) {
            uint32_t k = atomicAdd(&cnt->n_big_cells, 1u);
            big[k] = c;
            if (m > kBigCell) atomicOr(&cnt->err, kErrBigCell);
            continue;
        }
        uint32_t* a = order + cell_start[c];
        for (uint32_t i = 1; i < m; ++i) {
            uint32_t v = a[i];
            uint32_t j = i;
            while (j > 0 && a[j - 1] > v) { a[j] = a[j - 1]; --j; }
            a[j] = v;
        }
    }
}

// One block per queued cell: bitonic sort in shared memory (<= kBigCell entries).
__global__ void __launch_bounds__(1024) k_cell_sort_big(const uint32_t* __restrict__ cell_count,
                                                        const uint32_t* __restrict__ cell_start,
                                                        const uint32_t* __restrict__ big, const Counters* __restrict__ cnt,
                                                        uint32_t* __restrict__ order) {
    __shared__ uint32_t s[kBigCell];
    uint32_t nb = cnt->n_big_cells;
    for (uint32_t b = blockIdx.x; b < nb; b += gridDim.x) {
        uint32_t c = big[b];
        uint32_t m = cell_count[c];
        if (m > kBigCell) continue;
        uint32_t* a = order + cell_start[c];
        uint32_t p2 = 1;
        while (p2 < m) p2 <<= 1;
        for (uint32_t i = threadIdx.x; i < p2; i += blockDim.x) s[i] = i < m ? a[i] : 0xffffffffu;
        __syncthreads();
        for (uint32_t k = 2; k <= p2; k <<= 1) {
            for (uint32_t j = k >> 1; j > 0; j >>= 1) {
                for (uint32_t i = threadIdx.x; i < p2; i += blockDim.x) {
                    uint32_t l = i ^ j;
                    if (l > i) {
                        bool up = (i & k) == 0;
                        uint32_t x = s[i], y = s[l];
                        if ((x > y) == up) { s[i] = y; s[l] = x; }
                    }
                }
                __syncthreads();
            }
        }
        for (uint32_t i = threadIdx.x; i < m; i += blockDim.x) a[i] = s[i];
        __syncthreads();
    }
}

// Gathers the payload into sorted SoA arrays.
__global__ void __launch_bounds__(kThreads) k_gather(const uint32_t* __restrict__ order, const uint32_t* __restrict__ keys,
                                                     const float* __restrict__ pos, const float* __restrict__ vel,
                                                     uint32_t n, uint32_t* __restrict__ skeys, float4* __restrict__ spos,
                                                     float4* __restrict__ svel) {
    for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x) {
        uint32_t i = order[j];
        skeys[j] = keys[i];
        spos[j] = make_float4(pos[3 * (size_t)i], pos[3 * (size_t)i + 1], pos[3 * (size_t)i + 2], 0.f);
        svel[j] = make_float4(vel[3 * (size_t)i], vel[3 * (size_t)i + 1], vel[3 * (size_t)i + 2], 0.f);
    }
}

pms_status launch_hash_sort(pms_ctx* ctx) {
    const uint32_t n = ctx->n;
    const KGrid g = kgrid_of(ctx->grid);
    Counters* cnt = ctx->counters.as<Counters>();
    PMS_CUDA(ctx, cudaMemsetAsync(ctx->cell_count.p, 0, sizeof(uint32_t) * (size_t)g.sp_size, ctx->stream));
    const unsigned gb = grid_for(n, kThreads);
    k_hash_count<<<gb, kThreads, 0, ctx->stream>>>(g, ctx->in_pos.as<float>(), n, ctx->keys.as<uint32_t>(),
                                                   ctx->slot.as<uint32_t>(), ctx->cell_count.as<uint32_t>(), cnt);
    PMS_LAUNCHED(ctx);
    // cell_start[c + 1] - cell_start[c] is cell c's count for every c, and cell_start[sp_size] = n,
    // so the cells of a row segment form one contiguous particle range
    pms_status st = scan_u32(ctx, ctx->cell_count.as<uint32_t>(), ctx->cell_start.as<uint32_t>(), g.sp_size,
                             ctx->cell_start.as<uint32_t>() + g.sp_size);
    if (st != PMS_OK) return st;
    k_scatter<<<gb, kThreads, 0, ctx->stream>>>(ctx->keys.as<uint32_t>(), ctx->slot.as<uint32_t>(),
                                                ctx->cell_start.as<uint32_t>(), n, ctx->order.as<uint32_t>());
    PMS_LAUNCHED(ctx);
    k_cell_sort<<<grid_for(g.sp_size, kThreads), kThreads, 0, ctx->stream>>>(
        ctx->cell_count.as<uint32_t>(), ctx->cell_start.as<uint32_t>(), g.sp_size, ctx->order.as<uint32_t>(),
        ctx->big_cells.as<uint32_t>(), cnt);
    PMS_LAUNCHED(ctx);
    k_cell_sort_big<<<32, 1024, 0, ctx->stream>>>(ctx->cell_count.as<uint32_t>(), ctx->cell_start.as<uint32_t>(),
                                                   ctx->big_cells.as<uint32_t>(), cnt, ctx->order.as<uint32_t>());
    PMS_LAUNCHED(ctx);
    if (ctx->vel_pending) {
        PMS_CUDA(ctx, cudaStreamWaitEvent(ctx->stream, ctx->vel_ready, 0));   // the uploaded velocities
        ctx->vel_pending = false;
    }
    k_gather<<<gb, kThreads, 0, ctx->stream>>>(ctx->order.as<uint32_t>(), ctx->keys.as<uint32_t>(),
                                               ctx->in_pos.as<float>(), ctx->in_vel.as<float>(), n,
                                               ctx->skeys.as<uint32_t>(), ctx->spos.as<float4>(), ctx->svel.as<float4>());
    PMS_LAUNCHED(ctx);
    return PMS_OK;
}

// ---------------------------------------------------------------------------
// surface cells (estimationOfSurfaceParticles, Anisotropic_kernel.cuh:15-106):
// a non-empty cell with an empty cell in its clamped 3x3x3 neighbourhood.
// Writes numSurParticleGrid (surf_count) and the packed cell record
// cell_info = {start, count | surface << 31} read by the neighbour loops.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kThreads) k_surface_cells(KGrid g, const uint32_t* __restrict__ cell_count,
                                                            const uint32_t* __restrict__ cell_start,
                                                            uint32_t* __restrict__ surf_count, uint2* __restrict__ cell_info) {
    const uint32_t rx = g.spres[0], ry = g.spres[1], rz = g.spres[2], rxy = rx * ry;
    for (uint32_t c = blockIdx.x * blockDim.x + threadIdx.x; c < g.sp_size; c += gridDim.x * blockDim.x) {
        uint32_t m = cell_count[c];
        uint32_t s = cell_start[c];
        if (m == 0) { surf_count[c] = 0; cell_info[c] = make_uint2(s, 0u); continue; }
        uint32_t z = c / rxy, r = c - z * rxy, y = r / rx, x = r - y * rx;
        uint32_t lx = min(max(x - 1u, 0u), rx - 1u), hx = min(x + 1u, rx - 1u);
        uint32_t ly = min(max(y - 1u, 0u), ry - 1u), hy = min(y + 1u, ry - 1u);
        uint32_t lz = min(max(z - 1u, 0u), rz - 1u), hz = min(z + 1u, rz - 1u);
        bool surface = false;
        for (uint32_t cz = lz; cz <= hz && !surface; ++cz)
            for (uint32_t cy = ly; cy <= hy && !surface; ++cy)
                for (uint32_t cx = lx; cx <= hx; ++cx)
                    if (cell_count[cz * rxy + cy * rx + cx] == 0) { surface = true; break; }
        surf_count[c] = surface ? m : 0u;
        cell_info[c] = make_uint2(s, m | (surface ? 0x80000000u : 0u));
    }
}

// compactationOfParticles (Anisotropic_kernel.cuh:127-155), particle-parallel
__global__ void __launch_bounds__(kThreads) k_surface_list(const uint32_t* __restrict__ skeys, uint32_t n,
                                                           const uint2* __restrict__ cell_info,
                                                           const uint32_t* __restrict__ surf_start,
                                                           uint32_t* __restrict__ slist) {
    for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x) {
        uint32_t c = skeys[j];
        uint2 ci = cell_info[c];
        if (ci.y & 0x80000000u) slist[surf_start[c] + (j - ci.x)] = j;
    }
}

pms_status launch_surface_cells(pms_ctx* ctx) {
    const KGrid g = kgrid_of(ctx->grid);
    Counters* cnt = ctx->counters.as<Counters>();
    k_surface_cells<<<grid_for(g.sp_size, kThreads), kThreads, 0, ctx->stream>>>(
        g, ctx->cell_count.as<uint32_t>(), ctx->cell_start.as<uint32_t>(), ctx->surf_count.as<uint32_t>(),
        ctx->cell_info.as<uint2>());
    PMS_LAUNCHED(ctx);
    pms_status st = scan_u32(ctx, ctx->surf_count.as<uint32_t>(), ctx->surf_start.as<uint32_t>(), g.sp_size, &cnt->ns);
    if (st != PMS_OK) return st;
    k_surface_list<<<grid_for(ctx->n, kThreads), kThreads, 0, ctx->stream>>>(
        ctx->skeys.as<uint32_t>(), ctx->n, ctx->cell_info.as<uint2>(), ctx->surf_start.as<uint32_t>(),
        ctx->slist.as<uint32_t>());
    PMS_LAUNCHED(ctx);
    return PMS_OK;
}

}  // namespace pms
