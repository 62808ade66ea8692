// k_band.cu -- outer narrow band of scalar-grid vertices.
//
// Reference: Anisotropic_kernel.cuh:522-636 (estimationOfSurfaceVertices with
// LOWRES on, USING_GRID off) marks, for every surface particle, each scalar
// vertex v of the box idx +- ceil(h / cell) that lies inside the AABB p +- h
// and satisfies (flag || n . (v - p) > 0), plus the vertices one step along
// +x, +y and +z of it (the LOWRES dilation).  Marks go into a dense uint per
// vertex; thrust then scans all S_sc flags and compactationOfSurfaceVertices
// (Anisotropic_kernel.cuh:639-653) gathers the ascending vertex list.
//
// GB300 design: marks are bits, made tile by tile.  Neighbouring surface
// particles' boxes overlap heavily (each band vertex is marked by ~90 of them
// on a 2M-particle crown), so marking straight into the global bitmap costs a
// global atomic per particle and box row.  Instead the scalar grid is cut into
// tiles of 32 x 8 x 8 vertices (one 32-bit shared word per tile row); the
// tiles some surface particle's box reaches are listed first, then one block
// per tile stages the surface particles of the rows of spatial cells around it
// (contiguous stretches of the surface list) in shared memory, and each thread
// collects one tile row's marks from its share of them in a register, with the
// reference's own tests and roundings; each tile row then lands in the global
// bitmap with at most two atomics.  The dilation is a pass over the bitmap:
// B = B0 | B0<<1 | B0<<rx | B0<<(rx*ry) in linear bit order (the reference's
// index arithmetic, including its row wrap).  The compaction is a popcount per
// 32-bit word, one scan over words and a per-word bit extraction.  The bitmap
// (S_sc / 8 bytes) replaces three dense S_sc-sized uint arrays.
#include "pms_internal.h"
#include "k_common.cuh"

namespace pms {

// Tiles of the scalar grid: 32 vertices along x (one shared word per tile row) by 8 by 8.
static constexpr int kTileX = 32, kTileY = 8, kTileZ = 8;
static constexpr int kTileThreads = 256;

struct TileDims {
    uint32_t n[3];            // tiles per axis
};

// The clamped box [lo, hi] of scalar vertices a surface particle tests
// (estimationOfSurfaceVertices: idx +- ceil(h / cell), clamped to the grid).
__device__ __forceinline__ void particle_box(const KGrid& g, int ext, const float p[3], int lo[3], int hi[3]) {
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const int res = (int)g.scres[k];
        const int c = __float2int_rz(__fdiv_rn(__fsub_rn(p[k], g.scmin_pos[k]), g.sc_cs));
        lo[k] = min(max(c - ext, 0), res - 1);
        hi[k] = min(max(c + ext, 0), res - 1);
    }
}

// the tiles each surface particle's box reaches (read before the atomic: most are set already)
__global__ void __launch_bounds__(256) k_band_tile_mark(KGrid g, int ext, TileDims td, const uint32_t* __restrict__ slist,
                                                        const Counters* __restrict__ cnt, const float4* __restrict__ spos,
                                                        uint32_t* __restrict__ tbits) {
    const uint32_t ns = cnt->ns;
    for (uint32_t s = blockIdx.x * blockDim.x + threadIdx.x; s < ns; s += gridDim.x * blockDim.x) {
        const float4 p4 = __ldg(&spos[__ldg(&slist[s])]);
        const float p[3] = {p4.x, p4.y, p4.z};
        int lo[3], hi[3];
        particle_box(g, ext, p, lo, hi);
        for (int tz = lo[2] / kTileZ; tz <= hi[2] / kTileZ; ++tz)
            for (int ty = lo[1] / kTileY; ty <= hi[1] / kTileY; ++ty)
                for (int tx = lo[0] / kTileX; tx <= hi[0] / kTileX; ++tx) {
                    const uint32_t t = ((uint32_t)tz * td.n[1] + (uint32_t)ty) * td.n[0] + (uint32_t)tx;
                    const uint32_t bit = 1u << (t & 31u);
                    if (!(tbits[t >> 5] & bit)) atomicOr(&tbits[t >> 5], bit);
                }
    }
}

// Rows of spatial cells a tile block handles at once (their surface particles are
// spread over the block's threads), and surface particles staged in shared memory
// at once.
static constexpr int kTileRows = 256;
static constexpr int kTileChunk = 256;
static constexpr int kTileGroups = kTileThreads / (kTileZ * kTileY);   // threads per tile row

// One block per listed tile.  The rows of spatial cells whose particles can have a
// box reaching the tile (a cell of margin on each side covers the rounding of
// positions, keys and vertex coordinates) hold their surface particles as
// contiguous stretches of the surface list (it is in cell order: surf_start is
// the exclusive scan of the per-cell surface counts).  Those particles are staged
// in shared memory a chunk at a time with what a tile row needs of them (the
// part of their box inside the tile, their AABB p +- h, the x positions of the
// tile inside it); then every thread owns one tile row and a quarter of the
// chunk's particles and ORs into a register the vertices of its row that each of
// them marks: inside the AABB and (flag || n . (v - p) > 0), evaluated as
// estimationOfSurfaceVertices does (Anisotropic_kernel.cuh:551-606): vertex
// coordinates i * cell + min, each difference, product and sum rounded on its own.
__global__ void __launch_bounds__(kTileThreads) k_band_tiles(KGrid g, float h, int ext, TileDims td,
                                                              const uint32_t* __restrict__ n_tiles_dev,
                                                              const uint32_t* __restrict__ tiles,
                                                              const uint32_t* __restrict__ surf_start,
                                                              const uint32_t* __restrict__ surf_count,
                                                              const uint32_t* __restrict__ slist,
                                                              const float4* __restrict__ spos, const float4* __restrict__ nrm4,
                                                              uint32_t* __restrict__ bm0) {
    __shared__ uint32_t pre[kTileRows + 1];      // exclusive prefix of the rows' surface-particle counts
    __shared__ uint32_t first[kTileRows];        // each row's first surface-list entry
    __shared__ uint32_t wsum[kTileThreads / 32];
    __shared__ float vxs[kTileX];                // the tile's vertex x coordinates
    __shared__ float4 sp[kTileChunk];            // staged particle: p, and h (flag: n.w)
    __shared__ float4 sn[kTileChunk];            // its normal, w: flag
    __shared__ uint32_t sxin[kTileChunk];        // tile x positions inside its box and AABB (0: nothing to mark)
    __shared__ uint32_t syz[kTileChunk];         // its box inside the tile: y0 | y1 << 8 | z0 << 16 | z1 << 24
    __shared__ uint32_t red[kTileGroups][kTileZ * kTileY];
    __shared__ uint32_t s_nrel;                  // staged particles of the chunk whose box reaches the tile
    const uint32_t n_tiles = *n_tiles_dev;
    const uint32_t tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5;
    const uint32_t srx = g.spres[0], sry = g.spres[1];
    const uint64_t rxy = (uint64_t)g.scres[0] * g.scres[1];
    const int my_row = (int)(tid % (kTileZ * kTileY)), my_group = (int)(tid / (kTileZ * kTileY));
    const int my_y = my_row % kTileY, my_z = my_row / kTileY;
    for (uint32_t ti = blockIdx.x; ti < n_tiles; ti += gridDim.x) {
        const uint32_t t = __ldg(&tiles[ti]);
        const uint32_t tx = t % td.n[0], tyz = t / td.n[0], ty = tyz % td.n[1], tz = tyz / td.n[1];
        const int t0[3] = {(int)tx * kTileX, (int)ty * kTileY, (int)tz * kTileZ};
        const int t1[3] = {min(t0[0] + kTileX, (int)g.scres[0]) - 1, min(t0[1] + kTileY, (int)g.scres[1]) - 1,
                           min(t0[2] + kTileZ, (int)g.scres[2]) - 1};
        if (tid < kTileX) vxs[tid] = sc_coord_i(g, t0[0] + (int)tid, 0);
        // this thread's tile row
        const float vy = sc_coord_i(g, t0[1] + my_y, 1), vz = sc_coord_i(g, t0[2] + my_z, 2);
        const bool row_in = t0[1] + my_y <= t1[1] && t0[2] + my_z <= t1[2];
        uint32_t acc = 0u;
        // spatial cells of the particles whose box can reach the tile
        int slo[3], shi[3];
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            const float a = g.scmin_pos[k] + (float)(t0[k] - ext - 1) * g.sc_cs - g.min_pos[k];
            const float b = g.scmin_pos[k] + (float)(t1[k] + ext + 2) * g.sc_cs - g.min_pos[k];
            slo[k] = max((int)floorf(a / g.sp_cs) - 1, 0);
            shi[k] = min((int)floorf(b / g.sp_cs) + 1, (int)g.spres[k] - 1);
        }
        const int ny = shi[1] - slo[1] + 1, nz = shi[2] - slo[2] + 1;
        const int nrow = (ny > 0 && nz > 0 && shi[0] >= slo[0]) ? ny * nz : 0;
        for (int r0 = 0; r0 < nrow; r0 += kTileRows) {
            const int nr = min(kTileRows, nrow - r0);
            // each row's stretch of the surface list, and a block-wide exclusive scan of the lengths
            uint32_t len = 0u;
            if ((int)tid < nr) {
                const int r = r0 + (int)tid;
                const uint32_t row = ((uint32_t)(slo[2] + r / ny) * sry + (uint32_t)(slo[1] + r % ny)) * srx;
                const uint32_t c0 = row + (uint32_t)slo[0], c1 = row + (uint32_t)shi[0];
                const uint32_t a = __ldg(&surf_start[c0]);
                len = __ldg(&surf_start[c1]) + __ldg(&surf_count[c1]) - a;
                first[tid] = a;
            }
            uint32_t incl = len;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
                if (lane >= (uint32_t)o) incl += y;
            }
            if (lane == 31u) wsum[warp] = incl;
            __syncthreads();
            uint32_t wofs = 0u;
            for (uint32_t w = 0; w < warp; ++w) wofs += wsum[w];
            if ((int)tid < nr) pre[tid] = wofs + incl - len;
            if (tid == kTileThreads - 1) {
                uint32_t tot = 0u;
                for (uint32_t w = 0; w < kTileThreads / 32; ++w) tot += wsum[w];
                pre[nr] = tot;
            }
            __syncthreads();
            const uint32_t total = pre[nr];
            for (uint32_t c0 = 0; c0 < total; c0 += kTileChunk) {
                const uint32_t nc = min((uint32_t)kTileChunk, total - c0);
                if (tid == 0) s_nrel = 0u;
                __syncthreads();
                // stage the chunk: only particles whose box reaches the tile take a slot (the
                // cell rows around the tile hold about twice as many), so the rows' loops below
                // see no particle that marks nothing; marks are an OR, the slot order is free
                if (tid < nc) {
                    const uint32_t k = c0 + tid;
                    int lo = 0, hi = nr - 1;     // the row holding entry k: the last row whose prefix is <= k
                    while (lo < hi) {
                        const int mid = (lo + hi + 1) >> 1;
                        if (pre[mid] <= k) lo = mid; else hi = mid - 1;
                    }
                    const uint32_t j = __ldg(&slist[first[lo] + (k - pre[lo])]);
                    const float4 p4 = __ldg(&spos[j]);
                    const float4 n4 = __ldg(&nrm4[j]);
                    const float p[3] = {p4.x, p4.y, p4.z};
                    int blo[3], bhi[3];
                    particle_box(g, ext, p, blo, bhi);
                    const int x0 = max(blo[0], t0[0]), x1 = min(bhi[0], t1[0]);
                    const int y0 = max(blo[1], t0[1]), y1 = min(bhi[1], t1[1]);
                    const int z0 = max(blo[2], t0[2]), z1 = min(bhi[2], t1[2]);
                    uint32_t xin = 0u;
                    if (x0 <= x1 && y0 <= y1 && z0 <= z1) {
                        const float ax = __fsub_rn(p[0], h), bx = __fadd_rn(p[0], h);
                        for (int x = x0; x <= x1; ++x) {
                            const float vx = vxs[x - t0[0]];
                            if (!(vx < ax || vx > bx)) xin |= 1u << (x - t0[0]);
                        }
                    }
                    // the warp's lanes staging this chunk (tid < nc), named for the ballot
                    const uint32_t nin = min(32u, nc - (tid & ~31u));
                    const unsigned act = nin == 32u ? 0xffffffffu : ((1u << nin) - 1u);
                    const unsigned want = __ballot_sync(act, xin != 0u);
                    uint32_t slot0 = 0u;
                    const int leader = __ffs(act) - 1;
                    if ((int)lane == leader && want) slot0 = atomicAdd(&s_nrel, (uint32_t)__popc(want));
                    slot0 = __shfl_sync(act, slot0, leader);
                    if (xin) {
                        const uint32_t slot = slot0 + (uint32_t)__popc(want & ((1u << lane) - 1u));
                        sp[slot] = p4;
                        sn[slot] = n4;
                        sxin[slot] = xin;
                        syz[slot] = (uint32_t)(y0 - t0[1]) | (uint32_t)(y1 - t0[1]) << 8 | (uint32_t)(z0 - t0[2]) << 16 |
                                    (uint32_t)(z1 - t0[2]) << 24;
                    }
                }
                __syncthreads();
                const uint32_t nrel = s_nrel;
                // this thread's row against its share of the chunk
                if (row_in) {
                    for (uint32_t k = (uint32_t)my_group; k < nrel; k += kTileGroups) {
                        const uint32_t xin = sxin[k];
                        const uint32_t yz = syz[k];
                        if (!xin || my_y < (int)(yz & 0xffu) || my_y > (int)((yz >> 8) & 0xffu) ||
                            my_z < (int)((yz >> 16) & 0xffu) || my_z > (int)(yz >> 24))
                            continue;
                        // marks are an OR: a particle whose x positions in this row are all
                        // marked already (each band vertex is marked by dozens) adds nothing
                        if (!(xin & ~acc)) continue;
                        const float4 p4 = sp[k];
                        const float4 n4 = sn[k];
                        if (vy < __fsub_rn(p4.y, h) || vy > __fadd_rn(p4.y, h) || vz < __fsub_rn(p4.z, h) ||
                            vz > __fadd_rn(p4.z, h))
                            continue;
                        if (n4.w != 0.f) { acc |= xin; continue; }     // flag: the whole AABB part
                        const float by = __fmul_rn(n4.y, __fsub_rn(vy, p4.y));
                        const float cz = __fmul_rn(n4.z, __fsub_rn(vz, p4.z));
                        for (uint32_t m = xin & ~acc; m; m &= m - 1u) {
                            const int i = __ffs(m) - 1;
                            const float dot = __fadd_rn(__fadd_rn(__fmul_rn(n4.x, __fsub_rn(vxs[i], p4.x)), by), cz);
                            if (dot > 0.f) acc |= 1u << i;
                        }
                    }
                }
                __syncthreads();
            }
        }
        red[my_group][my_row] = acc;
        __syncthreads();
        if (tid < kTileZ * kTileY) {
            uint32_t m = 0u;
#pragma unroll
            for (int q = 0; q < kTileGroups; ++q) m |= red[q][tid];
            if (m) {
                const uint64_t bit = (uint64_t)(t0[2] + (int)tid / kTileY) * rxy +
                                     (uint64_t)(t0[1] + (int)tid % kTileY) * g.scres[0] + (uint64_t)t0[0];
                const uint64_t w = bit >> 5;
                const uint32_t sh = (uint32_t)(bit & 31u);
                atomicOr(&bm0[w], m << sh);
                if (sh && (m >> (32u - sh))) atomicOr(&bm0[w + 1], m >> (32u - sh));
            }
        }
        __syncthreads();
    }
}

// bits of `b` shifted up by s positions, as seen by word w
__device__ __forceinline__ uint32_t shifted_word(const uint32_t* __restrict__ b, uint64_t w, uint64_t s) {
    const uint64_t q = s >> 5;
    const uint32_t r = (uint32_t)(s & 31u);
    if (w < q) return 0u;
    uint32_t hi = b[w - q];
    if (r == 0) return hi;
    uint32_t lo = (w >= q + 1) ? b[w - q - 1] : 0u;
    return (hi << r) | (lo >> (32u - r));
}

// LOWRES dilation (Anisotropic_kernel.cuh:610-629) and popcount per word
__global__ void __launch_bounds__(256) k_band_dilate(const uint32_t* __restrict__ bm0, uint32_t* __restrict__ bm,
                                                     uint32_t* __restrict__ wcount, uint64_t nwords, uint64_t nbits,
                                                     uint64_t sy, uint64_t sz) {
    for (uint64_t w = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; w < nwords; w += (uint64_t)gridDim.x * blockDim.x) {
        uint32_t v = bm0[w] | shifted_word(bm0, w, 1) | shifted_word(bm0, w, sy) | shifted_word(bm0, w, sz);
        if (w == nwords - 1 && (nbits & 31u)) v &= (1u << (nbits & 31u)) - 1u;
        bm[w] = v;
        wcount[w] = __popc(v);
    }
}

// popcount per word
__global__ void __launch_bounds__(256) k_word_popc(const uint32_t* __restrict__ b, uint32_t* __restrict__ wcount,
                                                   uint64_t nwords) {
    for (uint64_t w = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; w < nwords; w += (uint64_t)gridDim.x * blockDim.x)
        wcount[w] = __popc(b[w]);
}

// ascending vertex list from the bitmap
__global__ void __launch_bounds__(256) k_band_list(const uint32_t* __restrict__ bm, const uint32_t* __restrict__ wprefix,
                                                   uint64_t nwords, uint32_t* __restrict__ vlist) {
    for (uint64_t w = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; w < nwords; w += (uint64_t)gridDim.x * blockDim.x) {
        uint32_t b = bm[w];
        uint32_t o = wprefix[w];
        while (b) {
            uint32_t bit = __ffs(b) - 1;
            vlist[o++] = (uint32_t)(w * 32u + bit);
            b &= b - 1u;
        }
    }
}

static TileDims tile_dims(const KGrid& g) {
    TileDims td;
    td.n[0] = (g.scres[0] + kTileX - 1) / kTileX;
    td.n[1] = (g.scres[1] + kTileY - 1) / kTileY;
    td.n[2] = (g.scres[2] + kTileZ - 1) / kTileZ;
    return td;
}

pms_status launch_band(pms_ctx* ctx) {
    const KGrid g = kgrid_of(ctx->grid);
    Counters* cnt = ctx->counters.as<Counters>();
    const uint64_t nbits = g.sc_size, nwords = (nbits + 31) / 32;
    const TileDims td = tile_dims(g);
    const uint64_t ntiles = (uint64_t)td.n[0] * td.n[1] * td.n[2];
    const uint64_t tw = (ntiles + 31) / 32;
    // sized with the grid (ensure_grid_buffers: a tile holds at least one vertex)
    if (ctx->tile_list.cap < 4 * ntiles || ctx->tile_bits.cap < 4 * tw)
        return pms_fail(ctx, PMS_ERR_STATE, "internal: band tile buffers not sized for the grid");
    PMS_CUDA(ctx, cudaMemsetAsync(ctx->tile_bits.p, 0, 4 * tw, ctx->stream));
    PMS_CUDA(ctx, cudaMemsetAsync(ctx->bm0.p, 0, sizeof(uint32_t) * nwords, ctx->stream));
    // extent = ceil(maxdistance / scGridSize) (Anisotropic_kernel.cuh:551), a correctly rounded float quotient
    const int ext_dev = (int)(uint32_t)ceilf(ctx->prm.h / g.sc_cs);
    k_band_tile_mark<<<grid_for(ctx->n, 256), 256, 0, ctx->stream>>>(g, ext_dev, td, ctx->slist.as<uint32_t>(), cnt,
                                                                     ctx->spos.as<float4>(), ctx->tile_bits.as<uint32_t>());
    PMS_LAUNCHED(ctx);
    k_word_popc<<<grid_for(tw, 256), 256, 0, ctx->stream>>>(ctx->tile_bits.as<uint32_t>(), ctx->tile_wc.as<uint32_t>(), tw);
    PMS_LAUNCHED(ctx);
    pms_status st = scan_u32(ctx, ctx->tile_wc.as<uint32_t>(), ctx->tile_wp.as<uint32_t>(), tw, &cnt->n_tiles);
    if (st != PMS_OK) return st;
    k_band_list<<<grid_for(tw, 256), 256, 0, ctx->stream>>>(ctx->tile_bits.as<uint32_t>(), ctx->tile_wp.as<uint32_t>(), tw,
                                                            ctx->tile_list.as<uint32_t>());
    PMS_LAUNCHED(ctx);
    k_band_tiles<<<grid_for(ntiles, 1, 152u * 8u), kTileThreads, 0, ctx->stream>>>(
        g, ctx->prm.h, ext_dev, td, &cnt->n_tiles, ctx->tile_list.as<uint32_t>(), ctx->surf_start.as<uint32_t>(),
        ctx->surf_count.as<uint32_t>(), ctx->slist.as<uint32_t>(), ctx->spos.as<float4>(), ctx->nrm4.as<float4>(),
        ctx->bm0.as<uint32_t>());
    PMS_LAUNCHED(ctx);
    const uint64_t sy = g.scres[0], sz = (uint64_t)g.scres[0] * g.scres[1];
    k_band_dilate<<<grid_for(nwords, 256), 256, 0, ctx->stream>>>(ctx->bm0.as<uint32_t>(), ctx->bm.as<uint32_t>(),
                                                                  ctx->wcount.as<uint32_t>(), nwords, nbits, sy, sz);
    PMS_LAUNCHED(ctx);
    return scan_u32(ctx, ctx->wcount.as<uint32_t>(), ctx->wprefix.as<uint32_t>(), nwords, &cnt->nv);
}

pms_status launch_bits_list(pms_ctx* ctx, const uint32_t* bm, const uint32_t* wprefix, uint32_t* vlist) {
    const uint64_t nwords = ((uint64_t)ctx->grid.sc_size + 31) / 32;
    k_band_list<<<grid_for(nwords, 256), 256, 0, ctx->stream>>>(bm, wprefix, nwords, vlist);
    PMS_LAUNCHED(ctx);
    return PMS_OK;
}

pms_status launch_band_list(pms_ctx* ctx) {
    const uint64_t nwords = ((uint64_t)ctx->grid.sc_size + 31) / 32;
    k_band_list<<<grid_for(nwords, 256), 256, 0, ctx->stream>>>(ctx->bm.as<uint32_t>(), ctx->wprefix.as<uint32_t>(),
                                                                nwords, ctx->vlist.as<uint32_t>());
    PMS_LAUNCHED(ctx);
    return PMS_OK;
}

}  // namespace pms
