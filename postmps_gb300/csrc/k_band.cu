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
// GB300 design: marks are bits.  One warp handles one surface particle and
// tests whole rows of its box at once; a ballot turns each row into a bit
// mask that lands with at most two atomicOr per row.  The dilation is then a
// pass over the bitmap: B = B0 | B0<<1 | B0<<rx | B0<<(rx*ry) in linear bit
// order (the reference's index arithmetic, including its row wrap).  The
// compaction is a popcount per 32-bit word, one scan over words and a
// per-word bit extraction.  The bitmap (S_sc / 8 bytes) replaces three dense
// S_sc-sized uint arrays.
#include "pms_internal.h"
#include "k_common.cuh"

namespace pms {

// one warp per surface particle; rows of the box packed into the 32 lanes
__global__ void __launch_bounds__(256) k_band_mark(KGrid g, float h, const uint32_t* __restrict__ slist,
                                                   const Counters* __restrict__ cnt, const float4* __restrict__ spos,
                                                   const float4* __restrict__ nrm4, uint32_t* __restrict__ bm0) {
    const uint32_t ns = cnt->ns;
    const int lane = threadIdx.x & 31;
    const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint32_t nwarps = (gridDim.x * blockDim.x) >> 5;
    const int rx = (int)g.scres[0], ry = (int)g.scres[1], rz = (int)g.scres[2];
    const uint64_t rxy = (uint64_t)g.scres[0] * g.scres[1];
    const uint64_t nbits = g.sc_size;
    // extent = ceil(maxdistance / scGridSize) (Anisotropic_kernel.cuh:551)
    const int ext = (int)(uint32_t)ceilf(__fdiv_rn(h, g.sc_cs));
    for (uint32_t s = warp; s < ns; s += nwarps) {
        const uint32_t i = slist[s];
        const float4 p4 = spos[i];
        const float4 n4 = nrm4[i];
        const bool flag = n4.w != 0.f;
        const float p[3] = {p4.x, p4.y, p4.z};
        int c[3], lo[3], hi[3];
        float aa[3], bb[3];
        const int res[3] = {rx, ry, rz};
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            c[k] = __float2int_rz(__fdiv_rn(__fsub_rn(p[k], g.scmin_pos[k]), g.sc_cs));
            lo[k] = min(max(c[k] - ext, 0), res[k] - 1);
            hi[k] = min(max(c[k] + ext, 0), res[k] - 1);
            aa[k] = __fsub_rn(p[k], h);
            bb[k] = __fadd_rn(p[k], h);
        }
        const int W = hi[0] - lo[0] + 1;            // row width
        if (W <= 0 || hi[1] < lo[1] || hi[2] < lo[2]) continue;
        const int ny = hi[1] - lo[1] + 1, nz = hi[2] - lo[2] + 1;
        const int nrows = ny * nz;
        for (int x0 = 0; x0 < W; x0 += 32) {        // row chunks of at most 32 vertices
            const int Wc = min(32, W - x0);
            const int rpi = 32 / Wc;                 // rows per warp pass
            const int my_row = lane / Wc, my_x = lane - my_row * Wc;
            for (int r0 = 0; r0 < nrows; r0 += rpi) {
                const int row = r0 + my_row;
                bool pass = false;
                int y = 0, z = 0;
                if (my_row < rpi && row < nrows) {
                    y = lo[1] + row % ny;
                    z = lo[2] + row / ny;
                    const int x = lo[0] + x0 + my_x;
                    const float vx = sc_coord_i(g, x, 0), vy = sc_coord_i(g, y, 1), vz = sc_coord_i(g, z, 2);
                    const bool outside = (vx < aa[0] || vy < aa[1] || vz < aa[2]) || (vx > bb[0] || vy > bb[1] || vz > bb[2]);
                    if (!outside) {
                        const float dx = __fsub_rn(vx, p[0]), dy = __fsub_rn(vy, p[1]), dz = __fsub_rn(vz, p[2]);
                        const float dot = __fadd_rn(__fadd_rn(__fmul_rn(n4.x, dx), __fmul_rn(n4.y, dy)), __fmul_rn(n4.z, dz));
                        pass = flag || dot > 0.f;
                    }
                }
                const uint32_t bal = __ballot_sync(0xffffffffu, pass);
                if (my_row < rpi && row < nrows && my_x == 0) {
                    const uint32_t mask = (Wc == 32) ? bal : ((bal >> (my_row * Wc)) & ((1u << Wc) - 1u));
                    if (mask) {
                        const uint64_t bit = (uint64_t)z * rxy + (uint64_t)y * (uint64_t)rx + (uint64_t)(lo[0] + x0);
                        const uint64_t w = bit >> 5;
                        const uint32_t sh = (uint32_t)(bit & 31u);
                        if (bit < nbits) atomicOr(&bm0[w], mask << sh);
                        if (sh && (mask >> (32u - sh)) && ((w + 1) << 5) < nbits) atomicOr(&bm0[w + 1], mask >> (32u - sh));
                    }
                }
            }
        }
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

pms_status launch_band(pms_ctx* ctx) {
    const KGrid g = kgrid_of(ctx->grid);
    Counters* cnt = ctx->counters.as<Counters>();
    const uint64_t nbits = g.sc_size, nwords = (nbits + 31) / 32;
    PMS_CUDA(ctx, cudaMemsetAsync(ctx->bm0.p, 0, sizeof(uint32_t) * nwords, ctx->stream));
    k_band_mark<<<grid_for((uint64_t)ctx->n * 32u, 256), 256, 0, ctx->stream>>>(
        g, ctx->prm.h, ctx->slist.as<uint32_t>(), cnt, ctx->spos.as<float4>(), ctx->nrm4.as<float4>(), ctx->bm0.as<uint32_t>());
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
