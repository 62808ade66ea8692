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

// ---------------------------------------------------------------------------
// Plain-band membership of single vertices, for the learned band: a vertex
// belongs to the band of k_band_mark + k_band_dilate when a surface particle
// marks it or the vertex one step lower in linear order along x, y or z (the
// dilation B0 | B0 << 1 | B0 << rx | B0 << rx*ry, row wrap included).  The
// test looks from the vertex at the surface cells within h instead of marking
// from every surface particle, and repeats k_band_mark's per-particle test
// with the same roundings, so it answers exactly what the bitmap would hold.
// ---------------------------------------------------------------------------

// k_band_mark's test of one (particle, vertex) pair: the AABB p +- h, the
// direction flag || n . (v - p) > 0, and the index box c +- ext clamped to the grid
__device__ __forceinline__ bool marks(const KGrid& g, float h, int ext, float4 p, float4 n, int ix, int iy, int iz,
                                      float vx, float vy, float vz) {
    if (vx < __fsub_rn(p.x, h) || vy < __fsub_rn(p.y, h) || vz < __fsub_rn(p.z, h) || vx > __fadd_rn(p.x, h) ||
        vy > __fadd_rn(p.y, h) || vz > __fadd_rn(p.z, h))
        return false;
    if (n.w == 0.f) {
        const float dx = __fsub_rn(vx, p.x), dy = __fsub_rn(vy, p.y), dz = __fsub_rn(vz, p.z);
        const float dot = __fadd_rn(__fadd_rn(__fmul_rn(n.x, dx), __fmul_rn(n.y, dy)), __fmul_rn(n.z, dz));
        if (!(dot > 0.f)) return false;
    }
    const int cx = __float2int_rz(__fdiv_rn(__fsub_rn(p.x, g.scmin_pos[0]), g.sc_cs));
    const int cy = __float2int_rz(__fdiv_rn(__fsub_rn(p.y, g.scmin_pos[1]), g.sc_cs));
    const int cz = __float2int_rz(__fdiv_rn(__fsub_rn(p.z, g.scmin_pos[2]), g.sc_cs));
    const int rx = (int)g.scres[0] - 1, ry = (int)g.scres[1] - 1, rz = (int)g.scres[2] - 1;
    return ix >= min(max(cx - ext, 0), rx) && ix <= min(max(cx + ext, 0), rx) && iy >= min(max(cy - ext, 0), ry) &&
           iy <= min(max(cy + ext, 0), ry) && iz >= min(max(cz - ext, 0), rz) && iz <= min(max(cz + ext, 0), rz);
}

// Does a particle of the surface cells [xa, xb) x [ya, yb) x [za, zb) mark one
// of the NT (1 or 3) target vertices?  Targets t with bit t of `use` clear are skipped.
template <int NT>
__device__ bool scan_cells(const KGrid& g, float h, int ext, const uint2* __restrict__ cell_info,
                           const float4* __restrict__ spos, const float4* __restrict__ nrm4, int xa, int xb, int ya,
                           int yb, int za, int zb, const int (&ix)[NT], const int (&iy)[NT], const int (&iz)[NT],
                           const float (&vx)[NT], const float (&vy)[NT], const float (&vz)[NT], uint32_t use) {
    for (int cz = za; cz < zb; ++cz)
        for (int cy = ya; cy < yb; ++cy) {
            const uint32_t row = ((uint32_t)cz * g.spres[1] + (uint32_t)cy) * g.spres[0];
            for (int cx = xa; cx < xb; ++cx) {
                const uint2 ci = __ldg(&cell_info[row + (uint32_t)cx]);
                if (!(ci.y & 0x80000000u)) continue;         // empty or not a surface cell
                const uint32_t j1 = ci.x + (ci.y & 0x7fffffffu);
                for (uint32_t j = ci.x; j < j1; ++j) {
                    const float4 p = __ldg(&spos[j]), n = __ldg(&nrm4[j]);
#pragma unroll
                    for (int t = 0; t < NT; ++t)
                        if (((use >> t) & 1u) && marks(g, h, ext, p, n, ix[t], iy[t], iz[t], vx[t], vy[t], vz[t]))
                            return true;
                }
            }
        }
    return false;
}

// the surface cells within h of the box [lo, hi]: every particle that can mark a vertex of the box
template <int NT>
__device__ __forceinline__ bool scan_marks(const KGrid& g, float h, int ext, const uint2* __restrict__ cell_info,
                                           const float4* __restrict__ spos, const float4* __restrict__ nrm4, float lox,
                                           float loy, float loz, float hix, float hiy, float hiz, const int (&ix)[NT],
                                           const int (&iy)[NT], const int (&iz)[NT], const float (&vx)[NT],
                                           const float (&vy)[NT], const float (&vz)[NT], uint32_t use) {
    const float inv = 1.f / g.sp_cs, r = h * inv + kRangeMargin;
    return scan_cells<NT>(g, h, ext, cell_info, spos, nrm4, max((int)floorf((lox - g.min_pos[0]) * inv - r), 0),
                          min((int)floorf((hix - g.min_pos[0]) * inv + r) + 1, (int)g.spres[0]),
                          max((int)floorf((loy - g.min_pos[1]) * inv - r), 0),
                          min((int)floorf((hiy - g.min_pos[1]) * inv + r) + 1, (int)g.spres[1]),
                          max((int)floorf((loz - g.min_pos[2]) * inv - r), 0),
                          min((int)floorf((hiz - g.min_pos[2]) * inv + r) + 1, (int)g.spres[2]), ix, iy, iz, vx, vy, vz, use);
}

// B0 at vertex (x, y, z)
__device__ __forceinline__ bool in_b0(const KGrid& g, float h, int ext, const uint2* __restrict__ cell_info,
                                      const float4* __restrict__ spos, const float4* __restrict__ nrm4, int x, int y, int z) {
    const int ix[1] = {x}, iy[1] = {y}, iz[1] = {z};
    const float vx[1] = {sc_coord_i(g, x, 0)}, vy[1] = {sc_coord_i(g, y, 1)}, vz[1] = {sc_coord_i(g, z, 2)};
    return scan_marks<1>(g, h, ext, cell_info, spos, nrm4, vx[0], vy[0], vz[0], vx[0], vy[0], vz[0], ix, iy, iz, vx, vy, vz, 1u);
}

// The quick side of the test: B0 at v, then at its three lower neighbours (no
// row wrap), from the 2 x 2 x 2 particle cells nearest to v -- most band
// vertices are marked by a particle there.  A vertex it cannot confirm goes to
// `rest` for the full test.
__global__ void __launch_bounds__(128) k_plain_quick(KGrid g, float h, const uint32_t* __restrict__ n_dev,
                                                     const uint32_t* __restrict__ list, const uint2* __restrict__ cell_info,
                                                     const float4* __restrict__ spos, const float4* __restrict__ nrm4,
                                                     uint32_t* __restrict__ rest, uint32_t* __restrict__ n_rest) {
    const uint32_t n = *n_dev;
    const int ext = (int)(uint32_t)ceilf(__fdiv_rn(h, g.sc_cs));   // as k_band_mark
    const uint32_t rx = g.scres[0], rxy = g.scres[0] * g.scres[1];
    const float inv = 1.f / g.sp_cs;
    const uint32_t lane = threadIdx.x & 31u;
    for (uint32_t t0 = blockIdx.x * blockDim.x; t0 < n; t0 += gridDim.x * blockDim.x) {
        const uint32_t t = t0 + threadIdx.x;
        bool open = false;
        uint32_t v = 0;
        if (t < n) {
            v = list[t];
            const int z = (int)(v / rxy), y = (int)((v - (uint32_t)z * rxy) / rx), x = (int)(v - (uint32_t)z * rxy - (uint32_t)y * rx);
            const int ix[1] = {x}, iy[1] = {y}, iz[1] = {z};
            const float vx[1] = {sc_coord_i(g, x, 0)}, vy[1] = {sc_coord_i(g, y, 1)}, vz[1] = {sc_coord_i(g, z, 2)};
            int a[3], b[3];
            const float u[3] = {(vx[0] - g.min_pos[0]) * inv, (vy[0] - g.min_pos[1]) * inv, (vz[0] - g.min_pos[2]) * inv};
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                const int c = (int)floorf(u[k]);
                const int lo = u[k] - (float)c < 0.5f ? c - 1 : c;
                a[k] = max(lo, 0);
                b[k] = min(lo + 2, (int)g.spres[k]);
            }
            open = !scan_cells<1>(g, h, ext, cell_info, spos, nrm4, a[0], b[0], a[1], b[1], a[2], b[2], ix, iy, iz, vx, vy,
                                  vz, 1u);
            const uint32_t use = (x > 0 ? 1u : 0u) | (y > 0 ? 2u : 0u) | (z > 0 ? 4u : 0u);
            if (open && use) {
                const int jx[3] = {x - 1, x, x}, jy[3] = {y, y - 1, y}, jz[3] = {z, z, z - 1};
                const float qx = sc_coord_i(g, x - 1, 0), qy = sc_coord_i(g, y - 1, 1), qz = sc_coord_i(g, z - 1, 2);
                const float wx[3] = {qx, vx[0], vx[0]}, wy[3] = {vy[0], qy, vy[0]}, wz[3] = {vz[0], vz[0], qz};
                open = !scan_cells<3>(g, h, ext, cell_info, spos, nrm4, a[0], b[0], a[1], b[1], a[2], b[2], jx, jy, jz, wx, wy,
                                      wz, use);
            }
        }
        // warp-aggregated append of the open vertices
        const uint32_t m = __ballot_sync(0xffffffffu, open);
        uint32_t base = 0;
        if (lane == 0 && m) base = atomicAdd(n_rest, (uint32_t)__popc(m));
        base = __shfl_sync(0xffffffffu, base, 0);
        if (open) rest[base + (uint32_t)__popc(m & ((1u << lane) - 1u))] = v;
    }
}

// membership of vertex v = (x, y, z) in the dilated band
__device__ bool in_plain_band(const KGrid& g, float h, int ext, const uint2* __restrict__ cell_info,
                              const float4* __restrict__ spos, const float4* __restrict__ nrm4, uint32_t v) {
    const uint32_t rx = g.scres[0], ry = g.scres[1], rxy = rx * ry;
    const int z = (int)(v / rxy), y = (int)((v - (uint32_t)z * rxy) / rx), x = (int)(v - (uint32_t)z * rxy - (uint32_t)y * rx);
    if (in_b0(g, h, ext, cell_info, spos, nrm4, x, y, z)) return true;
    // the lower neighbours v - 1, v - rx, v - rx*ry where they do not wrap, in one scan
    const uint32_t use = (x > 0 ? 1u : 0u) | (y > 0 ? 2u : 0u) | (z > 0 ? 4u : 0u);
    if (use) {
        const int ix[3] = {x - 1, x, x}, iy[3] = {y, y - 1, y}, iz[3] = {z, z, z - 1};
        const float px = sc_coord_i(g, x, 0), py = sc_coord_i(g, y, 1), pz = sc_coord_i(g, z, 2);
        const float qx = sc_coord_i(g, x - 1, 0), qy = sc_coord_i(g, y - 1, 1), qz = sc_coord_i(g, z - 1, 2);
        const float vx[3] = {qx, px, px}, vy[3] = {py, qy, py}, vz[3] = {pz, pz, qz};
        if (scan_marks<3>(g, h, ext, cell_info, spos, nrm4, (use & 1u) ? qx : px, (use & 2u) ? qy : py,
                          (use & 4u) ? qz : pz, px, py, pz, ix, iy, iz, vx, vy, vz, use))
            return true;
    }
    // at x == 0 (y == 0) the linear shift wraps to the row (slab) below; z == 0 has nothing below
    if (x == 0 && v >= 1) {
        const uint32_t u = v - 1, uz = u / rxy, uy = (u - uz * rxy) / rx;
        if (in_b0(g, h, ext, cell_info, spos, nrm4, (int)(u - uz * rxy - uy * rx), (int)uy, (int)uz)) return true;
    }
    if (y == 0 && v >= rx) {
        const uint32_t u = v - rx, uz = u / rxy, uy = (u - uz * rxy) / rx;
        if (in_b0(g, h, ext, cell_info, spos, nrm4, (int)(u - uz * rxy - uy * rx), (int)uy, (int)uz)) return true;
    }
    (void)ry;
    return false;
}

// The listed vertices outside the plain band leave the vertex set: the bit in
// vbm is cleared, the dense field value set to 0 (what a vertex off the band
// reads) and n_removed counts them.
__global__ void __launch_bounds__(128) k_plain_member(KGrid g, float h, const uint32_t* __restrict__ n_dev,
                                                      const uint32_t* __restrict__ list, const uint2* __restrict__ cell_info,
                                                      const float4* __restrict__ spos, const float4* __restrict__ nrm4,
                                                      uint32_t* __restrict__ vbm, float* __restrict__ fdense,
                                                      uint32_t* __restrict__ n_removed) {
    const uint32_t n = *n_dev;
    const int ext = (int)(uint32_t)ceilf(__fdiv_rn(h, g.sc_cs));   // as k_band_mark
    for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
        const uint32_t v = list[t];
        if (in_plain_band(g, h, ext, cell_info, spos, nrm4, v)) continue;
        atomicAnd(&vbm[v >> 5], ~(1u << (v & 31u)));
        fdense[v] = 0.f;
        atomicAdd(n_removed, 1u);
    }
}

pms_status launch_plain_member(pms_ctx* ctx, const uint32_t* list, const uint32_t* n_dev, uint32_t n_host, uint32_t* rest,
                               uint32_t* n_rest, uint32_t* n_removed) {
    const KGrid g = kgrid_of(ctx->grid);
    PMS_CUDA(ctx, cudaMemsetAsync(n_rest, 0, sizeof(uint32_t), ctx->stream));
    k_plain_quick<<<grid_for(n_host, 128), 128, 0, ctx->stream>>>(g, ctx->prm.h, n_dev, list, ctx->cell_info.as<uint2>(),
                                                                  ctx->spos.as<float4>(), ctx->nrm4.as<float4>(), rest, n_rest);
    PMS_LAUNCHED(ctx);
    k_plain_member<<<grid_for(n_host, 128), 128, 0, ctx->stream>>>(
        g, ctx->prm.h, n_rest, rest, ctx->cell_info.as<uint2>(), ctx->spos.as<float4>(), ctx->nrm4.as<float4>(),
        ctx->bm.as<uint32_t>(), ctx->fdense.as<float>(), n_removed);
    PMS_LAUNCHED(ctx);
    return PMS_OK;
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
