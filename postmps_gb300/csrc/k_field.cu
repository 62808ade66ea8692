// k_field.cu -- narrow-band scalar field.
//
// Reference: computationOfScalarFieldGrid, Anisotropic_kernel.cuh:656-777 with
// anisotropicW / anisotropicWOpt (myCuda.cuh:151-191).  For band vertex v at
// position x_v (float32 i*cell + min) in spatial cell c it sums, over cells
// z, y, x in the HALF-OPEN box [c - 2e, c + 2e) (clamped), in that order:
//   surface cell:  (m / rho_j) * sigma * det(G_j) * (1 - |G_j r|^2)^3
//                  if |r| < maxvalue_j * h and |G_j r|^2 < 1, r = x_j - x_v
//   other cell:    (m / rho_j) * sigma / h^3 * (1 - |r|^2 / h^2)^3   if |r| < h
// skipping particles with rho == 0, and after each CELL tests
// sum > 2 * iso, which breaks only the innermost (x) loop: once the sum has
// crossed the threshold, every later row adds exactly its first cell.
//
// GB300 design: thread per band vertex, consecutive threads on consecutive
// band vertices (neighbours along x share almost all cells, so the particle
// loads hit in L1).  Every particle carries its kernel in one packed form --
// symmetric G, h_s^2 and sigma*det(G), with G = I/h, h_s = h for particles of
// non-surface cells -- so one branch-free formula serves both kinds and the
// loads of consecutive particles overlap.  The cells x in [xa, xb) of a row are
// the contiguous particle range [cell_start[row + xa], cell_start[row + xb]);
// slabs and rows are cut to those the largest support can reach, each row to
// the cells its own largest support reaches, and a cell whose particles' bounding
// box lies beyond the support of every particle in it (h, or the cell's largest
// maxvalue * h recorded by the anisotropy pass) contributes exactly zero and is
// skipped.
// Adding a zero contribution leaves the sum unchanged, so no cut changes the
// reference's sum or its early exit: the threshold test after a skipped cell
// sees the same sum as the test before it.
//
// Sign certification (the learned band's exact fallback; no reference
// counterpart).  Every term of the sum is >= 0 and float addition of a
// non-negative term never decreases a sum, so a vertex is certainly above the
// iso-value -- marching-cubes corner bit clear, whatever the rest of its walk
// would add -- as soon as a part of its sum exceeds iso.  In this mode a vertex
// (1) first sums the particles of the 2 x 2 x 2 spatial cells nearest to it (in
// any order; the test then asks for iso * (1 + 2^-9), which covers the rounding
// of two float sums in different orders of up to ~30,000 non-zero terms each);
// (2) failing that, walks in the reference's order and stops as soon as its
// running sum exceeds iso -- that prefix is the reference's own, since the
// reference's early exit (2 * iso) cannot have fired before.  A vertex stopped
// either way gets a placeholder above iso (its partial sum) and a bit in
// `cert`; a vertex whose walk ran to the end has exactly the reference's value
// (no early exit fired, the sum never exceeded iso).
#include <type_traits>

#include "pms_internal.h"
#include "k_common.cuh"

namespace pms {

struct FieldParams {
    float h;                  // isotropic support, the smallest culling radius of a cell
    float thr;                // 2 * iso: the early-exit threshold (certification: iso)
    float grow;               // relative margin on culling radii
    float quick;              // certification: iso * (1 + 2^-9), the nearest-cells test
};

__device__ __forceinline__ float gap2_axis(float p, float lo, float cs, float pad) {
    float a = lo - pad, b = lo + cs + pad;
    float d = fmaxf(a - p, p - b);
    return d > 0.f ? d * d : 0.f;
}

// A particle adds sigma det(G) (m/rho) (1 - |G r|^2)^3 when |G r|^2 < 1
// (anisotropicW, myCuda.cuh:151-191); every other particle adds exactly 0.
// The reference also tests |r| < maxvalue * h first, which |G r| < 1 already
// implies (maxvalue * h = 1 / smallest singular value of G); at the very edge
// the two can differ only by rounding, where the contribution is ~0.  |G r|^2
// is evaluated as r^T M r with the packed M = G^T G (off-diagonals doubled)
// and the weight w = (m/rho) sigma det(G) stored per particle.
// A work item is a run of up to K band vertices that are neighbours along x
// (ids id0, id0 + 1, ...; one row of the scalar grid): item = first band index
// t0 | (count - 1) << 29.  The run shares the slabs and rows of its walk (same
// y and z), each cell's bounds and record loads and each particle's loads;
// every vertex keeps its own window, x range, sum and early exit, and adds its
// contributions in the reference's order, so each value is the one a walk of
// that vertex alone gives.
static constexpr uint32_t kItemShift = 29;

// BT threads per block (autotuned: 64, 128 or 256), K vertices per item (1, 2
// or 4, autotuned).  cell_rad holds sp_size per-cell support radii followed by
// one radius per row (z, y): the largest maxvalue * h of the row's particles
// (0 where none is anisotropic).  The z and y ranges are cut from the largest
// support of the frame, each row's x range from the row's own radius, and each
// non-empty cell by its record: the bounding box of its particles and its
// largest support.  The value goes to field[t] (band order; skipped when field
// is null) and to fdense[id] (the whole scalar grid).
// CERT: sign certification (above); cert receives a bit per vertex stopped above
// iso, n_cert their count.
template <int BT, int K, bool CERT>
__global__ void __launch_bounds__(BT, (K == 1 ? 1280 : 1024) / BT)
k_field(KGrid g, FieldParams fp, const Counters* __restrict__ cnt, const uint32_t* __restrict__ n_items_dev,
        const uint32_t* __restrict__ items, const uint32_t* __restrict__ vlist, const uint32_t* __restrict__ cell_start,
        const float* __restrict__ cell_rad, const float4* __restrict__ rec, const float4* __restrict__ spos,
        const float4* __restrict__ aniso, float* __restrict__ field, float* __restrict__ fdense,
        uint32_t* __restrict__ cert, uint32_t* __restrict__ n_cert, Counters* __restrict__ cnt_w) {
    const uint32_t n_items = *n_items_dev;
    uint32_t my_cert = 0;
    unsigned long long my_pairs = 0;         // (vertex, particle) pairs evaluated
    const uint32_t rx = g.scres[0], rxy = g.scres[0] * g.scres[1];
    const uint32_t srx = g.spres[0], sry = g.spres[1];
    const uint32_t e2 = 2u * (uint32_t)g.spexpand;
    const float pad = 1e-4f * g.sp_cs, inv_cs = 1.f / g.sp_cs;
    const float* __restrict__ row_rad = cell_rad + g.sp_size;
    // largest support of any particle this frame
    const float rmax = fmaxf(__uint_as_float(cnt->rad_max_bits), fp.h) * fp.grow;
    const float rmax2 = rmax * rmax;
    for (uint32_t it = blockIdx.x * blockDim.x + threadIdx.x; it < n_items; it += gridDim.x * blockDim.x) {
        const uint32_t item = items[it];
        const uint32_t t0 = item & ((1u << kItemShift) - 1u);
        const int m = (int)(item >> kItemShift) + 1;
        const uint32_t id = vlist[t0];
        const uint32_t iz = id / rxy, rem = id - iz * rxy, iy = rem / rx, ix = rem - iy * rx;
        const float vy = sc_coord(g, iy, 1), vz = sc_coord(g, iz, 2);
        float vx[K], ux[K], sum[K];
        int wlo[K], whi[K];                          // the vertices' x windows [c - 2e, c + 2e) (clamped)
        uint3 lo, hi;
#pragma unroll
        for (int k = 0; k < K; ++k) {
            vx[k] = sc_coord(g, ix + (uint32_t)k, 0);
            const uint3 c = sp_cell(g, vx[k], vy, vz);
            box_clamp(g, c, e2, lo, hi);             // y and z bounds agree for all vertices of the run
            wlo[k] = (int)lo.x;
            whi[k] = k < m ? (int)hi.x : (int)lo.x;  // vertices past the run: empty windows
            ux[k] = (vx[k] - g.min_pos[0]) * inv_cs;
            sum[k] = 0.f;
        }
        const float uy = (vy - g.min_pos[1]) * inv_cs, uz = (vz - g.min_pos[2]) * inv_cs;
        bool done[K];
#pragma unroll
        for (int k = 0; k < K; ++k) done[k] = false;
        if constexpr (CERT) {
            // the 2 x 2 x 2 cells nearest to each vertex (inside its window): the run
            // shares the two slabs and two rows, each vertex takes its own two x cells
            const int cz = (int)floorf(uz), cy = (int)floorf(uy);
            const int z2 = uz - (float)cz >= 0.5f ? cz + 1 : cz - 1, y2 = uy - (float)cy >= 0.5f ? cy + 1 : cy - 1;
            int qa[K], qb[K];
            int XA = 0x7fffffff, XB = -1;
#pragma unroll
            for (int k = 0; k < K; ++k) {
                const int cx = (int)floorf(ux[k]);
                const int x2 = ux[k] - (float)cx >= 0.5f ? cx + 1 : cx - 1;
                qa[k] = max(min(cx, x2), wlo[k]);
                qb[k] = min(max(cx, x2) + 1, whi[k]);
                if (qa[k] < qb[k]) { XA = min(XA, qa[k]); XB = max(XB, qb[k]); }
            }
#pragma unroll
            for (int s2 = 0; s2 < 4; ++s2) {
                const int z = (s2 >> 1) ? z2 : cz, y = (s2 & 1) ? y2 : cy;
                if (z < (int)lo.z || z >= (int)hi.z || y < (int)lo.y || y >= (int)hi.y) continue;
                const uint32_t row = ((uint32_t)z * sry + (uint32_t)y) * srx;
                for (int x = XA; x < XB; ++x) {
                    bool use[K];
#pragma unroll
                    for (int k = 0; k < K; ++k) use[k] = x >= qa[k] && x < qb[k];
                    const uint32_t j0 = __ldg(&cell_start[row + (uint32_t)x]), j1 = __ldg(&cell_start[row + (uint32_t)x + 1u]);
                    {
                        uint32_t nu = 0u;
#pragma unroll
                        for (int k = 0; k < K; ++k) nu += use[k] ? 1u : 0u;
                        my_pairs += (unsigned long long)(j1 - j0) * nu;
                    }
                    for (uint32_t j = j0; j < j1; ++j) {
                        const float4 q = __ldg(&spos[j]);
                        const float4 a0 = __ldg(&aniso[2 * (size_t)j]);
                        const float4 a1 = __ldg(&aniso[2 * (size_t)j + 1]);
                        const float ry = __fsub_rn(q.y, vy), rz = __fsub_rn(q.z, vz);
                        const float pyz = __fmaf_rn(rz, __fmul_rn(a1.z, rz), __fmul_rn(ry, __fmaf_rn(a1.x, ry, __fmul_rn(a1.y, rz))));
                        const float cyz = __fmaf_rn(a0.y, ry, __fmul_rn(a0.z, rz));
#pragma unroll
                        for (int k = 0; k < K; ++k) {
                            const float rxk = __fsub_rn(q.x, vx[k]);
                            const float d2 = __fmaf_rn(rxk, __fmaf_rn(a0.x, rxk, cyz), pyz);
                            const float xx = __fsub_rn(1.f, d2);
                            const float w = (d2 < 1.f) ? __fmul_rn(a1.w, __fmul_rn(__fmul_rn(xx, xx), xx)) : 0.f;
                            if (use[k]) sum[k] = __fadd_rn(sum[k], w);
                        }
                    }
                }
            }
            bool all = true;
#pragma unroll
            for (int k = 0; k < K; ++k) {
                if (k < m && sum[k] > fp.quick) {
                    done[k] = true;
                    whi[k] = wlo[k];                 // nothing left to walk
                } else {
                    sum[k] = 0.f;                    // the walk starts over in the reference's order
                    all = all && !(k < m);
                }
            }
            if (all) {
                uint32_t mask = 0u;
#pragma unroll
                for (int k = 0; k < K; ++k)
                    if (k < m) { fdense[id + k] = sum[k]; mask |= 1u << k; }
                const uint32_t w = id >> 5, sh = id & 31u;
                atomicOr(&cert[w], mask << sh);
                if (sh && (mask >> (32u - sh))) atomicOr(&cert[w + 1], mask >> (32u - sh));
                my_cert += (uint32_t)m;
                continue;
            }
        }
        int za, zb;
        cell_range(uz, rmax * inv_cs + kRangeMargin, lo.z, hi.z, za, zb);
        for (int z = za; z < zb; ++z) {
            const float gz = gap2_axis(vz, g.min_pos[2] + (float)z * g.sp_cs, g.sp_cs, pad);
            if (gz >= rmax2) continue;
            int ya, yb;
            cell_range(uy, sqrtf(rmax2 - gz) * inv_cs + kRangeMargin, lo.y, hi.y, ya, yb);
            for (int y = ya; y < yb; ++y) {
                const float gyz = gz + gap2_axis(vy, g.min_pos[1] + (float)y * g.sp_cs, g.sp_cs, pad);
                const uint32_t rowi = (uint32_t)z * sry + (uint32_t)y;
                const float rr = fmaxf(__ldg(&row_rad[rowi]), fp.h) * fp.grow;
                const float rr2 = rr * rr;
                if (gyz >= rr2) continue;           // every cell of the row adds 0
                const uint32_t row = rowi * srx;
                // each vertex's cells of this row: past the threshold, only the window's
                // first cell (the reference adds it, then breaks); else those the row's
                // largest support reaches
                const float rxc = sqrtf(rr2 - gyz) * inv_cs + kRangeMargin;
                int xs[K], xe[K];
                bool live[K];
                int X0 = 0x7fffffff, X1 = -1;
#pragma unroll
                for (int k = 0; k < K; ++k) {
                    if (!CERT && sum[k] > fp.thr) {
                        xs[k] = wlo[k];
                        xe[k] = min(wlo[k] + 1, whi[k]);
                    } else {
                        cell_range(ux[k], rxc, (uint32_t)wlo[k], (uint32_t)whi[k], xs[k], xe[k]);
                    }
                    live[k] = xs[k] < xe[k];
                    if (live[k]) { X0 = min(X0, xs[k]); X1 = max(X1, xe[k]); }
                }
                for (int x0 = X0; x0 < X1; x0 += 32) {
                    const int nx = min(X1 - x0, 32);
                    // cells of the chunk inside some live vertex's range (a vertex past the
                    // threshold needs only its window's first cell, which can sit well left
                    // of the others' ranges)
                    uint32_t need = 0u;
#pragma unroll
                    for (int k = 0; k < K; ++k) {
                        const int a = max(xs[k] - x0, 0), b = min(xe[k] - x0, nx);
                        if (live[k] && a < b) need |= (b - a == 32 ? ~0u : ((1u << (b - a)) - 1u)) << a;
                    }
                    // cells whose record each vertex reaches (independent loads)
                    uint32_t reach[K];
#pragma unroll
                    for (int k = 0; k < K; ++k) reach[k] = 0u;
                    for (uint32_t todo = need; todo; todo &= todo - 1u) {
                        const int i = __ffs(todo) - 1;
                        const int x = x0 + i;
                        const uint32_t c = row + (uint32_t)x;
                        const float4 b0 = __ldg(&rec[2 * (size_t)c]), b1 = __ldg(&rec[2 * (size_t)c + 1]);
                        const float dy = fmaxf(fmaxf(b0.y - vy, vy - b1.y), 0.f);
                        const float dz = fmaxf(fmaxf(b0.z - vz, vz - b1.z), 0.f);
                        const float dyz = dy * dy + dz * dz;
#pragma unroll
                        for (int k = 0; k < K; ++k) {
                            const float dx = fmaxf(fmaxf(b0.x - vx[k], vx[k] - b1.x), 0.f);
                            const bool in = live[k] && x >= xs[k] && x < xe[k] && dx * dx + dyz < b0.w;
                            reach[k] |= (in ? 1u : 0u) << i;
                        }
                    }
                    uint32_t any = 0u;
#pragma unroll
                    for (int k = 0; k < K; ++k) any |= reach[k];
                    // the reached cells in x order; a vertex stops for the row once its
                    // sum passes the threshold after one of its cells
                    while (any) {
                        const int i = __ffs(any) - 1;
                        const uint32_t bit = 1u << i;
                        const uint32_t c = row + (uint32_t)(x0 + i);
                        bool use[K];
#pragma unroll
                        for (int k = 0; k < K; ++k) use[k] = (reach[k] & bit) != 0u;
                        const uint32_t j0 = __ldg(&cell_start[c]), j1 = __ldg(&cell_start[c + 1u]);
                        {
                            uint32_t nu = 0u;
#pragma unroll
                            for (int k = 0; k < K; ++k) nu += use[k] ? 1u : 0u;
                            my_pairs += (unsigned long long)(j1 - j0) * nu;
                        }
#pragma unroll 1
                        for (uint32_t j = j0; j < j1; ++j) {
                            const float4 q = __ldg(&spos[j]);
                            const float4 a0 = __ldg(&aniso[2 * (size_t)j]);      // {m00, 2 m01, 2 m02, h_s^2}
                            const float4 a1 = __ldg(&aniso[2 * (size_t)j + 1]);  // {m11, 2 m12, m22, w}
                            // r^T M r with every rounding spelled out, so that the value does
                            // not depend on how many vertices share the loads
                            const float ry = __fsub_rn(q.y, vy), rz = __fsub_rn(q.z, vz);
                            const float pyz = __fmaf_rn(rz, __fmul_rn(a1.z, rz), __fmul_rn(ry, __fmaf_rn(a1.x, ry, __fmul_rn(a1.y, rz))));
                            const float cyz = __fmaf_rn(a0.y, ry, __fmul_rn(a0.z, rz));
#pragma unroll
                            for (int k = 0; k < K; ++k) {
                                const float rxk = __fsub_rn(q.x, vx[k]);
                                const float d2 = __fmaf_rn(rxk, __fmaf_rn(a0.x, rxk, cyz), pyz);
                                const float xx = __fsub_rn(1.f, d2);
                                const float w = (d2 < 1.f) ? __fmul_rn(a1.w, __fmul_rn(__fmul_rn(xx, xx), xx)) : 0.f;
                                if (use[k]) sum[k] = __fadd_rn(sum[k], w);
                            }
                        }
                        uint32_t still = 0u;
#pragma unroll
                        for (int k = 0; k < K; ++k) {
                            if (use[k] && sum[k] > fp.thr) {
                                reach[k] = 0u;
                                live[k] = false;
                                if constexpr (CERT) { done[k] = true; whi[k] = wlo[k]; }   // certified: stop for good
                            }
                            still |= reach[k];
                        }
                        any = still & ~((bit << 1) - 1u);   // i = 31: bit << 1 = 0, nothing left
                    }
                    bool more = false;
#pragma unroll
                    for (int k = 0; k < K; ++k) more |= live[k] && xe[k] > x0 + nx;
                    if (!more) break;
                }
            }
        }
        uint32_t mask = 0u;
#pragma unroll
        for (int k = 0; k < K; ++k)
            if (k < m) {
                if (field) field[t0 + k] = sum[k];
                fdense[id + k] = sum[k];
                if (done[k]) mask |= 1u << k;
            }
        if (CERT && mask) {
            const uint32_t w = id >> 5, sh = id & 31u;
            atomicOr(&cert[w], mask << sh);
            if (sh && (mask >> (32u - sh))) atomicOr(&cert[w + 1], mask >> (32u - sh));
            my_cert += (uint32_t)__popc(mask);
        }
    }
    if constexpr (CERT) {
        const uint32_t tot = __reduce_add_sync(0xffffffffu, my_cert);
        if ((threadIdx.x & 31u) == 0 && tot) atomicAdd(n_cert, tot);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) my_pairs += __shfl_xor_sync(0xffffffffu, my_pairs, o);
    if ((threadIdx.x & 31u) == 0 && my_pairs) atomicAdd(&cnt_w->n_pairs, my_pairs);
}

// Work items over vlist[0 .. *n_dev): group g = entries [g K, g K + K) splits
// into its runs of x-neighbours (id + 1 in the same row); count, then write.
__global__ void __launch_bounds__(256) k_field_items(const uint32_t* __restrict__ vlist, const uint32_t* __restrict__ n_dev,
                                                     uint32_t ngroups, uint32_t K, uint32_t rx,
                                                     const uint32_t* __restrict__ offs, uint32_t* __restrict__ out) {
    const uint32_t n = *n_dev;
    for (uint32_t g = blockIdx.x * blockDim.x + threadIdx.x; g < ngroups; g += gridDim.x * blockDim.x) {
        const uint32_t t0 = g * K, t1 = min(t0 + K, n);
        uint32_t runs = 0, start = t0, o = offs ? offs[g] : 0u;
        for (uint32_t t = t0; t < t1; ++t) {
            const uint32_t id = __ldg(&vlist[t]);
            const bool join = t > t0 && id == __ldg(&vlist[t - 1]) + 1u && id % rx != 0u;
            if (t > t0 && !join) {
                if (offs) out[o + runs] = start | ((t - start - 1u) << kItemShift);
                ++runs;
                start = t;
            }
        }
        if (t0 < t1) {
            if (offs) out[o + runs] = start | ((t1 - start - 1u) << kItemShift);
            ++runs;
        }
        if (!offs) out[g] = runs;
    }
}

pms_status launch_field_on(pms_ctx* ctx, const uint32_t* vlist, const uint32_t* n_dev, uint32_t n_host, float* out,
                           uint32_t* cert, uint32_t* n_cert) {
    const KGrid g = kgrid_of(ctx->grid);
    const pms_params& P = ctx->prm;
    FieldParams fp;
    fp.h = P.h;
    fp.thr = cert ? P.iso_value : 2.f * P.iso_value;
    fp.grow = kSupportGrow;
    fp.quick = P.iso_value * (1.f + 1.f / 512.f);
    Counters* cnt = ctx->counters.as<Counters>();
    if ((uint64_t)n_host >= (1ull << kItemShift)) return pms_fail(ctx, PMS_ERR_UNSUPPORTED, "band above 2^29 vertices");
    const uint32_t K = (uint32_t)ctx->tune.field_vpt;
    const uint32_t ngroups = (n_host + K - 1u) / K;
    PMS_CUDA(ctx, ctx->fitem_cnt.ensure(4 * ((size_t)ngroups + 1)));
    PMS_CUDA(ctx, ctx->fitem_off.ensure(4 * ((size_t)ngroups + 1)));
    PMS_CUDA(ctx, ctx->fitems.ensure(4 * ((size_t)n_host + 1)));
    const unsigned gb = grid_for(ngroups, 256);
    k_field_items<<<gb, 256, 0, ctx->stream>>>(vlist, n_dev, ngroups, K, g.scres[0], nullptr, ctx->fitem_cnt.as<uint32_t>());
    PMS_LAUNCHED(ctx);
    pms_status st = scan_u32(ctx, ctx->fitem_cnt.as<uint32_t>(), ctx->fitem_off.as<uint32_t>(), ngroups, &cnt->n_items);
    if (st != PMS_OK) return st;
    k_field_items<<<gb, 256, 0, ctx->stream>>>(vlist, n_dev, ngroups, K, g.scres[0], ctx->fitem_off.as<uint32_t>(),
                                               ctx->fitems.as<uint32_t>());
    PMS_LAUNCHED(ctx);
    const int bt = ctx->tune.field_threads;
    const unsigned per_sm = (K == 1 ? 1280u : 1024u) / (unsigned)bt;
    const unsigned blocks = grid_for(n_host, (unsigned)bt, 152u * (unsigned)ctx->tune.field_waves * per_sm);
    auto go = [&](auto kern) {
        kern<<<blocks, bt, 0, ctx->stream>>>(g, fp, cnt, &cnt->n_items, ctx->fitems.as<uint32_t>(), vlist,
                                             ctx->cell_start.as<uint32_t>(), ctx->cell_rad.as<float>(),
                                             ctx->cell_rec.as<float4>(), ctx->spos.as<float4>(), ctx->aniso.as<float4>(), out,
                                             ctx->fdense.as<float>(), cert, n_cert, cnt);
    };
    auto by_vpt = [&](auto bt_tag) {
        constexpr int B = decltype(bt_tag)::value;
        if (cert) {
            if (K == 1) go(k_field<B, 1, true>);
            else if (K == 4) go(k_field<B, 4, true>);
            else go(k_field<B, 2, true>);
        } else {
            if (K == 1) go(k_field<B, 1, false>);
            else if (K == 4) go(k_field<B, 4, false>);
            else go(k_field<B, 2, false>);
        }
    };
    if (bt == 64) by_vpt(std::integral_constant<int, 64>());
    else if (bt == 256) by_vpt(std::integral_constant<int, 256>());
    else by_vpt(std::integral_constant<int, 128>());
    PMS_LAUNCHED(ctx);
    return PMS_OK;
}

// the frame's first field evaluation: the dense field starts at 0 everywhere
pms_status launch_field(pms_ctx* ctx) {
    Counters* cnt = ctx->counters.as<Counters>();
    PMS_CUDA(ctx, cudaMemsetAsync(ctx->fdense.p, 0, 4 * (size_t)ctx->grid.sc_size, ctx->stream));
    return launch_field_on(ctx, ctx->vlist.as<uint32_t>(), &cnt->nv, ctx->nv, ctx->field.as<float>());
}

// field[t] = fdense[vlist[t]]: the band-order field of a vertex list whose values are all computed
__global__ void __launch_bounds__(256) k_field_gather(const uint32_t* __restrict__ vlist, const uint32_t* __restrict__ n_dev,
                                                      const float* __restrict__ fdense, float* __restrict__ field) {
    const uint32_t n = *n_dev;
    for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x)
        field[t] = __ldg(&fdense[__ldg(&vlist[t])]);
}

pms_status launch_field_gather(pms_ctx* ctx, const uint32_t* vlist, const uint32_t* n_dev, uint32_t n_host, float* out) {
    k_field_gather<<<grid_for(n_host, 256), 256, 0, ctx->stream>>>(vlist, n_dev, ctx->fdense.as<float>(), out);
    PMS_LAUNCHED(ctx);
    return PMS_OK;
}

}  // namespace pms
