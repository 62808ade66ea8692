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
#include "pms_internal.h"
#include "k_common.cuh"

namespace pms {

struct FieldParams {
    float h;                  // isotropic support, the smallest culling radius of a cell
    float thr;                // 2 * iso: the early-exit threshold
    float grow;               // relative margin on culling radii
};

__device__ __forceinline__ float gap2_axis(float p, float lo, float cs, float pad) {
    float a = lo - pad, b = lo + cs + pad;
    float d = fmaxf(a - p, p - b);
    return d > 0.f ? d * d : 0.f;
}

// true when vertex v is within the culling radius of cell c's particle box
// (cell records: {min xyz, r^2}, {max xyz, 0}; r^2 = -1 for an empty cell)
__device__ __forceinline__ bool cell_reaches(const float4* __restrict__ rec, uint32_t c, const float3 v) {
    const float4 b0 = __ldg(&rec[2 * (size_t)c]), b1 = __ldg(&rec[2 * (size_t)c + 1]);
    const float dx = fmaxf(fmaxf(b0.x - v.x, v.x - b1.x), 0.f);
    const float dy = fmaxf(fmaxf(b0.y - v.y, v.y - b1.y), 0.f);
    const float dz = fmaxf(fmaxf(b0.z - v.z, v.z - b1.z), 0.f);
    return dx * dx + dy * dy + dz * dz < b0.w;
}

// Sum of the contributions of particles [j0, j1) at vertex v.  A particle adds
// sigma det(G) (m/rho) (1 - |G r|^2)^3 when |G r|^2 < 1 (anisotropicW,
// myCuda.cuh:151-191); every other particle adds exactly 0.  The reference
// also tests |r| < maxvalue * h first, which |G r| < 1 already implies
// (maxvalue * h = 1 / smallest singular value of G); at the very edge the two
// can differ only by rounding, where the contribution is ~0.  |G r|^2 is
// evaluated as r^T M r with the packed M = G^T G (off-diagonals doubled) and
// the weight w = (m/rho) sigma det(G) stored per particle.
__device__ __forceinline__ float range_sum(uint32_t j0, uint32_t j1, const float3 v, const float4* __restrict__ spos,
                                           const float4* __restrict__ aniso, float sum) {
#pragma unroll 2
    for (uint32_t j = j0; j < j1; ++j) {
        const float4 q = __ldg(&spos[j]);
        const float4 a0 = __ldg(&aniso[2 * (size_t)j]);      // {m00, 2 m01, 2 m02, h_s^2}
        const float4 a1 = __ldg(&aniso[2 * (size_t)j + 1]);  // {m11, 2 m12, m22, w}
        const float rx = q.x - v.x, ry = q.y - v.y, rz = q.z - v.z;
        const float d2 = rx * (a0.x * rx + a0.y * ry + a0.z * rz) + ry * (a1.x * ry + a1.y * rz) + rz * (a1.z * rz);
        const float x = 1.f - d2;
        sum += (d2 < 1.f) ? a1.w * (x * x * x) : 0.f;
    }
    return sum;
}

// BT threads per block (autotuned: 64, 128 or 256), 48 registers per thread at most
// (40 resident warps per SM).
// cell_rad holds sp_size per-cell support radii followed by one radius per row
// (z, y): the largest maxvalue * h of the row's particles (0 where none is
// anisotropic).  The z and y ranges are cut from the largest support of the
// frame, each row's x range from the row's own radius, and each non-empty cell
// by its record: the bounding box of its particles and its largest support.
// The value goes to field[t] (band order; skipped when field is null) and to
// fdense[id] (the whole scalar grid).
template <int BT>
__global__ void __launch_bounds__(BT, 1280 / BT) k_field(KGrid g, FieldParams fp, const Counters* __restrict__ cnt,
                                                    const uint32_t* __restrict__ n_dev,
                                                    const uint32_t* __restrict__ vlist, const uint32_t* __restrict__ cell_start,
                                                    const float* __restrict__ cell_rad, const float4* __restrict__ rec,
                                                    const float4* __restrict__ spos, const float4* __restrict__ aniso,
                                                    float* __restrict__ field, float* __restrict__ fdense) {
    const uint32_t nv = *n_dev;
    const uint32_t rx = g.scres[0], rxy = g.scres[0] * g.scres[1];
    const uint32_t srx = g.spres[0], sry = g.spres[1];
    const uint32_t e2 = 2u * (uint32_t)g.spexpand;
    const float pad = 1e-4f * g.sp_cs, inv_cs = 1.f / g.sp_cs;
    const float* __restrict__ row_rad = cell_rad + g.sp_size;
    // largest support of any particle this frame
    const float rmax = fmaxf(__uint_as_float(cnt->rad_max_bits), fp.h) * fp.grow;
    const float rmax2 = rmax * rmax;
    for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < nv; t += gridDim.x * blockDim.x) {
        const uint32_t id = vlist[t];
        const uint32_t iz = id / rxy, rem = id - iz * rxy, iy = rem / rx, ix = rem - iy * rx;
        const float3 v = make_float3(sc_coord(g, ix, 0), sc_coord(g, iy, 1), sc_coord(g, iz, 2));
        const uint3 c = sp_cell(g, v.x, v.y, v.z);
        uint3 lo, hi;
        box_clamp(g, c, e2, lo, hi);             // the reference's loops run to hi exclusive
        const float ux = (v.x - g.min_pos[0]) * inv_cs, uy = (v.y - g.min_pos[1]) * inv_cs,
                    uz = (v.z - g.min_pos[2]) * inv_cs;
        float sum = 0.f;
        int za, zb;
        cell_range(uz, rmax * inv_cs + kRangeMargin, lo.z, hi.z, za, zb);
        for (int z = za; z < zb; ++z) {
            const float gz = gap2_axis(v.z, g.min_pos[2] + (float)z * g.sp_cs, g.sp_cs, pad);
            if (gz >= rmax2) continue;
            int ya, yb;
            cell_range(uy, sqrtf(rmax2 - gz) * inv_cs + kRangeMargin, lo.y, hi.y, ya, yb);
            for (int y = ya; y < yb; ++y) {
                const float gyz = gz + gap2_axis(v.y, g.min_pos[1] + (float)y * g.sp_cs, g.sp_cs, pad);
                const uint32_t rowi = (uint32_t)z * sry + (uint32_t)y;
                const float rr = fmaxf(__ldg(&row_rad[rowi]), fp.h) * fp.grow;
                const float rr2 = rr * rr;
                if (gyz >= rr2) continue;           // every cell of the row adds 0
                const uint32_t row = rowi * srx;
                if (sum > fp.thr) {
                    // threshold crossed: the reference adds this row's first cell, then breaks
                    if (lo.x < hi.x && cell_reaches(rec, row + lo.x, v))
                        sum = range_sum(__ldg(&cell_start[row + lo.x]), __ldg(&cell_start[row + lo.x + 1]), v, spos,
                                        aniso, sum);
                    continue;
                }
                // cells of the row the row's largest support can reach, 32 at a time:
                // first the cells whose record the vertex reaches (independent loads),
                // then their particles in x order until the threshold is crossed
                int xa, xb;
                cell_range(ux, sqrtf(rr2 - gyz) * inv_cs + kRangeMargin, lo.x, hi.x, xa, xb);
                for (int x0 = xa; x0 < xb; x0 += 32) {
                    const int nx = min(xb - x0, 32);
                    uint32_t reach = 0u;
                    for (int k = 0; k < nx; ++k)
                        reach |= (cell_reaches(rec, row + (uint32_t)(x0 + k), v) ? 1u : 0u) << k;
                    while (reach) {
                        const uint32_t cell = row + (uint32_t)(x0 + __ffs(reach) - 1);
                        reach &= reach - 1u;
                        sum = range_sum(__ldg(&cell_start[cell]), __ldg(&cell_start[cell + 1u]), v, spos, aniso, sum);
                        if (sum > fp.thr) break;
                    }
                    if (sum > fp.thr) break;
                }
            }
        }
        if (field) field[t] = sum;
        fdense[id] = sum;
    }
}

pms_status launch_field_on(pms_ctx* ctx, const uint32_t* vlist, const uint32_t* n_dev, uint32_t n_host, float* out) {
    const KGrid g = kgrid_of(ctx->grid);
    const pms_params& P = ctx->prm;
    FieldParams fp;
    fp.h = P.h;
    fp.thr = 2.f * P.iso_value;
    fp.grow = kSupportGrow;
    Counters* cnt = ctx->counters.as<Counters>();
    const int bt = ctx->tune.field_threads;
    const unsigned blocks = grid_for(n_host, (unsigned)bt, 152u * (unsigned)ctx->tune.field_waves * (1280u / (unsigned)bt));
    auto go = [&](auto kern) {
        kern<<<blocks, bt, 0, ctx->stream>>>(g, fp, cnt, n_dev, vlist, ctx->cell_start.as<uint32_t>(),
                                             ctx->cell_rad.as<float>(), ctx->cell_rec.as<float4>(), ctx->spos.as<float4>(),
                                             ctx->aniso.as<float4>(), out, ctx->fdense.as<float>());
    };
    if (bt == 64) go(k_field<64>);
    else if (bt == 256) go(k_field<256>);
    else go(k_field<128>);
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
