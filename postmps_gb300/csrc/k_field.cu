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
// loads hit in L1).  A cell whose box lies beyond the support of every
// particle in it (h for isotropic cells, the cell's largest maxvalue * h for
// anisotropic ones, recorded by the anisotropy pass) contributes exactly zero
// and is skipped, except that the first cell of a row is still visited once
// the threshold is crossed; both keep the reference's sum in its semantics.
// Particle data come from SoA float4 (x, y, z, m/rho) and two float4 of the
// symmetric G, h_s^2 and sigma*det precomputed per surface particle.
#include "pms_internal.h"
#include "k_common.cuh"

namespace pms {

static constexpr int kThreads = 128;
static constexpr float kSigma = 1.56668147f;

struct FieldParams {
    float h, h_sq, inv_h2, c_iso, thr;
    float r_iso2;             // culling radius of isotropic cells, squared
    float grow;               // relative margin on culling radii
};

__device__ __forceinline__ float gap2_axis(float p, float lo, float cs, float pad) {
    float a = lo - pad, b = lo + cs + pad;
    float d = fmaxf(a - p, p - b);
    return d > 0.f ? d * d : 0.f;
}

__device__ __forceinline__ float cell_sum(const uint2 ci, const float3 v, const FieldParams& fp,
                                          const float4* __restrict__ spos, const float4* __restrict__ aniso, float sum) {
    const uint32_t m = ci.y & 0x7fffffffu;
    if (ci.y & 0x80000000u) {
        for (uint32_t j = ci.x; j < ci.x + m; ++j) {
            const float4 q = __ldg(&spos[j]);
            const float rx = q.x - v.x, ry = q.y - v.y, rz = q.z - v.z;
            const float l2 = rx * rx + ry * ry + rz * rz;
            const float4 a0 = __ldg(&aniso[2 * (size_t)j]);
            if (l2 >= a0.w) continue;                    // |r| >= maxvalue * h
            const float4 a1 = __ldg(&aniso[2 * (size_t)j + 1]);
            const float tx = rx * a0.x + ry * a0.y + rz * a0.z;
            const float ty = rx * a0.y + ry * a1.x + rz * a1.y;
            const float tz = rx * a0.z + ry * a1.y + rz * a1.z;
            const float d2 = tx * tx + ty * ty + tz * tz;
            if (d2 >= 1.f) continue;
            const float x = 1.f - d2;
            sum += q.w * (a1.w * x * x * x);
        }
    } else {
        for (uint32_t j = ci.x; j < ci.x + m; ++j) {
            const float4 q = __ldg(&spos[j]);
            const float rx = q.x - v.x, ry = q.y - v.y, rz = q.z - v.z;
            const float l2 = rx * rx + ry * ry + rz * rz;
            if (l2 >= fp.h_sq) continue;
            const float x = 1.f - l2 * fp.inv_h2;
            sum += q.w * (fp.c_iso * x * x * x);
        }
    }
    return sum;
}

// culling radius of one cell: maxvalue * h of its particles (anisotropic cells) or h
__device__ __forceinline__ float cell_lim2(uint2 ci, const float* __restrict__ cell_rad, uint32_t c, const FieldParams& fp) {
    if (!(ci.y & 0x80000000u)) return fp.r_iso2;
    const float r = __ldg(&cell_rad[c]) * fp.grow;
    return r * r;
}

__global__ void __launch_bounds__(kThreads, 8) k_field(KGrid g, FieldParams fp, const Counters* __restrict__ cnt,
                                                    const uint32_t* __restrict__ vlist, const uint2* __restrict__ cell_info,
                                                    const float* __restrict__ cell_rad, const float4* __restrict__ spos,
                                                    const float4* __restrict__ aniso, float* __restrict__ field) {
    const uint32_t nv = cnt->nv;
    const uint32_t rx = g.scres[0], rxy = g.scres[0] * g.scres[1];
    const uint32_t srx = g.spres[0], srxy = g.spres[0] * g.spres[1];
    const uint32_t e2 = 2u * (uint32_t)g.spexpand;
    const float pad = 1e-4f * g.sp_cs;
    // largest support of any particle this frame
    const float rmax = fmaxf(__uint_as_float(cnt->rad_max_bits), fp.h) * fp.grow;
    const float rmax2 = rmax * rmax;
    for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < nv; t += gridDim.x * blockDim.x) {
        const uint32_t id = vlist[t];
        const uint32_t iz = id / rxy, rem = id - iz * rxy, iy = rem / rx, ix = rem - iy * rx;
        const float3 v = make_float3(sc_coord(g, ix, 0), sc_coord(g, iy, 1), sc_coord(g, iz, 2));
        const uint3 c = sp_cell(g, v.x, v.y, v.z);
        uint3 lo, hi;
        box_clamp(g, c, e2, lo, hi);
        float sum = 0.f;
        for (uint32_t z = lo.z; z < hi.z; ++z) {
            const float gz = gap2_axis(v.z, g.min_pos[2] + (float)z * g.sp_cs, g.sp_cs, pad);
            if (gz >= rmax2) continue;
            for (uint32_t y = lo.y; y < hi.y; ++y) {
                const float gyz = gz + gap2_axis(v.y, g.min_pos[1] + (float)y * g.sp_cs, g.sp_cs, pad);
                if (gyz >= rmax2) continue;
                const uint32_t row = z * srxy + y * srx;
                if (sum > fp.thr) {
                    // threshold crossed: the reference adds this row's first cell, then breaks
                    if (lo.x < hi.x) {
                        const float gx = gyz + gap2_axis(v.x, g.min_pos[0] + (float)lo.x * g.sp_cs, g.sp_cs, pad);
                        if (gx < rmax2) {
                            const uint2 ci = __ldg(&cell_info[row + lo.x]);
                            if (gx < cell_lim2(ci, cell_rad, row + lo.x, fp)) sum = cell_sum(ci, v, fp, spos, aniso, sum);
                        }
                    }
                    continue;
                }
                for (uint32_t x = lo.x; x < hi.x; ++x) {
                    const float gx = gyz + gap2_axis(v.x, g.min_pos[0] + (float)x * g.sp_cs, g.sp_cs, pad);
                    if (gx >= rmax2) continue;
                    const uint2 ci = __ldg(&cell_info[row + x]);
                    if ((ci.y & 0x7fffffffu) == 0 || gx >= cell_lim2(ci, cell_rad, row + x, fp)) continue;
                    sum = cell_sum(ci, v, fp, spos, aniso, sum);
                    if (sum > fp.thr) break;
                }
            }
        }
        field[t] = sum;
    }
}

pms_status launch_field(pms_ctx* ctx) {
    const KGrid g = kgrid_of(ctx->grid);
    const pms_params& P = ctx->prm;
    FieldParams fp;
    fp.h = P.h;
    fp.h_sq = P.h * P.h;
    const float inv = 1.f / P.h;
    fp.inv_h2 = inv * inv;
    fp.c_iso = kSigma * (inv * inv * inv);
    fp.thr = 2.f * P.iso_value;
    fp.grow = 1.0001f;
    const float ri = fp.grow * P.h;
    fp.r_iso2 = ri * ri;
    Counters* cnt = ctx->counters.as<Counters>();
    k_field<<<grid_for(ctx->nv, kThreads), kThreads, 0, ctx->stream>>>(
        g, fp, cnt, ctx->vlist.as<uint32_t>(), ctx->cell_info.as<uint2>(), ctx->cell_rad.as<float>(),
        ctx->spos.as<float4>(), ctx->aniso.as<float4>(), ctx->field.as<float>());
    PMS_LAUNCHED(ctx);
    return PMS_OK;
}

}  // namespace pms
