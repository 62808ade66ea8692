// k_common.cuh -- device helpers shared by the libpms kernels.
#pragma once
#include <cuda_runtime.h>
#include <cstdint>
#include "pms_internal.h"

namespace pms {

// Grid parameters passed to kernels by value (lives in the kernel's constant bank).
struct KGrid {
    float min_pos[3], scmin_pos[3];
    float sp_cs, sc_cs;
    uint32_t spres[3], scres[3];
    int32_t spexpand, scexpand, spexpand_diffuse;
    uint32_t sp_size, sc_size;
};

inline KGrid kgrid_of(const pms_grid& g) {
    KGrid k;
    for (int i = 0; i < 3; ++i) {
        k.min_pos[i] = g.min_pos[i];
        k.scmin_pos[i] = g.scmin_pos[i];
        k.spres[i] = g.spres[i];
        k.scres[i] = g.scres[i];
    }
    k.sp_cs = g.sp_grid_size;
    k.sc_cs = g.sc_grid_size;
    k.spexpand = g.spexpand;
    k.scexpand = g.scexpand;
    k.spexpand_diffuse = g.spexpand_diffuse;
    k.sp_size = g.sp_size;
    k.sc_size = g.sc_size;
    return k;
}

// float -> uint with the GPU's saturating conversion (cvt.rzi.u32.f32)
__device__ __forceinline__ uint32_t f2u(float x) { return __float2uint_rz(x); }

// Spatial cell of a position: uint((p - min) / cell) per axis, each operation
// rounded separately (getIndex3D, myCuda.cuh:55-59).
__device__ __forceinline__ uint3 sp_cell(const KGrid& g, float x, float y, float z) {
    return make_uint3(f2u(__fdiv_rn(__fsub_rn(x, g.min_pos[0]), g.sp_cs)),
                      f2u(__fdiv_rn(__fsub_rn(y, g.min_pos[1]), g.sp_cs)),
                      f2u(__fdiv_rn(__fsub_rn(z, g.min_pos[2]), g.sp_cs)));
}

__device__ __forceinline__ uint32_t lin3(uint32_t x, uint32_t y, uint32_t z, const uint32_t* res) {
    return z * res[0] * res[1] + y * res[0] + x;   // uint32 arithmetic as the reference
}

// Scalar-grid vertex position (float)i * cell + min, two roundings
// (getVertexPos, myCuda.cuh:121-131).
__device__ __forceinline__ float sc_coord(const KGrid& g, uint32_t i, int axis) {
    return __fadd_rn(__fmul_rn((float)i, g.sc_cs), g.scmin_pos[axis]);
}
__device__ __forceinline__ float sc_coord_i(const KGrid& g, int i, int axis) {
    return __fadd_rn(__fmul_rn((float)i, g.sc_cs), g.scmin_pos[axis]);
}

// [c - e, c + e] with uint wrap-around then clamp to [0, res-1]: the
// reference's neighbourhood bounds (Anisotropic_kernel.cuh:176-184).
__device__ __forceinline__ void box_clamp(const KGrid& g, uint3 c, uint32_t e, uint3& lo, uint3& hi) {
    lo.x = min(max(c.x - e, 0u), g.spres[0] - 1u);
    lo.y = min(max(c.y - e, 0u), g.spres[1] - 1u);
    lo.z = min(max(c.z - e, 0u), g.spres[2] - 1u);
    hi.x = min(max(c.x + e, 0u), g.spres[0] - 1u);
    hi.y = min(max(c.y + e, 0u), g.spres[1] - 1u);
    hi.z = min(max(c.z + e, 0u), g.spres[2] - 1u);
}

// Distance^2 from a point to the axis-aligned box of spatial cell index i along one axis
// (0 inside).  The box is widened by `pad` to cover rounding of the cell keys.
__device__ __forceinline__ float axis_gap(float p, float lo, float hi) {
    float d = fmaxf(lo - p, p - hi);
    return d > 0.f ? d : 0.f;
}

__device__ __forceinline__ uint32_t ordered_bits(float f) {
    uint32_t b = __float_as_uint(f);
    return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}
__device__ __forceinline__ float from_ordered_bits(uint32_t u) {
    uint32_t b = (u & 0x80000000u) ? (u & 0x7fffffffu) : ~u;
    return __uint_as_float(b);
}

// Squared distance from p to the box of spatial cell (x, y, z), the box widened
// by `pad` so particles whose key rounded into the cell from just outside are
// still covered.
__device__ __forceinline__ float cell_gap2(const KGrid& g, float3 p, uint32_t x, uint32_t y, uint32_t z, float pad) {
    const float x0 = g.min_pos[0] + (float)x * g.sp_cs - pad, x1 = x0 + g.sp_cs + 2.f * pad;
    const float y0 = g.min_pos[1] + (float)y * g.sp_cs - pad, y1 = y0 + g.sp_cs + 2.f * pad;
    const float z0 = g.min_pos[2] + (float)z * g.sp_cs - pad, z1 = z0 + g.sp_cs + 2.f * pad;
    const float dx = axis_gap(p.x, x0, x1), dy = axis_gap(p.y, y0, y1), dz = axis_gap(p.z, z0, z1);
    return dx * dx + dy * dy + dz * dz;
}

// Margin, in cells, added to every range that the neighbour walks cut from a
// support radius.  The ranges are computed from the point's position in cell
// units, u = (p - min) / cell, whose rounding error (like that of a particle's
// own key) stays below 1e-3 cells on grids of up to 8000 cells per axis; a cell
// left out by the cut therefore holds no particle within the support, and the
// cut changes no sum.
constexpr float kRangeMargin = 0.01f;

// Relative margin on support radii used for culling: a particle's kernel is
// non-zero only within its support (|G r| < 1 implies |r| < maxvalue * h), and
// float rounding of |G r|^2 moves that edge by ~1e-6 relative at most.
constexpr float kSupportGrow = 1.0001f;

// First and one-past-last cell of [u - rc, u + rc] along one axis, clipped to [lo, hi).
__device__ __forceinline__ void cell_range(float u, float rc, uint32_t lo, uint32_t hi, int& a, int& b) {
    a = max((int)floorf(u - rc), (int)lo);
    b = min((int)floorf(u + rc) + 1, (int)hi);
}

// Row-segment neighbour walk of one point.  Cells are sorted by key and key =
// (z * res_y + y) * res_x + x, so the cells x in [xa, xb) of one row hold the
// contiguous particle range [cell_start[row + xa], cell_start[row + xb]).  The
// walk visits only the slabs z and rows y of the window [lo, hi) (hi
// exclusive) that come within sqrt(r2) of p, each row cut to the cells the
// sphere reaches, and body(j) runs over the particle ranges in the reference's
// z, y, x, particle order.  cell_start must have sp_size + 1 entries.
template <class Body>
__device__ __forceinline__ void row_walk(const KGrid& g, float3 p, uint3 lo, uint3 hi, float r2, float pad,
                                         const uint32_t* __restrict__ cell_start, Body&& body) {
    const uint32_t srx = g.spres[0], srxy = g.spres[0] * g.spres[1];
    const float cs = g.sp_cs, inv = 1.f / g.sp_cs;
    const float ux = (p.x - g.min_pos[0]) * inv, uy = (p.y - g.min_pos[1]) * inv, uz = (p.z - g.min_pos[2]) * inv;
    int za, zb;
    cell_range(uz, sqrtf(r2) * inv + kRangeMargin, lo.z, hi.z, za, zb);
    for (int z = za; z < zb; ++z) {
        const float z0 = g.min_pos[2] + (float)z * cs;
        const float gz0 = axis_gap(p.z, z0 - pad, z0 + cs + pad);
        const float gz = gz0 * gz0;
        if (gz >= r2) continue;
        int ya, yb;
        cell_range(uy, sqrtf(r2 - gz) * inv + kRangeMargin, lo.y, hi.y, ya, yb);
        for (int y = ya; y < yb; ++y) {
            const float y0 = g.min_pos[1] + (float)y * cs;
            const float gy0 = axis_gap(p.y, y0 - pad, y0 + cs + pad);
            const float gyz = gz + gy0 * gy0;
            if (gyz >= r2) continue;
            int xa, xb;
            cell_range(ux, sqrtf(r2 - gyz) * inv + kRangeMargin, lo.x, hi.x, xa, xb);
            if (xa >= xb) continue;
            const uint32_t row = (uint32_t)z * srxy + (uint32_t)y * srx;
            const uint32_t ja = __ldg(&cell_start[row + (uint32_t)xa]), jb = __ldg(&cell_start[row + (uint32_t)xb]);
#pragma unroll 2
            for (uint32_t j = ja; j < jb; ++j) body(j);
        }
    }
}

// rank of bit `id` among set bits of a bitmap with exclusive word prefix sums
__device__ __forceinline__ uint32_t bit_rank(const uint32_t* bm, const uint32_t* wprefix, uint32_t id) {
    uint32_t w = id >> 5, b = id & 31u;
    return wprefix[w] + __popc(bm[w] & ((1u << b) - 1u));
}
__device__ __forceinline__ bool bit_get(const uint32_t* bm, uint64_t nbits, uint64_t id) {
    return id < nbits && ((bm[id >> 5] >> (id & 31u)) & 1u);
}

}  // namespace pms
