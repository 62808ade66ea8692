// k_aniso.cu -- density of every particle and the anisotropy of every surface
// particle (weighted mean, covariance, eigen decomposition, eigenvalue clamp,
// G matrix, oriented normal, thin-feature flag).
//
// Reference: Anisotropic_kernel.cuh:158-213 (calculationOfDensity),
// 216-281 (calculationOfSmoothed), 350-519 (calculationOfTransformMatrices),
// myCuda.cuh:84-119, 193-203, 403-415 (wij, matrixMul, determinant,
// wij_density), SVD3.cuh (a float32 3x3 SVD).
//
// GB300 design: one thread per particle walks the sorted cells around it;
// cells whose box lies beyond the kernel support are skipped (their
// contributions are exactly zero), so the (4e+1)^3 box shrinks to the cells
// that can matter.  The covariance is symmetric positive definite (it is seeded
// with h^2 I), so its SVD is its eigen decomposition: a cyclic Jacobi solver
// with exact rotations runs in float32, and covariances whose condition
// number exceeds cfg.fp64_svd_cond are re-solved in float64.  Sums are
// accumulated relative to the particle's own position for accuracy.
#include <cmath>

#include "pms_internal.h"
#include "k_common.cuh"

namespace pms {

static constexpr int kThreads = 128;
static constexpr float kSigma = 1.56668147f;      // Define.h:11, 315/(64 pi)

struct AnisoParams {
    float h, h_sq, h_inv, r2h, mass, kdens, inv_h2;
    float nn_d2;     // |u| <= h      <=>  |u|^2 <= nn_d2  (|u| = sqrt of |u|^2, rounded)
    float w_d2;      // |u| < 2h      <=>  |u|^2 <= w_d2
    int min_nn;
    uint32_t sp_size, spres_x;   // where the per-row radii start; cells per row
    double cond_limit;
};

// ---------------------------------------------------------------------------
// density (calculationOfDensity): rho_i = sum_j sigma/h^3 (1 - (d/h)^2)^3, d < h,
// over cells [c - e, c + e]; also stores m / rho into spos.w for the field.
// ---------------------------------------------------------------------------
template <int BT>
__global__ void __launch_bounds__(BT, 1024 / BT) k_density(KGrid g, AnisoParams ap, const uint32_t* __restrict__ skeys,
                                                      const uint32_t* __restrict__ cell_start, float4* __restrict__ spos,
                                                      float* __restrict__ rho, uint32_t n) {
    const uint32_t rx = g.spres[0], rxy = g.spres[0] * g.spres[1];
    const float pad = 1e-4f * g.sp_cs;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float4 pi4 = spos[i];
        const float3 p = make_float3(pi4.x, pi4.y, pi4.z);
        const uint32_t key = skeys[i];
        const uint3 c = make_uint3(key % rx, (key / rx) % g.spres[1], key / rxy);
        uint3 lo, hi;
        box_clamp(g, c, (uint32_t)g.spexpand, lo, hi);
        hi = make_uint3(hi.x + 1, hi.y + 1, hi.z + 1);
        // sum of max(1 - d^2/h^2, 0)^3, times sigma / h^3 once at the end
        float w = 0.f;
        row_walk(g, p, lo, hi, ap.h_sq, pad, cell_start, [&](uint32_t j) {
            const float4 q = __ldg(&spos[j]);
            const float dx = p.x - q.x, dy = p.y - q.y, dz = p.z - q.z;
            const float d2 = dx * dx + dy * dy + dz * dz;
            const float s = fmaxf(fmaf(-d2, ap.inv_h2, 1.f), 0.f);   // 0 beyond h: adds nothing
            w = fmaf(s * s, s, w);
        });
        rho[i] = ap.kdens * w;
    }
}

// m / rho into spos.w (0 for rho == 0: the field skips such particles), and the
// isotropic kernel of every particle in the field's packed form: M = G^T G
// with G = I / h (off-diagonals doubled), h_s^2 = h^2, and the weight
// (m / rho) sigma det(G) = (m / rho) sigma / h^3; the anisotropy pass
// overwrites the surface particles' entries.
__global__ void __launch_bounds__(kThreads) k_inv_density(float4* __restrict__ spos, const float* __restrict__ rho,
                                                          float4* __restrict__ aniso, AnisoParams ap, uint32_t n) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float r = rho[i];
        spos[i].w = r == 0.f ? 0.f : ap.mass / r;
        const float inv_h2 = ap.h_inv * ap.h_inv;
        aniso[2 * (size_t)i + 0] = make_float4(inv_h2, 0.f, 0.f, ap.h_sq);
        aniso[2 * (size_t)i + 1] = make_float4(inv_h2, 0.f, inv_h2, spos[i].w * ap.kdens);
    }
}

// ---------------------------------------------------------------------------
// symmetric 3x3 eigen decomposition, cyclic Jacobi with exact rotations
// (Golub & Van Loan, Algorithm 8.4.2 / the classical Jacobi method)
// ---------------------------------------------------------------------------
template <class T>
__device__ __forceinline__ void jacobi_rotate(T a[3][3], T v[3][3], int p, int q) {
    T apq = a[p][q];
    if (apq == T(0)) return;
    T theta = (a[q][q] - a[p][p]) / (T(2) * apq);
    T t = (theta >= T(0) ? T(1) : T(-1)) / (fabs(theta) + sqrt(theta * theta + T(1)));
    T c = T(1) / sqrt(t * t + T(1)), s = t * c;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        T akp = a[k][p], akq = a[k][q];
        a[k][p] = c * akp - s * akq;
        a[k][q] = s * akp + c * akq;
    }
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        T apk = a[p][k], aqk = a[q][k];
        a[p][k] = c * apk - s * aqk;
        a[q][k] = s * apk + c * aqk;
    }
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        T vkp = v[k][p], vkq = v[k][q];
        v[k][p] = c * vkp - s * vkq;
        v[k][q] = s * vkp + c * vkq;
    }
}

// On return e[0..2] are eigenvalues sorted by decreasing magnitude and
// column k of v the matching unit eigenvector.
template <class T>
__device__ __forceinline__ void eig_sym3(T a[3][3], T e[3], T v[3][3], T tol) {
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) v[i][j] = (i == j) ? T(1) : T(0);
    for (int sweep = 0; sweep < 12; ++sweep) {
        T off = fabs(a[0][1]) + fabs(a[0][2]) + fabs(a[1][2]);
        T dia = fabs(a[0][0]) + fabs(a[1][1]) + fabs(a[2][2]);
        if (off <= tol * dia) break;
        jacobi_rotate<T>(a, v, 0, 1);
        jacobi_rotate<T>(a, v, 0, 2);
        jacobi_rotate<T>(a, v, 1, 2);
    }
    T d[3] = {a[0][0], a[1][1], a[2][2]};
    int i0 = 0, i1 = 1, i2 = 2;
    if (fabs(d[i1]) > fabs(d[i0])) { int t = i0; i0 = i1; i1 = t; }
    if (fabs(d[i2]) > fabs(d[i0])) { int t = i0; i0 = i2; i2 = t; }
    if (fabs(d[i2]) > fabs(d[i1])) { int t = i1; i1 = i2; i2 = t; }
    int idx[3] = {i0, i1, i2};
    T w[3][3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        e[k] = d[idx[k]];
#pragma unroll
        for (int r = 0; r < 3; ++r) w[r][k] = v[r][idx[k]];
    }
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
        for (int k = 0; k < 3; ++k) v[r][k] = w[r][k];
}

// ---------------------------------------------------------------------------
// anisotropy, pass 1: weighted moments of the neighbourhood, one surface
// particle per thread, ONE walk over the cells.  With u = x_j - x_i and
// w = 1 - (|u| / 2h)^3 (wij with support 2h):
//   S0 = sum w, S1 = sum w u, S2 = sum w u u^T, J = #{|u| <= h}.
// The reference's two passes (mean, then covariance about the mean) follow
// from these: mean = x_i + S1/S0 and sum w (u - o)(u - o)^T = S2 - S1 S1^T / S0.
// The count and the support test compare |u|^2 with the exact bounds of the
// rounded square root (the same decisions as comparing |u|); the weight uses
// the hardware reciprocal square root (a few ulp, inside the weight's rounding).
// ---------------------------------------------------------------------------
template <int BT>
__global__ void __launch_bounds__(BT, 1024 / BT) k_moments(KGrid g, AnisoParams ap, const uint32_t* __restrict__ slist,
                                                      const Counters* __restrict__ cnt, const uint32_t* __restrict__ skeys,
                                                      const uint32_t* __restrict__ cell_start, const float4* __restrict__ spos,
                                                      float4* __restrict__ mom) {
    const uint32_t ns = cnt->ns;
    const uint32_t rx = g.spres[0], rxy = g.spres[0] * g.spres[1];
    const float pad = 1e-4f * g.sp_cs;
    const float r2h_sq = ap.r2h * ap.r2h;
    const float inv_r2h = 1.f / ap.r2h;
    for (uint32_t s = blockIdx.x * blockDim.x + threadIdx.x; s < ns; s += gridDim.x * blockDim.x) {
        const uint32_t i = slist[s];
        const float4 pi4 = spos[i];
        const float3 p = make_float3(pi4.x, pi4.y, pi4.z);
        const uint32_t key = skeys[i];
        const uint3 c = make_uint3(key % rx, (key / rx) % g.spres[1], key / rxy);
        uint3 lo, hi;
        box_clamp(g, c, 2u * (uint32_t)g.spexpand, lo, hi);
        hi = make_uint3(hi.x + 1, hi.y + 1, hi.z + 1);
        float s0 = 0.f, sx = 0.f, sy = 0.f, sz = 0.f;
        float sxx = 0.f, sxy = 0.f, sxz = 0.f, syy = 0.f, syz = 0.f, szz = 0.f;
        uint32_t nn = 0;
        row_walk(g, p, lo, hi, r2h_sq, pad, cell_start, [&](uint32_t j) {
            const float4 q = __ldg(&spos[j]);
            // |u| rounded operation by operation, as the reference's neighbour count sees it
            const float ux = __fsub_rn(q.x, p.x), uy = __fsub_rn(q.y, p.y), uz = __fsub_rn(q.z, p.z);
            const float d2 = __fadd_rn(__fadd_rn(__fmul_rn(ux, ux), __fmul_rn(uy, uy)), __fmul_rn(uz, uz));
            nn += (d2 <= ap.nn_d2) ? 1u : 0u;
            const float t = d2 * rsqrtf(d2) * inv_r2h;               // d2 = 0 gives NaN, selected away
            const float w = (d2 <= ap.w_d2 && d2 > 0.f) ? 1.f - t * t * t : (d2 > 0.f ? 0.f : 1.f);
            const float wx = w * ux, wy = w * uy, wz = w * uz;
            s0 += w; sx += wx; sy += wy; sz += wz;
            sxx += wx * ux; sxy += wx * uy; sxz += wx * uz;
            syy += wy * uy; syz += wy * uz; szz += wz * uz;
        });
        mom[3 * (size_t)s + 0] = make_float4(s0, sx, sy, sz);
        mom[3 * (size_t)s + 1] = make_float4(sxx, sxy, sxz, syy);
        mom[3 * (size_t)s + 2] = make_float4(syz, szz, __uint_as_float(nn), 0.f);
    }
}

// ---------------------------------------------------------------------------
// anisotropy, pass 2: covariance, eigen decomposition, clamp, G, normal, flag
// (Anisotropic_kernel.cuh:431-518) from the moments; also the per-cell
// and per-row support radius max(maxvalue * h) that lets the field skip far
// rows and cells.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kThreads) k_eigen(AnisoParams ap, const uint32_t* __restrict__ slist,
                                                    const Counters* __restrict__ cnt, const uint32_t* __restrict__ skeys,
                                                    const float4* __restrict__ spos, const float4* __restrict__ mom,
                                                    float4* __restrict__ aniso, float4* __restrict__ nrm4,
                                                    float4* __restrict__ mean4, float* __restrict__ gdebug,
                                                    uint32_t* __restrict__ nnb, float* __restrict__ cell_rad,
                                                    Counters* __restrict__ cnt_w) {
    const uint32_t ns = cnt->ns;
    for (uint32_t s = blockIdx.x * blockDim.x + threadIdx.x; s < ns; s += gridDim.x * blockDim.x) {
        const uint32_t i = slist[s];
        const float4 pi4 = spos[i];
        const float4 m0 = mom[3 * (size_t)s + 0], m1 = mom[3 * (size_t)s + 1], m2 = mom[3 * (size_t)s + 2];
        const float ws = m0.x;                               // >= 1: the particle itself
        const float ox = m0.y / ws, oy = m0.z / ws, oz = m0.w / ws;   // mean - p
        const uint32_t nn = __float_as_uint(m2.z);
        float G[3][3], nv[3], maxv, flag;
        if ((int)nn < ap.min_nn) {
            // isolated particle: isotropic kernel (Anisotropic_kernel.cuh:435-443)
#pragma unroll
            for (int a = 0; a < 3; ++a)
#pragma unroll
                for (int b = 0; b < 3; ++b) G[a][b] = (a == b) ? ap.h_inv : 0.f;
            maxv = 1.f; flag = 1.f; nv[0] = 1.f; nv[1] = 0.f; nv[2] = 0.f;
        } else {
            // (h^2 I + S2 - S1 S1^T / S0) / S0
            const float inv = 1.f / ws;
            const float c00 = (ap.h_sq + (m1.x - m0.y * ox)) * inv, c01 = (m1.y - m0.y * oy) * inv;
            const float c02 = (m1.z - m0.y * oz) * inv, c11 = (ap.h_sq + (m1.w - m0.z * oy)) * inv;
            const float c12 = (m2.x - m0.z * oz) * inv, c22 = (ap.h_sq + (m2.y - m0.w * oz)) * inv;
            float A[3][3] = {{c00, c01, c02}, {c01, c11, c12}, {c02, c12, c22}};
            float e[3], U[3][3];
            eig_sym3<float>(A, e, U, 1e-7f);
            float sv0 = fabsf(e[0]), sv1 = fabsf(e[1]), sv2 = fabsf(e[2]);
            if ((double)sv0 > ap.cond_limit * (double)sv2) {
                // ill-conditioned covariance: solve again in float64
                double Ad[3][3] = {{c00, c01, c02}, {c01, c11, c12}, {c02, c12, c22}};
                double ed[3], Ud[3][3];
                eig_sym3<double>(Ad, ed, Ud, 1e-15);
#pragma unroll
                for (int k = 0; k < 3; ++k) {
                    e[k] = (float)ed[k];
#pragma unroll
                    for (int r = 0; r < 3; ++r) U[r][k] = (float)Ud[r][k];
                }
                sv0 = fabsf(e[0]); sv1 = fabsf(e[1]); sv2 = fabsf(e[2]);
                atomicAdd(&cnt_w->n_fp64, 1u);
            }
            // clamp and scale (Anisotropic_kernel.cuh:459-509)
            const float smax = fmaxf(sv0, fmaxf(sv1, sv2)), smin = fminf(sv0, fminf(sv1, sv2));
            flag = (smin <= smax * 0.25f) ? 1.f : 0.f;
            const float lim = smax / 4.0f;
            sv0 = fmaxf(sv0, lim); sv1 = fmaxf(sv1, lim); sv2 = fmaxf(sv2, lim);
            const float scale = cbrtf(sv0 * sv1 * sv2);
            const float cof = ap.h_inv * scale;
            const float k0 = cof / sv0, k1 = cof / sv1, k2 = cof / sv2;
#pragma unroll
            for (int a = 0; a < 3; ++a)
#pragma unroll
                for (int b = 0; b < 3; ++b)
                    G[a][b] = U[a][0] * k0 * U[b][0] + U[a][1] * k1 * U[b][1] + U[a][2] * k2 * U[b][2];
            nv[0] = U[0][2]; nv[1] = U[1][2]; nv[2] = U[2][2];
            maxv = sv0 / scale;
        }
        // orient the normal away from the mean (Anisotropic_kernel.cuh:512-515)
        if (nv[0] * (-ox) + nv[1] * (-oy) + nv[2] * (-oz) < 0.f) { nv[0] = -nv[0]; nv[1] = -nv[1]; nv[2] = -nv[2]; }
        // determinant as the reference evaluates it (myCuda.cuh:193-203)
        const float det = G[0][0] * G[1][1] * G[2][2] + G[0][1] * G[1][2] * G[2][0] + G[0][2] * G[1][0] * G[2][1]
                        - G[0][0] * G[1][2] * G[2][1] - G[0][1] * G[1][0] * G[2][2] - G[0][2] * G[1][1] * G[2][0];
        const float hs = maxv * ap.h;
        // symmetric G packed in two float4: {g00, g01, g02, hs^2}, {g11, g12, g22, sigma * det}
        // the field's packed form: M = G^T G = G G (G is symmetric), off-diagonals doubled,
        // so |G r|^2 = r^T M r costs 9 multiply-adds; w = (m / rho) sigma det(G)
        float M[3][3];
#pragma unroll
        for (int a = 0; a < 3; ++a)
#pragma unroll
            for (int b = 0; b < 3; ++b) M[a][b] = G[a][0] * G[0][b] + G[a][1] * G[1][b] + G[a][2] * G[2][b];
        aniso[2 * (size_t)i + 0] = make_float4(M[0][0], 2.f * M[0][1], 2.f * M[0][2], hs * hs);
        aniso[2 * (size_t)i + 1] = make_float4(M[1][1], 2.f * M[1][2], M[2][2], pi4.w * (kSigma * det));
        nrm4[i] = make_float4(nv[0], nv[1], nv[2], flag);
        mean4[s] = make_float4(pi4.x + ox, pi4.y + oy, pi4.z + oz, ws);
        float* gd = gdebug + 10 * (size_t)s;
#pragma unroll
        for (int a = 0; a < 3; ++a)
#pragma unroll
            for (int b = 0; b < 3; ++b) gd[3 * a + b] = G[a][b];
        gd[9] = maxv;
        nnb[s] = nn;
        // per-cell, per-row and global support radius (positive floats order like their bits)
        const uint32_t key = skeys[i];
        atomicMax(reinterpret_cast<unsigned int*>(&cell_rad[key]), __float_as_uint(hs));
        atomicMax(reinterpret_cast<unsigned int*>(&cell_rad[ap.sp_size + key / ap.spres_x]), __float_as_uint(hs));
        atomicMax(&cnt_w->rad_max_bits, __float_as_uint(hs));
    }
}

// ---------------------------------------------------------------------------
// per-cell culling record for the field: the bounding box of the cell's
// particles and the square of the largest support among them (h, or the
// cell's largest maxvalue * h), grown by kSupportGrow.  A vertex farther than
// that from the box gets exactly 0 from every particle of the cell.  An empty
// cell gets r^2 = -1, which no vertex reaches.
// rec[2c] = {min x, min y, min z, r^2}, rec[2c + 1] = {max x, max y, max z, 0}.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kThreads) k_cell_records(const uint32_t* __restrict__ cell_start,
                                                           const float4* __restrict__ spos,
                                                           const float* __restrict__ cell_rad, float h, uint32_t S,
                                                           float4* __restrict__ rec) {
    for (uint32_t c = blockIdx.x * blockDim.x + threadIdx.x; c < S; c += gridDim.x * blockDim.x) {
        const uint32_t j0 = cell_start[c], j1 = cell_start[c + 1];
        if (j0 == j1) {
            rec[2 * (size_t)c] = make_float4(0.f, 0.f, 0.f, -1.f);
            continue;
        }
        const float4 q = spos[j0];
        float lx = q.x, ly = q.y, lz = q.z, hx = q.x, hy = q.y, hz = q.z;
        for (uint32_t j = j0 + 1; j < j1; ++j) {
            const float4 p = spos[j];
            lx = fminf(lx, p.x); ly = fminf(ly, p.y); lz = fminf(lz, p.z);
            hx = fmaxf(hx, p.x); hy = fmaxf(hy, p.y); hz = fmaxf(hz, p.z);
        }
        const float r = fmaxf(cell_rad[c], h) * kSupportGrow;
        rec[2 * (size_t)c] = make_float4(lx, ly, lz, r * r);
        rec[2 * (size_t)c + 1] = make_float4(hx, hy, hz, 0.f);
    }
}

// Largest float x >= 0 with sqrt(x) <= r (inclusive) or sqrt(x) < r (strict),
// sqrt correctly rounded: the rounded square root is non-decreasing, so
// sqrt(x) <= r exactly when x <= that bound.
static float sqrt_bound(float r, bool inclusive) {
    auto ok = [&](float x) { const float s = std::sqrt(x); return inclusive ? s <= r : s < r; };
    float x = r * r;
    while (x > 0.f && !ok(x)) x = std::nextafter(x, 0.f);
    while (ok(std::nextafter(x, INFINITY))) x = std::nextafter(x, INFINITY);
    return x;
}

pms_status launch_density_aniso(pms_ctx* ctx) {
    const KGrid g = kgrid_of(ctx->grid);
    const pms_params& P = ctx->prm;
    AnisoParams ap;
    ap.h = P.h; ap.h_sq = P.h_sq; ap.h_inv = P.h_inv; ap.r2h = P.aniso_radius; ap.mass = P.mass;
    ap.kdens = kSigma / (P.h * P.h * P.h);
    ap.inv_h2 = 1.f / (P.h * P.h);
    ap.min_nn = P.min_num_neighbors;
    ap.cond_limit = ctx->cfg.fp64_svd_cond;
    ap.nn_d2 = sqrt_bound(P.h, true);
    ap.w_d2 = sqrt_bound(P.aniso_radius, false);
    ap.sp_size = g.sp_size;
    ap.spres_x = g.spres[0];
    Counters* cnt = ctx->counters.as<Counters>();
    // block sizes of the neighbour walks are autotuned (64, 128 or 256 threads)
    const int bd = ctx->tune.density_threads, bm = ctx->tune.moments_threads;
    auto dens = [&](auto kern) {
        kern<<<grid_for(ctx->n, (unsigned)bd), bd, 0, ctx->stream>>>(g, ap, ctx->skeys.as<uint32_t>(),
                                                                    ctx->cell_start.as<uint32_t>(), ctx->spos.as<float4>(),
                                                                    ctx->rho.as<float>(), ctx->n);
    };
    if (bd == 64) dens(k_density<64>);
    else if (bd == 256) dens(k_density<256>);
    else dens(k_density<128>);
    PMS_LAUNCHED(ctx);
    k_inv_density<<<grid_for(ctx->n, kThreads), kThreads, 0, ctx->stream>>>(ctx->spos.as<float4>(), ctx->rho.as<float>(),
                                                                           ctx->aniso.as<float4>(), ap, ctx->n);
    PMS_LAUNCHED(ctx);
    // ns is on the device; grids are sized by the particle count (an upper bound)
    auto mom = [&](auto kern) {
        kern<<<grid_for(ctx->n, (unsigned)bm), bm, 0, ctx->stream>>>(g, ap, ctx->slist.as<uint32_t>(), cnt,
                                                                    ctx->skeys.as<uint32_t>(), ctx->cell_start.as<uint32_t>(),
                                                                    ctx->spos.as<float4>(), ctx->moments.as<float4>());
    };
    if (bm == 64) mom(k_moments<64>);
    else if (bm == 256) mom(k_moments<256>);
    else mom(k_moments<128>);
    PMS_LAUNCHED(ctx);
    PMS_CUDA(ctx, cudaMemsetAsync(ctx->cell_rad.p, 0,
                                  sizeof(float) * ((size_t)g.sp_size + (size_t)g.spres[1] * g.spres[2]), ctx->stream));
    k_eigen<<<grid_for(ctx->n, kThreads), kThreads, 0, ctx->stream>>>(
        ap, ctx->slist.as<uint32_t>(), cnt, ctx->skeys.as<uint32_t>(), ctx->spos.as<float4>(), ctx->moments.as<float4>(),
        ctx->aniso.as<float4>(), ctx->nrm4.as<float4>(), ctx->mean4.as<float4>(), ctx->gdebug.as<float>(),
        ctx->nnb.as<uint32_t>(), ctx->cell_rad.as<float>(), cnt);
    PMS_LAUNCHED(ctx);
    k_cell_records<<<grid_for(g.sp_size, kThreads), kThreads, 0, ctx->stream>>>(
        ctx->cell_start.as<uint32_t>(), ctx->spos.as<float4>(), ctx->cell_rad.as<float>(), P.h, g.sp_size,
        ctx->cell_rec.as<float4>());
    PMS_LAUNCHED(ctx);
    return PMS_OK;
}

}  // namespace pms
