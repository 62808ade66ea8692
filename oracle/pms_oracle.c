/*
 * pms_oracle.c -- CPU oracle for the particle-to-surface pipeline.
 *
 * TEST INFRASTRUCTURE ONLY (see pms_oracle.h).  Restates, loop for loop, the
 * reference's surface-reconstruction path:
 *   Params.cpp:24-152                parameter derivation
 *   FileData.cpp:239-283             per-frame bounding box and grid
 *   NeighborSearch_kernel.cuh:53-186 cell keys and cell ranges
 *   Thrust.cuh:40-50                 stable sort by key
 *   Anisotropic_kernel.cuh:15-777    surface cells, density, mean, covariance,
 *                                    G matrices, band vertices, scalar field
 *   myCuda.cuh:49-415                kernels W and helpers
 *   MarchingCube_kernel.cuh:20-157   marching-cubes classify and emit
 *
 * Compile with -ffp-contract=off: the float32 expressions that feed integer
 * decisions (cell keys, grid sizes, band tests, iso comparisons) must round
 * exactly like the reference's separate float32 operations.
 */
#include "pms_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <float.h>

#define ORC_SIGMA 1.56668147f          /* Define.h:11 */
#define ORC_EPS   1.0e-7               /* Define.h:10 (double literal) */

static inline uint32_t clampu(uint32_t v, uint32_t lo, uint32_t hi) { return v < lo ? lo : (v > hi ? hi : v); }
static inline int32_t clampi(int32_t v, int32_t lo, int32_t hi) { return v < lo ? lo : (v > hi ? hi : v); }

/* float -> uint conversion as the GPU does it (saturating); positions are
 * always inside the padded grid so the saturation never triggers.           */
static inline uint32_t f2u(float x) {
    if (!(x > 0.0f)) return 0u;
    if (x >= 4294967296.0f) return 0xffffffffu;
    return (uint32_t)x;
}

/* ------------------------------------------------------------------------ */
/* Params.cpp:53-118                                                         */
/* ------------------------------------------------------------------------ */
void orc_derive_params(const orc_config* c, orc_params* p)
{
    memset(p, 0, sizeof(*p));
    p->mass = (float)c->mass;
    p->particle_spacing = (float)c->particle_spacing;
    p->smoothing_radius_ratio = (int)c->smoothing_radius_ratio;
    /* int * float */
    p->h = (float)p->smoothing_radius_ratio * p->particle_spacing;
    p->h_inv = (float)(1.0 / (double)p->h);
    p->h_sq = p->h * p->h;
    p->aniso_radius = p->h * 2.0f;
    p->min_num_neighbors = (int)c->min_num_neighbors;
    p->isolate_num_neighbors = (int)c->isolate_num_neighbors;
    p->lambda_for_smoothed = (float)c->lambda_for_smoothed;
    p->iso_value = (float)c->iso_value;

    /* Params.cpp:75-99 */
    p->hd = (float)(1.732 * (double)p->particle_spacing);
    p->hd_inv = (float)(1.0 / (double)p->hd);
    p->hd_sq = p->hd * p->hd;
    p->hd_aniso = p->hd * 2.0f;
    {
        /* (4 / 3) is integer 1 in the reference; evaluation is float32 left to right */
        const float PI_F = 3.14159265f;
        float half = p->particle_spacing / 2.0f;
        float a = 1.0f * PI_F;
        a = a * powf(half, 3.0f);
        a = a * 315.0f;
        float b = 64.0f * PI_F;
        b = b * powf(p->hd, 9.0f);
        p->coefficient = a / b;
    }
    p->d_min_num_neighbors = (int)(signed char)c->min_num_neighbors;
    p->min_wc = (float)c->min_wave_crests;  p->max_wc = (float)c->max_wave_crests;
    p->min_ta = (float)c->min_trapped_air;  p->max_ta = (float)c->max_trapped_air;
    p->min_ke = (float)c->min_kinetic_energy; p->max_ke = (float)c->max_kinetic_energy;
    p->ta_mult = (int)c->trapped_air_multiplier;
    p->wc_mult = (int)c->wave_crests_multiplier;
    p->time_step = (float)c->time_step;
    p->life_time = (int)c->life_time;
    p->buoyancy = (float)c->buoyancy_control;
    p->drag = (float)c->drag_control;

    /* Params.cpp:105-118 */
    p->sp_scale = (int)c->sp_scale;
    p->sc_scale = (int)c->sc_scale;
    p->sp_grid_size = (float)((double)p->particle_spacing * 1.5);
    p->sc_grid_size = p->particle_spacing / (float)p->sc_scale;
    p->spexpand = (int)ceilf(p->h / p->sp_grid_size);
    p->scexpand = (int)ceilf(p->h / p->sc_grid_size);
    p->spexpand_diffuse = (int)ceilf(p->hd / p->sp_grid_size);
}

/* FileData.cpp:240-257 */
void orc_bbox(const float* pos, uint32_t n, float bmin[3], float bmax[3])
{
    for (int k = 0; k < 3; ++k) { bmin[k] = pos[k]; bmax[k] = pos[k]; }
    for (uint32_t i = 1; i < n; ++i) {
        for (int k = 0; k < 3; ++k) {
            float v = pos[3 * (size_t)i + k];
            if (bmax[k] <= v) bmax[k] = v;
            if (bmin[k] >= v) bmin[k] = v;
        }
    }
}

/* FileData.cpp:259-279 (NOBOUND path), float32 arithmetic, "+ 0.5" in double */
void orc_grid_from_bbox(const orc_params* p, const float bmin[3], const float bmax[3], orc_grid* g)
{
    memset(g, 0, sizeof(*g));
    float two_h = 2.0f * p->h, four_h = 4.0f * p->h;
    for (int k = 0; k < 3; ++k) {
        g->scmin_pos[k] = bmin[k] - two_h;
        g->scmax_pos[k] = bmax[k] + two_h;
        g->min_pos[k] = bmin[k] - four_h;
        g->max_pos[k] = bmax[k] + four_h;
    }
    g->sp_grid_size = p->sp_grid_size;
    g->sc_grid_size = p->sc_grid_size;
    for (int k = 0; k < 3; ++k) {
        float sp = (g->max_pos[k] - g->min_pos[k]) / g->sp_grid_size;
        g->spres[k] = f2u(sp);
        float sc = (g->scmax_pos[k] - g->scmin_pos[k]) / g->sc_grid_size;
        double scd = (double)sc + 0.5;
        g->scres[k] = (uint32_t)scd;
    }
    g->spexpand = p->spexpand;
    g->scexpand = p->scexpand;
    g->spexpand_diffuse = p->spexpand_diffuse;
    g->sp_size = g->spres[0] * g->spres[1] * g->spres[2];
    g->sc_size = g->scres[0] * g->scres[1] * g->scres[2];
}

/* ------------------------------------------------------------------------ */
/* NeighborSearch_kernel.cuh:129-152  getIndex3D myCuda.cuh:55-59           */
/* ------------------------------------------------------------------------ */
static inline void cell_of(const orc_grid* g, const float* p, uint32_t c[3])
{
    for (int k = 0; k < 3; ++k) c[k] = f2u((p[k] - g->min_pos[k]) / g->sp_grid_size);
}
static inline uint32_t lin3(uint32_t x, uint32_t y, uint32_t z, const uint32_t res[3])
{
    return z * res[0] * res[1] + y * res[0] + x;   /* uint32 wrap like the reference */
}

void orc_hash(const orc_grid* g, const float* pos, uint32_t n, uint32_t* keys)
{
    #pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < (int64_t)n; ++i) {
        uint32_t c[3];
        cell_of(g, pos + 3 * i, c);
        keys[i] = lin3(c[0], c[1], c[2], g->spres);
    }
}

/* Thrust.cuh:40-50: thrust::sort_by_key on uint keys is a stable radix sort.
 * Restated as a stable counting sort over [0, nkeys). */
void orc_stable_sort(const uint32_t* keys, uint32_t n, uint32_t nkeys, uint32_t* perm)
{
    uint32_t* cnt = (uint32_t*)calloc((size_t)nkeys + 1, sizeof(uint32_t));
    for (uint32_t i = 0; i < n; ++i) cnt[keys[i] + 1]++;
    for (uint32_t k = 0; k < nkeys; ++k) cnt[k + 1] += cnt[k];
    for (uint32_t i = 0; i < n; ++i) perm[cnt[keys[i]]++] = i;
    free(cnt);
}

/* NeighborSearch_kernel.cuh:154-186; cells without particles keep {0,0}
 * (GPUmemory.cpp:61 memsets dIndexRange). */
void orc_cell_ranges(const uint32_t* sk, uint32_t n, uint32_t nkeys, uint32_t* start, uint32_t* end)
{
    memset(start, 0, sizeof(uint32_t) * nkeys);
    memset(end, 0, sizeof(uint32_t) * nkeys);
    for (uint32_t i = 0; i < n; ++i) {
        uint32_t h = sk[i];
        if (i == 0 || h != sk[i - 1]) {
            start[h] = i;
            if (i > 0) end[sk[i - 1]] = i;
        }
        if (i == n - 1) end[h] = i + 1;
    }
}

/* ------------------------------------------------------------------------ */
/* Anisotropic_kernel.cuh:15-106 (uint wrap-then-clamp neighbourhood)        */
/* ------------------------------------------------------------------------ */
void orc_surface_cells(const orc_grid* g, const uint32_t* start, const uint32_t* end, uint32_t* surf_count)
{
    const uint32_t rx = g->spres[0], ry = g->spres[1], rz = g->spres[2];
    const uint32_t S = g->sp_size;
    #pragma omp parallel for schedule(static)
    for (int64_t t = 0; t < (int64_t)S; ++t) {
        uint32_t id = (uint32_t)t;
        surf_count[id] = 0;
        if (end[id] - start[id] == 0) continue;     /* spatialGrid.fluid */
        uint32_t z = id / (rx * ry), m = id % (rx * ry), y = m / rx, x = m % rx;
        uint32_t lo[3] = {x - 1u, y - 1u, z - 1u}, hi[3] = {x + 1u, y + 1u, z + 1u};
        uint32_t res[3] = {rx, ry, rz};
        for (int k = 0; k < 3; ++k) { lo[k] = clampu(lo[k], 0, res[k] - 1); hi[k] = clampu(hi[k], 0, res[k] - 1); }
        int surface = 0;
        for (uint32_t cz = lo[2]; cz <= hi[2]; ++cz)
            for (uint32_t cy = lo[1]; cy <= hi[1]; ++cy)
                for (uint32_t cx = lo[0]; cx <= hi[0]; ++cx) {
                    uint32_t q = lin3(cx, cy, cz, res);
                    if (end[q] - start[q] == 0) { surface = 1; break; }
                }
        if (surface) surf_count[id] = end[id] - start[id];
    }
}

uint64_t orc_exclusive_scan_u32(const uint32_t* in, uint64_t n, uint32_t* out)
{
    uint64_t acc = 0;
    for (uint64_t i = 0; i < n; ++i) { out[i] = (uint32_t)acc; acc += in[i]; }
    return acc;
}

/* Anisotropic_kernel.cuh:127-155 */
void orc_surface_list(const orc_grid* g, const uint32_t* surf_count, const uint32_t* surf_scan,
                      const uint32_t* start, uint32_t* list)
{
    for (uint32_t c = 0; c < g->sp_size; ++c) {
        if (surf_count[c] > 0) {
            for (uint32_t i = 0; i < surf_count[c]; ++i) list[surf_scan[c] + i] = start[c] + i;
        }
    }
}

/* ------------------------------------------------------------------------ */
/* neighbourhood [c-e, c+e] (inclusive) with uint wrap-then-clamp            */
/* ------------------------------------------------------------------------ */
static inline void box_incl(const orc_grid* g, const uint32_t c[3], uint32_t e, uint32_t lo[3], uint32_t hi[3])
{
    for (int k = 0; k < 3; ++k) {
        lo[k] = clampu(c[k] - e, 0, g->spres[k] - 1);
        hi[k] = clampu(c[k] + e, 0, g->spres[k] - 1);
    }
}

/* myCuda.cuh:403-415 wij_density, myCuda.cuh:84-94 wij (float64) */
static inline double w_density(double d, double r)
{
    if (d < r) { double s = 1.0 - (d / r) * (d / r); return (double)ORC_SIGMA / (r * r * r) * s * s * s; }
    return 0.0;
}
static inline double w_cubic(double d, double r)
{
    if (d < r) { double s = d / r; return 1.0 - s * s * s; }
    return 0.0;
}

/* Anisotropic_kernel.cuh:158-213 */
void orc_density(const orc_params* p, const orc_grid* g, const float* spos, uint32_t n,
                 const uint32_t* start, const uint32_t* end, double* rho)
{
    const double h = p->h;
    #pragma omp parallel for schedule(dynamic, 256)
    for (int64_t i = 0; i < (int64_t)n; ++i) {
        const float* pi = spos + 3 * i;
        uint32_t c[3], lo[3], hi[3];
        cell_of(g, pi, c);
        box_incl(g, c, (uint32_t)g->spexpand, lo, hi);
        double w = 0.0;
        for (uint32_t z = lo[2]; z <= hi[2]; ++z)
            for (uint32_t y = lo[1]; y <= hi[1]; ++y)
                for (uint32_t x = lo[0]; x <= hi[0]; ++x) {
                    uint32_t q = lin3(x, y, z, g->spres);
                    for (uint32_t j = start[q]; j < end[q]; ++j) {
                        const float* pj = spos + 3 * (size_t)j;
                        double dx = (double)pi[0] - pj[0], dy = (double)pi[1] - pj[1], dz = (double)pi[2] - pj[2];
                        w += w_density(sqrt(dx * dx + dy * dy + dz * dz), h);
                    }
                }
        rho[i] = w;
    }
}

/* Symmetric 3x3 eigen decomposition by cyclic Jacobi rotations (float64).
 * A is overwritten; on return eval[k] with evec column k (row-major 3x3),
 * sorted by decreasing |eval|. */
static void jacobi3(double A[3][3], double eval[3], double V[3][3])
{
    for (int i = 0; i < 3; ++i) for (int j = 0; j < 3; ++j) V[i][j] = (i == j);
    for (int sweep = 0; sweep < 64; ++sweep) {
        double off = fabs(A[0][1]) + fabs(A[0][2]) + fabs(A[1][2]);
        double scale = fabs(A[0][0]) + fabs(A[1][1]) + fabs(A[2][2]);
        if (off <= 1e-300 || off <= 1e-17 * scale) break;
        for (int p = 0; p < 2; ++p) for (int q = p + 1; q < 3; ++q) {
            double apq = A[p][q];
            if (apq == 0.0) continue;
            double theta = (A[q][q] - A[p][p]) / (2.0 * apq);
            double t = (theta >= 0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1.0));
            double cs = 1.0 / sqrt(t * t + 1.0), sn = t * cs;
            for (int k = 0; k < 3; ++k) {          /* A = A * J */
                double akp = A[k][p], akq = A[k][q];
                A[k][p] = cs * akp - sn * akq;
                A[k][q] = sn * akp + cs * akq;
            }
            for (int k = 0; k < 3; ++k) {          /* A = J^T * A */
                double apk = A[p][k], aqk = A[q][k];
                A[p][k] = cs * apk - sn * aqk;
                A[q][k] = sn * apk + cs * aqk;
            }
            for (int k = 0; k < 3; ++k) {          /* V = V * J */
                double vkp = V[k][p], vkq = V[k][q];
                V[k][p] = cs * vkp - sn * vkq;
                V[k][q] = sn * vkp + cs * vkq;
            }
        }
    }
    int idx[3] = {0, 1, 2};
    double d[3] = {A[0][0], A[1][1], A[2][2]};
    for (int a = 0; a < 2; ++a) for (int b = a + 1; b < 3; ++b)
        if (fabs(d[idx[b]]) > fabs(d[idx[a]])) { int t = idx[a]; idx[a] = idx[b]; idx[b] = t; }
    double W[3][3];
    for (int k = 0; k < 3; ++k) { eval[k] = d[idx[k]]; for (int r = 0; r < 3; ++r) W[r][k] = V[r][idx[k]]; }
    memcpy(V, W, sizeof(W));
}

/* Anisotropic_kernel.cuh:216-281 (mean) and 350-519 (covariance, G, normal) */
void orc_anisotropy(const orc_params* p, const orc_grid* g, const float* spos, uint32_t n,
                    const uint32_t* start, const uint32_t* end,
                    const uint32_t* list, uint32_t ns,
                    double* mean, double* Gout, double* maxv, double* nrm, uint8_t* flag,
                    uint32_t* nnb)
{
    (void)n;
    const double h = p->h, r2h = p->aniso_radius;
    const uint32_t e2 = 2u * (uint32_t)g->spexpand;
    #pragma omp parallel for schedule(dynamic, 64)
    for (int64_t s = 0; s < (int64_t)ns; ++s) {
        const float* pi = spos + 3 * (size_t)list[s];
        uint32_t c[3], lo[3], hi[3];
        cell_of(g, pi, c);
        box_incl(g, c, e2, lo, hi);
        /* pass 1: weighted mean, support 2h */
        double ws = 0, mx = 0, my = 0, mz = 0;
        for (uint32_t z = lo[2]; z <= hi[2]; ++z)
            for (uint32_t y = lo[1]; y <= hi[1]; ++y)
                for (uint32_t x = lo[0]; x <= hi[0]; ++x) {
                    uint32_t q = lin3(x, y, z, g->spres);
                    for (uint32_t j = start[q]; j < end[q]; ++j) {
                        const float* pj = spos + 3 * (size_t)j;
                        double dx = (double)pi[0] - pj[0], dy = (double)pi[1] - pj[1], dz = (double)pi[2] - pj[2];
                        double w = w_cubic(sqrt(dx * dx + dy * dy + dz * dz), r2h);
                        ws += w; mx += w * pj[0]; my += w * pj[1]; mz += w * pj[2];
                    }
                }
        double m[3] = {0, 0, 0};
        if (ws > 0) { m[0] = mx / ws; m[1] = my / ws; m[2] = mz / ws; }
        mean[3 * s + 0] = m[0]; mean[3 * s + 1] = m[1]; mean[3 * s + 2] = m[2];

        /* pass 2: covariance about the mean, neighbour count within h */
        double C[3][3] = {{h * h, 0, 0}, {0, h * h, 0}, {0, 0, h * h}};
        /* the reference seeds with smoothingRadiusSq (float32 h*h) */
        C[0][0] = C[1][1] = C[2][2] = (double)p->h_sq;
        double wsum = 0;
        uint32_t cnt = 0;
        for (uint32_t z = lo[2]; z <= hi[2]; ++z)
            for (uint32_t y = lo[1]; y <= hi[1]; ++y)
                for (uint32_t x = lo[0]; x <= hi[0]; ++x) {
                    uint32_t q = lin3(x, y, z, g->spres);
                    for (uint32_t j = start[q]; j < end[q]; ++j) {
                        const float* pj = spos + 3 * (size_t)j;
                        double ux = (double)pj[0] - pi[0], uy = (double)pj[1] - pi[1], uz = (double)pj[2] - pi[2];
                        double dist = sqrt(ux * ux + uy * uy + uz * uz);
                        if (dist <= h) ++cnt;
                        double v[3] = {(double)pj[0] - m[0], (double)pj[1] - m[1], (double)pj[2] - m[2]};
                        double w = w_cubic(dist, r2h);
                        wsum += w;
                        for (int a = 0; a < 3; ++a) for (int b = 0; b < 3; ++b) C[a][b] += w * v[a] * v[b];
                    }
                }
        nnb[s] = cnt;
        double G[3][3];
        double nv[3];
        double mval;
        uint8_t fl;
        if ((int)cnt < p->min_num_neighbors) {
            for (int a = 0; a < 3; ++a) for (int b = 0; b < 3; ++b) G[a][b] = (a == b) ? (double)p->h_inv : 0.0;
            mval = 1.0; fl = 1; nv[0] = 1; nv[1] = 0; nv[2] = 0;
        } else {
            for (int a = 0; a < 3; ++a) for (int b = 0; b < 3; ++b) C[a][b] /= wsum;
            double sv[3], U[3][3];
            jacobi3(C, sv, U);
            for (int k = 0; k < 3; ++k) sv[k] = fabs(sv[k]);
            double mx3 = fmax(sv[0], fmax(sv[1], sv[2]));
            double mn3 = fmin(sv[0], fmin(sv[1], sv[2]));
            fl = (mn3 <= mx3 * 0.25) ? 1 : 0;
            double lim = mx3 / 4.0;
            for (int k = 0; k < 3; ++k) sv[k] = fmax(sv[k], lim);
            double scale = cbrt(sv[0] * sv[1] * sv[2]);
            double cof = (double)p->h_inv * scale;
            double inv[3] = {cof / sv[0], cof / sv[1], cof / sv[2]};
            /* G = U diag(inv) U^T (U == V for a symmetric positive matrix) */
            for (int a = 0; a < 3; ++a) for (int b = 0; b < 3; ++b) {
                double acc = 0;
                for (int k = 0; k < 3; ++k) acc += U[a][k] * inv[k] * U[b][k];
                G[a][b] = acc;
            }
            nv[0] = U[0][2]; nv[1] = U[1][2]; nv[2] = U[2][2];
            mval = sv[0] / scale;
        }
        double dpm = nv[0] * ((double)pi[0] - m[0]) + nv[1] * ((double)pi[1] - m[1]) + nv[2] * ((double)pi[2] - m[2]);
        if (dpm < 0.0) { nv[0] = -nv[0]; nv[1] = -nv[1]; nv[2] = -nv[2]; }
        for (int a = 0; a < 3; ++a) for (int b = 0; b < 3; ++b) Gout[9 * s + 3 * a + b] = G[a][b];
        maxv[s] = mval;
        nrm[3 * s + 0] = nv[0]; nrm[3 * s + 1] = nv[1]; nrm[3 * s + 2] = nv[2];
        flag[s] = fl;
    }
}

/* ------------------------------------------------------------------------ */
/* Anisotropic_kernel.cuh:522-636 (LOWRES on, USING_GRID off), bit-exact:    */
/* float32 vertex positions i*cell+min and dot products without contraction  */
/* ------------------------------------------------------------------------ */
static inline void bm_set(uint32_t* bm, uint64_t nbits, uint64_t i)
{
    if (i < nbits) bm[i >> 5] |= 1u << (i & 31);
}

void orc_band_bitmap(const orc_grid* g, float h, const float* spos, const uint32_t* list,
                     uint32_t ns, const float* nrm, const uint8_t* flag, uint32_t* bitmap)
{
    const uint64_t nbits = g->sc_size;
    const int32_t rx = (int32_t)g->scres[0], ry = (int32_t)g->scres[1], rz = (int32_t)g->scres[2];
    const float cs = g->sc_grid_size;
    const uint32_t ext = (uint32_t)ceilf(h / cs);
    for (uint32_t s = 0; s < ns; ++s) {
        const float* p = spos + 3 * (size_t)list[s];
        const float* nv = nrm + 3 * (size_t)s;
        int fl = flag[s] != 0;
        int32_t c[3];
        for (int k = 0; k < 3; ++k) c[k] = (int32_t)((p[k] - g->scmin_pos[k]) / cs);   /* make_int3 truncation */
        float aa[3], bb[3];
        for (int k = 0; k < 3; ++k) { aa[k] = p[k] - h; bb[k] = p[k] + h; }
        int32_t lo[3], hi[3];
        int32_t res[3] = {rx, ry, rz};
        for (int k = 0; k < 3; ++k) {
            lo[k] = clampi(c[k] - (int32_t)ext, 0, res[k] - 1);
            hi[k] = clampi(c[k] + (int32_t)ext, 0, res[k] - 1);
        }
        for (int32_t z = lo[2]; z <= hi[2]; ++z)
            for (int32_t y = lo[1]; y <= hi[1]; ++y)
                for (int32_t x = lo[0]; x <= hi[0]; ++x) {
                    float v[3];
                    int32_t ix[3] = {x, y, z};
                    for (int k = 0; k < 3; ++k) {
                        volatile float t = (float)ix[k] * cs;
                        v[k] = t + g->scmin_pos[k];
                    }
                    int outside = (v[0] < aa[0] || v[1] < aa[1] || v[2] < aa[2]) ||
                                  (v[0] > bb[0] || v[1] > bb[1] || v[2] > bb[2]);
                    if (outside) continue;
                    float d0 = v[0] - p[0], d1 = v[1] - p[1], d2 = v[2] - p[2];
                    volatile float t0 = nv[0] * d0, t1 = nv[1] * d1, t2 = nv[2] * d2;
                    float dot = (t0 + t1) + t2;
                    if (fl || dot > 0.0f) {
                        uint64_t id = (uint64_t)(uint32_t)(z * rx * ry + y * rx + x);
                        bm_set(bitmap, nbits, id);
                        bm_set(bitmap, nbits, id + 1);                              /* +x */
                        bm_set(bitmap, nbits, id + (uint32_t)rx);                   /* +y */
                        bm_set(bitmap, nbits, id + (uint64_t)(uint32_t)(rx * ry)); /* +z */
                    }
                }
    }
}

uint64_t orc_bitmap_to_list(const uint32_t* bm, uint64_t nbits, uint32_t* list)
{
    uint64_t k = 0;
    for (uint64_t i = 0; i < nbits; ++i)
        if (bm[i >> 5] >> (i & 31) & 1u) { if (list) list[k] = (uint32_t)i; ++k; }
    return k;
}

/* ------------------------------------------------------------------------ */
/* Anisotropic_kernel.cuh:656-777, anisotropicW/anisotropicWOpt              */
/* myCuda.cuh:151-191 (float64)                                              */
/* ------------------------------------------------------------------------ */
void orc_field(const orc_params* p, const orc_grid* g, const float* spos, uint32_t n,
               const double* rho, const uint32_t* start, const uint32_t* end,
               const uint32_t* surf_count, const uint32_t* surf_scan,
               const double* Gs, const double* maxv,
               const uint32_t* verts, uint32_t nv, double* field)
{
    (void)n;
    const double h = p->h, mass = p->mass, thr = 2.0 * (double)p->iso_value;
    const double sig = (double)ORC_SIGMA;
    const uint32_t e2 = 2u * (uint32_t)g->spexpand;
    const uint32_t rx = g->scres[0], ry = g->scres[1];
    #pragma omp parallel for schedule(dynamic, 256)
    for (int64_t t = 0; t < (int64_t)nv; ++t) {
        uint32_t id = verts[t];
        uint32_t iz = id / (rx * ry), m = id % (rx * ry), iy = m / rx, ix = m % rx;
        /* vertex position as the reference computes it in float32 */
        float vp[3];
        uint32_t ii[3] = {ix, iy, iz};
        for (int k = 0; k < 3; ++k) { volatile float tt = (float)ii[k] * g->sc_grid_size; vp[k] = tt + g->scmin_pos[k]; }
        uint32_t c[3], lo[3], hi[3];
        cell_of(g, vp, c);
        box_incl(g, c, e2, lo, hi);
        double sum = 0.0;
        for (uint32_t z = lo[2]; z < hi[2]; ++z)
            for (uint32_t y = lo[1]; y < hi[1]; ++y)
                for (uint32_t x = lo[0]; x < hi[0]; ++x) {
                    uint32_t q = lin3(x, y, z, g->spres);
                    uint32_t cnt = end[q] - start[q];
                    if (surf_count[q] > 0) {
                        for (uint32_t i = 0; i < cnt; ++i) {
                            uint32_t sid = surf_scan[q] + i;
                            uint32_t j = start[q] + i;
                            if (rho[j] == 0.0) continue;
                            const float* pj = spos + 3 * (size_t)j;
                            double r[3] = {(double)pj[0] - vp[0], (double)pj[1] - vp[1], (double)pj[2] - vp[2]};
                            double len = sqrt(r[0] * r[0] + r[1] * r[1] + r[2] * r[2]);
                            double hs = maxv[sid] * h;
                            if (len >= hs) continue;
                            const double* G = Gs + 9 * (size_t)sid;
                            double tx = r[0] * G[0] + r[1] * G[1] + r[2] * G[2];
                            double ty = r[0] * G[3] + r[1] * G[4] + r[2] * G[5];
                            double tz = r[0] * G[6] + r[1] * G[7] + r[2] * G[8];
                            double d2 = tx * tx + ty * ty + tz * tz;
                            if (d2 >= 1.0) continue;
                            double det = G[0] * G[4] * G[8] + G[1] * G[5] * G[6] + G[2] * G[3] * G[7]
                                       - G[0] * G[5] * G[7] - G[1] * G[3] * G[8] - G[2] * G[4] * G[6];
                            double xx = 1.0 - d2;
                            sum += mass / rho[j] * (sig * det * xx * xx * xx);
                        }
                    } else {
                        for (uint32_t j = start[q]; j < end[q]; ++j) {
                            if (rho[j] == 0.0) continue;
                            const float* pj = spos + 3 * (size_t)j;
                            double r[3] = {(double)pj[0] - vp[0], (double)pj[1] - vp[1], (double)pj[2] - vp[2]};
                            double l2 = r[0] * r[0] + r[1] * r[1] + r[2] * r[2];
                            if (sqrt(l2) >= h) continue;
                            double inv = 1.0 / h;
                            double d2 = l2 * inv * inv;
                            double xx = 1.0 - d2;
                            sum += mass / rho[j] * (sig * inv * inv * inv * xx * xx * xx);
                        }
                    }
                    if (sum > thr) break;
                }
        field[t] = sum;
    }
}

/* ------------------------------------------------------------------------ */
/* MarchingCube_kernel.cuh:20-157, myCuda.cuh:205-339                         */
/* ------------------------------------------------------------------------ */
static uint32_t T_edge[256];
static int32_t  T_tri[256 * 16];
static uint32_t T_nv[256];
static uint32_t T_ev[24];
static const int CORNER[8][3] = {{0,0,0},{0,0,1},{0,1,1},{0,1,0},{1,0,0},{1,0,1},{1,1,1},{1,1,0}};

void orc_mc_set_tables(const uint32_t* e, const int32_t* t, const uint32_t* nvt, const uint32_t* ev)
{
    memcpy(T_edge, e, sizeof(T_edge));
    memcpy(T_tri, t, sizeof(T_tri));
    memcpy(T_nv, nvt, sizeof(T_nv));
    memcpy(T_ev, ev, sizeof(T_ev));
}

static inline int bm_get(const uint32_t* bm, uint64_t nbits, uint64_t i)
{
    return i < nbits ? (int)((bm[i >> 5] >> (i & 31)) & 1u) : 0;
}

/* rank of vertex id in the band list (binary search: verts is ascending) */
static inline int64_t band_rank(const uint32_t* verts, uint32_t nv, uint32_t id)
{
    uint32_t lo = 0, hi = nv;
    while (lo < hi) { uint32_t mid = lo + (hi - lo) / 2; if (verts[mid] < id) lo = mid + 1; else hi = mid; }
    return (lo < nv && verts[lo] == id) ? (int64_t)lo : -1;
}

uint64_t orc_mc_classify(const orc_grid* g, float iso, const uint32_t* bitmap,
                         const uint32_t* verts, uint32_t nv, const float* fieldv,
                         uint32_t* cases, uint32_t* nvert)
{
    const uint32_t rx = g->scres[0], ry = g->scres[1];
    const uint64_t nbits = g->sc_size;
    uint64_t total = 0;
    for (uint32_t t = 0; t < nv; ++t) {
        uint32_t id = verts[t];
        uint32_t z = id / (rx * ry), m = id % (rx * ry), y = m / rx, x = m % rx;
        uint32_t corner[8];
        int all = 1;
        for (int k = 0; k < 8; ++k) {
            corner[k] = (z + CORNER[k][2]) * rx * ry + (y + CORNER[k][1]) * rx + (x + CORNER[k][0]);
            if (!bm_get(bitmap, nbits, corner[k])) all = 0;
        }
        uint32_t cs = 0, nvx = 0;
        if (all) {
            for (int k = 0; k < 8; ++k) {
                int64_t r = band_rank(verts, nv, corner[k]);
                float f = fieldv[r];
                if (f <= iso) cs |= 1u << k;
            }
            nvx = T_nv[cs];
        }
        cases[t] = cs;
        nvert[t] = nvx;
        total += nvx;
    }
    return total;
}

static inline double fval(const orc_grid* g, const uint32_t* bitmap, const uint32_t* verts, uint32_t nv,
                          const double* fieldv, int64_t x, int64_t y, int64_t z)
{
    if (x < 0 || y < 0 || z < 0 || x >= g->scres[0] || y >= g->scres[1] || z >= g->scres[2]) return 0.0;
    uint64_t id = (uint64_t)z * g->scres[0] * g->scres[1] + (uint64_t)y * g->scres[0] + (uint64_t)x;
    if (!bm_get(bitmap, g->sc_size, id)) return 0.0;
    int64_t r = band_rank(verts, nv, (uint32_t)id);
    return r < 0 ? 0.0 : fieldv[r];
}

static inline void normalize3(double v[3])
{
    double l = sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    if (l > 0) { v[0] /= l; v[1] /= l; v[2] /= l; }
    else { v[0] = v[1] = v[2] = NAN; }
}

void orc_mc_emit(const orc_grid* g, float iso, const uint32_t* bitmap,
                 const uint32_t* verts, uint32_t nv, const double* fieldv,
                 const uint32_t* cases, const uint32_t* nvert, const uint64_t* offsets,
                 double* vpos, double* vnrm)
{
    const uint32_t rx = g->scres[0], ry = g->scres[1];
    const double cs = g->sc_grid_size;
    #pragma omp parallel for schedule(dynamic, 256)
    for (int64_t t = 0; t < (int64_t)nv; ++t) {
        if (nvert[t] == 0) continue;
        uint32_t id = verts[t];
        int64_t z = id / (rx * ry), m = id % (rx * ry), y = m / rx, x = m % rx;
        uint32_t cse = cases[t];
        double cp[8][3], cn[8][3], cf[8];
        for (int k = 0; k < 8; ++k) {
            int64_t X = x + CORNER[k][0], Y = y + CORNER[k][1], Z = z + CORNER[k][2];
            cp[k][0] = (double)X * cs + g->scmin_pos[0];
            cp[k][1] = (double)Y * cs + g->scmin_pos[1];
            cp[k][2] = (double)Z * cs + g->scmin_pos[2];
            cf[k] = fval(g, bitmap, verts, nv, fieldv, X, Y, Z);
            cn[k][0] = fval(g, bitmap, verts, nv, fieldv, X - 1, Y, Z) - fval(g, bitmap, verts, nv, fieldv, X + 1, Y, Z);
            cn[k][1] = fval(g, bitmap, verts, nv, fieldv, X, Y - 1, Z) - fval(g, bitmap, verts, nv, fieldv, X, Y + 1, Z);
            cn[k][2] = fval(g, bitmap, verts, nv, fieldv, X, Y, Z - 1) - fval(g, bitmap, verts, nv, fieldv, X, Y, Z + 1);
            normalize3(cn[k]);
        }
        double ip[12][3], in[12][3];
        double sign = (iso < 0.0f) ? -1.0 : 1.0;
        uint32_t ef = T_edge[cse];
        for (int i = 0; i < 12; ++i) {
            if (!(ef & (1u << i))) continue;
            uint32_t a = T_ev[2 * i], b = T_ev[2 * i + 1];
            double d = cf[b] - cf[a];
            double tt = (d > -ORC_EPS && d < ORC_EPS) ? 0.5 : ((double)iso - cf[a]) / d;
            double nn[3];
            for (int k = 0; k < 3; ++k) {
                ip[i][k] = cp[a][k] + tt * (cp[b][k] - cp[a][k]);
                nn[k] = cn[a][k] + tt * (cn[b][k] - cn[a][k]);
            }
            normalize3(nn);
            for (int k = 0; k < 3; ++k) in[i][k] = sign * nn[k];
        }
        uint64_t base = offsets[t];
        for (uint32_t v = 0; v < nvert[t]; ++v) {
            int e = T_tri[cse * 16 + v];
            for (int k = 0; k < 3; ++k) { vpos[3 * (base + v) + k] = ip[e][k]; vnrm[3 * (base + v) + k] = in[e][k]; }
        }
    }
}

/* ------------------------------------------------------------------------ */
/* Mesh distance: vertex-to-triangle distance over a uniform bucket grid      */
/* ------------------------------------------------------------------------ */
static double pt_tri_dist2(const double* p, const double* a, const double* b, const double* c)
{
    /* closest point on triangle (Ericson, Real-Time Collision Detection 5.1.5) */
    double ab[3], ac[3], ap[3];
    for (int k = 0; k < 3; ++k) { ab[k] = b[k] - a[k]; ac[k] = c[k] - a[k]; ap[k] = p[k] - a[k]; }
#define DOT(u, v) ((u)[0] * (v)[0] + (u)[1] * (v)[1] + (u)[2] * (v)[2])
    double d1 = DOT(ab, ap), d2 = DOT(ac, ap);
    double q[3];
    if (d1 <= 0 && d2 <= 0) { for (int k = 0; k < 3; ++k) q[k] = a[k]; goto done; }
    double bp[3]; for (int k = 0; k < 3; ++k) bp[k] = p[k] - b[k];
    double d3 = DOT(ab, bp), d4 = DOT(ac, bp);
    if (d3 >= 0 && d4 <= d3) { for (int k = 0; k < 3; ++k) q[k] = b[k]; goto done; }
    double vc = d1 * d4 - d3 * d2;
    if (vc <= 0 && d1 >= 0 && d3 <= 0) { double v = d1 / (d1 - d3); for (int k = 0; k < 3; ++k) q[k] = a[k] + v * ab[k]; goto done; }
    double cpv[3]; for (int k = 0; k < 3; ++k) cpv[k] = p[k] - c[k];
    double d5 = DOT(ab, cpv), d6 = DOT(ac, cpv);
    if (d6 >= 0 && d5 <= d6) { for (int k = 0; k < 3; ++k) q[k] = c[k]; goto done; }
    double vb = d5 * d2 - d1 * d6;
    if (vb <= 0 && d2 >= 0 && d6 <= 0) { double w = d2 / (d2 - d6); for (int k = 0; k < 3; ++k) q[k] = a[k] + w * ac[k]; goto done; }
    double va = d3 * d6 - d5 * d4;
    if (va <= 0 && (d4 - d3) >= 0 && (d5 - d6) >= 0) {
        double w = (d4 - d3) / ((d4 - d3) + (d5 - d6));
        for (int k = 0; k < 3; ++k) q[k] = b[k] + w * (c[k] - b[k]);
        goto done;
    }
    {
        double den = 1.0 / (va + vb + vc);
        double v = vb * den, w = vc * den;
        for (int k = 0; k < 3; ++k) q[k] = a[k] + ab[k] * v + ac[k] * w;
    }
done:;
    double dd[3] = {p[0] - q[0], p[1] - q[1], p[2] - q[2]};
    return DOT(dd, dd);
#undef DOT
}

double orc_hausdorff_vertices_to_mesh(const double* a, uint64_t na, const double* b, uint64_t nb, double cell)
{
    if (na == 0) return 0.0;
    if (nb < 3) return INFINITY;
    const uint64_t ntri = nb / 3;
    double lo[3] = {DBL_MAX, DBL_MAX, DBL_MAX}, hi[3] = {-DBL_MAX, -DBL_MAX, -DBL_MAX};
    for (uint64_t i = 0; i < nb; ++i)
        for (int k = 0; k < 3; ++k) { double v = b[3 * i + k]; if (v < lo[k]) lo[k] = v; if (v > hi[k]) hi[k] = v; }
    int64_t res[3];
    for (int k = 0; k < 3; ++k) { res[k] = (int64_t)((hi[k] - lo[k]) / cell) + 1; if (res[k] < 1) res[k] = 1; }
    const uint64_t nc = (uint64_t)res[0] * res[1] * res[2];
    uint32_t* cnt = (uint32_t*)calloc(nc + 1, sizeof(uint32_t));
    uint32_t* fill = (uint32_t*)calloc(nc, sizeof(uint32_t));
    uint32_t* items = NULL;
    /* bucket each triangle by its bounding box: pass 0 counts, pass 1 fills */
    for (int pass = 0; pass < 2; ++pass) {
        if (pass == 1) {
            for (uint64_t c = 0; c < nc; ++c) cnt[c + 1] += cnt[c];
            items = (uint32_t*)malloc(sizeof(uint32_t) * ((size_t)cnt[nc] + 1));
        }
        for (uint64_t t = 0; t < ntri; ++t) {
            int64_t l[3], u[3];
            for (int k = 0; k < 3; ++k) {
                double mn = b[9 * t + k], mx = mn;
                for (int v = 1; v < 3; ++v) { double x = b[9 * t + 3 * v + k]; if (x < mn) mn = x; if (x > mx) mx = x; }
                l[k] = (int64_t)((mn - lo[k]) / cell); u[k] = (int64_t)((mx - lo[k]) / cell);
                if (l[k] < 0) l[k] = 0;
                if (u[k] >= res[k]) u[k] = res[k] - 1;
            }
            for (int64_t z = l[2]; z <= u[2]; ++z)
                for (int64_t y = l[1]; y <= u[1]; ++y)
                    for (int64_t x = l[0]; x <= u[0]; ++x) {
                        uint64_t c = ((uint64_t)z * res[1] + y) * res[0] + x;
                        if (pass == 0) cnt[c + 1]++;
                        else items[cnt[c] + fill[c]++] = (uint32_t)t;
                    }
        }
    }
    double worst = 0.0;
    #pragma omp parallel for schedule(dynamic, 1024) reduction(max:worst)
    for (int64_t i = 0; i < (int64_t)na; ++i) {
        const double* p = a + 3 * i;
        int64_t c0[3];
        for (int k = 0; k < 3; ++k) c0[k] = (int64_t)floor((p[k] - lo[k]) / cell);
        double best = INFINITY;
        const int64_t rmax = res[0] + res[1] + res[2] + 2;
        for (int64_t r = 0; r <= rmax; ++r) {
            /* shell of Chebyshev radius r around the vertex's bucket */
            for (int64_t z = c0[2] - r; z <= c0[2] + r; ++z)
                for (int64_t y = c0[1] - r; y <= c0[1] + r; ++y)
                    for (int64_t x = c0[0] - r; x <= c0[0] + r; ++x) {
                        int64_t dz = llabs(z - c0[2]), dy = llabs(y - c0[1]), dx = llabs(x - c0[0]);
                        int64_t md = dx > dy ? dx : dy;
                        md = md > dz ? md : dz;
                        if (md != r) continue;
                        if (x < 0 || y < 0 || z < 0 || x >= res[0] || y >= res[1] || z >= res[2]) continue;
                        uint64_t c = ((uint64_t)z * res[1] + y) * res[0] + x;
                        for (uint32_t q = cnt[c]; q < cnt[c + 1]; ++q) {
                            const double* tr = b + 9 * (size_t)items[q];
                            double d2 = pt_tri_dist2(p, tr, tr + 3, tr + 6);
                            if (d2 < best) best = d2;
                        }
                    }
            /* every triangle not yet visited is at least r*cell away */
            double reach = (double)r * cell;
            if (best <= reach * reach) break;
        }
        double d = sqrt(best);
        if (d > worst) worst = d;
    }
    free(items); free(fill); free(cnt);
    return worst;
}

/* ------------------------------------------------------------------------ */
/* MarchingCube_kernel.cuh:161-233  estimationOfScalarValue (float64)        */
/* For mesh vertex v in spatial cell c: over cells [c - e, c + e) (clamped,  */
/* the upper bound exclusive as in the reference), w = 1 - (d/h)^3 for       */
/* d < h; rhop = sum w rho_j / sum w, vel = sum w vel_j / sum w (zero when   */
/* no particle is within h).  out: 5 per vertex {vel xyz, |vel|, rhop}.      */
/* ------------------------------------------------------------------------ */
void orc_scalar_values(const orc_params* p, const orc_grid* g, const float* spos, const float* svel,
                       const double* rho, const uint32_t* start, const uint32_t* end, const float* verts,
                       uint64_t m, double* out)
{
    const double h = p->h;
    #pragma omp parallel for schedule(dynamic, 256)
    for (int64_t t = 0; t < (int64_t)m; ++t) {
        const float* v = verts + 3 * t;
        uint32_t c[3], lo[3], hi[3];
        cell_of(g, v, c);
        box_incl(g, c, (uint32_t)g->spexpand, lo, hi);
        double ws = 0.0, rh = 0.0, vx = 0.0, vy = 0.0, vz = 0.0;
        for (uint32_t z = lo[2]; z < hi[2]; ++z)
            for (uint32_t y = lo[1]; y < hi[1]; ++y)
                for (uint32_t x = lo[0]; x < hi[0]; ++x) {
                    const uint32_t q = lin3(x, y, z, g->spres);
                    for (uint32_t j = start[q]; j < end[q]; ++j) {
                        const float* pj = spos + 3 * (size_t)j;
                        const double dx = (double)v[0] - pj[0], dy = (double)v[1] - pj[1], dz = (double)v[2] - pj[2];
                        const double d = sqrt(dx * dx + dy * dy + dz * dz);
                        if (d >= h) continue;
                        const double s = d / h, w = 1.0 - s * s * s;
                        rh += w * rho[j];
                        vx += w * svel[3 * (size_t)j]; vy += w * svel[3 * (size_t)j + 1]; vz += w * svel[3 * (size_t)j + 2];
                        ws += w;
                    }
                }
        double* o = out + 5 * t;
        if (ws > 0.0) {
            vx /= ws; vy /= ws; vz /= ws;
            o[0] = vx; o[1] = vy; o[2] = vz; o[3] = sqrt(vx * vx + vy * vy + vz * vz); o[4] = rh / ws;
        } else {
            o[0] = o[1] = o[2] = o[3] = o[4] = 0.0;
        }
    }
}

