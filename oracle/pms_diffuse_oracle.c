/*
 * pms_diffuse_oracle.c -- CPU oracle of the diffuse-particle stage.
 *
 * TEST INFRASTRUCTURE ONLY (see pms_oracle.h).  Restates
 * DiffuseGeneration_kernel.cuh:528-1199 and DiffuseGeneration.cu:187-442,
 * 760-867 with myCuda.cuh:341-401:
 *   normals, trapped air, energy, wave crests   float64
 *   spawn counts (phi clamps, floor)            float32, each operation rounded
 *                                               once, from given potentials
 *   spawn: velocities float64 from the float32 inputs; positions, TTL and
 *          types (neighbour counts, float32 distances) exact
 *   advection of old diffuse particles          float32 operation by operation
 *                                               (Wendland weights in float64, as
 *                                               the reference evaluates them)
 * The spawn uniforms use the same counter-based generator as the product
 * (splitmix64 of seed, frame and index), standing in for the reference's
 * std::random_device / mt19937 stream.
 */
#include "pms_oracle.h"

#include <math.h>
#include <string.h>
#include <stdlib.h>

#define D_EPS 1.0e-7
#define D_PI_F 3.14159265f
#define D_SPRAY 6
#define D_BUBBLE 20

static inline uint32_t clampu_d(uint32_t v, uint32_t lo, uint32_t hi) { return v < lo ? lo : (v > hi ? hi : v); }
static inline uint32_t f2u_d(float x) { if (!(x > 0.0f)) return 0u; if (x >= 4294967296.0f) return 0xffffffffu; return (uint32_t)x; }

static void dbox(const orc_grid* g, const float* p, uint32_t lo[3], uint32_t hi[3])
{
    for (int k = 0; k < 3; ++k) {
        uint32_t c = f2u_d((p[k] - g->min_pos[k]) / g->sp_grid_size);
        uint32_t e = (uint32_t)g->spexpand_diffuse;
        lo[k] = clampu_d(c - e, 0, g->spres[k] - 1);
        hi[k] = clampu_d(c + e, 0, g->spres[k] - 1);
    }
}
static inline uint32_t dlin(const orc_grid* g, uint32_t x, uint32_t y, uint32_t z)
{
    return z * g->spres[0] * g->spres[1] + y * g->spres[0] + x;
}

float orc_spawn_uniform(uint64_t seed, uint32_t frame, uint64_t idx)
{
    uint64_t x = seed * 0x9E3779B97F4A7C15ull + (uint64_t)frame * 0xD1B54A32D192ED03ull + idx;
    x ^= x >> 30; x *= 0xBF58476D1CE4E5B9ull;
    x ^= x >> 27; x *= 0x94D049BB133111EBull;
    x ^= x >> 31;
    return (float)((double)(x >> 40) * (1.0 / 16777216.0));
}

/* calculationofNormal (DiffuseGeneration_kernel.cuh:528-609), launched for
 * particles 0 .. nfree-1 (the reference indexes particles by thread id).
 * nrm: 3n, holds the starting normals on entry. */
void orc_df_normals(const orc_params* p, const orc_grid* g, const float* spos, uint32_t n,
                    const uint32_t* start, const uint32_t* end, uint32_t nfree, double* nrm)
{
    const double h = p->hd, h2 = p->hd_sq, coef = p->coefficient;
    if (nfree > n) nfree = n;
    #pragma omp parallel for schedule(dynamic, 256)
    for (int64_t t = 0; t < (int64_t)nfree; ++t) {
        const float* pi = spos + 3 * t;
        uint32_t lo[3], hi[3];
        dbox(g, pi, lo, hi);
        double nx = 0, ny = 0, nz = 0;
        for (uint32_t z = lo[2]; z <= hi[2]; ++z)
            for (uint32_t y = lo[1]; y <= hi[1]; ++y)
                for (uint32_t x = lo[0]; x <= hi[0]; ++x) {
                    uint32_t c = dlin(g, x, y, z);
                    for (uint32_t j = start[c]; j < end[c]; ++j) {
                        const float* pj = spos + 3 * (size_t)j;
                        double sx = (double)pi[0] - pj[0], sy = (double)pi[1] - pj[1], sz = (double)pi[2] - pj[2];
                        double mp2 = sx * sx + sy * sy + sz * sz, mp = sqrt(mp2), q = mp / h;
                        if (q > 0 && q < 1) {
                            double d = h2 - mp2, c6 = coef / mp * d * d * 6.0;
                            nx += c6 * sx; ny += c6 * sy; nz += c6 * sz;
                        }
                    }
                }
        double mn2 = nx * nx + ny * ny + nz * nz;
        if (mn2 < D_EPS) continue;
        double il = 1.0 / sqrt(mn2);
        nrm[3 * t] = nx * il; nrm[3 * t + 1] = ny * il; nrm[3 * t + 2] = nz * il;
    }
}

/* calculationofTrappedairpotential (:689-761) */
void orc_df_trapped(const orc_params* p, const orc_grid* g, const float* spos, const float* svel, uint32_t n,
                    const uint32_t* start, const uint32_t* end, double* ita, double* energy)
{
    const double h = p->hd;
    #pragma omp parallel for schedule(dynamic, 256)
    for (int64_t i = 0; i < (int64_t)n; ++i) {
        const float* pi = spos + 3 * i;
        const float* vi = svel + 3 * i;
        uint32_t lo[3], hi[3];
        dbox(g, pi, lo, hi);
        double acc = 0;
        for (uint32_t z = lo[2]; z <= hi[2]; ++z)
            for (uint32_t y = lo[1]; y <= hi[1]; ++y)
                for (uint32_t x = lo[0]; x <= hi[0]; ++x) {
                    uint32_t c = dlin(g, x, y, z);
                    for (uint32_t j = start[c]; j < end[c]; ++j) {
                        const float* pj = spos + 3 * (size_t)j;
                        const float* vj = svel + 3 * (size_t)j;
                        double sx = (double)pi[0] - pj[0], sy = (double)pi[1] - pj[1], sz = (double)pi[2] - pj[2];
                        double mp = sqrt(sx * sx + sy * sy + sz * sz);
                        if (mp > D_EPS && mp <= h) {
                            double ux = (double)vi[0] - vj[0], uy = (double)vi[1] - vj[1], uz = (double)vi[2] - vj[2];
                            double mv = ux * ux + uy * uy + uz * uz;
                            if (mv > D_EPS) {
                                mv = sqrt(mv);
                                double e = 1.0 - (ux / mv * (sx / mp) + uy / mv * (sy / mp) + uz / mv * (sz / mp));
                                acc += mv * e * (1.0 - mp / h);
                            }
                        }
                    }
                }
        ita[i] = acc;
        energy[i] = 0.5 * (double)p->mass * ((double)vi[0] * vi[0] + (double)vi[1] * vi[1] + (double)vi[2] * vi[2]);
    }
}

static inline float dot_rn3(const float* a, const float* b)
{
    volatile float x = a[0] * b[0], y = a[1] * b[1], z = a[2] * b[2];
    volatile float s = x + y;
    return s + z;
}

/* calculationofWavecrests (:611-687) for the free-surface list; nrm are the
 * float32 particle normals the crest sum reads. */
void orc_df_crests(const orc_params* p, const orc_grid* g, const float* spos, const float* svel,
                   const uint32_t* start, const uint32_t* end, const uint32_t* free_list, uint32_t nfree,
                   const float* nrm, double* wc)
{
    const double h = p->hd;
    #pragma omp parallel for schedule(dynamic, 256)
    for (int64_t t = 0; t < (int64_t)nfree; ++t) {
        uint32_t i = free_list[t];
        const float* pi = spos + 3 * (size_t)i;
        const float* vi = svel + 3 * (size_t)i;
        const float* ni = nrm + 3 * (size_t)i;
        if ((double)dot_rn3(ni, ni) <= D_EPS || (double)dot_rn3(vi, vi) <= D_EPS || (double)dot_rn3(vi, ni) < 0.6) {
            wc[i] = 0;
            continue;
        }
        uint32_t lo[3], hi[3];
        dbox(g, pi, lo, hi);
        double acc = 0;
        for (uint32_t z = lo[2]; z <= hi[2]; ++z)
            for (uint32_t y = lo[1]; y <= hi[1]; ++y)
                for (uint32_t x = lo[0]; x <= hi[0]; ++x) {
                    uint32_t c = dlin(g, x, y, z);
                    for (uint32_t j = start[c]; j < end[c]; ++j) {
                        const float* nj = nrm + 3 * (size_t)j;
                        if ((double)dot_rn3(nj, nj) <= D_EPS) continue;
                        const float* pj = spos + 3 * (size_t)j;
                        double dx = (double)pj[0] - pi[0], dy = (double)pj[1] - pi[1], dz = (double)pj[2] - pi[2];
                        double l = sqrt(dx * dx + dy * dy + dz * dz);
                        if (l == 0) continue;
                        double cth = (dx * ni[0] + dy * ni[1] + dz * ni[2]) / l;
                        if (cth < -D_EPS) {
                            double e1 = 1.0 - ((double)ni[0] * nj[0] + (double)ni[1] * nj[1] + (double)ni[2] * nj[2]);
                            double w = (l <= h && l > 0) ? 1.0 - l / h : 0.0;
                            acc += e1 * w;
                        }
                    }
                }
        wc[i] = acc;
    }
}

static inline float phi_f(float I, float tmin, float tmax)
{
    volatile float a = fminf(I, tmax) - fminf(I, tmin);
    volatile float b = tmax - tmin;
    return a / b;
}

/* calculateofNumberofdiffuseparticles (:763-791): pot_raw (3n float: waveCrest,
 * Ita, energy before the clamps) -> clamped potentials and counts. */
void orc_df_counts(const orc_params* p, const float* pot_raw, uint32_t n, float* pot_clamped, int32_t* num)
{
    for (uint32_t i = 0; i < n; ++i) {
        float wc = phi_f(pot_raw[3 * i], p->min_wc, p->max_wc);
        float ta = phi_f(pot_raw[3 * i + 1], p->min_ta, p->max_ta);
        float en = phi_f(pot_raw[3 * i + 2], p->min_ke, p->max_ke);
        pot_clamped[3 * i] = wc; pot_clamped[3 * i + 1] = ta; pot_clamped[3 * i + 2] = en;
        volatile float a = (float)p->ta_mult * ta, b = (float)p->wc_mult * wc;
        volatile float s = a + b;
        volatile float f = en * s;
        volatile float f2 = f * p->time_step;
        num[i] = (int32_t)floorf(f2);
    }
}

/* counts after the clamps only (the potentials the product reports are clamped) */
void orc_df_counts_from_clamped(const orc_params* p, const float* pot_clamped, uint32_t n, int32_t* num)
{
    for (uint32_t i = 0; i < n; ++i) {
        float wc = pot_clamped[3 * i], ta = pot_clamped[3 * i + 1], en = pot_clamped[3 * i + 2];
        volatile float a = (float)p->ta_mult * ta, b = (float)p->wc_mult * wc;
        volatile float s = a + b;
        volatile float f = en * s;
        volatile float f2 = f * p->time_step;
        num[i] = (int32_t)floorf(f2);
    }
}

/* neighbours within hd of x: squared != 0 compares |s|^2 <= hd^2 (generator),
 * otherwise |s| <= hd (advection); every float32 operation rounded once */
static int count_within(const orc_params* p, const orc_grid* g, const float* spos, const uint32_t* start,
                        const uint32_t* end, const float* x, int squared)
{
    uint32_t lo[3], hi[3];
    dbox(g, x, lo, hi);
    int count = 0;
    for (uint32_t zz = lo[2]; zz <= hi[2]; ++zz)
        for (uint32_t yy = lo[1]; yy <= hi[1]; ++yy)
            for (uint32_t xx = lo[0]; xx <= hi[0]; ++xx) {
                uint32_t c = dlin(g, xx, yy, zz);
                for (uint32_t j = start[c]; j < end[c]; ++j) {
                    const float* pj = spos + 3 * (size_t)j;
                    float s[3];
                    for (int k = 0; k < 3; ++k) { volatile float t = x[k] - pj[k]; s[k] = t; }
                    float d2 = dot_rn3(s, s);
                    if (squared ? (d2 <= p->hd_sq) : (sqrtf(d2) <= p->hd)) ++count;
                }
            }
    return count;
}

static inline int type_of(int d) { return d > D_BUBBLE ? 2 : (d < D_SPRAY ? 0 : 1); }

/* calculateofDiffusePosition + calculateofDiffuseType (:812-999).  num: per
 * sorted particle spawn counts; gen: 8 floats per generated particle
 * (pos, vel, ttl, type), in spawn order.  Returns the generated count. */
uint64_t orc_df_spawn(const orc_params* p, const orc_grid* g, const float* spos, const float* svel, uint32_t n,
                      const uint32_t* start, const uint32_t* end, const int32_t* num, uint64_t seed, uint32_t frame,
                      float* gen)
{
    uint64_t k = 0;
    for (uint32_t i = 0; i < n; ++i) {
        if (num[i] < 1) continue;
        const float* pp = spos + 3 * (size_t)i;
        const float* vv = svel + 3 * (size_t)i;
        double px = pp[0], py = pp[1], pz = pp[2], vx = vv[0], vy = vv[1], vz = vv[2];
        double e1[3];
        if (vv[0] != 0.f) { e1[0] = ((-(0.0 - pz) * vz - (1.0 - py) * vy) / vx) + px; e1[1] = 1; e1[2] = 0; }
        else if (vv[1] != 0.f) { e1[0] = 1; e1[2] = 0; e1[1] = ((-(1.0 - px) * vx - (0.0 - pz) * vz) / vy) + py; }
        else { e1[0] = 1; e1[1] = 0; e1[2] = ((-(1.0 - px) * vx - (0.0 - py) * vy) / vz) + pz; }
        double l = sqrt(e1[0] * e1[0] + e1[1] * e1[1] + e1[2] * e1[2]);
        for (int a = 0; a < 3; ++a) e1[a] /= l;
        double e2[3] = {e1[1] * vz - vy * e1[2], e1[0] * vz - vx * e1[2], e1[0] * vy - vx * e1[1]};
        l = sqrt(e2[0] * e2[0] + e2[1] * e2[1] + e2[2] * e2[2]);
        for (int a = 0; a < 3; ++a) e2[a] /= l;
        int type = type_of(count_within(p, g, spos, start, end, pp, 1));
        for (int c = 0; c < num[i]; ++c, ++k) {
            float u1 = orc_spawn_uniform(seed, frame, 3 * k + 1), u2 = orc_spawn_uniform(seed, frame, 3 * k + 2);
            double r = (double)p->hd * sqrt((double)u1);
            float theta = u2 * 2.0f * D_PI_F;
            double ct = cos((double)theta), st = sin((double)theta);
            float* o = gen + 8 * k;
            o[0] = pp[0]; o[1] = pp[1]; o[2] = pp[2];
            o[3] = (float)(r * ct * e1[0] + r * st * e2[0] + vx);
            o[4] = (float)(r * ct * e1[1] + r * st * e2[1] + vy);
            o[5] = (float)(r * ct * e1[2] + r * st * e2[2] + vz);
            o[6] = (float)(num[i] * p->life_time);
            o[7] = (float)type;
        }
    }
    return k;
}

static inline float wendland(float rx, float ry, float rz, float h)
{
    float r[3] = {rx, ry, rz};
    float mx = sqrtf(dot_rn3(r, r));
    volatile float q = mx / h;
    if (q >= 0.f && q <= 2.f) {
        /* ad and e1 are float variables initialised from double expressions; the
         * product runs in float until the double factor (2q + 1.) */
        volatile float ad = (float)(21.0 / (16.0 * (double)D_PI_F * (double)h * (double)h * (double)h));
        volatile float e1 = (float)(1.0 - ((double)q / 2.0));
        volatile float a = ad * e1;
        volatile float b = a * e1;
        volatile float c = b * e1;
        volatile float d = c * e1;
        return (float)((double)d * ((double)(2.0f * q) + 1.0));
    }
    return 0.f;
}

#define RN(x) ({ volatile float _t = (x); _t; })

/* updateDiffuseParticle (:1001-1199) on records of 8 floats (pos, vel, ttl, type),
 * in place.  bounds: the current frame's spatial grid min + 4.5 spacing, max - 4.5 spacing. */
void orc_df_update(const orc_params* p, const orc_grid* g, const float* spos, const float* svel,
                   const uint32_t* start, const uint32_t* end, float* rec, uint32_t n_old)
{
    const float m = (float)((double)p->particle_spacing * 4.5);
    float lob[3], hib[3];
    for (int k = 0; k < 3; ++k) { lob[k] = g->min_pos[k] + m; hib[k] = g->max_pos[k] - m; }
    const float dt = p->time_step, gz = -9.81f;
    for (uint32_t t = 0; t < n_old; ++t) {
        float* o = rec + 8 * (size_t)t;
        float pos[3] = {o[0], o[1], o[2]}, vel[3] = {o[3], o[4], o[5]};
        int ttl = (int)o[6], type;
        int density = count_within(p, g, spos, start, end, pos, 0);
        float num[3] = {0, 0, 0}, wsum = 0;
        if (density >= D_SPRAY) {
            uint32_t lo[3], hi[3];
            dbox(g, pos, lo, hi);
            for (uint32_t zz = lo[2]; zz <= hi[2]; ++zz)
                for (uint32_t yy = lo[1]; yy <= hi[1]; ++yy)
                    for (uint32_t xx = lo[0]; xx <= hi[0]; ++xx) {
                        uint32_t c = dlin(g, xx, yy, zz);
                        for (uint32_t j = start[c]; j < end[c]; ++j) {
                            const float* pj = spos + 3 * (size_t)j;
                            const float* vj = svel + 3 * (size_t)j;
                            float tv = wendland(RN(pos[0] - pj[0]), RN(pos[1] - pj[1]), RN(pos[2] - pj[2]), p->hd);
                            for (int k = 0; k < 3; ++k) num[k] = RN(num[k] + RN(vj[k] * tv));
                            wsum = RN(wsum + tv);
                        }
                    }
        }
        float nv[3] = {vel[0], vel[1], vel[2]}, np[3] = {pos[0], pos[1], pos[2]};
        if (density < D_SPRAY) {
            nv[0] = RN(nv[0] + RN(0.f * dt));
            nv[1] = RN(nv[1] + RN(0.f * dt));
            nv[2] = RN(nv[2] + RN(gz * dt));
            for (int k = 0; k < 3; ++k) np[k] = RN(np[k] + RN(dt * nv[k]));
        }
        if (density > D_BUBBLE) {
            float gg[3] = {0.f, 0.f, gz};
            for (int k = 0; k < 3; ++k) num[k] = RN(num[k] / wsum);
            for (int k = 0; k < 3; ++k)
                nv[k] = RN(vel[k] + RN(dt * RN(RN(-p->buoyancy * gg[k]) + RN(RN(p->drag * RN(num[k] - vel[k])) / dt))));
            for (int k = 0; k < 3; ++k) np[k] = RN(np[k] + RN(dt * nv[k]));
        }
        if (density <= D_BUBBLE && density >= D_SPRAY) {
            for (int k = 0; k < 3; ++k) num[k] = RN(num[k] / wsum);
            for (int k = 0; k < 3; ++k) { nv[k] = num[k]; np[k] = RN(np[k] + RN(dt * num[k])); }
            ttl -= 1;
        }
        int outside = (np[0] > hib[0] || np[1] > hib[1] || np[2] > hib[2]) || (np[0] < lob[0] || np[1] < lob[1] || np[2] < lob[2]);
        if (outside || ttl <= 0) { type = 3; ttl = 0; }
        else type = type_of(count_within(p, g, spos, start, end, np, 0));
        o[0] = np[0]; o[1] = np[1]; o[2] = np[2];
        o[3] = nv[0]; o[4] = nv[1]; o[5] = nv[2];
        o[6] = (float)ttl; o[7] = (float)type;
    }
}
