// k_diffuse.cu -- diffuse (spray / foam / bubble) particle generation.
//
// Reference: DiffuseGeneration::runsimulation (DiffuseGeneration.cu:89-104,
// 187-442, 760-867) with the kernels of DiffuseGeneration_kernel.cuh:18-118,
// 528-1199 and the helpers of myCuda.cuh:341-401.  Per frame:
//   free-surface particles  = particles of surface cells (:18-118)
//   colour-gradient normals  for particles 0 .. NumFree-1 -- the reference
//                            launches NumFree threads and indexes particles by
//                            thread id, not through the free-surface list
//                            (:528-609, DiffuseGeneration.cu:288-297); kept.
//   trapped air, energy      all particles (:689-761)
//   wave crests              free-surface particles (:611-687)
//   spawn counts             phi clamps, floor(E (kta Ita + kwc WC) dt) (:763-791)
//   spawn                    children sit on the parent, velocity jittered in
//                            the plane normal to v (:812-922)
//   classify                 neighbours within hd: spray < 6 <= foam <= 20 < bubble (:924-999)
//   advect last frame's      gravity / buoyancy-drag / Wendland-averaged fluid
//   diffuse particles        velocity, deletion out of bounds or TTL <= 0 (:1001-1199)
//   delete and append        generated then old, type 3 removed (DiffuseGeneration.cu:760-867)
//
// GB300 design differences: the spawn uniforms come from a counter-based
// generator on the device (seed, frame, index) instead of std::random_device
// on the host plus a host-to-device copy; delete/append and the split by type
// are a device stream compaction instead of a device-host-device round trip;
// a child's type depends only on its parent's position, so it is computed
// once per parent.  Operations that decide integers (thresholds, neighbour
// counts, floor) are rounded one by one so the oracle can mirror them.
#include "pms_internal.h"
#include "k_common.cuh"

#include <cmath>

namespace pms {

static constexpr int kThreads = 128;
static constexpr double kEps = 1.0e-7;          // EPSILON_, Define.h:10 (double)
// The reference compares float values with the double EPSILON_ (and 0.6).  For a
// float x, (double)x > E  <=>  x > down(E) and (double)x < E  <=>  x < up(E), with
// down / up the nearest floats below / above E, so these float constants give the
// same decisions without the FP64 pipe in the neighbour loops.
static constexpr float kEpsDown = 0x1.ad7f28p-24f;   // largest float <= 1e-7
static constexpr float kEpsUp = 0x1.ad7f2ap-24f;     // smallest float >= 1e-7
static constexpr float k06Up = 0x1.333334p-1f;       // smallest float >= 0.6
static constexpr float kPiF = 3.14159265f;      // PI, Define.h:9
static constexpr int kSpray = 6, kBubble = 20;  // SPARY, BUBBLE, Define.h:13-14

struct DiffuseParticle {   // 32 bytes: two float4-aligned halves
    float px, py, pz;
    int ttl;
    float vx, vy, vz;
    int type;
};

struct DiffuseParams {
    float hd, hd_sq, hd_inv, coefficient, mass, time_step, buoyancy, drag;
    float min_wc, max_wc, min_ta, max_ta, min_ke, max_ke;
    int ta_mult, wc_mult, life_time;
    float lo_bound[3], hi_bound[3];    // grid min + 4.5 spacing, grid max - 4.5 spacing
    // exact bounds on a squared distance x for the loops' distance tests (the square
    // root and the division correctly rounded, as the kernels compute them):
    float d2_eps;    // sqrt(x) > EPSILON_     <=>  x > d2_eps
    float d2_hd;     // sqrt(x) <= hd          <=>  x <= d2_hd
    float d2_q1;     // sqrt(x) / hd < 1       <=>  x <= d2_q1
    float w_ad;      // the Wendland kernel's factor 21 / (16 pi hd^3), rounded to float
    uint64_t seed;
    uint32_t frame;
};

// Counts of the delete/append step: given on the host (a single frame: exact, and the
// buffers sized to them) or read from the device and clamped to the buffers'
// capacities (a batched frame, captured into a graph); a count past a capacity sets
// kErrCapacity and the batch runs again with larger buffers.
struct DfN {
    uint32_t gen, old;                 // host counts, or the capacities when read from the device
    const uint32_t* gen_dev;           // generated particles (Counters::n_generated), or null
    const uint32_t* old_dev;           // carried particles, or null
    uint32_t out_cap;                  // capacity of the delete/append output
    uint32_t* err;                     // the frame's error word
};
__device__ __forceinline__ uint32_t df_gen(const DfN& c) { return c.gen_dev ? min(*c.gen_dev, c.gen) : c.gen; }
__device__ __forceinline__ uint32_t df_old(const DfN& c) { return c.old_dev ? min(*c.old_dev, c.old) : c.old; }

// counter-based uniform in [0, 1): splitmix64 finaliser of (seed, frame, index)
__host__ __device__ __forceinline__ float spawn_uniform(uint64_t seed, uint32_t frame, uint64_t idx) {
    uint64_t x = seed * 0x9E3779B97F4A7C15ull + (uint64_t)frame * 0xD1B54A32D192ED03ull + idx;
    x ^= x >> 30; x *= 0xBF58476D1CE4E5B9ull;
    x ^= x >> 27; x *= 0x94D049BB133111EBull;
    x ^= x >> 31;
    // a 24-bit integer times 2^-24: exact in float
    return (float)(uint32_t)(x >> 40) * 0x1p-24f;
}

// a.b with every product and sum rounded on its own (x, y, z order)
__device__ __forceinline__ float dot_rn(float ax, float ay, float az, float bx, float by, float bz) {
    return __fadd_rn(__fadd_rn(__fmul_rn(ax, bx), __fmul_rn(ay, by)), __fmul_rn(az, bz));
}

__device__ __forceinline__ void diffuse_box(const KGrid& g, float x, float y, float z, uint3& lo, uint3& hi) {
    const uint3 c = sp_cell(g, x, y, z);
    box_clamp(g, c, (uint32_t)g.spexpand_diffuse, lo, hi);
}

// ---------------------------------------------------------------------------
// free-surface list and the starting normals
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_df_free(const uint32_t* __restrict__ skeys, const uint2* __restrict__ cell_info,
                                                 const float4* __restrict__ nrm4, int have_surface_normals, uint32_t n,
                                                 uint32_t* __restrict__ isfree, float4* __restrict__ nrm) {
    for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x) {
        const bool surf = (cell_info[skeys[j]].y & 0x80000000u) != 0;
        isfree[j] = surf ? 1u : 0u;
        // the surface pass leaves normals on surface particles; other particles start at zero
        const float4 q = (surf && have_surface_normals) ? nrm4[j] : make_float4(0.f, 0.f, 0.f, 0.f);
        nrm[j] = make_float4(q.x, q.y, q.z, 0.f);
    }
}

__global__ void __launch_bounds__(256) k_df_freelist(const uint32_t* __restrict__ isfree, const uint32_t* __restrict__ scan,
                                                     uint32_t n, uint32_t* __restrict__ list) {
    for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x)
        if (isfree[j]) list[scan[j]] = j;
}

// calculationofNormal: thread t < NumFree computes the normal of particle t
__global__ void __launch_bounds__(kThreads, 8) k_df_normal(KGrid g, DiffuseParams dp, const Counters* __restrict__ cnt,
                                                        const uint32_t* __restrict__ cell_start,
                                                        const float4* __restrict__ spos, uint32_t n,
                                                        float4* __restrict__ nrm) {
    const uint32_t nf = min(cnt->n_free, n);
    const float pad = 1e-4f * g.sp_cs, r2 = dp.hd_sq;
    for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < nf; t += gridDim.x * blockDim.x) {
        const float4 p4 = spos[t];
        const float3 p = make_float3(p4.x, p4.y, p4.z);
        uint3 lo, hi;
        diffuse_box(g, p.x, p.y, p.z, lo, hi);
        hi = make_uint3(hi.x + 1, hi.y + 1, hi.z + 1);
        float nx = 0.f, ny = 0.f, nz = 0.f;
        row_walk(g, p, lo, hi, r2, pad, cell_start, [&](uint32_t j) {
            const float4 q = __ldg(&spos[j]);
            const float sx = p.x - q.x, sy = p.y - q.y, sz = p.z - q.z;
            const float mp2 = sx * sx + sy * sy + sz * sz;
            // q = |s| / hd in (0, 1), decided on |s|^2 before the square root
            if (mp2 > 0.f && mp2 <= dp.d2_q1) {
                const float mp = sqrtf(mp2);
                const float d = dp.hd_sq - mp2;
                const float derivative = d * d * 6.f;
                const float c = dp.coefficient / mp * derivative;
                nx += c * sx; ny += c * sy; nz += c * sz;
            }
        });
        const float mn2 = nx * nx + ny * ny + nz * nz;
        if (mn2 < kEpsUp) continue;              // keeps the previous normal
        const float inv = 1.f / sqrtf(mn2);
        nrm[t] = make_float4(nx * inv, ny * inv, nz * inv, 0.f);
    }
}

// ---------------------------------------------------------------------------
// potentials
// ---------------------------------------------------------------------------
__device__ __forceinline__ float phi_clamp(float I, float tmin, float tmax) {
    return __fdiv_rn(__fsub_rn(fminf(I, tmax), fminf(I, tmin)), __fsub_rn(tmax, tmin));
}

// calculationofTrappedairpotential: every particle.  A particle spawns
// floor(ke (ta_mult TA + wc_mult WC) dt) diffuse particles with ke its clamped kinetic
// energy: where ke clamps to 0 (a particle at rest) the count is 0 whatever its
// trapped air and wave crest, so those walks are skipped and the potentials left 0;
// every count, and so every output, is the reference's.
__global__ void __launch_bounds__(kThreads, 8) k_df_trapped(KGrid g, DiffuseParams dp, const uint32_t* __restrict__ cell_start,
                                                         const float4* __restrict__ spos, const float4* __restrict__ svel,
                                                         uint32_t n, float4* __restrict__ pot) {
    const float pad = 1e-4f * g.sp_cs, r2 = dp.hd_sq;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float4 p4 = spos[i], v = svel[i];
        const float3 p = make_float3(p4.x, p4.y, p4.z);
        // 0.5 * (double)m * (double)|v|^2 rounded to float: the double product of two floats
        // is exact and the halving too, so it is the float product rounded once, halved (the
        // two could differ only for energies below the normal float range, ~1e-38)
        const float ke = 0.5f * __fmul_rn(dp.mass, v.x * v.x + v.y * v.y + v.z * v.z);
        pot[i].z = ke;
        if (phi_clamp(ke, dp.min_ke, dp.max_ke) == 0.f) {
            pot[i].y = 0.f;
            continue;
        }
        uint3 lo, hi;
        diffuse_box(g, p.x, p.y, p.z, lo, hi);
        hi = make_uint3(hi.x + 1, hi.y + 1, hi.z + 1);
        float ita = 0.f;
        row_walk(g, p, lo, hi, r2, pad, cell_start, [&](uint32_t j) {
            const float4 q = __ldg(&spos[j]);
            const float4 w = __ldg(&svel[j]);
            const float sx = p.x - q.x, sy = p.y - q.y, sz = p.z - q.z;
            const float mp2 = sx * sx + sy * sy + sz * sz;
            // EPSILON_ < |s| <= hd, decided on |s|^2 before the square root
            if (mp2 > dp.d2_eps && mp2 <= dp.d2_hd) {
                const float mp = sqrtf(mp2);
                const float ux = v.x - w.x, uy = v.y - w.y, uz = v.z - w.z;
                float mv = ux * ux + uy * uy + uz * uz;
                if (mv > kEpsDown) {
                    mv = sqrtf(mv);
                    // (u/|u|) . (s/|s|) as one quotient: the reference's six divisions
                    // differ from it only in rounding
                    const float e = 1.f - (ux * sx + uy * sy + uz * sz) / (mv * mp);
                    const float wgt = 1.f - mp * dp.hd_inv;
                    ita += mv * e * wgt;
                }
            }
        });
        pot[i].y = ita;
    }
}

// calculationofWavecrests: free-surface particles
__global__ void __launch_bounds__(kThreads, 8) k_df_crests(KGrid g, DiffuseParams dp, const Counters* __restrict__ cnt,
                                                        const uint32_t* __restrict__ freelist,
                                                        const uint32_t* __restrict__ cell_start,
                                                        const float4* __restrict__ spos, const float4* __restrict__ svel,
                                                        const float4* __restrict__ nrm, float4* __restrict__ pot) {
    const uint32_t nf = cnt->n_free;
    const float pad = 1e-4f * g.sp_cs, r2 = dp.hd_sq;
    for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < nf; t += gridDim.x * blockDim.x) {
        const uint32_t i = freelist[t];
        const float4 p4 = spos[i], v = svel[i], ni = nrm[i];
        const float3 p = make_float3(p4.x, p4.y, p4.z);
        const float nn = dot_rn(ni.x, ni.y, ni.z, ni.x, ni.y, ni.z);
        const float vv = dot_rn(v.x, v.y, v.z, v.x, v.y, v.z);
        // the reference's zero cases, and a particle that spawns nothing (its clamped kinetic
        // energy, from the trapped-air pass, is 0)
        if (nn <= kEpsDown || vv <= kEpsDown || dot_rn(v.x, v.y, v.z, ni.x, ni.y, ni.z) < k06Up ||
            phi_clamp(pot[i].z, dp.min_ke, dp.max_ke) == 0.f) {
            pot[i].x = 0.f;
            continue;
        }
        uint3 lo, hi;
        diffuse_box(g, p.x, p.y, p.z, lo, hi);
        hi = make_uint3(hi.x + 1, hi.y + 1, hi.z + 1);
        float wc = 0.f;
        row_walk(g, p, lo, hi, r2, pad, cell_start, [&](uint32_t j) {
            const float4 nj = __ldg(&nrm[j]);
            const float4 q = __ldg(&spos[j]);
            if (dot_rn(nj.x, nj.y, nj.z, nj.x, nj.y, nj.z) <= kEpsDown) return;
            // crests2p: x_ji = normalize(x_j - x_i); counts if x_ji . n_i < -eps
            const float dx = q.x - p.x, dy = q.y - p.y, dz = q.z - p.z;
            const float l2 = dx * dx + dy * dy + dz * dz;
            if (l2 == 0.f) return;                      // normalize(0) is NaN: contributes 0
            if (l2 > dp.d2_hd) return;                  // |x_ij| > hd: the weight below is 0
            const float il = 1.f / sqrtf(l2);
            const float c = (dx * il) * ni.x + (dy * il) * ni.y + (dz * il) * ni.z;
            if (c < -kEpsDown) {
                // curvature2p: (1 - n_i . n_j) * Weend(x_i - x_j, h)
                const float e1 = 1.f - (ni.x * nj.x + ni.y * nj.y + ni.z * nj.z);
                const float mx = sqrtf(l2);
                const float w = (mx <= dp.hd && mx > 0.f) ? __fsub_rn(1.f, mx / dp.hd) : 0.f;   // 1 - q exact in double, then rounded
                wc += e1 * w;
            }
        });
        pot[i].x = wc;
    }
}


// calculateofNumberofdiffuseparticles; key = spawning << 32 | count for one 64-bit scan
__global__ void __launch_bounds__(256) k_df_count(DiffuseParams dp, float4* __restrict__ pot, uint32_t n,
                                                  int32_t* __restrict__ num, unsigned long long* __restrict__ key) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        float4 q = pot[i];
        q.x = phi_clamp(q.x, dp.min_wc, dp.max_wc);
        q.y = phi_clamp(q.y, dp.min_ta, dp.max_ta);
        q.z = phi_clamp(q.z, dp.min_ke, dp.max_ke);
        pot[i] = q;
        const float a = __fmul_rn((float)dp.ta_mult, q.y), b = __fmul_rn((float)dp.wc_mult, q.x);
        const float f = __fmul_rn(__fmul_rn(q.z, __fadd_rn(a, b)), dp.time_step);
        const int k = (int)floorf(f);
        num[i] = k;
        key[i] = k >= 1 ? ((1ull << 32) | (unsigned long long)(uint32_t)k) : 0ull;
    }
}

__global__ void k_df_totals(const unsigned long long* __restrict__ total, Counters* __restrict__ cnt) {
    const unsigned long long t = *total;
    cnt->n_spawning = (uint32_t)(t >> 32);
    cnt->n_generated = (uint32_t)(t & 0xffffffffull);
}

__global__ void __launch_bounds__(256) k_df_spawnlist(const unsigned long long* __restrict__ key,
                                                      const unsigned long long* __restrict__ off, uint32_t n,
                                                      uint32_t* __restrict__ list) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        if (key[i]) list[(uint32_t)(off[i] >> 32)] = i;
}

// Particles with |s|^2 <= hd^2 (the generator's test; calculateofDiffuseType) over the
// diffuse box, walking only the rows and cells of the box that come within hd: a cell
// left out holds no particle the count would take, so the count is the reference's.
__device__ __forceinline__ int count_within_gen(const KGrid& g, const DiffuseParams& dp,
                                                const uint32_t* __restrict__ cell_start, const float4* __restrict__ spos,
                                                float px, float py, float pz) {
    uint3 lo, hi;
    diffuse_box(g, px, py, pz, lo, hi);
    hi = make_uint3(hi.x + 1, hi.y + 1, hi.z + 1);          // row_walk takes [lo, hi)
    const float r = dp.hd * kSupportGrow;
    int count = 0;
    row_walk(g, make_float3(px, py, pz), lo, hi, r * r, 1e-4f * g.sp_cs, cell_start, [&](uint32_t j) {
        const float4 q = __ldg(&spos[j]);
        const float sx = __fsub_rn(px, q.x), sy = __fsub_rn(py, q.y), sz = __fsub_rn(pz, q.z);
        if (dot_rn(sx, sy, sz, sx, sy, sz) <= dp.hd_sq) ++count;
    });
    return count;
}

__device__ __forceinline__ int type_of(int density) { return density > kBubble ? 2 : (density < kSpray ? 0 : 1); }

// calculateofDiffusePosition + calculateofDiffuseType, one spawning parent per thread
__global__ void __launch_bounds__(kThreads, 8) k_df_spawn(KGrid g, DiffuseParams dp, const Counters* __restrict__ cnt,
                                                       const uint32_t* __restrict__ spawnlist,
                                                       const unsigned long long* __restrict__ off,
                                                       const int32_t* __restrict__ num, const uint32_t* __restrict__ cell_start,
                                                       const float4* __restrict__ spos, const float4* __restrict__ svel,
                                                       DiffuseParticle* __restrict__ gen, uint32_t gen_cap,
                                                       const uint32_t* __restrict__ frame_dev, uint32_t frame_off,
                                                       uint32_t* __restrict__ err) {
    const uint32_t ns = cnt->n_spawning;
    // a batched frame reads its number (the batch's first frame plus its place) from the device
    const uint32_t frame = frame_dev ? *frame_dev + frame_off : dp.frame;
    for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < ns; t += gridDim.x * blockDim.x) {
        const uint32_t i = spawnlist[t];
        const float4 p = spos[i], v = svel[i];
        // a vector normal to v (solveEq, myCuda.cuh:385-389), then the second axis
        float e1x, e1y, e1z;
        if (v.x != 0.f) {
            e1x = ((-(0.f - p.z) * v.z - (1.f - p.y) * v.y) / v.x) + p.x; e1y = 1.f; e1z = 0.f;
        } else if (v.y != 0.f) {
            e1x = 1.f; e1z = 0.f; e1y = ((-(1.f - p.x) * v.x - (0.f - p.z) * v.z) / v.y) + p.y;
        } else {
            e1x = 1.f; e1y = 0.f; e1z = ((-(1.f - p.x) * v.x - (0.f - p.y) * v.y) / v.z) + p.z;
        }
        float il = 1.f / sqrtf(e1x * e1x + e1y * e1y + e1z * e1z);
        e1x *= il; e1y *= il; e1z *= il;
        float e2x = e1y * v.z - v.y * e1z, e2y = e1x * v.z - v.x * e1z, e2z = e1x * v.y - v.x * e1y;
        il = 1.f / sqrtf(e2x * e2x + e2y * e2y + e2z * e2z);
        e2x *= il; e2y *= il; e2z *= il;
        const int k = num[i];
        const uint32_t start = (uint32_t)(off[i] & 0xffffffffull);
        const int type = type_of(count_within_gen(g, dp, cell_start, spos, p.x, p.y, p.z));
        for (int c = 0; c < k; ++c) {
            const uint64_t idif = (uint64_t)start + (uint64_t)c;
            const float u1 = spawn_uniform(dp.seed, frame, 3 * idif + 1);
            const float u2 = spawn_uniform(dp.seed, frame, 3 * idif + 2);
            const float r = dp.hd * sqrtf(u1);
            const float theta = u2 * 2.f * kPiF;
            // cos(theta) and sin(theta) of a float theta are the single-precision
            // functions in the reference's device code
            float st, ct;
            sincosf(theta, &st, &ct);
            DiffuseParticle d;
            d.px = p.x; d.py = p.y; d.pz = p.z;      // the reference overwrites the offset position with the parent's
            d.vx = __fadd_rn(__fadd_rn(__fmul_rn(__fmul_rn(r, ct), e1x), __fmul_rn(__fmul_rn(r, st), e2x)), v.x);
            d.vy = __fadd_rn(__fadd_rn(__fmul_rn(__fmul_rn(r, ct), e1y), __fmul_rn(__fmul_rn(r, st), e2y)), v.y);
            d.vz = __fadd_rn(__fadd_rn(__fmul_rn(__fmul_rn(r, ct), e1z), __fmul_rn(__fmul_rn(r, st), e2z)), v.z);
            d.ttl = k * dp.life_time;
            d.type = type;
            if (idif < gen_cap) gen[idif] = d;
            else atomicOr(err, kErrCapacity);
        }
    }
}

// The last factor of Wwendland, (float)((double)d * ((double)t + 1.0)) with d >= 0 and
// t = 2q in [0, 4] floats, without the FP64 pipe (GB300 runs FP64 at a small fraction
// of the FP32 rate, and this runs once per neighbour pair).  r = fma(d, t, d) is the
// exact product P = d (1 + t) rounded once.  The double form rounds P to 53 bits and
// then to 24; the two agree unless the 53-bit rounding lands exactly on a midpoint
// between two floats, which needs P within 2^-53 |P| of that midpoint.  The residual
// P - r is formed exactly from error-free transforms (TwoProduct by fma, Knuth's
// TwoSum) and summed in float (error below 2^-21 ulp(r)); when it lies within
// 2^-18 ulp(r) of half an ulp, or r is not a normal float well above the underflow
// range, the double form is evaluated instead.  For t < 2^-29 the double sum t + 1
// is itself rounded, but then P lies within 2^-29 |d| of the float d, far from any
// midpoint, and both forms return d.
#ifndef __CUDA_ARCH__
// host forms of the rounded operations that no compiler may contract into an fma
static inline float host_mul(float a, float b) { volatile float r = a * b; return r; }
static inline float host_add(float a, float b) { volatile float r = a + b; return r; }
static inline float host_sub(float a, float b) { volatile float r = a - b; return r; }
#endif

__host__ __device__ __forceinline__ float wendland_tail(float d, float t) {
#ifdef __CUDA_ARCH__
#define PMS_FMA(a, b, c) __fmaf_rn(a, b, c)
#define PMS_MUL(a, b) __fmul_rn(a, b)
#define PMS_ADD(a, b) __fadd_rn(a, b)
#define PMS_SUB(a, b) __fsub_rn(a, b)
#else
#define PMS_FMA(a, b, c) std::fma(a, b, c)
#define PMS_MUL(a, b) host_mul(a, b)
#define PMS_ADD(a, b) host_add(a, b)
#define PMS_SUB(a, b) host_sub(a, b)
#endif
    const float r = PMS_FMA(d, t, d);
    const float ph = PMS_MUL(d, t), pl = PMS_FMA(d, t, -ph);          // d t = ph + pl
    const float sm = PMS_ADD(d, ph), bb = PMS_SUB(sm, d);
    const float e = PMS_ADD(PMS_SUB(d, PMS_SUB(sm, bb)), PMS_SUB(ph, bb));   // d + ph = sm + e
    const float eps = PMS_ADD(PMS_ADD(PMS_SUB(sm, r), e), pl);              // P - r
    uint32_t rb;
    memcpy(&rb, &r, 4);
    const uint32_t ex = (rb >> 23) & 0xffu;
    bool exact_enough = ex >= 40u && ex < 255u && d >= 1.0e-30f;
    if (exact_enough) {
        const uint32_t hb = (ex - 24u) << 23;                            // half an ulp of r
        float half;
        memcpy(&half, &hb, 4);
        const float gap = PMS_SUB(eps < 0.f ? -eps : eps, half);
        exact_enough = (gap < 0.f ? -gap : gap) > PMS_MUL(half, 0x1p-17f);
    }
#undef PMS_FMA
#undef PMS_MUL
#undef PMS_ADD
#undef PMS_SUB
    return exact_enough ? r : (float)((double)d * ((double)t + 1.0));
}

// Wwendland, myCuda.cuh:391-401: ad and e1 are float variables set from double
// expressions; ad*e1^4 runs in float, the last factor (2q + 1.) in double.  ad is a
// constant of the frame (dp.w_ad, the same double expression evaluated on the host).
// e1 = (float)(1.0 - q/2.0) is computed in float: for q in [0, 2] the double
// difference is exact whenever q/2 >= 2^-30, and below that both forms give 1.0f, so
// the one float rounding is the double form's.
__device__ __forceinline__ float wendland(float rx, float ry, float rz, float h, float ad) {
    const float mx = __fsqrt_rn(dot_rn(rx, ry, rz, rx, ry, rz));
    const float q = __fdiv_rn(mx, h);
    if (q >= 0.f && q <= 2.f) {
        const float e1 = __fsub_rn(1.f, __fmul_rn(q, 0.5f));
        const float d = __fmul_rn(__fmul_rn(__fmul_rn(__fmul_rn(ad, e1), e1), e1), e1);
        return wendland_tail(d, __fmul_rn(2.0f, q));
    }
    return 0.f;
}

// The previous frame's particles grouped by their type (spray, foam, bubble; each
// group in stored order), as a permutation: spray particles in air walk almost
// empty cells while foam and bubbles walk dense ones, and a warp that mixes them
// runs at the pace of its slowest lane.  The particles stay where they are (the
// live set keeps the reference's generated-then-old order).
__global__ void __launch_bounds__(256) k_df_type_keys(const DiffuseParticle* __restrict__ old, DfN dn,
                                                      unsigned long long* __restrict__ key) {
    const uint32_t n_old = df_old(dn);
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n_old; i += gridDim.x * blockDim.x) {
        const int t = old[i].type;
        key[i] = t == 0 ? 1ull : (t == 1 ? (1ull << 32) : 0ull);
    }
}

__global__ void __launch_bounds__(256) k_df_type_perm(const unsigned long long* __restrict__ key,
                                                      const unsigned long long* __restrict__ scan,
                                                      const unsigned long long* __restrict__ total, DfN dn,
                                                      uint32_t* __restrict__ perm) {
    const uint32_t n_old = df_old(dn);
    const unsigned long long tot = *total;
    const uint32_t n0 = (uint32_t)(tot & 0xffffffffull), n1 = (uint32_t)(tot >> 32);
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n_old; i += gridDim.x * blockDim.x) {
        const unsigned long long k = key[i], sc = scan[i];
        const uint32_t s0 = (uint32_t)(sc & 0xffffffffull), s1 = (uint32_t)(sc >> 32);
        const uint32_t dest = (k & 1ull) ? s0 : (k ? n0 + s1 : n0 + n1 + (i - s0 - s1));
        perm[dest] = i;
    }
}

// Neighbours of x within hd (|s| <= hd, the advection's test), walking only the rows
// and cells of the diffuse box that come within hd of x: a cell left out holds no
// particle that the count would take, so the count is the reference's.
__device__ __forceinline__ int count_within_near(const KGrid& g, const DiffuseParams& dp,
                                                 const uint32_t* __restrict__ cell_start, const float4* __restrict__ spos,
                                                 float px, float py, float pz) {
    uint3 lo, hi;
    diffuse_box(g, px, py, pz, lo, hi);
    hi = make_uint3(hi.x + 1, hi.y + 1, hi.z + 1);          // row_walk takes [lo, hi)
    const float r = dp.hd * kSupportGrow;
    int count = 0;
    row_walk(g, make_float3(px, py, pz), lo, hi, r * r, 1e-4f * g.sp_cs, cell_start, [&](uint32_t j) {
        const float4 q = __ldg(&spos[j]);
        const float sx = __fsub_rn(px, q.x), sy = __fsub_rn(py, q.y), sz = __fsub_rn(pz, q.z);
        if (dot_rn(sx, sy, sz, sx, sy, sz) <= dp.d2_hd) ++count;   // |s| <= hd
    });
    return count;
}

// updateDiffuseParticle (DiffuseGeneration_kernel.cuh:1036-1199), one diffuse
// particle of the previous frame per thread.  The reference walks its cell box
// three times (neighbour count, velocity average, neighbour count at the new
// position); here the first two share one walk over the rows and cells within
// 2 hd (the Wendland support: every particle farther adds exactly 0 to the
// average, every particle the count takes lies within hd), in the reference's
// cell and particle order, and the last walk covers only what lies within hd.
__global__ void __launch_bounds__(kThreads, 8) k_df_update(KGrid g, DiffuseParams dp, DfN dn,
                                                        const uint32_t* __restrict__ cell_start,
                                                        const float4* __restrict__ spos,
                                                        const float4* __restrict__ svel, const uint32_t* __restrict__ perm,
                                                        DiffuseParticle* __restrict__ old) {
    const uint32_t n_old = df_old(dn);
    for (uint32_t tt = blockIdx.x * blockDim.x + threadIdx.x; tt < n_old; tt += gridDim.x * blockDim.x) {
        const uint32_t t = perm[tt];
        DiffuseParticle d = old[t];
        const float px = d.px, py = d.py, pz = d.pz, vx = d.vx, vy = d.vy, vz = d.vz;
        // a particle that was spray last frame most likely still is, and spray moves with
        // gravity alone: its neighbours within hd are counted first, and the walk over
        // 2 hd that the velocity average needs runs only when that count says foam or
        // bubble (then it counts again, the same particles in the same order)
        int density = d.type == 0 ? count_within_near(g, dp, cell_start, spos, px, py, pz) : kSpray;
        float nx = 0.f, ny = 0.f, nz = 0.f, wsum = 0.f;
        if (density >= kSpray) {
            density = 0;
            uint3 lo, hi;
            diffuse_box(g, px, py, pz, lo, hi);
            hi = make_uint3(hi.x + 1, hi.y + 1, hi.z + 1);
            const float r = 2.f * dp.hd * kSupportGrow;
            row_walk(g, make_float3(px, py, pz), lo, hi, r * r, 1e-4f * g.sp_cs, cell_start, [&](uint32_t j) {
                const float4 q = __ldg(&spos[j]);
                const float sx = __fsub_rn(px, q.x), sy = __fsub_rn(py, q.y), sz = __fsub_rn(pz, q.z);
                if (dot_rn(sx, sy, sz, sx, sy, sz) <= dp.d2_hd) ++density;   // |s| <= hd
                const float4 w = __ldg(&svel[j]);
                const float tv = wendland(sx, sy, sz, dp.hd, dp.w_ad);
                nx = __fadd_rn(nx, __fmul_rn(w.x, tv));
                ny = __fadd_rn(ny, __fmul_rn(w.y, tv));
                nz = __fadd_rn(nz, __fmul_rn(w.z, tv));
                wsum = __fadd_rn(wsum, tv);
            });
        }
        const float gz = -9.81f, dt = dp.time_step;
        if (density < kSpray) {
            d.vx = __fadd_rn(d.vx, __fmul_rn(0.f, dt));
            d.vy = __fadd_rn(d.vy, __fmul_rn(0.f, dt));
            d.vz = __fadd_rn(d.vz, __fmul_rn(gz, dt));
            d.px = __fadd_rn(d.px, __fmul_rn(dt, d.vx));
            d.py = __fadd_rn(d.py, __fmul_rn(dt, d.vy));
            d.pz = __fadd_rn(d.pz, __fmul_rn(dt, d.vz));
        }
        if (density > kBubble) {
            nx = __fdiv_rn(nx, wsum); ny = __fdiv_rn(ny, wsum); nz = __fdiv_rn(nz, wsum);
            // vel + dt * (-buoyancy * g + drag * (num - vel) / dt), per component
            d.vx = __fadd_rn(vx, __fmul_rn(dt, __fadd_rn(__fmul_rn(-dp.buoyancy, 0.f), __fdiv_rn(__fmul_rn(dp.drag, __fsub_rn(nx, vx)), dt))));
            d.vz = __fadd_rn(vz, __fmul_rn(dt, __fadd_rn(__fmul_rn(-dp.buoyancy, gz), __fdiv_rn(__fmul_rn(dp.drag, __fsub_rn(nz, vz)), dt))));
            d.vy = __fadd_rn(vy, __fmul_rn(dt, __fadd_rn(__fmul_rn(-dp.buoyancy, 0.f), __fdiv_rn(__fmul_rn(dp.drag, __fsub_rn(ny, vy)), dt))));
            d.px = __fadd_rn(d.px, __fmul_rn(dt, d.vx));
            d.py = __fadd_rn(d.py, __fmul_rn(dt, d.vy));
            d.pz = __fadd_rn(d.pz, __fmul_rn(dt, d.vz));
        }
        if (density <= kBubble && density >= kSpray) {
            nx = __fdiv_rn(nx, wsum); ny = __fdiv_rn(ny, wsum); nz = __fdiv_rn(nz, wsum);
            d.vx = nx; d.vy = ny; d.vz = nz;
            d.px = __fadd_rn(d.px, __fmul_rn(dt, nx));
            d.py = __fadd_rn(d.py, __fmul_rn(dt, ny));
            d.pz = __fadd_rn(d.pz, __fmul_rn(dt, nz));
            d.ttl -= 1;
        }
        const bool outside = (d.px > dp.hi_bound[0] || d.py > dp.hi_bound[1] || d.pz > dp.hi_bound[2]) ||
                             (d.px < dp.lo_bound[0] || d.py < dp.lo_bound[1] || d.pz < dp.lo_bound[2]);
        if (outside || d.ttl <= 0) {
            d.type = 3;
            d.ttl = 0;
        } else {
            d.type = type_of(count_within_near(g, dp, cell_start, spos, d.px, d.py, d.pz));
        }
        old[t] = d;
    }
}

// delete and append: generated then old, dropping type 3; per-type counts (summed per
// thread, then per warp, one atomic per warp and type)
__global__ void __launch_bounds__(256) k_df_keep(const DiffuseParticle* __restrict__ gen,
                                                 const DiffuseParticle* __restrict__ old, DfN dn,
                                                 uint32_t* __restrict__ keep, Counters* __restrict__ cnt) {
    const uint32_t n_gen = df_gen(dn), total = n_gen + df_old(dn);
    uint32_t c[4] = {0u, 0u, 0u, 0u};
    for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < total; k += gridDim.x * blockDim.x) {
        const int type = k < n_gen ? gen[k].type : old[k - n_gen].type;
        keep[k] = type != 3 ? 1u : 0u;
        c[type == 0 ? 0 : (type == 2 ? 2 : (type == 3 ? 3 : 1))]++;
    }
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const uint32_t w = __reduce_add_sync(0xffffffffu, c[i]);
        if ((threadIdx.x & 31u) == 0 && w) atomicAdd(&cnt->n_type[i], w);
    }
}

__global__ void __launch_bounds__(256) k_df_append(const DiffuseParticle* __restrict__ gen,
                                                   const DiffuseParticle* __restrict__ old, DfN dn,
                                                   const uint32_t* __restrict__ keep, const uint32_t* __restrict__ scan,
                                                   DiffuseParticle* __restrict__ out) {
    const uint32_t n_gen = df_gen(dn), total = n_gen + df_old(dn);
    for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < total; k += gridDim.x * blockDim.x)
        if (keep[k]) {
            const uint32_t dest = scan[k];
            if (dest < dn.out_cap) out[dest] = k < n_gen ? gen[k] : old[k - n_gen];
            else atomicOr(dn.err, kErrCapacity);
        }
}

// A batched frame's counts before delete/append: the carried count clamped to its
// buffer and the step's total (generated + carried).
__global__ void k_df_frame_counts(const uint32_t* __restrict__ old_dev, uint32_t old_cap, uint32_t gen_cap,
                                  Counters* __restrict__ cnt) {
    const uint32_t o = *old_dev, gnr = cnt->n_generated;
    cnt->n_old = min(o, old_cap);
    cnt->n_df_total = min(o, old_cap) + min(gnr, gen_cap);
    if (o > old_cap || gnr > gen_cap) atomicOr(&cnt->err, kErrCapacity);
}

// A batched frame's survivors: their count becomes the next frame's carried count and
// they take the next stretch of the batch's diffuse arena.
__global__ void k_df_carry(const Counters* __restrict__ cnt, uint32_t out_cap, uint32_t* __restrict__ old_dev,
                           unsigned long long* __restrict__ running, unsigned long long* __restrict__ base) {
    const uint32_t live = min(cnt->n_live, out_cap);
    *old_dev = live;
    *base = *running;
    *running += live;
}

__global__ void __launch_bounds__(256) k_df_export(const DiffuseParticle* __restrict__ live,
                                                   const uint32_t* __restrict__ n_dev,
                                                   const unsigned long long* __restrict__ base, uint64_t cap,
                                                   DiffuseParticle* __restrict__ arena, uint32_t* __restrict__ err) {
    const uint32_t n = *n_dev;
    const unsigned long long b = *base;
    for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        if (b + k < cap) arena[b + k] = live[k];
        else if (k == 0 || b + k == cap) atomicOr(err, kErrCapacity);
    }
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
// The largest float x >= 0 for which ok(x) holds, ok true up to some bound and
// false beyond it (monotone), searched from a nearby start.
template <class Ok>
static float largest_float_where(float start, Ok ok) {
    float x = start;
    while (x > 0.f && !ok(x)) x = std::nextafter(x, 0.f);
    while (ok(std::nextafter(x, INFINITY))) x = std::nextafter(x, INFINITY);
    return x;
}

static DiffuseParams diffuse_params(const pms_ctx* ctx) {
    const pms_params& P = ctx->prm;
    DiffuseParams d;
    d.hd = P.hd; d.hd_sq = P.hd_sq; d.hd_inv = 1.f / P.hd; d.coefficient = P.coefficient; d.mass = P.mass; d.time_step = P.time_step;
    d.buoyancy = P.buoyancy; d.drag = P.drag;
    d.min_wc = P.min_wc; d.max_wc = P.max_wc; d.min_ta = P.min_ta; d.max_ta = P.max_ta;
    d.min_ke = P.min_ke; d.max_ke = P.max_ke;
    d.ta_mult = P.ta_mult; d.wc_mult = P.wc_mult; d.life_time = P.life_time;
    // dGridParams.maxPos - particleSpacing * 4.5 (a double product passed as float)
    const float m = (float)((double)P.particle_spacing * 4.5);
    for (int k = 0; k < 3; ++k) { d.lo_bound[k] = ctx->grid.min_pos[k] + m; d.hi_bound[k] = ctx->grid.max_pos[k] - m; }
    d.d2_eps = largest_float_where(kEpsDown * kEpsDown, [](float x) { return std::sqrt(x) <= kEpsDown; });
    d.d2_hd = largest_float_where(d.hd * d.hd, [&](float x) { return std::sqrt(x) <= d.hd; });
    d.d2_q1 = largest_float_where(d.hd * d.hd, [&](float x) { return std::sqrt(x) / d.hd < 1.f; });
    d.w_ad = (float)(21.0 / (16.0 * (double)kPiF * (double)d.hd * (double)d.hd * (double)d.hd));
    d.seed = ctx->cfg.rng_seed;
    d.frame = ctx->frame_index;
    return d;
}

// Potentials, spawn counts and the spawn list of a frame: sizes from the frame's
// particle count (on the host for single and batched frames alike).
static pms_status diffuse_front(pms_ctx* ctx, const KGrid& g, const DiffuseParams& dp, Counters* cnt) {
    const uint32_t n = ctx->n;
    const size_t N = n;
    pms_status st;
    PMS_CUDA(ctx, ctx->d_isfree.ensure(4 * N));
    PMS_CUDA(ctx, ctx->d_freescan.ensure(4 * N));
    PMS_CUDA(ctx, ctx->d_freelist.ensure(4 * N));
    PMS_CUDA(ctx, ctx->d_nrm_free.ensure(16 * N));
    PMS_CUDA(ctx, ctx->d_pot.ensure(16 * N));
    PMS_CUDA(ctx, ctx->d_num.ensure(4 * N));
    PMS_CUDA(ctx, ctx->d_isdiff.ensure(8 * N));      // 64-bit spawn keys
    PMS_CUDA(ctx, ctx->d_isdiffscan.ensure(8 * N));
    PMS_CUDA(ctx, ctx->d_difflist.ensure(4 * N));
    const unsigned gb = grid_for(n, 256), gk = grid_for(n, kThreads);
    k_df_free<<<gb, 256, 0, ctx->stream>>>(ctx->skeys.as<uint32_t>(), ctx->cell_info.as<uint2>(), ctx->nrm4.as<float4>(),
                                           ctx->have_aniso ? 1 : 0, n, ctx->d_isfree.as<uint32_t>(), ctx->d_nrm_free.as<float4>());
    PMS_LAUNCHED(ctx);
    if ((st = scan_u32(ctx, ctx->d_isfree.as<uint32_t>(), ctx->d_freescan.as<uint32_t>(), n, &cnt->n_free))) return st;
    k_df_freelist<<<gb, 256, 0, ctx->stream>>>(ctx->d_isfree.as<uint32_t>(), ctx->d_freescan.as<uint32_t>(), n,
                                               ctx->d_freelist.as<uint32_t>());
    PMS_LAUNCHED(ctx);
    k_df_normal<<<gk, kThreads, 0, ctx->stream>>>(g, dp, cnt, ctx->cell_start.as<uint32_t>(), ctx->spos.as<float4>(), n,
                                                  ctx->d_nrm_free.as<float4>());
    PMS_LAUNCHED(ctx);
    PMS_CUDA(ctx, cudaMemsetAsync(ctx->d_pot.p, 0, 16 * N, ctx->stream));
    k_df_trapped<<<gk, kThreads, 0, ctx->stream>>>(g, dp, ctx->cell_start.as<uint32_t>(), ctx->spos.as<float4>(),
                                                   ctx->svel.as<float4>(), n, ctx->d_pot.as<float4>());
    PMS_LAUNCHED(ctx);
    k_df_crests<<<gk, kThreads, 0, ctx->stream>>>(g, dp, cnt, ctx->d_freelist.as<uint32_t>(), ctx->cell_start.as<uint32_t>(),
                                                  ctx->spos.as<float4>(), ctx->svel.as<float4>(),
                                                  ctx->d_nrm_free.as<float4>(), ctx->d_pot.as<float4>());
    PMS_LAUNCHED(ctx);
    k_df_count<<<gb, 256, 0, ctx->stream>>>(dp, ctx->d_pot.as<float4>(), n, ctx->d_num.as<int32_t>(),
                                            ctx->d_isdiff.as<unsigned long long>());
    PMS_LAUNCHED(ctx);
    if ((st = scan_u64(ctx, ctx->d_isdiff.as<unsigned long long>(), ctx->d_isdiffscan.as<unsigned long long>(), n,
                       ctx->tmp.as<unsigned long long>())))
        return st;
    k_df_totals<<<1, 1, 0, ctx->stream>>>(ctx->tmp.as<unsigned long long>(), cnt);
    PMS_LAUNCHED(ctx);
    k_df_spawnlist<<<gb, 256, 0, ctx->stream>>>(ctx->d_isdiff.as<unsigned long long>(),
                                                ctx->d_isdiffscan.as<unsigned long long>(), n, ctx->d_difflist.as<uint32_t>());
    PMS_LAUNCHED(ctx);
    return PMS_OK;
}

// Spawn, the carried particles' update and delete/append.  Single frames pass the exact
// counts (dn.gen_dev, dn.old_dev null), batched frames the capacities and device counts;
// launch grids follow the host values, kernels stop at the device counts.
static pms_status diffuse_tail(pms_ctx* ctx, const KGrid& g, const DiffuseParams& dp, Counters* cnt, const DfN& dn,
                               uint32_t spawn_bound, const uint32_t* frame_dev, uint32_t frame_off, uint32_t* live_out) {
    pms_status st;
    const uint32_t total = dn.gen + dn.old;
    if (spawn_bound)
        k_df_spawn<<<grid_for(spawn_bound, kThreads), kThreads, 0, ctx->stream>>>(
            g, dp, cnt, ctx->d_difflist.as<uint32_t>(), ctx->d_isdiffscan.as<unsigned long long>(), ctx->d_num.as<int32_t>(),
            ctx->cell_start.as<uint32_t>(), ctx->spos.as<float4>(), ctx->svel.as<float4>(), ctx->d_gen.as<DiffuseParticle>(),
            dn.gen, frame_dev, frame_off, &cnt->err);
    if (spawn_bound) PMS_LAUNCHED(ctx);
    if (dn.old) {
        const unsigned go = grid_for(dn.old, 256);
        k_df_type_keys<<<go, 256, 0, ctx->stream>>>(ctx->d_old.as<DiffuseParticle>(), dn, ctx->d_tkey.as<unsigned long long>());
        PMS_LAUNCHED(ctx);
        if ((st = scan_u64(ctx, ctx->d_tkey.as<unsigned long long>(), ctx->d_tscan.as<unsigned long long>(), dn.old,
                           ctx->tmp.as<unsigned long long>(), dn.old_dev ? &cnt->n_old : nullptr)))
            return st;
        k_df_type_perm<<<go, 256, 0, ctx->stream>>>(ctx->d_tkey.as<unsigned long long>(),
                                                    ctx->d_tscan.as<unsigned long long>(),
                                                    ctx->tmp.as<unsigned long long>(), dn, ctx->d_perm.as<uint32_t>());
        PMS_LAUNCHED(ctx);
        k_df_update<<<grid_for(dn.old, kThreads), kThreads, 0, ctx->stream>>>(
            g, dp, dn, ctx->cell_start.as<uint32_t>(), ctx->spos.as<float4>(), ctx->svel.as<float4>(),
            ctx->d_perm.as<uint32_t>(), ctx->d_old.as<DiffuseParticle>());
        PMS_LAUNCHED(ctx);
    }
    uint32_t* keep = ctx->d_typescan.as<uint32_t>();
    uint32_t* kscan = keep + (total ? total : 1);
    if (total) {
        k_df_keep<<<grid_for(total, 256), 256, 0, ctx->stream>>>(ctx->d_gen.as<DiffuseParticle>(),
                                                                 ctx->d_old.as<DiffuseParticle>(), dn, keep, cnt);
        PMS_LAUNCHED(ctx);
        if ((st = scan_u32(ctx, keep, kscan, total, live_out, dn.gen_dev ? &cnt->n_df_total : nullptr))) return st;
        k_df_append<<<grid_for(total, 256), 256, 0, ctx->stream>>>(ctx->d_gen.as<DiffuseParticle>(),
                                                                   ctx->d_old.as<DiffuseParticle>(), dn, keep, kscan,
                                                                   ctx->d_all.as<DiffuseParticle>());
        PMS_LAUNCHED(ctx);
    } else {
        PMS_CUDA(ctx, cudaMemsetAsync(live_out, 0, sizeof(uint32_t), ctx->stream));
    }
    return PMS_OK;
}

// The single-frame diffuse stage in three parts, each with at most one host
// synchronisation, at its start: the front (free surface, potentials, spawn counts),
// the tail (spawn, update, delete/append) once the counts are on the host, and the
// finish (the live count, the streamed copy).  A frame with surface reconstruction
// runs the parts on a stream of their own between the surface stages.
pms_status diffuse_part_front(pms_ctx* ctx) {
    ctx->df_run = ctx->n != 0;
    if (!ctx->df_run) { ctx->diffuse_old = 0; return PMS_OK; }
    const KGrid g = kgrid_of(ctx->grid);
    const DiffuseParams dp = diffuse_params(ctx);
    Counters* cnt = ctx->counters.as<Counters>();
    pms_status st;
    if (!ctx->have_aniso && (st = launch_surface_cells(ctx))) return st;
    // earlier frames' live particles (moved in place below) may still be on their way to the host
    PMS_CHECK(out_device_wait(ctx, ctx->diffuse_q));
    return diffuse_front(ctx, g, dp, cnt);
}

pms_status diffuse_part_tail(pms_ctx* ctx) {
    if (!ctx->df_run) return PMS_OK;
    const KGrid g = kgrid_of(ctx->grid);
    const DiffuseParams dp = diffuse_params(ctx);
    Counters* cnt = ctx->counters.as<Counters>();
    pms_status st;
    if ((st = sync_counters(ctx))) return st;
    const uint32_t n_gen = ctx->h_counters->n_generated, n_spawn = ctx->h_counters->n_spawning;
    const uint32_t n_old = ctx->diffuse_old;
    const size_t total = (size_t)n_gen + n_old;
    ctx->df_total = total;
    PMS_CUDA(ctx, ctx->d_gen.ensure_grow(sizeof(DiffuseParticle) * (n_gen ? n_gen : 1)));
    PMS_CUDA(ctx, ctx->d_all.ensure_grow(sizeof(DiffuseParticle) * (total ? total : 1)));
    PMS_CUDA(ctx, ctx->d_typescan.ensure_grow(8 * (total ? total : 1)));
    if (n_old) {
        PMS_CUDA(ctx, ctx->d_tkey.ensure_grow(8 * (size_t)n_old));
        PMS_CUDA(ctx, ctx->d_tscan.ensure_grow(8 * (size_t)n_old));
        PMS_CUDA(ctx, ctx->d_perm.ensure_grow(4 * (size_t)n_old));
    }
    const DfN dn = {n_gen, n_old, nullptr, nullptr, (uint32_t)(total ? total : 1), &cnt->err};
    return diffuse_tail(ctx, g, dp, cnt, dn, n_spawn, nullptr, 0, &cnt->n_live);
}

pms_status diffuse_part_finish(pms_ctx* ctx) {
    if (!ctx->df_run) return PMS_OK;
    pms_status st;
    if ((st = sync_counters(ctx))) return st;
    ctx->diffuse_old = ctx->df_total ? ctx->h_counters->n_live : 0;
    std::swap(ctx->d_all, ctx->d_old);               // the survivors are next frame's old particles
    if (ctx->dout) {
        // the live set to the registered host buffer, on the copy stream
        int slot;
        PMS_CHECK(out_begin(ctx, ctx->diffuse_q, ctx->dout, &slot));
        const uint64_t m = ctx->diffuse_old;
        PMS_CUDA(ctx, cudaEventRecord(ctx->diffuse_ready, ctx->stream));
        PMS_CUDA(ctx, cudaStreamWaitEvent(ctx->copy_stream, ctx->diffuse_ready, 0));
        if (m && m <= ctx->dout_cap)
            PMS_CUDA(ctx, cudaMemcpyAsync(ctx->dout, ctx->d_old.p, sizeof(DiffuseParticle) * m, cudaMemcpyDeviceToHost,
                                          ctx->copy_stream));
        PMS_CUDA(ctx, cudaEventRecord(ctx->diffuse_q.ev[slot], ctx->copy_stream));
        out_push(ctx->diffuse_q, slot, ctx->dout, m, ctx->dout_cap);
    }
    return PMS_OK;
}

pms_status launch_diffuse(pms_ctx* ctx) {
    PMS_CHECK(diffuse_part_front(ctx));
    PMS_CHECK(diffuse_part_tail(ctx));
    return diffuse_part_finish(ctx);
}

// every buffer of a batched frame's diffuse stage, for frames of up to nmax particles
pms_status ensure_diffuse_batch_buffers(pms_ctx* ctx, uint32_t nmax, uint32_t gen_cap, uint32_t old_cap) {
    const size_t N = nmax ? nmax : 1, G = gen_cap ? gen_cap : 1, O = old_cap ? old_cap : 1;
    for (DBuf* b : {&ctx->d_isfree, &ctx->d_freescan, &ctx->d_freelist, &ctx->d_num, &ctx->d_difflist})
        PMS_CUDA(ctx, b->ensure(4 * N));
    for (DBuf* b : {&ctx->d_nrm_free, &ctx->d_pot}) PMS_CUDA(ctx, b->ensure(16 * N));
    for (DBuf* b : {&ctx->d_isdiff, &ctx->d_isdiffscan}) PMS_CUDA(ctx, b->ensure(8 * N));
    PMS_CUDA(ctx, ctx->d_gen.ensure(sizeof(DiffuseParticle) * G));
    PMS_CUDA(ctx, ctx->d_all.ensure(sizeof(DiffuseParticle) * O));
    PMS_CUDA(ctx, ctx->d_old.ensure(sizeof(DiffuseParticle) * O));
    PMS_CUDA(ctx, ctx->d_typescan.ensure(8 * (G + O)));
    PMS_CUDA(ctx, ctx->d_tkey.ensure(8 * O));
    PMS_CUDA(ctx, ctx->d_tscan.ensure(8 * O));
    PMS_CUDA(ctx, ctx->d_perm.ensure(4 * O));
    return PMS_OK;
}

pms_status launch_diffuse_bounded(pms_ctx* ctx, const DiffuseBatch& db) {
    const uint32_t n = ctx->n;
    const KGrid g = kgrid_of(ctx->grid);
    const DiffuseParams dp = diffuse_params(ctx);
    Counters* cnt = ctx->counters.as<Counters>();
    pms_status st;
    if (n && (st = diffuse_front(ctx, g, dp, cnt))) return st;
    if (!n) PMS_CUDA(ctx, cudaMemsetAsync(&cnt->n_generated, 0, sizeof(uint32_t), ctx->stream));
    k_df_frame_counts<<<1, 1, 0, ctx->stream>>>(db.old_dev, db.old_cap, db.gen_cap, cnt);
    PMS_LAUNCHED(ctx);
    const DfN dn = {db.gen_cap, db.old_cap, &cnt->n_generated, &cnt->n_old, db.old_cap, &cnt->err};
    if ((st = diffuse_tail(ctx, g, dp, cnt, dn, n, db.frame_dev, db.frame_off, &cnt->n_live))) return st;
    std::swap(ctx->d_all, ctx->d_old);               // at capture: the next frame reads this frame's survivors
    k_df_carry<<<1, 1, 0, ctx->stream>>>(cnt, db.old_cap, db.old_dev, db.running, db.base);
    PMS_LAUNCHED(ctx);
    k_df_export<<<grid_for(db.old_cap, 256), 256, 0, ctx->stream>>>(ctx->d_old.as<DiffuseParticle>(), db.old_dev, db.base,
                                                                     db.arena_cap, static_cast<DiffuseParticle*>(db.arena),
                                                                     &cnt->err);
    PMS_LAUNCHED(ctx);
    return PMS_OK;
}

}  // namespace pms

using pms::DiffuseParticle;

pms_status pms::diffuse_debug(pms_ctx* ctx, int id, std::vector<uint8_t>& out) {
    if (!ctx->have_diffuse) return pms_fail(ctx, PMS_ERR_STATE, "no diffuse stage yet");
    const size_t n = ctx->n;
    const DBuf* src = nullptr;
    size_t bytes = 0;
    switch (id) {
        case PMS_ARRAY_DIFFUSE_POTENTIAL: src = &ctx->d_pot; bytes = 16 * n; break;
        case PMS_ARRAY_DIFFUSE_COUNT: src = &ctx->d_num; bytes = 4 * n; break;
        case PMS_ARRAY_FREE_NORMAL: src = &ctx->d_nrm_free; bytes = 16 * n; break;
        default: return pms_fail(ctx, PMS_ERR_INVALID_ARGUMENT, "unknown array id %d", id);
    }
    std::vector<uint8_t> raw(bytes);
    PMS_CUDA(ctx, cudaMemcpyAsync(raw.data(), src->p, bytes, cudaMemcpyDeviceToHost, ctx->stream));
    PMS_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    if (id == PMS_ARRAY_DIFFUSE_COUNT) { out.swap(raw); return PMS_OK; }
    // float4 -> xyz
    out.resize(12 * n);
    for (size_t i = 0; i < n; ++i) memcpy(out.data() + 12 * i, raw.data() + 16 * i, 12);
    return PMS_OK;
}

static pms_status download_live(pms_ctx* ctx, std::vector<DiffuseParticle>& v) {
    v.resize(ctx->diffuse_old);
    if (!v.empty())
        PMS_CUDA(ctx, cudaMemcpyAsync(v.data(), ctx->d_old.p, sizeof(DiffuseParticle) * v.size(), cudaMemcpyDeviceToHost,
                                      ctx->stream));
    PMS_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return PMS_OK;
}

static_assert(sizeof(DiffuseParticle) == sizeof(pms_diffuse_particle), "diffuse particle layout");

extern "C" pms_status pms_stream_diffuse_to_host(pms_ctx* ctx, pms_diffuse_particle* out, uint64_t cap) {
    if (!ctx) return PMS_ERR_INVALID_ARGUMENT;
    cudaSetDevice(ctx->device);
    // frames already on their way keep their own buffers
    if (out) PMS_CHECK(pms::copy_stream_ready(ctx));
    ctx->dout = out;
    ctx->dout_cap = out ? cap : 0;
    return PMS_OK;
}

extern "C" pms_status pms_wait_diffuse(pms_ctx* ctx, uint64_t* n) {
    if (!ctx) return PMS_ERR_INVALID_ARGUMENT;
    if (!ctx->diffuse_q.count) return pms_fail(ctx, PMS_ERR_STATE, "no diffuse particles streamed since the last wait");
    cudaSetDevice(ctx->device);
    uint64_t m = 0, cap = 0;
    bool overflow = false;
    PMS_CHECK(pms::out_wait(ctx, ctx->diffuse_q, &m, &overflow, &cap));
    if (n) *n = m;
    if (overflow)
        return pms_fail(ctx, PMS_ERR_CAPACITY, "%llu diffuse particles, the host buffer holds %llu",
                        (unsigned long long)m, (unsigned long long)cap);
    return PMS_OK;
}

// The float form of Wwendland's last factor evaluated on the host, for tests (exported,
// not part of pms.h's stable surface).
extern "C" void pms_debug_wendland_tail(const float* d, const float* t, float* out, uint64_t n) {
    for (uint64_t i = 0; i < n; ++i) out[i] = pms::wendland_tail(d[i], t[i]);
}

extern "C" pms_status pms_reset_diffuse(pms_ctx* ctx) {
    if (!ctx) return PMS_ERR_INVALID_ARGUMENT;
    cudaSetDevice(ctx->device);
    // the carried set is the source of streamed copies until they have landed; frames
    // streamed before the reset can still be waited for
    PMS_CHECK(pms::out_sync(ctx, ctx->diffuse_q));
    PMS_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    ctx->diffuse_old = 0;
    ctx->frame_index = 0;
    ctx->have_diffuse = false;
    return PMS_OK;
}

extern "C" pms_status pms_download_diffuse(pms_ctx* ctx, int type, float* pos, float* vel, int32_t* type_out,
                                           int32_t* ttl, float* wc, float* ta, float* en, uint32_t cap, uint32_t* n_out) {
    if (!ctx) return PMS_ERR_INVALID_ARGUMENT;
    if (type < -1 || type > 2) return pms_fail(ctx, PMS_ERR_INVALID_ARGUMENT, "diffuse type must be -1, 0, 1 or 2");
    cudaSetDevice(ctx->device);
    std::vector<DiffuseParticle> v;
    pms_status st = download_live(ctx, v);
    if (st) return st;
    uint32_t k = 0;
    for (const DiffuseParticle& d : v) {
        // the reference's split: 0 spray, 2 bubble, anything else foam (DiffuseGeneration.cu:808-826)
        const int cls = d.type == 0 ? 0 : (d.type == 2 ? 2 : 1);
        if (type != -1 && cls != type) continue;
        if (k < cap) {
            if (pos) { pos[3 * k] = d.px; pos[3 * k + 1] = d.py; pos[3 * k + 2] = d.pz; }
            if (vel) { vel[3 * k] = d.vx; vel[3 * k + 1] = d.vy; vel[3 * k + 2] = d.vz; }
            if (type_out) type_out[k] = d.type;
            if (ttl) ttl[k] = d.ttl;
            // the reference never fills a diffuse particle's waveCrest / Ita / energy (always 0)
            if (wc) wc[k] = 0.f;
            if (ta) ta[k] = 0.f;
            if (en) en[k] = 0.f;
        }
        ++k;
    }
    if (n_out) *n_out = k;
    if (k > cap && (pos || vel || type_out || ttl || wc || ta || en))
        return pms_fail(ctx, PMS_ERR_CAPACITY, "%u diffuse particles", k);
    return PMS_OK;
}

pms_status pms::diffuse_frame_output(pms_ctx* ctx, const pms_config& cfg, int frame, std::vector<std::vector<float>>& pos,
                                     std::vector<std::vector<float>>& vel, std::vector<std::string>& paths, float& size) {
    std::vector<DiffuseParticle> v;
    pms_status st = download_live(ctx, v);
    if (st) return st;
    static const char* prefixes[3] = {"PartSpary_", "PartFoam_", "PartBubble_"};
    pos.assign(3, {});
    vel.assign(3, {});
    paths.assign(3, {});
    for (const DiffuseParticle& d : v) {
        // the reference's split: 0 spray, 2 bubble, anything else foam (DiffuseGeneration.cu:808-826)
        const int c = d.type == 0 ? 0 : (d.type == 2 ? 2 : 1);
        pos[c].insert(pos[c].end(), {d.px, d.py, d.pz});
        vel[c].insert(vel[c].end(), {d.vx, d.vy, d.vz});
    }
    char num[64];
    snprintf(num, sizeof(num), "%.*d", cfg.num_zeros, frame);
    std::string dir = cfg.diffuse_path;
    if (!dir.empty() && dir.back() != '/') dir += "/";
    for (int cls = 0; cls < 3; ++cls) paths[cls] = dir + prefixes[cls] + num + ".vtk";
    size = ctx->prm.hd / 10.f;
    return PMS_OK;
}
