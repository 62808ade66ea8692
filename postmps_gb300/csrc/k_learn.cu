// k_learn.cu -- learned narrow band: a 64 -> 64 -> 1 ReLU MLP (BF16 weights,
// FP32 accumulate) that predicts which fine cubes of the scalar grid the
// surface crosses, its training kernels, and the exact border-check fallback.
// No counterpart in the reference: it replaces the band-vertex marking of
// estimationOfSurfaceVertices (Anisotropic_kernel.cuh:522-636) as the source
// of the vertices at which computationOfScalarFieldGrid
// (Anisotropic_kernel.cuh:656-777) is evaluated; the field, the marching-cubes
// classification and the triangle emission are the plain path's kernels.
//
// Features.  A coarse density grid has a vertex at every second scalar-grid
// vertex (coarse vertex c sits on fine vertex 2c).  Every particle is splatted
// onto the 8 coarse vertices around it with trilinear weights, accumulated in
// 20-bit fixed point (integer atomics, so the sums do not depend on the order
// of the additions).  Scaled by the particles a coarse cell holds at the
// lattice spacing, a vertex inside the fluid reads about 1 (the trilinear
// weights of a lattice sum to one) and a vertex in the air 0.  Fine cube c
// (origin vertex x) lies in coarse cell k = x >> 1 with parity s = x & 1 per
// axis; its 64 features are the densities of the 4 x 4 x 4 coarse vertices
// nearest to it, k - 1 + d for s = 0 and k + 2 - d for s = 1 (d = 0..3): the
// patch is reflected for odd cubes, so in the patch's own frame every cube
// sits at offsets -2.5, -0.5, 1.5, 3.5 fine cells from the patch's vertices.
// Feature index f = (dz * 4 + dy) * 4 + dx; value min(density, 64), rounded
// to bf16.
//
// Candidates.  Only cubes of coarse cells whose 4 x 4 x 4 patch holds a vertex
// above 0 and a vertex below 0.5 are evaluated (a uniformly full or uniformly
// empty neighbourhood is deep inside or far outside the fluid).
//
// Network.  h = relu(x W1 + b1), z = h . w2 + b2; the cube is predicted when
// z > threshold.  The first layer runs on the tensor cores, 16 cubes per warp
// per mma.sync.m16n8k16 (bf16 inputs, fp32 accumulate), weights held in
// registers as B fragments; the second layer is a quad shuffle reduction.
//
// Training.  Weighted binary cross-entropy on cubes the plain method labels
// (valid marching cube = 1).  Forward as above; backward dz = sigmoid(z) (pw y
// + 1 - y) - pw y (over the batch), dh = dz w2 [pre > 0], dW1 = X^T dh on the
// tensor cores (dh rounded to bf16, fp32 accumulate), db1, dw2, db2 in fp32;
// Adam on fp32 master weights, bf16 copies for the forward pass.
#include "pms_internal.h"
#include "k_common.cuh"
#include "learn_internal.h"
#include <cuda_bf16.h>

namespace pms {

// ---------------------------------------------------------------------------
// helpers
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
    __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<uint32_t*>(&v);
}
__device__ __forceinline__ uint32_t pack_raw(uint16_t lo, uint16_t hi) { return (uint32_t)lo | ((uint32_t)hi << 16); }
__device__ __forceinline__ float bf16_to_f(uint16_t b) { return __uint_as_float((uint32_t)b << 16); }

// D = A (16x16 bf16, row) * B (16x8 bf16, col) + C, fp32
__device__ __forceinline__ void mma_bf16(float (&d)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

static constexpr float kFixScale = 1048576.f;        // 2^20: fixed point of the splat weights
static constexpr float kFixInv = 1.f / 1048576.f;

// scaled density of a coarse vertex from its fixed-point sum (before bf16 rounding)
__device__ __forceinline__ float density_of(uint32_t sum, float inv_expected) {
    return fminf(__fmul_rn(__fmul_rn((float)sum, kFixInv), inv_expected), 64.f);
}
__device__ __forceinline__ float feature_of(uint32_t sum, float inv_expected) {
    return __bfloat162float(__float2bfloat16_rn(density_of(sum, inv_expected)));
}

// coarse vertex of canonical patch offset d (0..3) for a cube in coarse cell k
// with parity s along one axis
__device__ __forceinline__ int patch_cell(int k, int s, int d) { return s ? k + 2 - d : k - 1 + d; }

// ---------------------------------------------------------------------------
// coarse occupancy grid
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_coarse_count(KGrid g, LearnDims ld, const float4* __restrict__ spos, uint32_t n,
                                                      uint32_t* __restrict__ counts) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float4 p = spos[i];
        const float q[3] = {p.x, p.y, p.z};
        int k[3];
        float w1[3];
        bool ok = true;
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            // coarse coordinate: fine coordinate (p - min) / cell, halved
            const float u = __fmul_rn(__fdiv_rn(__fsub_rn(q[a], g.scmin_pos[a]), g.sc_cs), 0.5f);
            const float f0 = floorf(u);
            ok = ok && f0 >= 0.f && f0 < (float)(ld.cres[a] - 1u);
            k[a] = ok ? (int)f0 : 0;
            w1[a] = __fsub_rn(u, f0);
        }
        if (!ok) continue;
#pragma unroll
        for (int c = 0; c < 8; ++c) {
            const float wx = (c & 1) ? w1[0] : __fsub_rn(1.f, w1[0]);
            const float wy = (c & 2) ? w1[1] : __fsub_rn(1.f, w1[1]);
            const float wz = (c & 4) ? w1[2] : __fsub_rn(1.f, w1[2]);
            const uint32_t fix = __float2uint_rn(__fmul_rn(__fmul_rn(__fmul_rn(wx, wy), wz), kFixScale));
            if (fix)
                atomicAdd(&counts[((size_t)(k[2] + (c >> 2)) * ld.cres[1] + (k[1] + ((c >> 1) & 1))) * ld.cres[0] +
                                  (k[0] + (c & 1))],
                          fix);
        }
    }
}

// ---------------------------------------------------------------------------
// Densities as bf16 feature pairs over the coarse grid padded by one plane on
// the low side of every axis (patch vertex -1 lies there and reads 0):
// padded vertex p = ((cz + 1) * P1 + cy + 1) * P0 + cx + 1 with P = cres + 1,
// and dens2[p] = bf16(d(p)) | bf16(d(p + 1)) << 16, d = min(density, 64).
// ---------------------------------------------------------------------------
struct PadDims {
    uint32_t p0, p1, p2;
    size_t np;                // p0 * p1 * p2
};
__host__ __device__ inline PadDims pad_dims(const LearnDims& ld) {
    PadDims d;
    d.p0 = ld.cres[0] + 1; d.p1 = ld.cres[1] + 1; d.p2 = ld.cres[2] + 1;
    d.np = (size_t)d.p0 * d.p1 * d.p2;
    return d;
}

// (the padded grid holds fewer than 2^29 vertices: 32-bit index arithmetic)
__device__ __forceinline__ uint32_t padded_feature(const uint32_t* __restrict__ counts, const LearnDims& ld,
                                                   const PadDims& pd, uint32_t p) {
    if (p >= (uint32_t)pd.np) return 0u;
    const uint32_t row = p / pd.p0, px = p - row * pd.p0, pz = row / pd.p1, py = row - pz * pd.p1;
    if (px == 0 || py == 0 || pz == 0) return 0u;
    const size_t c = ((size_t)(pz - 1) * ld.cres[1] + (py - 1)) * ld.cres[0] + (px - 1);
    return __bfloat16_as_ushort(__float2bfloat16_rn(density_of(counts[c], ld.inv_expected)));
}

__global__ void __launch_bounds__(256) k_coarse_dens(const uint32_t* __restrict__ counts, LearnDims ld,
                                                     uint32_t* __restrict__ dens2) {
    const PadDims pd = pad_dims(ld);
    const uint32_t np = (uint32_t)pd.np;
    for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < np; p += gridDim.x * blockDim.x)
        dens2[p] = padded_feature(counts, ld, pd, p) | (padded_feature(counts, ld, pd, p + 1u) << 16);
}

// ---------------------------------------------------------------------------
// candidates over tiles of 4 x 4 x 4 coarse cells (8 x 8 x 8 fine cubes):
// each tile lists its candidate cubes and appends them to one list
// ---------------------------------------------------------------------------
static constexpr int kTile = 4;                 // coarse cells per tile axis
static constexpr int kHalo = 1;                 // patch vertices k - 1 .. k + 2 of the tile's cells k
static constexpr int kSm = 8;                   // tile + halo = 7 coarse vertices per axis, padded
static constexpr int kCandThreads = 128;

// clist[i] = {cube id, padded coarse vertex of the cube's coarse cell | parity
// x << 29 | parity y << 30 | parity z << 31}
__global__ void __launch_bounds__(kCandThreads) k_learn_cand(KGrid g, LearnDims ld, const uint32_t* __restrict__ counts,
                                                             uint2* __restrict__ clist, uint32_t* __restrict__ n_cand) {
    __shared__ float s_cnt[kSm][kSm][kSm];        // densities of the coarse vertices the tile's cubes read
    __shared__ uint8_t s_mixed[kTile * kTile * kTile];
    __shared__ uint16_t s_list[512];
    __shared__ uint32_t s_n, s_base;
    const int tid = threadIdx.x;
    const uint32_t tx = ld.tiles[0], ty = ld.tiles[1];
    const uint32_t tile = blockIdx.x;
    const int T0[3] = {(int)(tile % tx) * kTile, (int)((tile / tx) % ty) * kTile, (int)(tile / (tx * ty)) * kTile};
    if (T0[2] >= (int)ld.cres[2]) return;
    // the coarse densities of the tile plus halo (outside the grid: empty)
    int any = 0, all = 1;
    for (int e = tid; e < kSm * kSm * kSm; e += kCandThreads) {
        const int lx = e % kSm, ly = (e / kSm) % kSm, lz = e / (kSm * kSm);
        const int cx = T0[0] - kHalo + lx, cy = T0[1] - kHalo + ly, cz = T0[2] - kHalo + lz;
        uint32_t c = 0;
        // the padding plane (index 7) lies beyond every patch: load it as empty without a read
        if (lx < 7 && ly < 7 && lz < 7 && cx >= 0 && cy >= 0 && cz >= 0 && cx < (int)ld.cres[0] && cy < (int)ld.cres[1] &&
            cz < (int)ld.cres[2])
            c = __ldg(&counts[((size_t)cz * ld.cres[1] + cy) * ld.cres[0] + cx]);
        const float d = density_of(c, ld.inv_expected);
        s_cnt[lz][ly][lx] = d;
        if (lx < 7 && ly < 7 && lz < 7) {
            any |= d > 0.f;
            all &= d >= 0.5f;
        }
    }
    if (tid == 0) s_n = 0;
    const int any_b = __syncthreads_or(any), all_b = __syncthreads_and(all);
    if (!any_b || all_b) return;                 // uniformly empty or full: no candidates
    // mixed flag of each coarse cell of the tile over its 4^3 patch vertices
    if (tid < kTile * kTile * kTile) {
        const int cx = tid % kTile, cy = (tid / kTile) % kTile, cz = tid / (kTile * kTile);
        bool nz = false, lo = false;
        for (int dz = 0; dz < 4; ++dz)
            for (int dy = 0; dy < 4; ++dy)
                for (int dx = 0; dx < 4; ++dx) {
                    const float v = s_cnt[cz + dz][cy + dy][cx + dx];
                    nz |= v > 0.f;
                    lo |= v < 0.5f;
                }
        s_mixed[tid] = (nz && lo) ? 1 : 0;
    }
    __syncthreads();
    // candidate cubes of the tile (local index q = (lz * 8 + ly) * 8 + lx)
    const uint32_t rxy = g.scres[0] * g.scres[1];
    for (int q = tid; q < 512; q += kCandThreads) {
        const int lx = q & 7, ly = (q >> 3) & 7, lz = q >> 6;
        const int fx = 2 * T0[0] + lx, fy = 2 * T0[1] + ly, fz = 2 * T0[2] + lz;
        const bool in = fx < (int)g.scres[0] - 1 && fy < (int)g.scres[1] - 1 && fz < (int)g.scres[2] - 1;
        if (in && s_mixed[((lz >> 1) * kTile + (ly >> 1)) * kTile + (lx >> 1)]) s_list[atomicAdd(&s_n, 1u)] = (uint16_t)q;
    }
    __syncthreads();
    const uint32_t ncand = s_n;
    if (ncand == 0) return;
    if (tid == 0) s_base = atomicAdd(n_cand, ncand);
    __syncthreads();
    const PadDims pd = pad_dims(ld);
    for (uint32_t e = tid; e < ncand; e += kCandThreads) {
        const int q = s_list[e];
        const int lx = q & 7, ly = (q >> 3) & 7, lz = q >> 6;
        const uint32_t fx = 2 * T0[0] + lx, fy = 2 * T0[1] + ly, fz = 2 * T0[2] + lz;
        const uint32_t pv = (((fz >> 1) + 1) * pd.p1 + (fy >> 1) + 1) * pd.p0 + (fx >> 1) + 1;
        clist[s_base + e] = make_uint2(fz * rxy + fy * g.scres[0] + fx,
                                       pv | ((fx & 1u) << 29) | ((fy & 1u) << 30) | ((fz & 1u) << 31));
    }
}

// ---------------------------------------------------------------------------
// the network over the candidate list
// ---------------------------------------------------------------------------

struct PredictOut {
    uint32_t* q;              // cube bitmap (bit = origin vertex id); may be null
    uint32_t* cand;           // candidate cube ids; may be null
    float* logit;             // their logits; may be null
    uint32_t cand_cap;
    uint32_t* n_pred;         // device counter
};

// W1 as B fragments: b[kk][nt][0..1] for k-step kk (features 16kk..16kk+15) and
// n-tile nt (hidden 8nt..8nt+7)
__device__ __forceinline__ void load_w1_frags(const DevModel* __restrict__ m, uint32_t (&b)[4][8][2], int lane) {
    const uint16_t* w1 = m->w1;
    const int kq = (lane & 3) * 2, n = lane >> 2;
#pragma unroll
    for (int kk = 0; kk < 4; ++kk)
#pragma unroll
        for (int nt = 0; nt < 8; ++nt) {
            const int i0 = kk * 16 + kq, j = nt * 8 + n;
            b[kk][nt][0] = pack_raw(w1[(i0 + 0) * kHid + j], w1[(i0 + 1) * kHid + j]);
            b[kk][nt][1] = pack_raw(w1[(i0 + 8) * kHid + j], w1[(i0 + 9) * kHid + j]);
        }
}

// The A-fragment registers of one cube for a lane: features (dz, dy, dx) with
// dx in {dx0, dx0 + 1} (one dens2 pair) and dy in {dy0, dy0 + 2}, for dz = kk.
// Patch offset d of a cube with parity s lies at coarse offset d - 1 (s = 0)
// or 2 - d (s = 1) from its coarse cell: for s = 1 the pair runs backwards
// and its halves are swapped.
struct PatchRow {
    uint32_t base;            // padded index of the pair (dx0, dz = 0, dy = dy0)
    int dz, dy2;              // padded index steps for dz + 1 and dy + 2
    bool swap;
};

__device__ __forceinline__ void patch_row(uint32_t rec, int dx0, int dy0, uint32_t p0, uint32_t p01, PatchRow& r) {
    const int sx = (rec >> 29) & 1, sy = (rec >> 30) & 1, sz = (rec >> 31) & 1;
    const int pv = (int)(rec & 0x1fffffffu);
    const int xo = sx ? 1 - dx0 : dx0 - 1;
    const int yo = sy ? 2 - dy0 : dy0 - 1;
    const int zo = sz ? 2 : -1;
    r.base = (uint32_t)(pv + zo * (int)p01 + yo * (int)p0 + xo);
    r.dz = sz ? -(int)p01 : (int)p01;
    r.dy2 = sy ? -2 * (int)p0 : 2 * (int)p0;
    r.swap = sx;
}

__device__ __forceinline__ uint32_t patch_pair(const uint32_t* __restrict__ dens2, const PatchRow& r, int kk, int yi) {
    const uint32_t v = __ldg(&dens2[(int)r.base + kk * r.dz + yi * r.dy2]);
    return r.swap ? __byte_perm(v, 0u, 0x1032) : v;
}

// ---------------------------------------------------------------------------
// The first layer on the fifth-generation tensor cores.  A block takes tiles
// of 128 candidates.  Every thread gathers the 64 features of one candidate
// into registers and writes them to its lane of tensor memory (tcgen05.st
// 32x32b: row = lane, two bf16 of K per 32-bit column); one thread issues four
// tcgen05.mma (M 128, N 64, K 16; A from tensor memory, B = W1 from shared
// memory in the UMMA canonical K-major layout without swizzle, staged once per
// block; fp32 accumulator in tensor memory), their completion arrives on an
// mbarrier, and each warp reads its 32 rows of the accumulator back
// (tcgen05.ld 32x32b) for b1, ReLU, w2 and b2.  Two A buffers let the gathers
// of one tile overlap the MMA and the epilogue of the one before.  The dynamic
// shared memory a block asks for keeps at most four blocks on an SM, so their
// 4 x 128 tensor-memory columns fit the SM's 512 and no allocation waits.
// ---------------------------------------------------------------------------
static constexpr int kTcThreads = 128, kTcRows = 128;
// tensor-memory columns: the N fp32 accumulators (0..63), then two A buffers of
// 64 bf16 per row, two to a 32-bit column (64..95, 96..127)
static constexpr uint32_t kTcCols = 128, kTcColA = 64;
static constexpr uint32_t kTcBytesB = kHid * kIn * 2;
// 4 x (50 + 1) KiB fit an SM's 228 KiB, 5 x do not: four blocks per SM at most
static constexpr uint32_t kTcSmem = 50u * 1024u;
static constexpr uint32_t kTcSpin = 1u << 22;                   // bound on the polls of one mbarrier phase
static constexpr int kTcBlocksPerSm = 4;
static_assert(kTcBytesB + 2 * kHid * 4 + 64 + 1024 <= kTcSmem, "shared memory plan");
static_assert(kIn == 64 && kHid == 64, "the tile plan assumes 64 features and 64 hidden units");

// byte offset of element (row r, k) of a K-major operand with 64 K elements (bf16)
__device__ __forceinline__ uint32_t umma_off(uint32_t r, uint32_t k) {
    return ((((r >> 3) << 3) + (k >> 3)) << 7) + ((r & 7u) << 4) + ((k & 7u) << 1);
}

// shared-memory matrix descriptor: start, leading byte offset 128 (next core
// matrix along K), stride byte offset 1024 (next 8-row group), the fixed
// version bits 46-48 = 0b001, no swizzle
__device__ __forceinline__ uint64_t umma_desc(uint32_t saddr) {
    return (uint64_t)((saddr & 0x3FFFFu) >> 4) | ((uint64_t)(128u >> 4) << 16) | ((uint64_t)(1024u >> 4) << 32) |
           (1ull << 46);
}

// instruction descriptor of kind::f16: fp32 accumulator (bits 4-5 = 1), A and B
// bf16 (bits 7-9 = 1, 10-12 = 1), both K-major, N >> 3 at bit 17, M >> 4 at bit 24
constexpr uint32_t kTcIdesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(kHid >> 3) << 17) |
                              ((uint32_t)(kTcRows >> 4) << 24);

// A from tensor memory (lane = row, 16 bf16 of K in 8 columns), B from shared memory
__device__ __forceinline__ void tc_mma_ts(uint32_t d_tmem, uint32_t a_tmem, uint64_t b, uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], [%1], %2, %3, p;\n\t}\n" ::"r"(d_tmem),
        "r"(a_tmem), "l"(b), "r"(kTcIdesc), "r"(accumulate));
}
// 32 consecutive 32-bit columns of this thread's lane, waited for
__device__ __forceinline__ void tc_st32(uint32_t taddr, const uint32_t (&r)[32]) {
    asm volatile(
        "tcgen05.st.sync.aligned.32x32b.x32.b32 [%0], {%1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, "
        "%16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31, %32};\n\t"
        "tcgen05.wait::st.sync.aligned;" ::"r"(taddr),
        "r"(r[0]), "r"(r[1]), "r"(r[2]), "r"(r[3]), "r"(r[4]), "r"(r[5]), "r"(r[6]), "r"(r[7]), "r"(r[8]), "r"(r[9]),
        "r"(r[10]), "r"(r[11]), "r"(r[12]), "r"(r[13]), "r"(r[14]), "r"(r[15]), "r"(r[16]), "r"(r[17]), "r"(r[18]),
        "r"(r[19]), "r"(r[20]), "r"(r[21]), "r"(r[22]), "r"(r[23]), "r"(r[24]), "r"(r[25]), "r"(r[26]), "r"(r[27]),
        "r"(r[28]), "r"(r[29]), "r"(r[30]), "r"(r[31])
        : "memory");
}
__device__ __forceinline__ void tc_commit(uint32_t bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar) : "memory");
}
__device__ __forceinline__ void tc_before_sync() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_after_sync() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ bool mbar_try(uint32_t bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}\n"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    return ok != 0;
}
// 16 consecutive accumulator columns of this thread's lane, waited for
__device__ __forceinline__ void tc_ld16(uint32_t taddr, float (&v)[16]) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, "
        "[%16];\n\ttcgen05.wait::ld.sync.aligned;"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
          "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr)
        : "memory");
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

__global__ void __launch_bounds__(kTcThreads, kTcBlocksPerSm) k_learn_mlp(LearnDims ld, const uint32_t* __restrict__ dens2,
                                                          const uint2* __restrict__ clist, const uint32_t* __restrict__ n_dev,
                                                          const DevModel* __restrict__ model, int use_model, PredictOut out,
                                                          uint32_t* __restrict__ err, uint32_t wait_polls) {
    const uint32_t n = *n_dev;
    if (!use_model) {
        // collect only
        for (uint32_t e = blockIdx.x * blockDim.x + threadIdx.x; e < n && e < out.cand_cap; e += gridDim.x * blockDim.x)
            out.cand[e] = clist[e].x;
        if (blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(out.n_pred, n);
        return;
    }
    extern __shared__ uint8_t tc_smem[];
    uint8_t* sm = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(tc_smem) + 1023u) & ~(uintptr_t)1023u);
    uint8_t* sB = sm;
    float* s_b1 = reinterpret_cast<float*>(sB + kTcBytesB);
    float* s_w2 = s_b1 + kHid;
    uint64_t* s_bar = reinterpret_cast<uint64_t*>(s_w2 + kHid);
    uint32_t* s_tmem = reinterpret_cast<uint32_t*>(s_bar + 1);
    const uint32_t tid = threadIdx.x, warp = tid >> 5;
    const uint32_t b_saddr = (uint32_t)__cvta_generic_to_shared(sB);
    const uint32_t bar = (uint32_t)__cvta_generic_to_shared(s_bar);
    // W1 as the B operand (row j = hidden unit, K = input feature i)
    for (uint32_t e = tid; e < (uint32_t)(kHid * kIn / 2); e += kTcThreads) {
        const uint32_t j = e / (kIn / 2), i = (e % (kIn / 2)) * 2;
        *reinterpret_cast<uint32_t*>(sB + umma_off(j, i)) =
            pack_raw(model->w1[i * kHid + j], model->w1[(i + 1) * kHid + j]);
    }
    // {b1[j], b1[j + 1], w2[j], w2[j + 1]} for even j, one 16-byte load per two columns
    if (tid < (uint32_t)kHid / 2) {
        const uint32_t j = 2 * tid;
        reinterpret_cast<float4*>(s_b1)[tid] =
            make_float4(model->b1[j], model->b1[j + 1], bf16_to_f(model->w2[j]), bf16_to_f(model->w2[j + 1]));
    }
    if (tid == 0) mbar_init(bar, 1);
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                         (uint32_t)__cvta_generic_to_shared(s_tmem)),
                     "r"(kTcCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    fence_async_smem();
    tc_before_sync();
    __syncthreads();
    tc_after_sync();
    const uint32_t tmem = *s_tmem;
    const uint32_t t_row = tmem + ((warp * 32u) << 16);      // this warp's 32 lanes
    const float b2 = model->b2, thr = model->threshold;
    const PadDims pd = pad_dims(ld);
    const uint32_t p01 = pd.p0 * pd.p1;
    const uint32_t ntiles = (n + kTcRows - 1) / kTcRows;
    uint32_t phase = 0, npred = 0;
    bool ok = true;
    // Software pipeline: while the tensor cores work on tile t (A buffer t & 1),
    // the threads load tile t + 1's features into registers and finish tile t's
    // epilogue; then they store those features into the other buffer and one
    // thread issues tile t + 1's MMA.  Candidate records come one tile earlier.
    const uint32_t e_step = gridDim.x * (uint32_t)kTcRows;
    uint32_t g[32];
    auto gather = [&](uint2 c) {
        PatchRow r[4];
        patch_row(c.y, 0, 0, pd.p0, p01, r[0]);
        patch_row(c.y, 2, 0, pd.p0, p01, r[1]);
        patch_row(c.y, 0, 1, pd.p0, p01, r[2]);
        patch_row(c.y, 2, 1, pd.p0, p01, r[3]);
#pragma unroll
        for (int kk = 0; kk < 4; ++kk)
#pragma unroll
            for (int yi = 0; yi < 2; ++yi)
#pragma unroll
                for (int q = 0; q < 4; ++q) g[(kk * 2 + yi) * 4 + q] = patch_pair(dens2, r[q], kk, yi);
    };
    // this thread's row, features f = 16 dz + 4 dy + dx in K order: g[i] holds
    // f = 2i, 2i + 1, the 32-bit column i of the row's lane in an A buffer
    auto store = [&](uint32_t buf, bool live) {
        if (!live)
#pragma unroll
            for (int i = 0; i < 32; ++i) g[i] = 0u;
        tc_st32(t_row + kTcColA + 32u * buf, g);
    };
    auto issue = [&](uint32_t buf) {
        if (tid == 0) {
            tc_after_sync();
#pragma unroll
            for (uint32_t kk = 0; kk < 4; ++kk)
                tc_mma_ts(tmem, tmem + kTcColA + 32u * buf + 8u * kk, umma_desc(b_saddr + kk * 256u), kk);
            tc_commit(bar);
        }
    };
    uint32_t tile = blockIdx.x, buf = 0;
    uint32_t e = tile * kTcRows + tid;
    bool live = tile < ntiles && e < n;
    uint32_t id = 0;
    uint2 c_pref = make_uint2(0u, 0u);
    if (tile < ntiles) {
        if (live) {
            const uint2 c = __ldg(&clist[e]);
            id = c.x;
            gather(c);
        }
        if (e + e_step < n) c_pref = __ldg(&clist[e + e_step]);
        store(0, live);
        tc_before_sync();
        __syncthreads();
        issue(0);
    }
    for (; tile < ntiles; tile += gridDim.x) {
        const uint32_t tnext = tile + gridDim.x;
        const uint32_t e_n = e + e_step;
        const bool live_n = tnext < ntiles && e_n < n;
        const uint2 c_n = c_pref;
        uint32_t id_n = 0;
        if (live_n) {
            id_n = c_n.x;
            gather(c_n);                     // in flight during the wait and the epilogue
            if (e_n + e_step < n) c_pref = __ldg(&clist[e_n + e_step]);
        }
        bool done = false;
        for (uint32_t spins = 0; spins < wait_polls && !(done = mbar_try(bar, phase)); ++spins) {
        }
        ok = __syncthreads_and(done) != 0;
        if (!ok) {
            // give the MMA in flight a second bounded wait before its tensor memory is freed
            if (tid == 0) {
                uint32_t again = 0;
                bool landed = false;
                while (!(landed = mbar_try(bar, phase)) && ++again < kTcSpin) {
                }
                // the tensor memory is freed below either way: the host must not trust this context
                if (!landed) atomicOr(err, kErrTcLost);
            }
            __syncthreads();
            break;
        }
        phase ^= 1u;
        tc_after_sync();
        float z = b2;
#pragma unroll
        for (uint32_t q = 0; q < 4; ++q) {
            float v[16];
            tc_ld16(t_row + q * 16u, v);
#pragma unroll
            for (int i = 0; i < 16; i += 2) {
                const float4 bw = reinterpret_cast<const float4*>(s_b1)[(q * 16 + i) / 2];
                z += fmaxf(v[i] + bw.x, 0.f) * bw.z;
                z += fmaxf(v[i + 1] + bw.y, 0.f) * bw.w;
            }
        }
        if (live) {
            if (out.logit) {
                if (e < out.cand_cap) { out.cand[e] = id; out.logit[e] = z; }
                ++npred;
            } else if (z > thr) {
                atomicOr(&out.q[id >> 5], 1u << (id & 31u));
                ++npred;
            }
        }
        if (tnext < ntiles) {
            // the other buffer was read by the MMA two tiles back, finished before this wait
            store(buf ^ 1u, live_n);
        }
        tc_before_sync();                    // this tile's accumulator reads finish before the next MMA
        __syncthreads();
        if (tnext < ntiles) issue(buf ^ 1u);
        buf ^= 1u;
        e = e_n;
        live = live_n;
        id = id_n;
    }
    if (!ok && tid == 0) atomicOr(err, kErrTimeout);
    // one count per warp
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) npred += __shfl_xor_sync(0xffffffffu, npred, o);
    if ((tid & 31u) == 0 && npred) atomicAdd(out.n_pred, npred);
    tc_before_sync();
    __syncthreads();
    tc_after_sync();
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTcCols) : "memory");
}

// ---------------------------------------------------------------------------
// The band split: a cube marks its 8 corners (cube c is a corner's cube when c
// is the corner minus {0,1} along each axis), and the plain band U splits into
// the corners of predicted cubes E (evaluated exactly at once) and the rest N
// (certified); popcounts per word for the scans of both.
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t shifted(const uint32_t* __restrict__ b, uint64_t w, uint64_t s) {
    const uint64_t q = s >> 5;
    const uint32_t r = (uint32_t)(s & 31u);
    if (w < q) return 0u;
    const uint32_t hi = b[w - q];
    if (r == 0) return hi;
    const uint32_t lo = (w >= q + 1) ? b[w - q - 1] : 0u;
    return (hi << r) | (lo >> (32u - r));
}

// cubes null: no prediction, N = U
__global__ void __launch_bounds__(256) k_band_split(const uint32_t* __restrict__ cubes, const uint32_t* __restrict__ band,
                                                    uint32_t* __restrict__ e_bm, uint32_t* __restrict__ n_bm,
                                                    uint32_t* __restrict__ e_wc, uint32_t* __restrict__ n_wc, uint64_t nwords,
                                                    uint64_t nbits, uint64_t sy, uint64_t sz) {
    for (uint64_t w = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; w < nwords; w += (uint64_t)gridDim.x * blockDim.x) {
        uint32_t v = 0u;
        if (cubes)
            v = cubes[w] | shifted(cubes, w, 1) | shifted(cubes, w, sy) | shifted(cubes, w, sy + 1) |
                shifted(cubes, w, sz) | shifted(cubes, w, sz + 1) | shifted(cubes, w, sz + sy) | shifted(cubes, w, sz + sy + 1);
        uint32_t u = band[w];
        if (w == nwords - 1 && (nbits & 31u)) u &= (1u << (nbits & 31u)) - 1u;
        const uint32_t e = u & v, n = u & ~v;
        e_bm[w] = e;
        n_bm[w] = n;
        e_wc[w] = __popc(e);
        n_wc[w] = __popc(n);
    }
}

// The certified corners of the valid cubes (compaction records {vertex id,
// case, ...}): their bits move from `cert` to `recheck`, whose vertices are
// then evaluated exactly, so that `cert` ends holding the band vertices whose
// field is a placeholder.  A cube's corners lie in 4 rows of 2 neighbouring
// vertices.
__global__ void __launch_bounds__(256) k_recheck_bits(KGrid g, const Counters* __restrict__ cnt, const uint4* __restrict__ cube,
                                                      uint32_t* __restrict__ cert, uint32_t* __restrict__ recheck) {
    const uint32_t n = cnt->nvalid;
    const uint32_t rx = g.scres[0], rxy = g.scres[0] * g.scres[1];
    for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
        const uint32_t id = __ldg(&cube[t]).x;
#pragma unroll
        for (int r = 0; r < 4; ++r) {
            const uint32_t c = id + (uint32_t)(r & 1) * rx + (uint32_t)(r >> 1) * rxy;   // corners c, c + 1
            const uint32_t w = c >> 5, sh = c & 31u;
            const uint32_t pair = (cert[w] >> sh) & (sh == 31u ? 1u : 3u);
            const uint32_t hi = sh == 31u ? (cert[w + 1] & 1u) : 0u;
            if (pair) atomicOr(&recheck[w], pair << sh);
            if (hi) atomicOr(&recheck[w + 1], 1u);
            // those vertices get exact values: they leave the certified set
            if (pair) atomicAnd(&cert[w], ~(pair << sh));
            if (hi) atomicAnd(&cert[w + 1], ~1u);
        }
    }
}

// popcount per word of a bitmap
__global__ void __launch_bounds__(256) k_popc(const uint32_t* __restrict__ b, uint32_t* __restrict__ wcount, uint64_t nwords) {
    for (uint64_t w = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; w < nwords; w += (uint64_t)gridDim.x * blockDim.x)
        wcount[w] = __popc(b[w]);
}

// cube bitmap of the plain method's valid cubes (training labels)
__global__ void __launch_bounds__(256) k_label_bits(const uint32_t* __restrict__ n_dev, const uint32_t* __restrict__ vlist,
                                                    const unsigned long long* __restrict__ mc_key, uint32_t* __restrict__ lbm) {
    const uint32_t n = *n_dev;
    for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x)
        if (mc_key[t]) atomicOr(&lbm[vlist[t] >> 5], 1u << (vlist[t] & 31u));
}

// features of explicit cubes (bf16 bits, 64 per cube), for checks against the oracle
__global__ void __launch_bounds__(256) k_features(KGrid g, LearnDims ld, const uint32_t* __restrict__ counts,
                                                  const uint32_t* __restrict__ cubes, uint32_t n, uint16_t* __restrict__ x) {
    const uint32_t rx = g.scres[0], rxy = g.scres[0] * g.scres[1];
    for (uint64_t e = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; e < 64ull * n; e += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t s = (uint32_t)(e >> 6), f = (uint32_t)(e & 63u);
        const uint32_t id = cubes[s];
        const int c[3] = {(int)(id % rx), (int)((id / rx) % g.scres[1]), (int)(id / rxy)};
        const int d[3] = {(int)(f & 3u), (int)((f >> 2) & 3u), (int)(f >> 4)};
        int cc[3];
        bool in = true;
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            cc[a] = patch_cell(c[a] >> 1, c[a] & 1, d[a]);
            in = in && cc[a] >= 0 && cc[a] < (int)ld.cres[a];
        }
        const uint32_t cnt = in ? counts[((size_t)cc[2] * ld.cres[1] + cc[1]) * ld.cres[0] + cc[0]] : 0u;
        x[e] = __bfloat16_as_ushort(__float2bfloat16_rn(feature_of(cnt, ld.inv_expected)));
    }
}

// ---------------------------------------------------------------------------
// Training on the fifth-generation tensor cores: one block = 128 samples, one
// thread per sample (its tensor-memory lane).
//   forward   D1 (128 x 64, fp32, tensor memory) = X (128 x 64, bf16, tensor
//             memory, written by each thread to its own lane) . W1 (shared memory,
//             the inference kernel's K-major layout); each thread reads its row back
//             and forms pre, h, z, the loss and dz, dh = dz w2 [pre > 0].
//   backward  D2 (128 x 80) = A2 (128 x 128 samples) . B2 (128 samples x 80), both
//             K-major in shared memory (each thread writes its sample's column):
//             A2 rows j < 64 hold dh[:, j], rows 64 + j hold h[:, j]; B2 columns
//             f < 64 hold X[:, f], column 64 holds 1, column 65 dz, the rest 0.  So
//             D2[j][f] = sum_s dh[s][j] X[s][f] (dW1 transposed), D2[j][64] =
//             sum_s dh[s][j] (db1) and D2[64 + j][65] = sum_s h[s][j] dz[s] (dw2):
//             all three gradients from one accumulator (dh, h, dz rounded to bf16,
//             fp32 accumulation).  db2 and the loss are warp reductions.
// One thread issues the MMAs; their completion arrives on an mbarrier whose waits
// are bounded (a wait that runs out sets an error bit, waits once more for the
// MMA in flight and frees the tensor memory).
// ---------------------------------------------------------------------------
static constexpr int kTrainThreads = 128, kBlockSamples = 128;
static constexpr uint32_t kTrCols = 256;                 // tensor-memory columns of a block
static constexpr uint32_t kTrColA = 64, kTrColD2 = 128;  // X (32 columns), D2 (80 columns)
static constexpr uint32_t kTrN2 = 80;                     // D2 columns: 64 features, ones, dz, zero padding
static constexpr uint32_t kTrBytesA2 = 128u * 128u * 2u, kTrBytesB2 = kTrN2 * 128u * 2u;
static constexpr uint32_t kTrSmem = 1024u + kTcBytesB + kTrBytesA2 + kTrBytesB2 + kBlockSamples * kIn * 2 +
                                    kBlockSamples * 4 + 2 * kHid * 4 + 64;
constexpr uint32_t kTrIdesc2 = (1u << 4) | (1u << 7) | (1u << 10) | ((kTrN2 >> 3) << 17) | ((128u >> 4) << 24);
static_assert(kTrN2 % 16 == 0 && kTrColD2 + kTrN2 <= kTrCols && kTrColA + 32 <= kTrColD2, "tensor-memory plan");

struct TrainIn {
    // source A: sampled candidates of a frame
    const uint32_t* cand; uint32_t n_cand; const uint32_t* labels; const uint32_t* counts;
    // source B: explicit bf16 features and labels
    const uint16_t* x; const uint8_t* y;
    uint32_t batch; uint64_t seed; float pos_weight;
};

__device__ __forceinline__ uint64_t mix64(uint64_t z) {
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

// byte offset of element (row r, k) of a K-major operand with 128 K elements (bf16)
__device__ __forceinline__ uint32_t umma_off128(uint32_t r, uint32_t k) {
    return ((((r >> 3) << 4) + (k >> 3)) << 7) + ((r & 7u) << 4) + ((k & 7u) << 1);
}
// the descriptor of such an operand: core matrices 128 bytes apart along K, 8-row
// groups 2048 bytes apart
__device__ __forceinline__ uint64_t umma_desc128(uint32_t saddr) {
    return (uint64_t)((saddr & 0x3FFFFu) >> 4) | ((uint64_t)(128u >> 4) << 16) | ((uint64_t)(2048u >> 4) << 32) |
           (1ull << 46);
}
// A and B from shared memory
__device__ __forceinline__ void tc_mma_ss(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t idesc, uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(d_tmem),
        "l"(a), "l"(b), "r"(idesc), "r"(accumulate));
}

// a bounded wait on the mbarrier phase, block-wide; false when it ran out (then the
// MMA in flight had a second bounded wait and err holds the reason)
__device__ bool tr_wait(uint32_t bar, uint32_t parity, uint32_t* err) {
    bool done = false;
    for (uint32_t spins = 0; spins < kTcSpin && !(done = mbar_try(bar, parity)); ++spins) {
    }
    if (__syncthreads_and(done)) return true;
    if (threadIdx.x == 0) {
        uint32_t again = 0;
        bool landed = false;
        while (!(landed = mbar_try(bar, parity)) && ++again < kTcSpin) {
        }
        atomicOr(err, landed ? kErrTimeout : (kErrTimeout | kErrTcLost));
    }
    __syncthreads();
    return false;
}

__global__ void __launch_bounds__(kTrainThreads) k_learn_train(KGrid g, LearnDims ld, TrainIn in,
                                                               const DevModel* __restrict__ model, float* __restrict__ grad,
                                                               float* __restrict__ loss_sum, uint32_t* __restrict__ err) {
    extern __shared__ uint8_t tr_smem[];
    uint8_t* sm = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(tr_smem) + 1023u) & ~(uintptr_t)1023u);
    uint8_t* sW1 = sm;
    uint8_t* sA2 = sW1 + kTcBytesB;
    uint8_t* sB2 = sA2 + kTrBytesA2;
    uint16_t* s_x = reinterpret_cast<uint16_t*>(sB2 + kTrBytesB2);        // [sample][feature]
    float* s_y = reinterpret_cast<float*>(s_x + kBlockSamples * kIn);
    float* s_b1 = s_y + kBlockSamples;
    float* s_w2 = s_b1 + kHid;
    uint64_t* s_bar = reinterpret_cast<uint64_t*>(s_w2 + kHid);
    uint32_t* s_tmem = reinterpret_cast<uint32_t*>(s_bar + 1);
    const uint32_t tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5;
    const uint32_t s_base = blockIdx.x * kBlockSamples;
    const float inv_batch = 1.f / (float)in.batch;
    // features and labels of the block's samples (rows past the batch: zero, label -1)
    for (uint32_t e = tid; e < (uint32_t)(kBlockSamples * kIn); e += kTrainThreads) {
        const uint32_t r = e / kIn, f = e % kIn;
        const uint32_t s = s_base + r;
        uint16_t v = 0;
        float y = -1.f;
        if (s < in.batch) {
            if (in.x) {
                v = in.x[(size_t)s * kIn + f];
                y = in.y[s] ? 1.f : 0.f;
            } else {
                const uint32_t slot = (uint32_t)(mix64(in.seed ^ (0x9E3779B97F4A7C15ull * (s + 1))) % in.n_cand);
                const uint32_t id = in.cand[slot];
                const uint32_t rx = g.scres[0], rxy = g.scres[0] * g.scres[1];
                const int c[3] = {(int)(id % rx), (int)((id / rx) % g.scres[1]), (int)(id / rxy)};
                const int d[3] = {(int)(f & 3u), (int)((f >> 2) & 3u), (int)(f >> 4)};
                int cc[3];
                bool inside = true;
#pragma unroll
                for (int a = 0; a < 3; ++a) {
                    cc[a] = patch_cell(c[a] >> 1, c[a] & 1, d[a]);
                    inside = inside && cc[a] >= 0 && cc[a] < (int)ld.cres[a];
                }
                const uint32_t cnt = inside ? in.counts[((size_t)cc[2] * ld.cres[1] + cc[1]) * ld.cres[0] + cc[0]] : 0u;
                v = __bfloat16_as_ushort(__float2bfloat16_rn(feature_of(cnt, ld.inv_expected)));
                y = ((in.labels[id >> 5] >> (id & 31u)) & 1u) ? 1.f : 0.f;
            }
        }
        s_x[r * kIn + f] = v;
        if (f == 0) s_y[r] = y;
    }
    // W1 as the forward's B operand (row j = hidden unit, K = input feature i)
    for (uint32_t e = tid; e < (uint32_t)(kHid * kIn / 2); e += kTrainThreads) {
        const uint32_t j = e / (kIn / 2), i = (e % (kIn / 2)) * 2;
        *reinterpret_cast<uint32_t*>(sW1 + umma_off(j, i)) = pack_raw(model->w1[i * kHid + j], model->w1[(i + 1) * kHid + j]);
    }
    if (tid < (uint32_t)kHid) {
        s_b1[tid] = model->b1[tid];
        s_w2[tid] = bf16_to_f(model->w2[tid]);
    }
    const uint32_t bar = (uint32_t)__cvta_generic_to_shared(s_bar);
    if (tid == 0) mbar_init(bar, 1);
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                         (uint32_t)__cvta_generic_to_shared(s_tmem)),
                     "r"(kTrCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    fence_async_smem();
    tc_before_sync();
    __syncthreads();
    tc_after_sync();
    const uint32_t tmem = *s_tmem;
    const uint32_t t_row = tmem + ((warp * 32u) << 16);
    // forward: this sample's features into its lane, then D1 = X W1
    {
        uint32_t xr[32];
#pragma unroll
        for (int i = 0; i < 32; ++i) xr[i] = pack_raw(s_x[tid * kIn + 2 * i], s_x[tid * kIn + 2 * i + 1]);
        tc_st32(t_row + kTrColA, xr);
    }
    tc_before_sync();
    __syncthreads();
    if (tid == 0) {
        tc_after_sync();
        const uint32_t w_saddr = (uint32_t)__cvta_generic_to_shared(sW1);
#pragma unroll
        for (uint32_t kk = 0; kk < 4; ++kk) tc_mma_ts(tmem, tmem + kTrColA + 8u * kk, umma_desc(w_saddr + kk * 256u), kk);
        tc_commit(bar);
    }
    bool ok = tr_wait(bar, 0, err);
    float dz = 0.f, lsum = 0.f;
    if (ok) {
        tc_after_sync();
        float acc[kHid];
#pragma unroll
        for (uint32_t q = 0; q < 4; ++q) {
            float v[16];
            tc_ld16(t_row + q * 16u, v);
#pragma unroll
            for (int i = 0; i < 16; ++i) acc[q * 16 + i] = v[i] + s_b1[q * 16 + i];
        }
        float z = model->b2;
#pragma unroll
        for (int j = 0; j < kHid; ++j) z += fmaxf(acc[j], 0.f) * s_w2[j];
        const float y = s_y[tid];
        if (y >= 0.f) {
            const float p = 1.f / (1.f + expf(-z));
            const float wy = in.pos_weight * y;
            dz = (p * (wy + 1.f - y) - wy) * inv_batch;
            // softplus(-z) = -log sigmoid(z), softplus(z) = -log(1 - sigmoid(z))
            const float sp_pos = fmaxf(-z, 0.f) + log1pf(expf(-fabsf(z)));
            const float sp_neg = fmaxf(z, 0.f) + log1pf(expf(-fabsf(z)));
            lsum = (wy * sp_pos + (1.f - y) * sp_neg) * inv_batch;
        }
        // this sample's column of A2 (dh, then h) and of B2 (x, 1, dz, 0)
#pragma unroll
        for (int j = 0; j < kHid; ++j) {
            const float dh = acc[j] > 0.f ? dz * s_w2[j] : 0.f;
            *reinterpret_cast<uint16_t*>(sA2 + umma_off128((uint32_t)j, tid)) = __bfloat16_as_ushort(__float2bfloat16_rn(dh));
            *reinterpret_cast<uint16_t*>(sA2 + umma_off128((uint32_t)(kHid + j), tid)) =
                __bfloat16_as_ushort(__float2bfloat16_rn(fmaxf(acc[j], 0.f)));
        }
    }
#pragma unroll 8
    for (uint32_t n = 0; n < kTrN2; ++n) {
        const uint16_t v = n < (uint32_t)kIn ? s_x[tid * kIn + n]
                                             : (n == (uint32_t)kIn ? (uint16_t)0x3F80u
                                                                   : (n == (uint32_t)kIn + 1u ? __bfloat16_as_ushort(__float2bfloat16_rn(dz))
                                                                                              : (uint16_t)0u));
        *reinterpret_cast<uint16_t*>(sB2 + umma_off128(n, tid)) = v;
    }
    // db2 and the loss, one atomic per warp
    float gb2 = dz;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        gb2 += __shfl_xor_sync(0xffffffffu, gb2, o);
        lsum += __shfl_xor_sync(0xffffffffu, lsum, o);
    }
    if (ok && lane == 0) {
        atomicAdd(&grad[kOffB2], gb2);
        atomicAdd(loss_sum, lsum);
    }
    // backward: D2 = A2 B2 over the block's 128 samples
    fence_async_smem();
    tc_before_sync();
    __syncthreads();
    if (ok) {
        if (tid == 0) {
            tc_after_sync();
            const uint32_t a_saddr = (uint32_t)__cvta_generic_to_shared(sA2), b_saddr = (uint32_t)__cvta_generic_to_shared(sB2);
#pragma unroll
            for (uint32_t kk = 0; kk < 8; ++kk)
                tc_mma_ss(tmem + kTrColD2, umma_desc128(a_saddr + kk * 256u), umma_desc128(b_saddr + kk * 256u), kTrIdesc2, kk);
            tc_commit(bar);
        }
        ok = tr_wait(bar, 1, err);
    }
    if (ok) {
        tc_after_sync();
        if (warp < 2) {
            // row j = tid: dW1[f][j] for f < 64 and db1[j]
#pragma unroll
            for (uint32_t q = 0; q < 4; ++q) {
                float v[16];
                tc_ld16(t_row + kTrColD2 + q * 16u, v);
#pragma unroll
                for (int i = 0; i < 16; ++i) atomicAdd(&grad[(q * 16 + i) * kHid + tid], v[i]);
            }
            float v[16];
            tc_ld16(t_row + kTrColD2 + 64u, v);
            atomicAdd(&grad[kOffB1 + tid], v[0]);
        } else {
            // row 64 + j: dw2[j] in column 65
            float v[16];
            tc_ld16(t_row + kTrColD2 + 64u, v);
            atomicAdd(&grad[kOffW2 + tid - kHid], v[1]);
        }
    }
    tc_before_sync();
    __syncthreads();
    tc_after_sync();
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTrCols) : "memory");
}

// Adam on the fp32 master parameters, then the bf16 / fp32 model copy
__global__ void __launch_bounds__(256) k_adam(float* __restrict__ w, const float* __restrict__ grad, float* __restrict__ m,
                                              float* __restrict__ v, AdamParams ap, DevModel* __restrict__ model) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < kNumParams; i += gridDim.x * blockDim.x) {
        if (ap.lr != 0.f) {
            const float gi = grad[i];
            const float mi = ap.beta1 * m[i] + (1.f - ap.beta1) * gi;
            const float vi = ap.beta2 * v[i] + (1.f - ap.beta2) * gi * gi;
            m[i] = mi;
            v[i] = vi;
            w[i] -= ap.lr * (mi * ap.inv_bc1) / (sqrtf(vi * ap.inv_bc2) + ap.eps);
        }
        const float wi = w[i];
        if (i < kOffB1) model->w1[i] = __bfloat16_as_ushort(__float2bfloat16_rn(wi));
        else if (i < kOffW2) model->b1[i - kOffB1] = wi;
        else if (i < kOffB2) model->w2[i - kOffW2] = __bfloat16_as_ushort(__float2bfloat16_rn(wi));
        else model->b2 = wi;
    }
}

// ---------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------
LearnDims learn_dims(const pms_ctx* ctx) {
    const pms_grid& g = ctx->grid;
    LearnDims ld;
    for (int a = 0; a < 3; ++a) {
        ld.cres[a] = g.scres[a] / 2u + 2u;                        // coarse vertices per axis
        ld.tiles[a] = ((g.scres[a] + 1u) / 2u + kTile - 1) / kTile;  // tiles over the coarse cells holding cubes
    }
    const double side = 2.0 * (double)g.sc_grid_size, sp = (double)ctx->prm.particle_spacing;
    const double expected = (side / sp) * (side / sp) * (side / sp);
    ld.inv_expected = (float)(expected > 0.0 ? 1.0 / expected : 1.0);
    return ld;
}

pms_status launch_coarse_counts(pms_ctx* ctx) {
    const KGrid g = kgrid_of(ctx->grid);
    const LearnDims ld = learn_dims(ctx);
    const size_t nc = (size_t)ld.cres[0] * ld.cres[1] * ld.cres[2];
    PMS_CUDA(ctx, ctx->l_counts.ensure(4 * (nc ? nc : 1)));
    const PadDims pd = pad_dims(ld);
    if (pd.np >= (1ull << 29)) return pms_fail(ctx, PMS_ERR_UNSUPPORTED, "coarse grid too large");
    PMS_CUDA(ctx, ctx->l_dens.ensure(4 * pd.np));
    PMS_CUDA(ctx, cudaMemsetAsync(ctx->l_counts.p, 0, 4 * nc, ctx->stream));
    if (ctx->n) {
        k_coarse_count<<<grid_for(ctx->n, 256), 256, 0, ctx->stream>>>(g, ld, ctx->spos.as<float4>(), ctx->n,
                                                                         ctx->l_counts.as<uint32_t>());
        PMS_LAUNCHED(ctx);
    }
    k_coarse_dens<<<grid_for(pd.np, 256), 256, 0, ctx->stream>>>(ctx->l_counts.as<uint32_t>(), ld, ctx->l_dens.as<uint32_t>());
    PMS_LAUNCHED(ctx);
    return PMS_OK;
}

pms_status launch_predict(pms_ctx* ctx, int use_model, uint32_t* q, uint32_t* cand, float* logit, uint32_t cand_cap) {
    const KGrid g = kgrid_of(ctx->grid);
    const LearnDims ld = learn_dims(ctx);
    const uint64_t ntiles = (uint64_t)ld.tiles[0] * ld.tiles[1] * ld.tiles[2];
    if (ntiles >= (1ull << 31)) return pms_fail(ctx, PMS_ERR_UNSUPPORTED, "coarse grid too large");
    Counters* cnt = ctx->counters.as<Counters>();
    // candidates are distinct cubes: at most one per scalar-grid vertex
    PMS_CUDA(ctx, ctx->l_clist.ensure(8 * ((size_t)g.sc_size + 1)));
    k_learn_cand<<<(unsigned)ntiles, kCandThreads, 0, ctx->stream>>>(g, ld, ctx->l_counts.as<uint32_t>(),
                                                                    ctx->l_clist.as<uint2>(), &cnt->l_cand);
    PMS_LAUNCHED(ctx);
    PredictOut out;
    out.q = q; out.cand = cand; out.logit = logit; out.cand_cap = cand_cap;
    out.n_pred = &cnt->l_pred;
    PMS_CUDA(ctx, cudaFuncSetAttribute(k_learn_mlp, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kTcSmem));
    PMS_CUDA(ctx, cudaFuncSetAttribute(k_learn_mlp, cudaFuncAttributePreferredSharedMemoryCarveout,
                                       (int)cudaSharedmemCarveoutMaxShared));
    k_learn_mlp<<<152u * kTcBlocksPerSm, kTcThreads, kTcSmem, ctx->stream>>>(
        ld, ctx->l_dens.as<uint32_t>(), ctx->l_clist.as<uint2>(), &cnt->l_cand,
        ctx->l_model.as<DevModel>(), use_model, out, &cnt->err, ctx->tc_wait_polls ? ctx->tc_wait_polls - 1u : kTcSpin);
    PMS_LAUNCHED(ctx);
    return PMS_OK;
}

pms_status launch_band_split(pms_ctx* ctx, const uint32_t* cubes, uint32_t* e_bm, uint32_t* n_bm, uint32_t* e_wc,
                             uint32_t* n_wc) {
    const KGrid g = kgrid_of(ctx->grid);
    const uint64_t nbits = g.sc_size, nwords = (nbits + 31) / 32;
    const uint64_t sy = g.scres[0], sz = (uint64_t)g.scres[0] * g.scres[1];
    k_band_split<<<grid_for(nwords, 256), 256, 0, ctx->stream>>>(cubes, ctx->bm.as<uint32_t>(), e_bm, n_bm, e_wc, n_wc,
                                                                 nwords, nbits, sy, sz);
    PMS_LAUNCHED(ctx);
    return PMS_OK;
}

pms_status launch_bits_list(pms_ctx* ctx, const uint32_t* bm, const uint32_t* wprefix, uint32_t* vlist);

pms_status launch_recheck_bits(pms_ctx* ctx, uint32_t* cert, uint32_t* recheck) {
    const KGrid g = kgrid_of(ctx->grid);
    Counters* cnt = ctx->counters.as<Counters>();
    // ctx->nv bounds the valid cubes; the kernel reads their count
    k_recheck_bits<<<grid_for(ctx->nv, 256), 256, 0, ctx->stream>>>(g, cnt, ctx->cube.as<uint4>(), cert, recheck);
    PMS_LAUNCHED(ctx);
    return PMS_OK;
}

pms_status launch_popc(pms_ctx* ctx, const uint32_t* b, uint32_t* wcount) {
    const uint64_t nwords = ((uint64_t)ctx->grid.sc_size + 31) / 32;
    k_popc<<<grid_for(nwords, 256), 256, 0, ctx->stream>>>(b, wcount, nwords);
    PMS_LAUNCHED(ctx);
    return PMS_OK;
}

pms_status launch_label_bits(pms_ctx* ctx, uint32_t* lbm) {
    Counters* cnt = ctx->counters.as<Counters>();
    k_label_bits<<<grid_for(ctx->nv, 256), 256, 0, ctx->stream>>>(&cnt->nv, ctx->vlist.as<uint32_t>(),
                                                                   ctx->mc_key.as<unsigned long long>(), lbm);
    PMS_LAUNCHED(ctx);
    return PMS_OK;
}

pms_status launch_features(pms_ctx* ctx, const uint32_t* cubes, uint32_t n, uint16_t* x) {
    const KGrid g = kgrid_of(ctx->grid);
    const LearnDims ld = learn_dims(ctx);
    k_features<<<grid_for(64ull * n, 256), 256, 0, ctx->stream>>>(g, ld, ctx->l_counts.as<uint32_t>(), cubes, n, x);
    PMS_LAUNCHED(ctx);
    return PMS_OK;
}

cudaError_t launch_train(const pms_ctx* data, cudaStream_t stream, const TrainArgs& a, const DevModel* model, float* grad,
                         float* loss_sum, uint32_t* err) {
    KGrid g = {};
    LearnDims ld = {};
    TrainIn in = {};
    if (data) {
        g = kgrid_of(data->grid);
        ld = learn_dims(data);
        in.cand = data->l_cand.as<uint32_t>();
        in.n_cand = data->l_ncand;
        in.labels = data->l_label.as<uint32_t>();
        in.counts = data->l_counts.as<uint32_t>();
    }
    in.x = a.x;
    in.y = a.y;
    in.batch = a.batch;
    in.seed = a.seed;
    in.pos_weight = a.pos_weight;
    const unsigned blocks = (a.batch + kBlockSamples - 1) / kBlockSamples;
    const cudaError_t e = cudaFuncSetAttribute(k_learn_train, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kTrSmem);
    if (e != cudaSuccess) return e;
    k_learn_train<<<blocks, kTrainThreads, kTrSmem, stream>>>(g, ld, in, model, grad, loss_sum, err);
    return cudaGetLastError();
}

cudaError_t launch_adam(cudaStream_t stream, float* w, const float* grad, float* m, float* v, const AdamParams& ap,
                        DevModel* model) {
    k_adam<<<(kNumParams + 255) / 256, 256, 0, stream>>>(w, grad, m, v, ap, model);
    return cudaGetLastError();
}

}  // namespace pms
