// pms_internal.h -- shared declarations of libpms (context, device buffers,
// kernel launchers).  Not part of the public ABI (include/pms.h).
#pragma once

#include <cuda_runtime.h>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/pms.h"

namespace pms {

// ---------------------------------------------------------------------------
// device buffers: grow-only, contents not preserved across growth
// ---------------------------------------------------------------------------
struct DBuf {
    void* p = nullptr;
    size_t cap = 0;
    cudaError_t ensure(size_t bytes) {
        if (bytes <= cap && p) return cudaSuccess;
        if (p) { cudaFree(p); p = nullptr; cap = 0; }
        size_t want = bytes < 256 ? 256 : bytes;
        cudaError_t e = cudaMalloc(&p, want);
        if (e == cudaSuccess) cap = want;
        return e;
    }
    void release() { if (p) cudaFree(p); p = nullptr; cap = 0; }
    template <class T> T* as() const { return static_cast<T*>(p); }
};

// Counters kept on the device between stages (read back only on demand).
struct Counters {
    uint32_t n;             // particles
    uint32_t ns;            // surface particles
    uint32_t nv;            // band vertices
    uint32_t nvalid;        // valid cubes
    unsigned long long nmesh;  // mesh vertices
    uint32_t n_fp64;        // covariances solved in FP64
    uint32_t n_big_cells;   // cells with more particles than the per-thread sort handles
    uint32_t err;           // error bits (kErr*)
    uint32_t bbox_min[3];   // order-preserving integer encodings of the bbox
    uint32_t bbox_max[3];
    // diffuse
    uint32_t n_free;        // free-surface particles
    uint32_t n_spawning;    // particles that spawn diffuse particles
    uint32_t n_generated;   // generated diffuse particles
    uint32_t n_old;         // live diffuse particles carried from the last frame
    uint32_t n_live;        // after delete/append
    uint32_t n_type[4];     // spray, foam, bubble, deleted
    uint32_t rad_max_bits;  // largest anisotropic support maxvalue * h (float bits)
    uint32_t pad[1];
};

enum : uint32_t {
    kErrNonFinite = 1u,     // NaN/Inf particle position
    kErrKeyRange = 2u,      // a cell key outside the grid
    kErrBigCell = 4u,       // a cell above the largest supported occupancy
    kErrCapacity = 8u,      // a device-side capacity was exceeded
};

// Marching-cubes tables (see mc_tables.cu): 256 cases, corner order
// (x,y,z) offsets {000,001,011,010,100,101,111,110}, edge k joins
// corners kEdgeVertex[k][0..1].
struct McTables {
    uint32_t edge_flags[256];
    int32_t tri[256][16];
    uint32_t num_vertices[256];
    uint32_t edge_vertex[12][2];
};
const McTables& mc_tables_host();
const char* mc_tables_origin();

// Scan workspace.
struct ScanTemp {
    DBuf partial;           // per-block partial sums (u64 capable)
};

// Stage timing events.
enum Stage { kStageGrid = 0, kStageAniso, kStageBand, kStageField, kStageMc, kStageDiffuse, kNumStages };

}  // namespace pms

// ---------------------------------------------------------------------------
// the context
// ---------------------------------------------------------------------------
struct pms_ctx {
    pms_config cfg;
    pms_params prm;
    pms_grid grid;
    int device = 0;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    std::string last_error;
    uint64_t launches = 0;

    uint32_t n = 0;              // particles of the current frame
    bool have_particles = false, have_grid = false, have_aniso = false, have_band = false,
         have_field = false, have_mc = false, have_diffuse = false;
    // host mirrors of device counters, valid after the stage that syncs
    uint32_t ns = 0, nv = 0, nvalid = 0;
    uint64_t nmesh = 0;

    // particle inputs
    pms::DBuf in_pos, in_vel, in_rho;
    // hashing and sorted particle data
    pms::DBuf keys, slot, order, skeys, spos, svel, rho;
    pms::DBuf cell_count, cell_start, cell_info, surf_count, surf_start, big_cells;
    // anisotropy
    pms::DBuf slist, moments, aniso, nrm4, mean4, gdebug, nnb, cell_rad;
    // band
    pms::DBuf bm0, bm, wcount, wprefix, vlist;
    // field and marching cubes
    pms::DBuf field, mc_case, mc_key, mc_off, valid, vert, vnorm;
    // diffuse
    pms::DBuf d_isfree, d_freescan, d_freelist, d_pot, d_num, d_numscan, d_isdiff, d_isdiffscan,
              d_difflist, d_gen, d_old, d_all, d_rand, d_typescan, d_nrm_free;
    uint32_t diffuse_old = 0;    // live diffuse particles carried to the next frame
    uint32_t frame_index = 0;

    pms::DBuf counters;          // pms::Counters
    pms::Counters* h_counters = nullptr;  // pinned mirror
    pms::ScanTemp scan;
    pms::DBuf tmp;

    cudaEvent_t ev[pms::kNumStages + 1] = {};
    bool ev_recorded[pms::kNumStages] = {};
    int ev_from[pms::kNumStages] = {};
    int last_event = 0;
};

// ---------------------------------------------------------------------------
// error helpers
// ---------------------------------------------------------------------------
pms_status pms_fail(pms_ctx* ctx, pms_status s, const char* fmt, ...);
#define PMS_CUDA(ctx, call)                                                                    \
    do {                                                                                       \
        cudaError_t e__ = (call);                                                              \
        if (e__ != cudaSuccess)                                                                \
            return pms_fail((ctx), e__ == cudaErrorMemoryAllocation ? PMS_ERR_OUT_OF_MEMORY    \
                                                                    : PMS_ERR_CUDA,            \
                            "%s: %s (%s:%d)", #call, cudaGetErrorString(e__), __FILE__, __LINE__); \
    } while (0)
#define PMS_LAUNCHED(ctx)                                                                      \
    do {                                                                                       \
        (ctx)->launches++;                                                                     \
        cudaError_t e__ = cudaPeekAtLastError();                                               \
        if (e__ != cudaSuccess)                                                                \
            return pms_fail((ctx), PMS_ERR_CUDA, "kernel launch: %s (%s:%d)",                  \
                            cudaGetErrorString(e__), __FILE__, __LINE__);                      \
    } while (0)

namespace pms {
// launch helpers
inline unsigned grid_for(uint64_t n, unsigned block, unsigned max_blocks = 152u * 64u) {
    uint64_t b = (n + block - 1) / block;
    if (b < 1) b = 1;
    if (b > max_blocks) b = max_blocks;
    return (unsigned)b;
}

// scans (scan.cu): exclusive prefix sums of n elements; *total_dev receives the
// sum (may be null).  All asynchronous on the stream.
pms_status scan_u32(pms_ctx* ctx, const uint32_t* in, uint32_t* out, uint64_t n, uint32_t* total_dev);
pms_status scan_u64(pms_ctx* ctx, const unsigned long long* in, unsigned long long* out, uint64_t n,
                    unsigned long long* total_dev);

// stage launchers (one .cu each)
pms_status launch_bbox(pms_ctx* ctx);
pms_status launch_hash_sort(pms_ctx* ctx);
pms_status launch_surface_cells(pms_ctx* ctx);
pms_status launch_density_aniso(pms_ctx* ctx);
pms_status launch_band(pms_ctx* ctx);
pms_status launch_band_list(pms_ctx* ctx);
pms_status launch_field(pms_ctx* ctx);
pms_status launch_mc_classify(pms_ctx* ctx);
pms_status launch_mc_emit(pms_ctx* ctx);
pms_status launch_diffuse(pms_ctx* ctx);
pms_status upload_mc_tables(pms_ctx* ctx);

// host utilities
pms_status sync_counters(pms_ctx* ctx);
// diffuse results (k_diffuse.cu)
pms_status diffuse_debug(pms_ctx* ctx, int array_id, std::vector<uint8_t>& out);
pms_status write_diffuse_frame(pms_ctx* ctx, const pms_config& cfg, int frame);
}  // namespace pms
