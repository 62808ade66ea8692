// pms_internal.h -- shared declarations of libpms (context, device buffers,
// kernel launchers).  Not part of the public ABI (include/pms.h).
#pragma once

#include <cuda_runtime.h>
#include <atomic>
#include <cstdint>
#include <mutex>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/pms.h"

namespace pms {

// ---------------------------------------------------------------------------
// device buffers: grow-only, contents not preserved across growth
// ---------------------------------------------------------------------------
// A captured CUDA graph holds raw buffer addresses: it is captured again when the
// signature of the buffers it uses (dbuf_signature) has changed.
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
    // for sizes that grow from frame to frame (the carried diffuse set): half again as
    // much room, so that a slowly growing need does not reallocate (and synchronise) every frame
    cudaError_t ensure_grow(size_t bytes) {
        if (bytes <= cap && p) return cudaSuccess;
        return ensure(bytes + bytes / 2);
    }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        cap = 0;
    }
    template <class T> T* as() const { return static_cast<T*>(p); }
};

// Counters kept on the device between stages (read back only on demand).
static constexpr int kMaxMcPieces = 4;  // vertex ranges a streamed mesh is emitted in

struct Counters {
    uint32_t n;             // particles
    uint32_t ns;            // surface particles
    uint32_t nv;            // band vertices
    uint32_t nvalid;        // valid cubes
    unsigned long long nmesh;  // mesh vertices
    unsigned long long n_pairs;  // (vertex, particle) pairs the field launches evaluated
    uint32_t n_fp64;        // covariances solved in FP64
    uint32_t n_big_cells;   // cells with more particles than the per-thread sort handles
    uint32_t err;           // error bits (kErr*)
    uint32_t bbox_min[3];   // order-preserving integer encodings of the bbox
    uint32_t bbox_max[3];
    // diffuse
    uint32_t n_free;        // free-surface particles
    uint32_t n_spawning;    // particles that spawn diffuse particles
    uint32_t n_generated;   // generated diffuse particles
    uint32_t n_old;         // live diffuse particles carried from the last frame (batched frames)
    uint32_t n_live;        // after delete/append
    uint32_t n_type[4];     // spray, foam, bubble, deleted
    uint32_t rad_max_bits;  // largest anisotropic support maxvalue * h (float bits)
    // learned band (the first kLearnCounters fields are zeroed per frame)
    uint32_t l_cand;        // candidate cubes evaluated by the network
    uint32_t l_pred;        // predicted cubes (or candidate slots written)
    uint32_t l_exact;       // band vertices evaluated exactly first (corners of predicted cubes)
    uint32_t l_nlist;       // band vertices certified (the rest of the band)
    uint32_t l_cert;        // ... of which stopped above iso without an exact value
    uint32_t l_recheck;     // certified corners of valid cubes, evaluated exactly afterwards
    uint32_t n_items;       // work items of the last field launch
    uint32_t n_tiles;       // scalar-grid tiles the band marking visits
    uint32_t n_weld;        // vertices of the welded mesh (crossed grid edges)
    uint32_t n_df_total;    // generated + carried diffuse particles of a batched frame
    uint32_t mc_piece[kMaxMcPieces + 1];  // first cube of each streamed emission range, then nvalid
};
static constexpr int kLearnCounters = 6;

enum : uint32_t {
    kErrNonFinite = 1u,     // NaN/Inf particle position
    kErrKeyRange = 2u,      // a cell key outside the grid
    kErrBigCell = 4u,       // a cell above the largest supported occupancy
    kErrCapacity = 8u,      // a device-side capacity was exceeded
    kErrTimeout = 16u,      // a bounded wait on the tensor cores gave up
    kErrTcLost = 32u,       // ... and the MMA in flight outlived a second bounded wait
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

// Frames whose streamed output (mesh or diffuse particles) is on its way to a
// registered host buffer, oldest first.  Each record's event fires when its copies
// have landed; copies run in order on the copy stream, so the newest event covers
// every older one.
struct OutQueue {
    static constexpr int kSlots = 4;   // frames in flight at most
    cudaEvent_t ev[kSlots] = {};
    const void* host[kSlots] = {};     // the buffer the frame's copy writes
    uint64_t n[kSlots] = {}, cap[kSlots] = {};
    bool overflow[kSlots] = {};
    int head = 0, count = 0;           // oldest record, records pending
    int last = -1;                     // newest record ever made (its event may have fired)
};

// Scan workspace.
struct ScanTemp {
    DBuf partial;           // per-block partial sums (u64 capable)
};

// Launch shapes chosen by the autotuner (pms_autotune): threads per block of
// the neighbour walks and the field's resident-block cap (blocks per SM).
struct Tune {
    int field_threads = 128, field_waves = 8, density_threads = 128, moments_threads = 128, field_vpt = 2;
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
    // velocities uploaded on a stream of their own while the grid is built (the sort's
    // gather waits for them)
    cudaStream_t up_stream = nullptr;
    cudaEvent_t up_start = nullptr, vel_ready = nullptr;
    // staged upload (pms_stage_particles / pms_upload_staged): the next frame's inputs in a
    // second pair of device buffers, copied from pinned host staging on stage_stream
    std::mutex stage_mu;
    pms::DBuf st_pos, st_vel;
    float *stage_hpos = nullptr, *stage_hvel = nullptr;
    size_t stage_hcap = 0;
    cudaStream_t stage_stream = nullptr;
    cudaEvent_t stage_ready = nullptr, stage_free = nullptr;
    bool staged = false, stage_free_recorded = false;
    uint32_t staged_n = 0;
    bool vel_pending = false;
    // mesh streamed to registered host buffers on a copy stream while later stages (and,
    // with alternating buffers, later frames) run; out_* is the registration for the
    // frames to come, mesh_q the frames on their way
    cudaStream_t copy_stream = nullptr;
    cudaEvent_t mesh_ready = nullptr;
    float* out_pos = nullptr;
    float* out_nrm = nullptr;
    uint64_t out_cap = 0;
    pms::OutQueue mesh_q;
    // live diffuse particles streamed to a registered host buffer on the copy stream
    pms_diffuse_particle* dout = nullptr;
    uint64_t dout_cap = 0;
    cudaEvent_t diffuse_ready = nullptr;
    pms::OutQueue diffuse_q;
    // the diffuse stage beside the surface stages of a frame: its own stream and scan
    // scratch (swapped in while its parts are issued), fork and join events
    cudaStream_t df_stream = nullptr;
    cudaEvent_t df_fork = nullptr, df_join = nullptr;
    pms::ScanTemp df_scan;
    pms::DBuf df_tmp;
    bool df_run = false;               // the frame's diffuse parts have work (particles)
    size_t df_total = 0;               // generated + carried particles of the frame
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
    pms::DBuf slist, moments, aniso, nrm4, mean4, gdebug, nnb, cell_rad, cell_rec;
    // band (and the tiles of the scalar grid its marking visits)
    pms::DBuf bm0, bm, wcount, wprefix, vlist, tile_bits, tile_wc, tile_wp, tile_list;
    // field and marching cubes
    pms::DBuf field, mc_case, mc_key, mc_off, valid, vert, vnorm, sval;
    // the field over the whole scalar grid, 0 off the band (the marching cubes' lookups);
    // per valid cube {vertex id, case, first mesh vertex, 0}
    pms::DBuf fdense, cube;
    // welded mesh: crossed-edge bitmap (3 bits per scalar vertex), its word popcounts and
    // prefix, vertices, normals, triangle indices
    pms::DBuf w_bits, w_wc, w_wp, w_vert, w_vnorm, w_idx;
    uint64_t w_nvert = 0;
    bool have_weld = false, weld_normals = false;
    // field work items (runs of x-neighbouring band vertices)
    pms::DBuf fitems, fitem_cnt, fitem_off;
    bool have_values = false;
    // vertex normals of the current mesh: made by the emission only when a streamed
    // mesh asks for them, else on the first download that does
    bool mesh_normals = false;
    // diffuse
    pms::DBuf d_isfree, d_freescan, d_freelist, d_pot, d_num, d_numscan, d_isdiff, d_isdiffscan,
              d_difflist, d_gen, d_old, d_all, d_rand, d_typescan, d_nrm_free, d_tkey, d_tscan, d_perm;
    // learned band: coarse counts, model, cube bitmaps, merge buffers, training data
    pms::DBuf l_dens, l_clist;   // bf16 coarse density pairs (padded grid), candidate cube records
    // l_q: predicted cubes; l_cert: certified vertices; E / N: vertices evaluated exactly first /
    // certified (bitmaps, popcounts, prefixes, lists); the rechecked corners reuse E's buffers
    pms::DBuf l_counts, l_model, l_q, l_cert, l_e_bm, l_e_wc, l_e_wp, l_e_list, l_n_bm, l_n_wc, l_n_wp, l_n_list,
              l_field_new, l_cand, l_logit, l_label;
    bool have_model = false, band_learned = false, mc_classified = false, mc_compacted = false;
    // polls + 1 of the first bounded wait on the tensor cores (0: the default bound)
    uint32_t tc_wait_polls = 0;
    int band_mode = PMS_BAND_PLAIN;
    pms::Tune tune;
    // batched frames (pms_batch.cpp)
    void* batch = nullptr;
    uint64_t batch_launches = 0;         // kernels in the batch graph
    uint32_t l_ncand = 0, l_npred = 0, l_nexact = 0, l_ncert = 0, l_nrecheck = 0;
    uint32_t diffuse_old = 0;    // live diffuse particles carried to the next frame
    uint32_t frame_index = 0;

    pms::DBuf counters;          // pms::Counters
    pms::Counters* h_counters = nullptr;  // pinned mirror, mapped
    uint32_t* h_counters_dev = nullptr;   // ... its device address
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
#define PMS_CHECK(expr)                                                                        \
    do {                                                                                       \
        const pms_status s__ = (expr);                                                         \
        if (s__ != PMS_OK) return s__;                                                         \
    } while (0)
#define PMS_LAUNCHED(ctx)                                                                      \
    do {                                                                                       \
        (ctx)->launches++;                                                                     \
        cudaError_t e__ = cudaGetLastError();                                                  \
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
// sum (may be null); with n_dev, elements at and past *n_dev count as zero
// (n is then a bound).  All asynchronous on the stream.
pms_status scan_u32(pms_ctx* ctx, const uint32_t* in, uint32_t* out, uint64_t n, uint32_t* total_dev,
                    const uint32_t* n_dev = nullptr);
pms_status scan_u64(pms_ctx* ctx, const unsigned long long* in, unsigned long long* out, uint64_t n,
                    unsigned long long* total_dev, const uint32_t* n_dev = nullptr);

// stage launchers (one .cu each)
pms_status launch_bbox(pms_ctx* ctx);
// Streamed-output queues (pms_api.cpp).  copy_stream_ready creates the copy stream and
// both queues' events.  out_begin picks the record slot of a frame about to stream into
// `host`: records still pending on that buffer (and every older one) are waited for and
// dropped, as is the oldest when all slots are taken.  out_push files the frame after
// its copies and the slot's event were issued.  out_wait pops the oldest record.
// out_device_wait orders the context's stream after every copy issued so far (before a
// copy's device source is written again); out_sync waits on the host for them.
pms_status copy_stream_ready(pms_ctx* ctx);
pms_status out_begin(pms_ctx* ctx, OutQueue& q, const void* host, int* slot);
void out_push(OutQueue& q, int slot, const void* host, uint64_t n, uint64_t cap);
pms_status out_wait(pms_ctx* ctx, OutQueue& q, uint64_t* n, bool* overflow, uint64_t* cap);
pms_status out_device_wait(pms_ctx* ctx, const OutQueue& q);
pms_status out_sync(pms_ctx* ctx, const OutQueue& q);
// the counters into the mapped mirror h_counters (one small kernel on the context's stream)
pms_status launch_publish_counters(pms_ctx* ctx);
pms_status launch_hash_sort(pms_ctx* ctx);
pms_status launch_surface_cells(pms_ctx* ctx);
pms_status launch_density_aniso(pms_ctx* ctx);
pms_status launch_band(pms_ctx* ctx);
pms_status launch_band_list(pms_ctx* ctx);
pms_status launch_field(pms_ctx* ctx);
// field at the vertices vlist[0 .. *n_dev) into out (n_host: a bound for the grid); with
// cert, sign certification: vertices stopped above iso get a bit there, n_cert counts them
pms_status launch_field_on(pms_ctx* ctx, const uint32_t* vlist, const uint32_t* n_dev, uint32_t n_host, float* out,
                           uint32_t* cert = nullptr, uint32_t* n_cert = nullptr);
pms_status launch_field_gather(pms_ctx* ctx, const uint32_t* vlist, const uint32_t* n_dev, uint32_t n_host, float* out);
// ascending list of the set bits of a bitmap over the scalar grid
pms_status launch_bits_list(pms_ctx* ctx, const uint32_t* bm, const uint32_t* wprefix, uint32_t* vlist);
// marching-cube cases of the band vertices, then the scan and compaction; classify = both
pms_status launch_mc_cases(pms_ctx* ctx);
pms_status launch_mc_compact(pms_ctx* ctx);
pms_status launch_mc_classify(pms_ctx* ctx);
// the mesh in `pieces` vertex ranges [nmesh * q / pieces, nmesh * (q + 1) / pieces): the first
// cube of each range into Counters::mc_piece (pieces <= kMaxMcPieces)
pms_status launch_mc_piece_bounds(pms_ctx* ctx, uint32_t pieces);
// piece q emits the cubes whose first mesh vertex lies in range q (all cubes for piece < 0)
pms_status launch_mc_emit(pms_ctx* ctx, int piece = -1, uint32_t pieces = 1);
pms_status launch_scalar_values(pms_ctx* ctx);
// welded mesh from the valid-cube records (k_mc.cu): ebits of nw words zeroed and set,
// n_unique its vertex count; vert / vnorm / idx may be null
pms_status launch_weld(pms_ctx* ctx, uint32_t* ebits, uint32_t* wc, uint32_t* wprefix, uint64_t nw, uint32_t* n_unique,
                       uint64_t cap, float* vert, float* vnorm, uint32_t* idx);
// triangle soup into vert (+ 3 * *frame_base floats when frame_base is set), at most cap vertices
pms_status launch_mc_emit_to(pms_ctx* ctx, float* vert, float* vnorm, const unsigned long long* frame_base,
                             unsigned long long cap, int piece = -1, uint32_t pieces = 1);
pms_status launch_diffuse(pms_ctx* ctx);
// launch_diffuse's three parts (k_diffuse.cu): front, tail, finish
pms_status diffuse_part_front(pms_ctx* ctx);
pms_status diffuse_part_tail(pms_ctx* ctx);
pms_status diffuse_part_finish(pms_ctx* ctx);
// A batched frame's diffuse stage: every size is a capacity and every count lives on the
// device, so it can be captured into a graph.  The carried particles come from ctx->d_old
// (their count at *old_dev, set by the frame before), the survivors go to ctx->d_all and
// (the buffers then swap, on the host, at capture) their count to *old_dev, and a copy of
// them lands in the arena at a running offset.
struct DiffuseBatch {
    uint32_t gen_cap = 0, old_cap = 0;       // generated and carried particles a frame may hold
    uint32_t* old_dev = nullptr;             // carried count (in: this frame's; out: the next frame's)
    const uint32_t* frame_dev = nullptr;     // frame counter of the batch's first frame
    uint32_t frame_off = 0;                  // this frame's place in the batch
    unsigned long long* running = nullptr;   // arena fill (device)
    unsigned long long* base = nullptr;      // this frame's arena offset (device)
    void* arena = nullptr;                   // 32-byte diffuse records
    uint64_t arena_cap = 0;                  // records the arena holds
};
pms_status ensure_diffuse_batch_buffers(pms_ctx* ctx, uint32_t nmax, uint32_t gen_cap, uint32_t old_cap);
pms_status launch_diffuse_bounded(pms_ctx* ctx, const DiffuseBatch& db);
pms_status upload_mc_tables(pms_ctx* ctx);

// host utilities
pms_status sync_counters(pms_ctx* ctx);
// a hash of the addresses and sizes of a context's device buffers (without the
// diffuse stage's unless asked for)
uint64_t dbuf_signature(pms_ctx* c, bool diffuse);
}  // namespace pms
void pms_batch_release(pms_ctx* c);   // pms_batch.cpp
namespace pms {
// diffuse results (k_diffuse.cu)
pms_status diffuse_debug(pms_ctx* ctx, int array_id, std::vector<uint8_t>& out);
// the live diffuse particles split into the three files of a frame (FileData.cpp:945-1036):
// positions and velocities per class (spray, foam, bubble), their paths, the size value
pms_status diffuse_frame_output(pms_ctx* ctx, const pms_config& cfg, int frame, std::vector<std::vector<float>>& pos,
                                std::vector<std::vector<float>>& vel, std::vector<std::string>& paths, float& size);
}  // namespace pms
