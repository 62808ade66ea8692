// pms_batch.cpp -- many frames in one CUDA graph launch.  No counterpart in
// the reference: GPUPOST::runSimulation (GPUPOST.cpp:56-81) runs one frame at
// a time, synchronising with the host after almost every stage.
//
// A batch runs in two passes.  (1) All frames are copied into one device
// arena and their bounding boxes are computed (one synchronisation for the
// whole batch); the host derives each frame's grid from its box exactly as
// for a single frame.  (2) Every stage of every frame is captured, in order,
// into one CUDA graph whose kernels size their work from counts kept on the
// device -- one Counters record per frame -- with host-side launch grids and
// buffers sized by per-frame bounds, so nothing in the graph waits for the
// host.  Frames run one after another on the context's buffers; meshes land
// behind each other in one arena (the running offset lives on the device).
// The graph is kept and relaunched while the frames' grids stay the same.
// Frames are spread over lanes -- the context and up to three sub-contexts,
// each with its own buffers and stream -- that fork from and join the
// capture stream, so independent frames overlap on the GPU; a frame's mesh
// claims its stretch of the arena with an atomic add.
//
// With the learned band, the graph holds each frame's plain band, prediction,
// split, exact field at the predicted corners, sign certification of the rest,
// classification and exact field at the certified corners of valid cubes: the
// same launches as a single learned frame, every size a bound and every count
// on the device, so the batched result equals the single-frame result (and the
// plain band's).
//
// With diffuse generation on, a diffuse lane -- a further sub-context with its
// own stream -- runs every frame's diffuse stage in frame order, as the carried
// particles demand: frame f's stage waits for frame f's surface stages on their
// lane and reads that lane's grid buffers, and the lane's next frame waits for it
// before it overwrites them.  Sizes are capacities (generated and carried
// particles per frame), counts live on the device, the carried set alternates
// between two buffers, and each frame's survivors land in a diffuse arena; a
// count past a capacity sets an error bit and the batch runs again, from the
// same carried particles, with larger buffers.  The carried set enters from and
// returns to the context, so batches and single frames continue one sequence.
#include <algorithm>
#include <memory>
#include <cstdint>
#include <cstring>
#include <utility>

#include "pms_internal.h"
#include "learn_internal.h"

using namespace pms;

namespace pms {
pms_status ensure_band_buffers(pms_ctx* c, uint32_t nv);
pms_status ensure_particle_buffers(pms_ctx* c, uint32_t n);
pms_status ensure_grid_buffers(pms_ctx* c, const pms_grid& g);
pms_status launch_batch_base(pms_ctx* ctx, const Counters* cnt, unsigned long long* running, unsigned long long* base);
pms_status launch_batch_mesh_to_host(pms_ctx* ctx, const float* mesh, const unsigned long long* base_f,
                                     unsigned long long dev_cap, float* host, unsigned long long host_cap, uint32_t* trunc);
}  // namespace pms

struct BatchState {
    DBuf pos, vel, rho, cnt, base, mesh;
    std::vector<uint32_t> n;
    std::vector<uint64_t> off;
    std::vector<pms_grid> grid;
    std::vector<Counters> hcnt;
    std::vector<unsigned long long> hbase;
    std::vector<cudaEvent_t> ev, ev_end;         // per-frame start / end, recorded inside the graph
    std::vector<pms_ctx*> lanes;                 // sub-contexts (lane 0 is the context itself)
    std::vector<cudaEvent_t> join;
    cudaEvent_t fork = nullptr;
    cudaGraphExec_t exec = nullptr;
    int flags = -1;
    uint64_t mesh_cap = 0;
    uint32_t captures = 0;
    uint64_t sig = 0;                 // signature of the buffers the graph was captured against
    uint32_t nlanes_captured = 0;
    uint32_t wait_captured = 0;       // the debug wait limit baked into the captured launches
    // diffuse generation
    pms_ctx* dlane = nullptr;                    // the diffuse lane
    cudaEvent_t djoin = nullptr;
    std::vector<cudaEvent_t> ev_surf, ev_diff;   // per frame: grid and anisotropy done (the diffuse fork), diffuse done
    DBuf dcnt, drun, dbase, darena;              // {carried count, first frame's number}, arena fill, offsets, arena
    uint64_t darena_cap = 0;
    uint32_t gen_cap = 0, old_cap = 0;
    void *d_in = nullptr, *d_out = nullptr;      // carried buffer the graph reads first / holds the survivors last
    std::vector<unsigned long long> hdbase;
    // meshes streamed into a registered host arena inside the graph (pms_batch_stream_meshes)
    float* h_mesh = nullptr;                     // host address, for the caller
    float* h_mesh_dev = nullptr;                 // the same memory as the kernels see it
    uint64_t h_mesh_cap = 0;                     // vertices
    DBuf h_trunc;                                // set when a frame's soup did not fit the host arena
    ~BatchState() {
        if (exec) cudaGraphExecDestroy(exec);
        for (cudaEvent_t e : ev) cudaEventDestroy(e);
        for (cudaEvent_t e : ev_end) cudaEventDestroy(e);
        for (cudaEvent_t e : join) cudaEventDestroy(e);
        if (fork) cudaEventDestroy(fork);
        for (pms_ctx* l : lanes) pms_destroy(l);
        for (cudaEvent_t e : ev_surf) cudaEventDestroy(e);
        for (cudaEvent_t e : ev_diff) cudaEventDestroy(e);
        if (djoin) cudaEventDestroy(djoin);
        if (dlane) pms_destroy(dlane);
        for (DBuf* b : {&pos, &vel, &rho, &cnt, &base, &mesh, &dcnt, &drun, &dbase, &darena, &h_trunc}) b->release();
    }
};

static BatchState* batch_of(pms_ctx* c) {
    if (!c->batch) c->batch = new BatchState;
    return static_cast<BatchState*>(c->batch);
}

void pms_batch_release(pms_ctx* c) {
    delete static_cast<BatchState*>(c->batch);
    c->batch = nullptr;
}

static bool same_grid(const pms_grid& a, const pms_grid& b) { return memcmp(&a, &b, sizeof(a)) == 0; }

// Points the context at frame f of the arena (buffers borrowed, not owned).
struct FrameView {
    pms_ctx* c;
    DBuf pos, vel, rho, cnt;
    uint32_t n;
    pms_grid grid;
    explicit FrameView(pms_ctx* ctx) : c(ctx), pos(ctx->in_pos), vel(ctx->in_vel), rho(ctx->in_rho), cnt(ctx->counters),
                                       n(ctx->n), grid(ctx->grid) {}
    // the frame's grid is known only after the bounding-box pass (with_grid false there)
    void point(BatchState* b, uint32_t f, bool with_grid = true) {
        c->in_pos.p = b->pos.as<char>() + 12 * b->off[f];
        c->in_vel.p = b->vel.as<char>() + 12 * b->off[f];
        c->in_rho.p = b->rho.as<char>() + 4 * b->off[f];
        // borrowed: a capacity no request exceeds, so nothing frees or regrows them through the view
        c->in_pos.cap = c->in_vel.cap = c->in_rho.cap = SIZE_MAX;
        c->counters.p = b->cnt.as<Counters>() + f;
        c->counters.cap = SIZE_MAX;
        c->n = b->n[f];
        if (with_grid) c->grid = b->grid[f];
    }
    ~FrameView() {
        c->in_pos = pos; c->in_vel = vel; c->in_rho = rho; c->counters = cnt;
        c->n = n; c->grid = grid;
    }
};

// Points the diffuse lane at frame f: the grid buffers of the lane that built the
// frame, the frame's counters, size and grid (borrowed; restored on destruction).
struct DiffuseLaneView {
    pms_ctx* d;
    DBuf skeys, cell_info, nrm4, cell_start, spos, svel, cnt;
    uint32_t n;
    pms_grid grid;
    bool have_aniso;
    explicit DiffuseLaneView(pms_ctx* dl)
        : d(dl), skeys(dl->skeys), cell_info(dl->cell_info), nrm4(dl->nrm4), cell_start(dl->cell_start), spos(dl->spos),
          svel(dl->svel), cnt(dl->counters), n(dl->n), grid(dl->grid), have_aniso(dl->have_aniso) {}
    void point(const pms_ctx* lc, BatchState* b, uint32_t f) {
        d->skeys = lc->skeys; d->cell_info = lc->cell_info; d->nrm4 = lc->nrm4;
        d->cell_start = lc->cell_start; d->spos = lc->spos; d->svel = lc->svel;
        for (DBuf* x : {&d->skeys, &d->cell_info, &d->nrm4, &d->cell_start, &d->spos, &d->svel}) x->cap = SIZE_MAX;
        d->counters.p = b->cnt.as<Counters>() + f;
        d->counters.cap = SIZE_MAX;
        d->n = b->n[f];
        d->grid = b->grid[f];
        d->have_aniso = true;
    }
    ~DiffuseLaneView() {
        d->skeys = skeys; d->cell_info = cell_info; d->nrm4 = nrm4; d->cell_start = cell_start; d->spos = spos;
        d->svel = svel; d->counters = cnt; d->n = n; d->grid = grid; d->have_aniso = have_aniso;
    }
};

// Stages of one frame without host synchronisation (the context points at the frame).
// band: 0 plain, 1 learned (network + certification), 2 certification alone.
// fork (when set) is recorded once the frame's grid and anisotropy are made: all the
// diffuse stage reads, so the diffuse lane starts there, beside the band and field.
static pms_status capture_frame(pms_ctx* c, BatchState* b, uint32_t f, int band, cudaEvent_t fork) {
    pms_status st;
    Counters* cnt = c->counters.as<Counters>();
    const pms_grid& g = c->grid;
    c->nv = g.sc_size;                       // bounds for launch grids; kernels read the device counts
    c->nvalid = g.sc_size;
    if ((st = launch_bbox(c))) return st;    // resets the frame's counters
    if (c->n == 0) {
        if (fork) PMS_CUDA(c, cudaEventRecord(fork, c->stream));
        return PMS_OK;
    }
    if ((st = launch_hash_sort(c))) return st;
    if ((st = launch_surface_cells(c))) return st;
    if ((st = launch_density_aniso(c))) return st;
    if (fork) PMS_CUDA(c, cudaEventRecord(fork, c->stream));
    if (band) {
        if ((st = launch_band(c))) return st;
        if ((st = launch_band_list(c))) return st;
        if ((st = learned_split(c, band == 1))) return st;
        if ((st = learned_field(c))) return st;
    } else {
        if ((st = launch_band(c))) return st;
        if ((st = launch_band_list(c))) return st;
        if ((st = launch_field(c))) return st;
        if ((st = launch_mc_classify(c))) return st;
    }
    unsigned long long* base = b->base.as<unsigned long long>();
    if ((st = launch_batch_base(c, cnt, base + b->n.size(), base + f))) return st;
    if ((st = launch_mc_emit_to(c, b->mesh.as<float>(), nullptr, base + f, b->mesh_cap))) return st;
    if (b->h_mesh_dev)
        return launch_batch_mesh_to_host(c, b->mesh.as<float>(), base + f, b->mesh_cap, b->h_mesh_dev, b->h_mesh_cap,
                                         b->h_trunc.as<uint32_t>());
    return PMS_OK;
}

static constexpr uint32_t kBatchLanes = 4;

// lane l of the batch: the context itself for l = 0, else a sub-context
static pms_ctx* lane_ctx(pms_ctx* c, BatchState* b, uint32_t l) { return l == 0 ? c : b->lanes[l - 1]; }

static pms_status capture(pms_ctx* c, BatchState* b, int band, uint32_t nlanes, bool diffuse) {
    if (b->exec) { cudaGraphExecDestroy(b->exec); b->exec = nullptr; }
    const uint32_t k = (uint32_t)b->n.size();
    // frames to lanes, largest first onto the least loaded lane
    std::vector<uint32_t> order(k), lane_of(k);
    for (uint32_t f = 0; f < k; ++f) order[f] = f;
    std::stable_sort(order.begin(), order.end(), [&](uint32_t x, uint32_t y) { return b->n[x] > b->n[y]; });
    std::vector<uint64_t> load(nlanes, 0);
    for (uint32_t f : order) {
        const uint32_t l = (uint32_t)(std::min_element(load.begin(), load.end()) - load.begin());
        lane_of[f] = l;
        load[l] += b->n[f] + 1;
    }
    cudaGraph_t graph = nullptr;
    pms_ctx* dl = diffuse ? b->dlane : nullptr;
    std::vector<uint64_t> launches0(nlanes);
    for (uint32_t l = 0; l < nlanes; ++l) launches0[l] = lane_ctx(c, b, l)->launches;
    const uint64_t dlaunches0 = dl ? dl->launches : 0;
    PMS_CUDA(c, cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeRelaxed));
    pms_status st = PMS_OK;
    cudaError_t e = cudaMemsetAsync(b->base.as<unsigned long long>() + k, 0, sizeof(unsigned long long), c->stream);
    if (e == cudaSuccess && dl) e = cudaMemsetAsync(b->drun.p, 0, sizeof(unsigned long long), c->stream);
    if (e == cudaSuccess) e = cudaEventRecord(b->fork, c->stream);
    for (uint32_t l = 1; l < nlanes && e == cudaSuccess; ++l) e = cudaStreamWaitEvent(lane_ctx(c, b, l)->stream, b->fork, 0);
    if (e == cudaSuccess && dl) e = cudaStreamWaitEvent(dl->stream, b->fork, 0);
    if (e != cudaSuccess) st = PMS_ERR_CUDA;
    {
        // frames in order, each on its lane; with diffuse generation each frame's diffuse
        // stage follows on the diffuse lane, and the lane's next frame waits for it
        std::vector<std::unique_ptr<FrameView>> views;
        for (uint32_t l = 0; l < nlanes; ++l) views.emplace_back(new FrameView(lane_ctx(c, b, l)));
        std::unique_ptr<DiffuseLaneView> dview(dl ? new DiffuseLaneView(dl) : nullptr);
        std::vector<int> last(nlanes, -1);
        if (dl) b->d_in = dl->d_old.p;
        for (uint32_t f = 0; f < k && !st; ++f) {
            const uint32_t l = lane_of[f];
            pms_ctx* lc = lane_ctx(c, b, l);
            if (dl && last[l] >= 0 && cudaStreamWaitEvent(lc->stream, b->ev_diff[(uint32_t)last[l]], 0) != cudaSuccess) {
                st = PMS_ERR_CUDA;
                break;
            }
            views[l]->point(b, f);
            // external: recorded when the graph runs (a plain record inside a capture only orders work)
            if (cudaEventRecordWithFlags(b->ev[f], lc->stream, cudaEventRecordExternal) != cudaSuccess) { st = PMS_ERR_CUDA; break; }
            if ((st = capture_frame(lc, b, f, band, dl ? b->ev_surf[f] : nullptr))) break;
            if (cudaEventRecordWithFlags(b->ev_end[f], lc->stream, cudaEventRecordExternal) != cudaSuccess) { st = PMS_ERR_CUDA; break; }
            last[l] = (int)f;
            if (!dl) continue;
            if (cudaStreamWaitEvent(dl->stream, b->ev_surf[f], 0) != cudaSuccess) {
                st = PMS_ERR_CUDA;
                break;
            }
            dview->point(lc, b, f);
            DiffuseBatch db;
            db.gen_cap = b->gen_cap;
            db.old_cap = b->old_cap;
            db.old_dev = b->dcnt.as<uint32_t>();
            db.frame_dev = b->dcnt.as<uint32_t>() + 1;
            db.frame_off = f;
            db.running = b->drun.as<unsigned long long>();
            db.base = b->dbase.as<unsigned long long>() + f;
            db.arena = b->darena.p;
            db.arena_cap = b->darena_cap;
            if ((st = launch_diffuse_bounded(dl, db))) break;
            if (cudaEventRecord(b->ev_diff[f], dl->stream) != cudaSuccess) st = PMS_ERR_CUDA;
        }
        if (dl) b->d_out = dl->d_old.p;
    }
    for (uint32_t l = 1; l < nlanes && !st; ++l) {
        if (cudaEventRecord(b->join[l - 1], lane_ctx(c, b, l)->stream) != cudaSuccess ||
            cudaStreamWaitEvent(c->stream, b->join[l - 1], 0) != cudaSuccess)
            st = PMS_ERR_CUDA;
    }
    if (dl && !st &&
        (cudaEventRecord(b->djoin, dl->stream) != cudaSuccess || cudaStreamWaitEvent(c->stream, b->djoin, 0) != cudaSuccess))
        st = PMS_ERR_CUDA;
    c->batch_launches = 0;
    for (uint32_t l = 0; l < nlanes; ++l) {
        pms_ctx* lc = lane_ctx(c, b, l);
        c->batch_launches += lc->launches - launches0[l];
        lc->launches = launches0[l];          // counted when the graph runs
    }
    if (dl) {
        c->batch_launches += dl->launches - dlaunches0;
        dl->launches = dlaunches0;
    }
    e = cudaStreamEndCapture(c->stream, &graph);
    if (st) {
        if (graph) cudaGraphDestroy(graph);
        // a lane's failure message lives on the lane
        for (uint32_t l = 1; l < nlanes; ++l)
            if (!lane_ctx(c, b, l)->last_error.empty()) c->last_error = lane_ctx(c, b, l)->last_error;
        if (dl && !dl->last_error.empty()) c->last_error = dl->last_error;
        return st;
    }
    if (e != cudaSuccess) return pms_fail(c, PMS_ERR_CUDA, "batch graph capture: %s", cudaGetErrorString(e));
    e = cudaGraphInstantiate(&b->exec, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) { b->exec = nullptr; return pms_fail(c, PMS_ERR_CUDA, "batch graph instantiate: %s", cudaGetErrorString(e)); }
    b->captures++;
    return PMS_OK;
}

// every buffer a lane's frames need, sized for the largest frame (nothing may allocate inside the graph)
static pms_status ensure_lane(pms_ctx* lc, pms_ctx* c, uint32_t nmax, const pms_grid& gmax,
                              const std::vector<pms_grid>& grid, bool learned) {
    pms_status st;
    if ((st = ensure_particle_buffers(lc, nmax))) return st;
    if ((st = ensure_grid_buffers(lc, gmax))) return st;
    if ((st = ensure_band_buffers(lc, gmax.sc_size))) return st;
    PMS_CUDA(lc, lc->scan.partial.ensure(sizeof(unsigned long long) * 1024));
    lc->tune = c->tune;
    lc->tc_wait_polls = c->tc_wait_polls;     // the debug wait limit holds on every lane
    if (!learned) return PMS_OK;
    const size_t S = (size_t)gmax.sc_size + 1;
    if ((st = ensure_learned_buffers(lc, gmax.sc_size, gmax.sc_size))) return st;
    size_t ncoarse = 1;
    for (const pms_grid& g : grid)
        ncoarse = std::max(ncoarse, (size_t)(g.scres[0] / 2 + 2) * (g.scres[1] / 2 + 2) * (g.scres[2] / 2 + 2));
    PMS_CUDA(lc, lc->l_counts.ensure(4 * ncoarse));
    size_t npad = 1;
    for (const pms_grid& g : grid)
        npad = std::max(npad, (size_t)(g.scres[0] / 2 + 3) * (g.scres[1] / 2 + 3) * (g.scres[2] / 2 + 3));
    PMS_CUDA(lc, lc->l_dens.ensure(4 * npad));    // padded coarse grid: cres + 1 per axis
    PMS_CUDA(lc, lc->l_clist.ensure(8 * S));
    if (lc != c && c->have_model) {
        // the lane reads the context's model
        PMS_CUDA(lc, lc->l_model.ensure(sizeof(pms_band_model)));
        PMS_CUDA(lc, cudaMemcpyAsync(lc->l_model.p, c->l_model.p, sizeof(pms_band_model), cudaMemcpyDeviceToDevice, c->stream));
        PMS_CUDA(lc, cudaStreamSynchronize(c->stream));
        lc->have_model = true;
    }
    return PMS_OK;
}

static pms_status check_frame_errors(pms_ctx* c, const Counters& h, uint32_t f) {
    if (h.err & kErrNonFinite) return pms_fail(c, PMS_ERR_INVALID_ARGUMENT, "frame %u: positions contain NaN or Inf", f);
    if (h.err & kErrBigCell) return pms_fail(c, PMS_ERR_UNSUPPORTED, "frame %u: a spatial cell holds more than 4096 particles", f);
    if (h.err & kErrKeyRange) return pms_fail(c, PMS_ERR_CUDA, "frame %u: internal: a cell key fell outside the grid", f);
    if (h.err & kErrTcLost)
        return pms_fail(c, PMS_ERR_CUDA, "frame %u: a tensor-core operation outlived two bounded waits; destroy this context", f);
    if (h.err & kErrTimeout) return pms_fail(c, PMS_ERR_CUDA, "frame %u: internal: a wait on the tensor cores timed out", f);
    return PMS_OK;
}

static inline float decode_ordered(uint32_t u) {
    uint32_t b = (u & 0x80000000u) ? (u & 0x7fffffffu) : ~u;
    float f;
    memcpy(&f, &b, 4);
    return f;
}

// the buffers a batch graph holds: every lane's, the diffuse lane's and the batch's own
static uint64_t batch_signature(pms_ctx* c, BatchState* b, uint32_t nlanes, bool diffuse) {
    uint64_t h = 0;
    for (uint32_t l = 0; l < nlanes; ++l) h = h * 31u + dbuf_signature(lane_ctx(c, b, l), false);
    if (diffuse && b->dlane) h = h * 31u + dbuf_signature(b->dlane, true);
    for (DBuf* x : {&b->pos, &b->vel, &b->rho, &b->cnt, &b->base, &b->mesh, &b->dcnt, &b->drun, &b->dbase, &b->darena,
                    &b->h_trunc})
        h = (h * 1099511628211ull) ^ (uint64_t)(uintptr_t)x->p ^ ((uint64_t)x->cap << 1);
    h = (h * 1099511628211ull) ^ (uint64_t)(uintptr_t)b->h_mesh_dev ^ (b->h_mesh_cap << 1);
    return h;
}

extern "C" pms_status pms_run_batch(pms_ctx* c, const pms_frame* frames, uint32_t k, int flags) {
    if (!c || (k && !frames)) return PMS_ERR_INVALID_ARGUMENT;
    const int band = (flags & PMS_BATCH_LEARNED) ? 1 : (flags & PMS_BATCH_CERTIFIED) ? 2 : 0;
    const bool learned = band != 0;          // the learned band's buffers and launches
    const bool diffuse = c->cfg.is_diffuse != 0;
    const int shape_flags = flags | (diffuse ? (1 << 16) : 0);
    if (band == 1 && !c->have_model) return pms_fail(c, PMS_ERR_STATE, "learned batch without a model");
    for (uint32_t f = 0; f < k; ++f)
        if (frames[f].n && !frames[f].pos_xyz) return pms_fail(c, PMS_ERR_INVALID_ARGUMENT, "frame %u: no positions", f);
    cudaSetDevice(c->device);
    // a single frame's velocity upload may still be in flight: order it before the batch
    // (whose captured sort must not wait on work outside the capture)
    if (c->vel_pending) {
        PMS_CUDA(c, cudaStreamWaitEvent(c->stream, c->vel_ready, 0));
        c->vel_pending = false;
    }
    BatchState* b = batch_of(c);
    if (k == 0) { b->n.clear(); b->hcnt.clear(); return PMS_OK; }
    // ---- pass 1: arena, uploads, bounding boxes
    uint64_t total = 0;
    std::vector<uint64_t> off(k);
    std::vector<uint32_t> n(k);
    uint32_t nmax = 0;
    for (uint32_t f = 0; f < k; ++f) { off[f] = total; n[f] = frames[f].n; total += n[f]; nmax = std::max(nmax, n[f]); }
    const size_t T = total ? total : 1;
    PMS_CUDA(c, b->pos.ensure(12 * T));
    PMS_CUDA(c, b->vel.ensure(12 * T));
    PMS_CUDA(c, b->rho.ensure(4 * T));
    PMS_CUDA(c, b->cnt.ensure(sizeof(Counters) * (k ? k : 1)));
    PMS_CUDA(c, b->base.ensure(sizeof(unsigned long long) * (k + 1)));
    const bool shape_same = b->n == n && b->flags == shape_flags;
    for (uint32_t f = 0; f < k; ++f) {
        const size_t m = n[f];
        if (!m) continue;
        PMS_CUDA(c, cudaMemcpyAsync(b->pos.as<char>() + 12 * off[f], frames[f].pos_xyz, 12 * m, cudaMemcpyDefault, c->stream));
        if (frames[f].vel_xyz)
            PMS_CUDA(c, cudaMemcpyAsync(b->vel.as<char>() + 12 * off[f], frames[f].vel_xyz, 12 * m, cudaMemcpyDefault, c->stream));
        else
            PMS_CUDA(c, cudaMemsetAsync(b->vel.as<char>() + 12 * off[f], 0, 12 * m, c->stream));
        if (frames[f].rhop)
            PMS_CUDA(c, cudaMemcpyAsync(b->rho.as<char>() + 4 * off[f], frames[f].rhop, 4 * m, cudaMemcpyDefault, c->stream));
        else
            PMS_CUDA(c, cudaMemsetAsync(b->rho.as<char>() + 4 * off[f], 0, 4 * m, c->stream));
    }
    b->n = n;
    b->off = off;
    b->flags = shape_flags;
    pms_status st;
    {
        FrameView view(c);
        for (uint32_t f = 0; f < k; ++f) {
            view.point(b, f, false);
            if ((st = launch_bbox(c))) return st;
        }
    }
    b->hcnt.resize(k);
    if (k) PMS_CUDA(c, cudaMemcpyAsync(b->hcnt.data(), b->cnt.p, sizeof(Counters) * k, cudaMemcpyDeviceToHost, c->stream));
    PMS_CUDA(c, cudaStreamSynchronize(c->stream));
    std::vector<pms_grid> grid(k);
    pms_grid gmax = {};
    for (uint32_t f = 0; f < k; ++f) {
        if ((st = check_frame_errors(c, b->hcnt[f], f))) return st;
        if (!n[f]) { memset(&grid[f], 0, sizeof(pms_grid)); continue; }
        float bmin[3], bmax[3];
        for (int a = 0; a < 3; ++a) { bmin[a] = decode_ordered(b->hcnt[f].bbox_min[a]); bmax[a] = decode_ordered(b->hcnt[f].bbox_max[a]); }
        if ((st = pms_grid_from_bbox(&c->prm, bmin, bmax, &grid[f]))) return pms_fail(c, st, "frame %u: grid too large", f);
        gmax.sp_size = std::max(gmax.sp_size, grid[f].sp_size);
        gmax.sc_size = std::max(gmax.sc_size, grid[f].sc_size);
        // rows of the largest frame (the per-row radii follow the per-cell ones)
        gmax.spres[1] = 1;
        gmax.spres[2] = std::max(gmax.spres[2], grid[f].spres[1] * grid[f].spres[2]);
    }
    bool grids_same = shape_same && b->grid.size() == k;
    for (uint32_t f = 0; grids_same && f < k; ++f) grids_same = same_grid(b->grid[f], grid[f]);
    b->grid = grid;
    // ---- lanes and their capacities (nothing may allocate inside the graph)
    const uint32_t nlanes = std::min<uint32_t>(kBatchLanes, k);
    while (b->lanes.size() + 1 < nlanes) {
        pms_ctx* lc = nullptr;
        pms_config lcfg = c->cfg;
        lcfg.band_model[0] = 0;
        if ((st = pms_create(&lcfg, c->device, &lc))) return pms_fail(c, st, "batch lane context");
        b->lanes.push_back(lc);
        cudaEvent_t e;
        PMS_CUDA(c, cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
        b->join.push_back(e);
    }
    if (!b->fork) PMS_CUDA(c, cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming));
    for (uint32_t l = 0; l < nlanes; ++l)
        if ((st = ensure_lane(lane_ctx(c, b, l), c, nmax, gmax, grid, learned))) return st;
    if (diffuse) {
        if (!b->dlane) {
            pms_config lcfg = c->cfg;
            lcfg.band_model[0] = 0;
            if ((st = pms_create(&lcfg, c->device, &b->dlane))) return pms_fail(c, st, "batch diffuse lane context");
            PMS_CUDA(c, cudaEventCreateWithFlags(&b->djoin, cudaEventDisableTiming));
        }
        while (b->ev_surf.size() < k) {
            cudaEvent_t e0, e1;
            PMS_CUDA(c, cudaEventCreateWithFlags(&e0, cudaEventDisableTiming));
            PMS_CUDA(c, cudaEventCreateWithFlags(&e1, cudaEventDisableTiming));
            b->ev_surf.push_back(e0);
            b->ev_diff.push_back(e1);
        }
        // capacities: generated and carried particles per frame, and the arena of every
        // frame's survivors (grown, and the batch run again, when a frame exceeds them)
        b->gen_cap = std::max(b->gen_cap, std::max<uint32_t>(1u << 18, nmax / 4));
        b->old_cap = std::max(b->old_cap, std::max<uint32_t>(1u << 20, 2 * c->diffuse_old));
        b->darena_cap = std::max<uint64_t>(b->darena_cap, (uint64_t)k * (b->old_cap / 2));
    }
    if (nlanes != b->nlanes_captured || c->tc_wait_polls != b->wait_captured) grids_same = false;
    uint64_t want_cap = 0;
    for (uint32_t f = 0; f < k; ++f) {
        const uint64_t sx = grid[f].scres[0], sy = grid[f].scres[1], sz = grid[f].scres[2];
        want_cap += std::min<uint64_t>(15ull * grid[f].sc_size, std::max<uint64_t>(1u << 20, 24ull * (sx * sy + sy * sz + sx * sz)));
    }
    if (want_cap > b->mesh_cap) { b->mesh_cap = want_cap; grids_same = false; }
    PMS_CUDA(c, b->mesh.ensure(12 * (b->mesh_cap ? b->mesh_cap : 1)));
    while (b->ev.size() < k + 1) {
        cudaEvent_t e0, e1;
        PMS_CUDA(c, cudaEventCreate(&e0));
        PMS_CUDA(c, cudaEventCreate(&e1));
        b->ev.push_back(e0);
        b->ev_end.push_back(e1);
    }
    // ---- pass 2: the graph (captured again when the frames' grids or any buffer changed)
    const int attempts = diffuse ? 8 : 3;
    for (int attempt = 0; attempt < attempts; ++attempt) {
        if (diffuse) {
            pms_ctx* dl = b->dlane;
            if ((st = ensure_diffuse_batch_buffers(dl, nmax, b->gen_cap, b->old_cap))) return st;
            PMS_CUDA(c, dl->scan.partial.ensure(sizeof(unsigned long long) * 1024));
            PMS_CUDA(c, b->dcnt.ensure(2 * sizeof(uint32_t)));
            PMS_CUDA(c, b->drun.ensure(sizeof(unsigned long long)));
            PMS_CUDA(c, b->dbase.ensure(sizeof(unsigned long long) * k));
            PMS_CUDA(c, b->darena.ensure(32 * (b->darena_cap ? b->darena_cap : 1)));
        }
        if (!grids_same || !b->exec || b->sig != batch_signature(c, b, nlanes, diffuse)) {
            if ((st = capture(c, b, band, nlanes, diffuse))) return st;
            b->sig = batch_signature(c, b, nlanes, diffuse);
            b->nlanes_captured = nlanes;
            b->wait_captured = c->tc_wait_polls;
            grids_same = true;
        }
        if (diffuse) {
            // the context's carried particles and frame counter enter the batch
            const uint32_t in[2] = {c->diffuse_old, c->frame_index};
            if (c->diffuse_old)
                PMS_CUDA(c, cudaMemcpyAsync(b->d_in, c->d_old.p, 32 * (size_t)c->diffuse_old, cudaMemcpyDeviceToDevice, c->stream));
            PMS_CUDA(c, cudaMemcpyAsync(b->dcnt.p, in, sizeof(in), cudaMemcpyHostToDevice, c->stream));
        }
        if (b->h_mesh_dev) PMS_CUDA(c, cudaMemsetAsync(b->h_trunc.p, 0, sizeof(uint32_t), c->stream));
        PMS_CUDA(c, cudaGraphLaunch(b->exec, c->stream));
        c->launches += c->batch_launches;
        b->hbase.resize(k + 1);
        if (k) PMS_CUDA(c, cudaMemcpyAsync(b->hcnt.data(), b->cnt.p, sizeof(Counters) * k, cudaMemcpyDeviceToHost, c->stream));
        PMS_CUDA(c, cudaMemcpyAsync(b->hbase.data(), b->base.p, sizeof(unsigned long long) * (k + 1), cudaMemcpyDeviceToHost,
                                    c->stream));
        PMS_CUDA(c, cudaStreamSynchronize(c->stream));
        bool overflow = false;
        for (uint32_t f = 0; f < k; ++f) {
            if ((st = check_frame_errors(c, b->hcnt[f], f))) return st;
            overflow |= (b->hcnt[f].err & kErrCapacity) != 0;
        }
        unsigned long long dfill = 0;
        if (diffuse) PMS_CUDA(c, cudaMemcpy(&dfill, b->drun.p, sizeof(dfill), cudaMemcpyDeviceToHost));
        if (!overflow) {
            uint32_t trunc = 0;
            if (b->h_mesh_dev) PMS_CUDA(c, cudaMemcpy(&trunc, b->h_trunc.p, sizeof(trunc), cudaMemcpyDeviceToHost));
            if (trunc)
                return pms_fail(c, PMS_ERR_CAPACITY, "the batch's meshes have %llu vertices, the host arena holds %llu",
                                (unsigned long long)b->hbase[k], (unsigned long long)b->h_mesh_cap);
            break;
        }
        if (attempt == attempts - 1) return pms_fail(c, PMS_ERR_CAPACITY, "batch capacity overflow");
        if (b->hbase[k] > b->mesh_cap) {
            b->mesh_cap = std::max<uint64_t>(2 * b->mesh_cap, b->hbase[k] + (b->hbase[k] >> 2));
            PMS_CUDA(c, b->mesh.ensure(12 * b->mesh_cap));
        }
        if (diffuse) {
            // a frame past a capacity: its count (and every later frame's) is a lower bound
            uint32_t gmax_seen = 0, omax_seen = 0;
            bool hit = false;
            for (uint32_t f = 0; f < k; ++f) {
                const Counters& h = b->hcnt[f];
                gmax_seen = std::max(gmax_seen, h.n_generated);
                omax_seen = std::max(omax_seen, h.n_live);
                hit |= (h.err & kErrCapacity) != 0 && h.n_generated > b->gen_cap;
            }
            if (hit) b->gen_cap = std::max<uint32_t>(2 * b->gen_cap, gmax_seen + (gmax_seen >> 2));
            if (omax_seen >= b->old_cap || hit) b->old_cap = std::max<uint32_t>(2 * b->old_cap, omax_seen + (omax_seen >> 2));
            if (dfill >= b->darena_cap || hit || omax_seen >= b->old_cap)
                b->darena_cap = std::max<uint64_t>(2 * b->darena_cap, dfill + (dfill >> 2));
            b->darena_cap = std::max<uint64_t>(b->darena_cap, (uint64_t)k * (b->old_cap / 2));
        }
        grids_same = false;
    }
    if (diffuse) {
        // the last frame's survivors leave the batch: the context's carried particles and
        // frame counter continue the sequence
        b->hdbase.resize(k);
        PMS_CUDA(c, cudaMemcpy(b->hdbase.data(), b->dbase.p, sizeof(unsigned long long) * k, cudaMemcpyDeviceToHost));
        const uint32_t last = std::min(b->hcnt[k - 1].n_live, b->old_cap);
        PMS_CUDA(c, c->d_old.ensure(32 * (size_t)(last ? last : 1)));
        if (last) PMS_CUDA(c, cudaMemcpyAsync(c->d_old.p, b->d_out, 32 * (size_t)last, cudaMemcpyDeviceToDevice, c->stream));
        PMS_CUDA(c, cudaStreamSynchronize(c->stream));
        c->diffuse_old = last;
        c->frame_index += k;
        c->have_diffuse = true;
    }
    return PMS_OK;
}

extern "C" pms_status pms_batch_frame(pms_ctx* c, uint32_t f, pms_counts* out, float* ms) {
    if (!c || !c->batch) return PMS_ERR_INVALID_ARGUMENT;
    BatchState* b = static_cast<BatchState*>(c->batch);
    if (f >= b->n.size()) return PMS_ERR_INVALID_ARGUMENT;
    const Counters& h = b->hcnt[f];
    if (out) {
        memset(out, 0, sizeof(*out));
        out->n_particles = b->n[f];
        out->n_surface_particles = h.ns;
        out->n_band_vertices = h.nv;
        out->n_valid_cubes = h.nvalid;
        out->n_mesh_vertices = h.nmesh;
        out->n_fp64_svd = h.n_fp64;
        if (b->flags & (1 << 16)) {
            out->n_free_surface = h.n_free;
            out->n_spawning = h.n_spawning;
            out->n_generated_diffuse = h.n_generated;
            out->n_diffuse = h.n_live;
            out->n_spray = h.n_type[0];
            out->n_foam = h.n_type[1];
            out->n_bubble = h.n_type[2];
        }
        if (b->flags & (PMS_BATCH_LEARNED | PMS_BATCH_CERTIFIED)) {
            out->n_band_candidates = h.l_cand;
            out->n_band_predicted = h.l_pred;
            out->n_band_exact = h.l_exact;
            out->n_band_certified = h.l_cert;
            out->n_band_rechecked = h.l_recheck;
        }
    }
    if (ms) {
        *ms = 0.f;
        if (cudaEventElapsedTime(ms, b->ev[f], b->ev_end[f]) != cudaSuccess) {
            *ms = 0.f;
            cudaGetLastError();                      // a missing time is not a failure of later calls
        }
    }
    return PMS_OK;
}

extern "C" pms_status pms_batch_mesh(pms_ctx* c, uint32_t f, float* pos, uint64_t cap, uint64_t* n_out) {
    if (!c || !c->batch || !n_out) return PMS_ERR_INVALID_ARGUMENT;
    BatchState* b = static_cast<BatchState*>(c->batch);
    if (f >= b->n.size()) return PMS_ERR_INVALID_ARGUMENT;
    const uint64_t m = b->hcnt[f].nmesh;
    *n_out = m;
    if (!pos) return PMS_OK;
    if (cap < m) return PMS_ERR_CAPACITY;
    cudaSetDevice(c->device);
    if (m) PMS_CUDA(c, cudaMemcpyAsync(pos, b->mesh.as<float>() + 3 * b->hbase[f], 12 * m, cudaMemcpyDeviceToHost, c->stream));
    PMS_CUDA(c, cudaStreamSynchronize(c->stream));
    return PMS_OK;
}

extern "C" pms_status pms_batch_stream_meshes(pms_ctx* c, float* pos, uint64_t cap) {
    if (!c) return PMS_ERR_INVALID_ARGUMENT;
    cudaSetDevice(c->device);
    BatchState* b = batch_of(c);
    float* dev = nullptr;
    if (pos && cudaHostGetDevicePointer((void**)&dev, pos, 0) != cudaSuccess) {
        cudaGetLastError();
        return pms_fail(c, PMS_ERR_INVALID_ARGUMENT, "the host mesh arena is not mapped page-locked memory");
    }
    if (pos) PMS_CUDA(c, b->h_trunc.ensure(sizeof(uint32_t)));
    b->h_mesh = pos;
    b->h_mesh_dev = pos ? dev : nullptr;
    b->h_mesh_cap = pos ? cap : 0;
    return PMS_OK;
}

extern "C" pms_status pms_batch_mesh_range(pms_ctx* c, uint32_t f, uint64_t* first, uint64_t* n_out) {
    if (!c || !c->batch || !first || !n_out) return PMS_ERR_INVALID_ARGUMENT;
    BatchState* b = static_cast<BatchState*>(c->batch);
    if (f >= b->n.size() || b->hbase.size() <= f) return PMS_ERR_INVALID_ARGUMENT;
    *first = b->hbase[f];
    *n_out = b->hcnt[f].nmesh;
    return PMS_OK;
}

extern "C" pms_status pms_batch_diffuse(pms_ctx* c, uint32_t f, pms_diffuse_particle* out, uint64_t cap, uint64_t* n_out) {
    if (!c || !c->batch || !n_out) return PMS_ERR_INVALID_ARGUMENT;
    BatchState* b = static_cast<BatchState*>(c->batch);
    if (f >= b->n.size()) return PMS_ERR_INVALID_ARGUMENT;
    if (!(b->flags & (1 << 16)) || b->hdbase.size() != b->n.size())
        return pms_fail(c, PMS_ERR_STATE, "the last batch ran without diffuse generation");
    const uint64_t m = b->hcnt[f].n_live;
    *n_out = m;
    if (!out) return PMS_OK;
    if (cap < m) return PMS_ERR_CAPACITY;
    cudaSetDevice(c->device);
    if (m) PMS_CUDA(c, cudaMemcpyAsync(out, b->darena.as<char>() + 32 * b->hdbase[f], 32 * m, cudaMemcpyDeviceToHost, c->stream));
    PMS_CUDA(c, cudaStreamSynchronize(c->stream));
    return PMS_OK;
}

extern "C" pms_status pms_batch_info(pms_ctx* c, uint32_t* graph_kernels, uint32_t* captures) {
    if (!c) return PMS_ERR_INVALID_ARGUMENT;
    BatchState* b = static_cast<BatchState*>(c->batch);
    if (graph_kernels) *graph_kernels = (uint32_t)c->batch_launches;
    if (captures) *captures = b ? b->captures : 0;
    return PMS_OK;
}
