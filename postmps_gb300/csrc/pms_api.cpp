// pms_api.cpp -- the C ABI of libpms: context lifetime, frame upload, stage
// orchestration, result download.  Mirrors the reference's host class chain
// (GPUPOST.cpp:20-96, NeighborSearch.cu:37-76, Anisotropic.cu:30-254,
// MarchingCube.cu:32-197, GPUmemory.cpp) with these differences:
//   * device buffers are grow-only and reused across frames instead of
//     cudaMalloc/cudaFree per stage;
//   * counts stay on the device; the host reads them only where it must size
//     the next buffers (grid, band, mesh) or return results;
//   * every failure is a returned pms_status with a message, never an abort.
#include <thread>

#include "pms_internal.h"

#include <cstdarg>
#include <algorithm>

using namespace pms;

pms_status pms_fail(pms_ctx* ctx, pms_status s, const char* fmt, ...) {
    char buf[1024];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    if (ctx) ctx->last_error = buf;
    return s;
}

extern "C" const char* pms_status_string(pms_status s) {
    switch (s) {
        case PMS_OK: return "ok";
        case PMS_ERR_INVALID_ARGUMENT: return "invalid argument";
        case PMS_ERR_CUDA: return "CUDA error";
        case PMS_ERR_OUT_OF_MEMORY: return "out of memory";
        case PMS_ERR_CAPACITY: return "capacity exceeded";
        case PMS_ERR_IO: return "I/O error";
        case PMS_ERR_CONFIG: return "configuration error";
        case PMS_ERR_STATE: return "stage called out of order";
        case PMS_ERR_TIMEOUT: return "device wait timed out";
        case PMS_ERR_UNSUPPORTED: return "unsupported input";
    }
    return "unknown status";
}

extern "C" const char* pms_last_error(const pms_ctx* ctx) { return ctx ? ctx->last_error.c_str() : "null context"; }

extern "C" uint64_t pms_kernel_launches(const pms_ctx* ctx) { return ctx ? ctx->launches : 0; }

// ---------------------------------------------------------------------------
// lifetime
// ---------------------------------------------------------------------------
// every device buffer of a context: released together, and their addresses sign a
// captured batch graph (the staging pair, swapped with the inputs, is released apart)
template <class F>
static void for_each_dbuf(pms_ctx* c, F f) {
    DBuf* bufs[] = {&c->in_pos, &c->in_vel, &c->in_rho, &c->keys, &c->slot, &c->order, &c->skeys, &c->spos,
                    &c->svel, &c->rho, &c->cell_count, &c->cell_start, &c->cell_info, &c->surf_count,
                    &c->surf_start, &c->big_cells, &c->slist, &c->moments, &c->cell_rad, &c->cell_rec, &c->aniso, &c->nrm4, &c->mean4, &c->gdebug,
                    &c->nnb, &c->bm0, &c->bm, &c->wcount, &c->wprefix, &c->vlist, &c->field, &c->mc_case,
                    &c->mc_key, &c->mc_off, &c->valid, &c->fdense, &c->cube, &c->fitems, &c->fitem_cnt, &c->fitem_off, &c->vert, &c->vnorm, &c->sval, &c->d_isfree, &c->d_freescan,
                    &c->d_freelist, &c->d_pot, &c->d_num, &c->d_numscan, &c->d_isdiff, &c->d_isdiffscan,
                    &c->d_difflist, &c->d_gen, &c->d_old, &c->d_all, &c->d_rand, &c->d_typescan,
                    &c->d_nrm_free, &c->d_tkey, &c->d_tscan, &c->d_perm, &c->counters, &c->scan.partial, &c->tmp,
                    &c->df_scan.partial, &c->df_tmp,
                    &c->l_dens, &c->l_clist, &c->l_counts, &c->l_model, &c->l_q, &c->l_cert, &c->l_e_bm, &c->l_e_wc,
                    &c->l_e_wp, &c->l_e_list, &c->l_n_bm, &c->l_n_wc, &c->l_n_wp, &c->l_n_list, &c->l_field_new,
                    &c->l_cand, &c->l_logit, &c->l_label, &c->tile_bits, &c->tile_wc, &c->tile_wp, &c->tile_list,
                    &c->w_bits, &c->w_wc, &c->w_wp, &c->w_vert, &c->w_vnorm, &c->w_idx};
    for (DBuf* b : bufs) f(*b);
}

static void release_all(pms_ctx* c) {
    for_each_dbuf(c, [](DBuf& b) { b.release(); });
}

uint64_t pms::dbuf_signature(pms_ctx* c, bool diffuse) {
    // the diffuse stage's buffers (d_*): used by a graph only on its diffuse lane
    const DBuf* dfirst[] = {&c->d_isfree, &c->d_freescan, &c->d_freelist, &c->d_pot, &c->d_num, &c->d_numscan,
                            &c->d_isdiff, &c->d_isdiffscan, &c->d_difflist, &c->d_gen, &c->d_old, &c->d_all,
                            &c->d_rand, &c->d_typescan, &c->d_nrm_free, &c->d_tkey, &c->d_tscan, &c->d_perm};
    uint64_t h = 1469598103934665603ull;
    for_each_dbuf(c, [&](DBuf& b) {
        if (!diffuse)
            for (const DBuf* d : dfirst)
                if (d == &b) return;
        h = (h ^ (uint64_t)(uintptr_t)b.p) * 1099511628211ull;
        h = (h ^ (uint64_t)b.cap) * 1099511628211ull;
    });
    return h;
}

extern "C" pms_status pms_create(const pms_config* cfg, int device, pms_ctx** out) {
    if (!cfg || !out) return PMS_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    pms_ctx* c = new (std::nothrow) pms_ctx();
    if (!c) return PMS_ERR_OUT_OF_MEMORY;
    c->cfg = *cfg;
    pms_status st = pms_params_derive(cfg, &c->prm);
    if (st != PMS_OK) { delete c; return st; }
    c->device = device >= 0 ? device : cfg->gpu_id;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) { delete c; return PMS_ERR_CUDA; }
    if (c->device >= ndev) { delete c; return PMS_ERR_INVALID_ARGUMENT; }
    if (cudaSetDevice(c->device) != cudaSuccess) { delete c; return PMS_ERR_CUDA; }
    if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess) { delete c; return PMS_ERR_CUDA; }
    c->own_stream = true;
    if (cudaHostAlloc(&c->h_counters, sizeof(Counters), cudaHostAllocMapped) != cudaSuccess) {
        cudaStreamDestroy(c->stream);
        delete c;
        return PMS_ERR_OUT_OF_MEMORY;
    }
    if (cudaHostGetDevicePointer((void**)&c->h_counters_dev, c->h_counters, 0) != cudaSuccess) {
        cudaFreeHost(c->h_counters);
        cudaStreamDestroy(c->stream);
        delete c;
        return PMS_ERR_CUDA;
    }
    memset(c->h_counters, 0, sizeof(Counters));
    for (int i = 0; i <= kNumStages; ++i) cudaEventCreate(&c->ev[i]);
    if (c->counters.ensure(sizeof(Counters)) != cudaSuccess || c->tmp.ensure(64) != cudaSuccess) {
        pms_destroy(c);
        return PMS_ERR_OUT_OF_MEMORY;
    }
    cudaMemsetAsync(c->counters.p, 0, sizeof(Counters), c->stream);
    st = upload_mc_tables(c);
    if (st != PMS_OK) { pms_destroy(c); return st; }
    if (cfg->band_model[0]) {
        pms_band_model m;
        if ((st = pms_load_band_model(cfg->band_model, &m)) != PMS_OK) { pms_destroy(c); return PMS_ERR_CONFIG; }
        if ((st = pms_set_band_model(c, &m)) != PMS_OK) { pms_destroy(c); return st; }
        c->band_mode = PMS_BAND_LEARNED;
    }
    *out = c;
    return PMS_OK;
}

extern "C" void pms_destroy(pms_ctx* c) {
    if (!c) return;
    cudaSetDevice(c->device);
    if (c->stream) cudaStreamSynchronize(c->stream);
    if (c->copy_stream) { cudaStreamSynchronize(c->copy_stream); cudaStreamDestroy(c->copy_stream); }
    if (c->up_stream) { cudaStreamSynchronize(c->up_stream); cudaStreamDestroy(c->up_stream); }
    if (c->up_start) cudaEventDestroy(c->up_start);
    if (c->vel_ready) cudaEventDestroy(c->vel_ready);
    if (c->df_stream) { cudaStreamSynchronize(c->df_stream); cudaStreamDestroy(c->df_stream); }
    if (c->df_fork) cudaEventDestroy(c->df_fork);
    if (c->df_join) cudaEventDestroy(c->df_join);
    if (c->mesh_ready) cudaEventDestroy(c->mesh_ready);
    if (c->diffuse_ready) cudaEventDestroy(c->diffuse_ready);
    for (OutQueue* q : {&c->mesh_q, &c->diffuse_q})
        for (cudaEvent_t e : q->ev) if (e) cudaEventDestroy(e);
    if (c->stage_stream) { cudaStreamSynchronize(c->stage_stream); cudaStreamDestroy(c->stage_stream); }
    if (c->stage_ready) cudaEventDestroy(c->stage_ready);
    if (c->stage_free) cudaEventDestroy(c->stage_free);
    if (c->stage_hpos) cudaFreeHost(c->stage_hpos);
    if (c->stage_hvel) cudaFreeHost(c->stage_hvel);
    c->st_pos.release();
    c->st_vel.release();
    pms_batch_release(c);
    release_all(c);
    for (int i = 0; i <= kNumStages; ++i) if (c->ev[i]) cudaEventDestroy(c->ev[i]);
    if (c->h_counters) cudaFreeHost(c->h_counters);
    if (c->own_stream && c->stream) cudaStreamDestroy(c->stream);
    delete c;
}

extern "C" pms_status pms_set_stream(pms_ctx* c, void* s) {
    if (!c) return PMS_ERR_INVALID_ARGUMENT;
    cudaStream_t ns = (cudaStream_t)s;
    if (!ns) {
        if (!c->own_stream) {
            if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess) return PMS_ERR_CUDA;
            c->own_stream = true;
        }
        return PMS_OK;
    }
    if (c->own_stream && c->stream) { cudaStreamSynchronize(c->stream); cudaStreamDestroy(c->stream); }
    c->stream = ns;
    c->own_stream = false;
    return PMS_OK;
}

// ---------------------------------------------------------------------------
// capacity
// ---------------------------------------------------------------------------
namespace pms {
pms_status ensure_particle_buffers(pms_ctx* c, uint32_t n);
pms_status ensure_grid_buffers(pms_ctx* c, const pms_grid& g);
}  // namespace pms
static pms_status ensure_particles(pms_ctx* c, uint32_t n) { return pms::ensure_particle_buffers(c, n); }
static pms_status ensure_grid(pms_ctx* c, const pms_grid& g) { return pms::ensure_grid_buffers(c, g); }

pms_status pms::ensure_particle_buffers(pms_ctx* c, uint32_t n) {
    const size_t N = n ? n : 1;
    PMS_CUDA(c, c->in_pos.ensure(12 * N));
    PMS_CUDA(c, c->in_vel.ensure(12 * N));
    PMS_CUDA(c, c->in_rho.ensure(4 * N));
    PMS_CUDA(c, c->keys.ensure(4 * N));
    PMS_CUDA(c, c->slot.ensure(4 * N));
    PMS_CUDA(c, c->order.ensure(4 * N));
    PMS_CUDA(c, c->skeys.ensure(4 * N));
    PMS_CUDA(c, c->spos.ensure(16 * N));
    PMS_CUDA(c, c->svel.ensure(16 * N));
    PMS_CUDA(c, c->rho.ensure(4 * N));
    PMS_CUDA(c, c->slist.ensure(4 * N));
    PMS_CUDA(c, c->moments.ensure(48 * N));
    PMS_CUDA(c, c->aniso.ensure(32 * N));
    PMS_CUDA(c, c->nrm4.ensure(16 * N));
    PMS_CUDA(c, c->mean4.ensure(16 * N));
    PMS_CUDA(c, c->gdebug.ensure(40 * N));
    PMS_CUDA(c, c->nnb.ensure(4 * N));
    PMS_CUDA(c, c->big_cells.ensure(4 * (N / 64 + 2)));
    return PMS_OK;
}

pms_status pms::ensure_grid_buffers(pms_ctx* c, const pms_grid& g) {
    const size_t S = g.sp_size ? g.sp_size : 1;
    PMS_CUDA(c, c->cell_count.ensure(4 * S));
    PMS_CUDA(c, c->cell_start.ensure(4 * (S + 1)));   // cell_start[S] = n
    PMS_CUDA(c, c->cell_info.ensure(8 * S));
    PMS_CUDA(c, c->surf_count.ensure(4 * S));
    PMS_CUDA(c, c->surf_start.ensure(4 * S));
    PMS_CUDA(c, c->cell_rad.ensure(4 * (S + (size_t)g.spres[1] * g.spres[2])));   // per cell, then per row
    PMS_CUDA(c, c->cell_rec.ensure(32 * S));   // two float4 per cell
    PMS_CUDA(c, c->fdense.ensure(4 * ((size_t)g.sc_size + 1)));
    const size_t W = ((uint64_t)g.sc_size + 31) / 32 + 1;
    PMS_CUDA(c, c->bm0.ensure(4 * W));
    PMS_CUDA(c, c->bm.ensure(4 * W));
    PMS_CUDA(c, c->wcount.ensure(4 * W));
    PMS_CUDA(c, c->wprefix.ensure(4 * W));
    // the band marking's tiles of the scalar grid: at most one per vertex
    const size_t T = (size_t)g.sc_size + 1, TW = T / 32 + 2;
    PMS_CUDA(c, c->tile_bits.ensure(4 * TW));
    PMS_CUDA(c, c->tile_wc.ensure(4 * TW));
    PMS_CUDA(c, c->tile_wp.ensure(4 * TW));
    PMS_CUDA(c, c->tile_list.ensure(4 * T));
    return PMS_OK;
}

namespace pms {
pms_status ensure_band_buffers(pms_ctx* c, uint32_t nv);
void mark_stage(pms_ctx* c, int boundary);
pms_status plain_band(pms_ctx* c);
}  // namespace pms

// the band's size changes from frame to frame: its buffers grow with headroom
pms_status pms::ensure_band_buffers(pms_ctx* c, uint32_t nv) {
    const size_t V = nv ? nv : 1;
    PMS_CUDA(c, c->vlist.ensure_grow(4 * V));
    PMS_CUDA(c, c->field.ensure_grow(4 * V));
    PMS_CUDA(c, c->mc_case.ensure_grow(4 * V));
    PMS_CUDA(c, c->mc_key.ensure_grow(8 * V));
    PMS_CUDA(c, c->mc_off.ensure_grow(8 * V));
    PMS_CUDA(c, c->valid.ensure_grow(4 * V));
    PMS_CUDA(c, c->cube.ensure_grow(16 * V));
    PMS_CUDA(c, c->fitems.ensure_grow(4 * (V + 1)));
    PMS_CUDA(c, c->fitem_cnt.ensure_grow(4 * (V + 1)));
    PMS_CUDA(c, c->fitem_off.ensure_grow(4 * (V + 1)));
    return PMS_OK;
}

extern "C" pms_status pms_reserve(pms_ctx* c, uint32_t max_particles, uint64_t max_scalar_vertices) {
    if (!c) return PMS_ERR_INVALID_ARGUMENT;
    cudaSetDevice(c->device);
    if (max_particles) { pms_status st = ensure_particles(c, max_particles); if (st) return st; }
    if (max_scalar_vertices) {
        if (max_scalar_vertices >= (1ull << 32)) return pms_fail(c, PMS_ERR_INVALID_ARGUMENT, "scalar grid above 2^32 vertices");
        pms_grid g = {};
        g.sc_size = (uint32_t)max_scalar_vertices;
        g.sp_size = (uint32_t)std::min<uint64_t>(max_scalar_vertices, 0xffffffffu);
        pms_status st = ensure_grid(c, g);
        if (st) return st;
    }
    return PMS_OK;
}

namespace pms {
pms_status copy_stream_ready(pms_ctx* c) {
    if (c->copy_stream) return PMS_OK;
    PMS_CUDA(c, cudaStreamCreateWithFlags(&c->copy_stream, cudaStreamNonBlocking));
    PMS_CUDA(c, cudaEventCreateWithFlags(&c->mesh_ready, cudaEventDisableTiming));
    PMS_CUDA(c, cudaEventCreateWithFlags(&c->diffuse_ready, cudaEventDisableTiming));
    for (OutQueue* q : {&c->mesh_q, &c->diffuse_q})
        for (cudaEvent_t& e : q->ev) PMS_CUDA(c, cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    return PMS_OK;
}

pms_status out_begin(pms_ctx* c, OutQueue& q, const void* host, int* slot) {
    int drop = 0;                          // records to drop from the head
    for (int i = 0; i < q.count; ++i)
        if (q.host[(q.head + i) % OutQueue::kSlots] == host) drop = i + 1;
    if (q.count - drop == OutQueue::kSlots) drop = 1;
    if (drop) PMS_CUDA(c, cudaEventSynchronize(q.ev[(q.head + drop - 1) % OutQueue::kSlots]));
    q.head = (q.head + drop) % OutQueue::kSlots;
    q.count -= drop;
    *slot = (q.head + q.count) % OutQueue::kSlots;
    return PMS_OK;
}

void out_push(OutQueue& q, int slot, const void* host, uint64_t n, uint64_t cap) {
    q.host[slot] = host;
    q.n[slot] = n;
    q.cap[slot] = cap;
    q.overflow[slot] = n > cap;
    q.last = slot;
    q.count++;
}

pms_status out_wait(pms_ctx* c, OutQueue& q, uint64_t* n, bool* overflow, uint64_t* cap) {
    const int h = q.head;
    PMS_CUDA(c, cudaEventSynchronize(q.ev[h]));
    q.head = (h + 1) % OutQueue::kSlots;
    q.count--;
    *n = q.n[h];
    *overflow = q.overflow[h];
    *cap = q.cap[h];
    return PMS_OK;
}

pms_status out_device_wait(pms_ctx* c, const OutQueue& q) {
    if (q.last >= 0) PMS_CUDA(c, cudaStreamWaitEvent(c->stream, q.ev[q.last], 0));
    return PMS_OK;
}

pms_status out_sync(pms_ctx* c, const OutQueue& q) {
    if (q.last >= 0) PMS_CUDA(c, cudaEventSynchronize(q.ev[q.last]));
    return PMS_OK;
}

pms_status sync_counters(pms_ctx* c) {
    pms_status st = launch_publish_counters(c);
    if (st) return st;
    PMS_CUDA(c, cudaStreamSynchronize(c->stream));
    return PMS_OK;
}
}  // namespace pms

static pms_status check_device_errors(pms_ctx* c) {
    const uint32_t e = c->h_counters->err;
    if (e & kErrNonFinite) return pms_fail(c, PMS_ERR_INVALID_ARGUMENT, "particle positions contain NaN or Inf");
    if (e & kErrBigCell)
        return pms_fail(c, PMS_ERR_UNSUPPORTED, "a spatial cell holds more than 4096 particles (particles nearly coincide)");
    if (e & kErrKeyRange) return pms_fail(c, PMS_ERR_CUDA, "internal: a cell key fell outside the grid");
    if (e & kErrCapacity) return pms_fail(c, PMS_ERR_CAPACITY, "internal: device capacity exceeded");
    if (e & kErrTcLost)
        return pms_fail(c, PMS_ERR_CUDA, "a tensor-core operation outlived two bounded waits; destroy this context");
    if (e & kErrTimeout) return pms_fail(c, PMS_ERR_CUDA, "internal: a wait on the tensor cores timed out");
    return PMS_OK;
}

// Stage timing: ev[0] opens a frame, ev[k + 1] closes stage k; a stage's time
// runs from the most recent earlier event.
void pms::mark_stage(pms_ctx* c, int boundary) {
    cudaEventRecord(c->ev[boundary], c->stream);
    if (boundary == 0) {
        c->last_event = 0;
        for (int i = 0; i < kNumStages; ++i) c->ev_recorded[i] = false;
        return;
    }
    c->ev_from[boundary - 1] = c->last_event;
    c->ev_recorded[boundary - 1] = true;
    c->last_event = boundary;
}
static void mark(pms_ctx* c, int boundary) { mark_stage(c, boundary); }
static pms_status ensure_band(pms_ctx* c, uint32_t nv) { return ensure_band_buffers(c, nv); }

// ---------------------------------------------------------------------------
// upload (FileData::loadFluidFile + GPUmemory::memAlcandCpy_fluid)
// ---------------------------------------------------------------------------
// a new frame's inputs are in place: every result of the last frame is stale
static void begin_frame(pms_ctx* c, uint32_t n) {
    c->n = n;
    c->have_particles = true;
    c->have_grid = c->have_aniso = c->have_band = c->have_field = c->have_mc = c->have_values = c->have_weld = false;
    c->band_learned = c->mc_classified = c->mc_compacted = false;
    c->l_ncand = c->l_npred = c->l_nexact = c->l_ncert = c->l_nrecheck = 0;
    c->ns = c->nv = c->nvalid = 0;
    c->nmesh = 0;
    for (int i = 0; i < kNumStages; ++i) c->ev_recorded[i] = false;
}

static pms_status upload_common(pms_ctx* c, const float* pos, const float* vel, const float* rho, uint32_t n,
                                cudaMemcpyKind kind) {
    if (!c || (n && !pos)) return PMS_ERR_INVALID_ARGUMENT;
    cudaSetDevice(c->device);
    pms_status st = ensure_particles(c, n);
    if (st) return st;
    if (n) {
        PMS_CUDA(c, cudaMemcpyAsync(c->in_pos.p, pos, 12 * (size_t)n, kind, c->stream));
        if (vel) {
            // the velocities are first read by the sort's gather: they travel on their own
            // stream while the bounding box, keys and counting sort run
            if (!c->up_stream) {
                PMS_CUDA(c, cudaStreamCreateWithFlags(&c->up_stream, cudaStreamNonBlocking));
                PMS_CUDA(c, cudaEventCreateWithFlags(&c->up_start, cudaEventDisableTiming));
                PMS_CUDA(c, cudaEventCreateWithFlags(&c->vel_ready, cudaEventDisableTiming));
            }
            PMS_CUDA(c, cudaEventRecord(c->up_start, c->stream));
            PMS_CUDA(c, cudaStreamWaitEvent(c->up_stream, c->up_start, 0));
            PMS_CUDA(c, cudaMemcpyAsync(c->in_vel.p, vel, 12 * (size_t)n, kind, c->up_stream));
            PMS_CUDA(c, cudaEventRecord(c->vel_ready, c->up_stream));
            c->vel_pending = true;
        } else {
            PMS_CUDA(c, cudaMemsetAsync(c->in_vel.p, 0, 12 * (size_t)n, c->stream));
            c->vel_pending = false;
        }
        // the input density is not read: every stage uses the density recomputed from
        // the positions (the reference overwrites Rhop before its first use,
        // Anisotropic_kernel.cuh:212), so it is not copied
        (void)rho;
    }
    begin_frame(c, n);
    return PMS_OK;
}

extern "C" pms_status pms_upload_particles(pms_ctx* c, const float* pos, const float* vel, const float* rho, uint32_t n) {
    return upload_common(c, pos, vel, rho, n, cudaMemcpyHostToDevice);
}
extern "C" pms_status pms_upload_particles_device(pms_ctx* c, const float* pos, const float* vel, const float* rho, uint32_t n) {
    return upload_common(c, pos, vel, rho, n, cudaMemcpyDeviceToDevice);
}

// host copy split over the host's threads (the staging copy of a multi-megabyte frame)
static void copy_parallel(void* dst, const void* src, size_t bytes) {
    const unsigned hw = std::thread::hardware_concurrency();
    const size_t T = std::max<size_t>(1, std::min<size_t>(hw ? hw : 1, bytes >> 22));
    if (T == 1) { memcpy(dst, src, bytes); return; }
    std::vector<std::thread> th;
    for (size_t k = 0; k < T; ++k)
        th.emplace_back([=]() {
            const size_t a = bytes * k / T, b = bytes * (k + 1) / T;
            memcpy(static_cast<char*>(dst) + a, static_cast<const char*>(src) + a, b - a);
        });
    for (std::thread& t : th) t.join();
}

// The staged upload.  Staging touches only its own members (pinned host buffers, a
// second pair of device input buffers, its stream and events, under stage_mu), so a
// thread may stage frame k + 1 while another runs frame k on the same context; it
// reports failures by status only (the message slot belongs to the frame's thread).
extern "C" pms_status pms_stage_particles(pms_ctx* c, const float* pos, const float* vel, const float* rho, uint32_t n) {
    if (!c || (n && !pos)) return PMS_ERR_INVALID_ARGUMENT;
    (void)rho;                                   // recomputed, as for pms_upload_particles
    if (cudaSetDevice(c->device) != cudaSuccess) return PMS_ERR_CUDA;
    std::lock_guard<std::mutex> lock(c->stage_mu);
    if (c->staged) return PMS_ERR_STATE;         // the frame staged before was not taken yet
    if (!c->stage_stream) {
        if (cudaStreamCreateWithFlags(&c->stage_stream, cudaStreamNonBlocking) != cudaSuccess ||
            cudaEventCreateWithFlags(&c->stage_ready, cudaEventDisableTiming) != cudaSuccess ||
            cudaEventCreateWithFlags(&c->stage_free, cudaEventDisableTiming) != cudaSuccess)
            return PMS_ERR_CUDA;
    }
    const size_t bytes = 12 * (size_t)n;
    // the previous staged copy has left the pinned buffers before they are refilled
    if (cudaStreamSynchronize(c->stage_stream) != cudaSuccess) return PMS_ERR_CUDA;
    if (c->stage_hcap < bytes) {
        if (c->stage_hpos) cudaFreeHost(c->stage_hpos);
        if (c->stage_hvel) cudaFreeHost(c->stage_hvel);
        c->stage_hpos = c->stage_hvel = nullptr;
        c->stage_hcap = 0;
        if (cudaMallocHost(&c->stage_hpos, bytes) != cudaSuccess || cudaMallocHost(&c->stage_hvel, bytes) != cudaSuccess)
            return PMS_ERR_OUT_OF_MEMORY;
        c->stage_hcap = bytes;
    }
    if (c->st_pos.ensure(bytes ? bytes : 12) != cudaSuccess || c->st_vel.ensure(bytes ? bytes : 12) != cudaSuccess)
        return PMS_ERR_OUT_OF_MEMORY;
    // the device buffers held the inputs of a frame that pms_upload_staged retired
    if (c->stage_free_recorded && cudaStreamWaitEvent(c->stage_stream, c->stage_free, 0) != cudaSuccess) return PMS_ERR_CUDA;
    if (n) {
        copy_parallel(c->stage_hpos, pos, bytes);
        if (vel) copy_parallel(c->stage_hvel, vel, bytes);
        else memset(c->stage_hvel, 0, bytes);
        if (cudaMemcpyAsync(c->st_pos.p, c->stage_hpos, bytes, cudaMemcpyHostToDevice, c->stage_stream) != cudaSuccess ||
            cudaMemcpyAsync(c->st_vel.p, c->stage_hvel, bytes, cudaMemcpyHostToDevice, c->stage_stream) != cudaSuccess)
            return PMS_ERR_CUDA;
    }
    if (cudaEventRecord(c->stage_ready, c->stage_stream) != cudaSuccess) return PMS_ERR_CUDA;
    c->staged_n = n;
    c->staged = true;
    return PMS_OK;
}

extern "C" pms_status pms_upload_staged(pms_ctx* c) {
    if (!c) return PMS_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lock(c->stage_mu);
    if (!c->staged) return pms_fail(c, PMS_ERR_STATE, "pms_upload_staged without a frame from pms_stage_particles");
    cudaSetDevice(c->device);
    const uint32_t n = c->staged_n;
    // a velocity copy of a direct upload may still be in flight into the buffer retired below
    if (c->vel_pending) {
        PMS_CUDA(c, cudaStreamWaitEvent(c->stream, c->vel_ready, 0));
        c->vel_pending = false;
    }
    // the staged buffers become the inputs (they hold n particles, so nothing regrows them)
    std::swap(c->in_pos, c->st_pos);
    std::swap(c->in_vel, c->st_vel);
    c->staged = false;
    pms_status st = ensure_particles(c, n);
    if (st) return st;
    PMS_CUDA(c, cudaStreamWaitEvent(c->stream, c->stage_ready, 0));
    // the retired buffers are free once the work enqueued before this point has run
    PMS_CUDA(c, cudaEventRecord(c->stage_free, c->stream));
    c->stage_free_recorded = true;
    begin_frame(c, n);
    return PMS_OK;
}

// ---------------------------------------------------------------------------
// stages
// ---------------------------------------------------------------------------
static inline float decode_ordered(uint32_t u) {
    uint32_t b = (u & 0x80000000u) ? (u & 0x7fffffffu) : ~u;
    float f;
    memcpy(&f, &b, 4);
    return f;
}

extern "C" pms_status pms_build_grid(pms_ctx* c) {
    if (!c) return PMS_ERR_INVALID_ARGUMENT;
    if (!c->have_particles) return pms_fail(c, PMS_ERR_STATE, "pms_build_grid before pms_upload_particles");
    cudaSetDevice(c->device);
    mark(c, kStageGrid);
    pms_status st = launch_bbox(c);
    if (st) return st;
    if ((st = sync_counters(c))) return st;
    if ((st = check_device_errors(c))) return st;
    if (c->n == 0) {
        memset(&c->grid, 0, sizeof(c->grid));
        c->have_grid = true;
        mark(c, kStageGrid + 1);
        return PMS_OK;
    }
    float bmin[3], bmax[3];
    for (int k = 0; k < 3; ++k) { bmin[k] = decode_ordered(c->h_counters->bbox_min[k]); bmax[k] = decode_ordered(c->h_counters->bbox_max[k]); }
    if ((st = pms_grid_from_bbox(&c->prm, bmin, bmax, &c->grid))) return pms_fail(c, st, "grid: domain too large for 32-bit cell indices");
    if ((st = ensure_grid(c, c->grid))) return st;
    if ((st = launch_hash_sort(c))) return st;
    c->have_grid = true;
    mark(c, kStageGrid + 1);
    return PMS_OK;
}

extern "C" pms_status pms_anisotropy(pms_ctx* c) {
    if (!c) return PMS_ERR_INVALID_ARGUMENT;
    if (!c->have_grid) return pms_fail(c, PMS_ERR_STATE, "pms_anisotropy before pms_build_grid");
    cudaSetDevice(c->device);
    if (c->n == 0) { c->have_aniso = true; return PMS_OK; }
    pms_status st;
    if ((st = launch_surface_cells(c))) return st;
    if ((st = launch_density_aniso(c))) return st;
    c->have_aniso = true;
    mark(c, kStageAniso + 1);
    return PMS_OK;
}

// The plain band's bitmap, count and ascending vertex list (one synchronisation).
pms_status pms::plain_band(pms_ctx* c) {
    pms_status st;
    if ((st = launch_band(c))) return st;
    if ((st = sync_counters(c))) return st;
    if ((st = check_device_errors(c))) return st;
    c->ns = c->h_counters->ns;
    c->nv = c->h_counters->nv;
    if ((st = ensure_band(c, c->nv))) return st;
    return launch_band_list(c);
}

extern "C" pms_status pms_band(pms_ctx* c) {
    if (!c) return PMS_ERR_INVALID_ARGUMENT;
    if (!c->have_aniso) return pms_fail(c, PMS_ERR_STATE, "pms_band before pms_anisotropy");
    cudaSetDevice(c->device);
    c->band_learned = c->mc_classified = c->mc_compacted = false;
    c->l_ncand = c->l_npred = c->l_nexact = c->l_ncert = c->l_nrecheck = 0;
    if (c->n == 0) { c->nv = 0; c->have_band = true; return PMS_OK; }
    pms_status st;
    if ((st = plain_band(c))) return st;
    c->have_band = true;
    mark(c, kStageBand + 1);
    return PMS_OK;
}

extern "C" pms_status pms_field(pms_ctx* c) {
    if (!c) return PMS_ERR_INVALID_ARGUMENT;
    if (!c->have_band) return pms_fail(c, PMS_ERR_STATE, "pms_field before pms_band");
    cudaSetDevice(c->device);
    if (c->nv) { pms_status st = launch_field(c); if (st) return st; }
    c->have_field = true;
    mark(c, kStageField + 1);
    return PMS_OK;
}

extern "C" pms_status pms_marching_cubes(pms_ctx* c) {
    if (!c) return PMS_ERR_INVALID_ARGUMENT;
    if (!c->have_field) return pms_fail(c, PMS_ERR_STATE, "pms_marching_cubes before pms_field");
    cudaSetDevice(c->device);
    c->nvalid = 0;
    c->nmesh = 0;
    c->have_weld = false;
    int slot = -1;                     // the frame's record in the streamed-mesh queue
    if (c->nv) {
        pms_status st;
        // the learned band's last border check already computed the final vertex set's cases
        if (!c->mc_classified && (st = launch_mc_cases(c))) return st;
        if (!(c->mc_classified && c->mc_compacted)) {
            if ((st = launch_mc_compact(c))) return st;
            if ((st = sync_counters(c))) return st;
        }
        c->nvalid = c->h_counters->nvalid;
        c->nmesh = c->h_counters->nmesh;
        const size_t M = c->nmesh ? c->nmesh : 1;
        // earlier frames' meshes may still be on their way to the host: a buffer that
        // grows waits for them on the host (its old allocation is freed), the emission
        // on the device
        c->mesh_normals = c->out_pos && c->out_nrm;
        if (c->vert.cap < 12 * M || (c->mesh_normals && c->vnorm.cap < 12 * M)) PMS_CHECK(out_sync(c, c->mesh_q));
        PMS_CUDA(c, c->vert.ensure_grow(12 * M));
        if (c->mesh_normals) PMS_CUDA(c, c->vnorm.ensure_grow(12 * M));
        PMS_CHECK(out_device_wait(c, c->mesh_q));
        // a streamed mesh goes in pieces: the emission runs in vertex ranges and each
        // piece travels on the copy stream while the next is made and the stages after run
        if (c->out_pos) PMS_CHECK(out_begin(c, c->mesh_q, c->out_pos, &slot));
        const bool copy = c->out_pos && c->nmesh <= c->out_cap;
        // with an earlier frame's mesh still pending, the caller keeps frames in flight and this
        // copy overlaps the next frame: one range, without the ranges' bounds and extra launches
        const bool in_flight = c->mesh_q.count > 0;
        const uint32_t pieces = copy ? (c->nmesh >= (1u << 16) && !in_flight ? (uint32_t)kMaxMcPieces : 1u) : 0u;
        if (!pieces && (st = launch_mc_emit(c))) return st;
        if (pieces > 1u && (st = launch_mc_piece_bounds(c, pieces))) return st;
        for (uint32_t q = 0; q < pieces; ++q) {
            const uint32_t v_lo = (uint32_t)((uint64_t)c->nmesh * q / pieces);
            const uint32_t v_end = (uint32_t)((uint64_t)c->nmesh * (q + 1) / pieces);
            if ((st = launch_mc_emit(c, pieces > 1u ? (int)q : -1, pieces))) return st;
            PMS_CUDA(c, cudaEventRecord(c->mesh_ready, c->stream));
            PMS_CUDA(c, cudaStreamWaitEvent(c->copy_stream, c->mesh_ready, 0));
            PMS_CUDA(c, cudaMemcpyAsync(c->out_pos + 3 * (size_t)v_lo, c->vert.as<float>() + 3 * (size_t)v_lo,
                                        12 * (size_t)(v_end - v_lo), cudaMemcpyDeviceToHost, c->copy_stream));
            if (c->out_nrm)
                PMS_CUDA(c, cudaMemcpyAsync(c->out_nrm + 3 * (size_t)v_lo, c->vnorm.as<float>() + 3 * (size_t)v_lo,
                                            12 * (size_t)(v_end - v_lo), cudaMemcpyDeviceToHost, c->copy_stream));
        }
    }
    if (c->out_pos) {
        if (slot < 0) PMS_CHECK(out_begin(c, c->mesh_q, c->out_pos, &slot));
        PMS_CUDA(c, cudaEventRecord(c->mesh_q.ev[slot], c->copy_stream));
        out_push(c->mesh_q, slot, c->out_pos, c->nmesh, c->out_cap);
    }
    c->have_mc = true;
    mark(c, kStageMc + 1);
    return PMS_OK;
}

extern "C" pms_status pms_scalar_values(pms_ctx* c) {
    if (!c) return PMS_ERR_INVALID_ARGUMENT;
    if (!c->have_mc) return pms_fail(c, PMS_ERR_STATE, "pms_scalar_values before pms_marching_cubes");
    cudaSetDevice(c->device);
    PMS_CUDA(c, c->sval.ensure(20 * (size_t)(c->nmesh ? c->nmesh : 1)));
    if (c->nmesh) { pms_status st = launch_scalar_values(c); if (st) return st; }
    c->have_values = true;
    return PMS_OK;
}

extern "C" pms_status pms_download_scalar_values(pms_ctx* c, float* vel_xyz, float* vel_len, float* rhop, uint64_t cap,
                                                 uint64_t* n_out) {
    if (!c || !n_out) return PMS_ERR_INVALID_ARGUMENT;
    if (!c->have_values) return pms_fail(c, PMS_ERR_STATE, "pms_download_scalar_values before pms_scalar_values");
    cudaSetDevice(c->device);
    const uint64_t m = c->nmesh;
    *n_out = m;
    if (!vel_xyz && !vel_len && !rhop) return PMS_OK;
    if (cap < m) return PMS_ERR_CAPACITY;
    std::vector<float> sv(5 * (size_t)m);
    if (m) PMS_CUDA(c, cudaMemcpyAsync(sv.data(), c->sval.p, 20 * (size_t)m, cudaMemcpyDeviceToHost, c->stream));
    PMS_CUDA(c, cudaStreamSynchronize(c->stream));
    for (uint64_t i = 0; i < m; ++i) {
        if (vel_xyz) { vel_xyz[3 * i] = sv[5 * i]; vel_xyz[3 * i + 1] = sv[5 * i + 1]; vel_xyz[3 * i + 2] = sv[5 * i + 2]; }
        if (vel_len) vel_len[i] = sv[5 * i + 3];
        if (rhop) rhop[i] = sv[5 * i + 4];
    }
    return PMS_OK;
}

extern "C" pms_status pms_surface(pms_ctx* c) {
    pms_status st;
    if ((st = pms_anisotropy(c))) return st;
    if ((st = pms_band(c))) return st;
    if ((st = pms_field(c))) return st;
    return pms_marching_cubes(c);
}

extern "C" pms_status pms_diffuse(pms_ctx* c) {
    if (!c) return PMS_ERR_INVALID_ARGUMENT;
    if (!c->have_grid) return pms_fail(c, PMS_ERR_STATE, "pms_diffuse before pms_build_grid");
    cudaSetDevice(c->device);
    pms_status st = launch_diffuse(c);
    if (st) return st;
    c->have_diffuse = true;
    mark(c, kStageDiffuse + 1);
    return PMS_OK;
}

// The diffuse parts are issued on the context's diffuse stream with their own scan
// scratch: the context's stream and scratch are swapped for them while in scope.
namespace {
struct OnDiffuseStream {
    pms_ctx* c;
    explicit OnDiffuseStream(pms_ctx* ctx) : c(ctx) { swap(); }
    ~OnDiffuseStream() { swap(); }
    void swap() {
        std::swap(c->stream, c->df_stream);
        std::swap(c->scan.partial, c->df_scan.partial);
        std::swap(c->tmp, c->df_tmp);
    }
};

// Joins the diffuse stream back into the context's stream when the frame ends, on
// every path: work of a frame that failed half way must not run into the next one.
struct DiffuseJoin {
    pms_ctx* c;
    ~DiffuseJoin() {
        cudaEventRecord(c->df_join, c->df_stream);
        cudaStreamWaitEvent(c->stream, c->df_join, 0);
    }
};
}  // namespace

// A frame with surface reconstruction and diffuse generation: the diffuse stage
// depends only on the grid and the anisotropy pass, and the surface stages only on
// those too, so after the anisotropy the diffuse parts run on a stream of their own
// beside the band, field and marching cubes.  Each part is issued where the surface
// chain has a long stretch of work queued: the front before the band's
// synchronisation, the tail after the field is queued, the finish after the emission.
// Results are those of the stages one after the other (no stage reads what the other
// chain writes; counters are separate fields, errors are OR-ed).
static pms_status run_frame_overlapped(pms_ctx* c) {
    pms_status st;
    if (!c->df_stream) {
        int lo = 0, hi = 0;
        PMS_CUDA(c, cudaDeviceGetStreamPriorityRange(&lo, &hi));
        PMS_CUDA(c, cudaStreamCreateWithPriority(&c->df_stream, cudaStreamNonBlocking, lo));
        PMS_CUDA(c, cudaEventCreateWithFlags(&c->df_fork, cudaEventDisableTiming));
        PMS_CUDA(c, cudaEventCreateWithFlags(&c->df_join, cudaEventDisableTiming));
        PMS_CUDA(c, c->df_tmp.ensure(64));
    }
    if ((st = pms_anisotropy(c))) return st;
    PMS_CUDA(c, cudaEventRecord(c->df_fork, c->stream));
    PMS_CUDA(c, cudaStreamWaitEvent(c->df_stream, c->df_fork, 0));
    DiffuseJoin join{c};
    {
        OnDiffuseStream d(c);
        if ((st = diffuse_part_front(c))) return st;
    }
    if (c->band_mode != PMS_BAND_PLAIN) {
        if ((st = pms_band_learned(c))) return st;
    } else {
        if ((st = pms_band(c))) return st;
        if ((st = pms_field(c))) return st;
    }
    {
        OnDiffuseStream d(c);
        if ((st = diffuse_part_tail(c))) return st;
    }
    if ((st = pms_marching_cubes(c))) return st;
    {
        OnDiffuseStream d(c);
        if ((st = diffuse_part_finish(c))) return st;
        // the diffuse stage's time runs from the anisotropy's end, where it forked
        PMS_CUDA(c, cudaEventRecord(c->ev[kStageDiffuse + 1], c->stream));
    }
    c->ev_from[kStageDiffuse] = kStageAniso + 1;
    c->ev_recorded[kStageDiffuse] = true;
    c->have_diffuse = true;
    return PMS_OK;                     // join: the frame's stream waits for the diffuse stream
}

extern "C" pms_status pms_run_frame(pms_ctx* c) {
    if (!c) return PMS_ERR_INVALID_ARGUMENT;
    pms_status st;
    if ((st = pms_build_grid(c))) return st;
    if (c->cfg.is_surface && c->cfg.is_diffuse) {
        if ((st = run_frame_overlapped(c))) return st;
    } else {
        if (c->cfg.is_surface && (st = c->band_mode != PMS_BAND_PLAIN ? pms_surface_learned(c) : pms_surface(c))) return st;
        if (c->cfg.is_diffuse && (st = pms_diffuse(c))) return st;
    }
    c->frame_index++;
    return PMS_OK;
}

// ---------------------------------------------------------------------------
// results
// ---------------------------------------------------------------------------
extern "C" pms_status pms_get_counts(pms_ctx* c, pms_counts* out) {
    if (!c || !out) return PMS_ERR_INVALID_ARGUMENT;
    cudaSetDevice(c->device);
    pms_status st = sync_counters(c);
    if (st) return st;
    const Counters& h = *c->h_counters;
    memset(out, 0, sizeof(*out));
    out->n_particles = c->n;
    out->n_surface_particles = c->have_aniso ? h.ns : 0;
    out->n_band_vertices = c->have_band ? h.nv : 0;
    out->n_valid_cubes = c->have_mc ? h.nvalid : 0;
    out->n_mesh_vertices = c->have_mc ? h.nmesh : 0;
    out->n_fp64_svd = h.n_fp64;
    out->n_field_pairs = c->have_field ? h.n_pairs : 0;
    out->n_free_surface = h.n_free;
    out->n_generated_diffuse = h.n_generated;
    out->n_spawning = h.n_spawning;
    out->n_diffuse = c->diffuse_old;
    out->n_spray = h.n_type[0];
    out->n_foam = h.n_type[1];
    out->n_bubble = h.n_type[2];
    if (c->band_learned) {
        out->n_band_candidates = c->l_ncand;
        out->n_band_predicted = c->l_npred;
        out->n_band_exact = c->l_nexact;
        out->n_band_certified = c->l_ncert;
        out->n_band_rechecked = c->l_nrecheck;
    }
    return check_device_errors(c);
}

extern "C" pms_status pms_get_grid(pms_ctx* c, pms_grid* out) {
    if (!c || !out) return PMS_ERR_INVALID_ARGUMENT;
    if (!c->have_grid) return pms_fail(c, PMS_ERR_STATE, "no grid yet");
    *out = c->grid;
    return PMS_OK;
}

extern "C" pms_status pms_download_mesh(pms_ctx* c, float* pos, float* nrm, uint64_t cap, uint64_t* n_out) {
    if (!c) return PMS_ERR_INVALID_ARGUMENT;
    if (!c->have_mc) return pms_fail(c, PMS_ERR_STATE, "no mesh yet");
    cudaSetDevice(c->device);
    if (n_out) *n_out = c->nmesh;
    if (c->nmesh == 0) return PMS_OK;
    if (cap < c->nmesh || !pos) return pms_fail(c, PMS_ERR_CAPACITY, "mesh has %llu vertices", (unsigned long long)c->nmesh);
    if (nrm && !c->mesh_normals) {
        // the normals on demand: the emission once more, with them (same positions)
        PMS_CHECK(out_sync(c, c->mesh_q));
        PMS_CUDA(c, c->vnorm.ensure(12 * c->nmesh));
        c->mesh_normals = true;
        pms_status st = launch_mc_emit(c);
        if (st) return st;
    }
    PMS_CUDA(c, cudaMemcpyAsync(pos, c->vert.p, 12 * c->nmesh, cudaMemcpyDeviceToHost, c->stream));
    if (nrm) PMS_CUDA(c, cudaMemcpyAsync(nrm, c->vnorm.p, 12 * c->nmesh, cudaMemcpyDeviceToHost, c->stream));
    PMS_CUDA(c, cudaStreamSynchronize(c->stream));
    return PMS_OK;
}

extern "C" pms_status pms_weld_mesh(pms_ctx* c, int normals) {
    if (!c) return PMS_ERR_INVALID_ARGUMENT;
    if (!c->have_mc) return pms_fail(c, PMS_ERR_STATE, "pms_weld_mesh before pms_marching_cubes");
    cudaSetDevice(c->device);
    c->w_nvert = 0;
    c->weld_normals = normals != 0;
    if (c->nmesh) {
        const uint64_t nw = (3ull * c->grid.sc_size + 31) / 32;
        PMS_CUDA(c, c->w_bits.ensure(4 * (nw + 1)));
        PMS_CUDA(c, c->w_wc.ensure(4 * (nw + 1)));
        PMS_CUDA(c, c->w_wp.ensure(4 * (nw + 1)));
        // at most one welded vertex per soup vertex
        PMS_CUDA(c, c->w_vert.ensure(12 * c->nmesh));
        if (normals) PMS_CUDA(c, c->w_vnorm.ensure(12 * c->nmesh));
        PMS_CUDA(c, c->w_idx.ensure(4 * c->nmesh));
        Counters* cnt = c->counters.as<Counters>();
        pms_status st = launch_weld(c, c->w_bits.as<uint32_t>(), c->w_wc.as<uint32_t>(), c->w_wp.as<uint32_t>(), nw,
                                    &cnt->n_weld, c->nmesh, c->w_vert.as<float>(), normals ? c->w_vnorm.as<float>() : nullptr,
                                    c->w_idx.as<uint32_t>());
        if (st) return st;
        if ((st = sync_counters(c))) return st;
        c->w_nvert = c->h_counters->n_weld;
        if (c->w_nvert > c->nmesh) return pms_fail(c, PMS_ERR_CAPACITY, "welded mesh has more vertices than the soup");
    }
    c->have_weld = true;
    return PMS_OK;
}

extern "C" pms_status pms_download_welded_mesh(pms_ctx* c, float* pos, float* nrm, uint64_t cap_vertices, uint32_t* indices,
                                               uint64_t cap_indices, uint64_t* n_vertices, uint64_t* n_indices) {
    if (!c) return PMS_ERR_INVALID_ARGUMENT;
    if (!c->have_weld) return pms_fail(c, PMS_ERR_STATE, "pms_download_welded_mesh before pms_weld_mesh");
    if (nrm && !c->weld_normals) return pms_fail(c, PMS_ERR_STATE, "the welded mesh was made without normals");
    cudaSetDevice(c->device);
    if (n_vertices) *n_vertices = c->w_nvert;
    if (n_indices) *n_indices = c->nmesh;
    if ((pos || nrm) && cap_vertices < c->w_nvert)
        return pms_fail(c, PMS_ERR_CAPACITY, "welded mesh has %llu vertices", (unsigned long long)c->w_nvert);
    if (indices && cap_indices < c->nmesh)
        return pms_fail(c, PMS_ERR_CAPACITY, "welded mesh has %llu indices", (unsigned long long)c->nmesh);
    if (pos && c->w_nvert) PMS_CUDA(c, cudaMemcpyAsync(pos, c->w_vert.p, 12 * c->w_nvert, cudaMemcpyDeviceToHost, c->stream));
    if (nrm && c->w_nvert) PMS_CUDA(c, cudaMemcpyAsync(nrm, c->w_vnorm.p, 12 * c->w_nvert, cudaMemcpyDeviceToHost, c->stream));
    if (indices && c->nmesh) PMS_CUDA(c, cudaMemcpyAsync(indices, c->w_idx.p, 4 * c->nmesh, cudaMemcpyDeviceToHost, c->stream));
    PMS_CUDA(c, cudaStreamSynchronize(c->stream));
    return PMS_OK;
}

extern "C" pms_status pms_stream_mesh_to_host(pms_ctx* c, float* pos, float* nrm, uint64_t cap) {
    if (!c || (!pos && nrm)) return PMS_ERR_INVALID_ARGUMENT;
    cudaSetDevice(c->device);
    // frames already on their way keep their own buffers
    if (pos) PMS_CHECK(copy_stream_ready(c));
    c->out_pos = pos;
    c->out_nrm = pos ? nrm : nullptr;
    c->out_cap = pos ? cap : 0;
    return PMS_OK;
}

extern "C" pms_status pms_wait_mesh(pms_ctx* c, uint64_t* n_vertices) {
    if (!c) return PMS_ERR_INVALID_ARGUMENT;
    if (!c->mesh_q.count) return pms_fail(c, PMS_ERR_STATE, "no mesh streamed since the last wait");
    cudaSetDevice(c->device);
    uint64_t n = 0, cap = 0;
    bool overflow = false;
    PMS_CHECK(out_wait(c, c->mesh_q, &n, &overflow, &cap));
    if (n_vertices) *n_vertices = n;
    if (overflow)
        return pms_fail(c, PMS_ERR_CAPACITY, "mesh has %llu vertices, the host buffers %llu", (unsigned long long)n,
                        (unsigned long long)cap);
    return PMS_OK;
}

extern "C" pms_status pms_stage_times(pms_ctx* c, float* ms, int count) {
    if (!c || !ms) return PMS_ERR_INVALID_ARGUMENT;
    cudaSetDevice(c->device);
    PMS_CUDA(c, cudaStreamSynchronize(c->stream));
    for (int i = 0; i < count && i < kNumStages; ++i) {
        ms[i] = 0.f;
        if (!c->ev_recorded[i]) continue;
        float t = 0.f;
        if (cudaEventElapsedTime(&t, c->ev[c->ev_from[i]], c->ev[i + 1]) == cudaSuccess) ms[i] = t;
    }
    return PMS_OK;
}

// ---------------------------------------------------------------------------
// debug downloads
// ---------------------------------------------------------------------------
template <class T>
static pms_status d2h(pms_ctx* c, std::vector<T>& v, const void* src, size_t count) {
    v.resize(count);
    if (count) PMS_CUDA(c, cudaMemcpyAsync(v.data(), src, sizeof(T) * count, cudaMemcpyDeviceToHost, c->stream));
    PMS_CUDA(c, cudaStreamSynchronize(c->stream));
    return PMS_OK;
}

extern "C" pms_status pms_debug_set_wait_limit(pms_ctx* c, int64_t polls) {
    // the stored value is polls + 1 (0 selects the default bound), so polls stays below 2^32 - 1
    if (!c || polls >= 0xffffffffll) return PMS_ERR_INVALID_ARGUMENT;
    c->tc_wait_polls = polls < 0 ? 0u : (uint32_t)polls + 1u;
    return PMS_OK;
}

extern "C" pms_status pms_debug_download(pms_ctx* c, int id, void* dst, uint64_t cap, uint64_t* needed) {
    if (!c) return PMS_ERR_INVALID_ARGUMENT;
    cudaSetDevice(c->device);
    pms_status st = sync_counters(c);
    if (st) return st;
    const uint32_t n = c->n, ns = c->h_counters->ns, nv = c->h_counters->nv, S = c->grid.sp_size;
    std::vector<uint8_t> out;
    auto put = [&](const void* p, size_t bytes) { out.resize(bytes); if (bytes) memcpy(out.data(), p, bytes); };
    switch (id) {
        case PMS_ARRAY_KEYS_SORTED: case PMS_ARRAY_PERM: case PMS_ARRAY_DENSITY: {
            if (!c->have_grid) return PMS_ERR_STATE;
            if (id == PMS_ARRAY_DENSITY && !c->have_aniso) return PMS_ERR_STATE;
            const DBuf& b = id == PMS_ARRAY_KEYS_SORTED ? c->skeys : id == PMS_ARRAY_PERM ? c->order : c->rho;
            std::vector<uint32_t> v;
            if ((st = d2h(c, v, b.p, n))) return st;
            put(v.data(), 4 * (size_t)n);
            break;
        }
        case PMS_ARRAY_POS_SORTED: {
            if (!c->have_grid) return PMS_ERR_STATE;
            std::vector<float> v;
            if ((st = d2h(c, v, c->spos.p, 4 * (size_t)n))) return st;
            std::vector<float> o(3 * (size_t)n);
            for (size_t i = 0; i < n; ++i) for (int k = 0; k < 3; ++k) o[3 * i + k] = v[4 * i + k];
            put(o.data(), 4 * o.size());
            break;
        }
        case PMS_ARRAY_CELL_START: case PMS_ARRAY_CELL_END: {
            if (!c->have_grid) return PMS_ERR_STATE;
            std::vector<uint32_t> s, m;
            if ((st = d2h(c, s, c->cell_start.p, S))) return st;
            if ((st = d2h(c, m, c->cell_count.p, S))) return st;
            std::vector<uint32_t> o(S);
            for (size_t i = 0; i < S; ++i) o[i] = m[i] ? (id == PMS_ARRAY_CELL_START ? s[i] : s[i] + m[i]) : 0u;
            put(o.data(), 4 * o.size());
            break;
        }
        case PMS_ARRAY_SURF_COUNT: {
            if (!c->have_aniso) return PMS_ERR_STATE;
            std::vector<uint32_t> v;
            if ((st = d2h(c, v, c->surf_count.p, S))) return st;
            put(v.data(), 4 * v.size());
            break;
        }
        case PMS_ARRAY_SURF_LIST: case PMS_ARRAY_NEIGHBORS: {
            if (!c->have_aniso) return PMS_ERR_STATE;
            std::vector<uint32_t> v;
            if ((st = d2h(c, v, id == PMS_ARRAY_SURF_LIST ? c->slist.p : c->nnb.p, ns))) return st;
            put(v.data(), 4 * v.size());
            break;
        }
        case PMS_ARRAY_MEAN: {
            if (!c->have_aniso) return PMS_ERR_STATE;
            std::vector<float> v;
            if ((st = d2h(c, v, c->mean4.p, 4 * (size_t)ns))) return st;
            std::vector<float> o(3 * (size_t)ns);
            for (size_t i = 0; i < ns; ++i) for (int k = 0; k < 3; ++k) o[3 * i + k] = v[4 * i + k];
            put(o.data(), 4 * o.size());
            break;
        }
        case PMS_ARRAY_G: {
            if (!c->have_aniso) return PMS_ERR_STATE;
            std::vector<float> v;
            if ((st = d2h(c, v, c->gdebug.p, 10 * (size_t)ns))) return st;
            put(v.data(), 4 * v.size());
            break;
        }
        case PMS_ARRAY_NORMAL: case PMS_ARRAY_FLAG: {
            if (!c->have_aniso) return PMS_ERR_STATE;
            std::vector<uint32_t> sl;
            std::vector<float> nr;
            if ((st = d2h(c, sl, c->slist.p, ns))) return st;
            if ((st = d2h(c, nr, c->nrm4.p, 4 * (size_t)n))) return st;
            if (id == PMS_ARRAY_NORMAL) {
                std::vector<float> o(3 * (size_t)ns);
                for (size_t s = 0; s < ns; ++s) for (int k = 0; k < 3; ++k) o[3 * s + k] = nr[4 * (size_t)sl[s] + k];
                put(o.data(), 4 * o.size());
            } else {
                std::vector<uint8_t> o(ns);
                for (size_t s = 0; s < ns; ++s) o[s] = nr[4 * (size_t)sl[s] + 3] != 0.f;
                put(o.data(), o.size());
            }
            break;
        }
        case PMS_ARRAY_BAND_CERTIFIED: {
            if (!c->have_field) return PMS_ERR_STATE;
            std::vector<uint32_t> v(((uint64_t)c->grid.sc_size + 31) / 32, 0u);
            if (c->band_learned && c->nv && (st = d2h(c, v, c->l_cert.p, v.size()))) return st;
            put(v.data(), 4 * v.size());
            break;
        }
        case PMS_ARRAY_BAND_BITMAP: {
            if (!c->have_band) return PMS_ERR_STATE;
            std::vector<uint32_t> v;
            if ((st = d2h(c, v, c->bm.p, ((uint64_t)c->grid.sc_size + 31) / 32))) return st;
            put(v.data(), 4 * v.size());
            break;
        }
        case PMS_ARRAY_BAND_LIST: case PMS_ARRAY_FIELD: case PMS_ARRAY_CUBE_CASE: {
            const bool ok = id == PMS_ARRAY_BAND_LIST ? c->have_band : id == PMS_ARRAY_FIELD ? c->have_field : c->have_mc;
            if (!ok) return PMS_ERR_STATE;
            const DBuf& b = id == PMS_ARRAY_BAND_LIST ? c->vlist : id == PMS_ARRAY_FIELD ? c->field : c->mc_case;
            std::vector<uint32_t> v;
            if ((st = d2h(c, v, b.p, nv))) return st;
            put(v.data(), 4 * v.size());
            break;
        }
        case PMS_ARRAY_CUBE_NVERT: {
            if (!c->have_mc) return PMS_ERR_STATE;
            std::vector<unsigned long long> v;
            if ((st = d2h(c, v, c->mc_key.p, nv))) return st;
            std::vector<uint32_t> o(nv);
            for (size_t i = 0; i < nv; ++i) o[i] = (uint32_t)(v[i] & 0xffffffffull);
            put(o.data(), 4 * o.size());
            break;
        }
        default: {
            st = diffuse_debug(c, id, out);
            if (st) return st;
        }
    }
    if (needed) *needed = out.size();
    if (!dst || cap < out.size()) return dst ? PMS_ERR_CAPACITY : PMS_OK;
    if (!out.empty()) memcpy(dst, out.data(), out.size());
    return PMS_OK;
}
