// pms_learn.cpp -- host side of the learned narrow band: the band + field
// stage driven by the network with its border-check fallback, training-data
// preparation, and the trainer.  No counterpart in the reference (see k_learn.cu).
#include <algorithm>
#include <cmath>
#include <cstddef>
#include <utility>

#include "pms_internal.h"
#include "learn_internal.h"

using namespace pms;

// defined in pms_api.cpp
namespace pms {
pms_status ensure_band_buffers(pms_ctx* c, uint32_t nv);
void mark_stage(pms_ctx* c, int boundary);
}  // namespace pms

static constexpr uint32_t kMaxBorderRounds = 256;

static pms_status zero_learn_counters(pms_ctx* c) {
    PMS_CUDA(c, cudaMemsetAsync(reinterpret_cast<char*>(c->counters.p) + offsetof(Counters, l_cand), 0,
                                sizeof(uint32_t) * 5, c->stream));
    return PMS_OK;
}

static uint64_t words_of(const pms_ctx* c) { return ((uint64_t)c->grid.sc_size + 31) / 32; }

extern "C" pms_status pms_set_band_model(pms_ctx* c, const pms_band_model* m) {
    if (!c || !m) return PMS_ERR_INVALID_ARGUMENT;
    cudaSetDevice(c->device);
    PMS_CUDA(c, c->l_model.ensure(sizeof(pms_band_model)));
    PMS_CUDA(c, cudaMemcpyAsync(c->l_model.p, m, sizeof(pms_band_model), cudaMemcpyHostToDevice, c->stream));
    PMS_CUDA(c, cudaStreamSynchronize(c->stream));
    c->have_model = true;
    return PMS_OK;
}

extern "C" pms_status pms_set_band_mode(pms_ctx* c, int mode) {
    if (!c || (mode != PMS_BAND_PLAIN && mode != PMS_BAND_LEARNED)) return PMS_ERR_INVALID_ARGUMENT;
    if (mode == PMS_BAND_LEARNED && !c->have_model) return pms_fail(c, PMS_ERR_STATE, "learned band without a model");
    c->band_mode = mode;
    return PMS_OK;
}

static const char kModelMagic[8] = {'P', 'M', 'S', 'B', 'A', 'N', 'D', '1'};

extern "C" pms_status pms_save_band_model(const char* path, const pms_band_model* m, const char* meta) {
    if (!path || !m) return PMS_ERR_INVALID_ARGUMENT;
    FILE* f = fopen(path, "wb");
    if (!f) return PMS_ERR_IO;
    const uint32_t hdr[2] = {1u, (uint32_t)sizeof(pms_band_model)};
    const uint32_t ml = meta ? (uint32_t)strlen(meta) : 0u;
    bool ok = fwrite(kModelMagic, 1, 8, f) == 8 && fwrite(hdr, 4, 2, f) == 2 && fwrite(m, sizeof(*m), 1, f) == 1 &&
              fwrite(&ml, 4, 1, f) == 1 && (ml == 0 || fwrite(meta, 1, ml, f) == ml);
    ok = (fclose(f) == 0) && ok;
    return ok ? PMS_OK : PMS_ERR_IO;
}

extern "C" pms_status pms_load_band_model(const char* path, pms_band_model* out) {
    if (!path || !out) return PMS_ERR_INVALID_ARGUMENT;
    FILE* f = fopen(path, "rb");
    if (!f) return PMS_ERR_IO;
    char magic[8];
    uint32_t hdr[2];
    bool ok = fread(magic, 1, 8, f) == 8 && memcmp(magic, kModelMagic, 8) == 0 && fread(hdr, 4, 2, f) == 2 &&
              hdr[0] == 1u && hdr[1] == sizeof(pms_band_model) && fread(out, sizeof(*out), 1, f) == 1;
    fclose(f);
    if (!ok) return PMS_ERR_IO;
    for (int j = 0; j < kHid; ++j)
        if (!std::isfinite(out->b1[j])) return PMS_ERR_IO;
    return std::isfinite(out->b2) && !std::isnan(out->threshold) ? PMS_OK : PMS_ERR_IO;
}

// vertex list, nv and band buffers of the bitmap in c->bm (popcounts in c->wcount)
static pms_status finish_vertex_set(pms_ctx* c) {
    Counters* cnt = c->counters.as<Counters>();
    const uint64_t W = words_of(c);
    pms_status st = scan_u32(c, c->wcount.as<uint32_t>(), c->wprefix.as<uint32_t>(), W, &cnt->nv);
    if (st) return st;
    if ((st = sync_counters(c))) return st;
    c->nv = c->h_counters->nv;
    if ((st = ensure_band_buffers(c, c->nv))) return st;
    return launch_bits_list(c, c->bm.as<uint32_t>(), c->wprefix.as<uint32_t>(), c->vlist.as<uint32_t>());
}

// The corners of the compacted valid cubes (cube bitmap from their records,
// then the list of its corners), each tested against the plain band's rule; those
// outside leave the vertex set and l_removed counts them.  Corners of valid
// cubes are band vertices, so c->nv bounds the list.
pms_status pms::plain_band_filter(pms_ctx* c) {
    Counters* cnt = c->counters.as<Counters>();
    const uint64_t W = words_of(c);
    pms_status st;
    PMS_CUDA(c, c->l_vlist_new.ensure(4 * ((size_t)c->nv + 1)));
    PMS_CUDA(c, c->l_vlist_m.ensure(4 * ((size_t)c->nv + 1)));
    PMS_CUDA(c, cudaMemsetAsync(c->l_q.p, 0, 4 * W, c->stream));
    PMS_CUDA(c, cudaMemsetAsync(&cnt->l_removed, 0, sizeof(uint32_t), c->stream));
    if ((st = launch_valid_bits(c, c->l_q.as<uint32_t>()))) return st;
    if ((st = launch_corner_list(c, c->l_q.as<uint32_t>(), c->l_vlist_new.as<uint32_t>(), &cnt->l_nnew))) return st;
    return launch_plain_member(c, c->l_vlist_new.as<uint32_t>(), &cnt->l_nnew, c->nv, c->l_vlist_m.as<uint32_t>(),
                               &cnt->l_open, &cnt->l_removed);
}

extern "C" pms_status pms_band_learned(pms_ctx* c) {
    if (!c) return PMS_ERR_INVALID_ARGUMENT;
    if (!c->have_aniso) return pms_fail(c, PMS_ERR_STATE, "pms_band_learned before pms_anisotropy");
    if (!c->have_model) return pms_fail(c, PMS_ERR_STATE, "pms_band_learned without a model (pms_set_band_model)");
    cudaSetDevice(c->device);
    c->l_ncand = c->l_npred = c->l_nadded = c->l_iters = c->l_nremoved = 0;
    c->band_learned = true;
    c->mc_classified = c->mc_compacted = false;
    if (c->n == 0) { c->nv = 0; c->have_band = c->have_field = true; return PMS_OK; }
    Counters* cnt = c->counters.as<Counters>();
    const uint64_t W = words_of(c);
    pms_status st;
    PMS_CUDA(c, c->l_q.ensure(4 * (W + 1)));
    PMS_CUDA(c, c->l_qadd.ensure(4 * (W + 1)));
    if ((st = zero_learn_counters(c))) return st;
    // predicted cubes -> their corners -> vertex list
    if ((st = launch_coarse_counts(c))) return st;
    PMS_CUDA(c, cudaMemsetAsync(c->l_q.p, 0, 4 * W, c->stream));
    if ((st = launch_predict(c, 1, c->l_q.as<uint32_t>(), nullptr, nullptr, 0))) return st;
    if ((st = launch_cube_corners(c, c->l_q.as<uint32_t>(), nullptr, c->bm.as<uint32_t>(), c->wcount.as<uint32_t>())))
        return st;
    if ((st = finish_vertex_set(c))) return st;
    c->l_ncand = c->h_counters->l_cand;
    c->l_npred = c->h_counters->l_pred;
    c->have_band = true;
    mark_stage(c, kStageBand + 1);
    // exact field at those vertices, then the border check until no cube is missing:
    // a full check over every valid cube queues the cubes across crossed faces whose
    // corners lack a value; each round evaluates the queued cubes' new corners (set in
    // the vertex bitmap and listed as they are found) and checks only those cubes, one
    // synchronisation per round; when a round queues nothing, the sorted vertex list
    // is rebuilt from the bitmap and one more full check catches cubes whose corners
    // other cubes' rounds completed
    if (c->nv && (st = launch_field(c))) return st;
    uint64_t nv_bound = c->nv;                 // host bound on the vertex count while rounds run
    uint32_t added = 0;
    // queue lists: grow-only; a check whose queue overflowed its list runs again
    auto qcap_of = [](const DBuf& d) { return (uint32_t)std::min<size_t>(d.cap / 4, 0xffffffffu); };
    PMS_CUDA(c, c->l_qlist.ensure(4 * std::max<size_t>(1u << 16, nv_bound / 16)));
    PMS_CUDA(c, c->l_qnext.ensure(c->l_qlist.cap));
    auto run_check = [&](auto&& launch) -> pms_status {
        pms_status s2;
        for (int pass = 0; pass < 2; ++pass) {
            PMS_CUDA(c, cudaMemsetAsync(c->l_qadd.p, 0, 4 * W, c->stream));
            PMS_CUDA(c, cudaMemsetAsync(&cnt->l_added, 0, sizeof(uint32_t), c->stream));
            if ((s2 = launch())) return s2;
            if ((s2 = sync_counters(c))) return s2;
            added = c->h_counters->l_added;
            if (added <= qcap_of(c->l_qnext)) return PMS_OK;
            PMS_CUDA(c, c->l_qnext.ensure(4 * (size_t)added));
        }
        return pms_fail(c, PMS_ERR_CAPACITY, "border queue outgrew its list");
    };
    auto full_check = [&]() -> pms_status {
        pms_status s2;
        c->nv = (uint32_t)nv_bound;
        // classification (cases, scan, compaction: the valid-cube records), then the
        // border check over those records
        if ((s2 = launch_mc_classify(c))) return s2;
        if ((s2 = run_check([&] { return launch_border(c, c->l_qadd.as<uint32_t>(), c->l_qnext.as<uint32_t>(),
                                                       qcap_of(c->l_qnext)); })))
            return s2;
        c->mc_compacted = true;
        c->nv = c->h_counters->nv;
        nv_bound = c->nv;
        std::swap(c->l_qlist, c->l_qnext);
        return PMS_OK;
    };
    if (c->nv && (st = full_check())) return st;
    for (uint32_t round = 0; added && round < kMaxBorderRounds; ++round) {
        c->l_nadded += added;
        c->l_iters++;
        const uint32_t nq = added;
        // the queued cubes' corners without a value, and the field there
        const uint64_t nnew_bound = std::min<uint64_t>(8ull * nq, (uint64_t)c->grid.sc_size);
        PMS_CUDA(c, c->l_vlist_new.ensure(4 * (nnew_bound + 1)));
        PMS_CUDA(c, cudaMemsetAsync(&cnt->l_nnew, 0, sizeof(uint32_t), c->stream));
        if ((st = launch_queue_corners(c, c->l_qlist.as<uint32_t>(), nq, c->l_vlist_new.as<uint32_t>(), &cnt->l_nnew)))
            return st;
        if ((st = launch_field_on(c, c->l_vlist_new.as<uint32_t>(), &cnt->l_nnew, (uint32_t)nnew_bound, nullptr)))
            return st;
        nv_bound = std::min<uint64_t>(nv_bound + nnew_bound, (uint64_t)c->grid.sc_size);
        // border check of the queued cubes, now evaluated
        if ((st = run_check([&] { return launch_border_list(c, c->l_qlist.as<uint32_t>(), nq, c->l_qadd.as<uint32_t>(),
                                                            nullptr, c->l_qnext.as<uint32_t>(), qcap_of(c->l_qnext)); })))
            return st;
        std::swap(c->l_qlist, c->l_qnext);
        if (!added) {
            // the sorted vertex list of the grown set, then one full check
            if ((st = launch_popc(c, c->bm.as<uint32_t>(), c->wcount.as<uint32_t>()))) return st;
            if ((st = finish_vertex_set(c))) return st;
            nv_bound = c->nv;
            if ((st = full_check())) return st;
        }
    }
    if (added) {
        // round limit reached: the vertex list still covers every value computed
        if ((st = launch_popc(c, c->bm.as<uint32_t>(), c->wcount.as<uint32_t>()))) return st;
        if ((st = finish_vertex_set(c))) return st;
        if (c->nv && (st = launch_mc_classify(c))) return st;
    }
    // the plain band's membership test of the valid cubes' corners: a corner the
    // plain band lacks leaves the set, so that every cube classified valid is one
    // the plain band holds; the set then gets its sorted list again
    uint32_t removed = 0;
    if (c->nv) {
        if ((st = plain_band_filter(c))) return st;
        if ((st = sync_counters(c))) return st;
        removed = c->l_nremoved = c->h_counters->l_removed;
        if (removed) {
            if ((st = launch_popc(c, c->bm.as<uint32_t>(), c->wcount.as<uint32_t>()))) return st;
            if ((st = finish_vertex_set(c))) return st;
        }
    }
    c->nv = c->h_counters->nv;
    if ((st = ensure_band_buffers(c, c->nv))) return st;
    // the band-order field of the final vertex set (the rounds work on the dense field)
    if ((c->l_iters || removed) && c->nv && (st = launch_field_gather(c, c->vlist.as<uint32_t>(), &cnt->nv, c->nv, c->field.as<float>())))
        return st;
    // the last full check (or classification) computed the final vertex set's cases
    // unless corners were removed since
    c->mc_classified = removed == 0;
    c->mc_compacted = c->mc_classified;
    c->have_field = true;
    mark_stage(c, kStageField + 1);
    return PMS_OK;
}

extern "C" pms_status pms_surface_learned(pms_ctx* c) {
    pms_status st;
    if ((st = pms_anisotropy(c))) return st;
    if ((st = pms_band_learned(c))) return st;
    return pms_marching_cubes(c);
}

// ---------------------------------------------------------------------------
// training data
// ---------------------------------------------------------------------------
extern "C" pms_status pms_learn_prepare(pms_ctx* c, uint32_t* n_candidates, uint32_t* n_valid) {
    if (!c) return PMS_ERR_INVALID_ARGUMENT;
    if (!c->have_mc || c->band_learned) return pms_fail(c, PMS_ERR_STATE, "pms_learn_prepare needs a plain pms_surface");
    cudaSetDevice(c->device);
    const uint64_t W = words_of(c);
    pms_status st;
    PMS_CUDA(c, c->l_label.ensure(4 * (W + 1)));
    PMS_CUDA(c, cudaMemsetAsync(c->l_label.p, 0, 4 * W, c->stream));
    if (c->nv && (st = launch_label_bits(c, c->l_label.as<uint32_t>()))) return st;
    if ((st = launch_coarse_counts(c))) return st;
    if ((st = zero_learn_counters(c))) return st;
    if ((st = launch_predict(c, 0, nullptr, nullptr, nullptr, 0))) return st;
    if ((st = sync_counters(c))) return st;
    const uint32_t nc = c->h_counters->l_cand;
    PMS_CUDA(c, c->l_cand.ensure(4 * (size_t)(nc ? nc : 1)));
    if ((st = zero_learn_counters(c))) return st;
    if ((st = launch_predict(c, 0, nullptr, c->l_cand.as<uint32_t>(), nullptr, nc))) return st;
    if ((st = sync_counters(c))) return st;
    c->l_ncand = nc;
    if (n_candidates) *n_candidates = nc;
    if (n_valid) *n_valid = c->nvalid;
    return PMS_OK;
}

static pms_status download_labels(pms_ctx* c, std::vector<uint32_t>& lbm) {
    const uint64_t W = words_of(c);
    lbm.resize(W);
    PMS_CUDA(c, cudaMemcpyAsync(lbm.data(), c->l_label.p, 4 * W, cudaMemcpyDeviceToHost, c->stream));
    PMS_CUDA(c, cudaStreamSynchronize(c->stream));
    return PMS_OK;
}

extern "C" pms_status pms_learn_candidates(pms_ctx* c, uint32_t* ids, float* logits, uint8_t* labels, uint32_t cap,
                                           uint32_t* n) {
    if (!c || !n) return PMS_ERR_INVALID_ARGUMENT;
    if (!c->l_ncand && !c->l_label.p) return pms_fail(c, PMS_ERR_STATE, "pms_learn_candidates before pms_learn_prepare");
    cudaSetDevice(c->device);
    const uint32_t nc = c->l_ncand;
    *n = nc;
    if (nc > cap) return PMS_ERR_CAPACITY;
    const size_t NC = nc ? nc : 1;
    PMS_CUDA(c, c->l_logit.ensure(4 * NC));
    PMS_CUDA(c, c->l_vlist_new.ensure(4 * NC));
    pms_status st;
    if ((st = zero_learn_counters(c))) return st;
    if (logits) {
        if (!c->have_model) return pms_fail(c, PMS_ERR_STATE, "logits need a model (pms_set_band_model)");
        if ((st = launch_predict(c, 1, nullptr, c->l_vlist_new.as<uint32_t>(), c->l_logit.as<float>(), nc))) return st;
    } else {
        if ((st = launch_predict(c, 0, nullptr, c->l_vlist_new.as<uint32_t>(), nullptr, nc))) return st;
    }
    // candidates come back in the order the tiles finished: sort by cube id
    std::vector<uint32_t> id(nc);
    std::vector<float> lg(logits ? nc : 0);
    if (nc) {
        PMS_CUDA(c, cudaMemcpyAsync(id.data(), c->l_vlist_new.p, 4 * (size_t)nc, cudaMemcpyDeviceToHost, c->stream));
        if (logits) PMS_CUDA(c, cudaMemcpyAsync(lg.data(), c->l_logit.p, 4 * (size_t)nc, cudaMemcpyDeviceToHost, c->stream));
    }
    PMS_CUDA(c, cudaStreamSynchronize(c->stream));
    std::vector<uint32_t> order(nc);
    for (uint32_t i = 0; i < nc; ++i) order[i] = i;
    std::sort(order.begin(), order.end(), [&](uint32_t a, uint32_t b) { return id[a] < id[b]; });
    std::vector<uint32_t> lbm;
    if (labels && (st = download_labels(c, lbm))) return st;
    for (uint32_t i = 0; i < nc; ++i) {
        const uint32_t k = order[i];
        if (ids) ids[i] = id[k];
        if (logits) logits[i] = lg[k];
        if (labels) labels[i] = (uint8_t)((lbm[id[k] >> 5] >> (id[k] & 31u)) & 1u);
    }
    return PMS_OK;
}

extern "C" pms_status pms_learn_features(pms_ctx* c, const uint32_t* ids, uint32_t n, uint16_t* x) {
    if (!c || (n && (!ids || !x))) return PMS_ERR_INVALID_ARGUMENT;
    if (!c->l_counts.p) return pms_fail(c, PMS_ERR_STATE, "pms_learn_features before pms_learn_prepare");
    for (uint32_t i = 0; i < n; ++i)
        if (ids[i] >= c->grid.sc_size) return pms_fail(c, PMS_ERR_INVALID_ARGUMENT, "cube id outside the scalar grid");
    if (!n) return PMS_OK;
    cudaSetDevice(c->device);
    PMS_CUDA(c, c->l_vlist_new.ensure(4 * (size_t)n));
    PMS_CUDA(c, c->l_field_new.ensure(128 * (size_t)n));
    PMS_CUDA(c, cudaMemcpyAsync(c->l_vlist_new.p, ids, 4 * (size_t)n, cudaMemcpyHostToDevice, c->stream));
    pms_status st = launch_features(c, c->l_vlist_new.as<uint32_t>(), n, c->l_field_new.as<uint16_t>());
    if (st) return st;
    PMS_CUDA(c, cudaMemcpyAsync(x, c->l_field_new.p, 128 * (size_t)n, cudaMemcpyDeviceToHost, c->stream));
    PMS_CUDA(c, cudaStreamSynchronize(c->stream));
    return PMS_OK;
}

// ---------------------------------------------------------------------------
// trainer
// ---------------------------------------------------------------------------
struct pms_trainer {
    int device = 0;
    cudaStream_t stream = nullptr;
    DBuf w, m, v, grad, model, loss, x, y;
    uint64_t step = 0;
};

static uint64_t splitmix(uint64_t& s) {
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

static pms_status refresh_model(pms_trainer* t) {
    AdamParams ap = {0.f, 0.9f, 0.999f, 1e-8f, 1.f, 1.f};
    if (launch_adam(t->stream, t->w.as<float>(), t->grad.as<float>(), t->m.as<float>(), t->v.as<float>(), ap,
                    t->model.as<DevModel>()) != cudaSuccess)
        return PMS_ERR_CUDA;
    return cudaStreamSynchronize(t->stream) == cudaSuccess ? PMS_OK : PMS_ERR_CUDA;
}

extern "C" pms_status pms_trainer_create(int device, uint64_t seed, pms_trainer** out) {
    if (!out) return PMS_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    if (cudaSetDevice(device) != cudaSuccess) return PMS_ERR_CUDA;
    pms_trainer* t = new pms_trainer;
    t->device = device;
    const size_t P = sizeof(float) * kNumParams;
    bool ok = cudaStreamCreateWithFlags(&t->stream, cudaStreamNonBlocking) == cudaSuccess && t->w.ensure(P) == cudaSuccess &&
              t->m.ensure(P) == cudaSuccess && t->v.ensure(P) == cudaSuccess && t->grad.ensure(P) == cudaSuccess &&
              t->model.ensure(sizeof(DevModel)) == cudaSuccess && t->loss.ensure(sizeof(float)) == cudaSuccess;
    if (ok) {
        // He-uniform first layer, small second layer, zero biases
        std::vector<float> w(kNumParams, 0.f);
        uint64_t s = seed;
        const float a1 = std::sqrt(6.f / (float)kIn), a2 = std::sqrt(6.f / (float)kHid) * 0.1f;
        for (int i = 0; i < kOffB1; ++i) w[i] = a1 * (2.f * (float)((splitmix(s) >> 40) * (1.0 / 16777216.0)) - 1.f);
        for (int j = 0; j < kHid; ++j) w[kOffW2 + j] = a2 * (2.f * (float)((splitmix(s) >> 40) * (1.0 / 16777216.0)) - 1.f);
        ok = cudaMemcpy(t->w.p, w.data(), P, cudaMemcpyHostToDevice) == cudaSuccess &&
             cudaMemset(t->m.p, 0, P) == cudaSuccess && cudaMemset(t->v.p, 0, P) == cudaSuccess &&
             cudaMemset(t->grad.p, 0, P) == cudaSuccess && cudaMemset(t->model.p, 0, sizeof(DevModel)) == cudaSuccess &&
             refresh_model(t) == PMS_OK;
    }
    if (!ok) { pms_trainer_destroy(t); return PMS_ERR_CUDA; }
    *out = t;
    return PMS_OK;
}

extern "C" void pms_trainer_destroy(pms_trainer* t) {
    if (!t) return;
    cudaSetDevice(t->device);
    if (t->stream) cudaStreamSynchronize(t->stream);
    for (DBuf* b : {&t->w, &t->m, &t->v, &t->grad, &t->model, &t->loss, &t->x, &t->y}) b->release();
    if (t->stream) cudaStreamDestroy(t->stream);
    delete t;
}

extern "C" pms_status pms_trainer_step(pms_trainer* t, pms_ctx* c, uint32_t batch, uint64_t seed, float lr,
                                       float pos_weight, float* loss) {
    if (!t || !c || batch == 0) return PMS_ERR_INVALID_ARGUMENT;
    if (!c->l_ncand || !c->l_cand.p) return pms_fail(c, PMS_ERR_STATE, "pms_trainer_step before pms_learn_prepare");
    if (c->device != t->device) return pms_fail(c, PMS_ERR_INVALID_ARGUMENT, "trainer and context on different devices");
    cudaSetDevice(c->device);
    const size_t P = sizeof(float) * kNumParams;
    // the step runs on the data context's stream, after the frame's own work
    PMS_CUDA(c, cudaMemsetAsync(t->grad.p, 0, P, c->stream));
    PMS_CUDA(c, cudaMemsetAsync(t->loss.p, 0, sizeof(float), c->stream));
    TrainArgs a;
    a.batch = batch;
    a.seed = seed;
    a.pos_weight = pos_weight;
    PMS_CUDA(c, launch_train(c, c->stream, a, t->model.as<DevModel>(), t->grad.as<float>(), t->loss.as<float>()));
    c->launches++;
    t->step++;
    AdamParams ap;
    ap.lr = lr; ap.beta1 = 0.9f; ap.beta2 = 0.999f; ap.eps = 1e-8f;
    ap.inv_bc1 = (float)(1.0 / (1.0 - std::pow(0.9, (double)t->step)));
    ap.inv_bc2 = (float)(1.0 / (1.0 - std::pow(0.999, (double)t->step)));
    PMS_CUDA(c, launch_adam(c->stream, t->w.as<float>(), t->grad.as<float>(), t->m.as<float>(), t->v.as<float>(), ap,
                            t->model.as<DevModel>()));
    c->launches++;
    if (loss) {
        PMS_CUDA(c, cudaMemcpyAsync(loss, t->loss.p, sizeof(float), cudaMemcpyDeviceToHost, c->stream));
        PMS_CUDA(c, cudaStreamSynchronize(c->stream));
    }
    return PMS_OK;
}

extern "C" pms_status pms_trainer_grad(pms_trainer* t, const uint16_t* x, const uint8_t* y, uint32_t batch,
                                       float pos_weight, float* grad, float* loss) {
    if (!t || !x || !y || !grad || batch == 0) return PMS_ERR_INVALID_ARGUMENT;
    cudaSetDevice(t->device);
    const size_t P = sizeof(float) * kNumParams;
    if (t->x.ensure(128 * (size_t)batch) != cudaSuccess || t->y.ensure(batch) != cudaSuccess) return PMS_ERR_OUT_OF_MEMORY;
    TrainArgs a;
    a.x = t->x.as<uint16_t>();
    a.y = t->y.as<uint8_t>();
    a.batch = batch;
    a.pos_weight = pos_weight;
    float l = 0.f;
    if (cudaMemcpyAsync(t->x.p, x, 128 * (size_t)batch, cudaMemcpyHostToDevice, t->stream) != cudaSuccess ||
        cudaMemcpyAsync(t->y.p, y, batch, cudaMemcpyHostToDevice, t->stream) != cudaSuccess ||
        cudaMemsetAsync(t->grad.p, 0, P, t->stream) != cudaSuccess ||
        cudaMemsetAsync(t->loss.p, 0, sizeof(float), t->stream) != cudaSuccess ||
        launch_train(nullptr, t->stream, a, t->model.as<DevModel>(), t->grad.as<float>(), t->loss.as<float>()) != cudaSuccess ||
        cudaMemcpyAsync(grad, t->grad.p, P, cudaMemcpyDeviceToHost, t->stream) != cudaSuccess ||
        cudaMemcpyAsync(&l, t->loss.p, sizeof(float), cudaMemcpyDeviceToHost, t->stream) != cudaSuccess ||
        cudaStreamSynchronize(t->stream) != cudaSuccess)
        return PMS_ERR_CUDA;
    if (loss) *loss = l;
    return PMS_OK;
}

extern "C" pms_status pms_trainer_get_params(pms_trainer* t, float* params) {
    if (!t || !params) return PMS_ERR_INVALID_ARGUMENT;
    cudaSetDevice(t->device);
    if (cudaStreamSynchronize(t->stream) != cudaSuccess ||
        cudaMemcpy(params, t->w.p, sizeof(float) * kNumParams, cudaMemcpyDeviceToHost) != cudaSuccess)
        return PMS_ERR_CUDA;
    return PMS_OK;
}

extern "C" pms_status pms_trainer_set_params(pms_trainer* t, const float* params) {
    if (!t || !params) return PMS_ERR_INVALID_ARGUMENT;
    cudaSetDevice(t->device);
    if (cudaStreamSynchronize(t->stream) != cudaSuccess ||
        cudaMemcpy(t->w.p, params, sizeof(float) * kNumParams, cudaMemcpyHostToDevice) != cudaSuccess)
        return PMS_ERR_CUDA;
    return refresh_model(t);
}

extern "C" pms_status pms_trainer_get_model(pms_trainer* t, pms_band_model* out) {
    if (!t || !out) return PMS_ERR_INVALID_ARGUMENT;
    cudaSetDevice(t->device);
    if (cudaDeviceSynchronize() != cudaSuccess ||
        cudaMemcpy(out, t->model.p, sizeof(DevModel), cudaMemcpyDeviceToHost) != cudaSuccess)
        return PMS_ERR_CUDA;
    out->threshold = 0.f;
    return PMS_OK;
}
