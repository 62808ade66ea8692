// pms_learn.cpp -- host side of the learned narrow band: the band + field
// stage driven by the network with the exact sign certification of the rest of
// the band, training-data preparation, and the trainer.  No counterpart in the
// reference (see k_learn.cu, k_field.cu).
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
pms_status plain_band(pms_ctx* c);
}  // namespace pms

static pms_status zero_learn_counters(pms_ctx* c) {
    PMS_CUDA(c, cudaMemsetAsync(reinterpret_cast<char*>(c->counters.p) + offsetof(Counters, l_cand), 0,
                                sizeof(uint32_t) * kLearnCounters, c->stream));
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
    if (!c || (mode != PMS_BAND_PLAIN && mode != PMS_BAND_LEARNED && mode != PMS_BAND_CERTIFIED))
        return PMS_ERR_INVALID_ARGUMENT;
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

// Buffers of the split and the certification: a scalar grid of sc_size vertices, a band
// of at most nv of them.
pms_status pms::ensure_learned_buffers(pms_ctx* c, uint64_t sc_size, uint32_t nv) {
    const uint64_t W = (sc_size + 31) / 32 + 1;
    for (DBuf* d : {&c->l_q, &c->l_cert, &c->l_e_bm, &c->l_e_wc, &c->l_e_wp, &c->l_n_bm, &c->l_n_wc, &c->l_n_wp})
        PMS_CUDA(c, d->ensure(4 * W));
    for (DBuf* d : {&c->l_e_list, &c->l_n_list}) PMS_CUDA(c, d->ensure(4 * ((size_t)nv + 1)));
    return PMS_OK;
}

// The network's prediction (when asked) and the split of the plain band into the
// corners of predicted cubes E and the rest N, both as ascending lists.
pms_status pms::learned_split(pms_ctx* c, bool predict) {
    Counters* cnt = c->counters.as<Counters>();
    const uint64_t W = words_of(c);
    pms_status st;
    if ((st = zero_learn_counters(c))) return st;
    if (predict) {
        if ((st = launch_coarse_counts(c))) return st;
        PMS_CUDA(c, cudaMemsetAsync(c->l_q.p, 0, 4 * W, c->stream));
        if ((st = launch_predict(c, 1, c->l_q.as<uint32_t>(), nullptr, nullptr, 0))) return st;
    }
    if ((st = launch_band_split(c, predict ? c->l_q.as<uint32_t>() : nullptr, c->l_e_bm.as<uint32_t>(),
                                c->l_n_bm.as<uint32_t>(), c->l_e_wc.as<uint32_t>(), c->l_n_wc.as<uint32_t>())))
        return st;
    if ((st = scan_u32(c, c->l_e_wc.as<uint32_t>(), c->l_e_wp.as<uint32_t>(), W, &cnt->l_exact))) return st;
    if ((st = scan_u32(c, c->l_n_wc.as<uint32_t>(), c->l_n_wp.as<uint32_t>(), W, &cnt->l_nlist))) return st;
    if ((st = launch_bits_list(c, c->l_e_bm.as<uint32_t>(), c->l_e_wp.as<uint32_t>(), c->l_e_list.as<uint32_t>()))) return st;
    return launch_bits_list(c, c->l_n_bm.as<uint32_t>(), c->l_n_wp.as<uint32_t>(), c->l_n_list.as<uint32_t>());
}

// The field stage of the learned band: the exact field at E, signs at N, the
// classification of every band cube (the signs are those of the exact field
// everywhere), the exact field at the certified corners of the valid cubes, and
// the band-order field.  c->nv bounds every list.
pms_status pms::learned_field(pms_ctx* c) {
    Counters* cnt = c->counters.as<Counters>();
    const uint64_t W = words_of(c);
    const uint32_t nvb = c->nv;
    pms_status st;
    PMS_CUDA(c, cudaMemsetAsync(c->fdense.p, 0, 4 * (size_t)c->grid.sc_size, c->stream));
    PMS_CUDA(c, cudaMemsetAsync(c->l_cert.p, 0, 4 * W, c->stream));
    if ((st = launch_field_on(c, c->l_e_list.as<uint32_t>(), &cnt->l_exact, nvb, nullptr))) return st;
    if ((st = launch_field_on(c, c->l_n_list.as<uint32_t>(), &cnt->l_nlist, nvb, nullptr, c->l_cert.as<uint32_t>(),
                              &cnt->l_cert)))
        return st;
    if ((st = launch_mc_classify(c))) return st;
    // the certified corners of valid cubes: E's buffers hold them from here on
    PMS_CUDA(c, cudaMemsetAsync(c->l_e_bm.p, 0, 4 * W, c->stream));
    if ((st = launch_recheck_bits(c, c->l_cert.as<uint32_t>(), c->l_e_bm.as<uint32_t>()))) return st;
    if ((st = launch_popc(c, c->l_e_bm.as<uint32_t>(), c->l_e_wc.as<uint32_t>()))) return st;
    if ((st = scan_u32(c, c->l_e_wc.as<uint32_t>(), c->l_e_wp.as<uint32_t>(), W, &cnt->l_recheck))) return st;
    if ((st = launch_bits_list(c, c->l_e_bm.as<uint32_t>(), c->l_e_wp.as<uint32_t>(), c->l_e_list.as<uint32_t>()))) return st;
    if ((st = launch_field_on(c, c->l_e_list.as<uint32_t>(), &cnt->l_recheck, nvb, nullptr))) return st;
    return launch_field_gather(c, c->vlist.as<uint32_t>(), &cnt->nv, nvb, c->field.as<float>());
}

extern "C" pms_status pms_band_learned(pms_ctx* c) {
    if (!c) return PMS_ERR_INVALID_ARGUMENT;
    if (!c->have_aniso) return pms_fail(c, PMS_ERR_STATE, "pms_band_learned before pms_anisotropy");
    const bool predict = c->band_mode != PMS_BAND_CERTIFIED;
    if (predict && !c->have_model)
        return pms_fail(c, PMS_ERR_STATE, "pms_band_learned without a model (pms_set_band_model)");
    cudaSetDevice(c->device);
    c->l_ncand = c->l_npred = c->l_nexact = c->l_ncert = c->l_nrecheck = 0;
    c->band_learned = true;
    c->mc_classified = c->mc_compacted = false;
    if (c->n == 0) { c->nv = 0; c->have_band = c->have_field = true; return PMS_OK; }
    pms_status st;
    // the plain band: where the field exists (a cube with a corner off it is never valid)
    if ((st = plain_band(c))) return st;
    if ((st = ensure_learned_buffers(c, c->grid.sc_size, c->nv))) return st;
    if (c->nv && (st = learned_split(c, predict))) return st;
    c->have_band = true;
    mark_stage(c, kStageBand + 1);
    if (c->nv && (st = learned_field(c))) return st;
    // the classification and compaction are the marching cubes' own
    if ((st = sync_counters(c))) return st;
    const Counters& h = *c->h_counters;
    c->l_ncand = h.l_cand;
    c->l_npred = h.l_pred;
    c->l_nexact = h.l_exact;
    c->l_ncert = h.l_cert;
    c->l_nrecheck = h.l_recheck;
    if (h.err & kErrTcLost)
        return pms_fail(c, PMS_ERR_CUDA, "a tensor-core operation outlived two bounded waits; destroy this context");
    if (h.err & kErrTimeout) return pms_fail(c, PMS_ERR_CUDA, "internal: a wait on the tensor cores timed out");
    c->mc_classified = c->mc_compacted = c->nv != 0;
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
    PMS_CUDA(c, c->l_e_list.ensure(4 * NC));
    pms_status st;
    if ((st = zero_learn_counters(c))) return st;
    if (logits) {
        if (!c->have_model) return pms_fail(c, PMS_ERR_STATE, "logits need a model (pms_set_band_model)");
        if ((st = launch_predict(c, 1, nullptr, c->l_e_list.as<uint32_t>(), c->l_logit.as<float>(), nc))) return st;
    } else {
        if ((st = launch_predict(c, 0, nullptr, c->l_e_list.as<uint32_t>(), nullptr, nc))) return st;
    }
    // candidates come back in the order the tiles finished: sort by cube id
    std::vector<uint32_t> id(nc);
    std::vector<float> lg(logits ? nc : 0);
    if (nc) {
        PMS_CUDA(c, cudaMemcpyAsync(id.data(), c->l_e_list.p, 4 * (size_t)nc, cudaMemcpyDeviceToHost, c->stream));
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
    PMS_CUDA(c, c->l_e_list.ensure(4 * (size_t)n));
    PMS_CUDA(c, c->l_field_new.ensure(128 * (size_t)n));
    PMS_CUDA(c, cudaMemcpyAsync(c->l_e_list.p, ids, 4 * (size_t)n, cudaMemcpyHostToDevice, c->stream));
    pms_status st = launch_features(c, c->l_e_list.as<uint32_t>(), n, c->l_field_new.as<uint16_t>());
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
    DBuf w, m, v, grad, model, loss, x, y, err;
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
              t->model.ensure(sizeof(DevModel)) == cudaSuccess && t->loss.ensure(sizeof(float)) == cudaSuccess &&
              t->err.ensure(sizeof(uint32_t)) == cudaSuccess;
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
             cudaMemset(t->err.p, 0, sizeof(uint32_t)) == cudaSuccess &&
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
    for (DBuf* b : {&t->w, &t->m, &t->v, &t->grad, &t->model, &t->loss, &t->x, &t->y, &t->err}) b->release();
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
    PMS_CUDA(c, launch_train(c, c->stream, a, t->model.as<DevModel>(), t->grad.as<float>(), t->loss.as<float>(),
                             t->err.as<uint32_t>()));
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
        uint32_t e = 0;
        PMS_CUDA(c, cudaMemcpyAsync(&e, t->err.p, sizeof(uint32_t), cudaMemcpyDeviceToHost, c->stream));
        PMS_CUDA(c, cudaStreamSynchronize(c->stream));
        if (e) return pms_fail(c, PMS_ERR_CUDA, "a wait on the tensor cores timed out in a training step%s",
                               (e & kErrTcLost) ? "; destroy this context" : "");
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
    uint32_t e = 0;
    if (cudaMemcpyAsync(t->x.p, x, 128 * (size_t)batch, cudaMemcpyHostToDevice, t->stream) != cudaSuccess ||
        cudaMemcpyAsync(t->y.p, y, batch, cudaMemcpyHostToDevice, t->stream) != cudaSuccess ||
        cudaMemsetAsync(t->grad.p, 0, P, t->stream) != cudaSuccess ||
        cudaMemsetAsync(t->loss.p, 0, sizeof(float), t->stream) != cudaSuccess ||
        launch_train(nullptr, t->stream, a, t->model.as<DevModel>(), t->grad.as<float>(), t->loss.as<float>(),
                     t->err.as<uint32_t>()) != cudaSuccess ||
        cudaMemcpyAsync(grad, t->grad.p, P, cudaMemcpyDeviceToHost, t->stream) != cudaSuccess ||
        cudaMemcpyAsync(&l, t->loss.p, sizeof(float), cudaMemcpyDeviceToHost, t->stream) != cudaSuccess ||
        cudaMemcpyAsync(&e, t->err.p, sizeof(uint32_t), cudaMemcpyDeviceToHost, t->stream) != cudaSuccess ||
        cudaStreamSynchronize(t->stream) != cudaSuccess)
        return PMS_ERR_CUDA;
    if (e) return PMS_ERR_TIMEOUT;
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
