// pms_tune.cpp -- the project's autotuner: picks launch shapes of the
// neighbour-walk kernels (threads per block, the field's resident-block cap and
// vertices per work item)
// by timing every candidate on the frame the context holds.  No counterpart
// in the reference, whose launches use fixed block sizes.
#include <algorithm>
#include <vector>

#include "pms_internal.h"

using namespace pms;

static pms_status time_ms(pms_ctx* c, int reps, float* out, pms_status (*fn)(pms_ctx*)) {
    cudaEvent_t a, b;
    PMS_CUDA(c, cudaEventCreate(&a));
    PMS_CUDA(c, cudaEventCreate(&b));
    std::vector<float> t;
    pms_status st = PMS_OK;
    for (int r = 0; r < reps && !st; ++r) {
        cudaEventRecord(a, c->stream);
        st = fn(c);
        cudaEventRecord(b, c->stream);
        if (!st && cudaEventSynchronize(b) != cudaSuccess) st = PMS_ERR_CUDA;
        float ms = 0.f;
        if (!st) cudaEventElapsedTime(&ms, a, b);
        t.push_back(ms);
    }
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    if (st) return st;
    std::sort(t.begin(), t.end());
    *out = t[t.size() / 2];
    return PMS_OK;
}

extern "C" pms_status pms_autotune(pms_ctx* c, pms_tune* out) {
    if (!c) return PMS_ERR_INVALID_ARGUMENT;
    if (!c->have_field || c->n == 0) return pms_fail(c, PMS_ERR_STATE, "pms_autotune needs a reconstructed frame");
    cudaSetDevice(c->device);
    // the re-runs below bump device counters (FP64 solves); keep the frame's
    Counters saved;
    PMS_CUDA(c, cudaMemcpyAsync(&saved, c->counters.p, sizeof(Counters), cudaMemcpyDeviceToHost, c->stream));
    PMS_CUDA(c, cudaStreamSynchronize(c->stream));
    const int sizes[3] = {64, 128, 256};
    const int waves[4] = {1, 2, 4, 8};
    const int vpts[3] = {1, 2, 4};
    pms_status st;
    Tune best = c->tune;
    float best_aniso = 1e30f, best_field = 1e30f;
    for (int bd : sizes)
        for (int bm : sizes) {
            c->tune.density_threads = bd;
            c->tune.moments_threads = bm;
            float ms;
            if ((st = time_ms(c, 3, &ms, launch_density_aniso))) return st;
            if (ms < best_aniso) { best_aniso = ms; best.density_threads = bd; best.moments_threads = bm; }
        }
    c->tune.density_threads = best.density_threads;
    c->tune.moments_threads = best.moments_threads;
    if (c->nv) {
        for (int k : vpts)
            for (int bt : sizes)
                for (int w : waves) {
                    c->tune.field_vpt = k;
                    c->tune.field_threads = bt;
                    c->tune.field_waves = w;
                    float ms;
                    if ((st = time_ms(c, 3, &ms, launch_field))) return st;
                    if (ms < best_field) {
                        best_field = ms; best.field_threads = bt; best.field_waves = w; best.field_vpt = k;
                    }
                }
    }
    c->tune = best;
    // leave the frame's results as they were (the last re-runs used other shapes; values are identical)
    if ((st = launch_density_aniso(c))) return st;
    if (c->nv && (st = launch_field(c))) return st;
    PMS_CUDA(c, cudaMemcpyAsync(c->counters.p, &saved, sizeof(Counters), cudaMemcpyHostToDevice, c->stream));
    PMS_CUDA(c, cudaStreamSynchronize(c->stream));
    if (out) {
        out->field_threads = best.field_threads;
        out->field_waves = best.field_waves;
        out->field_vpt = best.field_vpt;
        out->density_threads = best.density_threads;
        out->moments_threads = best.moments_threads;
        out->anisotropy_ms = best_aniso;
        out->field_ms = c->nv ? best_field : 0.f;
    }
    return PMS_OK;
}

static bool valid_threads(int t) { return t == 64 || t == 128 || t == 256; }

extern "C" pms_status pms_set_tune(pms_ctx* c, const pms_tune* t) {
    if (!c || !t) return PMS_ERR_INVALID_ARGUMENT;
    if (!valid_threads(t->field_threads) || !valid_threads(t->density_threads) || !valid_threads(t->moments_threads) ||
        t->field_waves < 1 || t->field_waves > 64 || (t->field_vpt != 1 && t->field_vpt != 2 && t->field_vpt != 4))
        return pms_fail(c, PMS_ERR_INVALID_ARGUMENT, "launch shape outside the tuned set");
    c->tune.field_threads = t->field_threads;
    c->tune.field_waves = t->field_waves;
    c->tune.field_vpt = t->field_vpt;
    c->tune.density_threads = t->density_threads;
    c->tune.moments_threads = t->moments_threads;
    return PMS_OK;
}

extern "C" pms_status pms_get_tune(pms_ctx* c, pms_tune* out) {
    if (!c || !out) return PMS_ERR_INVALID_ARGUMENT;
    out->field_threads = c->tune.field_threads;
    out->field_waves = c->tune.field_waves;
    out->field_vpt = c->tune.field_vpt;
    out->density_threads = c->tune.density_threads;
    out->moments_threads = c->tune.moments_threads;
    out->anisotropy_ms = out->field_ms = 0.f;
    return PMS_OK;
}
