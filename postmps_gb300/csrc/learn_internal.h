// learn_internal.h -- learned narrow band: device model layout, trainer state
// and launchers shared by k_learn.cu and pms_learn.cpp.
#pragma once
#include "pms_internal.h"

namespace pms {

static constexpr int kIn = PMS_BAND_MLP_INPUTS, kHid = PMS_BAND_MLP_HIDDEN;
// parameter vector (fp32 master weights and gradients):
// W1[i * 64 + j] (input i -> hidden j), b1[64], w2[64], b2
static constexpr int kOffB1 = kIn * kHid, kOffW2 = kOffB1 + kHid, kOffB2 = kOffW2 + kHid;
static constexpr int kNumParams = PMS_BAND_MLP_PARAMS;
static_assert(kOffB2 + 1 == kNumParams, "parameter layout");

// the device copy of the model has the public struct's layout
using DevModel = pms_band_model;

// coarse density grid: a vertex on every second scalar-grid vertex
struct LearnDims {
    uint32_t cres[3];        // coarse vertices per axis
    uint32_t tiles[3];       // prediction tiles per axis (4 coarse cells each)
    float inv_expected;      // 1 / particles per coarse cell at the lattice spacing
};

struct AdamParams {
    float lr, beta1, beta2, eps, inv_bc1, inv_bc2;
};

struct TrainArgs {
    const uint16_t* x = nullptr;   // explicit features (bf16 bits, 64 per sample), or null
    const uint8_t* y = nullptr;    // explicit labels
    uint32_t batch = 0;
    uint64_t seed = 0;
    float pos_weight = 1.f;
};

LearnDims learn_dims(const pms_ctx* ctx);
pms_status launch_coarse_counts(pms_ctx* ctx);
pms_status launch_predict(pms_ctx* ctx, int use_model, uint32_t* q, uint32_t* cand, float* logit, uint32_t cand_cap);
// the plain band (ctx->bm) split into the corners of the cubes of a cube bitmap (E,
// evaluated exactly at once) and the rest (N, certified); cubes null: E empty
pms_status launch_band_split(pms_ctx* ctx, const uint32_t* cubes, uint32_t* e_bm, uint32_t* n_bm, uint32_t* e_wc,
                             uint32_t* n_wc);
// the certified corners (bits of cert) of the classified valid cubes move to recheck
pms_status launch_recheck_bits(pms_ctx* ctx, uint32_t* cert, uint32_t* recheck);
pms_status launch_popc(pms_ctx* ctx, const uint32_t* b, uint32_t* wcount);
pms_status launch_label_bits(pms_ctx* ctx, uint32_t* lbm);
// the learned band after the plain band (ctx->bm, ctx->vlist; ctx->nv its count, or a
// bound for batched frames): prediction and split, then the field stage (exact field
// at E, certification of N, classification, exact field at the rechecked corners,
// band-order field); no host synchronisation
pms_status ensure_learned_buffers(pms_ctx* ctx, uint64_t sc_size, uint32_t nv);
pms_status learned_split(pms_ctx* ctx, bool predict);
pms_status learned_field(pms_ctx* ctx);
pms_status launch_features(pms_ctx* ctx, const uint32_t* cubes, uint32_t n, uint16_t* x);
// one training pass over a batch on the tensor cores; err collects kErrTimeout /
// kErrTcLost when a bounded wait on the MMAs ran out
cudaError_t launch_train(const pms_ctx* data, cudaStream_t stream, const TrainArgs& a, const DevModel* model, float* grad,
                         float* loss_sum, uint32_t* err);
cudaError_t launch_adam(cudaStream_t stream, float* w, const float* grad, float* m, float* v, const AdamParams& ap,
                        DevModel* model);

}  // namespace pms
