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
pms_status launch_cube_corners(pms_ctx* ctx, const uint32_t* cubes, const uint32_t* exclude, uint32_t* out,
                               uint32_t* wcount);
// the corners of the cubes of a bitmap, listed in no particular order; *n_list their count
pms_status launch_corner_list(pms_ctx* ctx, const uint32_t* cubes, uint32_t* list, uint32_t* n_list);
pms_status launch_bits_or(pms_ctx* ctx, const uint32_t* a, const uint32_t* b, uint32_t* out, uint32_t* wcount);
// border checks queue cubes in qadd (a bitmap) and, when qlist is given, in a
// list of at most qcap entries; the count (l_added) may exceed qcap
pms_status launch_border(pms_ctx* ctx, uint32_t* qadd, uint32_t* qlist = nullptr, uint32_t qcap = 0);
// corners of n queued cubes not yet in the vertex bitmap: set there and appended to vnew
pms_status launch_queue_corners(pms_ctx* ctx, const uint32_t* cubes, uint32_t n, uint32_t* vnew, uint32_t* n_new);
pms_status launch_label_bits(pms_ctx* ctx, uint32_t* lbm);
// cube bitmap of the compacted valid-cube records (bits: zeroed)
pms_status launch_valid_bits(pms_ctx* ctx, uint32_t* bits);
// n: the list length, or a bound when n_dev holds it on the device
pms_status launch_border_list(pms_ctx* ctx, const uint32_t* cubes, uint32_t n, uint32_t* qadd,
                              const uint32_t* n_dev = nullptr, uint32_t* qlist = nullptr, uint32_t qcap = 0);
pms_status launch_popc(pms_ctx* ctx, const uint32_t* b, uint32_t* wcount);
// corners of the classified valid cubes outside the plain band leave the vertex
// set (bitmap and dense field); Counters::l_removed counts them
pms_status plain_band_filter(pms_ctx* ctx);
pms_status launch_features(pms_ctx* ctx, const uint32_t* cubes, uint32_t n, uint16_t* x);
cudaError_t launch_train(const pms_ctx* data, cudaStream_t stream, const TrainArgs& a, const DevModel* model, float* grad,
                         float* loss_sum);
cudaError_t launch_adam(cudaStream_t stream, float* w, const float* grad, float* m, float* v, const AdamParams& ap,
                        DevModel* model);

}  // namespace pms
