// k_diffuse.cu -- diffuse (spray / foam / bubble) particle generation.
// (stage entry points; kernels follow)
#include "pms_internal.h"
#include "k_common.cuh"

namespace pms {
pms_status launch_diffuse(pms_ctx* ctx) {
    return pms_fail(ctx, PMS_ERR_UNSUPPORTED, "diffuse generation is not built yet");
}
}  // namespace pms

pms_status pms::diffuse_debug(pms_ctx* ctx, int id, std::vector<uint8_t>& out) {
    (void)out;
    return pms_fail(ctx, PMS_ERR_INVALID_ARGUMENT, "unknown array id %d", id);
}

pms_status pms::write_diffuse_frame(pms_ctx* ctx, const pms_config& cfg, int frame) {
    (void)cfg; (void)frame;
    return pms_fail(ctx, PMS_ERR_UNSUPPORTED, "diffuse generation is not built yet");
}

extern "C" pms_status pms_download_diffuse(pms_ctx* ctx, int type, float* pos, float* vel, int32_t* type_out,
                                           int32_t* ttl, float* wc, float* ta, float* en, uint32_t cap, uint32_t* n_out) {
    (void)type; (void)pos; (void)vel; (void)type_out; (void)ttl; (void)wc; (void)ta; (void)en; (void)cap;
    if (n_out) *n_out = 0;
    return pms_fail(ctx, PMS_ERR_UNSUPPORTED, "diffuse generation is not built yet");
}
