// American exercise by least-squares Monte Carlo (placeholder until the LSMC kernels land).
#include "../../include/kgpu.h"
#include "api_internal.h"

extern "C" kgpu_status kgpu_lsmc_price(kgpu_context* ctx, const kgpu_model* model, double strike,
                                       double sign, double expiry, const kgpu_lsmc_settings* settings,
                                       uint64_t fresh_seed, kgpu_lsmc_result* out) {
    (void)model; (void)strike; (void)sign; (void)expiry; (void)settings; (void)fresh_seed; (void)out;
    if (ctx) ctx->error = "LSMC is not built in this library";
    return KGPU_UNSUPPORTED_OPERATION;
}
