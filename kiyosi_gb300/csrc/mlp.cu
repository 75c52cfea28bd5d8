// MLP continuation regression for LSMC (placeholder until the tensor-core kernels land).
#include "../../include/kgpu.h"
#include "api_internal.h"

kgpu_status kgpu_lsmc_mlp(kgpu_context* ctx, const kgpu_model*, double, double, double,
                          const kgpu_lsmc_settings*, uint64_t, kgpu_lsmc_result*) {
    ctx->error = "the MLP continuation basis is not built in this library";
    return KGPU_UNSUPPORTED_OPERATION;
}
