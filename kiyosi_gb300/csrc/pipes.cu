// Pipe throughput of the device, measured: the denominators of the path kernels' op-model
// roofline (FP32 fused multiply-add, its packed two-lane form, integer logic, the
// multi-function unit's base-2 logarithm, L1-resident loads).  Each kernel runs many
// independent chains of one operation per thread at full occupancy; the rate is the
// operations completed per second, timed with CUDA events on the context's stream.
#include <cuda_runtime.h>

#include "../../include/kgpu.h"
#include "api_internal.h"

namespace {

constexpr int kChains = 8;      // independent dependency chains per thread
constexpr int kIterations = 4096;
constexpr int kBlock = 256;

__global__ void __launch_bounds__(kBlock) ffma_kernel(float* sink, float a, float b) {
    float x[kChains];
    for (int c = 0; c < kChains; ++c) x[c] = float(threadIdx.x + c);
    for (int i = 0; i < kIterations; ++i)
#pragma unroll
        for (int c = 0; c < kChains; ++c) asm volatile("fma.rn.f32 %0, %0, %1, %2;" : "+f"(x[c]) : "f"(a), "f"(b));
    float s = 0.f;
    for (int c = 0; c < kChains; ++c) s += x[c];
    if (s == 1234.5f) sink[threadIdx.x] = s;
}

__global__ void __launch_bounds__(kBlock) ffma2_kernel(float* sink, float a, float b) {
    float2 x[kChains];
    for (int c = 0; c < kChains; ++c) x[c] = make_float2(float(threadIdx.x + c), float(c));
    const float2 va = make_float2(a, a), vb = make_float2(b, b);
    for (int i = 0; i < kIterations; ++i)
#pragma unroll
        for (int c = 0; c < kChains; ++c) x[c] = __ffma2_rn(x[c], va, vb);
    float s = 0.f;
    for (int c = 0; c < kChains; ++c) s += x[c].x + x[c].y;
    if (s == 1234.5f) sink[threadIdx.x] = s;
}

__global__ void __launch_bounds__(kBlock) lop3_kernel(unsigned* sink, unsigned a, unsigned b) {
    unsigned x[kChains];
    for (int c = 0; c < kChains; ++c) x[c] = threadIdx.x * 2654435761u + c;
    for (int i = 0; i < kIterations; ++i)
#pragma unroll
        for (int c = 0; c < kChains; ++c)
            asm volatile("lop3.b32 %0, %0, %1, %2, 0x96;" : "+r"(x[c]) : "r"(a), "r"(b));
    unsigned s = 0;
    for (int c = 0; c < kChains; ++c) s ^= x[c];
    if (s == 12345u) sink[threadIdx.x] = s;
}

__global__ void __launch_bounds__(kBlock) lg2_kernel(float* sink) {
    float x[kChains];
    for (int c = 0; c < kChains; ++c) x[c] = 1.5f + float(threadIdx.x + c);
    for (int i = 0; i < kIterations; ++i)
#pragma unroll
        for (int c = 0; c < kChains; ++c) asm volatile("lg2.approx.f32 %0, %0;" : "+f"(x[c]));
    float s = 0.f;
    for (int c = 0; c < kChains; ++c) s += x[c];
    if (s == 1234.5f) sink[threadIdx.x] = s;
}

// 32-bit loads that hit L1, every lane of a warp at the same address (the path kernels'
// table reads are broadcasts): each warp walks a 4 KiB table with a dependent index, as
// kChains independent walks.
__global__ void __launch_bounds__(kBlock) load_kernel(const unsigned* table, unsigned* sink) {
    unsigned x[kChains];
    for (int c = 0; c < kChains; ++c) x[c] = ((threadIdx.x >> 5) * 61u + 37u * c) & 1023u;
    for (int i = 0; i < kIterations; ++i)
#pragma unroll
        for (int c = 0; c < kChains; ++c) x[c] = __ldg(table + x[c]);
    unsigned s = 0;
    for (int c = 0; c < kChains; ++c) s ^= x[c];
    if (s == 12345u) sink[threadIdx.x] = s;
}

__global__ void fill_table_kernel(unsigned* table) {
    const unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < 1024) table[i] = (i * 613u + 17u) & 1023u;
}

}  // namespace

extern "C" kgpu_status kgpu_pipe_rates(kgpu_context* ctx, double* rates, int32_t count) {
    if (!ctx || !rates || count < 1) return KGPU_INVALID_INPUT;
    std::lock_guard<std::mutex> lock(ctx->mu);
    if (cudaSetDevice(ctx->device) != cudaSuccess) return KGPU_DEVICE_ERROR;
    if (ctx->stream_out.ensure(64 * 1024)) return KGPU_DEVICE_ERROR;
    unsigned* table = static_cast<unsigned*>(ctx->stream_out.ptr);
    float* sink = reinterpret_cast<float*>(table + 2048);
    const int blocks = ctx->sm_count * 8;  // 2048 threads per SM
    const double threads = double(blocks) * kBlock;
    const double ops = threads * kChains * double(kIterations);
    fill_table_kernel<<<4, 256, 0, ctx->stream>>>(table);
    cudaEvent_t start, stop;
    if (cudaEventCreate(&start) != cudaSuccess || cudaEventCreate(&stop) != cudaSuccess) return KGPU_DEVICE_ERROR;
    auto timed = [&](int which) -> double {
        float best = 0.f;
        for (int rep = 0; rep < 3; ++rep) {
            cudaEventRecord(start, ctx->stream);
            switch (which) {
                case 0: ffma_kernel<<<blocks, kBlock, 0, ctx->stream>>>(sink, 1.0000001f, 0.5f); break;
                case 1: ffma2_kernel<<<blocks, kBlock, 0, ctx->stream>>>(sink, 1.0000001f, 0.5f); break;
                case 2: lop3_kernel<<<blocks, kBlock, 0, ctx->stream>>>(table + 1024, 0x9e3779b9u, 0x7f4a7c15u); break;
                case 3: lg2_kernel<<<blocks, kBlock, 0, ctx->stream>>>(sink); break;
                default: load_kernel<<<blocks, kBlock, 0, ctx->stream>>>(table, table + 1024); break;
            }
            cudaEventRecord(stop, ctx->stream);
            cudaEventSynchronize(stop);
            float ms = 0.f;
            cudaEventElapsedTime(&ms, start, stop);
            if (rep == 0 || ms < best) best = ms;
        }
        const double per = which == 1 ? 2.0 : 1.0;  // FFMA2: two lanes of FMA per operation
        return best > 0.f ? ops * per / (double(best) * 1e-3) : 0.0;
    };
    // rates[0] FFMA, [1] FFMA2 (FMAs), [2] LOP3, [3] MUFU lg2, [4] L1-hit broadcast
    // loads; thread operations per second.
    for (int i = 0; i < count && i < 5; ++i) rates[i] = timed(i);
    for (int i = 5; i < count; ++i) rates[i] = 0.0;
    cudaEventDestroy(start);
    cudaEventDestroy(stop);
    return cudaGetLastError() == cudaSuccess ? KGPU_OK : KGPU_DEVICE_ERROR;
}
