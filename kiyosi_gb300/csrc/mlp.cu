// Least-squares Monte Carlo with a learned continuation value.
//
// At each exercise date the continuation value is the reference's least-squares
// polynomial (crates/kiyosi/src/engines/monte_carlo/american.rs:1347-1417, the cubic
// (S/K, v/theta) basis of the Heston path store) plus a small network
// f(x) = w3 . relu(W2 relu(W1 x + b1) + b2) + b3 with 3 inputs (log moneyness, variance,
// time), two hidden layers of 64 and one output, fitted by Adam on the mean squared error
// to what the polynomial leaves unexplained: the in-the-money paths' discounted cash
// flows minus the polynomial's fit.  A network that learns nothing leaves the
// polynomial method exactly.  Exercise decisions, the date-0 estimate and the
// out-of-sample lower bound follow the polynomial method step for step with the sum in
// place of the polynomial.
//
// Training runs on the fifth-generation tensor cores: one CTA holds 128 samples; the
// 64 x 64 layer's forward product, the backward product through it and every gradient's
// sum over the samples (W2 and b2; W1 and b1; w3) are tcgen05 MMAs (BF16 operands in
// shared memory, FP32 accumulators in tensor memory); the 3 -> 64 and 64 -> 1 layers'
// forward values and the activations run on the CUDA cores in FP32.  Per-CTA gradient
// partials are summed in a fixed order before Adam, so training is deterministic.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <mutex>
#include <vector>

#include "../../include/kgpu.h"
#include "api_internal.h"
#include "lsmc_common.cuh"
#include "tcgen05.cuh"

#include <cooperative_groups.h>

namespace kgpu {
namespace {

constexpr int kHidden = 64;
constexpr int kRows = 128;  // samples per training CTA (the MMA's M)
constexpr int kThreadsTrain = 256;  // two threads per sample, one per half of the hidden units
// Parameter vector: W1[64][3], b1[64], W2[64][64] (row = output unit), b2[64], w3[64], b3.
constexpr int kPW1 = 0, kPB1 = 192, kPW2 = 256, kPB2 = 4352, kPW3 = 4416, kPB3 = 4480;
constexpr int kParams = 4481;
constexpr int kStride = 4484;  // per-CTA partial: kParams gradients, then the loss sum; also the
                               // 16-byte-aligned stride of every parameter-sized region
constexpr int kLossSlot = 4481;
// Tensor memory: [0,64) Z2, [64,128) dH1, [128,208) dW2 and db2, [256,272) the small
// gradients (dW1, db1 in lanes 0..63; dW3 in lanes 64..127).
constexpr uint32_t kTmemColumns = 512;
constexpr uint32_t kColZ2 = 0, kColDH1 = 64, kColDW2 = 128, kColSmall = 256;
constexpr int kH1Rows = kHidden + 16;  // H1^T, a row of ones (db2) and 15 zero rows: N = 80

// Every sum over a tile's rows is a tensor-core product with the rows as K:
//   [dW2 | db2]  = dZ2^T (outputs, padded to M = 128) . [H1 | 1]       (N = 80)
//   [dW1 | db1]  = dZ1^T . [x0 x1 x2 1]   and   dW3 = relu(Z2)^T . dout,
// the last two as one product: A stacks dZ1^T (units 0..63) on relu(Z2)^T (64..127), B
// holds the rows' x0, x1, x2, 1 and dout (N = 16).  BF16 operands, FP32 sums.
struct __align__(1024) TrainSmem {
    __nv_bfloat16 h1[kRows * kHidden];       // A of the forward product: rows x inputs
    __nv_bfloat16 h1t[kH1Rows * kRows];      // B of [dW2 | db2]: inputs, ones, zeros x rows
    __nv_bfloat16 dz2[kRows * kHidden];      // A of the backward product: rows x outputs
    __nv_bfloat16 dz2t[kRows * kRows];       // A of [dW2 | db2]: outputs (64 + 64 zero) x rows
    __nv_bfloat16 gt[kRows * kRows];         // A of the small gradients: dZ1^T, relu(Z2)^T x rows
    __nv_bfloat16 xe[16 * kRows];            // B of the small gradients: x0, x1, x2, 1, dout, zeros x rows
    __nv_bfloat16 w2f[kHidden * kHidden];    // B forward: outputs x inputs
    __nv_bfloat16 w2b[kHidden * kHidden];    // B backward: inputs x outputs
    float4 l1[kHidden];  // layer 1 of unit j: W1[j][0..2], b1[j] (one 16-byte load)
    float b2[kHidden], w3[kHidden];
    float b3;
    // The clustered trainer's gradient sums of this CTA and its published parameters,
    // both in slot order (see slot_of).
    alignas(16) float acc[kStride];
    alignas(16) float pub[kStride];
    float red[16];       // per-warp sums of db3 and of the squared residuals
    float xch[256];      // output halves exchanged between the two threads of a row
    uint64_t bar;
    uint32_t tmem;
    int failed;
};

constexpr size_t kTrainSmemBytes = sizeof(TrainSmem) + 1024;

__device__ __forceinline__ float bf16_round(float x) { return __bfloat162float(__float2bfloat16_rn(x)); }

// Prepares a training CTA: tensor memory, the completion barrier and the constant rows
// of the gradient operands (rows 64..127 of dz2t, rows 64..79 of h1t, rows 5..15 of xe;
// they stay unchanged across steps).
__device__ __forceinline__ void train_setup(TrainSmem& s) {
    const int t = threadIdx.x;
    if ((t >> 5) == 0) {
        tc::tmem_alloc(&s.tmem, kTmemColumns);
        tc::tmem_relinquish();
    }
    if (t == 0) {
        tc::mbar_init(&s.bar, 1);
        s.failed = 0;
    }
    const __nv_bfloat16 zero = __float2bfloat16_rn(0.0f), one = __float2bfloat16_rn(1.0f);
    for (int i = t; i < kHidden * kRows; i += kThreadsTrain) s.dz2t[kHidden * kRows + i] = zero;
    for (int i = t; i < 16 * kRows; i += kThreadsTrain) {
        const int r = kHidden + i / kRows, c = i % kRows;
        s.h1t[tc::kmajor(r, c, kRows)] = r == kHidden ? one : zero;
        if (i / kRows >= 5) s.xe[tc::kmajor(i / kRows, c, kRows)] = zero;
    }
}

__device__ __forceinline__ void train_release(TrainSmem& s) {
    tc::fence_before_sync();
    __syncthreads();
    if ((threadIdx.x >> 5) == 0) tc::tmem_dealloc(s.tmem, kTmemColumns);
}

// Slot order of the clustered trainer's gradient sums and parameters: W2 transposed
// (slot in * 64 + o for W2[o][in]; a warp's 32 output units are 32 consecutive slots),
// then W1, b1, b2, w3, b3 (slots 4096..4480), the loss (4481) and two unused slots.
__host__ __device__ constexpr int slot_of(int param) {
    return param >= kPW2 && param < kPB2 ? ((param - kPW2) & 63) * kHidden + ((param - kPW2) >> 6)
           : param < kPW2               ? kHidden * kHidden + param
                                        : kHidden * kHidden + kPW2 + (param - kPB2);
}
__host__ __device__ constexpr int param_of_slot(int slot) {
    return slot < kHidden * kHidden ? kPW2 + (slot & 63) * kHidden + (slot >> 6)
           : slot < kHidden * kHidden + kPW2 ? slot - kHidden * kHidden
           : slot < kHidden * kHidden + kPW2 + (kParams - kPB2) ? kPB2 + slot - kHidden * kHidden - kPW2
                                                                 : -1;
}
static_assert(slot_of(kPB3) == 4480 && param_of_slot(4480) == kPB3 && param_of_slot(slot_of(kPW2 + 70)) == kPW2 + 70,
              "slot order");

// One batch's gradient partial of this CTA: it covers samples
// [first + 128 blockIdx.x, first + 128 blockIdx.x + 128) of the batch [first, first + count)
// and writes to `partial` (element stride `pstride`) its share of the gradient of
// (1 / count) sum (f(x) - y)^2 and its sum of squared residuals.  Thread t owns row
// t % 128 and hidden units [32 h, 32 h + 32) with h = t / 128; warps w and w + 4 read the
// same tensor-memory lanes, one column half each.  `phase` is the completion barrier's
// next parity (two completions per step).  Returns false, on every thread, when a
// tensor-core wait gave up.
template <bool kLocal>
__device__ bool grad_step(TrainSmem& s, const float* __restrict__ params, const uint4* __restrict__ w2_tiles,
                          const float4* __restrict__ samples, int first, int count, float inv_count,
                          float* __restrict__ partial, int pstride, uint32_t& phase) {
    const int t = threadIdx.x, warp = t >> 5;
    const int row = t & (kRows - 1), half = t >> 7, j0 = 32 * half;
    // A gradient value: to the partial (parameter order, stride pstride), or with kLocal
    // to this CTA's sums in shared memory (slot order).
    auto put = [&](int param, float value) {
        if (kLocal) s.acc[slot_of(param)] = value;
        else partial[size_t(param) * pstride] = value;
    };
    if (!kLocal) {
    // Parameters are read past L1 (ld.global.cg): the persistent trainer rewrites them
    // from other SMs between steps.
    if (t < kHidden) {
        s.l1[t] = make_float4(__ldcg(params + kPW1 + 3 * t), __ldcg(params + kPW1 + 3 * t + 1),
                              __ldcg(params + kPW1 + 3 * t + 2), __ldcg(params + kPB1 + t));
        s.b2[t] = __ldcg(params + kPB2 + t);
        s.w3[t] = __ldcg(params + kPW3 + t);
    }
    s.b3 = __ldcg(params + kPB3);
    if (w2_tiles) {
        // Both BF16 operand tiles of W2, already in shared-memory order (16 KB).
        uint4* dst = reinterpret_cast<uint4*>(s.w2f);  // w2f and w2b are contiguous
        for (int i = t; i < 2 * kHidden * kHidden / 8; i += kThreadsTrain) dst[i] = __ldcg(w2_tiles + i);
    } else {
        for (int i = t; i < kHidden * kHidden; i += kThreadsTrain) {
            const int o = i >> 6, in = i & 63;
            const __nv_bfloat16 w = __float2bfloat16_rn(__ldcg(params + kPW2 + i));
            s.w2f[tc::kmajor(o, in, kHidden)] = w;
            s.w2b[tc::kmajor(in, o, kHidden)] = w;
        }
    }
    }  // the clustered trainer keeps the network in shared memory
    const int local = blockIdx.x * kRows + row;
    const bool valid = local < count;
    const float4 x = valid ? samples[first + local] : make_float4(0.f, 0.f, 0.f, 0.f);
    __syncthreads();

    // Layer 1 on the CUDA cores for this thread's 32 units; H1 goes to shared memory in
    // both operand layouts (8 consecutive units of a row are one 16-byte store).
    uint32_t mask1 = 0;
#pragma unroll
    for (int g = 0; g < 4; ++g) {
        __align__(16) __nv_bfloat16 pack[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) {
            const int j = j0 + 8 * g + u;
            const float4 w = s.l1[j];
            const float z = fmaf(w.x, x.x, fmaf(w.y, x.y, fmaf(w.z, x.z, w.w)));
            if (z > 0.f) mask1 |= 1u << (8 * g + u);
            pack[u] = __float2bfloat16_rn(valid && z > 0.f ? z : 0.f);
            s.h1t[tc::kmajor(j, row, kRows)] = pack[u];
        }
        *reinterpret_cast<uint4*>(&s.h1[tc::kmajor(row, j0 + 8 * g, kHidden)]) = *reinterpret_cast<const uint4*>(pack);
    }
    // The row's inputs of the small gradients (zero past the batch).
    if (half == 0) {
        s.xe[tc::kmajor(0, row, kRows)] = __float2bfloat16_rn(x.x);
        s.xe[tc::kmajor(1, row, kRows)] = __float2bfloat16_rn(x.y);
        s.xe[tc::kmajor(2, row, kRows)] = __float2bfloat16_rn(x.z);
        s.xe[tc::kmajor(3, row, kRows)] = __float2bfloat16_rn(valid ? 1.0f : 0.0f);
    }
    tc::fence_async_smem();
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tmem = s.tmem;
    const uint32_t idesc = tc::idesc_bf16(kRows, kHidden);
    if (t == 0) {
        const uint32_t a0 = tc::smem_u32(s.h1), b0 = tc::smem_u32(s.w2f);
        for (int k = 0; k < kHidden / 16; ++k)
            tc::mma_bf16(tmem + kColZ2, tc::smem_desc(a0 + 256 * k, 128, kHidden * 16),
                         tc::smem_desc(b0 + 256 * k, 128, kHidden * 16), idesc, k > 0);
        tc::mma_commit(&s.bar);
    }
    bool ok = tc::mbar_wait(&s.bar, phase);
    phase ^= 1u;
    if (__syncthreads_or(!ok)) return false;
    tc::fence_after_sync();
    // Z2 of this row's 32 units (TMEM lane = row).
    const uint32_t lane_base = uint32_t((warp & 3) * 32) << 16;
    float z2[32];
    tc::tmem_load32(tmem + lane_base + kColZ2 + j0, z2);
    float out = 0.f;
#pragma unroll
    for (int u = 0; u < 32; ++u) {
        z2[u] += s.b2[j0 + u];
        out = fmaf(z2[u] > 0.f ? z2[u] : 0.f, s.w3[j0 + u], out);
    }
    // The output needs both halves: exchange through shared memory.
    s.xch[t] = out;
    __syncthreads();
    out = (s.b3 + s.xch[row]) + s.xch[row + kRows];
    const float res = valid ? out - x.w : 0.f;
    const float dout = 2.f * res * inv_count;
    // dZ2 in both operand layouts, relu(Z2)^T, and dout.
#pragma unroll
    for (int g = 0; g < 4; ++g) {
        __align__(16) __nv_bfloat16 pack[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) {
            const int k = 8 * g + u, j = j0 + k;
            const bool on = z2[k] > 0.f;
            pack[u] = __float2bfloat16_rn(on ? dout * s.w3[j] : 0.f);
            s.dz2t[tc::kmajor(j, row, kRows)] = pack[u];
            s.gt[tc::kmajor(kHidden + j, row, kRows)] = __float2bfloat16_rn(on ? z2[k] : 0.f);
        }
        *reinterpret_cast<uint4*>(&s.dz2[tc::kmajor(row, j0 + 8 * g, kHidden)]) = *reinterpret_cast<const uint4*>(pack);
    }
    if (half == 0) s.xe[tc::kmajor(4, row, kRows)] = __float2bfloat16_rn(dout);
    tc::fence_async_smem();
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    if (t == 0) {
        const uint32_t ad = tc::smem_u32(s.dz2), bw = tc::smem_u32(s.w2b);
        for (int k = 0; k < kHidden / 16; ++k)
            tc::mma_bf16(tmem + kColDH1, tc::smem_desc(ad + 256 * k, 128, kHidden * 16),
                         tc::smem_desc(bw + 256 * k, 128, kHidden * 16), idesc, k > 0);
        const uint32_t at = tc::smem_u32(s.dz2t), bh = tc::smem_u32(s.h1t);
        const uint32_t idesc80 = tc::idesc_bf16(kRows, kH1Rows);
        for (int k = 0; k < kRows / 16; ++k)
            tc::mma_bf16(tmem + kColDW2, tc::smem_desc(at + 256 * k, 128, kRows * 16),
                         tc::smem_desc(bh + 256 * k, 128, kRows * 16), idesc80, k > 0);
        tc::mma_commit(&s.bar);
    }
    // db3 and the loss: half 0 holds one copy of every row.
    float d3 = half == 0 ? dout : 0.f, l2 = half == 0 ? res * res : 0.f;
    for (int o = 16; o >= 1; o >>= 1) {
        d3 += __shfl_xor_sync(0xffffffffu, d3, o);
        l2 += __shfl_xor_sync(0xffffffffu, l2, o);
    }
    if ((t & 31) == 0 && half == 0) {
        s.red[warp] = d3;
        s.red[8 + warp] = l2;
    }
    ok = tc::mbar_wait(&s.bar, phase);
    phase ^= 1u;
    if (__syncthreads_or(!ok)) return false;
    tc::fence_after_sync();
    if (t == 0) {
        put(kPB3, ((s.red[0] + s.red[1]) + s.red[2]) + s.red[3]);
        if (kLocal) s.acc[kLossSlot] = ((s.red[8] + s.red[9]) + s.red[10]) + s.red[11];
        else partial[size_t(kLossSlot) * pstride] = ((s.red[8] + s.red[9]) + s.red[10]) + s.red[11];
    }
    // dZ1^T (rows 0..63 of the small gradients' A operand).
    {
        float dh1[32];
        tc::tmem_load32(tmem + lane_base + kColDH1 + j0, dh1);
#pragma unroll
        for (int k = 0; k < 32; ++k)
            s.gt[tc::kmajor(j0 + k, row, kRows)] = __float2bfloat16_rn(((mask1 >> k) & 1u) ? dh1[k] : 0.f);
    }
    tc::fence_async_smem();
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    if (t == 0) {
        const uint32_t ag = tc::smem_u32(s.gt), bx = tc::smem_u32(s.xe);
        const uint32_t idesc16 = tc::idesc_bf16(kRows, 16);
        for (int k = 0; k < kRows / 16; ++k)
            tc::mma_bf16(tmem + kColSmall, tc::smem_desc(ag + 256 * k, 128, kRows * 16),
                         tc::smem_desc(bx + 256 * k, 128, kRows * 16), idesc16, k > 0);
        tc::mma_commit(&s.bar);
    }
    // dW2 and db2 while the tensor cores run: TMEM lanes 0..63 hold rows = output units;
    // warps 0, 1 (inputs 0..31, and db2) and 4, 5 (inputs 32..63) read them.
    if ((warp & 3) < 2) {
        const int unit = row;  // output unit
        float g2[32];
        tc::tmem_load32(tmem + lane_base + kColDW2 + j0, g2);
        if (kLocal) {
            // Slot (j0 + q) * 64 + unit: consecutive lanes, consecutive words.
#pragma unroll
            for (int q = 0; q < 32; ++q) s.acc[(j0 + q) * kHidden + unit] = g2[q];
        } else if (pstride == 1) {
            float4* dst = reinterpret_cast<float4*>(partial + kPW2 + unit * kHidden + j0);
#pragma unroll
            for (int q = 0; q < 8; ++q) dst[q] = make_float4(g2[4 * q], g2[4 * q + 1], g2[4 * q + 2], g2[4 * q + 3]);
        } else {
#pragma unroll
            for (int q = 0; q < 32; ++q) partial[size_t(kPW2 + unit * kHidden + j0 + q) * pstride] = g2[q];
        }
        if (half == 0) {
            float b[4];
            tc::tmem_load4(tmem + lane_base + kColDW2 + kHidden, b);
            put(kPB2 + unit, b[0]);
        }
    }
    ok = tc::mbar_wait(&s.bar, phase);
    phase ^= 1u;
    if (__syncthreads_or(!ok)) return false;
    tc::fence_after_sync();
    if (warp < 4) {
        float gv[4];
        if (warp < 2) {
            // dW1 (columns 0..2) and db1 (column 3) of units 0..63.
            tc::tmem_load4(tmem + lane_base + kColSmall, gv);
            const int unit = 32 * warp + (t & 31);
#pragma unroll
            for (int c = 0; c < 3; ++c) put(kPW1 + 3 * unit + c, gv[c]);
            put(kPB1 + unit, gv[3]);
        } else {
            // dW3 (column 4) of units 0..63, in lanes 64..127.
            tc::tmem_load4(tmem + lane_base + kColSmall + 4, gv);
            put(kPW3 + 32 * (warp - 2) + (t & 31), gv[0]);
        }
    }
    return true;
}

// One batch's gradient partials (partials[b] for CTA b); used for gradient checks.
__global__ void __launch_bounds__(kThreadsTrain, 1) mlp_grad_kernel(const float* __restrict__ params,
                                                            const float4* __restrict__ samples, int first,
                                                            int count, float inv_count, float* __restrict__ partials,
                                                            int* __restrict__ error) {
    extern __shared__ unsigned char smem_raw[];
    TrainSmem& s = *reinterpret_cast<TrainSmem*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    train_setup(s);
    uint32_t phase = 0;
    if (!grad_step<false>(s, params, nullptr, samples, first, count, inv_count, partials + size_t(blockIdx.x) * kStride, 1,
                   phase) &&
        threadIdx.x == 0)
        atomicExch(error, 1);
    train_release(s);
}

// Adam (Kingma and Ba, 2015) on the summed CTA partials, in FP32.
__global__ void mlp_adam_kernel(const float* __restrict__ partials, int blocks, float* __restrict__ params,
                                float* __restrict__ m, float* __restrict__ v, float lr, float beta1, float beta2,
                                float eps, float bias1, float bias2) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= kParams) return;
    float g = 0.f;
    for (int b = 0; b < blocks; ++b) g += partials[size_t(b) * kStride + i];
    const float mi = beta1 * m[i] + (1.f - beta1) * g;
    const float vi = beta2 * v[i] + (1.f - beta2) * g * g;
    m[i] = mi;
    v[i] = vi;
    params[i] -= lr * (mi / bias1) / (sqrtf(vi / bias2) + eps);
}

// Grid barrier of a cooperative launch (every CTA resident): arrive on a counter, the
// last arrival advances the generation.  A wait that outlives ~`max_cycles` sets
// `*error` and returns false so the kernel can stop instead of hanging.
struct GridBarrier {
    unsigned int count;
    unsigned int generation;
};

__device__ __forceinline__ bool grid_barrier(GridBarrier* bar, unsigned int ctas, int* error,
                                             long long max_cycles = 2000000000LL) {
    __shared__ int ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        ok = 1;
        volatile unsigned int* gen = &bar->generation;
        const unsigned int g = *gen;
        __threadfence();
        if (atomicAdd(&bar->count, 1u) == ctas - 1) {
            bar->count = 0;
            __threadfence();
            atomicAdd(&bar->generation, 1u);
        } else {
            const long long start = clock64();
            while (*gen == g) {
                if (clock64() - start > max_cycles || *reinterpret_cast<volatile int*>(error)) {
                    atomicExch(error, 1);
                    ok = 0;
                    break;
                }
            }
        }
        __threadfence();
    }
    __syncthreads();
    return ok != 0;
}

struct TrainArgs {
    float* params;
    __nv_bfloat16* w2_tiles;  // [2][64 * 64]: forward then backward operand order
    float* m;
    float* v;
    const float4* samples;
    float* partials;
    GridBarrier* barrier;
    int* error;
    int itm, batch, steps, first_step;  // first_step: Adam steps taken before this launch
    float lr, beta1, beta2, eps;
};

// Every Adam step of one exercise date in one cooperative launch: each step computes
// the batch's gradient partials (one CTA per 128 samples), then every CTA sums the
// partials of its slice of the parameters in CTA order and applies Adam to it.
__global__ void __launch_bounds__(kThreadsTrain, 1) mlp_train_kernel(TrainArgs a) {
    extern __shared__ unsigned char smem_raw[];
    TrainSmem& s = *reinterpret_cast<TrainSmem*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    train_setup(s);
    const unsigned int ctas = gridDim.x;
    const int per_epoch = (a.itm + a.batch - 1) / a.batch;
    const int chunk = (kParams + int(ctas) - 1) / int(ctas);
    const int lo = int(blockIdx.x) * chunk, hi = min(kParams, lo + chunk);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    // W2's BF16 operand tiles for the first step: each CTA lays out its slice.
    for (int i = max(lo, kPW2) + int(threadIdx.x); i < min(hi, kPB2); i += kThreadsTrain) {
        const int w = i - kPW2, o = w >> 6, in = w & 63;
        const __nv_bfloat16 b = __float2bfloat16_rn(__ldcg(a.params + i));
        a.w2_tiles[tc::kmajor(o, in, kHidden)] = b;
        a.w2_tiles[kHidden * kHidden + tc::kmajor(in, o, kHidden)] = b;
    }
    __threadfence();
    uint32_t phase = 0;
    bool ok = grid_barrier(a.barrier, ctas, a.error);
    for (int step = 0; ok && step < a.steps; ++step) {
        const int first = (step % per_epoch) * a.batch;
        const int count = min(a.batch, a.itm - first);
        if (!grad_step<false>(s, a.params, reinterpret_cast<const uint4*>(a.w2_tiles), a.samples, first, count,
                       1.0f / float(count), a.partials + blockIdx.x, int(ctas), phase)) {
            if (threadIdx.x == 0) atomicExch(a.error, 1);
            break;
        }
        if (!grid_barrier(a.barrier, ctas, a.error)) break;
        const float tstep = float(a.first_step + step + 1);
        const float bias1 = 1.0f - powf(a.beta1, tstep), bias2 = 1.0f - powf(a.beta2, tstep);
        const int blocks = (count + kRows - 1) / kRows;
        // Adam on this CTA's slice.  Partials are parameter-major ([param][CTA], at most 64
        // CTAs), so a warp fetches one parameter's partials with two coalesced loads per
        // lane; six parameters per warp are in flight at once, with their Adam state.  The
        // sums use a fixed shuffle tree (deterministic).  Everything here was written by
        // other SMs: it is read past L1.
        for (int i0 = lo + warp * 6; i0 < hi; i0 += (kThreadsTrain / 32) * 6) {
            float g[6], state_m = 0.f, state_v = 0.f, state_w = 0.f;
            const int mine = i0 + lane;
            if (lane < 6 && mine < hi) {
                state_m = __ldcg(a.m + mine);
                state_v = __ldcg(a.v + mine);
                state_w = __ldcg(a.params + mine);
            }
#pragma unroll
            for (int u = 0; u < 6; ++u) {
                const int i = i0 + u;
                const float* row = a.partials + size_t(i < hi ? i : lo) * ctas;
                const float x0 = (i < hi && lane < blocks) ? __ldcg(row + lane) : 0.f;
                const float x1 = (i < hi && lane + 32 < blocks) ? __ldcg(row + lane + 32) : 0.f;
                g[u] = x0 + x1;
            }
#pragma unroll
            for (int u = 0; u < 6; ++u)
                for (int off = 16; off > 0; off >>= 1) g[u] += __shfl_xor_sync(0xffffffffu, g[u], off);
            float gi = g[0];
#pragma unroll
            for (int u = 1; u < 6; ++u) gi = lane == u ? g[u] : gi;
            if (lane < 6 && mine < hi) {
                const float mi = a.beta1 * state_m + (1.f - a.beta1) * gi;
                const float vi = a.beta2 * state_v + (1.f - a.beta2) * gi * gi;
                a.m[mine] = mi;
                a.v[mine] = vi;
                const float w = state_w - a.lr * (mi / bias1) / (sqrtf(vi / bias2) + a.eps);
                a.params[mine] = w;
                if (mine >= kPW2 && mine < kPB2) {
                    const int k = mine - kPW2, o = k >> 6, in = k & 63;
                    const __nv_bfloat16 b = __float2bfloat16_rn(w);
                    a.w2_tiles[tc::kmajor(o, in, kHidden)] = b;
                    a.w2_tiles[kHidden * kHidden + tc::kmajor(in, o, kHidden)] = b;
                }
            }
        }
        __threadfence();
        ok = grid_barrier(a.barrier, ctas, a.error);
    }
    train_release(s);
}

// ---------------------------------------------------------------------------------
// The clustered trainer: the cooperative trainer's 64 CTAs (one 128-sample tile each)
// as 8 thread-block clusters of 8, with the network, the Adam state and the gradient
// sums kept on chip.  Each step:
//   1. every CTA computes its tile's gradient sums into shared memory (slot order);
//   2. cluster barrier; CTA r of a cluster adds the sums of its slice of the slots over
//      the cluster's CTAs in rank order (distributed shared memory) and publishes the
//      cluster's slice to global memory with a flag (step number, release);
//   3. it waits (bounded) for the same slice's flags of the other clusters, adds the
//      8 cluster sums in cluster order and applies Adam to the slice: every cluster
//      computes the same update, and each slot's value and moments stay in the
//      registers of its owning thread;
//   4. cluster barrier; every CTA pulls the whole updated network from the 8 owners
//      of its cluster (16-byte distributed-shared-memory loads) into its copy.
// So a step has two cluster barriers and one point-to-point exchange per slice, no
// grid barrier, and no global traffic but the samples and the 8 x 4484 slice sums.
// The slice sums are double-buffered by step parity: a cluster can run at most one
// step ahead of the slowest, which has read the older buffer by then.
// Every CTA runs the same steps and barriers whatever happens: a tensor-core wait or a
// flag wait that gives up stops the dependent work and raises the error flag.
constexpr int kClusterCtas = 8;
constexpr int kSliceSlots = ((kStride + kClusterCtas - 1) / kClusterCtas + 3) & ~3;  // 564

struct ClusterTrainArgs {
    float* params;    // parameter order; read at the start, written at the end
    float* m;
    float* v;
    const float4* samples;
    float* exchange;  // [2][clusters][kStride] cluster sums of each slice
    int* flags;       // [clusters][kClusterCtas]: last step whose slice sums are published
    int* error;
    int itm, batch, steps, first_step;
    float lr, beta1, beta2, eps;
};

__device__ __forceinline__ uint32_t cluster_address(uint32_t local, int rank) {
    uint32_t out;
    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(out) : "r"(local), "r"(rank));
    return out;
}
__device__ __forceinline__ float4 dsmem_load4(uint32_t addr) {
    float4 v;
    asm volatile("ld.shared::cluster.v4.f32 {%0, %1, %2, %3}, [%4];"
                 : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w)
                 : "r"(addr)
                 : "memory");
    return v;
}
__device__ __forceinline__ void flag_release(int* flag, int value) {
    asm volatile("st.release.gpu.global.s32 [%0], %1;" ::"l"(flag), "r"(value) : "memory");
}
__device__ __forceinline__ int flag_acquire(const int* flag) {
    int v;
    asm volatile("ld.acquire.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(flag) : "memory");
    return v;
}

// Writes a slot's value into this CTA's copy of the network.
__device__ __forceinline__ void set_slot(TrainSmem& s, int slot, float w) {
    if (slot < kHidden * kHidden) {
        const int in = slot >> 6, o = slot & 63;
        const __nv_bfloat16 b = __float2bfloat16_rn(w);
        s.w2f[tc::kmajor(o, in, kHidden)] = b;
        s.w2b[tc::kmajor(in, o, kHidden)] = b;
        return;
    }
    const int p = param_of_slot(slot);
    if (p < 0) return;
    if (p < kPB1) reinterpret_cast<float*>(&s.l1[(p - kPW1) / 3])[(p - kPW1) % 3] = w;
    else if (p < kPW2) s.l1[p - kPB1].w = w;
    else if (p < kPW3) s.b2[p - kPB2] = w;
    else if (p < kPB3) s.w3[p - kPW3] = w;
    else s.b3 = w;
}

__global__ void __launch_bounds__(kThreadsTrain, 1) mlp_train_cluster_kernel(ClusterTrainArgs a) {
    namespace cg = cooperative_groups;
    cg::cluster_group cluster = cg::this_cluster();
    extern __shared__ unsigned char smem_raw[];
    TrainSmem& s = *reinterpret_cast<TrainSmem*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    train_setup(s);
    const int t = threadIdx.x;
    const int rank = int(cluster.block_rank());
    const int clusters = int(gridDim.x) / kClusterCtas, me = int(blockIdx.x) / kClusterCtas;
    for (int slot = t; slot < kStride; slot += kThreadsTrain) {
        const int p = param_of_slot(slot);
        if (p >= 0) set_slot(s, slot, a.params[p]);
    }
    // The four slots this thread owns: value and Adam moments in registers.
    const int s0 = rank * kSliceSlots + 4 * t;
    const bool owner = 4 * t < kSliceSlots && s0 < kStride;
    float master[4], mom1[4], mom2[4];
#pragma unroll
    for (int c = 0; c < 4; ++c) {
        const int p = owner ? param_of_slot(s0 + c) : -1;
        master[c] = p >= 0 ? a.params[p] : 0.f;
        mom1[c] = p >= 0 ? a.m[p] : 0.f;
        mom2[c] = p >= 0 ? a.v[p] : 0.f;
    }
    tc::fence_async_smem();
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const int per_epoch = (a.itm + a.batch - 1) / a.batch;
    uint32_t phase = 0;
    bool ok = true;
    for (int step = 0; step < a.steps; ++step) {
        const int first = (step % per_epoch) * a.batch;
        const int count = min(a.batch, a.itm - first);
        if (ok)
            ok = grad_step<true>(s, nullptr, nullptr, a.samples, first, count, 1.0f / float(count), nullptr, 0, phase);
        tc::fence_before_sync();
        cluster.sync();
        tc::fence_after_sync();
        float* ex = a.exchange + size_t(step & 1) * clusters * kStride;
        if (owner) {
            const uint32_t local = tc::smem_u32(&s.acc[s0]);
            float4 sum = dsmem_load4(cluster_address(local, 0));
#pragma unroll
            for (int q = 1; q < kClusterCtas; ++q) {
                const float4 v = dsmem_load4(cluster_address(local, q));
                sum.x += v.x;
                sum.y += v.y;
                sum.z += v.z;
                sum.w += v.w;
            }
            *reinterpret_cast<float4*>(ex + size_t(me) * kStride + s0) = sum;
        }
        __syncthreads();
        // Publish this slice, then wait for the other clusters' (lane c of warp 0 polls
        // cluster c's flag, all at once).
        if (t == 0) {
            __threadfence();
            flag_release(a.flags + me * kClusterCtas + rank, step);
        }
        bool arrived = true;
        if (t < 32 && ok) {
            __syncwarp();
            if (t < clusters && t != me) {
                const long long start = clock64();
                while (flag_acquire(a.flags + t * kClusterCtas + rank) < step) {
                    if (clock64() - start > 2000000000LL) {
                        arrived = false;
                        break;
                    }
                }
            }
        }
        ok = !__syncthreads_or(!arrived) && ok;
        const float tstep = float(a.first_step + step + 1);
        const float bias1 = 1.0f - powf(a.beta1, tstep), bias2 = 1.0f - powf(a.beta2, tstep);
        if (owner) {
            // The 8 clusters' sums, loaded together, added in cluster order.
            float4 part[8];
#pragma unroll
            for (int c = 0; c < 8; ++c)
                part[c] = c < clusters ? __ldcg(reinterpret_cast<const float4*>(ex + size_t(c) * kStride + s0))
                                       : make_float4(0.f, 0.f, 0.f, 0.f);
            float4 g = part[0];
#pragma unroll
            for (int c = 1; c < 8; ++c) {
                if (c >= clusters) break;
                g.x += part[c].x;
                g.y += part[c].y;
                g.z += part[c].z;
                g.w += part[c].w;
            }
            const float gs[4] = {g.x, g.y, g.z, g.w};
            float w[4];
#pragma unroll
            for (int c = 0; c < 4; ++c) {
                mom1[c] = a.beta1 * mom1[c] + (1.f - a.beta1) * gs[c];
                mom2[c] = a.beta2 * mom2[c] + (1.f - a.beta2) * gs[c] * gs[c];
                w[c] = master[c] - a.lr * (mom1[c] / bias1) / (sqrtf(mom2[c] / bias2) + a.eps);
                master[c] = w[c];
            }
            *reinterpret_cast<float4*>(&s.pub[s0]) = make_float4(w[0], w[1], w[2], w[3]);
        }
        cluster.sync();
        // Pull the updated network from the cluster's owners (all loads in flight first).
        constexpr int kPulls = (kStride / 4 + kThreadsTrain - 1) / kThreadsTrain;
        float4 pulled[kPulls];
#pragma unroll
        for (int u = 0; u < kPulls; ++u) {
            const int slot = 4 * (t + kThreadsTrain * u);
            pulled[u] = slot < kStride
                            ? dsmem_load4(cluster_address(tc::smem_u32(&s.pub[slot]), slot / kSliceSlots))
                            : make_float4(0.f, 0.f, 0.f, 0.f);
        }
#pragma unroll
        for (int u = 0; u < kPulls; ++u) {
            const int slot = 4 * (t + kThreadsTrain * u);
            if (slot < kStride) {
                set_slot(s, slot, pulled[u].x);
                set_slot(s, slot + 1, pulled[u].y);
                set_slot(s, slot + 2, pulled[u].z);
                set_slot(s, slot + 3, pulled[u].w);
            }
        }
        tc::fence_async_smem();
        __syncthreads();
    }
    if (me == 0 && owner) {
#pragma unroll
        for (int c = 0; c < 4; ++c) {
            const int p = param_of_slot(s0 + c);
            if (p >= 0) {
                a.params[p] = master[c];
                a.m[p] = mom1[c];
                a.v[p] = mom2[c];
            }
        }
    }
    if (t == 0 && !ok) atomicExch(a.error, 1);
    // The last pulls read the owners' shared memory: no CTA leaves before they are done.
    cluster.sync();
    train_release(s);
}

// Target normalisation of one date: the network fits (y - mean) / scale.
struct TargetNorm {
    double mean, scale;
};

// Copies the trained parameters into the per-date store: W2 rounded to BF16 as the
// training kernel multiplies it, the output layer scaled back to cash units
// (w3 * scale, b3 * scale + mean), so the stored network predicts y itself.
__global__ void mlp_snapshot_kernel(const float* __restrict__ params, const TargetNorm* __restrict__ norm,
                                    float* __restrict__ net) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= kParams) return;
    const float scale = float(norm->scale), mean = float(norm->mean);
    float w = params[i];
    if (i >= kPW2 && i < kPB2) w = bf16_round(w);
    else if (i >= kPW3 && i < kPB3) w *= scale;
    else if (i == kPB3) w = fmaf(w, scale, mean);
    net[i] = w;
}


// Network inputs of a path at exercise date k.
struct Features {
    float spot_scale;  // 1 / (sigma_ref sqrt(T)) applied to log(S/K)
    float v_center, v_scale;
    float time_scale;  // dt / T
};

template <bool TWO>
__device__ __forceinline__ float4 features(const LsmcParams<float>& p, const Features& f, int k, float a, float b) {
    const float spot = spot_at_date<float, TWO>(p, k, a);
    const float x0 = logf(spot / p.strike) * f.spot_scale;
    const float x1 = TWO ? (b - f.v_center) * f.v_scale : 0.f;
    return make_float4(x0, x1, float(k + 1) * f.time_scale, spot);
}

// Polynomial part of the continuation at date k (zero when the date has no fit).
template <bool TWO>
__device__ __forceinline__ float poly_part(const LsmcParams<float>& p, const double* coefs, const int* have, int k,
                                           float spot, float v) {
    if (!have[k]) return 0.f;
    float cn[TWO ? 10 : 3];
#pragma unroll
    for (int j = 0; j < (TWO ? 10 : 3); ++j) cn[j] = float(coefs[size_t(k) * kMaxTerms + j]);
    return continuation<float, TWO>(p, cn, spot / p.strike, TWO ? v * p.y_scale : 0.f);
}

// The fitted network on compacted samples, on the tensor cores: 128 samples per CTA,
// layer 1 on the CUDA cores, the 64 x 64 product as four tcgen05 MMAs (BF16 operands,
// FP32 accumulator in 64 TMEM columns), the output layer in FP32 -- the training
// kernel's forward arithmetic on a stored network (W2 already BF16-rounded, output
// layer in cash units).  out[j] = f(samples[j].xyz).
struct __align__(1024) InferSmem {
    __nv_bfloat16 h1[kRows * kHidden];
    __nv_bfloat16 w2f[kHidden * kHidden];
    float w1[3 * kHidden], b1[kHidden], b2[kHidden], w3[kHidden];
    uint64_t bar;
    uint32_t tmem;
};
constexpr size_t kInferSmemBytes = sizeof(InferSmem) + 1024;

__global__ void __launch_bounds__(kRows) mlp_infer_kernel(const float* __restrict__ net,
                                                          const float4* __restrict__ samples, int count,
                                                          float* __restrict__ out, int* __restrict__ error) {
    extern __shared__ unsigned char smem_raw[];
    InferSmem& s = *reinterpret_cast<InferSmem*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    const int t = threadIdx.x, warp = t >> 5;
    if (warp == 0) {
        tc::tmem_alloc(&s.tmem, 64);
        tc::tmem_relinquish();
    }
    if (t == 0) tc::mbar_init(&s.bar, 1);
    for (int i = t; i < 3 * kHidden; i += kRows) s.w1[i] = net[kPW1 + i];
    if (t < kHidden) {
        s.b1[t] = net[kPB1 + t];
        s.b2[t] = net[kPB2 + t];
        s.w3[t] = net[kPW3 + t];
    }
    for (int i = t; i < kHidden * kHidden; i += kRows)
        s.w2f[tc::kmajor(i >> 6, i & 63, kHidden)] = __float2bfloat16_rn(net[kPW2 + i]);
    const int row = blockIdx.x * kRows + t;
    const bool valid = row < count;
    const float4 x = valid ? samples[row] : make_float4(0.f, 0.f, 0.f, 0.f);
    __syncthreads();
#pragma unroll
    for (int g = 0; g < 8; ++g) {
        __align__(16) __nv_bfloat16 pack[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) {
            const int j = 8 * g + u;
            const float z = fmaf(s.w1[3 * j], x.x, fmaf(s.w1[3 * j + 1], x.y, fmaf(s.w1[3 * j + 2], x.z, s.b1[j])));
            pack[u] = __float2bfloat16_rn(z > 0.f ? z : 0.f);
        }
        *reinterpret_cast<uint4*>(&s.h1[tc::kmajor(t, 8 * g, kHidden)]) = *reinterpret_cast<const uint4*>(pack);
    }
    tc::fence_async_smem();
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tmem = s.tmem;
    if (t == 0) {
        const uint32_t a0 = tc::smem_u32(s.h1), b0 = tc::smem_u32(s.w2f);
        for (int k = 0; k < kHidden / 16; ++k)
            tc::mma_bf16(tmem, tc::smem_desc(a0 + 256 * k, 128, kHidden * 16), tc::smem_desc(b0 + 256 * k, 128, kHidden * 16),
                         tc::idesc_bf16(kRows, kHidden), k > 0);
        tc::mma_commit(&s.bar);
    }
    const bool ok = tc::mbar_wait(&s.bar, 0);
    if (!__syncthreads_or(!ok)) {
        tc::fence_after_sync();
        float z2[32];
        float y = net[kPB3];
        const uint32_t lane_base = uint32_t(warp * 32) << 16;
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            tc::tmem_load32(tmem + lane_base + 32 * h, z2);
#pragma unroll
            for (int u = 0; u < 32; ++u) {
                const float z = z2[u] + s.b2[32 * h + u];
                y = fmaf(z > 0.f ? z : 0.f, s.w3[32 * h + u], y);
            }
        }
        if (valid) out[row] = y;
    } else if (t == 0) {
        atomicExch(error, 1);
    }
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(tmem, 64);
}

// Exercise decisions of date k on its compacted in-the-money paths: exercise when the
// intrinsic value beats the polynomial plus the network's output (computed by
// mlp_infer_kernel into `net_out`).  Writes the cash of exercising paths.
template <bool TWO>
__global__ void __launch_bounds__(256) mlp_exercise_kernel(LsmcParams<float> p, int date, int count,
                                                           const int* __restrict__ sample_path,
                                                           const float* __restrict__ net_out,
                                                           const double* __restrict__ coefs,
                                                           const int* __restrict__ have, const float* __restrict__ a,
                                                           const float* __restrict__ b, float* __restrict__ cash) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= count) return;
    const int i = sample_path[j];
    const size_t at = size_t(date) * p.paths + i;
    const float spot = spot_at_date<float, TWO>(p, date, a[at]);
    const float v = TWO ? b[at] : 0.f;
    const float e = intrinsic(p, spot);
    if (e > 0.f && e / p.strike > poly_part<TWO>(p, coefs, have, date, spot, v) + net_out[j]) cash[i] = e;
}

__global__ void mlp_discount_kernel(float* __restrict__ cash, int n, float discount) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) cash[i] *= discount;
}

// Normal equations of the in-the-money paths at date k (the accumulation of
// lsmc_backward, with the cash already decided and discounted to date k).
template <bool TWO>
__global__ void __launch_bounds__(kLsmcThreads) mlp_poly_sums_kernel(LsmcParams<float> p, int date,
                                                                     const float* __restrict__ a,
                                                                     const float* __restrict__ b,
                                                                     const float* __restrict__ cash,
                                                                     double* __restrict__ partials) {
    constexpr int T = TWO ? 10 : 3;
    constexpr int S = sum_count(T);
    float acc[S];
#pragma unroll
    for (int j = 0; j < S; ++j) acc[j] = 0.f;
    const float inv_k = 1.f / p.strike;
    // One CTA per SM fits the accumulators: loads of kPrefetch paths are issued before
    // the sums, in grid-stride order (the accumulation order is unchanged).
    constexpr int kPrefetch = 4;
    const int stride = gridDim.x * blockDim.x;
    for (int base = blockIdx.x * blockDim.x + threadIdx.x; base < p.paths; base += kPrefetch * stride) {
        float av[kPrefetch], bv[kPrefetch], cv[kPrefetch];
#pragma unroll
        for (int u = 0; u < kPrefetch; ++u) {
            const int i = base + u * stride;
            if (i < p.paths) {
                const size_t at = size_t(date) * p.paths + i;
                av[u] = a[at];
                bv[u] = TWO ? b[at] : 0.f;
                cv[u] = cash[i];
            }
        }
#pragma unroll
        for (int u = 0; u < kPrefetch; ++u) {
            if (base + u * stride >= p.paths) break;
            const float s = spot_at_date<float, TWO>(p, date, av[u]);
            if (intrinsic(p, s) > 0.f) {
                float f[T];
                lsmc_basis<float, TWO>(s * inv_k, TWO ? bv[u] * p.y_scale : 0.f, f);
                const float target = cv[u] * inv_k;
                int q = 0;
#pragma unroll
                for (int r = 0; r < T; ++r)
#pragma unroll
                    for (int col = r; col < T; ++col) acc[q++] += f[r] * f[col];
#pragma unroll
                for (int r = 0; r < T; ++r) acc[q++] += f[r] * target;
            }
        }
    }
    block_sums<float, S>(acc, partials);
}

// In-the-money samples of date k in path order: per-block counts and target sums, a
// block-ordered scan (offsets, the date's target mean and scale), then the scatter.
struct BlockStats {
    double count, sum, sumsq;
};

template <bool TWO>
__global__ void __launch_bounds__(256) mlp_count_kernel(LsmcParams<float> p, int date, const float* __restrict__ a,
                                                        const float* __restrict__ b, const float* __restrict__ cash,
                                                        const double* __restrict__ coefs, const int* __restrict__ have,
                                                        BlockStats* __restrict__ stats) {
    __shared__ double ws[8][3];
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    double c = 0.0, y = 0.0;
    if (i < p.paths) {
        const size_t at = size_t(date) * p.paths + i;
        const float spot = spot_at_date<float, TWO>(p, date, a[at]);
        if (intrinsic(p, spot) > 0.f) {
            c = 1.0;
            y = double(cash[i] / p.strike - poly_part<TWO>(p, coefs, have, date, spot, TWO ? b[at] : 0.f));
        }
    }
    double y2 = y * y;
    for (int o = 16; o >= 1; o >>= 1) {
        c += __shfl_xor_sync(0xffffffffu, c, o);
        y += __shfl_xor_sync(0xffffffffu, y, o);
        y2 += __shfl_xor_sync(0xffffffffu, y2, o);
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) {
        ws[warp][0] = c;
        ws[warp][1] = y;
        ws[warp][2] = y2;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        BlockStats b{0.0, 0.0, 0.0};
        for (int w = 0; w < 8; ++w) {
            b.count += ws[w][0];
            b.sum += ws[w][1];
            b.sumsq += ws[w][2];
        }
        stats[blockIdx.x] = b;
    }
}

// Exclusive offsets in block order, the in-the-money total and the target normalisation,
// by one CTA of kScanThreads: each thread owns a contiguous run of blocks; counts are
// scanned exactly, the sums reduced in a fixed tree (deterministic).
constexpr int kScanThreads = 1024;

__global__ void __launch_bounds__(kScanThreads) mlp_scan_kernel(const BlockStats* __restrict__ stats, int blocks,
                                                                int* __restrict__ offsets, int* __restrict__ total,
                                                                TargetNorm* __restrict__ norm) {
    __shared__ int run_count[kScanThreads];
    __shared__ double run_sum[kScanThreads], run_sq[kScanThreads];
    const int t = threadIdx.x;
    const int per = (blocks + kScanThreads - 1) / kScanThreads;
    const int lo = min(blocks, t * per), hi = min(blocks, lo + per);
    int c = 0;
    double sum = 0.0, sq = 0.0;
    for (int b = lo; b < hi; ++b) {
        c += int(stats[b].count);
        sum += stats[b].sum;
        sq += stats[b].sumsq;
    }
    run_count[t] = c;
    run_sum[t] = sum;
    run_sq[t] = sq;
    __syncthreads();
    // Inclusive scan of the counts (Hillis-Steele on integers).
    for (int d = 1; d < kScanThreads; d <<= 1) {
        const int add = t >= d ? run_count[t - d] : 0;
        __syncthreads();
        run_count[t] += add;
        __syncthreads();
    }
    int base = t > 0 ? run_count[t - 1] : 0;
    for (int b = lo; b < hi; ++b) {
        offsets[b] = base;
        base += int(stats[b].count);
    }
    // Tree reduction of the target sums.
    for (int d = kScanThreads / 2; d > 0; d >>= 1) {
        if (t < d) {
            run_sum[t] += run_sum[t + d];
            run_sq[t] += run_sq[t + d];
        }
        __syncthreads();
    }
    if (t == 0) {
        const int n = run_count[kScanThreads - 1];
        *total = n;
        TargetNorm tn{0.0, 1.0};
        if (n > 0) {
            tn.mean = run_sum[0] / n;
            const double var = run_sq[0] / n - tn.mean * tn.mean;
            tn.scale = var > 1e-12 ? sqrt(var) : 1.0;
        }
        *norm = tn;
    }
}

template <bool TWO>
__global__ void __launch_bounds__(256) mlp_scatter_kernel(LsmcParams<float> p, Features f, int date,
                                                          const float* __restrict__ a, const float* __restrict__ b,
                                                          const float* __restrict__ cash, const double* __restrict__ coefs,
                                                          const int* __restrict__ have, const int* __restrict__ offsets,
                                                          const TargetNorm* __restrict__ norm,
                                                          float4* __restrict__ samples, int* __restrict__ sample_path) {
    __shared__ int warp_base[8];
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    float4 x = make_float4(0.f, 0.f, 0.f, 0.f);
    bool itm = false;
    float v = 0.f;
    if (i < p.paths) {
        const size_t at = size_t(date) * p.paths + i;
        v = TWO ? b[at] : 0.f;
        x = features<TWO>(p, f, date, a[at], v);
        itm = intrinsic(p, x.w) > 0.f;
    }
    const unsigned ballot = __ballot_sync(0xffffffffu, itm);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) warp_base[warp] = __popc(ballot);
    __syncthreads();
    if (threadIdx.x == 0) {
        int run = 0;
        for (int w = 0; w < 8; ++w) {
            const int c = warp_base[w];
            warp_base[w] = run;
            run += c;
        }
    }
    __syncthreads();
    if (itm) {
        const int pos = offsets[blockIdx.x] + warp_base[warp] + __popc(ballot & ((1u << lane) - 1u));
        const float y = cash[i] / p.strike - poly_part<TWO>(p, coefs, have, date, x.w, v);
        samples[pos] = make_float4(x.x, x.y, x.z, float((double(y) - norm->mean) / norm->scale));
        sample_path[pos] = i;
    }
}

// The cash moments at date 0, after its decision (FP64 partials per block).
__global__ void __launch_bounds__(256) mlp_final_kernel(const float* __restrict__ cash, int paths,
                                                        double* __restrict__ partials) {
    __shared__ double w0[8], w1[8];
    double s0 = 0.0, s1 = 0.0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < paths; i += gridDim.x * blockDim.x) {
        const double c = double(cash[i]);
        s0 += c;
        s1 += c * c;
    }
    for (int o = 16; o >= 1; o >>= 1) {
        s0 += __shfl_xor_sync(0xffffffffu, s0, o);
        s1 += __shfl_xor_sync(0xffffffffu, s1, o);
    }
    if ((threadIdx.x & 31) == 0) {
        w0[threadIdx.x >> 5] = s0;
        w1[threadIdx.x >> 5] = s1;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double t0 = 0.0, t1 = 0.0;
        for (int w = 0; w < 8; ++w) {
            t0 += w0[w];
            t1 += w1[w];
        }
        partials[2 * blockIdx.x] = t0;
        partials[2 * blockIdx.x + 1] = t1;
    }
}

// The fitted policy on fresh paths (american.rs:574-637), date by date so that the
// network runs on the tensor cores: every path carries its state (log spot, variance,
// value -- negative while alive -- and its PCG32 stream position) from one exercise
// date to the next; at each date the alive in-the-money paths are compacted, the
// network evaluates them (mlp_infer_kernel) and those whose intrinsic value beats the
// continuation stop.
struct FreshPaths {
    float* x;
    float* v;
    float* value;
    Pcg* pcg;
    float* spare;
    int* has_spare;
};

template <bool TWO>
__global__ void __launch_bounds__(256) mlp_fresh_advance_kernel(LsmcParams<float> p, uint64_t seed, int date,
                                                                float df, FreshPaths st, BlockStats* __restrict__ stats) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    bool itm = false;
    if (i < p.paths) {
        float value = date == 0 ? -1.f : st.value[i];
        if (value < 0.f) {
            PcgSource<float> n;
            float x, v;
            if (date == 0) {
                n.start(seed, uint64_t(i), TWO ? p.dates * p.substeps * 2 : p.dates);
                x = 0.f;
                v = p.v0;
            } else {
                n.g = st.pcg[i];
                n.spare = st.spare[i];
                n.has_spare = st.has_spare[i] != 0;
                x = st.x[i];
                v = st.v[i];
            }
            if (!TWO) {
                x += n.normal();
            } else {
                for (int j = 0; j < p.substeps; ++j) {
                    const float z1 = n.normal(), z2 = n.normal();
                    const float vp = v > 0.f ? v : 0.f;
                    const float sv = xsqrt(vp) * p.sqrt_h;
                    x += (p.rate - p.dividend - 0.5f * vp) * p.h + sv * z1;
                    v += p.kappa * (p.theta - vp) * p.h + p.xi * sv * (p.rho * z1 + p.rho_bar * z2);
                }
            }
            const float e = intrinsic(p, spot_at_date<float, TWO>(p, date, x));
            if (date == p.dates - 1) {
                value = e > 0.f ? e * df : 0.f;  // the last date exercises whenever in the money
            } else {
                itm = e > 0.f;
                st.pcg[i] = n.g;
                st.spare[i] = n.spare;
                st.has_spare[i] = n.has_spare;
            }
            st.x[i] = x;
            st.v[i] = v;
            st.value[i] = value;
        }
    }
    const int c = __syncthreads_count(itm);
    if (threadIdx.x == 0) stats[blockIdx.x] = BlockStats{double(c), 0.0, 0.0};
}

template <bool TWO>
__global__ void __launch_bounds__(256) mlp_fresh_scatter_kernel(LsmcParams<float> p, Features f, int date,
                                                                FreshPaths st, const int* __restrict__ offsets,
                                                                float4* __restrict__ samples,
                                                                int* __restrict__ sample_path) {
    __shared__ int warp_base[8];
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    float4 x = make_float4(0.f, 0.f, 0.f, 0.f);
    bool itm = false;
    if (i < p.paths && st.value[i] < 0.f && date < p.dates - 1) {
        x = features<TWO>(p, f, date, st.x[i], TWO ? st.v[i] : 0.f);
        itm = intrinsic(p, x.w) > 0.f;
    }
    const unsigned ballot = __ballot_sync(0xffffffffu, itm);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) warp_base[warp] = __popc(ballot);
    __syncthreads();
    if (threadIdx.x == 0) {
        int run = 0;
        for (int w = 0; w < 8; ++w) {
            const int c = warp_base[w];
            warp_base[w] = run;
            run += c;
        }
    }
    __syncthreads();
    if (itm) {
        const int pos = offsets[blockIdx.x] + warp_base[warp] + __popc(ballot & ((1u << lane) - 1u));
        samples[pos] = make_float4(x.x, x.y, x.z, 0.f);
        sample_path[pos] = i;
    }
}

template <bool TWO>
__global__ void __launch_bounds__(256) mlp_fresh_exercise_kernel(LsmcParams<float> p, int date, float df, int count,
                                                                 const int* __restrict__ sample_path,
                                                                 const float* __restrict__ net_out,
                                                                 const double* __restrict__ coefs,
                                                                 const int* __restrict__ have, FreshPaths st) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= count) return;
    const int i = sample_path[j];
    const float spot = spot_at_date<float, TWO>(p, date, st.x[i]);
    const float v = TWO ? st.v[i] : 0.f;
    const float e = intrinsic(p, spot);
    if (e > 0.f && e / p.strike > poly_part<TWO>(p, coefs, have, date, spot, v) + net_out[j]) st.value[i] = e * df;
}

// Deterministic initial weights: uniform(-sqrt(6 / fan_in), sqrt(6 / fan_in)) from a
// splitmix64 stream of `seed` for the hidden layers, zero biases and a zero output layer,
// so the untrained network adds nothing to the polynomial.
void initial_params(uint64_t seed, std::vector<float>& w) {
    w.assign(kParams, 0.0f);
    uint64_t state = seed;
    auto next = [&]() {
        uint64_t z = (state += 0x9E3779B97F4A7C15ULL);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
        z ^= z >> 31;
        return double(z >> 11) * (1.0 / 9007199254740992.0);
    };
    auto fill = [&](int at, int n, double fan_in) {
        const double r = std::sqrt(6.0 / fan_in);
        for (int i = 0; i < n; ++i) w[at + i] = float((2.0 * next() - 1.0) * r);
    };
    fill(kPW1, 3 * kHidden, 3.0);
    fill(kPW2, kHidden * kHidden, double(kHidden));
}

bool configure_train_kernel() {
    static bool done = false;
    if (done) return true;
    done = cudaFuncSetAttribute(mlp_grad_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, int(kTrainSmemBytes)) ==
               cudaSuccess &&
           cudaFuncSetAttribute(mlp_train_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, int(kTrainSmemBytes)) ==
               cudaSuccess &&
           cudaFuncSetAttribute(mlp_infer_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, int(kInferSmemBytes)) ==
               cudaSuccess;
    return done;
}

// Whether `ctas` training CTAs can all be resident at once (cooperative launch).
bool cooperative_fits(int device, int ctas) {
    int coop = 0, sms = 0, per_sm = 0;
    if (cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, device) != cudaSuccess || !coop) return false;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess) return false;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, mlp_train_kernel, kThreadsTrain, kTrainSmemBytes) != cudaSuccess)
        return false;
    return ctas <= per_sm * sms;
}

struct Adam {
    float lr, beta1 = 0.9f, beta2 = 0.999f, eps = 1e-8f;
    int step = 0;
};

// The clustered trainer: whether `ctas` CTAs (a multiple of kClusterCtas) fit at once;
// it stays off once a launch of it has been refused.
bool cluster_trainer_off = false;

bool cluster_trainer_fits(int ctas) {
    static int max_clusters = -1;
    if (max_clusters < 0) {
        max_clusters = 0;
        if (cudaFuncSetAttribute(mlp_train_cluster_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 int(kTrainSmemBytes)) == cudaSuccess) {
            cudaLaunchConfig_t cfg = {};
            cudaLaunchAttribute attr[1];
            attr[0].id = cudaLaunchAttributeClusterDimension;
            attr[0].val.clusterDim.x = kClusterCtas;
            attr[0].val.clusterDim.y = 1;
            attr[0].val.clusterDim.z = 1;
            cfg.gridDim = dim3(kClusterCtas);
            cfg.blockDim = dim3(kThreadsTrain);
            cfg.dynamicSmemBytes = kTrainSmemBytes;
            cfg.attrs = attr;
            cfg.numAttrs = 1;
            int n = 0;
            if (cudaOccupancyMaxActiveClusters(&n, mlp_train_cluster_kernel, &cfg) == cudaSuccess) max_clusters = n;
        }
        cudaGetLastError();
    }
    return !cluster_trainer_off && ctas % kClusterCtas == 0 && ctas <= 64 && ctas / kClusterCtas <= max_clusters;
}

// CTAs of the clustered trainer for a batch: one per 128 samples, rounded up to whole
// clusters.
int cluster_trainer_ctas(int batch) {
    return ((batch + kRows - 1) / kRows + kClusterCtas - 1) / kClusterCtas * kClusterCtas;
}

// Launches it (a cooperative launch of 8-CTA clusters: every CTA resident).  Resets the
// exchange flags first.  A refused launch turns it off and returns the error cleared.
cudaError_t launch_cluster_trainer(cudaStream_t st, int ctas, const ClusterTrainArgs& ca, bool& launched) {
    launched = false;
    if (cudaMemsetAsync(ca.flags, 0xFF, size_t(ctas) * sizeof(int), st) != cudaSuccess) return cudaGetLastError();
    cudaLaunchConfig_t cfg = {};
    cudaLaunchAttribute attr[2];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = kClusterCtas;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    attr[1].id = cudaLaunchAttributeCooperative;
    attr[1].val.cooperative = 1;
    cfg.gridDim = dim3(unsigned(ctas));
    cfg.blockDim = dim3(kThreadsTrain);
    cfg.dynamicSmemBytes = kTrainSmemBytes;
    cfg.stream = st;
    cfg.attrs = attr;
    cfg.numAttrs = 2;
    if (cudaLaunchKernelEx(&cfg, mlp_train_cluster_kernel, ca) != cudaSuccess) {
        cudaGetLastError();
        cluster_trainer_off = true;
        return cudaSuccess;
    }
    launched = true;
    return cudaSuccess;
}

// One optimiser step on samples [first, first + count).
cudaError_t train_step(cudaStream_t st, float* params, float* m, float* v, Adam& adam, const float4* samples, int first,
                       int count, float* partials, int* error) {
    const int blocks = (count + kRows - 1) / kRows;
    mlp_grad_kernel<<<blocks, kThreadsTrain, kTrainSmemBytes, st>>>(params, samples, first, count, 1.0f / float(count),
                                                            partials, error);
    adam.step += 1;
    const float bias1 = 1.0f - std::pow(adam.beta1, float(adam.step));
    const float bias2 = 1.0f - std::pow(adam.beta2, float(adam.step));
    mlp_adam_kernel<<<(kParams + 255) / 256, 256, 0, st>>>(partials, blocks, params, m, v, adam.lr, adam.beta1,
                                                           adam.beta2, adam.eps, bias1, bias2);
    return cudaGetLastError();
}

template <bool TWO>
kgpu_status mlp_run(kgpu_context* ctx, const kgpu_model* model, double strike, double sign, double expiry,
                    const kgpu_lsmc_settings* s, uint64_t fresh_seed, kgpu_lsmc_result* out) {
    const bool standalone = s->basis == KGPU_BASIS_MLP_STANDALONE;
    const LsmcParams<float> p = make_lsmc_params<float>(model, strike, sign, expiry, s);
    const size_t n = size_t(p.paths), d = size_t(p.dates);
    const int batch = s->mlp_batch > 0 ? s->mlp_batch : 8192;
    const int epochs = s->mlp_epochs > 0 ? s->mlp_epochs : 5;
    if (s->mlp_hidden != 0 && s->mlp_hidden != kHidden) {
        ctx->error = "the continuation network has 64 hidden units per layer";
        return KGPU_UNSUPPORTED_OPERATION;
    }
    Features f;
    const double sigma_ref = TWO ? std::sqrt(std::max(model->theta, 1e-8)) : model->volatility;
    f.spot_scale = float(1.0 / (std::max(sigma_ref, 1e-4) * std::sqrt(expiry)));
    f.v_center = TWO ? float(model->theta) : 0.f;
    f.v_scale = TWO ? float(1.0 / std::max(model->theta, 1e-8)) : 0.f;
    f.time_scale = float(1.0 / p.dates);
    const int pblocks = int((n + 255) / 256);
    const int max_train_blocks = (batch + kRows - 1) / kRows;
    const int fblocks = std::min(ctx->sm_count * 8, pblocks);
    const int sblocks = std::min<int>(ctx->sm_count * 4, int((n + kLsmcThreads - 1) / kLsmcThreads));
    // Buffers: path store, cash, samples, counts, parameters and Adam state, per-date
    // networks, gradient partials, estimate partials.
    // The path store; afterwards it holds the fresh paths' state (10 floats per path).
    const size_t store_bytes = std::max(n * d * (TWO ? 2 : 1), 10 * n) * sizeof(float);
    const size_t net_bytes = size_t(kParams) * sizeof(float);
    const size_t misc_floats = (size_t(3) + d) * kStride + size_t(max_train_blocks) * kStride + 2 * kHidden * kHidden +
                               size_t(2) * 8 * kStride + 64;
    if (ctx->lsmc_store.ensure(store_bytes) || ctx->lsmc_cash.ensure(n * sizeof(float)) ||
        ctx->mlp_scratch.ensure(n * (sizeof(float4) + sizeof(int) + sizeof(float)) +
                                size_t(pblocks) * (sizeof(BlockStats) + sizeof(int)) + d * sizeof(TargetNorm) + 256) ||
        ctx->mlp_params.ensure(misc_floats * sizeof(float)) ||
        ctx->lsmc_misc.ensure(size_t(fblocks) * 2 * sizeof(double) * 2 + 64) ||
        ctx->lsmc_sums.ensure((size_t(sblocks) + 1) * kMaxSums * sizeof(double)) ||
        ctx->lsmc_coef.ensure(d * kMaxTerms * sizeof(double) + d * sizeof(int) + 16))
        return KGPU_DEVICE_ERROR;
    if (!configure_train_kernel()) {
        ctx->error = "cannot configure the training kernel's shared memory";
        return KGPU_DEVICE_ERROR;
    }
    float* a = static_cast<float*>(ctx->lsmc_store.ptr);
    float* b = TWO ? a + n * d : nullptr;
    float* cash = static_cast<float*>(ctx->lsmc_cash.ptr);
    float4* samples = static_cast<float4*>(ctx->mlp_scratch.ptr);
    BlockStats* stats = reinterpret_cast<BlockStats*>(samples + n);
    TargetNorm* norms = reinterpret_cast<TargetNorm*>(stats + pblocks);
    int* counts = reinterpret_cast<int*>(norms + d);
    int* total = counts + pblocks;
    int* error = total + 1;
    GridBarrier* barrier = reinterpret_cast<GridBarrier*>(error + 1);
    int* sample_path = reinterpret_cast<int*>(barrier + 1);  // path of each compacted sample
    float* net_out = reinterpret_cast<float*>(sample_path + n);  // the network on the samples
    const bool cooperative = max_train_blocks <= 64 && cooperative_fits(ctx->device, max_train_blocks);
    // Regions of kStride floats keep every one 16-byte aligned (the gradient partials are
    // written as float4).
    float* params = static_cast<float*>(ctx->mlp_params.ptr);
    float* m = params + kStride;
    float* v = m + kStride;
    float* nets = v + kStride;
    float* partials = nets + d * kStride;
    __nv_bfloat16* w2_tiles = reinterpret_cast<__nv_bfloat16*>(partials + size_t(max_train_blocks) * kStride);
    float* exchange = reinterpret_cast<float*>(w2_tiles + 2 * kHidden * kHidden);  // clustered trainer
    int* flags = reinterpret_cast<int*>(exchange + size_t(2) * 8 * kStride);
    const int cluster_ctas = cluster_trainer_ctas(batch);
    double* finals = static_cast<double*>(ctx->lsmc_misc.ptr);
    double* lower_partials = finals + 2 * fblocks;
    double* coefs = static_cast<double*>(ctx->lsmc_coef.ptr);
    int* have = reinterpret_cast<int*>(coefs + d * kMaxTerms);
    int* poly_failed = have + d;
    double* poly_partials = static_cast<double*>(ctx->lsmc_sums.ptr);
    double* poly_reduced = poly_partials + size_t(sblocks) * kMaxSums;  // one partial per sum
    cudaStream_t st = ctx->stream;
    std::vector<float> init;
    initial_params(s->mlp_seed, init);
    Adam adam;
    adam.lr = float(s->mlp_learning_rate > 0.0 ? s->mlp_learning_rate : 1e-3);
    cudaEvent_t e0, e1, e2, e3;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaEventCreate(&e2);
    cudaEventCreate(&e3);
    auto cleanup = [&]() {
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        cudaEventDestroy(e2);
        cudaEventDestroy(e3);
    };
#define MLP_TRY(x)                                       \
    do {                                                 \
        cudaError_t rc_ = (x);                           \
        if (rc_ != cudaSuccess) {                        \
            ctx->error = cudaGetErrorString(rc_);        \
            cleanup();                                   \
            return KGPU_DEVICE_ERROR;                    \
        }                                                \
    } while (0)
    MLP_TRY(cudaMemcpyAsync(params, init.data(), net_bytes, cudaMemcpyHostToDevice, st));
    MLP_TRY(cudaMemsetAsync(m, 0, 2 * kStride * sizeof(float), st));
    MLP_TRY(cudaMemsetAsync(nets, 0, d * kStride * sizeof(float), st));
    MLP_TRY(cudaMemsetAsync(error, 0, sizeof(int) + sizeof(GridBarrier), st));
    MLP_TRY(cudaMemsetAsync(coefs, 0, d * kMaxTerms * sizeof(double) + d * sizeof(int) + sizeof(int), st));
    MLP_TRY(cudaEventRecord(e0, st));
    lsmc_forward<float, TWO><<<unsigned(pblocks), 256, 0, st>>>(p, s->seed, a, b, cash);
    MLP_TRY(cudaGetLastError());
    MLP_TRY(cudaEventRecord(e1, st));
    int launches = 1;
    int itm_next = 0;  // in-the-money samples of date + 1, still compacted in `samples`
    // Exercise decisions of date k with its fitted network on the tensor cores: the
    // compacted in-the-money samples of k go through mlp_infer_kernel, then
    // mlp_exercise_kernel compares with the intrinsic values.
    auto decide_at = [&](int k, int count) -> cudaError_t {
        if (count <= 0) return cudaSuccess;
        mlp_infer_kernel<<<(count + kRows - 1) / kRows, kRows, kInferSmemBytes, st>>>(nets + size_t(k) * kStride,
                                                                                      samples, count, net_out, error);
        mlp_exercise_kernel<TWO><<<(count + 255) / 256, 256, 0, st>>>(p, k, count, sample_path, net_out, coefs, have,
                                                                      a, b, cash);
        launches += 2;
        return cudaGetLastError();
    };
    for (int date = p.dates - 2; date >= 0; --date) {
        // Date + 1's decision (none at expiry, where the cash already is the intrinsic
        // value), then the cash discounted to this date (american.rs:1347-1362).
        if (date + 1 <= p.dates - 2) MLP_TRY(decide_at(date + 1, itm_next));
        mlp_discount_kernel<<<pblocks, 256, 0, st>>>(cash, p.paths, p.discount);
        ++launches;
        // The polynomial fit of this date (lsmc_solve: block-ordered merge, pivoted FP64
        // elimination with degree fallback), then the residual samples.  The standalone
        // network fits no polynomial: `have` stays 0, so the targets are the discounted
        // cash flows themselves and the network alone is the continuation value.
        if (!standalone) {
            mlp_poly_sums_kernel<TWO><<<sblocks, kLsmcThreads, 0, st>>>(p, date, a, b, cash, poly_partials);
            reduce_partials_kernel<<<sum_count(TWO ? 10 : 3), 32, 0, st>>>(poly_partials, sblocks, poly_reduced);
            lsmc_solve<TWO><<<1, kSolveThreads, 0, st>>>(poly_reduced, 1, p.max_degree,
                                                         coefs + size_t(date) * kMaxTerms, have + date, poly_failed);
            launches += 3;
        }
        mlp_count_kernel<TWO><<<pblocks, 256, 0, st>>>(p, date, a, b, cash, coefs, have, stats);
        mlp_scan_kernel<<<1, kScanThreads, 0, st>>>(stats, pblocks, counts, total, norms + date);
        mlp_scatter_kernel<TWO><<<pblocks, 256, 0, st>>>(p, f, date, a, b, cash, coefs, have, counts, norms + date,
                                                        samples, sample_path);
        launches += 3;
        MLP_TRY(cudaGetLastError());
        int itm = 0;
        MLP_TRY(cudaMemcpyAsync(&itm, total, sizeof(int), cudaMemcpyDeviceToHost, st));
        MLP_TRY(cudaStreamSynchronize(st));
        itm_next = itm;
        // Training samples: the first `mlp_samples` in-the-money paths (an i.i.d.
        // subsample, the paths being independent), or all of them.
        if (s->mlp_samples > 0 && itm > s->mlp_samples) itm = s->mlp_samples;
        if (itm > 0) {
            // The first fitted date starts from the initial weights: it trains four times
            // as long; later dates start from the previous date's network.
            const int date_epochs = adam.step == 0 ? 4 * epochs : epochs;
            const int steps = date_epochs * ((itm + batch - 1) / batch);
            bool clustered = false;
            if (cluster_trainer_fits(cluster_ctas)) {
                ClusterTrainArgs ca{params, m, v, samples, exchange, flags, error, itm, batch, steps,
                                    adam.step, adam.lr, adam.beta1, adam.beta2, adam.eps};
                MLP_TRY(launch_cluster_trainer(st, cluster_ctas, ca, clustered));
            }
            if (clustered) {
                adam.step += steps;
                launches += 1;
            } else if (cooperative) {
                TrainArgs ta{params, w2_tiles, m, v, samples, partials, barrier, error, itm, batch, steps,
                             adam.step, adam.lr, adam.beta1, adam.beta2, adam.eps};
                void* args[] = {&ta};
                MLP_TRY(cudaLaunchCooperativeKernel(reinterpret_cast<const void*>(mlp_train_kernel),
                                                    dim3(max_train_blocks), dim3(kThreadsTrain), args, kTrainSmemBytes, st));
                adam.step += steps;
                launches += 1;
            } else {
                for (int epoch = 0; epoch < date_epochs; ++epoch)
                    for (int first = 0; first < itm; first += batch) {
                        MLP_TRY(train_step(st, params, m, v, adam, samples, first, std::min(batch, itm - first),
                                           partials, error));
                        launches += 2;
                    }
            }
        }
        // The network of this date (kept when no path is in the money: the previous
        // date's weights continue).
        mlp_snapshot_kernel<<<(kParams + 255) / 256, 256, 0, st>>>(params, norms + date, nets + size_t(date) * kStride);
        ++launches;
    }
    // Date 0's decision on its compacted samples, then the cash moments.
    MLP_TRY(decide_at(0, itm_next));
    mlp_final_kernel<<<fblocks, 256, 0, st>>>(cash, p.paths, finals);
    ++launches;
    MLP_TRY(cudaGetLastError());
    MLP_TRY(cudaEventRecord(e2, st));
    const bool lower = fresh_seed != s->seed;
    if (lower) {
        // Fresh paths, date by date; the path store's buffer is free again and holds
        // their state.
        FreshPaths fp;
        fp.x = a;
        fp.v = a + n;
        fp.value = a + 2 * n;
        fp.pcg = reinterpret_cast<Pcg*>(a + 4 * n);  // 16-byte aligned: 4 n floats in
        fp.spare = a + 8 * n;
        fp.has_spare = reinterpret_cast<int*>(a + 9 * n);
        float df = 1.f;
        for (int k = 0; k < p.dates; ++k) {
            df *= p.discount;
            mlp_fresh_advance_kernel<TWO><<<pblocks, 256, 0, st>>>(p, fresh_seed, k, df, fp, stats);
            launches += 1;
            if (k == p.dates - 1) break;
            mlp_scan_kernel<<<1, kScanThreads, 0, st>>>(stats, pblocks, counts, total, norms + k);
            mlp_fresh_scatter_kernel<TWO><<<pblocks, 256, 0, st>>>(p, f, k, fp, counts, samples, sample_path);
            launches += 2;
            MLP_TRY(cudaGetLastError());
            int alive = 0;
            MLP_TRY(cudaMemcpyAsync(&alive, total, sizeof(int), cudaMemcpyDeviceToHost, st));
            MLP_TRY(cudaStreamSynchronize(st));
            if (alive > 0) {
                mlp_infer_kernel<<<(alive + kRows - 1) / kRows, kRows, kInferSmemBytes, st>>>(
                    nets + size_t(k) * kStride, samples, alive, net_out, error);
                mlp_fresh_exercise_kernel<TWO><<<(alive + 255) / 256, 256, 0, st>>>(p, k, df, alive, sample_path,
                                                                                    net_out, coefs, have, fp);
                launches += 2;
            }
        }
        mlp_final_kernel<<<fblocks, 256, 0, st>>>(fp.value, p.paths, lower_partials);
        ++launches;
        MLP_TRY(cudaGetLastError());
    }
    MLP_TRY(cudaEventRecord(e3, st));
    std::vector<double> fin(size_t(fblocks) * 4);
    int failed = 0, fit_failed = 0;
    MLP_TRY(cudaMemcpyAsync(fin.data(), finals, fin.size() * sizeof(double), cudaMemcpyDeviceToHost, st));
    MLP_TRY(cudaMemcpyAsync(&failed, error, sizeof(int), cudaMemcpyDeviceToHost, st));
    MLP_TRY(cudaMemcpyAsync(&fit_failed, poly_failed, sizeof(int), cudaMemcpyDeviceToHost, st));
    MLP_TRY(cudaStreamSynchronize(st));
    float ms_total = 0, ms_store = 0, ms_regress = 0;
    cudaEventElapsedTime(&ms_total, e0, e3);
    cudaEventElapsedTime(&ms_store, e0, e1);
    cudaEventElapsedTime(&ms_regress, e1, e2);
    cleanup();
#undef MLP_TRY
    if (failed) {
        ctx->error = "a tensor-core wait gave up in the training kernel";
        return KGPU_DEVICE_ERROR;
    }
    if (fit_failed) {
        ctx->error = "Monte Carlo produced a non-finite parameter, path or result";
        return KGPU_COMPUTATION_FAILURE;
    }
    ctx->last_launches = launches;
    ctx->last_kernel_ms = ms_total;
    auto moments = [&](const double* part, double* mean, double* err, double scale) {
        double s0 = 0.0, s1 = 0.0;
        for (int blk = 0; blk < fblocks; ++blk) {
            s0 += part[2 * blk];
            s1 += part[2 * blk + 1];
        }
        const double mu = s0 / double(n);
        const double var = n > 1 ? std::max(0.0, (s1 - s0 * mu) / double(n - 1)) : 0.0;
        *mean = mu * scale;
        *err = std::sqrt(var / double(n)) * scale;
    };
    const double disc0 = std::exp(-model->rate * (expiry / p.dates));
    const double immediate = std::max(0.0, sign * (model->spot - strike));
    double mean = 0.0, se = 0.0;
    moments(fin.data(), &mean, &se, disc0);
    out->price = std::max(immediate, mean);
    out->standard_error = se;
    out->out_of_sample = std::nan("");
    out->out_of_sample_error = std::nan("");
    if (lower) {
        double lm = 0.0, le = 0.0;
        moments(fin.data() + 2 * fblocks, &lm, &le, 1.0);
        out->out_of_sample = std::max(immediate, lm);
        out->out_of_sample_error = le;
    }
    out->wall_ms = ms_total;
    out->path_store_ms = ms_store;
    out->regression_ms = ms_regress;
    if (!std::isfinite(out->price)) {
        ctx->error = "Monte Carlo produced a non-finite parameter, path or result";
        return KGPU_COMPUTATION_FAILURE;
    }
    return KGPU_OK;
}

}  // namespace
}  // namespace kgpu

// LSMC with the continuation network (called by kgpu_lsmc_price for KGPU_BASIS_MLP and
// KGPU_BASIS_MLP_STANDALONE).
kgpu_status kgpu_lsmc_mlp(kgpu_context* ctx, const kgpu_model* model, double strike, double sign, double expiry,
                          const kgpu_lsmc_settings* settings, uint64_t fresh_seed, kgpu_lsmc_result* out) {
    if (cudaSetDevice(ctx->device) != cudaSuccess) return KGPU_DEVICE_ERROR;
    if (settings->precision != KGPU_PRECISION_FP32) {
        ctx->error = "the continuation network trains on an FP32 path store (precision must be FP32)";
        return KGPU_UNSUPPORTED_OPERATION;
    }
    return model->kind == KGPU_MODEL_HESTON
               ? kgpu::mlp_run<true>(ctx, model, strike, sign, expiry, settings, fresh_seed, out)
               : kgpu::mlp_run<false>(ctx, model, strike, sign, expiry, settings, fresh_seed, out);
}

extern "C" kgpu_status kgpu_mlp_train(kgpu_context* ctx, float* params, const float* samples, int32_t count,
                                      int32_t batch, int32_t steps, double learning_rate, int32_t trainer) {
    using namespace kgpu;
    if (!ctx || !params || !samples || count < 1 || batch < 1 || steps < 1 || !(learning_rate > 0.0) ||
        (trainer != KGPU_TRAINER_CLUSTER && trainer != KGPU_TRAINER_GRID))
        return KGPU_INVALID_INPUT;
    if (batch > 64 * kRows) {
        ctx->error = "the training batch is at most 8192 samples";
        return KGPU_INVALID_INPUT;
    }
    std::lock_guard<std::mutex> lock(ctx->mu);
    ctx->error.clear();
    if (cudaSetDevice(ctx->device) != cudaSuccess) return KGPU_DEVICE_ERROR;
    if (!configure_train_kernel()) {
        ctx->error = "cannot configure the training kernel's shared memory";
        return KGPU_DEVICE_ERROR;
    }
    const int blocks = (std::min(batch, count) + kRows - 1) / kRows;
    const int cluster_ctas = cluster_trainer_ctas(std::min(batch, count));
    if (trainer == KGPU_TRAINER_CLUSTER ? !cluster_trainer_fits(cluster_ctas) : !cooperative_fits(ctx->device, blocks)) {
        ctx->error = "the training kernel's CTAs do not fit the device at once";
        return KGPU_UNSUPPORTED_OPERATION;
    }
    // Parameters, Adam moments, gradient partials ([parameter][CTA]), W2 tiles, the
    // clustered trainer's slice sums and flags, the samples, the error word and the grid
    // barrier.
    const size_t floats = size_t(3) * kStride + size_t(blocks) * kStride + 2 * kHidden * kHidden +
                          size_t(2) * 8 * kStride + 64;
    const size_t bytes = floats * 4 + size_t(count) * 16 + 64;
    if (ctx->mlp_scratch.ensure(bytes)) return KGPU_DEVICE_ERROR;
    float* dparams = static_cast<float*>(ctx->mlp_scratch.ptr);
    float* dm = dparams + kStride;
    float* dv = dm + kStride;
    float* dpartials = dv + kStride;
    __nv_bfloat16* w2_tiles = reinterpret_cast<__nv_bfloat16*>(dpartials + size_t(blocks) * kStride);
    float* exchange = reinterpret_cast<float*>(w2_tiles + 2 * kHidden * kHidden);
    int* flags = reinterpret_cast<int*>(exchange + size_t(2) * 8 * kStride);
    float4* dsamples = reinterpret_cast<float4*>(flags + 64);
    int* derror = reinterpret_cast<int*>(dsamples + count);
    GridBarrier* barrier = reinterpret_cast<GridBarrier*>(derror + 2);
    cudaStream_t st = ctx->stream;
    if (cudaMemcpyAsync(dsamples, samples, size_t(count) * 16, cudaMemcpyHostToDevice, st) != cudaSuccess ||
        cudaMemcpyAsync(dparams, params, size_t(kParams) * 4, cudaMemcpyHostToDevice, st) != cudaSuccess ||
        cudaMemsetAsync(dm, 0, size_t(2) * kStride * 4, st) != cudaSuccess ||
        cudaMemsetAsync(derror, 0, 8 + sizeof(GridBarrier), st) != cudaSuccess)
        return KGPU_DEVICE_ERROR;
    Adam adam;
    TrainArgs ta{dparams, w2_tiles, dm, dv, dsamples, dpartials, barrier, derror, count, batch, steps,
                 0, float(learning_rate), adam.beta1, adam.beta2, adam.eps};
    void* args[] = {&ta};
    int failed = 0;
    bool clustered = false;
    if (trainer == KGPU_TRAINER_CLUSTER) {
        ClusterTrainArgs ca{dparams, dm, dv, dsamples, exchange, flags, derror, count, batch, steps,
                            0, float(learning_rate), adam.beta1, adam.beta2, adam.eps};
        if (launch_cluster_trainer(st, cluster_ctas, ca, clustered) != cudaSuccess) return KGPU_DEVICE_ERROR;
        if (!clustered) {
            ctx->error = "the device refused the clustered trainer's cooperative cluster launch";
            return KGPU_UNSUPPORTED_OPERATION;
        }
    }
    ctx->last_launches = 1;
    if ((!clustered && cudaLaunchCooperativeKernel(reinterpret_cast<const void*>(mlp_train_kernel), dim3(blocks),
                                                   dim3(kThreadsTrain), args, kTrainSmemBytes, st) != cudaSuccess) ||
        cudaMemcpyAsync(params, dparams, size_t(kParams) * 4, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaMemcpyAsync(&failed, derror, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess) {
        ctx->error = "training kernel failed";
        return KGPU_DEVICE_ERROR;
    }
    if (failed) {
        ctx->error = "a tensor-core wait or grid barrier gave up in the training kernel";
        return KGPU_DEVICE_ERROR;
    }
    return KGPU_OK;
}

extern "C" kgpu_status kgpu_mlp_gradients(kgpu_context* ctx, const float* params, const float* samples, int32_t count,
                                          float* grads, double* loss) {
    using namespace kgpu;
    if (!ctx || !params || !samples || !grads || !loss || count < 1) return KGPU_INVALID_INPUT;
    std::lock_guard<std::mutex> lock(ctx->mu);
    ctx->error.clear();
    if (cudaSetDevice(ctx->device) != cudaSuccess) return KGPU_DEVICE_ERROR;
    if (!configure_train_kernel()) {
        ctx->error = "cannot configure the training kernel's shared memory";
        return KGPU_DEVICE_ERROR;
    }
    const int blocks = (count + kRows - 1) / kRows;
    const size_t bytes = size_t(kParams) * 4 + size_t(count) * 16 + size_t(blocks) * kStride * 4 + 64;
    if (ctx->mlp_scratch.ensure(bytes)) return KGPU_DEVICE_ERROR;
    char* base = static_cast<char*>(ctx->mlp_scratch.ptr);
    float4* dsamples = reinterpret_cast<float4*>(base);
    float* dpartials = reinterpret_cast<float*>(base + size_t(count) * 16);
    float* dparams = dpartials + size_t(blocks) * kStride;
    int* derror = reinterpret_cast<int*>(dparams + kParams);
    cudaStream_t st = ctx->stream;
    std::vector<float> part(size_t(blocks) * kStride);
    int failed = 0;
    if (cudaMemcpyAsync(dsamples, samples, size_t(count) * 16, cudaMemcpyHostToDevice, st) != cudaSuccess ||
        cudaMemcpyAsync(dparams, params, size_t(kParams) * 4, cudaMemcpyHostToDevice, st) != cudaSuccess ||
        cudaMemsetAsync(derror, 0, sizeof(int), st) != cudaSuccess)
        return KGPU_DEVICE_ERROR;
    mlp_grad_kernel<<<blocks, kThreadsTrain, kTrainSmemBytes, st>>>(dparams, dsamples, 0, count, 1.0f / float(count), dpartials,
                                                            derror);
    if (cudaGetLastError() != cudaSuccess ||
        cudaMemcpyAsync(part.data(), dpartials, part.size() * 4, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaMemcpyAsync(&failed, derror, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess) {
        ctx->error = "training kernel failed";
        return KGPU_DEVICE_ERROR;
    }
    if (failed) {
        ctx->error = "a tensor-core wait gave up in the training kernel";
        return KGPU_DEVICE_ERROR;
    }
    double l = 0.0;
    for (int i = 0; i < kParams; ++i) {
        double g = 0.0;
        for (int blk = 0; blk < blocks; ++blk) g += part[size_t(blk) * kStride + i];
        grads[i] = float(g);
    }
    for (int blk = 0; blk < blocks; ++blk) l += part[size_t(blk) * kStride + kLossSlot];
    *loss = l / double(count);
    return KGPU_OK;
}
