// American exercise by least-squares Monte Carlo (Longstaff-Schwartz) on the GPU.
//
// Reference method: MonteCarloVanillaEngine::american_scenarios,
// crates/kiyosi/src/engines/monte_carlo/american.rs:955-1455, and solve_quadratic
// (1693-1749).  BSM with the quadratic basis {1, S/K, (S/K)^2} follows it step for step:
// per path the cumulative Brownian coordinate at each exercise date from the block
// streams (Pcg32::new(seed, path / 256), path-major, `dates` normals per path), spots
// S0 exp(drift (k+1)) exp(diffusion W_k), backward induction regressing discounted cash
// on the basis over in-the-money paths, exercise when intrinsic/K > continuation.
// Heston uses full-truncation Euler paths (`substeps` per exercise interval, two normals
// per step) and the ten monomials of degree <= 3 in (S/K, v/theta), with the same
// pivoted elimination and degree fallback.
//
// Kernels: lsmc_forward writes the path store [date][path] (coalesced); per date,
// lsmc_backward applies the next date's decision, discounts the cash and accumulates
// the in-the-money normal equations (products in the store's precision, FP64 across
// warps and blocks), lsmc_solve merges the block partials in block order and solves in
// FP64; lsmc_final and lsmc_lower_bound reduce the estimates.  The whole sequence is
// captured in a CUDA graph and replayed while the problem is unchanged (a changed one is
// re-captured and updates the executable graph in place).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <vector>

#include "../../include/kgpu.h"
#include "api_internal.h"
#include "lsmc_common.cuh"

namespace kgpu {
namespace {

// One exercise date of the backward induction (american.rs:1347-1417).
template <class Real, bool TWO>
__device__ __forceinline__ void backward_body(const LsmcParams<Real>& p, int date, const double* coef_next,
                                              const int* have_next, const Real* a, const Real* b, Real* cash,
                                              double* partials) {
    constexpr int T = TWO ? 10 : 3;
    constexpr int S = sum_count(T);
    Real acc[S];
#pragma unroll
    for (int j = 0; j < S; ++j) acc[j] = Real(0);
    const bool decide = coef_next != nullptr && *have_next;
    Real cn[T];
#pragma unroll
    for (int j = 0; j < T; ++j) cn[j] = decide ? Real(coef_next[j]) : Real(0);
    const Real inv_k = Real(1) / p.strike;
    // The 65-sum accumulator allows one CTA per SM, so the loop is latency-bound; each
    // thread loads kPrefetch paths before working through them in grid-stride order,
    // which keeps every thread's accumulation order (and the sums) unchanged.
    constexpr int kPrefetch = 4;
    const int stride = gridDim.x * blockDim.x;
    for (int base = blockIdx.x * blockDim.x + threadIdx.x; base < p.paths; base += kPrefetch * stride) {
        Real c_in[kPrefetch], a0[kPrefetch], b0[kPrefetch], a1[kPrefetch], b1[kPrefetch];
#pragma unroll
        for (int u = 0; u < kPrefetch; ++u) {
            const int i = base + u * stride;
            if (i < p.paths) {
                c_in[u] = cash[i];
                a0[u] = a[size_t(date) * p.paths + i];
                b0[u] = TWO ? b[size_t(date) * p.paths + i] : Real(0);
                a1[u] = decide ? a[size_t(date + 1) * p.paths + i] : Real(0);
                b1[u] = (decide && TWO) ? b[size_t(date + 1) * p.paths + i] : Real(0);
            }
        }
#pragma unroll
        for (int u = 0; u < kPrefetch; ++u) {
            const int i = base + u * stride;
            if (i >= p.paths) break;
            Real c = c_in[u];
            if (decide) {
                const Real s1 = spot_at_date<Real, TWO>(p, date + 1, a1[u]);
                const Real y1 = TWO ? b1[u] * p.y_scale : Real(0);
                const Real e = intrinsic(p, s1);
                if (e > Real(0) && e * inv_k > continuation<Real, TWO>(p, cn, s1 * inv_k, y1)) c = e;
            }
            c *= p.discount;
            cash[i] = c;
            const Real s = spot_at_date<Real, TWO>(p, date, a0[u]);
            if (intrinsic(p, s) > Real(0)) {
                Real f[T];
                lsmc_basis<Real, TWO>(s * inv_k, TWO ? b0[u] * p.y_scale : Real(0), f);
                const Real target = c * inv_k;
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
    block_sums<Real, S>(acc, partials);
}

template <class Real, bool TWO>
__global__ void __launch_bounds__(kLsmcThreads) lsmc_backward(LsmcParams<Real> p, int date, const double* coef_next,
                                                              const int* have_next, const Real* a, const Real* b,
                                                              Real* cash, double* partials) {
    backward_body<Real, TWO>(p, date, coef_next, have_next, a, b, cash, partials);
}

// One date of a BSM scenario batch: CTA row y is scenario y, with its cash
// ([scenario][path]), coefficients ([scenario][date][term]), flags ([scenario][date]) and
// partials ([scenario][sum][block]); the store is shared.
template <class Real>
__global__ void __launch_bounds__(kLsmcThreads) lsmc_backward_batch(const __grid_constant__ LsmcBatch<Real> batch,
                                                                    int date, const double* coef_next,
                                                                    const int* have_next, const Real* a, Real* cash,
                                                                    double* partials) {
    const int y = blockIdx.y;
    const LsmcParams<Real> p = batch.p[y];
    backward_body<Real, false>(p, date, coef_next ? coef_next + size_t(y) * p.dates * kMaxTerms : nullptr,
                               have_next ? have_next + size_t(y) * p.dates : nullptr, a, nullptr,
                               cash + size_t(y) * p.paths, partials + size_t(y) * sum_count(3) * gridDim.x);
}

// Date-0 decision and the mean of the cash (FP64 block partials: sum, sum of squares).
template <class Real, bool TWO>
__device__ __forceinline__ void final_body(const LsmcParams<Real>& p, const double* coef0, const int* have0,
                                           const Real* a, const Real* b, const Real* cash, double* partials) {
    constexpr int T = TWO ? 10 : 3;
    Real cn[T];
    const bool decide = *have0;
#pragma unroll
    for (int j = 0; j < T; ++j) cn[j] = decide ? Real(coef0[j]) : Real(0);
    const Real inv_k = Real(1) / p.strike;
    double s0 = 0.0, s1 = 0.0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < p.paths; i += gridDim.x * blockDim.x) {
        Real c = cash[i];
        if (decide) {
            const Real s = spot_at_date<Real, TWO>(p, 0, a[i]);
            const Real y = TWO ? b[i] * p.y_scale : Real(0);
            const Real e = intrinsic(p, s);
            if (e > Real(0) && e * inv_k > continuation<Real, TWO>(p, cn, s * inv_k, y)) c = e;
        }
        s0 += double(c);
        s1 += double(c) * double(c);
    }
    for (int off = 16; off > 0; off >>= 1) {
        s0 += __shfl_xor_sync(0xffffffffu, s0, off);
        s1 += __shfl_xor_sync(0xffffffffu, s1, off);
    }
    __shared__ double w0[kLsmcThreads / 32], w1[kLsmcThreads / 32];
    if ((threadIdx.x & 31) == 0) {
        w0[threadIdx.x >> 5] = s0;
        w1[threadIdx.x >> 5] = s1;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double t0 = 0.0, t1 = 0.0;
        for (int w = 0; w < kLsmcThreads / 32; ++w) {
            t0 += w0[w];
            t1 += w1[w];
        }
        partials[2 * blockIdx.x] = t0;
        partials[2 * blockIdx.x + 1] = t1;
    }
}

template <class Real, bool TWO>
__global__ void __launch_bounds__(kLsmcThreads) lsmc_final(LsmcParams<Real> p, const double* coef0, const int* have0,
                                                           const Real* a, const Real* b, const Real* cash,
                                                           double* partials) {
    final_body<Real, TWO>(p, coef0, have0, a, b, cash, partials);
}

template <class Real>
__global__ void __launch_bounds__(kLsmcThreads) lsmc_final_batch(const __grid_constant__ LsmcBatch<Real> batch,
                                                                 const double* coefs, const int* have, const Real* a,
                                                                 const Real* cash, double* partials) {
    const int y = blockIdx.y;
    const LsmcParams<Real> p = batch.p[y];
    final_body<Real, false>(p, coefs + size_t(y) * p.dates * kMaxTerms, have + size_t(y) * p.dates, a, nullptr,
                            cash + size_t(y) * p.paths, partials + size_t(y) * 2 * gridDim.x);
}

// Lower bound on fresh paths: the fitted policy applied forward (american.rs:574-637).
// The fitted FP64 coefficients in the path store's precision, for the forward pass.
template <class Real>
__global__ void coef_table_kernel(const double* coefs, Real* table, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) table[i] = Real(coefs[i]);
}

template <class Real, bool TWO>
__device__ __forceinline__ void lower_bound_body(const LsmcParams<Real>& p, uint64_t seed, const Real* table,
                                                 const int* have, double* partials) {
    const int dims = TWO ? p.dates * p.substeps * 2 : p.dates;
    const Real inv_k = Real(1) / p.strike;
    double s0 = 0.0, s1 = 0.0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < p.paths; i += gridDim.x * blockDim.x) {
        PcgSource<Real> n;
        n.start(seed, uint64_t(i), dims);
        Real x = Real(0), v = p.v0, value = Real(0), df = Real(1);
        for (int k = 0; k < p.dates; ++k) {
            if (!TWO) {
                x += n.normal();
            } else {
                for (int j = 0; j < p.substeps; ++j) {
                    const Real z1 = n.normal(), z2 = n.normal();
                    const Real vp = v > Real(0) ? v : Real(0);
                    const Real sv = xsqrt(vp) * p.sqrt_h;
                    x += (p.rate - p.dividend - Real(0.5) * vp) * p.h + sv * z1;
                    v += p.kappa * (p.theta - vp) * p.h + p.xi * sv * (p.rho * z1 + p.rho_bar * z2);
                }
            }
            df *= p.discount;
            const Real s = spot_at_date<Real, TWO>(p, k, x);
            const Real e = intrinsic(p, s);
            if (e > Real(0)) {
                bool stop = k == p.dates - 1;
                if (!stop && have[k]) {
                    stop = e * inv_k > continuation<Real, TWO>(p, table + k * kMaxTerms, s * inv_k,
                                                               TWO ? v * p.y_scale : Real(0));
                }
                if (stop) {
                    value = e * df;
                    break;
                }
            }
        }
        s0 += double(value);
        s1 += double(value) * double(value);
    }
    for (int off = 16; off > 0; off >>= 1) {
        s0 += __shfl_xor_sync(0xffffffffu, s0, off);
        s1 += __shfl_xor_sync(0xffffffffu, s1, off);
    }
    __shared__ double w0[kLsmcThreads / 32], w1[kLsmcThreads / 32];
    if ((threadIdx.x & 31) == 0) {
        w0[threadIdx.x >> 5] = s0;
        w1[threadIdx.x >> 5] = s1;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double t0 = 0.0, t1 = 0.0;
        for (int w = 0; w < kLsmcThreads / 32; ++w) {
            t0 += w0[w];
            t1 += w1[w];
        }
        partials[2 * blockIdx.x] = t0;
        partials[2 * blockIdx.x + 1] = t1;
    }
}

template <class Real, bool TWO>
__global__ void __launch_bounds__(kLsmcThreads) lsmc_lower_bound(LsmcParams<Real> p, uint64_t seed,
                                                                 const Real* table, const int* have,
                                                                 double* partials) {
    lower_bound_body<Real, TWO>(p, seed, table, have, partials);
}

template <class Real>
__global__ void __launch_bounds__(kLsmcThreads) lsmc_lower_bound_batch(const __grid_constant__ LsmcBatch<Real> batch,
                                                                       uint64_t seed, const Real* table,
                                                                       const int* have, double* partials) {
    const int y = blockIdx.y;
    const LsmcParams<Real> p = batch.p[y];
    lower_bound_body<Real, false>(p, seed, table + size_t(y) * p.dates * kMaxTerms, have + size_t(y) * p.dates,
                                  partials + size_t(y) * 2 * gridDim.x);
}

}  // namespace

// Runs one LSMC pricing in precision Real, or a batch of `count` BSM scenarios that share
// the path store (one result each, equal to the scalar pricing of that scenario); all
// device buffers come from the context.
template <class Real>
static kgpu_status lsmc_run(kgpu_context* ctx, const kgpu_model* models, int count, double strike, double sign,
                            double expiry, const kgpu_lsmc_settings* s, uint64_t fresh_seed, kgpu_lsmc_result* out) {
    const kgpu_model* model = models;
    const bool two = model->kind == KGPU_MODEL_HESTON;
    const bool batch = count > 1;
    LsmcBatch<Real> pb{};
    for (int y = 0; y < count; ++y) pb.p[y] = make_lsmc_params<Real>(models + y, strike, sign, expiry, s);
    const LsmcParams<Real>& p = pb.p[0];
    const int S = sum_count(p.terms);
    const size_t n = size_t(p.paths), d = size_t(p.dates), ns = size_t(count);
    const int blocks = std::min<int>(ctx->sm_count * 4, int((n + kLsmcThreads - 1) / kLsmcThreads));
    if (ctx->lsmc_store.ensure(n * d * sizeof(Real) * (two ? 2 : 1)) || ctx->lsmc_cash.ensure(ns * n * sizeof(Real)) ||
        ctx->lsmc_sums.ensure(ns * (size_t(blocks) + 1) * kMaxSums * sizeof(double)) ||
        ctx->lsmc_coef.ensure(ns * d * kMaxTerms * (sizeof(double) + sizeof(Real)) + ns * d * sizeof(int) + 64) ||
        ctx->lsmc_misc.ensure(ns * size_t(blocks) * 2 * sizeof(double) + 16))
        return KGPU_DEVICE_ERROR;
    Real* a = static_cast<Real*>(ctx->lsmc_store.ptr);
    Real* b = two ? a + n * d : nullptr;
    Real* cash = static_cast<Real*>(ctx->lsmc_cash.ptr);
    double* coefs = static_cast<double*>(ctx->lsmc_coef.ptr);
    int* have = reinterpret_cast<int*>(coefs + ns * d * kMaxTerms);
    int* failed = have + ns * d;
    // Converted coefficients after `failed`, aligned to 16 bytes.
    Real* table = reinterpret_cast<Real*>(
        (reinterpret_cast<uintptr_t>(failed + 1) + 15) & ~uintptr_t(15));
    double* partials = static_cast<double*>(ctx->lsmc_sums.ptr);
    double* reduced = partials + ns * size_t(blocks) * kMaxSums;  // one partial per sum and scenario
    double* finals = static_cast<double*>(ctx->lsmc_misc.ptr);
    cudaStream_t st = ctx->stream;
    const bool lower = fresh_seed != s->seed;
    double* lp = nullptr;
    if (lower) {
        if (ctx->mlp_scratch.ensure(ns * size_t(blocks) * 2 * sizeof(double))) return KGPU_DEVICE_ERROR;
        lp = static_cast<double*>(ctx->mlp_scratch.ptr);
    }
    for (cudaEvent_t& e : ctx->lsmc_events)
        if (!e && cudaEventCreate(&e) != cudaSuccess) return KGPU_DEVICE_ERROR;
    cudaEvent_t e0 = ctx->lsmc_events[0], e1 = ctx->lsmc_events[1], e2 = ctx->lsmc_events[2],
                e3 = ctx->lsmc_events[3];
    int launches = 0;
    // The whole launch sequence: captured once per problem into a CUDA graph and replayed.
    auto enqueue = [&]() {
        launches = 0;
        cudaMemsetAsync(coefs, 0, ns * d * kMaxTerms * sizeof(double) + ns * d * sizeof(int) + sizeof(int), st);
        if (batch)
            lsmc_forward_batch<Real><<<unsigned((n + 255) / 256), 256, 0, st>>>(pb, count, s->seed, a, cash);
        else if (two)
            lsmc_forward<Real, true><<<unsigned((n + 255) / 256), 256, 0, st>>>(p, s->seed, a, b, cash);
        else
            lsmc_forward<Real, false><<<unsigned((n + 255) / 256), 256, 0, st>>>(p, s->seed, a, b, cash);
        ++launches;
        cudaEventRecordWithFlags(e1, st, cudaEventRecordExternal);
        for (int date = p.dates - 2; date >= 0; --date) {
            const double* cnext = date + 1 <= p.dates - 2 ? coefs + size_t(date + 1) * kMaxTerms : nullptr;
            const int* hnext = date + 1 <= p.dates - 2 ? have + date + 1 : nullptr;
            if (batch) {
                lsmc_backward_batch<Real><<<dim3(blocks, count), kLsmcThreads, 0, st>>>(pb, date, cnext, hnext, a, cash,
                                                                                       partials);
                reduce_partials_kernel<<<dim3(S, count), 32, 0, st>>>(partials, blocks, reduced);
                lsmc_solve<false><<<count, kSolveThreads, 0, st>>>(reduced, 1, p.max_degree,
                                                                   coefs + size_t(date) * kMaxTerms, have + date,
                                                                   failed, int(d) * kMaxTerms, int(d));
            } else if (two) {
                lsmc_backward<Real, true><<<blocks, kLsmcThreads, 0, st>>>(p, date, cnext, hnext, a, b, cash, partials);
                reduce_partials_kernel<<<S, 32, 0, st>>>(partials, blocks, reduced);
                lsmc_solve<true><<<1, kSolveThreads, 0, st>>>(reduced, 1, p.max_degree, coefs + size_t(date) * kMaxTerms,
                                                    have + date, failed);
            } else {
                lsmc_backward<Real, false><<<blocks, kLsmcThreads, 0, st>>>(p, date, cnext, hnext, a, b, cash,
                                                                            partials);
                reduce_partials_kernel<<<S, 32, 0, st>>>(partials, blocks, reduced);
                lsmc_solve<false><<<1, kSolveThreads, 0, st>>>(reduced, 1, p.max_degree, coefs + size_t(date) * kMaxTerms,
                                                     have + date, failed);
            }
            launches += 3;
        }
        if (batch)
            lsmc_final_batch<Real><<<dim3(blocks, count), kLsmcThreads, 0, st>>>(pb, coefs, have, a, cash, finals);
        else if (two)
            lsmc_final<Real, true><<<blocks, kLsmcThreads, 0, st>>>(p, coefs, have, a, b, cash, finals);
        else
            lsmc_final<Real, false><<<blocks, kLsmcThreads, 0, st>>>(p, coefs, have, a, b, cash, finals);
        ++launches;
        cudaEventRecordWithFlags(e2, st, cudaEventRecordExternal);
        if (lower) {
            const int terms = count * int(d) * kMaxTerms;
            coef_table_kernel<Real><<<(terms + 255) / 256, 256, 0, st>>>(coefs, table, terms);
            if (batch)
                lsmc_lower_bound_batch<Real><<<dim3(blocks, count), kLsmcThreads, 0, st>>>(pb, fresh_seed, table,
                                                                                          have, lp);
            else if (two)
                lsmc_lower_bound<Real, true><<<blocks, kLsmcThreads, 0, st>>>(p, fresh_seed, table, have, lp);
            else
                lsmc_lower_bound<Real, false><<<blocks, kLsmcThreads, 0, st>>>(p, fresh_seed, table, have, lp);
            launches += 2;
        }
    };
    // Key of the captured sequence: every argument its launches bake in.
    std::vector<unsigned char> key;
    {
        const void* ptrs[] = {a, b, cash, coefs, partials, finals, lp};
        const uint64_t tail[] = {s->seed, fresh_seed, uint64_t(blocks) | (uint64_t(sizeof(Real)) << 32),
                                 uint64_t(count)};
        key.resize(sizeof(LsmcParams<Real>) * ns + sizeof(ptrs) + sizeof(tail));
        unsigned char* k = key.data();
        std::memcpy(k, pb.p, sizeof(LsmcParams<Real>) * ns);
        std::memcpy(k + sizeof(LsmcParams<Real>) * ns, ptrs, sizeof(ptrs));
        std::memcpy(k + sizeof(LsmcParams<Real>) * ns + sizeof(ptrs), tail, sizeof(tail));
    }
    if (!(ctx->lsmc_exec && ctx->lsmc_key == key)) {
        cudaGraph_t graph = nullptr;
        bool captured = cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal) == cudaSuccess;
        if (captured) {
            enqueue();
            captured = cudaStreamEndCapture(st, &graph) == cudaSuccess && graph;
        }
        if (captured) {
            cudaGraphExecUpdateResultInfo info;
            if (!ctx->lsmc_exec || cudaGraphExecUpdate(ctx->lsmc_exec, graph, &info) != cudaSuccess) {
                cudaGetLastError();
                if (ctx->lsmc_exec) cudaGraphExecDestroy(ctx->lsmc_exec);
                ctx->lsmc_exec = nullptr;
                if (cudaGraphInstantiate(&ctx->lsmc_exec, graph, 0) != cudaSuccess) ctx->lsmc_exec = nullptr;
            }
            cudaGraphDestroy(graph);
        }
        ctx->lsmc_key = ctx->lsmc_exec ? key : std::vector<unsigned char>();
    } else {
        // Replaying: count the launches the sequence holds.
        launches = 3 * (p.dates - 1) + 2 + (lower ? 2 : 0);
    }
    cudaGetLastError();  // a refused capture or update leaves nothing behind
    cudaEventRecord(e0, st);
    if (ctx->lsmc_exec) {
        if (cudaGraphLaunch(ctx->lsmc_exec, st) != cudaSuccess) {
            ctx->error = "CUDA graph launch failed";
            return KGPU_DEVICE_ERROR;
        }
    } else {
        enqueue();  // capture unavailable: launch directly
    }
    cudaEventRecord(e3, st);
    std::vector<double> lower_partials;
    if (lower) {
        lower_partials.resize(ns * size_t(blocks) * 2);
        cudaMemcpyAsync(lower_partials.data(), lp, lower_partials.size() * sizeof(double), cudaMemcpyDeviceToHost, st);
    }
    std::vector<double> fin(ns * size_t(blocks) * 2);
    int fail_flag = 0;
    cudaMemcpyAsync(fin.data(), finals, fin.size() * sizeof(double), cudaMemcpyDeviceToHost, st);
    cudaMemcpyAsync(&fail_flag, failed, sizeof(int), cudaMemcpyDeviceToHost, st);
    cudaError_t err = cudaStreamSynchronize(st);
    // Timing: the whole call from stream events around the graph; the path store and the
    // regression from the events the graph records (NaN when a query is refused; the
    // refusal is cleared so it cannot surface in a later call).
    float ms_total = 0, ms_store = 0, ms_regress = 0;
    if (cudaEventElapsedTime(&ms_total, e0, e3) != cudaSuccess) ms_total = std::nanf("");
    if (cudaEventElapsedTime(&ms_store, e0, e1) != cudaSuccess) ms_store = std::nanf("");
    if (cudaEventElapsedTime(&ms_regress, e1, e2) != cudaSuccess) ms_regress = std::nanf("");
    cudaGetLastError();
    if (err != cudaSuccess) {
        ctx->error = cudaGetErrorString(err);
        return KGPU_DEVICE_ERROR;
    }
    if (fail_flag) {
        ctx->error = "Monte Carlo produced a non-finite parameter, path or result";
        return KGPU_COMPUTATION_FAILURE;
    }
    ctx->last_launches = launches;
    ctx->last_kernel_ms = ms_total;
    for (int y = 0; y < count; ++y) {
        const kgpu_model* m = models + y;
        const double* fy = fin.data() + size_t(y) * blocks * 2;
        double s0 = 0.0, s1 = 0.0;
        for (int blk = 0; blk < blocks; ++blk) {
            s0 += fy[2 * blk];
            s1 += fy[2 * blk + 1];
        }
        const double disc0 = std::exp(-m->rate * (expiry / s->exercise_dates));
        const double mean = s0 / double(n);
        const double var = n > 1 ? std::max(0.0, (s1 - s0 * mean) / double(n - 1)) : 0.0;
        const double immediate = std::max(0.0, sign * (m->spot - strike));
        kgpu_lsmc_result& o = out[y];
        o.price = std::max(immediate, mean * disc0);
        o.standard_error = std::sqrt(var / double(n)) * disc0;
        o.out_of_sample = std::nan("");
        o.out_of_sample_error = std::nan("");
        if (lower) {
            const double* ly = lower_partials.data() + size_t(y) * blocks * 2;
            double l0 = 0.0, l1 = 0.0;
            for (int blk = 0; blk < blocks; ++blk) {
                l0 += ly[2 * blk];
                l1 += ly[2 * blk + 1];
            }
            const double lm = l0 / double(n);
            const double lv = n > 1 ? std::max(0.0, (l1 - l0 * lm) / double(n - 1)) : 0.0;
            o.out_of_sample = std::max(immediate, lm);
            o.out_of_sample_error = std::sqrt(lv / double(n));
        }
        o.wall_ms = ms_total;
        o.path_store_ms = ms_store;
        o.regression_ms = ms_regress;
        if (!std::isfinite(o.price)) {
            ctx->error = "Monte Carlo produced a non-finite parameter, path or result";
            return KGPU_COMPUTATION_FAILURE;
        }
    }
    return KGPU_OK;
}

}  // namespace kgpu

kgpu_status kgpu_lsmc_mlp(kgpu_context* ctx, const kgpu_model* model, double strike, double sign, double expiry,
                          const kgpu_lsmc_settings* settings, uint64_t fresh_seed, kgpu_lsmc_result* out);

// Checks shared by the scalar and the scenario entry points.
static kgpu_status lsmc_check(kgpu_context* ctx, const kgpu_model* model, double strike, double sign, double expiry,
                              const kgpu_lsmc_settings* settings) {
    auto bad = [&](const char* msg) {
        ctx->error = msg;
        return KGPU_INVALID_INPUT;
    };
    if (settings->exercise_dates < 2) return bad("American Monte Carlo requires at least two exercise intervals");
    if (settings->path_count < 1) return bad("path_count must be positive");
    if (!(strike > 0.0) || !(expiry > 0.0) || (sign != 1.0 && sign != -1.0)) return bad("invalid option terms");
    if (settings->sampling != KGPU_SAMPLING_PSEUDO_RANDOM) {
        ctx->error = "GPU LSMC samples pseudo-random paths";
        return KGPU_UNSUPPORTED_OPERATION;
    }
    if (model->kind == KGPU_MODEL_LOCAL_VOL) {
        ctx->error = "GPU LSMC supports BSM and Heston";
        return KGPU_UNSUPPORTED_OPERATION;
    }
    if (settings->basis < KGPU_BASIS_QUADRATIC || settings->basis > KGPU_BASIS_MLP_STANDALONE)
        return bad("unknown basis");
    const bool heston = model->kind == KGPU_MODEL_HESTON;
    if (settings->basis != KGPU_BASIS_MLP && settings->basis != KGPU_BASIS_MLP_STANDALONE &&
        (settings->basis == KGPU_BASIS_QUADRATIC) == heston)
        return bad("the quadratic basis prices BSM, the cubic (S/K, v) basis Heston");
    return KGPU_OK;
}

extern "C" kgpu_status kgpu_lsmc_price(kgpu_context* ctx, const kgpu_model* model, double strike, double sign,
                                       double expiry, const kgpu_lsmc_settings* settings, uint64_t fresh_seed,
                                       kgpu_lsmc_result* out) {
    if (!ctx || !model || !settings || !out) return KGPU_INVALID_INPUT;
    std::lock_guard<std::mutex> lock(ctx->mu);
    ctx->error.clear();
    if (const kgpu_status st = lsmc_check(ctx, model, strike, sign, expiry, settings)) return st;
    if (settings->basis == KGPU_BASIS_MLP || settings->basis == KGPU_BASIS_MLP_STANDALONE) {
        return kgpu_lsmc_mlp(ctx, model, strike, sign, expiry, settings, fresh_seed, out);
    }
    if (cudaSetDevice(ctx->device) != cudaSuccess) return KGPU_DEVICE_ERROR;
    return settings->precision == KGPU_PRECISION_FP64
               ? kgpu::lsmc_run<double>(ctx, model, 1, strike, sign, expiry, settings, fresh_seed, out)
               : kgpu::lsmc_run<float>(ctx, model, 1, strike, sign, expiry, settings, fresh_seed, out);
}

extern "C" kgpu_status kgpu_lsmc_price_scenarios(kgpu_context* ctx, const kgpu_model* models, int32_t count,
                                                 double strike, double sign, double expiry,
                                                 const kgpu_lsmc_settings* settings, uint64_t fresh_seed,
                                                 kgpu_lsmc_result* out) {
    if (!ctx || !models || !settings || !out) return KGPU_INVALID_INPUT;
    std::lock_guard<std::mutex> lock(ctx->mu);
    ctx->error.clear();
    if (count < 1 || count > kgpu::kMaxLsmcScenarios) {
        ctx->error = "an LSMC scenario batch holds 1 to 16 scenarios";
        return KGPU_INVALID_INPUT;
    }
    for (int y = 0; y < count; ++y) {
        if (const kgpu_status st = lsmc_check(ctx, models + y, strike, sign, expiry, settings)) return st;
        if (models[y].kind != KGPU_MODEL_BSM) {
            ctx->error = "LSMC scenario batches price Black-Scholes-Merton scenarios";
            return KGPU_UNSUPPORTED_OPERATION;
        }
    }
    if (settings->basis != KGPU_BASIS_QUADRATIC) {
        ctx->error = "LSMC scenario batches use the quadratic basis";
        return KGPU_UNSUPPORTED_OPERATION;
    }
    if (cudaSetDevice(ctx->device) != cudaSuccess) return KGPU_DEVICE_ERROR;
    return settings->precision == KGPU_PRECISION_FP64
               ? kgpu::lsmc_run<double>(ctx, models, count, strike, sign, expiry, settings, fresh_seed, out)
               : kgpu::lsmc_run<float>(ctx, models, count, strike, sign, expiry, settings, fresh_seed, out);
}
