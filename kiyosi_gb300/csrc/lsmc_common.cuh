// Path store shared by the LSMC regressions (polynomial in lsmc.cu, the continuation
// network in mlp.cu): parameters, the forward kernel and spot/intrinsic helpers.
#pragma once
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>

#include "../../include/kgpu.h"
#include "path_engine.cuh"

namespace kgpu {
namespace {

template <class Real>
struct LsmcParams {
    Real spot, strike, sign, drift, diffusion, discount;
    Real rate, dividend, kappa, theta, xi, rho, rho_bar, v0, h, sqrt_h, y_scale;
    int dates, substeps, paths, terms, max_degree;
};

template <class Real, bool TWO>
__device__ __forceinline__ Real spot_at_date(const LsmcParams<Real>& p, int k, Real a) {
    if (!TWO) return p.spot * xexp(p.drift * Real(k + 1)) * xexp(p.diffusion * a);
    return p.spot * xexp(a);
}

template <class Real>
__device__ __forceinline__ Real intrinsic(const LsmcParams<Real>& p, Real spot) {
    const Real v = p.sign * (spot - p.strike);
    return v > Real(0) ? v : Real(0);
}

// Host-side parameters of one pricing (exercise grid, Euler substeps, basis size).
template <class Real>
LsmcParams<Real> make_lsmc_params(const kgpu_model* model, double strike, double sign, double expiry,
                                  const kgpu_lsmc_settings* s) {
    const bool two = model->kind == KGPU_MODEL_HESTON;
    LsmcParams<Real> p{};
    const double dt = expiry / s->exercise_dates;
    p.spot = Real(model->spot);
    p.strike = Real(strike);
    p.sign = Real(sign);
    p.drift = Real((model->rate - model->dividend - 0.5 * model->volatility * model->volatility) * dt);
    p.diffusion = Real(model->volatility * std::sqrt(dt));
    p.discount = Real(std::exp(-model->rate * dt));
    p.rate = Real(model->rate);
    p.dividend = Real(model->dividend);
    p.kappa = Real(model->kappa);
    p.theta = Real(model->theta);
    p.xi = Real(model->xi);
    p.rho = Real(model->rho);
    p.rho_bar = Real(std::sqrt(1.0 - model->rho * model->rho));
    p.v0 = Real(model->v0);
    p.substeps = two ? std::max(1, s->substeps) : 1;
    p.h = Real(dt / p.substeps);
    p.sqrt_h = Real(std::sqrt(dt / p.substeps));
    p.y_scale = Real(two && model->theta > 0.0 ? 1.0 / model->theta : 1.0);
    p.dates = s->exercise_dates;
    p.paths = s->path_count;
    p.terms = two ? 10 : 3;
    p.max_degree = two ? 3 : 2;
    return p;
}

// Scenarios of one batched pricing (bumped BSM contexts sharing the random numbers) and
// their parameters, passed by value to the batch kernels; blockIdx.y selects one.
constexpr int kMaxLsmcScenarios = 16;

template <class Real>
struct LsmcBatch {
    LsmcParams<Real> p[kMaxLsmcScenarios];
};

constexpr int kLsmcThreads = 128;
constexpr int kMaxTerms = 10;
constexpr int kMaxSums = kMaxTerms * (kMaxTerms + 1) / 2 + kMaxTerms;  // upper triangle + rhs

__host__ __device__ constexpr int sum_count(int terms) { return terms * (terms + 1) / 2 + terms; }

template <class Real, bool TWO>
__device__ __forceinline__ void lsmc_basis(Real x, Real y, Real* f) {
    f[0] = Real(1);
    f[1] = x;
    if (!TWO) {
        f[2] = x * x;
        return;
    }
    f[2] = y;
    f[3] = x * x;
    f[4] = x * y;
    f[5] = y * y;
    f[6] = x * x * x;
    f[7] = x * x * y;
    f[8] = x * y * y;
    f[9] = y * y * y;
}

// `coef` in the path store's precision (converted from the FP64 fit once per thread or
// block, not per path: on GB300 a double-to-float conversion issues on the FP64 pipe).
template <class Real, bool TWO>
__device__ __forceinline__ Real continuation(const LsmcParams<Real>& p, const Real* coef, Real x, Real y) {
    Real f[kMaxTerms];
    lsmc_basis<Real, TWO>(x, y, f);
    Real c = Real(0);
#pragma unroll
    for (int i = 0; i < (TWO ? 10 : 3); ++i) c += coef[i] * f[i];
    return c;
}

// The block's FP64 partial of each normal-equation sum, written sum-major (the solve
// reads each sum coalesced).  FP32 accumulators go through shared memory and each sum
// is added by one thread in thread order: 65 x 128 FP64 additions per block instead of
// a 5-step butterfly on every lane (GB300's FP64 pipe is the slow one).  FP64
// accumulators keep the butterfly (their staging would not fit in shared memory).
template <class Real, int S>
__device__ __forceinline__ void block_sums(const Real (&acc)[S], double* partials) {
    if constexpr (sizeof(Real) == 4) {
        __shared__ float staged[S][kLsmcThreads + 1];  // padded: row reads hit distinct banks
#pragma unroll
        for (int j = 0; j < S; ++j) staged[j][threadIdx.x] = acc[j];
        __syncthreads();
        for (int j = threadIdx.x; j < S; j += blockDim.x) {
            double v = 0.0;
            for (int t = 0; t < kLsmcThreads; ++t) v += double(staged[j][t]);
            partials[size_t(j) * gridDim.x + blockIdx.x] = v;
        }
    } else {
        __shared__ double warp_sums[kLsmcThreads / 32][S];
        const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
        for (int j = 0; j < S; ++j) {
            double v = double(acc[j]);
            for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
            if (lane == 0) warp_sums[warp][j] = v;
        }
        __syncthreads();
        for (int j = threadIdx.x; j < S; j += blockDim.x) {
            double v = 0.0;
            for (int w = 0; w < kLsmcThreads / 32; ++w) v += warp_sums[w][j];
            partials[size_t(j) * gridDim.x + blockIdx.x] = v;
        }
    }
}

// Sums each normal-equation sum's block partials, one warp per sum on its own SM: lanes
// stride over the partials in a fixed order and a fixed shuffle tree adds the lanes.
// The solve then reads one partial per sum, so these sums are its inputs bit for bit,
// while the FP64 additions are spread over many SMs (one SM's FP64 pipe is slow).
// A grid with blockIdx.y > 0 reduces scenario y's sums ([S][blocks] partials each).
__global__ void __launch_bounds__(32) reduce_partials_kernel(const double* partials, int blocks, double* sums) {
    const int j = blockIdx.x, lane = threadIdx.x;
    partials += size_t(blockIdx.y) * gridDim.x * blocks;
    sums += size_t(blockIdx.y) * gridDim.x;
    double v = 0.0;
    for (int base = lane; base < blocks; base += 8 * 32) {
        double chunk[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) {
            const int blk = base + 32 * u;
            chunk[u] = blk < blocks ? partials[size_t(j) * blocks + blk] : 0.0;
        }
#pragma unroll
        for (int u = 0; u < 8; ++u)
            if (base + 32 * u < blocks) v += chunk[u];
    }
    for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
    if (lane == 0) sums[j] = v;
}

// Merges the block partials in block order and solves the normal equations with pivoting
// and degree fallback (solve_quadratic, american.rs:1693-1749), in FP64.
// Threads of the solve's launch: 16 warps read the block partials of the normal-equation
// sums concurrently (the order of each sum's additions does not depend on the warp
// count); 512 threads leave the elimination its 128 registers.
constexpr int kSolveThreads = 512;

// A grid of several CTAs solves one system per scenario: CTA y reads its partials at
// y S blocks and writes its coefficients at y coef_stride, its flag at y have_stride.
template <bool TWO>
__global__ void __launch_bounds__(kSolveThreads) lsmc_solve(const double* partials, int blocks, int max_degree, double* coef, int* have,
                           int* failed, int coef_stride = 0, int have_stride = 0) {
    constexpr int T = TWO ? 10 : 3;
    constexpr int S = sum_count(T);
    partials += size_t(blockIdx.x) * S * blocks;
    coef += size_t(blockIdx.x) * coef_stride;
    have += size_t(blockIdx.x) * have_stride;
    __shared__ double sums[S];
    // Each warp owns the sums j = warp + 16 q.  Lanes stride over the block partials of
    // a sum in a fixed order, then a fixed shuffle tree adds the lanes (deterministic).
    // The loads of eight partials of all of a warp's sums are issued before they are
    // added, so the reduction is not one load latency per partial.
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, warps = blockDim.x >> 5;
    constexpr int kPerWarp = (S + kSolveThreads / 32 - 1) / (kSolveThreads / 32);
    double v[kPerWarp];
#pragma unroll
    for (int q = 0; q < kPerWarp; ++q) v[q] = 0.0;
    for (int base = lane; base < blocks; base += 8 * 32) {
        double chunk[kPerWarp][8];
#pragma unroll
        for (int q = 0; q < kPerWarp; ++q) {
            const int j = warp + warps * q;
#pragma unroll
            for (int u = 0; u < 8; ++u) {
                const int blk = base + 32 * u;
                chunk[q][u] = (j < S && blk < blocks) ? partials[size_t(j) * blocks + blk] : 0.0;
            }
        }
#pragma unroll
        for (int q = 0; q < kPerWarp; ++q)
#pragma unroll
            for (int u = 0; u < 8; ++u)
                if (base + 32 * u < blocks) v[q] += chunk[q][u];
    }
#pragma unroll
    for (int q = 0; q < kPerWarp; ++q) {
        const int j = warp + warps * q;
        double t = v[q];
        for (int off = 16; off > 0; off >>= 1) t += __shfl_xor_sync(0xffffffffu, t, off);
        if (lane == 0 && j < S) sums[j] = t;
    }
    __syncthreads();
    // Pivoted elimination by one warp: lane r holds row r of the augmented system (the
    // right-hand side at index T).  Each element is updated with the same operations as
    // the sequential elimination; the pivot is the last row with the largest magnitude,
    // as there.
    if (threadIdx.x >= 32) return;
    if (lane == 0) {
        for (int j = 0; j < kMaxTerms; ++j) coef[j] = 0.0;
        *have = 0;
    }
    if (sums[0] == 0.0) return;
    double full[T + 1];
#pragma unroll
    for (int c = 0; c < T; ++c) {
        const int r0 = lane < c ? lane : c, c0 = lane < c ? c : lane;
        full[c] = lane < T ? sums[r0 * T - r0 * (r0 - 1) / 2 + (c0 - r0)] : 0.0;
    }
    full[T] = lane < T ? sums[T * (T + 1) / 2 + lane] : 0.0;
    for (int degree = max_degree; degree >= 0; --degree) {
        const int k = TWO ? (degree + 1) * (degree + 2) / 2 : degree + 1;
        double m[T + 1];
#pragma unroll
        for (int c = 0; c <= T; ++c) m[c] = (c < k || c == T) ? full[c] : 0.0;
        double scale = 0.0;
        if (lane < k) {
#pragma unroll
            for (int c = 0; c < T; ++c)
                if (c < k) scale = fmax(scale, fabs(m[c]));
        }
        for (int off = 16; off > 0; off >>= 1) scale = fmax(scale, __shfl_xor_sync(0xffffffffu, scale, off));
        bool singular = false;
#pragma unroll
        for (int col = 0; col < T; ++col) {
            if (col >= k) break;
            double best = (lane >= col && lane < k) ? fabs(m[col]) : -1.0;
            int pivot = lane;
            for (int off = 16; off > 0; off >>= 1) {
                const double ob = __shfl_xor_sync(0xffffffffu, best, off);
                const int op = __shfl_xor_sync(0xffffffffu, pivot, off);
                if (ob > best || (ob == best && op > pivot)) {
                    best = ob;
                    pivot = op;
                }
            }
            const double pv = __shfl_sync(0xffffffffu, m[col], pivot);
            if (!isfinite(pv)) {
                if (lane == 0) *failed = 1;
                return;
            }
            if (fabs(pv) <= 1e-14 * scale) {
                singular = true;
                break;
            }
            const int src = lane == col ? pivot : (lane == pivot ? col : lane);
            double prow[T + 1];
#pragma unroll
            for (int c = 0; c <= T; ++c) {
                m[c] = __shfl_sync(0xffffffffu, m[c], src);
                prow[c] = __shfl_sync(0xffffffffu, m[c], col);
            }
            if (lane > col && lane < k) {
                const double factor = m[col] / prow[col];
#pragma unroll
                for (int c = 0; c < T; ++c)
                    if (c >= col && c < k) m[c] -= factor * prow[c];
                m[T] -= factor * prow[T];
            }
        }
        if (singular) continue;
        double x[T];
        bool finite = true;
#pragma unroll
        for (int r = T - 1; r >= 0; --r) {
            x[r] = 0.0;
            if (r >= k) continue;
            double v = m[T];
#pragma unroll
            for (int c = 0; c < T; ++c)
                if (c > r && c < k) v -= m[c] * x[c];
            x[r] = __shfl_sync(0xffffffffu, v / m[r], r);
            finite = finite && isfinite(x[r]);
        }
        if (lane == 0) {
            if (!finite) {
                *failed = 1;
                return;
            }
            for (int r = 0; r < k; ++r) coef[r] = x[r];
            *have = 1;
        }
        return;
    }
    if (lane == 0) *failed = 1;
}

// Forward pass: the path store and the terminal cash.
template <class Real, bool TWO>
__global__ void __launch_bounds__(256) lsmc_forward(LsmcParams<Real> p, uint64_t seed, Real* a, Real* b,
                                                    Real* cash) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= p.paths) return;
    const int dims = TWO ? p.dates * p.substeps * 2 : p.dates;
    PcgSource<Real> n;
    n.start(seed, uint64_t(i), dims);
    Real x = Real(0), v = p.v0;
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
            b[size_t(k) * p.paths + i] = v;
        }
        a[size_t(k) * p.paths + i] = x;
    }
    cash[i] = intrinsic(p, spot_at_date<Real, TWO>(p, p.dates - 1, x));
}

// Forward pass of a BSM scenario batch: the store holds the cumulative Brownian
// coordinate, which every scenario shares (its spot, rate, dividend and volatility enter
// only through spot_at_date), so it is written once; each scenario gets its own terminal
// cash ([scenario][path]).  The draws and the store are those of lsmc_forward.
template <class Real>
__global__ void __launch_bounds__(256) lsmc_forward_batch(const __grid_constant__ LsmcBatch<Real> batch, int count,
                                                          uint64_t seed, Real* a, Real* cash) {
    const LsmcParams<Real>& p0 = batch.p[0];
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= p0.paths) return;
    PcgSource<Real> n;
    n.start(seed, uint64_t(i), p0.dates);
    Real x = Real(0);
    for (int k = 0; k < p0.dates; ++k) {
        x += n.normal();
        a[size_t(k) * p0.paths + i] = x;
    }
    for (int y = 0; y < count; ++y) {
        const LsmcParams<Real> p = batch.p[y];
        cash[size_t(y) * p.paths + i] = intrinsic(p, spot_at_date<Real, false>(p, p.dates - 1, x));
    }
}

}  // namespace
}  // namespace kgpu
