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

template <class Real, bool TWO>
__device__ __forceinline__ Real continuation(const LsmcParams<Real>& p, const double* coef, Real x, Real y) {
    Real f[kMaxTerms];
    lsmc_basis<Real, TWO>(x, y, f);
    Real c = Real(0);
#pragma unroll
    for (int i = 0; i < (TWO ? 10 : 3); ++i) c += Real(coef[i]) * f[i];
    return c;
}

// Merges the block partials in block order and solves the normal equations with pivoting
// and degree fallback (solve_quadratic, american.rs:1693-1749), in FP64.
template <bool TWO>
__global__ void lsmc_solve(const double* partials, int blocks, int max_degree, double* coef, int* have,
                           int* failed) {
    constexpr int T = TWO ? 10 : 3;
    constexpr int S = sum_count(T);
    __shared__ double sums[S];
    // One warp per sum: lanes stride over the block partials, then a fixed shuffle tree
    // (deterministic, and short enough that the solve is not latency-bound on it).
    const int lane = threadIdx.x & 31, warps = blockDim.x >> 5;
    for (int j = threadIdx.x >> 5; j < S; j += warps) {
        double v = 0.0;
        for (int blk = lane; blk < blocks; blk += 32) v += partials[size_t(blk) * S + j];
        for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
        if (lane == 0) sums[j] = v;
    }
    __syncthreads();
    if (threadIdx.x != 0) return;
    for (int j = 0; j < kMaxTerms; ++j) coef[j] = 0.0;
    *have = 0;
    if (sums[0] == 0.0) return;
    double full[T][T + 1];
    int q = 0;
    for (int r = 0; r < T; ++r)
        for (int c = r; c < T; ++c) {
            full[r][c] = sums[q];
            full[c][r] = sums[q];
            ++q;
        }
    for (int r = 0; r < T; ++r) full[r][T] = sums[q++];
    for (int degree = max_degree; degree >= 0; --degree) {
        const int k = TWO ? (degree + 1) * (degree + 2) / 2 : degree + 1;
        double m[T][T + 1];
        for (int r = 0; r < k; ++r) {
            for (int c = 0; c < k; ++c) m[r][c] = full[r][c];
            m[r][k] = full[r][T];
        }
        double scale = 0.0;
        for (int r = 0; r < k; ++r)
            for (int c = 0; c < k; ++c) scale = fmax(scale, fabs(m[r][c]));
        bool singular = false;
        for (int col = 0; col < k && !singular; ++col) {
            int pivot = col;
            for (int r = col + 1; r < k; ++r)
                if (fabs(m[r][col]) >= fabs(m[pivot][col])) pivot = r;
            if (!isfinite(m[pivot][col])) {
                *failed = 1;
                return;
            }
            if (fabs(m[pivot][col]) <= 1e-14 * scale) {
                singular = true;
                break;
            }
            if (pivot != col)
                for (int c = 0; c <= k; ++c) {
                    double t = m[col][c];
                    m[col][c] = m[pivot][c];
                    m[pivot][c] = t;
                }
            for (int r = col + 1; r < k; ++r) {
                const double factor = m[r][col] / m[col][col];
                for (int c = col; c < k; ++c) m[r][c] -= factor * m[col][c];
                m[r][k] -= factor * m[col][k];
            }
        }
        if (singular) continue;
        double x[T];
        for (int r = k - 1; r >= 0; --r) {
            double v = m[r][k];
            for (int c = r + 1; c < k; ++c) v -= m[r][c] * x[c];
            x[r] = v / m[r][r];
        }
        for (int r = 0; r < k; ++r) {
            if (!isfinite(x[r])) {
                *failed = 1;
                return;
            }
            coef[r] = x[r];
        }
        *have = 1;
        return;
    }
    *failed = 1;
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

}  // namespace
}  // namespace kgpu
