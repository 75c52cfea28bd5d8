// TEST INFRASTRUCTURE -- FP64 CPU oracle of least-squares Monte Carlo (Longstaff-Schwartz).
//
// BSM, quadratic basis: restates MonteCarloVanillaEngine::american_scenarios for one
// contract in its forward (non-reverse, normalized) mode, crates/kiyosi/src/engines/
// monte_carlo/american.rs:955-1455, with solve_quadratic (1693-1749): cumulative
// Brownian coordinates per path from the block streams, spots reconstructed per date
// as S0 exp(drift (k+1)) exp(diffusion W_k), in-the-money regression of discounted cash
// on {1, S/K, (S/K)^2} merged in block order, exercise when intrinsic/K > continuation.
//
// Heston, cubic basis: the same backward induction on full-truncation Euler paths
// (`substeps` Euler steps per exercise interval, two normals per step: spot, then the
// independent variance shock), with the ten monomials of degree <= 3 in (S/K, v/theta)
// and the same pivoted elimination with degree fallback (3 -> 2 -> 1 -> 0).  The
// reference has no Heston Monte Carlo; this follows its LSMC method on a new model.
//
// Only tests, the smoke check and bench.py's CPU leg use this file.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <thread>
#include <vector>

#include "../include/kgpu.h"
#include "oracle_core.h"

namespace kor {
namespace {

template <class F>
void parallel_blocks(size_t blocks, int threads, F&& f) {
    if (threads <= 0) threads = int(std::max(1u, std::thread::hardware_concurrency()));
    threads = int(std::min<size_t>(size_t(threads), std::max<size_t>(blocks, 1)));
    if (threads <= 1) {
        for (size_t b = 0; b < blocks; ++b) f(b);
        return;
    }
    size_t chunk = (blocks + threads - 1) / threads;
    std::vector<std::thread> pool;
    for (int t = 0; t < threads; ++t) {
        size_t begin = size_t(t) * chunk, end = std::min(blocks, begin + chunk);
        if (begin >= end) break;
        pool.emplace_back([&, begin, end]() {
            for (size_t b = begin; b < end; ++b) f(b);
        });
    }
    for (auto& th : pool) th.join();
}

// Number of basis terms by degree for one and two variables.
int terms(int degree, bool two) {
    if (!two) return degree + 1;
    return (degree + 1) * (degree + 2) / 2;
}

// Monomials of degree <= 3 in (x, y), graded: 1, x, y, x2, xy, y2, x3, x2y, xy2, y3.
void basis(double x, double y, bool two, double* out) {
    if (!two) {
        out[0] = 1.0;
        out[1] = x;
        out[2] = x * x;
        out[3] = x * x * x;
        return;
    }
    out[0] = 1.0;
    out[1] = x;
    out[2] = y;
    out[3] = x * x;
    out[4] = x * y;
    out[5] = y * y;
    out[6] = x * x * x;
    out[7] = x * x * y;
    out[8] = x * y * y;
    out[9] = y * y * y;
}

// Pivoted Gaussian elimination of the normal equations with degree fallback, as
// solve_quadratic (american.rs:1693-1749): a pivot at or below 1e-14 times the largest
// entry of the truncated system drops one degree.  `a` is k x (k+1), row-major, with
// k = terms(max_degree).  Returns the number of coefficients solved (0 on failure).
int solve(const std::vector<double>& sums, int max_degree, bool two, double* coef) {
    const int kmax = terms(max_degree, two);
    for (int degree = max_degree; degree >= 0; --degree) {
        const int k = terms(degree, two);
        std::vector<double> m(size_t(k) * (k + 1));
        for (int r = 0; r < k; ++r) {
            for (int c = 0; c < k; ++c) m[size_t(r) * (k + 1) + c] = sums[size_t(r) * (kmax + 1) + c];
            m[size_t(r) * (k + 1) + k] = sums[size_t(r) * (kmax + 1) + kmax];
        }
        double scale = 0.0;
        for (int r = 0; r < k; ++r)
            for (int c = 0; c < k; ++c) scale = std::max(scale, std::fabs(m[size_t(r) * (k + 1) + c]));
        bool singular = false;
        for (int col = 0; col < k; ++col) {
            // max_by with total_cmp keeps the last of equal maxima
            int pivot = col;
            for (int r = col + 1; r < k; ++r)
                if (std::fabs(m[size_t(r) * (k + 1) + col]) >= std::fabs(m[size_t(pivot) * (k + 1) + col])) pivot = r;
            double pv = m[size_t(pivot) * (k + 1) + col];
            if (!std::isfinite(pv)) return 0;
            if (std::fabs(pv) <= 1e-14 * scale) {
                singular = true;
                break;
            }
            if (pivot != col)
                for (int c = 0; c <= k; ++c)
                    std::swap(m[size_t(col) * (k + 1) + c], m[size_t(pivot) * (k + 1) + c]);
            for (int r = col + 1; r < k; ++r) {
                double factor = m[size_t(r) * (k + 1) + col] / m[size_t(col) * (k + 1) + col];
                for (int c = col; c < k; ++c) m[size_t(r) * (k + 1) + c] -= factor * m[size_t(col) * (k + 1) + c];
                m[size_t(r) * (k + 1) + k] -= factor * m[size_t(col) * (k + 1) + k];
            }
        }
        if (singular) continue;
        for (int r = k - 1; r >= 0; --r) {
            double v = m[size_t(r) * (k + 1) + k];
            for (int c = r + 1; c < k; ++c) v -= m[size_t(r) * (k + 1) + c] * coef[c];
            coef[r] = v / m[size_t(r) * (k + 1) + r];
        }
        for (int r = 0; r < k; ++r)
            if (!std::isfinite(coef[r])) return 0;
        for (int r = k; r < kmax; ++r) coef[r] = 0.0;
        return k;
    }
    return 0;
}

struct Problem {
    const kgpu_model* m;
    double strike, sign, expiry;
    int dates, substeps, paths;
    bool heston, two;
    int max_degree;
    double dt_date, discount;  // per exercise interval
    double drift, diffusion;   // BSM per interval
    double y_scale;            // 1/theta for the Heston basis
};

// Forward pass: per path, state at each exercise date.  BSM stores the Brownian
// coordinate (sum of normals), Heston stores log(S/S0) and v.  Layout [date][path].
void simulate(const Problem& p, uint64_t seed, int threads, std::vector<double>& a, std::vector<double>& b) {
    const int n = p.dates, paths = p.paths;
    a.assign(size_t(n) * paths, 0.0);
    if (p.heston) b.assign(size_t(n) * paths, 0.0);
    size_t blocks = size_t((paths + kBlockSize - 1) / kBlockSize);
    const kgpu_model* m = p.m;
    const double h = p.dt_date / p.substeps, sq = std::sqrt(h);
    const double rho_bar = std::sqrt(1.0 - m->rho * m->rho);
    parallel_blocks(blocks, threads, [&](size_t blk) {
        BlockDraws draws(seed, blk, nullptr);
        const int first = int(blk) * kBlockSize;
        const int last = std::min(first + kBlockSize, paths);
        for (int path = first; path < last; ++path) {
            if (!p.heston) {
                double w = 0.0;
                for (int k = 0; k < n; ++k) {
                    w += draws.normal();
                    a[size_t(k) * paths + path] = w;
                }
            } else {
                double x = 0.0, v = m->v0;
                for (int k = 0; k < n; ++k) {
                    for (int j = 0; j < p.substeps; ++j) {
                        double z1 = draws.normal(), z2 = draws.normal();
                        double vp = v > 0.0 ? v : 0.0;
                        double sv = std::sqrt(vp) * sq;
                        x += (m->rate - m->dividend - 0.5 * vp) * h + sv * z1;
                        v += m->kappa * (m->theta - vp) * h + m->xi * sv * (m->rho * z1 + rho_bar * z2);
                    }
                    a[size_t(k) * paths + path] = x;
                    b[size_t(k) * paths + path] = v;
                }
            }
            draws.skip(0);
        }
    });
}

inline double spot_of(const Problem& p, int k, double a) {
    if (!p.heston) return p.m->spot * std::exp(p.drift * double(k + 1)) * std::exp(p.diffusion * a);
    return p.m->spot * std::exp(a);
}

inline double payoff(const Problem& p, double spot) {
    double v = p.sign * (spot - p.strike);
    return v > 0.0 ? v : 0.0;
}

double continuation(const Problem& p, const double* coef, double x, double y) {
    double f[10];
    basis(x, y, p.two, f);
    int k = terms(p.max_degree, p.two);
    double c = 0.0;
    for (int i = 0; i < k; ++i) c += coef[i] * f[i];
    return c;
}

}  // namespace
}  // namespace kor

using namespace kor;

extern "C" int kor_lsmc_price(const kgpu_model* model, double strike, double sign, double expiry,
                              const kgpu_lsmc_settings* settings, uint64_t fresh_seed,
                              kgpu_lsmc_result* out, int threads) {
    Problem p;
    p.m = model;
    p.strike = strike;
    p.sign = sign;
    p.expiry = expiry;
    p.dates = settings->exercise_dates;
    p.substeps = settings->substeps > 0 ? settings->substeps : 1;
    p.paths = settings->path_count;
    p.heston = model->kind == KGPU_MODEL_HESTON;
    p.two = p.heston;
    p.max_degree = p.heston ? 3 : 2;
    if (p.dates < 2 || p.paths < 1) return KGPU_INVALID_INPUT;
    p.dt_date = expiry / p.dates;
    p.discount = std::exp(-model->rate * p.dt_date);
    p.drift = (model->rate - model->dividend - 0.5 * model->volatility * model->volatility) * p.dt_date;
    p.diffusion = model->volatility * std::sqrt(p.dt_date);
    p.y_scale = (p.heston && model->theta > 0.0) ? 1.0 / model->theta : 1.0;
    const int n = p.dates, paths = p.paths;
    const int k = terms(p.max_degree, p.two);
    std::vector<double> a, b;
    simulate(p, settings->seed, threads, a, b);
    auto state = [&](int date, int path, double* spot, double* y) {
        double s = spot_of(p, date, a[size_t(date) * paths + path]);
        *spot = s;
        *y = p.heston ? b[size_t(date) * paths + path] * p.y_scale : 0.0;
    };
    std::vector<double> cash(paths);
    for (int i = 0; i < paths; ++i) {
        double s, y;
        state(n - 1, i, &s, &y);
        cash[i] = payoff(p, s);
    }
    std::vector<double> coefs(size_t(n) * 10, 0.0);
    std::vector<int> have(n, 0);
    std::vector<double> sums(size_t(k) * (k + 1));
    size_t blocks = size_t((paths + kBlockSize - 1) / kBlockSize);
    std::vector<std::vector<double>> partial(blocks, std::vector<double>(size_t(k) * (k + 1)));
    for (int date = n - 2; date >= 0; --date) {
        const double* next_coef = &coefs[size_t(date + 1) * 10];
        const bool decide = date + 1 <= n - 2 && have[date + 1];
        parallel_blocks(blocks, threads, [&](size_t blk) {
            std::vector<double>& acc = partial[blk];
            std::fill(acc.begin(), acc.end(), 0.0);
            const int first = int(blk) * kBlockSize, last = std::min(first + kBlockSize, paths);
            double f[10];
            for (int i = first; i < last; ++i) {
                double s, y;
                if (decide) {
                    state(date + 1, i, &s, &y);
                    double intrinsic = payoff(p, s);
                    if (intrinsic > 0.0 && intrinsic / p.strike > continuation(p, next_coef, s / p.strike, y))
                        cash[i] = intrinsic;
                }
                cash[i] *= p.discount;
                state(date, i, &s, &y);
                if (payoff(p, s) > 0.0) {
                    basis(s / p.strike, y, p.two, f);
                    double target = cash[i] / p.strike;
                    for (int r = 0; r < k; ++r) {
                        for (int c = 0; c < k; ++c) acc[size_t(r) * (k + 1) + c] += f[r] * f[c];
                        acc[size_t(r) * (k + 1) + k] += f[r] * target;
                    }
                }
            }
        });
        std::fill(sums.begin(), sums.end(), 0.0);
        for (auto& acc : partial)
            for (size_t j = 0; j < sums.size(); ++j) sums[j] += acc[j];
        if (sums[0] != 0.0) {
            int solved = solve(sums, p.max_degree, p.two, &coefs[size_t(date) * 10]);
            if (solved == 0) return KGPU_COMPUTATION_FAILURE;
            have[date] = 1;
        }
    }
    // Date 0 decision, then one more interval of discounting to the valuation time.
    Moments mean;
    for (int i = 0; i < paths; ++i) {
        double s, y;
        if (have[0]) {
            state(0, i, &s, &y);
            double intrinsic = payoff(p, s);
            if (intrinsic > 0.0 && intrinsic / p.strike > continuation(p, &coefs[0], s / p.strike, y))
                cash[i] = intrinsic;
        }
        mean.add(cash[i], true);
    }
    const double immediate = payoff(p, model->spot);
    out->price = std::max(immediate, discounted_product(mean.scale, mean.mean, -model->rate * p.dt_date));
    out->standard_error =
        paths > 1 ? discounted_product(mean.scale, std::sqrt(mean.m2 / double(paths - 1) / double(paths)),
                                       -model->rate * p.dt_date)
                  : 0.0;
    out->out_of_sample = std::nan("");
    out->out_of_sample_error = std::nan("");
    if (fresh_seed != settings->seed) {
        // Lower bound: the fitted policy applied forward on fresh paths
        // (price_american_out_of_sample, american.rs:574-637).
        std::vector<double> fa, fb;
        simulate(p, fresh_seed, threads, fa, fb);
        Moments lower;
        for (int i = 0; i < paths; ++i) {
            double value = 0.0;
            for (int date = 0; date < n; ++date) {
                double s = spot_of(p, date, fa[size_t(date) * paths + i]);
                double y = p.heston ? fb[size_t(date) * paths + i] * p.y_scale : 0.0;
                double intrinsic = payoff(p, s);
                bool last = date == n - 1;
                if (intrinsic > 0.0 &&
                    (last || (have[date] && intrinsic / p.strike >
                                                continuation(p, &coefs[size_t(date) * 10], s / p.strike, y)))) {
                    value = intrinsic * std::exp(-model->rate * p.dt_date * double(date + 1));
                    break;
                }
            }
            lower.add(value, true);
        }
        out->out_of_sample = std::max(immediate, lower.scale * lower.mean);
        out->out_of_sample_error =
            paths > 1 ? lower.scale * std::sqrt(lower.m2 / double(paths - 1) / double(paths)) : 0.0;
    }
    out->wall_ms = out->path_store_ms = out->regression_ms = 0.0;
    return KGPU_OK;
}
