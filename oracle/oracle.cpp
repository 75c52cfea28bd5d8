// TEST INFRASTRUCTURE -- FP64 CPU oracle for kiyosi's Monte Carlo hot path.
//
// Restates the reference engines (kiyosi 0.23.0, paths inside crates/kiyosi/src) on the
// plan structs of include/kgpu.h.  Used only by tests/, the smoke check and the CPU
// baseline of bench.py; the product never links it.  Build with -ffp-contract=off.
#include "oracle_core.h"

#include <algorithm>
#include <array>
#include <atomic>
#include <cstring>
#include <limits>
#include <memory>
#include <mutex>
#include <thread>

#include "../include/kgpu.h"

namespace kor {

#include "../kiyosi_gb300/csrc/joe_kuo_6_21201.inc"

const uint32_t* joe_kuo_table() { return kgpu_joe_kuo_table; }

// --------------------------------------------------------------------------------------
// Cephes ndtri (engines/monte_carlo/sobol.rs:253-346; Cephes by S. L. Moshier).
// --------------------------------------------------------------------------------------
static double poly(double value, const double* c, int n, double leading) {
    double r = leading;
    for (int i = 0; i < n; ++i) r = r * value + c[i];
    return r;
}

double inverse_normal_cdf(double probability) {
    static const double P0[] = {-59.96335010141079, 98.00107541859997, -56.67628574690703,
                                13.931260938727968, -1.2391658386738125};
    static const double Q0[] = {1.9544885833814176, 4.676279128988815,  86.36024213908905,
                                -225.46268785411937, 200.26021238006066, -82.03722561683334,
                                15.90562251262117,   -1.1833162112133};
    static const double P1[] = {4.0554489230596245,  31.525109459989388,  57.16281922464213,
                                44.08050738932008,   14.684956192885803,  2.1866330685079025,
                                -0.1402560791713545, -0.03504246268278482,
                                -0.0008574567851546854};
    static const double Q1[] = {15.779988325646675,   45.39076351288792,   41.3172038254672,
                                15.04253856929075,    2.504649462083094,   -0.14218292285478779,
                                -0.03808064076915783, -0.0009332594808954574};
    static const double P2[] = {3.2377489177694603,     6.915228890689842,
                                3.9388102529247444,     1.3330346081580755,
                                0.20148538954917908,    0.012371663481782003,
                                0.00030158155350823543, 2.6580697468673755e-06,
                                6.239745391849833e-09};
    static const double Q2[] = {6.02427039364742,      3.6798356385616087,
                                1.3770209948908132,    0.21623699359449663,
                                0.013420400608854318,  0.00032801446468212774,
                                2.8924786474538068e-06, 6.790194080099813e-09};
    const double tail_boundary = 0.1353352832366127;
    bool upper = probability > 1.0 - tail_boundary;
    double tail = upper ? 1.0 - probability : probability;
    if (tail > tail_boundary) {
        double centered = tail - 0.5;
        double square = centered * centered;
        return (centered + centered * square * poly(square, P0, 5, 0.0) / poly(square, Q0, 8, 1.0)) *
               std::sqrt(2.0 * 3.141592653589793);
    }
    double root = std::sqrt(-2.0 * std::log(tail));
    double inverse = 1.0 / root;
    double correction = inverse * (root < 8.0 ? poly(inverse, P1, 9, 0.0) / poly(inverse, Q1, 8, 1.0)
                                              : poly(inverse, P2, 9, 0.0) / poly(inverse, Q2, 8, 1.0));
    double quantile = root - std::log(root) / root - correction;
    return upper ? quantile : -quantile;
}

// --------------------------------------------------------------------------------------
// SobolSequence::new (sobol.rs:85-134)
// --------------------------------------------------------------------------------------
SobolSequence::SobolSequence(int dims, uint64_t seed) : dimensions(dims) {
    directions.assign(size_t(dims) * kSobolBits, 0);
    shifts.resize(dims);
    const uint32_t* polynomial = kgpu_joe_kuo_table;
    for (int dimension = 0; dimension < dims; ++dimension) {
        uint64_t raw[kSobolBits];
        if (dimension == 0) {
            for (int column = 0; column < kSobolBits; ++column)
                raw[column] = uint64_t(1) << (kSobolBits - column - 1);
        } else {
            int degree = int(polynomial[0]);
            uint32_t coefficients = polynomial[1];
            for (int column = 0; column < degree; ++column)
                raw[column] = uint64_t(polynomial[column + 2]) << (kSobolBits - column - 1);
            polynomial += degree + 2;
            for (int column = degree; column < kSobolBits; ++column) {
                uint64_t direction = raw[column - degree] ^ (raw[column - degree] >> degree);
                for (int offset = 1; offset < degree; ++offset)
                    if ((coefficients >> (degree - offset - 1)) & 1) direction ^= raw[column - offset];
                raw[column] = direction;
            }
        }
        Pcg32 generator(seed, uint64_t(dimension));
        auto word = [&]() {
            uint64_t hi = generator.next();
            uint64_t lo = generator.next();
            return (hi << 32) | lo;
        };
        shifts[dimension] = word() & kSobolMask;
        uint64_t matrix[kSobolBits];
        for (int row = 0; row < kSobolBits; ++row) {
            int bit = kSobolBits - row - 1;
            matrix[row] = (word() & (kSobolMask << (bit + 1))) | (uint64_t(1) << bit);
        }
        for (int column = 0; column < kSobolBits; ++column) {
            uint64_t scrambled = 0;
            for (int row = 0; row < kSobolBits; ++row)
                scrambled |= uint64_t(__builtin_popcountll(raw[column] & matrix[row]) & 1)
                             << (kSobolBits - row - 1);
            directions[size_t(column) * dims + dimension] = scrambled;
        }
    }
}

// --------------------------------------------------------------------------------------
// Worker pool over fixed blocks, merged in block order (monte_carlo.rs:1914-1997).
// --------------------------------------------------------------------------------------
template <class F>
static void run_blocks(size_t blocks, int threads, F&& simulate) {
    if (threads <= 0) threads = int(std::max(1u, std::thread::hardware_concurrency()));
    threads = int(std::min<size_t>(size_t(threads), blocks));
    if (threads <= 1) {
        for (size_t b = 0; b < blocks; ++b) simulate(b);
        return;
    }
    // Contiguous chunks, one per worker, as par_chunks_mut does.
    size_t chunk = (blocks + threads - 1) / threads;
    std::vector<std::thread> pool;
    for (int t = 0; t < threads; ++t) {
        size_t begin = size_t(t) * chunk, end = std::min(blocks, begin + chunk);
        if (begin >= end) break;
        pool.emplace_back([&, begin, end]() {
            for (size_t b = begin; b < end; ++b) simulate(b);
        });
    }
    for (auto& th : pool) th.join();
}

// --------------------------------------------------------------------------------------
// Path normals of one sample: lazy draws with skip (LazyPath / SkippingPath,
// monte_carlo.rs:1621-1676) or the eager buffer of an antithetic pair.
// --------------------------------------------------------------------------------------
struct PathNormals {
    BlockDraws* draws;
    const double* cache;  // antithetic pair: all dimensions drawn eagerly
    int used = 0;
    double sign = 1.0;
    double normal() {
        double z = cache ? cache[used] : draws->normal();
        ++used;
        return sign * z;
    }
    void skip(int count) {
        if (count <= 0) return;
        if (!cache) draws->skip(uint64_t(count));
        used += count;
    }
};

struct Failure {
    bool failed = false;
};

static inline double spot_at(double initial, double log_return) {
    return discounted_product(initial, 1.0, log_return);  // scaled_value(initial, 1, lr)
}

// Local volatility lookup (market/local_volatility.rs:322-359).
struct LocalVol {
    int nt = 0, ns = 0;
    const double* times = nullptr;
    const double* spots = nullptr;
    const double* values = nullptr;
    std::vector<double> years;
    static void bracket(const double* nodes, int n, double value, int* left, double* weight) {
        int count = int(std::upper_bound(nodes, nodes + n, value) - nodes);  // partition_point(<=)
        int l = std::min(std::max(count - 1, 0), n - 2);
        double w = (value - nodes[l]) / (nodes[l + 1] - nodes[l]);
        *left = l;
        *weight = std::min(std::max(w, 0.0), 1.0);
    }
    static double interpolate(double low, double high, double weight) {
        return weight <= 0.5 ? low + weight * (high - low) : high + (1.0 - weight) * (low - high);
    }
    double at(double time, double spot) const {
        int row, column;
        double tw, sw;
        bracket(years.data(), nt, time, &row, &tw);
        bracket(spots, ns, spot, &column, &sw);
        const double* r0 = values + size_t(row) * ns;
        const double* r1 = values + size_t(row + 1) * ns;
        return interpolate(interpolate(r0[column], r0[column + 1], sw),
                           interpolate(r1[column], r1[column + 1], sw), tw);
    }
};

struct Model {
    const kgpu_model* m;
    LocalVol lv;
    explicit Model(const kgpu_model* model) : m(model) {
        if (m->kind == KGPU_MODEL_LOCAL_VOL) {
            lv.nt = m->lv_time_count;
            lv.ns = m->lv_spot_count;
            lv.times = m->lv_times;
            lv.spots = m->lv_spots;
            lv.values = m->lv_values;
            lv.years.resize(lv.nt);
            for (int i = 0; i < lv.nt; ++i) lv.years[i] = lv.times[i] - lv.times[0];
        }
    }
    int normals_per_step() const { return m->kind == KGPU_MODEL_HESTON ? 2 : 1; }
};

// One grid step of the state (log return relative to the valuation spot, variance).
// BSM: the reference's `log_return += diffusion.mul_add(normal, drift)`.
// Heston: full-truncation Euler in log spot; local vol: Euler in log spot with the
// surface read at the step's start.
struct State {
    double lr = 0.0;
    double v = 0.0;
};

static inline void step_state(const Model& model, const kgpu_step& st, State& s, PathNormals& n) {
    const kgpu_model* m = model.m;
    if (m->kind == KGPU_MODEL_BSM) {
        s.lr += std::fma(st.diffusion, n.normal(), st.drift);
    } else if (m->kind == KGPU_MODEL_HESTON) {
        double z1 = n.normal();
        double z2 = n.normal();
        double dt = st.drift, sq = st.diffusion;
        double vp = s.v > 0.0 ? s.v : 0.0;
        double sv = std::sqrt(vp) * sq;
        double zv = m->rho * z1 + std::sqrt(1.0 - m->rho * m->rho) * z2;
        s.lr += (m->rate - m->dividend - 0.5 * vp) * dt + sv * z1;
        s.v += m->kappa * (m->theta - vp) * dt + m->xi * sv * zv;
    } else {
        double spot = m->spot * std::exp(s.lr);
        double sigma = model.lv.at(st.time, spot);
        double dt = st.drift, sq = st.diffusion;
        s.lr += (m->rate - m->dividend - 0.5 * sigma * sigma) * dt + sigma * sq * n.normal();
    }
}

// --------------------------------------------------------------------------------------
// Payoff families on one path.
// --------------------------------------------------------------------------------------
struct Plan {
    const kgpu_book* book;
    const kgpu_contract* c;
    const kgpu_step* steps;
    const uint8_t* flags;
    const kgpu_event* events;
    const kgpu_bridge_interval* intervals;
    const kgpu_bridge_daily* daily;
};

// TerminalPayoff::at_normal (monte_carlo.rs:1238-1251)
static double european_payoff(const kgpu_contract* c, double z, Failure& f) {
    double distance = std::fma(c->diffusion, z, c->moneyness);
    double payoff;
    if (c->sign * distance <= 0.0)
        payoff = 0.0;
    else if (c->sign < 0.0)
        payoff = -std::expm1(distance);
    else
        payoff = -std::expm1(-distance) * std::exp(std::fma(c->diffusion, z, -c->half_variance));
    if (!std::isfinite(payoff)) f.failed = true;
    return payoff;
}

// The sample a path reports: its payoff, or its native delta or gamma sample.
static int output_of(const kgpu_contract* c) {
    return (c->flags & KGPU_C_OUTPUT_DELTA) ? 1 : ((c->flags & KGPU_C_OUTPUT_GAMMA) ? 2 : 0);
}

// Digital terminal payoff (digital.rs:111-140): moneyness = d2, diffusion = width,
// log_scale = exponent offset, strike = paid amount; with the likelihood-ratio delta
// and gamma samples of the same normal.
static double digital_payoff(const kgpu_contract* c, double z) {
    double distance = c->moneyness + z;
    bool call = c->sign > 0.0;
    if (!(call ? distance > 0.0 : distance < 0.0)) return 0.0;
    double exponent = c->log_scale + ((c->flags & KGPU_C_ASSET_DIGITAL) ? c->diffusion * z : 0.0);
    const int output = output_of(c);
    if (output == 0) return discounted_product(c->strike, 1.0, exponent);
    const double log_payoff = c->greek_log_amount + exponent;
    if (output == 1)
        return z != 0.0 ? std::copysign(std::exp(log_payoff + std::log(std::fabs(z)) - c->greek_log_spot -
                                                 c->greek_log_width),
                                        z)
                        : 0.0;
    const double score = std::fma(-c->diffusion, z, z * z - 1.0);
    return score != 0.0 ? std::copysign(std::exp(log_payoff + std::log(std::fabs(score)) - 2.0 * c->greek_log_spot -
                                                 2.0 * c->greek_log_width),
                                        score)
                        : 0.0;
}

// The barrier sampler's delta and gamma from the first normal's score plus the survival
// weight's spot derivatives (barrier.rs:455-470).
static double barrier_greek(int output, double value, double first, double second, double z, double width,
                            double spot) {
    const double score = z / width;
    if (output == 1) return (value * score + first) / spot;
    const double second_score = ((z * z - 1.0) / width - z) / width;
    return ((value * second_score + first * (2.0 * score - 1.0) + second) / spot) / spot;
}

// The `weighted` helper of the barrier sampler (barrier.rs:328-330):
// scaled_value(|amount|, signum(amount), log_weight).
static double weighted(double amount, double log_weight) {
    return discounted_product(std::fabs(amount), std::signbit(amount) ? -1.0 : 1.0, log_weight);
}

// Continuously monitored single barrier (barrier.rs:306-452), one terminal draw.
static double barrier_payoff(const kgpu_contract* c, double z, Failure& f) {
    const double noise = std::fma(c->diffusion, z, 0.0);
    const double terminal = c->barrier_drift + noise;
    const double asset = discounted_product(c->spot, 1.0, terminal);
    if (!std::isfinite(asset)) f.failed = true;
    const double distance = c->moneyness + noise;
    const double payoff = std::fabs(distance) < 0.5 ? c->strike * std::expm1(distance) : asset - c->strike;
    const double intrinsic = std::max(c->sign * payoff, 0.0);
    const double to_barrier = c->barrier_moneyness + noise;
    const bool up = c->flags & KGPU_C_BARRIER_UP;
    const bool in = c->flags & KGPU_C_BARRIER_IN;
    const bool live = up ? to_barrier < 0.0 : to_barrier > 0.0;
    const double slope = live ? 2.0 * (std::fabs(to_barrier) / c->diffusion) / c->diffusion : 0.0;
    const double exponent = -c->barrier_distance * slope;
    const double survival = live ? std::log(-std::expm1(exponent)) : -INFINITY;
    const double value = weighted(intrinsic, c->log_discount + (in ? exponent : survival)) +
                         weighted(c->rebate, c->log_discount + (in ? survival : exponent));
    if (!std::isfinite(value)) f.failed = true;
    const int output = output_of(c);
    if (output == 0) return value;
    double first = 0.0, second = 0.0;
    if (slope > 0.0 && exponent > -INFINITY) {
        const double difference = (in ? -1.0 : 1.0) * (intrinsic - c->rebate);
        first = weighted(up ? -difference : difference, c->log_discount + (exponent + std::log(slope)));
        if (output == 2) second = weighted(-difference, c->log_discount + (exponent + 2.0 * std::log(slope)));
    }
    const double greek = barrier_greek(output, value, first, second, z, c->diffusion, c->spot);
    if (!std::isfinite(greek)) f.failed = true;
    return greek;
}

// normal_cdf, log_normal_cdf, log_normal_tail and weighted_cdf (numerics.rs:192-224).
static double normal_cdf(double x) { return 0.5 * std::erfc(-x * 0.70710678118654752440); }

static double log_normal_cdf(double x) {
    if (x >= -10.0) return std::log(normal_cdf(x));
    const double inverse_square = (1.0 / x) / x;
    double term = 1.0, sum = 1.0;
    for (int k = 1; k <= 20; ++k) {
        term *= -double(2 * k - 1) * inverse_square;
        sum += term;
    }
    return -0.5 * x * x - std::log(-x) + std::log(sum / std::sqrt(2.0 * M_PI));
}

static double weighted_cdf(double amount, double exponent, double argument) {
    const double discount = std::exp(exponent);
    const double discounted = amount * discount;
    if (argument < -10.0 || !std::isnormal(discount) || !std::isfinite(discounted))
        return std::exp(std::log(amount) + exponent + log_normal_cdf(argument));
    return discounted * normal_cdf(argument);
}

// lognormal_price (engines/analytic/european.rs:317-403), the branch for widths of at
// least 1e-5 (plans with narrower conditioned widths are rejected before sampling).
static double lognormal_price(double spot, double strike, double log_moneyness, double asset_log,
                              double risk_log, double volatility, double root_time, double sign,
                              Failure& f) {
    const double width = volatility * root_time;
    if (!(width >= 1e-5)) {
        f.failed = true;
        return 0.0;
    }
    const double standardized = log_moneyness / width;
    const double d1 = standardized + 0.5 * width, d2 = standardized - 0.5 * width;
    const double asset = weighted_cdf(spot, asset_log, sign * d1);
    const double cash = weighted_cdf(strike, risk_log, sign * d2);
    const double direct = sign * (asset - cash);
    if (std::isfinite(direct)) return direct;
    const double la = log_moneyness + log_normal_cdf(sign * d1), lc = log_normal_cdf(sign * d2);
    const double hi = sign > 0.0 ? la : lc, lo = sign > 0.0 ? lc : la;
    const double difference = hi == -INFINITY ? -INFINITY : hi + std::log(-std::expm1(lo - hi));
    const double value = std::exp(std::log(strike) + risk_log + difference);
    if (!std::isfinite(value)) f.failed = true;
    return value;
}

// Scheduled single barrier (barrier.rs:240-449 without Greeks): one normal per date,
// noise = sum(width z) against each observed date's touch level; a knock-out stops at the
// hit with its rebate; a knock-in hit with more than 8 dates left is priced analytically
// from the hit (`condition_on_hit`); otherwise the expiry payoff or the expiry rebate.
static double barrier_discrete_payoff(const Plan& p, PathNormals& n, Failure& f) {
    const kgpu_contract* c = p.c;
    const bool up = c->flags & KGPU_C_BARRIER_UP;
    const bool in = c->flags & KGPU_C_BARRIER_IN;
    const bool condition = c->flags & KGPU_C_CONDITION_ON_HIT;
    double noise = 0.0, terminal = 0.0, first_normal = 0.0;
    bool touched = false;
    const int output = output_of(c);
    // The delta / gamma samples score the first normal (barrier.rs:455-470).
    auto finish = [&](double value) {
        return output == 0 ? value
                           : barrier_greek(output, value, 0.0, 0.0, first_normal, p.steps[0].diffusion, c->spot);
    };
    for (int i = 0; i < c->step_count; ++i) {
        const kgpu_step& st = p.steps[i];
        const kgpu_event& e = p.events[i];
        const double z = n.normal();
        if (i == 0) first_normal = z;
        noise = std::fma(st.diffusion, z, noise);
        terminal = st.drift + noise;
        if (c->flags & KGPU_C_CHECK_STEPS) {
            const double spot_now = discounted_product(c->spot, 1.0, terminal);
            if (!std::isfinite(spot_now) || spot_now <= 0.0) {
                f.failed = true;
                return 0.0;
            }
        }
        const bool touch = (c->flags & KGPU_C_DOUBLE) ? (noise <= e.knock_out || noise >= e.payment[3])
                                                       : (up ? noise >= e.knock_out : noise <= e.knock_out);
        if (e.has_knock_out && touch) {
            touched = true;
            if (condition && c->step_count - i > 8) {
                const double asset = discounted_product(c->spot, 1.0, terminal);
                return finish(lognormal_price(asset, c->strike,
                                              c->moneyness + noise + c->half_variance * e.coupon_barrier,
                                              e.payment[1], c->log_discount, c->volatility, e.payment[2], c->sign, f));
            }
        }
        if (touched && !in) {
            const double rebate =
                discounted_product(c->rebate, 1.0, (c->flags & KGPU_C_REBATE_AT_HIT) ? e.payment[0] : c->log_discount);
            if (!std::isfinite(rebate)) f.failed = true;
            return finish(rebate);
        }
    }
    const double asset = discounted_product(c->spot, 1.0, terminal);
    if (!std::isfinite(asset)) f.failed = true;
    const double distance = c->moneyness + noise;
    const double payoff = std::fabs(distance) < 0.5 ? c->strike * std::expm1(distance) : asset - c->strike;
    const double intrinsic = std::max(c->sign * payoff, 0.0);
    const double value = weighted(touched == in ? intrinsic : c->rebate, c->log_discount);
    if (!std::isfinite(value)) f.failed = true;
    return finish(value);
}

// log_add (numerics.rs:320-327).
static double log_add(double a, double b) {
    const double high = std::max(a, b);
    if (high == -INFINITY) return high;
    return high + std::log1p(std::exp(-std::fabs(a - b)));
}

// positive_difference (asian.rs:972-985): exp(a) - exp(b), floored at zero.
static double positive_difference(double a, double b) {
    if (a == INFINITY) return a;
    if (b == -INFINITY) return std::exp(a);
    const double difference = -std::expm1(b - a);
    return difference > 0.0 ? std::exp(a + std::log(difference)) : 0.0;
}

// ArithmeticParameters::geometric_values (asian.rs:1062-1085): the geometric
// control's [price, delta, gamma].
static void geometric_values(const kgpu_contract* c, double log_forward, double log_strike, double width,
                             double out[3]) {
    const double d1 = (log_forward - log_strike) / width + 0.5 * width;
    const double d2 = d1 - width;
    const double log_asset = log_forward + c->log_discount + log_normal_cdf(c->sign * d1);
    const double log_cash = log_strike + c->log_discount + log_normal_cdf(c->sign * d2);
    out[0] = c->sign > 0.0 ? positive_difference(log_asset, log_cash) : positive_difference(log_cash, log_asset);
    const double log_spot = c->avg_log_spot;
    out[1] = c->sign * std::exp(log_asset - log_spot);
    out[2] = std::exp(log_forward + c->log_discount - 2.0 * log_spot - std::log(width) - 0.5 * d1 * d1 -
                      0.5 * std::log(2.0 * M_PI));
}

// Continuous arithmetic average (asian.rs:636-711 ArithmeticGrid::path, then
// 1087-1178 ArithmeticParameters::arithmetic), flat rates, no realized history,
// interval widths of at least 1e-5 (plans reject narrower ones): the price or its native
// delta / gamma sample.
static double average_arithmetic_payoff(const kgpu_contract* c, PathNormals& n, Failure& f) {
    const bool lead = c->flags & KGPU_C_AVERAGE_LEAD;
    const bool control = c->flags & KGPU_C_AVERAGE_CONTROL;
    const int output = output_of(c);
    const int normals = c->step_count - (lead ? 1 : 0);  // step_count (n) - 1 increments
    const double lead_normal = lead ? n.normal() : 0.0;
    const double lead_growth = c->avg_lead_drift + c->avg_lead_width * lead_normal;
    double growth = 0.0, relative_sum = 0.0, log_sum = -INFINITY, geometric_growth = 0.0;
    for (int index = 0; index < normals; ++index) {
        const double normal = n.normal();
        growth += c->avg_drift + c->avg_width * normal;
        const bool last = index + 1 == normals;
        const double fraction = last ? c->avg_half : c->avg_fraction;
        if (control) geometric_growth += fraction * growth;
        if (growth > 600.0 || log_sum != -INFINITY) {
            if (log_sum == -INFINITY) log_sum = std::log(c->avg_rest + relative_sum);
            log_sum = log_add(log_sum, (last ? c->avg_log_half : c->avg_log_fraction) + growth);
        } else {
            relative_sum += fraction * std::expm1(growth);
        }
    }
    const double log_spot = c->avg_log_spot;
    const double log_rest =
        log_sum == -INFINITY ? c->avg_log_rest + std::log1p(relative_sum / c->avg_rest) : log_sum;
    const double log_q = c->avg_log_scale + lead_growth + log_rest + c->avg_interval_forward;
    const double log_c = c->avg_log_scale + lead_growth + c->avg_log_half;
    const double log_accrued = log_add(-INFINITY, log_c);
    double residual[3] = {0.0, 0.0, 0.0};
    if (control) {
        const double width = c->control_first_weight * c->avg_width;
        const double log_forward = c->control_log_asset_scale + lead_growth + geometric_growth +
                                   c->control_first_weight * c->avg_drift + 0.5 * width * width;
        geometric_values(c, log_forward, c->control_log_strike, width, residual);
    }
    double values[3] = {0.0, 0.0, 0.0};
    const double log_strike = c->avg_log_strike;
    const double ld = c->log_discount;
    if (log_accrued >= log_strike) {
        if (c->sign > 0.0) {
            values[0] = std::exp(log_q + ld) + positive_difference(log_accrued + ld, log_strike + ld);
            values[1] = std::exp(log_q + ld - log_spot) + std::exp(log_c + ld - log_spot);
        }
    } else {
        const double log_b = log_strike + std::log(-std::expm1(log_accrued - log_strike));
        double forward = log_q - log_b;
        if (log_sum == -INFINITY) {
            const double extra = std::expm1(lead_growth) +
                                 std::exp(lead_growth) * (c->avg_rest * std::expm1(c->avg_interval_forward) +
                                                          relative_sum * std::exp(c->avg_interval_forward));
            const double excess = c->avg_baseline + c->avg_weight * extra;
            const double b = std::exp(log_b - log_spot);
            if (b > 0.0 && std::fabs(excess / b) < 0.5) forward = std::log1p(excess / b);
        }
        const double center = forward / c->avg_width;
        const double d1 = center + 0.5 * c->avg_width;
        const double d2 = center - 0.5 * c->avg_width;
        const double log_asset = log_q + ld + log_normal_cdf(c->sign * d1);
        const double log_cash = log_b + ld + log_normal_cdf(c->sign * d2);
        values[0] = c->sign > 0.0 ? positive_difference(log_asset, log_cash) : positive_difference(log_cash, log_asset);
        values[1] = c->sign * (std::exp(log_c + ld - log_spot + log_normal_cdf(c->sign * d2)) +
                               std::exp(log_q + ld - log_spot + log_normal_cdf(c->sign * d1)));
        values[2] = std::exp(ld + 2.0 * log_strike - 2.0 * log_spot - log_b - c->greek_log_width - 0.5 * d2 * d2 -
                             0.5 * std::log(2.0 * M_PI));
    }
    const double value = values[output] - residual[output];
    if (!std::isfinite(value)) f.failed = true;
    return value;
}

// GeometricParameters::geometric (asian.rs:740-784): moneyness = initial moneyness +
// drift, diffusion = width, log_scale = log width; the price or its delta / gamma.
static double average_geometric_payoff(const kgpu_contract* c, double normal, Failure& f) {
    const double distance = c->moneyness + c->diffusion * normal;
    const double standardized = c->moneyness / c->diffusion + normal;
    if (c->sign * standardized <= 0.0) return 0.0;
    const double log_strike = c->avg_log_strike;
    double log_payoff;
    if (std::fabs(distance) < 1e-5 && std::isfinite(standardized))
        log_payoff = log_strike + c->log_scale + std::log(std::fabs(standardized)) +
                     (distance == 0.0 ? 0.0 : std::log(std::fabs(std::expm1(distance)) / std::fabs(distance)));
    else if (c->sign > 0.0)
        log_payoff = log_strike + distance + std::log(-std::expm1(-distance));
    else
        log_payoff = log_strike + std::log(-std::expm1(distance));
    const double log_asset = log_strike + distance + c->log_discount + c->greek_log_weight;
    const double numerator = normal - std::exp(c->greek_log_base_width);
    double value;
    switch (output_of(c)) {
        case 1:
            value = c->sign * std::exp(log_asset - c->greek_log_spot);
            break;
        case 2:
            value = numerator != 0.0 ? c->sign * std::copysign(std::exp(log_asset - 2.0 * c->greek_log_spot +
                                                                        std::log(std::fabs(numerator)) -
                                                                        c->greek_log_base_width),
                                                               numerator)
                                     : 0.0;
            break;
        default:
            value = std::exp(log_payoff + c->log_discount);
    }
    if (!std::isfinite(value)) f.failed = true;
    return value;
}

// survival (double_barrier.rs:6-112): the probability that a Brownian bridge between
// log distances `initial` and `terminal` above the lower barrier stays inside (0, band),
// in out[0], and with `derivatives` its first and second derivatives in the initial log
// spot in out[1], out[2].  Returns false when the series does not converge or leaves
// [0, 1] (the reference's unstable() error).
static bool double_survival(double initial, double terminal, double band, double deviation, bool derivatives,
                            double out[3]) {
    out[0] = out[1] = out[2] = 0.0;
    if (terminal <= 0.0 || terminal >= band) return true;
    double x = initial / band, y = terminal / band;
    const double ratio = deviation / band;
    const double variance = ratio * ratio;
    if (variance == 0.0) {
        out[0] = 1.0;
        return true;
    }
    if (!std::isfinite(variance) || variance <= 0.0) return false;
    const bool reflected = x + y > 1.0;
    if (reflected) {
        x = 1.0 - x;
        y = 1.0 - y;
    }
    double sum[3] = {0.0, 0.0, 0.0};
    bool converged = false;
    if (variance < 0.25) {
        const double inverse_variance = std::isnormal(variance) ? 1.0 / variance : INFINITY;
        sum[0] = -std::expm1(-2.0 * (x / ratio) * (y / ratio));
        // One image term: k shifts the band; direct images add, reflected ones subtract.
        auto term = [&](double k, bool direct) {
            const double exponent = direct ? -2.0 * (k / ratio) * ((y - x + k) / ratio)
                                           : -2.0 * ((x + k) / ratio) * ((y + k) / ratio);
            const double sign = direct ? 1.0 : -1.0;
            const double weight = std::exp(exponent);
            if (k != 0.0) sum[0] += sign * weight;
            if (derivatives) {
                const double numerator = direct ? 2.0 * k : -2.0 * (y + k);
                if (numerator != 0.0) {
                    const double slope = numerator * inverse_variance;
                    const double first = weight * slope;
                    const double second = first * slope;
                    if (std::isnormal(weight) && std::isnormal(first) && std::isnormal(second)) {
                        sum[1] += sign * first;
                        sum[2] += sign * second;
                    } else {
                        const double log_slope = std::log(std::fabs(numerator)) - 2.0 * std::log(ratio);
                        sum[1] += sign * std::copysign(std::exp(exponent + log_slope), numerator);
                        sum[2] += sign * std::exp(exponent + 2.0 * log_slope);
                    }
                }
            }
            return weight;
        };
        term(0.0, false);
        for (int n = 1; n <= 64; ++n) {
            const double k = double(n);
            const double a = term(k, true);
            const double b = term(k, false);
            const double c = term(-k, true);
            const double d = term(-k, false);
            if (n >= 2 && a + b + c + d < 1e-18) {
                converged = true;
                break;
            }
        }
    } else {
        const double distance = y - x;
        const double log_scale = std::log(2.0 * std::sqrt(2.0 * M_PI) * ratio) + 0.5 * distance * distance / variance;
        for (int n = 1; n <= 256; ++n) {
            const double frequency = double(n) * M_PI;
            const double exponent = log_scale - 0.5 * frequency * frequency * variance;
            const double weight = std::exp(exponent);
            const double sy = std::sin(frequency * y);
            const double product = std::sin(frequency * x) * sy;
            sum[0] += weight * product;
            if (derivatives) {
                const double first = frequency * std::cos(frequency * x) * sy;
                const double score = -distance / variance;
                sum[1] += weight * (first + score * product);
                sum[2] += weight * (2.0 * score * first + (score * score + 1.0 / variance - frequency * frequency) * product);
            }
            if (n >= 4 && exponent + 4.0 * std::log(frequency) < -40.0) {
                converged = true;
                break;
            }
        }
    }
    if (!converged || !(sum[0] >= -1e-13 && sum[0] <= 1.0 + 1e-13)) return false;
    out[0] = std::min(std::max(sum[0], 0.0), 1.0);
    if (derivatives) {
        out[1] = (reflected ? -sum[1] : sum[1]) / band;
        out[2] = (sum[2] / band) / band;
    }
    return true;
}

// Continuously monitored double barrier (barrier.rs:341-390), value only.
static double double_barrier_payoff(const kgpu_contract* c, double z, Failure& f) {
    const double noise = std::fma(c->diffusion, z, 0.0);
    const double terminal = c->barrier_drift + noise;
    const double asset = discounted_product(c->spot, 1.0, terminal);
    if (!std::isfinite(asset)) f.failed = true;
    const double distance = c->moneyness + noise;
    const double payoff = std::fabs(distance) < 0.5 ? c->strike * std::expm1(distance) : asset - c->strike;
    const double intrinsic = std::max(c->sign * payoff, 0.0);
    const int output = output_of(c);
    double survival[3];
    if (!double_survival(c->band_initial, c->barrier_moneyness + noise, c->band, c->diffusion, output != 0,
                         survival)) {
        f.failed = true;
        return 0.0;
    }
    const bool in = c->flags & KGPU_C_BARRIER_IN;
    const double rebate = (!in && (c->flags & KGPU_C_REBATE_AT_HIT)) ? 0.0 : c->rebate;
    const double value =
        weighted(intrinsic, c->log_discount + (in ? std::log1p(-survival[0]) : std::log(survival[0]))) +
        weighted(rebate, c->log_discount + (in ? std::log(survival[0]) : std::log1p(-survival[0])));
    if (!std::isfinite(value)) f.failed = true;
    if (output == 0) return value;
    // derivative(weight) of barrier.rs:366-372
    const double difference = (in ? -1.0 : 1.0) * (intrinsic - rebate);
    auto derivative = [&](double weight) {
        const double sign = (std::signbit(difference) ? -1.0 : 1.0) * (std::signbit(weight) ? -1.0 : 1.0);
        return discounted_product(std::fabs(difference), sign, c->log_discount + std::log(std::fabs(weight)));
    };
    const double first = derivative(survival[1]);
    const double second = output == 2 ? derivative(survival[2]) : 0.0;
    const double greek = barrier_greek(output, value, first, second, z, c->diffusion, c->spot);
    if (!std::isfinite(greek)) f.failed = true;
    return greek;
}

// AutocallableNote::terminal (instruments/autocallable.rs:1396-1414)
static inline double autocallable_terminal(const kgpu_contract* c, double spot, bool knocked_in) {
    if (knocked_in) {
        if (c->flags & KGPU_C_DOWNSIDE) {
            double clamped = std::min(std::max(spot, c->downside_lower), c->downside_upper);
            return c->terminal_base + (clamped - c->downside_upper) / c->downside_initial;
        }
        return c->terminal_fixed;
    }
    return c->terminal_plain;
}

// PathPlan::payoff (autocallable.rs:823-862), one note, forward stepping.
static double autocallable_forward(const Plan& p, const Model& model, PathNormals& n) {
    const kgpu_contract* c = p.c;
    bool has_ki = c->flags & KGPU_C_HAS_KNOCK_IN;
    State s;
    s.v = model.m->v0;
    bool knocked_in = c->flags & KGPU_C_KNOCKED_IN;
    double cash = c->initial_cash;
    int ev = 0;
    for (int i = 0; i < c->step_count; ++i) {
        step_state(model, p.steps[i], s, n);
        uint8_t fl = p.flags[i];
        if (fl & KGPU_STEP_KNOCK_IN) knocked_in |= has_ki && s.lr < c->knock_in;
        if (fl & KGPU_STEP_EVENT) {
            const kgpu_event& e = p.events[ev++];
            bool coupon_due = s.lr >= e.coupon_barrier;
            bool knocked_out = e.has_knock_out && s.lr >= e.knock_out;
            cash += e.payment[int(coupon_due) | (int(knocked_out) << 1)];
            if (knocked_out) return cash;
        }
    }
    knocked_in |= (c->flags & KGPU_C_EXPIRY_KNOCK_IN) && has_ki && s.lr < c->knock_in;
    double spot = spot_at(c->spot, s.lr);
    cash += autocallable_terminal(c, spot, knocked_in) * c->final_discount;
    return cash;
}

// PathPlan::bridge_payoffs::<1, true> (autocallable.rs:628-736).
static double autocallable_bridge(const Plan& p, const Model& model, PathNormals& n) {
    const kgpu_contract* c = p.c;
    bool has_ki = c->flags & KGPU_C_HAS_KNOCK_IN;
    double cash = c->initial_cash;
    bool knocked_in = c->flags & KGPU_C_KNOCKED_IN;
    bool monitoring = !knocked_in && has_ki;
    const double level = c->knock_in;
    int start = 0;
    double lr = 0.0;
    int ev = 0;
    for (int k = 0; k < c->bridge_count; ++k) {
        const kgpu_bridge_interval& iv = p.intervals[k];
        double target = lr + std::fma(iv.diffusion, n.normal(), iv.drift);
        double minimum = std::numeric_limits<double>::infinity();
        for (int i = start; i < iv.end; ++i) {
            if (!monitoring || minimum < level) {
                n.skip(iv.end - i);
                break;
            }
            double z = n.normal();
            const kgpu_bridge_daily& d = p.daily[i];
            lr += std::fma(d.weight, target - lr, d.width * z);
            minimum = std::min(minimum, lr);
        }
        lr = target;
        start = iv.end + 1;
        uint8_t fl = p.flags[iv.end];
        if (monitoring && (minimum < level || ((fl & KGPU_STEP_KNOCK_IN) && lr < level))) {
            monitoring = false;
            knocked_in = true;
        }
        if (fl & KGPU_STEP_EVENT) {
            const kgpu_event& e = p.events[ev++];
            bool hit = e.has_knock_out && lr >= e.knock_out;
            cash += e.payment[int(lr >= e.coupon_barrier) | (int(hit) << 1)];
            if (hit) return cash;
        }
    }
    bool hit = knocked_in || ((c->flags & KGPU_C_EXPIRY_KNOCK_IN) && has_ki && lr < level);
    cash += autocallable_terminal(c, spot_at(c->spot, lr), hit) * c->final_discount;
    return cash;
}

// Vanilla payoff after stepping every grid step, and the arithmetic average of the
// fixing spots (Asian).
static double path_vanilla(const Plan& p, const Model& model, PathNormals& n, bool asian) {
    const kgpu_contract* c = p.c;
    State s;
    s.v = model.m->v0;
    double sum = 0.0;
    int fixings = 0;
    for (int i = 0; i < c->step_count; ++i) {
        step_state(model, p.steps[i], s, n);
        if (asian && (p.flags[i] & KGPU_STEP_FIXING)) {
            sum += spot_at(c->spot, s.lr);
            ++fixings;
        }
    }
    double underlying = asian ? sum / double(fixings) : spot_at(c->spot, s.lr);
    double value = c->sign * (underlying - c->strike);
    return (value > 0.0 ? value : 0.0) * c->final_discount;
}

// MonteCarloAccumulatorEngine path (accumulator.rs:160-216) without fixed purchase events.
static double accumulator_path(const Plan& p, const Model& model, PathNormals& n) {
    const kgpu_contract* c = p.c;
    State s;
    s.v = model.m->v0;
    double quantity = c->quantity;
    auto unit = [&](double lr) {
        double distance = lr - c->log_strike;
        if (std::fabs(distance) < 0.5) return c->sign * c->strike * std::expm1(distance);
        double spot = spot_at(c->spot, lr);
        return c->sign > 0.0 ? spot - c->strike : c->strike - spot;
    };
    for (int i = 0; i < c->step_count; ++i) {
        step_state(model, p.steps[i], s, n);
        uint8_t fl = p.flags[i];
        if ((fl & KGPU_STEP_EVENT) && c->sign * s.lr >= c->sign * c->knock_out)
            return quantity * unit(s.lr) * p.steps[i].discount;
        if (fl & KGPU_STEP_ACCUMULATE)
            quantity += c->daily_quantity *
                        (c->sign * s.lr < c->sign * c->log_strike ? c->acceleration : 1.0);
    }
    return quantity * unit(s.lr) * c->final_discount;
}

static bool terminal_payoff(const kgpu_contract* c) {
    return c->payoff == KGPU_PAYOFF_EUROPEAN || c->payoff == KGPU_PAYOFF_DIGITAL || c->payoff == KGPU_PAYOFF_BARRIER ||
           c->payoff == KGPU_PAYOFF_AVERAGE_GEOMETRIC || c->payoff == KGPU_PAYOFF_DOUBLE_BARRIER;
}

static int dimensions_of(const kgpu_contract* c, const Model& model) {
    if (terminal_payoff(c)) return 1;
    if (c->dimensions > 0) return c->dimensions;
    return c->step_count * model.normals_per_step();
}

static double evaluate(const Plan& p, const Model& model, PathNormals& n, Failure& f) {
    const kgpu_contract* c = p.c;
    switch (c->payoff) {
        case KGPU_PAYOFF_EUROPEAN:
            return european_payoff(c, n.normal(), f);
        case KGPU_PAYOFF_DIGITAL:
            return digital_payoff(c, n.normal());
        case KGPU_PAYOFF_BARRIER:
            return barrier_payoff(c, n.normal(), f);
        case KGPU_PAYOFF_BARRIER_DISCRETE:
            return barrier_discrete_payoff(p, n, f);
        case KGPU_PAYOFF_AVERAGE_ARITHMETIC:
            return average_arithmetic_payoff(c, n, f);
        case KGPU_PAYOFF_AVERAGE_GEOMETRIC:
            return average_geometric_payoff(c, n.normal(), f);
        case KGPU_PAYOFF_DOUBLE_BARRIER:
            return double_barrier_payoff(c, n.normal(), f);
        case KGPU_PAYOFF_VANILLA_PATH:
            return path_vanilla(p, model, n, false);
        case KGPU_PAYOFF_ASIAN:
            return path_vanilla(p, model, n, true);
        case KGPU_PAYOFF_AUTOCALLABLE:
            return (c->flags & KGPU_C_BRIDGE) ? autocallable_bridge(p, model, n)
                                              : autocallable_forward(p, model, n);
        case KGPU_PAYOFF_ACCUMULATOR:
            return accumulator_path(p, model, n);
    }
    f.failed = true;
    return 0.0;
}

struct BlockResult {
    Moments moments, pairs;
    Moments variance;  // i.i.d. sample moments with variance, for the sample error
    uint64_t steps = 0;
};

// sample_paths (monte_carlo.rs:1761-1811) for one contract.
static int price_contract(const Model& model, const Plan& p, const kgpu_settings* settings,
                          int threads, kgpu_estimate* out) {
    const kgpu_contract* c = p.c;
    int64_t paths = c->path_count > 0 ? c->path_count : settings->path_count;
    if (paths < 1) return KGPU_INVALID_INPUT;
    bool sobol = settings->sampling == KGPU_SAMPLING_SOBOL;
    bool antithetic = settings->antithetic != 0;
    if (c->dimensions < 0 || (c->dimensions > 0 && c->dimensions < c->step_count * model.normals_per_step()))
        return KGPU_INVALID_INPUT;
    int dims = dimensions_of(c, model);
    // sobol::sequence rejects dimensions beyond the Joe-Kuo table (sobol.rs).
    if (sobol && (dims < 1 || dims > 21201)) return KGPU_INVALID_INPUT;
    int64_t samples = antithetic ? (paths + 1) / 2 : paths;
    size_t blocks = size_t((samples + kBlockSize - 1) / kBlockSize);
    std::unique_ptr<SobolSequence> seq;
    if (sobol) seq.reset(new SobolSequence(dims, settings->seed));
    bool statistics = !sobol && (!antithetic || paths % 2 == 0);
    bool variance = statistics && !antithetic;
    std::vector<BlockResult> partials(blocks);
    std::atomic<bool> failed{false};
    run_blocks(blocks, threads, [&](size_t b) {
        BlockResult r;
        BlockDraws draws(settings->seed, b, seq.get());
        std::vector<double> buffer(dims);
        Failure f;
        int64_t first = int64_t(b) * kBlockSize;
        int64_t last = std::min<int64_t>(first + kBlockSize, samples);
        for (int64_t sample = first; sample < last; ++sample) {
            bool paired = antithetic && sample < paths / 2;
            double positive, negative = 0.0;
            if (paired) {
                for (int d = 0; d < dims; ++d) buffer[d] = draws.normal();
                PathNormals n{&draws, buffer.data()};
                positive = evaluate(p, model, n, f);
                PathNormals m{&draws, buffer.data()};
                m.sign = -1.0;
                negative = evaluate(p, model, m, f);
                r.steps += uint64_t(std::max(n.used, m.used));
            } else {
                PathNormals n{&draws, nullptr};
                positive = evaluate(p, model, n, f);
                r.steps += uint64_t(n.used);
                n.skip(dims - n.used);
            }
            if (!std::isfinite(positive) || !std::isfinite(negative)) f.failed = true;
            r.moments.add(positive, variance);
            r.variance.add(positive, true);
            if (paired) {
                r.moments.add(negative, variance);
                r.variance.add(negative, true);
                if (statistics) r.pairs.add(midpoint(positive, negative), true);
            }
            draws.next_path();
        }
        if (f.failed) failed = true;
        partials[b] = r;
    });
    if (failed) return KGPU_COMPUTATION_FAILURE;
    Moments total, pairs, var;
    uint64_t executed = 0;
    for (auto& r : partials) {
        total.merge(r.moments, variance);
        var.merge(r.variance, true);
        if (statistics && antithetic) pairs.merge(r.pairs, true);
        executed += r.steps;
    }
    double log_discount = (c->payoff == KGPU_PAYOFF_EUROPEAN) ? c->log_scale : 0.0;
    double price = discounted_product(total.scale, total.mean, log_discount);
    if (!std::isfinite(price)) return KGPU_COMPUTATION_FAILURE;
    // sampling_standard_error (monte_carlo.rs:1435-1452) and from_sampling (939-963).
    const Moments& u = antithetic ? pairs : total;
    // ArithmeticGrid::sample (asian.rs:616-621): residual samples plus the control's mean.
    if (c->payoff == KGPU_PAYOFF_AVERAGE_ARITHMETIC && (c->flags & KGPU_C_AVERAGE_CONTROL))
        price += c->control_mean;
    out->price = price;
    out->seed = settings->seed;
    out->standard_error = 0.0;
    bool have = statistics && u.count >= 2;
    if (have) {
        double deviation = std::sqrt(std::max(u.m2, 0.0) / double(u.count - 1) / double(u.count));
        double se = discounted_product(u.scale, deviation, log_discount);
        if (se == 0.0) {
            out->uncertainty_status = KGPU_UNCERTAINTY_ZERO_OBSERVED_VARIANCE;
        } else {
            out->standard_error = se;
            out->uncertainty_status = KGPU_UNCERTAINTY_AVAILABLE;
        }
    } else if (sobol) {
        out->uncertainty_status = KGPU_UNCERTAINTY_UNSUPPORTED_SAMPLING;
    } else if (antithetic && paths % 2 != 0) {
        out->uncertainty_status = KGPU_UNCERTAINTY_INCOMPLETE_ANTITHETIC_PAIR;
    } else {
        out->uncertainty_status = KGPU_UNCERTAINTY_INSUFFICIENT_OBSERVATIONS;
    }
    out->sample_error =
        var.count >= 2
            ? discounted_product(var.scale,
                                 std::sqrt(std::max(var.m2, 0.0) / double(var.count - 1) /
                                           double(var.count)),
                                 log_discount)
            : 0.0;
    int grid = terminal_payoff(c) ? 1 : c->step_count;
    out->path_steps = double(paths) * double(grid);
    out->executed_steps = double(executed) / double(model.normals_per_step());
    return KGPU_OK;
}

// --------------------------------------------------------------------------------------
// Lanes of one shared daily grid on one path loop (engines/monte_carlo/autocallable/
// portfolio.rs).  SharedEvents::new (903-1047) builds the interval plan from the union
// of the lanes' cash and maturity dates; shared_payoffs (1275-1439) walks every lane
// along one path; price_with_strips (1150-1258) turns the threshold-strip bucket sums
// into prices.  Each lane is a contract of the book whose steps are a prefix of the
// longest lane's grid; its own interval plan is not read here.
// --------------------------------------------------------------------------------------

// numerics::Sum: Neumaier-compensated addition.
struct CompensatedSum {
    double value = 0.0, correction = 0.0;
    void add(double term) {
        double next = value + term;
        correction += std::fabs(value) >= std::fabs(term) ? (value - next) + term : (term - next) + value;
        value = next;
    }
    double total() const { return value + correction; }
    void merge(const CompensatedSum& other) {
        add(other.value);
        add(other.correction);
    }
};

enum { kStripNone = 0, kStripKnockOut = 1, kStripKnockIn = 2 };

struct SharedGroup {
    const kgpu_book* book;
    int lanes = 0;
    const kgpu_step* steps = nullptr;  // the longest lane's grid
    const uint8_t* flags = nullptr;
    int step_count = 0;
    struct Action {
        int lane, event;  // event < 0: the lane's maturity
    };
    struct Interval {
        int step, end;
        double drift, diffusion;
    };
    std::vector<Action> actions;
    std::vector<Interval> intervals;
    std::vector<std::array<double, 2>> daily;
    std::vector<std::pair<double, int>> barriers;  // live knock-in levels, ascending
    const int32_t *kind, *offset, *length;
    const double* levels;
};

struct LaneState {
    double cash;
    bool monitoring, knocked_in, terminated;
    int next_threshold;
};

static void build_shared_group(SharedGroup& g, double safe_low, double safe_high) {
    const kgpu_book* b = g.book;
    int base = 0;
    for (int l = 0; l < g.lanes; ++l)
        if (b->contracts[l].step_count >= b->contracts[base].step_count) base = l;  // max_by_key keeps the last
    const kgpu_contract& bc = b->contracts[base];
    g.steps = b->steps + bc.step_offset;
    g.flags = b->step_flags + bc.step_offset;
    g.step_count = bc.step_count;
    const int n = g.step_count;
    std::vector<std::vector<SharedGroup::Action>> buckets(n);
    for (int l = 0; l < g.lanes; ++l) {
        const kgpu_contract& c = b->contracts[l];
        if ((c.flags & KGPU_C_HAS_KNOCK_IN) && !(c.flags & KGPU_C_KNOCKED_IN)) g.barriers.push_back({c.knock_in, l});
        int ev = 0;
        for (int i = 0; i < c.step_count; ++i)
            if (b->step_flags[c.step_offset + i] & KGPU_STEP_EVENT) buckets[i].push_back({l, ev++});
        buckets[c.step_count - 1].push_back({l, -1});
    }
    std::vector<int> ends;
    for (int i = 0; i < n; ++i) {
        for (auto& a : buckets[i]) g.actions.push_back(a);
        ends.push_back(int(g.actions.size()));
    }
    double excursion = 0.0;
    for (int i = 0; i < n; ++i) excursion += std::fabs(g.steps[i].drift) + 20.0 * g.steps[i].diffusion;
    const bool bridge = safe_low <= excursion && excursion <= safe_high && safe_low <= -excursion &&
                        -excursion <= safe_high;
    g.daily.assign(size_t(n), std::array<double, 2>{0.0, 0.0});
    int first = 0, previous = 0;
    for (int step = 0; step < n; ++step) {
        const int end = ends[step];
        if (end == previous && step + 1 < n) continue;
        if (bridge && step - first >= 8) {
            double drift = g.steps[step].drift, width = g.steps[step].diffusion;
            double variance = width * width;
            for (int i = step - 1; i >= first; --i) {
                const double mean = g.steps[i].drift, w = g.steps[i].diffusion;
                const double next = std::fma(w, w, variance);
                g.daily[i] = {(w * w) / next, w * std::sqrt(variance / next)};
                drift += mean;
                variance = next;
            }
            const double diffusion = std::sqrt(variance);
            bool usable = std::isnormal(diffusion) && std::isfinite(drift);
            for (int i = first; i < step && usable; ++i) usable = g.daily[i][0] > 0.0 && g.daily[i][1] > 0.0;
            if (usable) {
                g.intervals.push_back({step, end, drift, diffusion});
                first = step + 1;
                previous = end;
                continue;
            }
        }
        for (int i = first; i <= step; ++i)
            g.intervals.push_back({i, i == step ? end : previous, g.steps[i].drift, g.steps[i].diffusion});
        first = step + 1;
        previous = end;
    }
    std::stable_sort(g.barriers.begin(), g.barriers.end(),
                     [](const std::pair<double, int>& a, const std::pair<double, int>& b) { return a.first < b.first; });
}

// One path of every lane; false when a lane's cash is not finite.
static bool shared_path(const SharedGroup& g, PathNormals& n, std::vector<LaneState>& st,
                        std::vector<CompensatedSum>& sums) {
    const kgpu_book* b = g.book;
    for (int l = 0; l < g.lanes; ++l) {
        const kgpu_contract& c = b->contracts[l];
        const bool knocked = c.flags & KGPU_C_KNOCKED_IN;
        st[l] = {c.initial_cash, (c.flags & KGPU_C_HAS_KNOCK_IN) && !knocked, knocked, false, 0};
    }
    double lr = 0.0, minimum = std::numeric_limits<double>::infinity();
    int first = 0, first_step = 0, remaining = g.lanes;
    size_t cursor = 0;
    bool ok = true;
    auto strip_end = [&](const double* lv, int from, int len, double value) {
        // partition_point(level <= value) over the ascending levels[from..len)
        return int(std::upper_bound(lv + from, lv + len, value) - lv);
    };
    for (const auto& iv : g.intervals) {
        const double target = lr + std::fma(iv.diffusion, n.normal(), iv.drift);
        if (first_step < iv.step) {
            while (cursor < g.barriers.size() && st[g.barriers[cursor].second].terminated) ++cursor;
            const double floor =
                cursor < g.barriers.size() ? g.barriers[cursor].first : std::numeric_limits<double>::infinity();
            for (int i = first_step; i < iv.step; ++i) {
                if (minimum < floor || floor == std::numeric_limits<double>::infinity()) {
                    n.skip(iv.step - i);
                    break;
                }
                const double z = n.normal();
                lr += std::fma(g.daily[i][0], target - lr, g.daily[i][1] * z);
                if (g.flags[i] & KGPU_STEP_KNOCK_IN) minimum = std::min(minimum, lr);
            }
        }
        lr = target;
        if (g.flags[iv.step] & KGPU_STEP_KNOCK_IN) minimum = std::min(minimum, lr);
        for (int q = first; q < iv.end; ++q) {
            const auto& a = g.actions[q];
            LaneState& L = st[a.lane];
            if (L.terminated) continue;
            const kgpu_contract& c = b->contracts[a.lane];
            const int kind = g.kind ? g.kind[a.lane] : kStripNone;
            const double* lv = kind ? g.levels + g.offset[a.lane] : nullptr;
            const int len = kind ? g.length[a.lane] : 0;
            CompensatedSum* bucket = kind ? sums.data() + g.offset[a.lane] : nullptr;
            bool terminated;
            if (a.event >= 0) {
                const kgpu_event& e = b->events[c.event_offset + a.event];
                if (kind == kStripKnockOut) {
                    const int crossed = strip_end(lv, L.next_threshold, len, lr);
                    if (crossed > L.next_threshold) {
                        const double cash = L.cash + e.payment[2];  // knocked out, coupon not due
                        if (!std::isfinite(cash)) ok = false;
                        bucket[L.next_threshold].add(cash);
                        if (crossed < len) bucket[crossed].add(-cash);
                        L.next_threshold = crossed;
                    }
                    terminated = crossed == len;
                } else {
                    const bool hit = e.has_knock_out && lr >= e.knock_out;
                    L.cash += e.payment[int(lr >= e.coupon_barrier) | (int(hit) << 1)];
                    if (!std::isfinite(L.cash)) ok = false;
                    terminated = hit;
                }
            } else {
                const double discount = g.steps[c.step_count - 1].discount;
                const double floor = (c.flags & KGPU_C_EXPIRY_KNOCK_IN) ? std::min(minimum, lr) : minimum;
                if (L.monitoring && floor < c.knock_in) {
                    L.monitoring = false;
                    L.knocked_in = true;
                }
                const double spot = spot_at(c.spot, lr);
                const double cash = L.cash + autocallable_terminal(&c, spot, L.knocked_in) * discount;
                if (!std::isfinite(cash)) ok = false;
                if (kind == kStripKnockOut) {
                    bucket[L.next_threshold].add(cash);
                } else {
                    if (kind == kStripKnockIn && !L.knocked_in) {
                        const int start = strip_end(lv, 0, len, floor);
                        if (start < len) {
                            const double hit = L.cash + autocallable_terminal(&c, spot, true) * discount;
                            if (!std::isfinite(hit - cash)) ok = false;
                            bucket[start].add(hit - cash);
                        }
                    }
                    L.cash = cash;
                }
                terminated = true;
            }
            if (terminated) {
                L.terminated = true;
                --remaining;
            }
        }
        if (remaining == 0) return ok;
        first = iv.end;
        first_step = iv.step + 1;
    }
    return false;
}

static int price_shared_group(const Model& model, SharedGroup& g, const kgpu_settings* settings, int strip_total,
                              double* lane_prices, double* strip_prices, int threads) {
    const kgpu_book* b = g.book;
    const int64_t paths = settings->path_count;
    if (paths < 1 || g.lanes < 1) return KGPU_INVALID_INPUT;
    const bool sobol = settings->sampling == KGPU_SAMPLING_SOBOL;
    const bool antithetic = settings->antithetic != 0;
    const int dims = g.step_count * model.normals_per_step();
    if (sobol && dims > 21201) return KGPU_INVALID_INPUT;
    const int64_t samples = antithetic ? (paths + 1) / 2 : paths;
    const size_t blocks = size_t((samples + kBlockSize - 1) / kBlockSize);
    std::unique_ptr<SobolSequence> seq;
    if (sobol) seq.reset(new SobolSequence(dims, settings->seed));
    struct Partial {
        std::vector<Moments> moments;
        std::vector<CompensatedSum> sums;
    };
    std::vector<Partial> partials(blocks);
    std::atomic<bool> failed{false};
    run_blocks(blocks, threads, [&](size_t blk) {
        Partial r;
        r.moments.assign(g.lanes, Moments());
        r.sums.assign(size_t(strip_total), CompensatedSum());
        std::vector<LaneState> st(g.lanes);
        BlockDraws draws(settings->seed, blk, seq.get());
        std::vector<double> buffer(dims);
        bool ok = true;
        const int64_t first = int64_t(blk) * kBlockSize;
        const int64_t last = std::min<int64_t>(first + kBlockSize, samples);
        for (int64_t sample = first; sample < last; ++sample) {
            const bool paired = antithetic && sample < paths / 2;
            auto record = [&]() {
                for (int l = 0; l < g.lanes; ++l) r.moments[l].add(st[l].cash, false);
            };
            if (paired) {
                for (int d = 0; d < dims; ++d) buffer[d] = draws.normal();
                PathNormals pn{&draws, buffer.data()};
                ok &= shared_path(g, pn, st, r.sums);
                record();
                PathNormals mn{&draws, buffer.data()};
                mn.sign = -1.0;
                ok &= shared_path(g, mn, st, r.sums);
                record();
            } else {
                PathNormals pn{&draws, nullptr};
                ok &= shared_path(g, pn, st, r.sums);
                record();
                pn.skip(dims - pn.used);
            }
            draws.next_path();
        }
        if (!ok) failed = true;
        partials[blk] = std::move(r);
    });
    if (failed) return KGPU_COMPUTATION_FAILURE;
    std::vector<Moments> total(g.lanes);
    std::vector<CompensatedSum> adjustments(static_cast<size_t>(strip_total));
    for (auto& r : partials) {
        for (int k = 0; k < strip_total; ++k) adjustments[k].merge(r.sums[k]);
        for (int l = 0; l < g.lanes; ++l) total[l].merge(r.moments[l], false);
    }
    for (int l = 0; l < g.lanes; ++l) {
        lane_prices[l] = discounted_product(total[l].scale, total[l].mean, 0.0);
        if (!std::isfinite(lane_prices[l])) return KGPU_COMPUTATION_FAILURE;
    }
    for (int l = 0; l < g.lanes; ++l) {
        if (!g.kind || g.kind[l] == kStripNone) continue;
        const double base = g.kind[l] == kStripKnockOut ? 0.0 : lane_prices[l];
        CompensatedSum prefix;
        for (int i = 0; i < g.length[l]; ++i) {
            prefix.merge(adjustments[g.offset[l] + i]);
            const double delta = prefix.total() / double(paths);
            const double price = base + delta;
            if (!std::isfinite(price) || (delta != 0.0 && std::fabs(price) < 1e-10 * (std::fabs(base) + std::fabs(delta))))
                return KGPU_COMPUTATION_FAILURE;
            strip_prices[g.offset[l] + i] = price;
        }
    }
    (void)b;
    return KGPU_OK;
}

}  // namespace kor

using namespace kor;

extern "C" {

int kor_price_book(const kgpu_model* model, const kgpu_book* book, const kgpu_settings* settings,
                   kgpu_estimate* out, int threads) {
    Model m(model);
    for (int i = 0; i < book->contract_count; ++i) {
        const kgpu_contract* c = &book->contracts[i];
        Plan p{book,
               c,
               book->steps + c->step_offset,
               book->step_flags + c->step_offset,
               book->events ? book->events + c->event_offset : nullptr,
               book->intervals ? book->intervals + c->bridge_offset : nullptr,
               book->bridge_daily ? book->bridge_daily + c->step_offset : nullptr};
        int status = price_contract(m, p, settings, threads, &out[i]);
        if (status != KGPU_OK) return status;
    }
    return KGPU_OK;
}

// The lanes of one shared daily grid (contracts of `book`), with optional threshold
// strips: lane l with kind[l] != 0 represents the ascending log levels
// levels[offset[l] .. offset[l] + length[l]), whose prices land in strip_prices at the
// same positions.  safe_low / safe_high bound the log returns that keep the spot finite.
int kor_price_shared_group(const kgpu_model* model, const kgpu_book* book, const kgpu_settings* settings,
                           double safe_low, double safe_high, const int32_t* kind, const int32_t* offset,
                           const int32_t* length, const double* levels, int strip_total, double* lane_prices,
                           double* strip_prices, int threads) {
    if (model->kind != KGPU_MODEL_BSM || book->contract_count < 1) return KGPU_INVALID_INPUT;
    for (int l = 0; l < book->contract_count; ++l)
        if (book->contracts[l].payoff != KGPU_PAYOFF_AUTOCALLABLE) return KGPU_INVALID_INPUT;
    Model m(model);
    SharedGroup g;
    g.book = book;
    g.lanes = book->contract_count;
    g.kind = kind;
    g.offset = offset;
    g.length = length;
    g.levels = levels;
    build_shared_group(g, safe_low, safe_high);
    return price_shared_group(m, g, settings, strip_total, lane_prices, strip_prices, threads);
}

// Raw PCG32 words of stream `stream` from word `first`.
void kor_pcg_words(uint64_t seed, uint64_t stream, uint64_t first, int64_t count, uint32_t* out) {
    Pcg32 g(seed, stream);
    g.advance(first);
    for (int64_t i = 0; i < count; ++i) out[i] = g.next();
}

// Normals `first .. first+count` of block `block` (NormalDraws with skip_normals).
void kor_pcg_normals(uint64_t seed, uint64_t block, uint64_t first, int64_t count, double* out) {
    BlockDraws d(seed, block, nullptr);
    d.skip(first);
    for (int64_t i = 0; i < count; ++i) out[i] = d.normal();
}

void kor_sobol_points(uint64_t seed, int dims, int dim, uint64_t first, int64_t count,
                      uint64_t* bits, double* normals) {
    SobolSequence s(dims, seed);
    for (int64_t i = 0; i < count; ++i) {
        uint64_t v = s.point(first + uint64_t(i), dim);
        if (bits) bits[i] = v;
        if (normals) normals[i] = normal_from_bits(v);
    }
}

void kor_sin_cos_turns(double turns, double* s, double* c) { sin_cos_turns(turns, s, c); }
double kor_ndtri(double p) { return inverse_normal_cdf(p); }

// European MC price with the terminal payoff of the kiyosi 0.19.0 build that produced
// benchmarks/quantlib/calibration/monte_carlo.json: max(sign (S_T - K), 0) with
// S_T = S exp(fma(sigma sqrt(T), z, (r - q - sigma^2/2) T)), discounted by exp(-r T)
// after the block-ordered Welford merge.  It uses the same normal stream and block
// structure as the 0.23.0 engine, so the recorded per-seed prices pin that stream.
double kor_golden_european_v019(uint64_t seed, int64_t paths, double spot, double strike,
                                double rate, double dividend, double sigma, double time, int call,
                                int threads) {
    double diffusion = sigma * std::sqrt(time);
    double drift = (rate - dividend - 0.5 * sigma * sigma) * time;
    double sign = call ? 1.0 : -1.0;
    size_t blocks = size_t((paths + kBlockSize - 1) / kBlockSize);
    std::vector<Moments> partial(blocks);
    run_blocks(blocks, threads, [&](size_t b) {
        BlockDraws d(seed, b, nullptr);
        Moments m;
        int64_t first = int64_t(b) * kBlockSize, last = std::min<int64_t>(first + kBlockSize, paths);
        for (int64_t s = first; s < last; ++s) {
            double st = spot * std::exp(std::fma(diffusion, d.normal(), drift));
            double v = sign * (st - strike);
            m.add(v > 0.0 ? v : 0.0, false);
        }
        partial[b] = m;
    });
    Moments total;
    for (auto& m : partial) total.merge(m, false);
    return discounted_product(total.scale, total.mean, -rate * time);
}

}  // extern "C"
