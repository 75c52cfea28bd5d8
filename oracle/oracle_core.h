// TEST INFRASTRUCTURE -- the FP64 CPU oracle for kiyosi's Monte Carlo hot path.
//
// This is a restatement, in C++, of the reference's Rust sampler (kiyosi 0.23.0).  Only
// tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use it, as the checker
// and as the timed CPU baseline; the product library never links it.  Rust's
// f64::{ln, exp, exp_m1, ln_1p, sqrt} are glibc's log/exp/expm1/log1p/sqrt on Linux, and
// f64::mul_add is std::fma; every other product and sum is rounded separately, so this
// file must be compiled with -ffp-contract=off.
#pragma once

#include <cmath>
#include <cstdint>
#include <vector>

namespace kor {

constexpr int kBlockSize = 256;  // BLOCK_SIZE, engines/monte_carlo.rs:20
constexpr int kSobolBits = 52;   // sobol.rs:5
constexpr uint64_t kSobolMask = (uint64_t(1) << kSobolBits) - 1;

// PCG-XSH-RR 64/32 (engines/monte_carlo.rs:2224-2277).
struct Pcg32 {
    static constexpr uint64_t kMultiplier = 6364136223846793005ULL;
    uint64_t state = 0;
    uint64_t increment = 1;

    Pcg32() = default;
    // Pcg32::new (monte_carlo.rs:2247-2256)
    Pcg32(uint64_t seed, uint64_t stream) : state(0), increment((stream << 1) | 1) {
        next();
        state += seed;
        next();
    }
    // Pcg32::next (monte_carlo.rs:2261-2267)
    uint32_t next() {
        uint64_t previous = state;
        state = previous * kMultiplier + increment;
        uint32_t x = uint32_t(((previous >> 18) ^ previous) >> 27);
        uint32_t r = uint32_t(previous >> 59);
        return (x >> r) | (x << ((32 - r) & 31));
    }
    // Pcg32::advance (monte_carlo.rs:2233-2245): affine squaring.
    void advance(uint64_t distance) {
        uint64_t multiplier = kMultiplier, inc = increment;
        while (distance != 0) {
            if (distance & 1) state = state * multiplier + inc;
            inc = inc * (multiplier + 1);
            multiplier = multiplier * multiplier;
            distance >>= 1;
        }
    }
    // Pcg32::uniform (monte_carlo.rs:2272-2276)
    double uniform() {
        uint64_t hi = next();
        uint64_t lo = next();
        uint64_t bits = (hi << 20) | (lo >> 12);
        return (double(bits) + 0.5) / 4503599627370496.0;
    }
};

// sin_cos_turns (monte_carlo.rs:1852-1894): quadrant reduction in turns, then Taylor
// polynomials evaluated with separate multiply and add roundings.
inline void sin_cos_turns(double turns, double* s, double* c) {
    static const double kSine[7] = {-1.0 / 1307674368000.0, 1.0 / 6227020800.0,
                                    -1.0 / 39916800.0,     1.0 / 362880.0,
                                    -1.0 / 5040.0,         1.0 / 120.0,
                                    -1.0 / 6.0};
    static const double kCosine[8] = {1.0 / 20922789888000.0, -1.0 / 87178291200.0,
                                      1.0 / 479001600.0,      -1.0 / 3628800.0,
                                      1.0 / 40320.0,          -1.0 / 720.0,
                                      1.0 / 24.0,             -0.5};
    const double tau = 6.283185307179586;
    uint32_t quadrant = uint32_t(turns * 4.0 + 0.5);
    double angle = tau * (turns - 0.25 * double(quadrant));
    double square = angle * angle;
    double ps = 0.0, pc = 0.0;
    for (double k : kSine) ps = ps * square + k;
    for (double k : kCosine) pc = pc * square + k;
    double sn = angle + angle * square * ps;
    double cs = 1.0 + square * pc;
    if (quadrant & 1) {
        double t = sn;
        sn = cs;
        cs = -t;
    }
    if (quadrant & 2) {
        sn = -sn;
        cs = -cs;
    }
    *s = sn;
    *c = cs;
}

// Cephes ndtri as restated in sobol.rs:253-346.
double inverse_normal_cdf(double probability);

// normal_from_bits (sobol.rs:249-252)
inline double normal_from_bits(uint64_t bits) {
    return inverse_normal_cdf((double(bits) + 0.5) / 4503599627370496.0);
}

// SobolSequence::new (sobol.rs:85-134): direction numbers scrambled by a random
// lower-triangular matrix (LMS) and a digital shift drawn from Pcg32::new(seed, dim).
struct SobolSequence {
    int dimensions = 0;
    std::vector<uint64_t> directions;  // [column * dimensions + dimension]
    std::vector<uint64_t> shifts;
    SobolSequence(int dims, uint64_t seed);
    uint64_t point(uint64_t index, int dimension) const {
        uint64_t value = shifts[dimension];
        uint64_t gray = index ^ (index >> 1);
        while (gray) {
            value ^= directions[size_t(__builtin_ctzll(gray)) * dimensions + dimension];
            gray &= gray - 1;
        }
        return value;
    }
};

// Scaled Welford moments (monte_carlo.rs:2155-2222).
struct Moments {
    uint64_t count = 0;
    double scale = 0.0, mean = 0.0, m2 = 0.0;
    void add(double value, bool variance) {
        if (std::fabs(value) > scale) {
            double ratio = scale / std::fabs(value);
            mean *= ratio;
            if (variance) m2 *= ratio * ratio;
            scale = std::fabs(value);
        }
        count += 1;
        double v = scale == 0.0 ? 0.0 : value / scale;
        double delta = v - mean;
        mean += delta / double(count);
        if (variance) m2 += delta * (v - mean);
    }
    void merge(const Moments& other, bool variance) {
        if (count == 0) {
            *this = other;
            return;
        }
        double sc = scale > other.scale ? scale : other.scale;
        double left = sc == 0.0 ? 0.0 : scale / sc;
        double right = sc == 0.0 ? 0.0 : other.scale / sc;
        double delta = other.mean * right - mean * left;
        uint64_t total = count + other.count;
        mean = mean * left + delta * (double(other.count) / double(total));
        if (variance)
            m2 = m2 * left * left + other.m2 * right * right +
                 delta * delta * (double(count) * (double(other.count) / double(total)));
        count = total;
        scale = sc;
    }
};

// discounted_product (numerics.rs:226-238)
inline double discounted_product(double scale, double weight, double log_discount) {
    double value = scale * weight;
    double discount = std::exp(log_discount);
    if (scale == 0.0 || weight == 0.0) return 0.0;
    if (std::isnormal(discount) && std::isnormal(value)) return value * discount;
    return std::copysign(std::exp(std::log(scale) + std::log(std::fabs(weight)) + log_discount),
                         weight);
}

// log_ratio (numerics.rs:80-92)
inline double log_ratio(double numerator, double denominator) {
    double relative = (numerator - denominator) / denominator;
    if (std::fabs(relative) < 0.5) return std::log1p(relative);
    double ratio = numerator / denominator;
    if (std::isnormal(ratio)) return std::log(ratio);
    return std::log(numerator) - std::log(denominator);
}

// Rust f64::midpoint for finite values of moderate size.
inline double midpoint(double a, double b) {
    const double lo = 2.2250738585072014e-308 * 2.0, hi = 1.7976931348623157e308 / 2.0;
    double aa = std::fabs(a), ab = std::fabs(b);
    if (aa <= hi && ab <= hi) return (a + b) / 2.0;
    if (aa < lo) return a + b / 2.0;
    if (ab < lo) return a / 2.0 + b;
    return a / 2.0 + b / 2.0;
}

// Normal draws of one block (NormalDraws, monte_carlo.rs:1678-1703) with the Sobol
// cursor of the block's first point (sobol.rs:136-243).
struct BlockDraws {
    Pcg32 generator;
    bool has_spare = false;
    double spare = 0.0;
    const SobolSequence* sobol = nullptr;
    std::vector<uint64_t> values;  // Sobol cursor state of the current point
    uint64_t index = 0;
    int dimension = 0;

    BlockDraws(uint64_t seed, uint64_t block, const SobolSequence* seq) : generator(seed, block),
                                                                          sobol(seq) {
        if (sobol) {
            index = block * kBlockSize;
            values.resize(sobol->dimensions);
            for (int d = 0; d < sobol->dimensions; ++d) values[d] = sobol->point(index, d);
        }
    }
    // sample_normal (monte_carlo.rs:1830-1845)
    double normal() {
        if (sobol) return normal_from_bits(values[dimension++]);
        if (has_spare) {
            has_spare = false;
            return spare;
        }
        double radius = std::sqrt(-2.0 * std::log(generator.uniform()));
        double s, c;
        sin_cos_turns(generator.uniform(), &s, &c);
        spare = radius * s;
        has_spare = true;
        return radius * c;
    }
    // NormalDraws::skip_normals (monte_carlo.rs:1689-1703); SobolCursor::seek for Sobol.
    void skip(uint64_t remaining) {
        if (sobol) {
            dimension += int(remaining);
            return;
        }
        if (remaining == 0) return;
        if (has_spare) {
            has_spare = false;
            remaining -= 1;
        }
        generator.advance((remaining / 2) * 4);
        if (remaining % 2 != 0) normal();
    }
    // SobolCursor::next_path (sobol.rs:206-218); positions of the PCG stream are kept by
    // the caller skipping the unused dimensions of each path.
    void next_path() {
        if (!sobol) return;
        index += 1;
        dimension = 0;
        int column = __builtin_ctzll(index);
        const uint64_t* dir = &sobol->directions[size_t(column) * sobol->dimensions];
        for (int d = 0; d < sobol->dimensions; ++d) values[d] ^= dir[d];
    }
    void seek(int dim) { dimension = dim; }
};

extern const uint32_t* joe_kuo_table();

}  // namespace kor
