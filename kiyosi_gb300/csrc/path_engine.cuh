// Path engine: one Monte Carlo path as a resumable state machine, shared by the plain
// (one thread per sample, one contract per launch) and persistent (lane-refill work
// queue) kernels.  Templated on the arithmetic type, the model and the sampler.
//
// Reference semantics, per payoff family (paths inside crates/kiyosi/src):
//   European terminal      engines/monte_carlo.rs:1238-1251 (TerminalPayoff::at_normal)
//   digital terminal       engines/monte_carlo/digital.rs:111-121
//   autocallable forward   engines/monte_carlo/autocallable.rs:823-862 (PathPlan::payoff)
//   autocallable bridge    engines/monte_carlo/autocallable.rs:628-736 (bridge_payoffs)
//   accumulator            engines/monte_carlo/accumulator.rs:160-216
//   vanilla / Asian path   path_samples with transition(), monte_carlo.rs:1498,2123
// Normal positions follow the reference's block streams: sample s of a contract uses
// normals [ (s % 256) * D, (s % 256 + 1) * D ) of stream Pcg32::new(seed, s / 256), or
// Sobol point s, dimensions 0..D-1; skipped normals keep later positions unchanged
// (LazyPath::finish / SkippingPath::skip, monte_carlo.rs:1591-1676).
//
// Plans are read in the kernel's own precision: FP64 kernels read the caller's kgpu_*
// arrays directly (identical layouts), FP32 kernels read single-precision copies made
// on the device by compile_plan_kernel, so no FP64 instruction runs per step.
#pragma once
#include <cstdint>

#include "../../include/kgpu.h"
#include "device_rng.cuh"

namespace kgpu {

template <class Real>
struct StepT {
    Real drift, diffusion, time, discount;
};
template <class Real>
struct EventT {
    Real knock_out, coupon_barrier;
    Real payment[4];
    int32_t has_knock_out, step;
};
template <class Real>
struct DailyT {
    Real weight, width;
};
template <class Real>
struct IntervalT {
    int32_t end, reserved;
    Real drift, diffusion;
};
static_assert(sizeof(StepT<double>) == sizeof(kgpu_step), "step layout");
static_assert(sizeof(EventT<double>) == sizeof(kgpu_event), "event layout");
static_assert(sizeof(DailyT<double>) == sizeof(kgpu_bridge_daily), "daily layout");
static_assert(sizeof(IntervalT<double>) == sizeof(kgpu_bridge_interval), "interval layout");

// One position of a bridged path (persistent kernels): position `start` of an interval
// draws the interval end (a = diffusion, b = drift), positions start+1..end are the
// daily bridge steps (a = width, b = weight).  Compiled on the device from the
// reference's BridgePlan intervals and daily weights.
template <class Real>
struct UnitT {
    Real a, b;
    int32_t end;    // last position of the interval
    int32_t flags;  // kUnitBegin | kUnitLast | kUnitKnockOut | end step flags << 8
};
constexpr int32_t kUnitBegin = 1;
constexpr int32_t kUnitLast = 2;
constexpr int32_t kUnitKnockOut = 4;  // the interval's end has a knock-out level

// Cash event of an interval's end, stored at the interval's last position.
template <class Real>
struct EndT {
    Real knock_out, coupon_barrier;
    Real payment[4];
    Real pad[2];
};

// A contract's scalars in the kernel's precision.
template <class Real>
struct ContractT {
    int32_t payoff, flags, step_count, event_count, bridge_count, reserved;
    int64_t step_offset;
    int32_t event_offset, bridge_offset;
    Real strike, sign, diffusion, half_variance, moneyness, log_scale;
    Real knock_in, initial_cash, terminal_base, terminal_plain, terminal_fixed;
    Real downside_lower, downside_upper, downside_initial, final_discount;
    Real knock_out, quantity, daily_quantity, acceleration, log_strike;
    Real barrier_drift, barrier_distance, barrier_moneyness, rebate, spot, log_discount;
    Real volatility, dividend;
    Real avg_drift, avg_width, avg_lead_drift, avg_lead_width, avg_interval_forward, avg_weight;
    Real avg_log_spot, avg_log_scale, avg_log_strike, avg_fraction, avg_half, avg_log_fraction, avg_log_half;
    Real avg_rest, avg_log_rest, avg_baseline;
    Real control_log_strike, control_log_asset_scale, control_first_weight, control_mean;
    Real band, band_initial;
    Real greek_log_spot, greek_log_width, greek_log_amount, greek_log_base_width, greek_log_weight;
};

// Device view of the book in the kernel's precision.
template <class Real>
struct DevBook {
    const ContractT<Real>* contracts;
    const StepT<Real>* steps;
    const uint8_t* flags;
    const EventT<Real>* events;
    const IntervalT<Real>* intervals;
    const DailyT<Real>* daily;
    const UnitT<Real>* units;  // per-position bridge units (persistent kernels), may be null
    const EndT<Real>* ends;    // per-position interval-end events (persistent kernels)
};

// Device view of the model.  The local-volatility surface is staged in shared memory
// by the kernels (`lv` points there).
template <class Real>
struct DevModel {
    int kind;
    int nt, ns;
    Real spot, rate, dividend;
    Real v0, kappa, theta, xi, rho, rho_bar;
    const Real* lv;  // [nt] years since the first node, [ns] spots, [nt*ns] values
};

// ------------------------------------------------------------------------------------
// Normal sources.
// ------------------------------------------------------------------------------------
// EXACT_RADIUS: the FP32 Box-Muller radius by IEEE sqrtf instead of the SFU root.
template <class Real, bool EXACT_RADIUS = false>
struct PcgSource {
    Pcg g;
    Real spare;
    bool has_spare;

    __device__ __forceinline__ void draw(Real& c, Real& s) {
        uint64_t b1 = pcg_bits52(g);
        uint64_t b2 = pcg_bits52(g);
        box_muller(b1, b2, &c, &s, EXACT_RADIUS);
    }
    // Positions the stream at the first normal of `sample` (dims normals per sample).
    __device__ __forceinline__ void start(uint64_t seed, uint64_t sample, int dims) {
        uint64_t block = sample / kBlockSize;
        uint64_t first = (sample % kBlockSize) * uint64_t(dims);
        g = pcg_new(seed, block);
        pcg_advance(g, (first / 2) * 4);
        has_spare = false;
        if (first & 1) {
            Real c, s;
            draw(c, s);
            spare = s;
            has_spare = true;
        }
    }
    __device__ __forceinline__ Real normal() {
        if (has_spare) {
            has_spare = false;
            return spare;
        }
        Real c, s;
        draw(c, s);
        spare = s;
        has_spare = true;
        return c;
    }
    __device__ __forceinline__ Real normal_if(bool need) { return need ? normal() : Real(0); }
    __device__ __forceinline__ void skip(int remaining) {
        if (remaining <= 0) return;
        if (has_spare) {
            has_spare = false;
            --remaining;
        }
        pcg_advance(g, uint64_t(remaining / 2) * 4);
        if (remaining & 1) normal();
    }
};

// Sobol point: the bits of dimension d are high[d] ^ nib[d][g & 15] ^ nib[d][16 + (g >> 4)]
// where high[] holds the shift and the directions of the gray-code bits >= 8 shared by
// the 256 points of one reference block, g the low 8 gray-code bits of the point, and
// nib[] the XORs of direction rows 0-3 and 4-7 for each 4-bit pattern.
template <class Real>
struct SobolSource {
    const uint64_t* high;
    const uint64_t* __restrict__ nib;  // [dims][32]
    int dims;
    int used;
    uint32_t lo, hi;

    __device__ __forceinline__ void start(uint64_t sample) {
        uint64_t gray = sample ^ (sample >> 1);
        lo = uint32_t(gray & 0xF);
        hi = uint32_t((gray >> 4) & 0xF) + 16;
        used = 0;
    }
    __device__ __forceinline__ uint64_t bits(int d) const {
        const uint64_t* row = nib + size_t(d) * 32;
        return high[d] ^ __ldg(row + lo) ^ __ldg(row + hi);
    }
    __device__ __forceinline__ Real normal() { return sobol_normal(bits(used++), Real()); }
    // Evaluates the next dimension whether or not it is needed (a pure function of the
    // point), so the warp computes the quantile converged; consumes it only if needed.
    __device__ __forceinline__ Real normal_if(bool need) {
        const Real z = sobol_normal(bits(used < dims ? used : dims - 1), Real());
        used += need ? 1 : 0;
        return z;
    }
    __device__ __forceinline__ void skip(int remaining) { used += remaining > 0 ? remaining : 0; }
};

// FP32 Sobol point from the top 32 of its 52 bits: high32[] and nib32[] hold the top 32
// bits of the block's high part and of the nibble tables (truncation commutes with XOR),
// halving the table bytes the path kernel reads.  The quantile needs the lower bits
// only in the extreme tails (t < 2^-20, about 2e-6 of draws), where the full 52-bit
// integer is rebuilt from the 64-bit directions.
struct SobolSource32 {
    const uint32_t* __restrict__ high32;  // this point's block row of the high table
    const uint32_t* __restrict__ nib32;     // [dims][32]
    const uint64_t* __restrict__ dirs64;    // [column * dims + dim]
    const uint64_t* __restrict__ shifts64;  // [dim]
    int dims;
    int used;
    uint32_t lo, hi;
    uint64_t gray;

    __device__ __forceinline__ void start(uint64_t sample) {
        gray = sample ^ (sample >> 1);
        lo = uint32_t(gray & 0xF);
        hi = uint32_t((gray >> 4) & 0xF) + 16;
        used = 0;
    }
    __device__ __forceinline__ float normal() {
        const int d = used++;
        const uint32_t* row = nib32 + size_t(d) * 32;
        const uint32_t v = high32[d] ^ __ldg(row + lo) ^ __ldg(row + hi);
        const bool upper = (v >> 31) != 0;
        const uint32_t k = upper ? ~v : v;  // top 32 bits of the 52-bit tail integer
        if (k < (1u << 12)) {
            uint64_t x = shifts64[d];
            for (uint64_t g = gray; g; g &= g - 1) x ^= dirs64[size_t(__ffsll(g) - 1) * dims + d];
            return sobol_normal(x, 0.0f);
        }
        return normal_from_tail32(k, upper);
    }
    __device__ __forceinline__ float normal_if(bool need) { return need ? normal() : 0.0f; }
    __device__ __forceinline__ void skip(int remaining) { used += remaining > 0 ? remaining : 0; }
};

// ------------------------------------------------------------------------------------
// Arithmetic helpers: FP64 keeps the reference's rounding; FP32 uses fast intrinsics.
// ------------------------------------------------------------------------------------
__device__ __forceinline__ double xfma(double a, double b, double c) { return fma(a, b, c); }
__device__ __forceinline__ float xfma(float a, float b, float c) { return fmaf(a, b, c); }
__device__ __forceinline__ double xabs(double x) { return fabs(x); }
__device__ __forceinline__ float xabs(float x) { return fabsf(x); }
__device__ __forceinline__ double xexp(double x) { return exp(x); }
__device__ __forceinline__ float xexp(float x) { return __expf(x); }
__device__ __forceinline__ double xexpm1(double x) { return expm1(x); }
__device__ __forceinline__ float xexpm1(float x) { return expm1f(x); }
__device__ __forceinline__ double xlog(double x) { return log(x); }
__device__ __forceinline__ float xlog(float x) { return __logf(x); }
__device__ __forceinline__ double xlog1p(double x) { return log1p(x); }
__device__ __forceinline__ float xlog1p(float x) { return log1pf(x); }
__device__ __forceinline__ double xsin(double x) { return sin(x); }
__device__ __forceinline__ float xsin(float x) { return sinf(x); }
__device__ __forceinline__ double xsqrt(double x) { return sqrt(x); }
__device__ __forceinline__ float xsqrt(float x) { return sqrt_approx(x); }
__device__ __forceinline__ double xinf(double) { return __longlong_as_double(0x7ff0000000000000LL); }
__device__ __forceinline__ float xinf(float) { return __int_as_float(0x7f800000); }
__device__ __forceinline__ double xnan(double) { return __longlong_as_double(0x7ff8000000000000LL); }
__device__ __forceinline__ float xnan(float) { return __int_as_float(0x7fc00000); }

// scaled_value(initial, 1, log_return) for ordinary magnitudes (numerics.rs:226-238).
template <class Real>
__device__ __forceinline__ Real spot_at(Real initial, Real log_return) {
    return initial * xexp(log_return);
}

// LocalVolatilitySurface::at_year (market/local_volatility.rs:322-359)
template <class Real>
__device__ __forceinline__ void lv_bracket(const Real* nodes, int n, Real value, int& left,
                                           Real& weight) {
    // partition_point(node <= value) - 1, clamped to [0, n-2].  `left` on entry is the
    // bracket of a previous value of the same path (or < 0): a path's spot moves little
    // per step and its time only forward, so walking from there usually takes no step;
    // the walk ends on the same bracket as the search.
    int l = left;
    if (l < 0) {
        int lo = 0, hi = n;
        while (lo < hi) {
            int mid = (lo + hi) >> 1;
            if (nodes[mid] <= value)
                lo = mid + 1;
            else
                hi = mid;
        }
        l = lo - 1;
        l = l < 0 ? 0 : (l > n - 2 ? n - 2 : l);
    } else {
        while (l > 0 && !(nodes[l] <= value)) --l;
        while (l < n - 2 && nodes[l + 1] <= value) ++l;
    }
    Real w;
    if constexpr (sizeof(Real) == 4)
        w = __fdividef(value - nodes[l], nodes[l + 1] - nodes[l]);
    else
        w = (value - nodes[l]) / (nodes[l + 1] - nodes[l]);
    weight = w < Real(0) ? Real(0) : (w > Real(1) ? Real(1) : w);
    left = l;
}

template <class Real>
__device__ __forceinline__ Real lv_interpolate(Real low, Real high, Real weight) {
    return weight <= Real(0.5) ? low + weight * (high - low) : high + (Real(1) - weight) * (low - high);
}

template <class Real>
__device__ __forceinline__ Real lv_at(const DevModel<Real>& m, Real time, Real spot, int& row, int& col) {
    const Real* years = m.lv;
    const Real* spots = m.lv + m.nt;
    const Real* values = m.lv + m.nt + m.ns;
    Real tw, sw;
    lv_bracket(years, m.nt, time, row, tw);
    lv_bracket(spots, m.ns, spot, col, sw);
    const Real* r0 = values + row * m.ns;
    const Real* r1 = r0 + m.ns;
    return lv_interpolate(lv_interpolate(r0[col], r0[col + 1], sw),
                          lv_interpolate(r1[col], r1[col + 1], sw), tw);
}

// ------------------------------------------------------------------------------------
// Path state.
// ------------------------------------------------------------------------------------
template <class Real>
struct PathState {
    Real lr;       // log return relative to the valuation spot
    Real v;        // Heston variance
    Real acc;      // Asian running sum / accumulator quantity
    Real cash;     // autocallable discounted cash
    Real target;   // bridge interval end
    Real minimum;  // bridge running minimum
    int i;         // next grid step
    int ev;        // next event (relative to the contract's first event)
    int k;         // next bridge interval
    int end;       // grid step ending the current bridge interval (-1: not started)
    int fixings;
    int executed;  // grid steps simulated
    int lv_row, lv_col;  // local volatility: the surface cell of the previous step (-1: none)
    bool knocked_in;
    bool monitoring;
    bool knocked_out;
};

template <class Real>
__device__ __forceinline__ void path_init(PathState<Real>& s, const ContractT<Real>& c, Real v0) {
    s.lr = Real(0);
    s.v = v0;
    s.acc = c.payoff == KGPU_PAYOFF_ACCUMULATOR ? c.quantity : Real(0);
    s.cash = c.initial_cash;
    s.target = Real(0);
    s.minimum = Real(0);
    s.i = 0;
    s.ev = 0;
    s.k = 0;
    s.end = -1;
    s.fixings = 0;
    s.executed = 0;
    s.lv_row = s.lv_col = -1;
    s.knocked_in = (c.flags & KGPU_C_KNOCKED_IN) != 0;
    s.monitoring = !s.knocked_in && (c.flags & KGPU_C_HAS_KNOCK_IN);
    s.knocked_out = false;
    if (c.payoff == KGPU_PAYOFF_AVERAGE_ARITHMETIC) {
        // growth (lr), relative sum (acc), log sum (cash), geometric growth (target) and
        // the lead growth (minimum; the lead normal is 0 without a lead interval).
        s.cash = -xinf(Real(0));
        s.minimum = c.avg_lead_drift + c.avg_lead_width * Real(0);
    }
}

// One grid step of the state.  BSM: `log_return += diffusion.mul_add(normal, drift)`;
// Heston: full-truncation Euler in log spot (two normals per step: spot, then the
// independent variance shock); local volatility: Euler in log spot with the surface
// read at the step's start.
template <class Real, int MODEL, class Source>
__device__ __forceinline__ void model_step(const DevModel<Real>& m, const StepT<Real>& st,
                                           PathState<Real>& s, Source& n) {
    if (MODEL == KGPU_MODEL_BSM) {
        Real t = xfma(st.diffusion, n.normal(), st.drift);
        s.lr = s.lr + t;
    } else if (MODEL == KGPU_MODEL_HESTON) {
        Real z1 = n.normal();
        Real z2 = n.normal();
        Real dt = st.drift, sq = st.diffusion;
        Real vp = s.v > Real(0) ? s.v : Real(0);
        Real sv = xsqrt(vp) * sq;
        Real zv = m.rho * z1 + m.rho_bar * z2;
        s.lr += (m.rate - m.dividend - Real(0.5) * vp) * dt + sv * z1;
        s.v += m.kappa * (m.theta - vp) * dt + m.xi * sv * zv;
    } else {
        Real spot = m.spot * xexp(s.lr);
        Real sigma = lv_at(m, st.time, spot, s.lv_row, s.lv_col);
        Real dt = st.drift, sq = st.diffusion;
        s.lr += (m.rate - m.dividend - Real(0.5) * sigma * sigma) * dt + sigma * sq * n.normal();
    }
}

// AutocallableNote::terminal (instruments/autocallable.rs:1396-1414)
template <class Real>
__device__ __forceinline__ Real autocallable_terminal(const ContractT<Real>& c, Real spot, bool ki) {
    if (ki) {
        if (c.flags & KGPU_C_DOWNSIDE) {
            Real clamped = spot < c.downside_lower ? c.downside_lower
                                                   : (spot > c.downside_upper ? c.downside_upper : spot);
            return c.terminal_base + (clamped - c.downside_upper) / c.downside_initial;
        }
        return c.terminal_fixed;
    }
    return c.terminal_plain;
}

template <class Real>
__device__ __forceinline__ Real european_value(const ContractT<Real>& c, Real z) {
    Real distance = xfma(c.diffusion, z, c.moneyness);
    if (c.sign * distance <= Real(0)) return Real(0);
    if (c.sign < Real(0)) return -xexpm1(distance);
    return -xexpm1(-distance) * xexp(xfma(c.diffusion, z, -c.half_variance));
}

// Which sample a path reports: 0 its payoff, 1 its delta sample, 2 its gamma sample.
__device__ __forceinline__ int output_of(int flags) {
    return (flags & KGPU_C_OUTPUT_DELTA) ? 1 : ((flags & KGPU_C_OUTPUT_GAMMA) ? 2 : 0);
}

// The barrier sampler's likelihood-ratio delta and gamma (barrier.rs:455-470): `z` is
// the first normal and `width` its standard deviation; `first` and `second` are the
// survival weight's spot derivatives (zero for scheduled monitoring).
template <class Real>
__device__ __forceinline__ Real likelihood_greek(int output, Real value, Real first, Real second, Real z, Real width,
                                                 Real spot) {
    const Real score = z / width;
    if (output == 1) return (value * score + first) / spot;
    const Real second_score = ((z * z - Real(1)) / width - z) / width;
    return ((value * second_score + first * (Real(2) * score - Real(1)) + second) / spot) / spot;
}

// MonteCarloDigitalEngine's native delta and gamma samples (digital.rs:116-140).
template <class Real>
__device__ __noinline__ Real digital_greek(const ContractT<Real>& c, Real z, Real exponent) {
    const Real log_payoff = c.greek_log_amount + exponent;
    if (output_of(c.flags) == 1) {
        if (z == Real(0)) return Real(0);
        return copysign(xexp(log_payoff + xlog(xabs(z)) - c.greek_log_spot - c.greek_log_width), z);
    }
    const Real score = xfma(-c.diffusion, z, z * z - Real(1));
    if (score == Real(0)) return Real(0);
    return copysign(xexp(log_payoff + xlog(xabs(score)) - Real(2) * c.greek_log_spot - Real(2) * c.greek_log_width),
                    score);
}

template <class Real>
__device__ __forceinline__ Real digital_value(const ContractT<Real>& c, Real z) {
    Real distance = c.moneyness + z;
    bool call = c.sign > Real(0);
    if (!(call ? distance > Real(0) : distance < Real(0))) return Real(0);
    Real exponent = c.log_scale + ((c.flags & KGPU_C_ASSET_DIGITAL) ? c.diffusion * z : Real(0));
    if (c.flags & (KGPU_C_OUTPUT_DELTA | KGPU_C_OUTPUT_GAMMA)) return digital_greek(c, z, exponent);
    return c.strike * xexp(exponent);
}

// Normal (finite, nonzero, not subnormal) test written with comparisons only; NaN fails
// every comparison.
__device__ __forceinline__ bool xnormal(double x) {
    const double a = fabs(x);
    return a >= 2.2250738585072014e-308 && a <= 1.7976931348623157e308;
}
__device__ __forceinline__ bool xnormal(float x) {
    const float a = fabsf(x);
    return a >= 1.17549435e-38f && a <= 3.40282347e38f;
}

// discounted_product(|amount|, signum(amount), log_weight) (numerics.rs:226-238), the
// `weighted` helper of barrier.rs:328-330.
template <class Real>
__device__ __forceinline__ Real weighted_amount(Real amount, Real log_weight) {
    const Real scale = xabs(amount);
    const Real weight = amount < Real(0) ? Real(-1) : Real(1);
    if (scale == Real(0)) return Real(0);
    const Real discount = xexp(log_weight);
    const Real value = scale * weight;
    if (xnormal(discount) && xnormal(value)) return value * discount;
    return copysign(xexp(xlog(scale) + log_weight), weight);
}

// Continuously monitored single barrier (barrier.rs:306-452): one terminal draw; the
// vanilla leg is weighted by the Brownian-bridge survival probability (knock-out) or
// the hit probability (knock-in), the expiry rebate by the other.
template <class Real>
__device__ __forceinline__ Real barrier_value(const ContractT<Real>& c, Real z) {
    const Real noise = xfma(c.diffusion, z, Real(0));
    const Real terminal = c.barrier_drift + noise;
    const Real distance = c.moneyness + noise;
    const Real payoff = xabs(distance) < Real(0.5) ? c.strike * xexpm1(distance)
                                                   : weighted_amount(c.spot, terminal) - c.strike;
    Real intrinsic = c.sign * payoff;
    intrinsic = intrinsic > Real(0) ? intrinsic : Real(0);
    const Real to_barrier = c.barrier_moneyness + noise;
    const bool up = (c.flags & KGPU_C_BARRIER_UP) != 0;
    const bool in = (c.flags & KGPU_C_BARRIER_IN) != 0;
    const bool live = up ? to_barrier < Real(0) : to_barrier > Real(0);
    const Real slope = live ? Real(2) * (xabs(to_barrier) / c.diffusion) / c.diffusion : Real(0);
    const Real exponent = -c.barrier_distance * slope;
    const Real survival = live ? xlog(-xexpm1(exponent)) : -xinf(Real(0));
    const Real value = weighted_amount(intrinsic, c.log_discount + (in ? exponent : survival)) +
                       weighted_amount(c.rebate, c.log_discount + (in ? survival : exponent));
    const int output = output_of(c.flags);
    if (output == 0) return value;
    Real first = Real(0), second = Real(0);
    if (slope > Real(0) && exponent > -xinf(Real(0))) {
        const Real difference = (in ? Real(-1) : Real(1)) * (intrinsic - c.rebate);
        first = weighted_amount(up ? -difference : difference, c.log_discount + (exponent + xlog(slope)));
        if (output == 2) second = weighted_amount(-difference, c.log_discount + (exponent + Real(2) * xlog(slope)));
    }
    return likelihood_greek(output, value, first, second, z, c.diffusion, c.spot);
}

__device__ __forceinline__ double xerfc(double x) { return erfc(x); }
__device__ __forceinline__ float xerfc(float x) { return erfcf(x); }

// normal_cdf, log_normal_cdf, log_normal_tail, weighted_cdf (numerics.rs:192-224).
template <class Real>
__device__ __forceinline__ Real normal_cdf_of(Real x) {
    return Real(0.5) * xerfc(-x * Real(0.70710678118654752440));
}

template <class Real>
__device__ Real log_normal_cdf_of(Real x) {
    if (x >= Real(-10)) return xlog(normal_cdf_of(x));
    const Real inverse_square = (Real(1) / x) / x;
    Real term = Real(1), sum = Real(1);
    for (int k = 1; k <= 20; ++k) {
        term *= -Real(2 * k - 1) * inverse_square;
        sum += term;
    }
    return Real(-0.5) * x * x - xlog(-x) + xlog(sum / Real(2.5066282746310002));
}

template <class Real>
__device__ __forceinline__ Real weighted_cdf_of(Real amount, Real exponent, Real argument) {
    const Real discount = xexp(exponent);
    const Real discounted = amount * discount;
    if (argument < Real(-10) || !xnormal(discount) || !(xabs(discounted) <= xinf(Real(0))))
        return xexp(xlog(amount) + exponent + log_normal_cdf_of(argument));
    return discounted * normal_cdf_of(argument);
}

// lognormal_price (engines/analytic/european.rs:317-403) for widths of at least 1e-5
// (narrower ones return NaN, reported as a computation failure).  Out of line: it runs
// once per conditioned path, and inlining it would raise the stepping loop's registers.
template <class Real>
__device__ __noinline__ Real lognormal_price_of(Real spot, Real strike, Real log_moneyness, Real asset_log, Real risk_log,
                                   Real volatility, Real root_time, Real sign) {
    const Real width = volatility * root_time;
    if (!(width >= Real(1e-5))) return xnan(Real(0));
    const Real standardized = log_moneyness / width;
    const Real d1 = standardized + Real(0.5) * width, d2 = standardized - Real(0.5) * width;
    const Real asset = weighted_cdf_of(spot, asset_log, sign * d1);
    const Real cash = weighted_cdf_of(strike, risk_log, sign * d2);
    const Real direct = sign * (asset - cash);
    if (xabs(direct) <= xinf(Real(0))) return direct;
    const Real la = log_moneyness + log_normal_cdf_of(sign * d1), lc = log_normal_cdf_of(sign * d2);
    const Real hi = sign > Real(0) ? la : lc, lo = sign > Real(0) ? lc : la;
    const Real difference = hi == -xinf(Real(0)) ? hi : hi + xlog(-xexpm1(lo - hi));
    return xexp(xlog(strike) + risk_log + difference);
}

// log_add (numerics.rs:320-327) and positive_difference (asian.rs:972-985).
template <class Real>
__device__ __forceinline__ Real log_add_of(Real a, Real b) {
    const Real high = a > b ? a : b;
    if (high == -xinf(Real(0))) return high;
    return high + xlog1p(xexp(-xabs(a - b)));
}

template <class Real>
__device__ __forceinline__ Real positive_difference_of(Real a, Real b) {
    if (a == xinf(Real(0))) return a;
    if (b == -xinf(Real(0))) return xexp(a);
    const Real difference = -xexpm1(b - a);
    return difference > Real(0) ? xexp(a + xlog(difference)) : Real(0);
}

constexpr double kHalfLog2Pi = 0.9189385332046727;  // ln(2 pi) / 2

// ArithmeticParameters::geometric_values (asian.rs:1062-1085): the geometric control's
// price, delta or gamma (`output` 0, 1, 2).
template <class Real>
__device__ Real average_geometric_values(const ContractT<Real>& c, Real log_forward, Real log_strike, Real width,
                                         int output) {
    const Real d1 = (log_forward - log_strike) / width + Real(0.5) * width;
    const Real d2 = d1 - width;
    const Real log_asset = log_forward + c.log_discount + log_normal_cdf_of(c.sign * d1);
    if (output == 1) return c.sign * xexp(log_asset - c.avg_log_spot);
    if (output == 2)
        return xexp(log_forward + c.log_discount - Real(2) * c.avg_log_spot - xlog(width) - Real(0.5) * d1 * d1 -
                    Real(kHalfLog2Pi));
    const Real log_cash = log_strike + c.log_discount + log_normal_cdf_of(c.sign * d2);
    return c.sign > Real(0) ? positive_difference_of(log_asset, log_cash) : positive_difference_of(log_cash, log_asset);
}

// ArithmeticParameters::arithmetic without realized history, for widths of at least
// 1e-5 (asian.rs:1087-1178): the first interval integrated in closed form given the
// path's other increments, minus the geometric control on the same path.  Returns the
// price, or the native delta or gamma sample (KGPU_C_OUTPUT_*).
template <class Real>
__device__ __noinline__ Real average_arithmetic_value(const ContractT<Real>& c, Real lead_growth, Real log_sum,
                                                      Real relative_sum, Real geometric_growth) {
    const int output = output_of(c.flags);
    const bool summed = log_sum == -xinf(Real(0));
    const Real log_rest = summed ? c.avg_log_rest + xlog1p(relative_sum / c.avg_rest) : log_sum;
    const Real log_q = ((c.avg_log_scale + lead_growth) + log_rest) + c.avg_interval_forward;
    const Real log_c = (c.avg_log_scale + lead_growth) + c.avg_log_half;
    const Real log_accrued = log_c;  // log_add(no history, log_c)
    Real control = Real(0);
    if (c.flags & KGPU_C_AVERAGE_CONTROL) {
        const Real width = c.control_first_weight * c.avg_width;
        const Real log_forward = (((c.control_log_asset_scale + lead_growth) + geometric_growth) +
                                  c.control_first_weight * c.avg_drift) +
                                 Real(0.5) * width * width;
        control = average_geometric_values(c, log_forward, c.control_log_strike, width, output);
    }
    const Real log_strike = c.avg_log_strike;
    const Real ld = c.log_discount;
    if (log_accrued >= log_strike) {
        if (c.sign < Real(0)) return Real(0) - control;
        if (output == 1) return (xexp(log_q + ld - c.avg_log_spot) + xexp(log_c + ld - c.avg_log_spot)) - control;
        if (output == 2) return Real(0) - control;
        const Real cash = positive_difference_of(log_accrued + ld, log_strike + ld);
        return (xexp(log_q + ld) + cash) - control;
    }
    const Real log_b = log_strike + xlog(-xexpm1(log_accrued - log_strike));
    Real forward = log_q - log_b;
    if (summed) {
        const Real extra = xexpm1(lead_growth) +
                           xexp(lead_growth) * (c.avg_rest * xexpm1(c.avg_interval_forward) +
                                                relative_sum * xexp(c.avg_interval_forward));
        const Real excess = c.avg_baseline + c.avg_weight * extra;
        const Real b = xexp(log_b - c.avg_log_spot);
        if (b > Real(0) && xabs(excess / b) < Real(0.5)) forward = xlog1p(excess / b);
    }
    const Real center = forward / c.avg_width;
    const Real d1 = center + Real(0.5) * c.avg_width, d2 = center - Real(0.5) * c.avg_width;
    if (output == 1)
        return c.sign * (xexp(log_c + ld - c.avg_log_spot + log_normal_cdf_of(c.sign * d2)) +
                         xexp(log_q + ld - c.avg_log_spot + log_normal_cdf_of(c.sign * d1))) -
               control;
    if (output == 2)
        return xexp(ld + Real(2) * log_strike - Real(2) * c.avg_log_spot - log_b - c.greek_log_width -
                    Real(0.5) * d2 * d2 - Real(kHalfLog2Pi)) -
               control;
    const Real log_asset = log_q + ld + log_normal_cdf_of(c.sign * d1);
    const Real log_cash = log_b + ld + log_normal_cdf_of(c.sign * d2);
    const Real price = c.sign > Real(0) ? positive_difference_of(log_asset, log_cash)
                                        : positive_difference_of(log_cash, log_asset);
    return price - control;
}

// GeometricParameters::geometric (asian.rs:740-784): moneyness holds the initial
// moneyness plus the drift, diffusion the width, log_scale the log width.  Returns the
// price, or the native delta or gamma sample.
template <class Real>
__device__ __noinline__ Real average_geometric_value(const ContractT<Real>& c, Real normal) {
    const Real distance = c.moneyness + c.diffusion * normal;
    const Real center = c.moneyness / c.diffusion;
    const Real standardized = center + normal;
    if (c.sign * standardized <= Real(0)) return Real(0);
    const Real log_strike = c.avg_log_strike;
    const int output = output_of(c.flags);
    if (output != 0) {
        const Real log_asset = log_strike + distance + c.log_discount + c.greek_log_weight;
        if (output == 1) return c.sign * xexp(log_asset - c.greek_log_spot);
        const Real numerator = normal - xexp(c.greek_log_base_width);
        if (numerator == Real(0)) return Real(0);
        return c.sign * copysign(xexp(log_asset - Real(2) * c.greek_log_spot + xlog(xabs(numerator)) -
                                      c.greek_log_base_width),
                                 numerator);
    }
    Real log_payoff;
    if (xabs(distance) < Real(1e-5) && xabs(standardized) < xinf(Real(0))) {
        log_payoff = log_strike + c.log_scale + xlog(xabs(standardized)) +
                     (distance == Real(0) ? Real(0) : xlog(xabs(xexpm1(distance)) / xabs(distance)));
    } else if (c.sign > Real(0)) {
        log_payoff = log_strike + distance + xlog(-xexpm1(-distance));
    } else {
        log_payoff = log_strike + xlog(-xexpm1(distance));
    }
    return xexp(log_payoff + c.log_discount);
}

// One image term's contribution to the survival derivatives (double_barrier.rs:37-65).
template <class Real>
__device__ __forceinline__ void image_derivatives(Real exponent, Real weight, Real numerator, Real sign,
                                                  Real inverse_variance, Real ratio, Real* d1, Real* d2) {
    if (numerator == Real(0)) return;
    const Real slope = numerator * inverse_variance;
    const Real first = weight * slope;
    const Real second = first * slope;
    if (xnormal(weight) && xnormal(first) && xnormal(second)) {
        *d1 += sign * first;
        *d2 += sign * second;
    } else {
        // Preserve derivatives when variance or weight underflows.
        const Real log_slope = xlog(xabs(numerator)) - Real(2) * xlog(ratio);
        *d1 += sign * copysign(xexp(exponent + log_slope), numerator);
        *d2 += sign * xexp(exponent + Real(2) * log_slope);
    }
}

// survival (double_barrier.rs:6-112): the probability that a Brownian path from
// `initial` to `terminal` (log distances above the lower barrier) over a standard
// deviation `deviation` stays inside (0, band), and with `derivatives` its first and
// second derivatives in the initial log spot.  Small variances sum the method of images,
// large ones the spectral (sine) series.  NaN when the series does not converge or
// leaves [0, 1] (a computation failure).
template <class Real>
__device__ __noinline__ Real double_survival(Real initial, Real terminal, Real band, Real deviation, bool derivatives,
                                             Real* d1, Real* d2) {
    *d1 = Real(0);
    *d2 = Real(0);
    if (terminal <= Real(0) || terminal >= band) return Real(0);
    Real x = initial / band, y = terminal / band;
    const Real ratio = deviation / band;
    const Real variance = ratio * ratio;
    if (variance == Real(0)) return Real(1);
    if (!(variance > Real(0) && variance < xinf(Real(0)))) return xnan(Real(0));
    const bool reflected = x + y > Real(1);
    if (reflected) {
        x = Real(1) - x;
        y = Real(1) - y;
    }
    Real sum = Real(0);
    bool converged = false;
    if (variance < Real(0.25)) {
        const Real inverse_variance = xnormal(variance) ? Real(1) / variance : xinf(Real(0));
        // The k = 0 terms: the direct one is 1, the reflected one is folded into expm1.
        sum = -xexpm1(Real(-2) * (x / ratio) * (y / ratio));
        if (derivatives) {
            const Real e0 = Real(-2) * ((x + Real(0)) / ratio) * ((y + Real(0)) / ratio);
            image_derivatives(e0, xexp(e0), Real(-2) * (y + Real(0)), Real(-1), inverse_variance, ratio, d1, d2);
        }
        for (int n = 1; n <= 64; ++n) {
            const Real k = Real(n);
            const Real e1 = Real(-2) * (k / ratio) * ((y - x + k) / ratio);
            const Real e2 = Real(-2) * ((x + k) / ratio) * ((y + k) / ratio);
            const Real e3 = Real(-2) * (-k / ratio) * ((y - x - k) / ratio);
            const Real e4 = Real(-2) * ((x - k) / ratio) * ((y - k) / ratio);
            const Real w1 = xexp(e1), w2 = xexp(e2), w3 = xexp(e3), w4 = xexp(e4);
            sum += w1;
            if (derivatives) image_derivatives(e1, w1, Real(2) * k, Real(1), inverse_variance, ratio, d1, d2);
            sum -= w2;
            if (derivatives) image_derivatives(e2, w2, Real(-2) * (y + k), Real(-1), inverse_variance, ratio, d1, d2);
            sum += w3;
            if (derivatives) image_derivatives(e3, w3, Real(2) * -k, Real(1), inverse_variance, ratio, d1, d2);
            sum -= w4;
            if (derivatives) image_derivatives(e4, w4, Real(-2) * (y - k), Real(-1), inverse_variance, ratio, d1, d2);
            if (n >= 2 && ((w1 + w2) + w3) + w4 < Real(1e-18)) {
                converged = true;
                break;
            }
        }
    } else {
        const Real distance = y - x;
        const Real log_scale = xlog(Real(2) * Real(2.5066282746310002) * ratio) + Real(0.5) * distance * distance / variance;
        for (int n = 1; n <= 256; ++n) {
            const Real frequency = Real(n) * Real(3.141592653589793);
            const Real exponent = log_scale - Real(0.5) * frequency * frequency * variance;
            const Real weight = xexp(exponent);
            const Real sy = xsin(frequency * y);
            const Real product = xsin(frequency * x) * sy;
            sum += weight * product;
            if (derivatives) {
                const Real first = frequency * cos(frequency * x) * sy;
                const Real score = -distance / variance;
                *d1 += weight * (first + score * product);
                *d2 += weight * (Real(2) * score * first + (score * score + Real(1) / variance - frequency * frequency) * product);
            }
            if (n >= 4 && exponent + Real(4) * xlog(frequency) < Real(-40)) {
                converged = true;
                break;
            }
        }
    }
    if (!converged || !(sum >= Real(-1e-13) && sum <= Real(1) + Real(1e-13))) return xnan(Real(0));
    if (derivatives) {
        *d1 = (reflected ? -*d1 : *d1) / band;
        *d2 = (*d2 / band) / band;
    }
    return sum < Real(0) ? Real(0) : (sum > Real(1) ? Real(1) : sum);
}

// The continuous double barrier's sample (barrier.rs:341-390), value only.
template <class Real>
__device__ __noinline__ Real double_barrier_value(const ContractT<Real>& c, Real z) {
    const Real noise = xfma(c.diffusion, z, Real(0));
    const Real terminal = c.barrier_drift + noise;
    const Real distance = c.moneyness + noise;
    const Real payoff = xabs(distance) < Real(0.5) ? c.strike * xexpm1(distance)
                                                   : weighted_amount(c.spot, terminal) - c.strike;
    Real intrinsic = c.sign * payoff;
    intrinsic = intrinsic > Real(0) ? intrinsic : Real(0);
    const int output = output_of(c.flags);
    Real ds1, ds2;
    const Real survival =
        double_survival(c.band_initial, c.barrier_moneyness + noise, c.band, c.diffusion, output != 0, &ds1, &ds2);
    const bool in = (c.flags & KGPU_C_BARRIER_IN) != 0;
    const Real rebate = (!in && (c.flags & KGPU_C_REBATE_AT_HIT)) ? Real(0) : c.rebate;
    const Real log_survival = xlog(survival), log_hit = xlog1p(-survival);
    const Real value = weighted_amount(intrinsic, c.log_discount + (in ? log_hit : log_survival)) +
                       weighted_amount(rebate, c.log_discount + (in ? log_survival : log_hit));
    if (output == 0) return value;
    // derivative(weight) of barrier.rs:366-372
    const Real difference = (in ? Real(-1) : Real(1)) * (intrinsic - rebate);
    const Real ad = xabs(difference), sd = difference < Real(0) ? Real(-1) : Real(1);
    const Real first =
        weighted_amount(ad * (sd * (ds1 < Real(0) ? Real(-1) : Real(1))), c.log_discount + xlog(xabs(ds1)));
    const Real second = output == 2 ? weighted_amount(ad * (sd * (ds2 < Real(0) ? Real(-1) : Real(1))),
                                                      c.log_discount + xlog(xabs(ds2)))
                                    : Real(0);
    return likelihood_greek(output, value, first, second, z, c.diffusion, c.spot);
}

template <class Real>
struct PlanPtrs {
    const StepT<Real>* __restrict__ steps;
    const uint8_t* __restrict__ flags;
    const EventT<Real>* __restrict__ events;
    const IntervalT<Real>* __restrict__ intervals;
    const DailyT<Real>* __restrict__ daily;
    const UnitT<Real>* __restrict__ units;
    const EndT<Real>* __restrict__ ends;
};

template <class Real>
__device__ __forceinline__ PlanPtrs<Real> plan_of(const DevBook<Real>& b, const ContractT<Real>& c) {
    PlanPtrs<Real> p;
    p.steps = b.steps + c.step_offset;
    p.flags = b.flags + c.step_offset;
    p.events = b.events ? b.events + c.event_offset : nullptr;
    p.intervals = b.intervals ? b.intervals + c.bridge_offset : nullptr;
    p.daily = b.daily ? b.daily + c.step_offset : nullptr;
    p.units = b.units ? b.units + c.step_offset : nullptr;
    p.ends = b.ends ? b.ends + c.step_offset : nullptr;
    return p;
}

// Advances one path by one unit of work (a grid step, or a bridge interval end).
template <class Real, int MODEL, class Source>
__device__ __forceinline__ bool grid_step(const DevModel<Real>& m, const ContractT<Real>& c,
                                          const PlanPtrs<Real>& p, PathState<Real>& s, Source& n,
                                          Real& value);

// Returns true when the path has finished; its payoff is then in `value`.
// EXT: the extended payoff set (scheduled barriers, continuous averages) is compiled in.
template <class Real, int MODEL, bool EXT = true, class Source>
__device__ __forceinline__ bool path_step(const DevModel<Real>& m, const ContractT<Real>& c,
                                          const PlanPtrs<Real>& p, PathState<Real>& s, Source& n,
                                          Real& value) {
    const int payoff = c.payoff;
    // The grid-stepping families first: they take a step per call, the others mostly one
    // call per path.
    if (payoff == KGPU_PAYOFF_VANILLA_PATH || payoff == KGPU_PAYOFF_ASIAN || payoff == KGPU_PAYOFF_ACCUMULATOR ||
        (payoff == KGPU_PAYOFF_AUTOCALLABLE && !(c.flags & KGPU_C_BRIDGE)))
        return grid_step<Real, MODEL>(m, c, p, s, n, value);
    if (payoff == KGPU_PAYOFF_AUTOCALLABLE && (c.flags & KGPU_C_BRIDGE)) {
        // bridge_payoffs::<1, true>: the interval end is drawn first, then daily bridge
        // steps until knock-in is decided, then the interval end.  Each call evaluates at
        // most one normal, at a single call site, so lanes in different phases of their
        // paths still share the quantile evaluation.
        const Real level = c.knock_in;
        const bool begin = s.end < 0;
        const bool daily = !begin && s.i < s.end && s.monitoring && !(s.minimum < level);
        const Real z = n.normal_if(begin || daily);
        if (begin) {
            const IntervalT<Real> iv = p.intervals[s.k];
            s.target = s.lr + xfma(iv.diffusion, z, iv.drift);
            s.minimum = xinf(Real());
            s.end = iv.end;
            if (s.i < s.end && s.monitoring) return false;
        } else if (daily) {
            const DailyT<Real> d = p.daily[s.i];
            s.lr = s.lr + xfma(d.weight, s.target - s.lr, d.width * z);
            s.minimum = s.lr < s.minimum ? s.lr : s.minimum;
            ++s.i;
            ++s.executed;
            if (s.i < s.end) return false;
        }
        if (s.i < s.end) {
            // knock-in decided (or never monitored): skip the interval's daily normals
            n.skip(s.end - s.i);
            s.i = s.end;
        }
        // interval end
        const int end = s.end;
        s.lr = s.target;
        s.end = -1;
        ++s.executed;
        const uint8_t fl = p.flags[end];
        if (s.monitoring && (s.minimum < level || ((fl & KGPU_STEP_KNOCK_IN) && s.lr < level))) {
            s.monitoring = false;
            s.knocked_in = true;
        }
        s.i = end + 1;
        s.k += 1;
        if (fl & KGPU_STEP_EVENT) {
            const EventT<Real>& e = p.events[s.ev++];
            const bool hit = e.has_knock_out && s.lr >= e.knock_out;
            s.cash += e.payment[int(s.lr >= e.coupon_barrier) | (int(hit) << 1)];
            if (hit) {
                value = s.cash;
                return true;
            }
        }
        if (s.k < c.bridge_count) return false;
        const bool hit = s.knocked_in ||
                         ((c.flags & KGPU_C_EXPIRY_KNOCK_IN) && (c.flags & KGPU_C_HAS_KNOCK_IN) && s.lr < level);
        value = s.cash + autocallable_terminal(c, spot_at(c.spot, s.lr), hit) * c.final_discount;
        return true;
    }
    if (payoff == KGPU_PAYOFF_EUROPEAN) {
        value = european_value(c, n.normal());
        s.executed = 1;
        return true;
    }
    if (payoff == KGPU_PAYOFF_DIGITAL) {
        value = digital_value(c, n.normal());
        s.executed = 1;
        return true;
    }
    if (payoff == KGPU_PAYOFF_BARRIER) {
        value = barrier_value(c, n.normal());
        s.executed = 1;
        return true;
    }
    if (EXT && payoff == KGPU_PAYOFF_DOUBLE_BARRIER) {
        value = double_barrier_value(c, n.normal());
        s.executed = 1;
        return true;
    }
    if (EXT && payoff == KGPU_PAYOFF_AVERAGE_GEOMETRIC) {
        value = average_geometric_value(c, n.normal());
        s.executed = 1;
        return true;
    }
    if (EXT && payoff == KGPU_PAYOFF_AVERAGE_ARITHMETIC) {
        // ArithmeticGrid::path (asian.rs:636-711): one normal per interval after the
        // first; the last one carries the end fixing's half weight.
        const Real z = n.normal();
        const int i = s.i;
        s.i = i + 1;
        s.executed += 1;
        if (i == 0 && (c.flags & KGPU_C_AVERAGE_LEAD)) {
            s.minimum = c.avg_lead_drift + c.avg_lead_width * z;
        } else {
            const Real growth = s.lr + (c.avg_drift + c.avg_width * z);
            s.lr = growth;
            const Real fraction = s.i == c.step_count ? c.avg_half : c.avg_fraction;
            if (c.flags & KGPU_C_AVERAGE_CONTROL) s.target += fraction * growth;
            const Real growth_bound = sizeof(Real) == 8 ? Real(600) : Real(80);
            if (growth > growth_bound || s.cash != -xinf(Real(0))) {
                // Above the bound, unit offsets fall below the type's precision.
                if (s.cash == -xinf(Real(0))) s.cash = xlog(c.avg_rest + s.acc);
                s.cash = log_add_of(s.cash, (s.i == c.step_count ? c.avg_log_half : c.avg_log_fraction) + growth);
            } else {
                s.acc += fraction * xexpm1(growth);
            }
        }
        if (s.i < c.step_count) return false;
        value = average_arithmetic_value(c, s.minimum, s.cash, s.acc, s.target);
        return true;
    }
    if (EXT && payoff == KGPU_PAYOFF_BARRIER_DISCRETE) {
        // Scheduled monitoring (barrier.rs:306-449): the noise sum(width z) against each
        // observed date's touch level; a knock-out stops at its hit, a knock-in with more
        // than 8 dates left is priced analytically from its hit.
        const int i = s.i;
        const StepT<Real> st = p.steps[i];
        const Real z = n.normal();
        if (i == 0) s.v = z;  // the first normal carries the likelihood-ratio score
        s.lr = xfma(st.diffusion, z, s.lr);
        s.i = i + 1;
        s.executed += 1;
        // Native delta / gamma samples: the first normal's score (barrier.rs:455-470).
        const auto finish = [&]() {
            const int output = output_of(c.flags);
            if (output != 0)
                value = likelihood_greek(output, value, Real(0), Real(0), s.v, p.steps[0].diffusion, c.spot);
            return true;
        };
        if (c.flags & KGPU_C_CHECK_STEPS) {
            const Real spot_now = weighted_amount(c.spot, st.drift + s.lr);
            if (!(spot_now > Real(0) && spot_now < xinf(Real(0)))) {
                value = xnan(Real(0));  // unrepresentable path: reported as a computation failure
                return true;
            }
        }
        const EventT<Real> e = p.events[i];
        const bool in = (c.flags & KGPU_C_BARRIER_IN) != 0;
        const bool touched_now = (c.flags & KGPU_C_DOUBLE) ? (s.lr <= e.knock_out || s.lr >= e.payment[3])
                                 : (c.flags & KGPU_C_BARRIER_UP) ? s.lr >= e.knock_out
                                                                 : s.lr <= e.knock_out;
        if (e.has_knock_out && touched_now) {
            s.knocked_in = true;  // touched
            if ((c.flags & KGPU_C_CONDITION_ON_HIT) && c.step_count - i > 8) {
                const Real asset = weighted_amount(c.spot, st.drift + s.lr);
                value = lognormal_price_of(asset, c.strike, c.moneyness + s.lr + c.half_variance * e.coupon_barrier,
                                           e.payment[1], c.log_discount, c.volatility, e.payment[2], c.sign);
                return finish();
            }
            if (!in) {
                value = weighted_amount(c.rebate, (c.flags & KGPU_C_REBATE_AT_HIT) ? e.payment[0] : c.log_discount);
                return finish();
            }
        }
        if (s.i < c.step_count) return false;
        const Real asset = weighted_amount(c.spot, st.drift + s.lr);
        const Real distance = c.moneyness + s.lr;
        const Real payoff_value = xabs(distance) < Real(0.5) ? c.strike * xexpm1(distance) : asset - c.strike;
        Real intrinsic = c.sign * payoff_value;
        intrinsic = intrinsic > Real(0) ? intrinsic : Real(0);
        value = weighted_amount(s.knocked_in == in ? intrinsic : c.rebate, c.log_discount);
        return finish();
    }
    // Grid-stepping families.
    return grid_step<Real, MODEL>(m, c, p, s, n, value);
}

// The per-step rule of an Asian on its fixings (the spot added at each fixing step) and of
// a vanilla path (none).
template <class Real>
__device__ __forceinline__ void fixing_rule(const ContractT<Real>& c, uint8_t fl, PathState<Real>& s) {
    if (c.payoff == KGPU_PAYOFF_ASIAN && (fl & KGPU_STEP_FIXING)) {
        s.acc += spot_at(c.spot, s.lr);
        s.fixings += 1;
    }
}

// Their payoff after the last step: the call or put on the fixings' average (Asian) or on
// the terminal spot (vanilla path), discounted.
template <class Real>
__device__ __forceinline__ Real fixing_value(const ContractT<Real>& c, const PathState<Real>& s) {
    Real underlying = c.payoff == KGPU_PAYOFF_ASIAN ? s.acc / Real(s.fixings) : spot_at(c.spot, s.lr);
    Real x = c.sign * (underlying - c.strike);
    return (x > Real(0) ? x : Real(0)) * c.final_discount;
}

// One grid step of the grid-stepping families (vanilla path, Asian on fixings, forward
// autocallable, accumulator): model step, then the family's per-step rule.
template <class Real, int MODEL, class Source>
__device__ __forceinline__ bool grid_step(const DevModel<Real>& m, const ContractT<Real>& c,
                                          const PlanPtrs<Real>& p, PathState<Real>& s, Source& n,
                                          Real& value) {
    const int payoff = c.payoff;
    const int i = s.i;
    const StepT<Real> st = p.steps[i];
    model_step<Real, MODEL>(m, st, s, n);
    const uint8_t fl = p.flags[i];
    s.i = i + 1;
    s.executed += 1;
    const bool last = s.i == c.step_count;
    if (payoff == KGPU_PAYOFF_AUTOCALLABLE) {
        if (fl & KGPU_STEP_KNOCK_IN) s.knocked_in |= (c.flags & KGPU_C_HAS_KNOCK_IN) && s.lr < c.knock_in;
        if (fl & KGPU_STEP_EVENT) {
            const EventT<Real>& e = p.events[s.ev++];
            const bool coupon_due = s.lr >= e.coupon_barrier;
            const bool knocked_out = e.has_knock_out && s.lr >= e.knock_out;
            s.cash += e.payment[int(coupon_due) | (int(knocked_out) << 1)];
            if (knocked_out) {
                value = s.cash;
                return true;
            }
        }
        if (!last) return false;
        const bool ki = s.knocked_in || ((c.flags & KGPU_C_EXPIRY_KNOCK_IN) &&
                                         (c.flags & KGPU_C_HAS_KNOCK_IN) && s.lr < c.knock_in);
        value = s.cash + autocallable_terminal(c, spot_at(c.spot, s.lr), ki) * c.final_discount;
        return true;
    }
    if (payoff == KGPU_PAYOFF_ACCUMULATOR) {
        const Real sign = c.sign;
        auto unit = [&](Real lr) {
            Real distance = lr - c.log_strike;
            if (xabs(distance) < Real(0.5)) return sign * c.strike * xexpm1(distance);
            Real spot = spot_at(c.spot, lr);
            return sign > Real(0) ? spot - c.strike : c.strike - spot;
        };
        if ((fl & KGPU_STEP_EVENT) && sign * s.lr >= sign * c.knock_out) {
            value = s.acc * unit(s.lr) * st.discount;
            return true;
        }
        if (fl & KGPU_STEP_ACCUMULATE)
            s.acc += c.daily_quantity * (sign * s.lr < sign * c.log_strike ? c.acceleration : Real(1));
        if (!last) return false;
        value = s.acc * unit(s.lr) * c.final_discount;
        return true;
    }
    fixing_rule(c, fl, s);
    if (!last) return false;
    value = fixing_value(c, s);
    return true;
}

// The bridged autocallable as one uniform unit of work per path position (persistent
// kernels).  Same arithmetic and normal positions as the bridge branch of path_step: a
// unit is the interval-end draw (the interval's first position) or one daily bridge
// step.  Every call evaluates one normal and both unit formulas and selects; when the
// interval's end is due (its last position, or knock-in decided so the remaining daily
// normals are skipped) the interval end is settled in the same call, with selects and
// predicated loads rather than a separate phase, so lanes at different positions of
// their paths stay converged.  Returns true when the path has finished.
template <class Real, class Source>
__device__ __forceinline__ bool bridge_unit_step(const ContractT<Real>& c, const PlanPtrs<Real>& p,
                                                 PathState<Real>& s, Source& n) {
    const int q = s.i;
    const UnitT<Real> u = p.units[q];
    const Real z = n.normal();
    const bool begin = (u.flags & kUnitBegin) != 0;
    const Real target = s.lr + xfma(u.a, z, u.b);
    const Real daily = s.lr + xfma(u.b, s.target - s.lr, u.a * z);
    s.target = begin ? target : s.target;
    s.lr = begin ? s.lr : daily;
    s.minimum = begin ? xinf(Real()) : (daily < s.minimum ? daily : s.minimum);
    s.executed += 1;
    const Real level = c.knock_in;
    const bool due = (u.flags & kUnitLast) || !s.monitoring || s.minimum < level;
    // Interval end, evaluated with selects: skip the remaining daily normals, settle
    // knock-in and the cash event.  Lanes without an event read one shared record.
    const int end = u.end;
    const int next = due ? end + 1 : q + 1;
    n.skip(next - (q + 1));
    s.i = next;
    const Real lr = due ? s.target : s.lr;
    s.lr = lr;
    const int fl = u.flags >> 8;
    const bool ki = due && s.monitoring && (s.minimum < level || ((fl & KGPU_STEP_KNOCK_IN) && lr < level));
    s.knocked_in = s.knocked_in || ki;
    s.monitoring = s.monitoring && !ki;
    bool hit = false;
    if (due && (fl & KGPU_STEP_EVENT)) {
        const EndT<Real> e = p.ends[end];
        hit = (u.flags & kUnitKnockOut) && lr >= e.knock_out;
        const bool coupon = lr >= e.coupon_barrier;
        s.cash += hit ? (coupon ? e.payment[3] : e.payment[2]) : (coupon ? e.payment[1] : e.payment[0]);
    }
    s.knocked_out = hit;
    return due && (hit || end + 1 >= c.step_count);
}

// Payoff of a finished bridged path: the cash collected, plus the discounted terminal
// redemption when the note reached expiry (discounted_terminal, autocallable.rs:797).
template <class Real>
__device__ __forceinline__ Real bridge_value(const DevModel<Real>& m, const ContractT<Real>& c,
                                             const PathState<Real>& s) {
    if (s.knocked_out) return s.cash;
    const bool in = s.knocked_in || ((c.flags & KGPU_C_EXPIRY_KNOCK_IN) && (c.flags & KGPU_C_HAS_KNOCK_IN) &&
                                     s.lr < c.knock_in);
    return s.cash + autocallable_terminal(c, spot_at(c.spot, s.lr), in) * c.final_discount;
}

// Scaled Welford moments (monte_carlo.rs:2155-2222), used by the plain schedule.
struct Moments {
    double count, scale, mean, m2;
};

__device__ __forceinline__ void moments_add(Moments& m, double value, bool variance) {
    double a = fabs(value);
    if (a > m.scale) {
        double ratio = m.scale / a;
        m.mean = m.mean * ratio;
        if (variance) m.m2 = m.m2 * (ratio * ratio);
        m.scale = a;
    }
    m.count += 1.0;
    double v = m.scale == 0.0 ? 0.0 : value / m.scale;
    double delta = v - m.mean;
    m.mean = m.mean + delta / m.count;
    if (variance) m.m2 = m.m2 + delta * (v - m.mean);
}

__device__ __forceinline__ void moments_merge(Moments& a, const Moments& b, bool variance) {
    if (a.count == 0.0) {
        a = b;
        return;
    }
    double sc = a.scale > b.scale ? a.scale : b.scale;
    double left = sc == 0.0 ? 0.0 : a.scale / sc;
    double right = sc == 0.0 ? 0.0 : b.scale / sc;
    double delta = b.mean * right - a.mean * left;
    double total = a.count + b.count;
    a.mean = a.mean * left + delta * (b.count / total);
    if (variance)
        a.m2 = a.m2 * left * left + b.m2 * right * right + delta * delta * (a.count * (b.count / total));
    a.count = total;
    a.scale = sc;
}

}  // namespace kgpu
