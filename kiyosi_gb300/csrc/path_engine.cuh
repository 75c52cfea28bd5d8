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
#pragma once
#include <cstdint>

#include "../../include/kgpu.h"
#include "device_rng.cuh"

namespace kgpu {

// Device view of the book (device pointers).
struct DevBook {
    const kgpu_contract* contracts;
    const kgpu_step* steps;
    const uint8_t* flags;
    const kgpu_event* events;
    const kgpu_bridge_interval* intervals;
    const kgpu_bridge_daily* daily;
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
template <class Real>
struct PcgSource {
    Pcg g;
    Real spare;
    bool has_spare;

    __device__ __forceinline__ void draw(Real& c, Real& s) {
        uint64_t b1 = pcg_bits52(g);
        uint64_t b2 = pcg_bits52(g);
        box_muller(b1, b2, &c, &s);
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

// Sobol point: bits of dimension d are high[d] ^ XOR_{c in low gray bits} low[c*D + d],
// where high[] holds the shift and the directions of the gray-code bits shared by the
// 256 points of one reference block (bits >= 8), and low[] the first 8 direction rows.
template <class Real>
struct SobolSource {
    const uint64_t* high;
    const uint64_t* low;
    int dims;
    int used;
    uint32_t gray_low;

    __device__ __forceinline__ void start(uint64_t sample) {
        uint64_t gray = sample ^ (sample >> 1);
        gray_low = uint32_t(gray & 0xFF);
        used = 0;
    }
    __device__ __forceinline__ uint64_t bits(int d) const {
        uint64_t x = high[d];
        uint32_t g = gray_low;
        while (g) {
            int c = __ffs(g) - 1;
            x ^= low[c * dims + d];
            g &= g - 1;
        }
        return x;
    }
    __device__ __forceinline__ Real normal() { return sobol_normal(bits(used++), Real()); }
    __device__ __forceinline__ void skip(int remaining) {
        if (remaining > 0) used += remaining;
    }
};

// ------------------------------------------------------------------------------------
// Arithmetic helpers: FP64 keeps the reference's rounding; FP32 uses fast intrinsics.
// ------------------------------------------------------------------------------------
__device__ __forceinline__ double xexp(double x) { return exp(x); }
__device__ __forceinline__ float xexp(float x) { return __expf(x); }
__device__ __forceinline__ double xexpm1(double x) { return expm1(x); }
__device__ __forceinline__ float xexpm1(float x) { return expm1f(x); }
__device__ __forceinline__ double xsqrt(double x) { return sqrt(x); }
__device__ __forceinline__ float xsqrt(float x) { return sqrtf(x); }

// scaled_value(initial, 1, log_return) for ordinary magnitudes (numerics.rs:226-238).
template <class Real>
__device__ __forceinline__ Real spot_at(Real initial, Real log_return) {
    return initial * xexp(log_return);
}

// LocalVolatilitySurface::at_year (market/local_volatility.rs:322-359)
template <class Real>
__device__ __forceinline__ void lv_bracket(const Real* nodes, int n, Real value, int& left,
                                           Real& weight) {
    // partition_point(node <= value) - 1, clamped to [0, n-2]
    int lo = 0, hi = n;
    while (lo < hi) {
        int mid = (lo + hi) >> 1;
        if (nodes[mid] <= value)
            lo = mid + 1;
        else
            hi = mid;
    }
    int l = lo - 1;
    l = l < 0 ? 0 : (l > n - 2 ? n - 2 : l);
    Real w = (value - nodes[l]) / (nodes[l + 1] - nodes[l]);
    weight = w < Real(0) ? Real(0) : (w > Real(1) ? Real(1) : w);
    left = l;
}

template <class Real>
__device__ __forceinline__ Real lv_interpolate(Real low, Real high, Real weight) {
    return weight <= Real(0.5) ? low + weight * (high - low) : high + (Real(1) - weight) * (low - high);
}

template <class Real>
__device__ __forceinline__ Real lv_at(const DevModel<Real>& m, Real time, Real spot) {
    const Real* years = m.lv;
    const Real* spots = m.lv + m.nt;
    const Real* values = m.lv + m.nt + m.ns;
    int row, col;
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
    int fixings;
    int executed;  // grid steps simulated
    bool knocked_in;
    bool monitoring;
    bool in_interval;
};

template <class Real>
__device__ __forceinline__ void path_init(PathState<Real>& s, const kgpu_contract& c, Real v0) {
    s.lr = Real(0);
    s.v = v0;
    s.acc = Real(c.payoff == KGPU_PAYOFF_ACCUMULATOR ? c.quantity : 0.0);
    s.cash = Real(c.initial_cash);
    s.target = Real(0);
    s.minimum = Real(0);
    s.i = 0;
    s.ev = 0;
    s.k = 0;
    s.fixings = 0;
    s.executed = 0;
    s.knocked_in = (c.flags & KGPU_C_KNOCKED_IN) != 0;
    s.monitoring = !s.knocked_in && (c.flags & KGPU_C_HAS_KNOCK_IN);
    s.in_interval = false;
}

// One grid step of the state.  BSM: `log_return += diffusion.mul_add(normal, drift)`;
// Heston: full-truncation Euler in log spot (two normals per step: spot, then the
// independent variance shock); local volatility: Euler in log spot with the surface
// read at the step's start.
template <class Real, int MODEL, class Source>
__device__ __forceinline__ void model_step(const DevModel<Real>& m, const kgpu_step& st,
                                           PathState<Real>& s, Source& n) {
    if (MODEL == KGPU_MODEL_BSM) {
        Real t = fma(Real(st.diffusion), n.normal(), Real(st.drift));
        s.lr = s.lr + t;
    } else if (MODEL == KGPU_MODEL_HESTON) {
        Real z1 = n.normal();
        Real z2 = n.normal();
        Real dt = Real(st.drift), sq = Real(st.diffusion);
        Real vp = s.v > Real(0) ? s.v : Real(0);
        Real sv = xsqrt(vp) * sq;
        Real zv = m.rho * z1 + m.rho_bar * z2;
        s.lr += (m.rate - m.dividend - Real(0.5) * vp) * dt + sv * z1;
        s.v += m.kappa * (m.theta - vp) * dt + m.xi * sv * zv;
    } else {
        Real spot = m.spot * xexp(s.lr);
        Real sigma = lv_at(m, Real(st.time), spot);
        Real dt = Real(st.drift), sq = Real(st.diffusion);
        s.lr += (m.rate - m.dividend - Real(0.5) * sigma * sigma) * dt + sigma * sq * n.normal();
    }
}

// AutocallableNote::terminal (instruments/autocallable.rs:1396-1414)
template <class Real>
__device__ __forceinline__ Real autocallable_terminal(const kgpu_contract& c, Real spot, bool ki) {
    if (ki) {
        if (c.flags & KGPU_C_DOWNSIDE) {
            Real lower = Real(c.downside_lower), upper = Real(c.downside_upper);
            Real clamped = spot < lower ? lower : (spot > upper ? upper : spot);
            return Real(c.terminal_base) + (clamped - upper) / Real(c.downside_initial);
        }
        return Real(c.terminal_fixed);
    }
    return Real(c.terminal_plain);
}

template <class Real>
__device__ __forceinline__ Real european_value(const kgpu_contract& c, Real z) {
    Real distance = fma(Real(c.diffusion), z, Real(c.moneyness));
    if (Real(c.sign) * distance <= Real(0)) return Real(0);
    if (c.sign < 0.0) return -xexpm1(distance);
    return -xexpm1(-distance) * xexp(fma(Real(c.diffusion), z, -Real(c.half_variance)));
}

template <class Real>
__device__ __forceinline__ Real digital_value(const kgpu_contract& c, Real z) {
    Real distance = Real(c.moneyness) + z;
    bool call = c.sign > 0.0;
    if (!(call ? distance > Real(0) : distance < Real(0))) return Real(0);
    Real exponent = Real(c.log_scale) + ((c.flags & KGPU_C_ASSET_DIGITAL) ? Real(c.diffusion) * z : Real(0));
    return Real(c.strike) * xexp(exponent);
}

// Advances one path by one unit of work (a grid step, or a bridge interval end).
// Returns true when the path has finished; its payoff is then in `value`.
template <class Real, int MODEL, class Source>
__device__ __forceinline__ bool path_step(const DevModel<Real>& m, const kgpu_contract& c,
                                          const kgpu_step* __restrict__ steps,
                                          const uint8_t* __restrict__ flags,
                                          const kgpu_event* __restrict__ events,
                                          const kgpu_bridge_interval* __restrict__ intervals,
                                          const kgpu_bridge_daily* __restrict__ daily,
                                          PathState<Real>& s, Source& n, Real& value) {
    const int payoff = c.payoff;
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
    if (payoff == KGPU_PAYOFF_AUTOCALLABLE && (c.flags & KGPU_C_BRIDGE)) {
        // bridge_payoffs::<1, true>: interval end drawn first, then daily bridge steps
        // until knock-in is decided, then the interval end.
        const kgpu_bridge_interval iv = intervals[s.k];
        const Real level = Real(c.knock_in);
        if (!s.in_interval) {
            s.target = s.lr + fma(Real(iv.diffusion), n.normal(), Real(iv.drift));
            s.minimum = Real(__int_as_float(0x7f800000));
            s.in_interval = true;
        }
        if (s.i < iv.end) {
            if (!s.monitoring || s.minimum < level) {
                n.skip(iv.end - s.i);
                s.i = iv.end;
            } else {
                Real z = n.normal();
                const kgpu_bridge_daily d = daily[s.i];
                s.lr = s.lr + fma(Real(d.weight), s.target - s.lr, Real(d.width) * z);
                s.minimum = s.lr < s.minimum ? s.lr : s.minimum;
                ++s.i;
                ++s.executed;
                if (s.i < iv.end) return false;
            }
        }
        // interval end
        s.lr = s.target;
        s.in_interval = false;
        ++s.executed;
        const uint8_t fl = flags[iv.end];
        if (s.monitoring && (s.minimum < level || ((fl & KGPU_STEP_KNOCK_IN) && s.lr < level))) {
            s.monitoring = false;
            s.knocked_in = true;
        }
        s.i = iv.end + 1;
        s.k += 1;
        if (fl & KGPU_STEP_EVENT) {
            const kgpu_event& e = events[s.ev++];
            bool hit = e.has_knock_out && s.lr >= Real(e.knock_out);
            s.cash += Real(e.payment[int(s.lr >= Real(e.coupon_barrier)) | (int(hit) << 1)]);
            if (hit) {
                value = s.cash;
                return true;
            }
        }
        if (s.k < c.bridge_count) return false;
        bool hit = s.knocked_in ||
                   ((c.flags & KGPU_C_EXPIRY_KNOCK_IN) && (c.flags & KGPU_C_HAS_KNOCK_IN) && s.lr < level);
        value = s.cash + autocallable_terminal(c, spot_at(m.spot, s.lr), hit) * Real(c.final_discount);
        return true;
    }
    // Grid-stepping families.
    const int i = s.i;
    const kgpu_step st = steps[i];
    model_step<Real, MODEL>(m, st, s, n);
    const uint8_t fl = flags[i];
    s.i = i + 1;
    s.executed += 1;
    const bool last = s.i == c.step_count;
    if (payoff == KGPU_PAYOFF_AUTOCALLABLE) {
        if (fl & KGPU_STEP_KNOCK_IN)
            s.knocked_in |= (c.flags & KGPU_C_HAS_KNOCK_IN) && s.lr < Real(c.knock_in);
        if (fl & KGPU_STEP_EVENT) {
            const kgpu_event& e = events[s.ev++];
            bool coupon_due = s.lr >= Real(e.coupon_barrier);
            bool knocked_out = e.has_knock_out && s.lr >= Real(e.knock_out);
            s.cash += Real(e.payment[int(coupon_due) | (int(knocked_out) << 1)]);
            if (knocked_out) {
                value = s.cash;
                return true;
            }
        }
        if (!last) return false;
        bool ki = s.knocked_in || ((c.flags & KGPU_C_EXPIRY_KNOCK_IN) &&
                                   (c.flags & KGPU_C_HAS_KNOCK_IN) && s.lr < Real(c.knock_in));
        value = s.cash + autocallable_terminal(c, spot_at(m.spot, s.lr), ki) * Real(c.final_discount);
        return true;
    }
    if (payoff == KGPU_PAYOFF_ACCUMULATOR) {
        const Real sign = Real(c.sign);
        auto unit = [&](Real lr) {
            Real distance = lr - Real(c.log_strike);
            if (fabs(distance) < Real(0.5)) return sign * Real(c.strike) * xexpm1(distance);
            Real spot = spot_at(m.spot, lr);
            return c.sign > 0.0 ? spot - Real(c.strike) : Real(c.strike) - spot;
        };
        if ((fl & KGPU_STEP_EVENT) && sign * s.lr >= sign * Real(c.knock_out)) {
            value = s.acc * unit(s.lr) * Real(st.discount);
            return true;
        }
        if (fl & KGPU_STEP_ACCUMULATE)
            s.acc += Real(c.daily_quantity) *
                     (sign * s.lr < sign * Real(c.log_strike) ? Real(c.acceleration) : Real(1));
        if (!last) return false;
        value = s.acc * unit(s.lr) * Real(c.final_discount);
        return true;
    }
    if (payoff == KGPU_PAYOFF_ASIAN && (fl & KGPU_STEP_FIXING)) {
        s.acc += spot_at(m.spot, s.lr);
        s.fixings += 1;
    }
    if (!last) return false;
    Real underlying = payoff == KGPU_PAYOFF_ASIAN ? s.acc / Real(s.fixings) : spot_at(m.spot, s.lr);
    Real x = Real(c.sign) * (underlying - Real(c.strike));
    value = (x > Real(0) ? x : Real(0)) * Real(c.final_discount);
    return true;
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
