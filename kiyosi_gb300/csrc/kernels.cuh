// Plain and persistent Monte Carlo kernels (templates; instantiated per precision in
// kernels_fp64.cu, compiled with --fmad=false, and kernels_fp32.cu).
#pragma once
#include <cstdint>

#include "path_engine.cuh"

namespace kgpu {

constexpr int kThreads = 256;  // one CUDA block = one reference block of 256 samples
constexpr int kWarps = kThreads / 32;
// Path units a warp runs in lockstep between lane refills (persistent kernel).
constexpr int kRefill = 16;

// Partial result of one reference block (plain schedule).
struct BlockPartial {
    Moments moments;   // merged like the reference (variance only when it has one)
    Moments pairs;     // antithetic pair means
    Moments sample;    // i.i.d. moments with variance, for the sample error
    double executed;
};

// Partial sums of one work item (persistent schedule).
struct TilePartial {
    double sum, sumsq, count, executed;
};

// Sobol tables of one sequence: directions [column * dims + dim], shifts [dim] and the
// 4-bit nibble XOR tables of direction rows 0-7, [dim][32].
struct SobolTables {
    const uint64_t* directions;
    const uint64_t* shifts;
    const uint64_t* nibbles;
    const uint32_t* directions32;  // top 32 of the 52 bits, same layouts
    const uint32_t* shifts32;
    const uint32_t* nibbles32;
    const uint32_t* high32;  // [block][dims]: the high part of every reference block in use
    int dims;
};

// The caller's plan (kgpu_* arrays, device pointers).
struct RawBook {
    const kgpu_contract* contracts;
    const kgpu_step* steps;
    const uint8_t* flags;
    const kgpu_event* events;
    const kgpu_bridge_interval* intervals;
    const kgpu_bridge_daily* daily;
    int contract_count;
    int64_t step_total;
    int event_total, interval_total;
};

template <class Real>
struct PlainArgs {
    DevBook<Real> book;
    int contract;
    int dims;
    int64_t paths;
    int64_t samples;
    uint64_t seed;
    int antithetic;
    int statistics;  // pseudo-random with a variance estimate
    int variance;    // the reference keeps m2 (statistics && !antithetic)
    SobolTables sobol;
    BlockPartial* partials;
};

template <class Real>
struct PersistentArgs {
    DevBook<Real> book;
    const int4* items;  // (contract, first sample, sample count, dims), grouped by contract
    const int* order;   // dispatch order of the items (longest contracts first)
    int item_count;
    int* queue;         // work-queue head
    uint64_t seed;
    SobolTables sobol;
    Real* values;                  // per-path payoffs
    const int64_t* value_offset;   // per contract: first slot of its samples in `values`
    unsigned long long* executed;  // per contract: grid steps simulated
    const volatile int* cancel;    // host-mapped cancellation word (may be null)
    int* aborted;
    int refill;                    // path units between lane refills
};

// ------------------------------------------------------------------------------------
// Plan compilation: the caller's FP64 plan into the kernel's precision.
// ------------------------------------------------------------------------------------
template <class Real>
__global__ void compile_contracts_kernel(const kgpu_contract* in, int n, ContractT<Real>* out) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const kgpu_contract c = in[i];
    ContractT<Real> o;
    o.payoff = c.payoff;
    o.flags = c.flags;
    o.step_count = c.step_count;
    o.event_count = c.event_count;
    o.bridge_count = c.bridge_count;
    o.reserved = 0;
    o.step_offset = c.step_offset;
    o.event_offset = c.event_offset;
    o.bridge_offset = c.bridge_offset;
    o.strike = Real(c.strike);
    o.sign = Real(c.sign);
    o.diffusion = Real(c.diffusion);
    o.half_variance = Real(c.half_variance);
    o.moneyness = Real(c.moneyness);
    o.log_scale = Real(c.log_scale);
    o.knock_in = Real(c.knock_in);
    o.initial_cash = Real(c.initial_cash);
    o.terminal_base = Real(c.terminal_base);
    o.terminal_plain = Real(c.terminal_plain);
    o.terminal_fixed = Real(c.terminal_fixed);
    o.downside_lower = Real(c.downside_lower);
    o.downside_upper = Real(c.downside_upper);
    o.downside_initial = Real(c.downside_initial);
    o.final_discount = Real(c.final_discount);
    o.knock_out = Real(c.knock_out);
    o.quantity = Real(c.quantity);
    o.daily_quantity = Real(c.daily_quantity);
    o.acceleration = Real(c.acceleration);
    o.log_strike = Real(c.log_strike);
    o.barrier_drift = Real(c.barrier_drift);
    o.barrier_distance = Real(c.barrier_distance);
    o.barrier_moneyness = Real(c.barrier_moneyness);
    o.rebate = Real(c.rebate);
    o.spot = Real(c.spot);
    o.log_discount = Real(c.log_discount);
    o.volatility = Real(c.volatility);
    o.dividend = Real(c.dividend);
    o.avg_drift = Real(c.avg_drift);
    o.avg_width = Real(c.avg_width);
    o.avg_lead_drift = Real(c.avg_lead_drift);
    o.avg_lead_width = Real(c.avg_lead_width);
    o.avg_interval_forward = Real(c.avg_interval_forward);
    o.avg_weight = Real(c.avg_weight);
    o.avg_log_spot = Real(c.avg_log_spot);
    o.avg_log_scale = Real(c.avg_log_scale);
    o.avg_log_strike = Real(c.avg_log_strike);
    o.avg_fraction = Real(c.avg_fraction);
    o.avg_half = Real(c.avg_half);
    o.avg_log_fraction = Real(c.avg_log_fraction);
    o.avg_log_half = Real(c.avg_log_half);
    o.avg_rest = Real(c.avg_rest);
    o.avg_log_rest = Real(c.avg_log_rest);
    o.avg_baseline = Real(c.avg_baseline);
    o.control_log_strike = Real(c.control_log_strike);
    o.control_log_asset_scale = Real(c.control_log_asset_scale);
    o.control_first_weight = Real(c.control_first_weight);
    o.control_mean = Real(c.control_mean);
    o.band = Real(c.band);
    o.band_initial = Real(c.band_initial);
    o.greek_log_spot = Real(c.greek_log_spot);
    o.greek_log_width = Real(c.greek_log_width);
    o.greek_log_amount = Real(c.greek_log_amount);
    o.greek_log_base_width = Real(c.greek_log_base_width);
    o.greek_log_weight = Real(c.greek_log_weight);
    out[i] = o;
}

// Steps, events, intervals and bridge weights to single precision (grid-stride).
static __global__ void compile_arrays_fp32_kernel(RawBook b, StepT<float>* steps, EventT<float>* events,
                                                  IntervalT<float>* intervals, DailyT<float>* daily) {
    const int64_t stride = int64_t(gridDim.x) * blockDim.x;
    const int64_t first = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    for (int64_t i = first; i < b.step_total; i += stride) {
        const kgpu_step s = b.steps[i];
        steps[i] = StepT<float>{float(s.drift), float(s.diffusion), float(s.time), float(s.discount)};
        if (b.daily) daily[i] = DailyT<float>{float(b.daily[i].weight), float(b.daily[i].width)};
    }
    for (int64_t i = first; i < b.event_total; i += stride) {
        const kgpu_event e = b.events[i];
        EventT<float> o;
        o.knock_out = float(e.knock_out);
        o.coupon_barrier = float(e.coupon_barrier);
        for (int k = 0; k < 4; ++k) o.payment[k] = float(e.payment[k]);
        o.has_knock_out = e.has_knock_out;
        o.step = e.step;
        events[i] = o;
    }
    for (int64_t i = first; i < b.interval_total; i += stride) {
        const kgpu_bridge_interval v = b.intervals[i];
        intervals[i] = IntervalT<float>{v.end, 0, float(v.drift), float(v.diffusion)};
    }
}

// Per-position bridge units of every bridged contract, one CTA per contract.  The CTA
// stages the contract's interval ends and the running count of cash events at them in
// shared memory (up to kUnitsStaged intervals; longer plans are walked interval by
// interval), then every thread fills positions, finding its interval by bisection.
constexpr int kUnitsStaged = 2048;

template <class Real>
__global__ void __launch_bounds__(256) compile_units_kernel(const kgpu_contract* contracts,
                                                            const kgpu_bridge_interval* intervals,
                                                            const kgpu_bridge_daily* daily, const uint8_t* flags,
                                                            const kgpu_event* events, UnitT<Real>* units,
                                                            EndT<Real>* ends) {
    __shared__ int end_of[kUnitsStaged];
    __shared__ int event_before[kUnitsStaged];  // cash events at interval ends before interval k
    __shared__ int warp_total[8];
    const kgpu_contract c = contracts[blockIdx.x];
    if (!(c.flags & KGPU_C_BRIDGE)) return;
    auto unit_at = [&](int q, int k, int start, int ev) {
        const kgpu_bridge_interval iv = intervals[c.bridge_offset + k];
        const int fl = flags[c.step_offset + iv.end];
        const bool event = (fl & KGPU_STEP_EVENT) != 0;
        UnitT<Real> u;
        if (q == start) {
            u.a = Real(iv.diffusion);
            u.b = Real(iv.drift);
            u.flags = kUnitBegin;
        } else {
            const kgpu_bridge_daily d = daily[c.step_offset + q - 1];
            u.a = Real(d.width);
            u.b = Real(d.weight);
            u.flags = 0;
        }
        u.end = iv.end;
        u.flags |= fl << 8;
        if (q == iv.end) u.flags |= kUnitLast;
        EndT<Real> o{};
        if (event) {
            const kgpu_event e = events[ev];
            if (e.has_knock_out) u.flags |= kUnitKnockOut;
            if (q == iv.end) {
                o.knock_out = Real(e.knock_out);
                o.coupon_barrier = Real(e.coupon_barrier);
                for (int j = 0; j < 4; ++j) o.payment[j] = Real(e.payment[j]);
            }
        }
        units[c.step_offset + q] = u;
        ends[c.step_offset + q] = o;
    };
    const int n = c.bridge_count;
    if (n > kUnitsStaged) {
        // Long plans: interval by interval, positions of an interval in parallel.
        int start = 0, ev = c.event_offset;
        for (int k = 0; k < n; ++k) {
            const int e = intervals[c.bridge_offset + k].end;
            for (int q = start + int(threadIdx.x); q <= e; q += blockDim.x) unit_at(q, k, start, ev);
            ev += (flags[c.step_offset + e] & KGPU_STEP_EVENT) ? 1 : 0;
            start = e + 1;
        }
        return;
    }
    // Interval ends and an exclusive scan of the event flags at them (8 per thread).
    constexpr int kPer = kUnitsStaged / 256;
    int local[kPer];
    int sum = 0;
    for (int j = 0; j < kPer; ++j) {
        const int k = int(threadIdx.x) * kPer + j;
        int is_event = 0;
        if (k < n) {
            const int e = intervals[c.bridge_offset + k].end;
            end_of[k] = e;
            is_event = (flags[c.step_offset + e] & KGPU_STEP_EVENT) ? 1 : 0;
        }
        local[j] = sum;
        sum += is_event;
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int inclusive = sum;
    for (int o = 1; o < 32; o <<= 1) {
        const int v = __shfl_up_sync(0xffffffffu, inclusive, o);
        if (lane >= o) inclusive += v;
    }
    if (lane == 31) warp_total[warp] = inclusive;
    __syncthreads();
    int base = inclusive - sum;
    for (int w = 0; w < warp; ++w) base += warp_total[w];
    for (int j = 0; j < kPer; ++j) {
        const int k = int(threadIdx.x) * kPer + j;
        if (k < n) event_before[k] = base + local[j];
    }
    __syncthreads();
    for (int q = threadIdx.x; q < c.step_count; q += blockDim.x) {
        int lo = 0, hi = n - 1;  // first interval whose end is >= q
        while (lo < hi) {
            const int mid = (lo + hi) >> 1;
            if (end_of[mid] >= q) hi = mid; else lo = mid + 1;
        }
        const int start = lo == 0 ? 0 : end_of[lo - 1] + 1;
        unit_at(q, lo, start, c.event_offset + event_before[lo]);
    }
}

// The 32-bit high part of every reference block: row b holds, per dimension, the shift
// XOR the directions of the gray-code bits >= 8 of block b's points.
static __global__ void sobol_high_table_kernel(SobolTables t, int blocks, uint32_t* out) {
    const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= int64_t(blocks) * t.dims) return;
    const int b = int(i / t.dims), d = int(i % t.dims);
    const uint64_t first = uint64_t(b) * kBlockSize;
    uint64_t g = (first ^ (first >> 1)) >> 8;
    uint32_t x = t.shifts32[d];
    for (; g; g &= g - 1) x ^= t.directions32[size_t(__ffsll(g) - 1 + 8) * t.dims + d];
    out[i] = x;
}

// Top 32 of the 52 bits of a 64-bit Sobol table.
static __global__ void sobol_top32_kernel(const uint64_t* in, int64_t n, uint32_t* out) {
    const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i < n) out[i] = uint32_t(in[i] >> 20);
}

// Nibble tables of a Sobol sequence: for each dimension, the XOR of direction rows 0-3
// selected by a 4-bit pattern (16 entries) then rows 4-7 (16 entries).
static __global__ void sobol_nibbles_kernel(const uint64_t* directions, int dims, uint64_t* out) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= dims * 32) return;
    const int d = i / 32, e = i % 32;
    const int base = e < 16 ? 0 : 4;
    const int pattern = e & 15;
    uint64_t x = 0;
    for (int b = 0; b < 4; ++b)
        if ((pattern >> b) & 1) x ^= directions[size_t(base + b) * dims + d];
    out[i] = x;
}

template <class Real>
__device__ __forceinline__ void load_model(DevModel<Real>& m, const kgpu_model& src, Real* smem_lv,
                                           const double* lv_dev) {
    m.kind = src.kind;
    m.spot = Real(src.spot);
    m.rate = Real(src.rate);
    m.dividend = Real(src.dividend);
    m.v0 = Real(src.v0);
    m.kappa = Real(src.kappa);
    m.theta = Real(src.theta);
    m.xi = Real(src.xi);
    m.rho = Real(src.rho);
    m.rho_bar = Real(sqrt(1.0 - src.rho * src.rho));
    m.nt = src.lv_time_count;
    m.ns = src.lv_spot_count;
    m.lv = smem_lv;
    if (src.kind == KGPU_MODEL_LOCAL_VOL) {
        int total = m.nt + m.ns + m.nt * m.ns;
        for (int i = threadIdx.x; i < total; i += blockDim.x) smem_lv[i] = Real(lv_dev[i]);
    }
}

// Shift and directions of the gray-code bits >= 8 shared by the points of block `block`.
__device__ __forceinline__ void sobol_high(const SobolTables& t, uint64_t block, uint64_t* high,
                                           int lane, int width) {
    uint64_t first = block * kBlockSize;
    uint64_t gray = (first ^ (first >> 1)) >> 8;
    for (int d = lane; d < t.dims; d += width) {
        uint64_t x = t.shifts[d];
        uint64_t g = gray;
        while (g) {
            int c = __ffsll(g) - 1 + 8;
            x ^= t.directions[size_t(c) * t.dims + d];
            g &= g - 1;
        }
        high[d] = x;
    }
}

// The same from the 32-bit tables.
__device__ __forceinline__ void sobol_high(const SobolTables& t, uint64_t block, uint32_t* high,
                                           int lane, int width) {
    uint64_t first = block * kBlockSize;
    uint64_t gray = (first ^ (first >> 1)) >> 8;
    for (int d = lane; d < t.dims; d += width) {
        uint32_t x = t.shifts32[d];
        uint64_t g = gray;
        while (g) {
            int c = __ffsll(g) - 1 + 8;
            x ^= t.directions32[size_t(c) * t.dims + d];
            g &= g - 1;
        }
        high[d] = x;
    }
}

// The Sobol source and high-table word of each precision: FP32 kernels use the 32-bit
// tables, FP64 kernels the full 52-bit ones.
template <class Real>
struct SobolKind;
template <>
struct SobolKind<double> {
    using Word = uint64_t;
    using Source = SobolSource<double>;
    static __device__ __forceinline__ Source make(const SobolTables& t, const Word* high) {
        return Source{high, t.nibbles, t.dims, 0, 0, 0};
    }
    static constexpr bool global_high = false;
    static __device__ __forceinline__ void set_row(Source&, const SobolTables&, uint64_t) {}
};
template <>
struct SobolKind<float> {
    using Word = uint32_t;
    using Source = SobolSource32;
    static __device__ __forceinline__ Source make(const SobolTables& t, const Word* high) {
        return Source{high, t.nibbles32, t.directions, t.shifts, t.dims, 0, 0, 0, 0};
    }
    static constexpr bool global_high = true;
    static __device__ __forceinline__ void set_row(Source& n, const SobolTables& t, uint64_t sample) {
        n.high32 = t.high32 + size_t(sample / kBlockSize) * t.dims;
    }
};

template <class S, class Real>
struct Negated {
    S& s;
    __device__ __forceinline__ Real normal() { return -s.normal(); }
    __device__ __forceinline__ Real normal_if(bool need) { return -s.normal_if(need); }
    __device__ __forceinline__ void skip(int n) { s.skip(n); }
};

// Runs one whole path to completion.
template <class Real, int MODEL, class Source>
__device__ __forceinline__ Real run_path(const DevModel<Real>& m, const ContractT<Real>& c,
                                         const PlanPtrs<Real>& p, Source& n, int& executed) {
    PathState<Real> s;
    path_init(s, c, m.v0);
    Real value = Real(0);
    // Every path ends within step_count + bridge_count units of work.
    int guard = 2 * c.step_count + 2 * c.bridge_count + 2;
    while (!path_step<Real, MODEL>(m, c, p, s, n, value)) {
        if (--guard == 0) {
            value = xnan(Real());  // reported as a computation failure
            break;
        }
    }
    executed = s.executed;
    return value;
}

// Plain schedule: thread = sample, CUDA block = reference block; the block's moments are
// accumulated sequentially in sample order as sample_paths does (monte_carlo.rs:1778-1798).
template <class Real, int MODEL, bool SOBOL>
__global__ void __launch_bounds__(kThreads) plain_kernel(PlainArgs<Real> a, kgpu_model model,
                                                         const double* lv_dev) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    double* values = reinterpret_cast<double*>(smem_raw);          // [2 * kThreads]
    int* used = reinterpret_cast<int*>(values + 2 * kThreads);     // [kThreads]
    uint64_t* high = reinterpret_cast<uint64_t*>(used + kThreads);  // [dims] (Sobol)
    Real* lv = reinterpret_cast<Real*>(high + (SOBOL ? a.dims : 0));
    DevModel<Real> m;
    load_model(m, model, lv, lv_dev);
    const uint64_t block = blockIdx.x;
    if (SOBOL) sobol_high(a.sobol, block, high, threadIdx.x, blockDim.x);
    __syncthreads();
    // A reference into the compiled book (not a local copy): out-of-line payoff pieces
    // receive it without a stack copy of the contract.
    const ContractT<Real>& c = a.book.contracts[a.contract];
    const PlanPtrs<Real> plan = plan_of(a.book, c);
    const int64_t sample = int64_t(block) * kBlockSize + threadIdx.x;
    double positive = 0.0, negative = 0.0;
    int executed = 0;
    if (sample < a.samples) {
        const bool paired = a.antithetic && sample < a.paths / 2;
        int e1 = 0, e2 = 0;
        if (SOBOL) {
            SobolSource<Real> n{high, a.sobol.nibbles, a.dims, 0, 0, 0};
            n.start(uint64_t(sample));
            positive = double(run_path<Real, MODEL>(m, c, plan, n, e1));
            if (paired) {
                n.start(uint64_t(sample));
                Negated<SobolSource<Real>, Real> neg{n};
                negative = double(run_path<Real, MODEL>(m, c, plan, neg, e2));
            }
        } else {
            PcgSource<Real> n;
            n.start(a.seed, uint64_t(sample), a.dims);
            positive = double(run_path<Real, MODEL>(m, c, plan, n, e1));
            if (paired) {
                n.start(a.seed, uint64_t(sample), a.dims);
                Negated<PcgSource<Real>, Real> neg{n};
                negative = double(run_path<Real, MODEL>(m, c, plan, neg, e2));
            }
        }
        executed = e1 > e2 ? e1 : e2;
    }
    values[threadIdx.x] = positive;
    values[kThreads + threadIdx.x] = negative;
    used[threadIdx.x] = executed;
    __syncthreads();
    if (threadIdx.x == 0) {
        BlockPartial p;
        p.moments = Moments{0, 0, 0, 0};
        p.pairs = Moments{0, 0, 0, 0};
        p.sample = Moments{0, 0, 0, 0};
        double total_steps = 0.0;
        const int64_t first = int64_t(block) * kBlockSize;
        const int64_t remaining = a.samples - first;
        const int count = remaining < kThreads ? int(remaining) : kThreads;
        for (int j = 0; j < count; ++j) {
            const bool paired = a.antithetic && first + j < a.paths / 2;
            double pv = values[j];
            moments_add(p.moments, pv, a.variance);
            moments_add(p.sample, pv, true);
            if (paired) {
                double nv = values[kThreads + j];
                moments_add(p.moments, nv, a.variance);
                moments_add(p.sample, nv, true);
                if (a.statistics) moments_add(p.pairs, (pv + nv) / 2.0, true);
            }
            total_steps += double(used[j]);
        }
        p.executed = total_steps;
        a.partials[block] = p;
    }
}

// Merges the block partials of one contract in block order (monte_carlo.rs:1800-1809).
// The merge is a dependent chain, but its divisions depend only on prefix sums of the
// block counts and prefix maxima of the block scales, both exact in any order.  The
// CTA's threads compute a chunk's weights in parallel; then one thread per chain (the
// price moments, the i.i.d. sample moments, the antithetic pair moments) walks the
// chunk with them.  Every operation is the sequential merge's, rounded separately
// (__dmul_rn and friends, never contracted), so the result is bit-identical to it.
constexpr int kMergeThreads = 256;

struct MergeStep {
    double left, right, w, u, mean, m2;  // left < 0 marks "copy the block" (empty state)
};

__device__ __forceinline__ const Moments& merge_chain(const BlockPartial& p, int c) {
    return c == 0 ? p.moments : (c == 1 ? p.sample : p.pairs);
}

static __global__ void __launch_bounds__(kMergeThreads)
    merge_blocks_kernel(const BlockPartial* partials, int blocks, int variance, int statistics, int antithetic,
                        BlockPartial* out) {
    __shared__ MergeStep steps[3][kMergeThreads];
    __shared__ double scan_count[kMergeThreads], scan_scale[kMergeThreads];
    __shared__ double carry_count[3], carry_scale[3], executed_part[kMergeThreads];
    const int t = threadIdx.x;
    const int chains = (statistics && antithetic) ? 3 : 2;
    if (t < 3) {
        carry_count[t] = 0.0;
        carry_scale[t] = 0.0;
    }
    double mean = 0.0, m2 = 0.0, executed = 0.0;  // chain state of threads 0..2
    for (int base = 0; base < blocks; base += kMergeThreads) {
        const int g = base + t;
        const int n = min(kMergeThreads, blocks - base);
        if (g < blocks) executed = __dadd_rn(executed, partials[g].executed);
        for (int c = 0; c < chains; ++c) {
            __syncthreads();
            const Moments b = g < blocks ? merge_chain(partials[g], c) : Moments{0, 0, 0, 0};
            scan_count[t] = b.count;
            scan_scale[t] = b.scale;
            __syncthreads();
            // Inclusive scans (sum of integer counts, max of scales): exact.
            for (int d = 1; d < kMergeThreads; d <<= 1) {
                const double pc = t >= d ? scan_count[t - d] : 0.0;
                const double ps = t >= d ? scan_scale[t - d] : 0.0;
                __syncthreads();
                scan_count[t] = __dadd_rn(scan_count[t], pc);
                scan_scale[t] = fmax(scan_scale[t], ps);
                __syncthreads();
            }
            if (g < blocks) {
                const double a_count = __dadd_rn(carry_count[c], t > 0 ? scan_count[t - 1] : 0.0);
                const double a_scale = fmax(carry_scale[c], t > 0 ? scan_scale[t - 1] : 0.0);
                MergeStep st;
                st.mean = b.mean;
                st.m2 = b.m2;
                if (a_count == 0.0) {
                    st.left = -1.0;
                    st.right = st.w = st.u = 0.0;
                } else {
                    const double sc = a_scale > b.scale ? a_scale : b.scale;
                    st.left = sc == 0.0 ? 0.0 : __ddiv_rn(a_scale, sc);
                    st.right = sc == 0.0 ? 0.0 : __ddiv_rn(b.scale, sc);
                    const double total = __dadd_rn(a_count, b.count);
                    st.w = __ddiv_rn(b.count, total);
                    st.u = __dmul_rn(a_count, st.w);
                }
                steps[c][t] = st;
            }
            __syncthreads();
            if (t == 0) {
                carry_count[c] = __dadd_rn(carry_count[c], scan_count[n - 1]);
                carry_scale[c] = fmax(carry_scale[c], scan_scale[n - 1]);
            }
        }
        __syncthreads();
        if (t < chains) {
            const bool with_variance = t == 0 ? variance != 0 : true;
            for (int i = 0; i < n; ++i) {
                const MergeStep st = steps[t][i];
                if (st.left < 0.0) {
                    mean = st.mean;
                    m2 = st.m2;
                    continue;
                }
                const double ml = __dmul_rn(mean, st.left);
                const double delta = __dsub_rn(__dmul_rn(st.mean, st.right), ml);
                mean = __dadd_rn(ml, __dmul_rn(delta, st.w));
                if (with_variance)
                    m2 = __dadd_rn(__dadd_rn(__dmul_rn(__dmul_rn(m2, st.left), st.left),
                                             __dmul_rn(__dmul_rn(st.m2, st.right), st.right)),
                                   __dmul_rn(__dmul_rn(delta, delta), st.u));
            }
        }
    }
    executed_part[t] = executed;
    __syncthreads();
    if (t < 3) {
        Moments m{0, 0, 0, 0};
        if (t < chains) m = Moments{carry_count[t], carry_scale[t], mean, m2};
        if (t == 0) out->moments = m;
        if (t == 1) out->sample = m;
        if (t == 2) out->pairs = m;
    }
    if (t == 0) {
        // Integer-valued counts: exact in any summation order.
        double total = 0.0;
        for (int i = 0; i < kMergeThreads; ++i) total = __dadd_rn(total, executed_part[i]);
        out->executed = total;
    }
}

__device__ __forceinline__ unsigned lanemask_lt() {
    unsigned m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

// Persistent schedule.  Warps pull (contract, tile) items from a device queue and hand
// the item's samples to lanes one at a time: lanes run kRefill path units in lockstep,
// then every lane whose path has finished takes the next unstarted sample -- of the
// current item, or of the next queued one -- so a warp never waits for an item to drain
// while work is queued.  Lanes may therefore hold paths of different items (and
// contracts); each lane keeps its own contract and plan.  Sobol points read the high
// part of their reference block from a global table (FP32) or, in FP64, from the
// warp's shared copy (FP64 keeps one item per warp).  Each finished path writes its
// payoff to values[value_offset[contract] + sample]; reduce_values_kernel sums them in a
// fixed order, so results do not depend on which warp ran which path.
// Resident CTAs the register budget is cut for: FP32 paths fit 64 registers (four
// CTAs per SM); FP64 state needs twice the registers, so it keeps two CTAs.
template <class Real>
constexpr int kPersistentMinBlocks = sizeof(Real) == 4 ? 4 : 2;

template <class Real, int MODEL, bool SOBOL, bool EXT>
__global__ void __launch_bounds__(kThreads, kPersistentMinBlocks<Real>) persistent_kernel(PersistentArgs<Real> a,
                                                                                          kgpu_model model,
                                                              const double* lv_dev) {
    using Kind = SobolKind<Real>;
    using Word = typename Kind::Word;
    constexpr bool kGlobalHigh = Kind::global_high;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    Word* highs = reinterpret_cast<Word*>(smem_raw);
    const int dims = SOBOL ? a.sobol.dims : 0;
    const int shared_dims = (SOBOL && !kGlobalHigh) ? dims : 0;
    Real* lv = reinterpret_cast<Real*>(highs + kWarps * shared_dims);
    DevModel<Real> m;
    load_model(m, model, lv, lv_dev);
    __syncthreads();
    const int warp = threadIdx.x >> 5;
    const int lane = threadIdx.x & 31;
    const unsigned below = lanemask_lt();
    Word* high = highs + warp * shared_dims;

    // Current item of the warp (uniform).
    int item_contract = 0, item_dims = 0;
    int64_t next = 0, end = 0;
    bool have = false;
    auto fetch = [&]() {
        int it = -1;
        if (lane == 0) {
            int q = atomicAdd(a.queue, 1);
            if (a.cancel && *a.cancel) {
                atomicExch(a.aborted, 1);
                q = a.item_count;
            }
            it = q < a.item_count ? a.order[q] : -1;
        }
        it = __shfl_sync(0xffffffffu, it, 0);
        have = it >= 0;
        if (!have) return;
        const int4 w = a.items[it];
        item_contract = w.x;
        item_dims = w.w;
        next = w.y;
        end = int64_t(w.y) + w.z;
        if (SOBOL && !kGlobalHigh) {
            __syncwarp();
            sobol_high(a.sobol, uint64_t(w.y) / kBlockSize, high, lane, 32);
            __syncwarp();
        }
    };
    fetch();

    // Per-lane path.
    bool active = false;
    int contract = 0;
    int64_t sample = 0;
    int guard = 0;
    bool bridged = false;
    PlanPtrs<Real> plan{};
    PathState<Real> s;
    PcgSource<Real> pn;
    typename Kind::Source sn = Kind::make(a.sobol, high);
    unsigned long long exec = 0;
    int exec_contract = -1;

    for (;;) {
        // Refill: idle lanes take unstarted samples in lane order, crossing into the next
        // queued item when the current one runs out.  FP64 Sobol keeps one item per warp
        // (its high part is a per-warp shared copy), so it crosses only once all lanes idle.
        unsigned want = __ballot_sync(0xffffffffu, !active);
        while (want && have) {
            if (SOBOL && !kGlobalHigh && next == end) {
                if (want != 0xffffffffu) break;
                fetch();
                continue;
            }
            const int64_t avail = end - next;
            const int rank = __popc(want & below);
            if (!active && rank < avail) {
                sample = next + rank;
                if (contract != item_contract || exec_contract < 0) {
                    if (exec) atomicAdd(a.executed + exec_contract, exec);
                    exec = 0;
                }
                contract = item_contract;
                exec_contract = item_contract;
                const ContractT<Real>& c = a.book.contracts[contract];
                plan = plan_of(a.book, c);
                bridged = MODEL == KGPU_MODEL_BSM && c.payoff == KGPU_PAYOFF_AUTOCALLABLE &&
                          (c.flags & KGPU_C_BRIDGE) && plan.units != nullptr;
                guard = 2 * c.step_count + 2 * c.bridge_count + 2;
                path_init(s, c, m.v0);
                if (SOBOL) {
                    Kind::set_row(sn, a.sobol, uint64_t(sample));
                    sn.start(uint64_t(sample));
                } else {
                    pn.start(a.seed, uint64_t(sample), item_dims);
                }
                active = true;
            }
            const int taken = __popc(want);
            const int64_t take = taken < avail ? taken : avail;
            next += take;
            want = __ballot_sync(0xffffffffu, !active);
            if (next == end && !(SOBOL && !kGlobalHigh)) fetch();
        }
        if (!__any_sync(0xffffffffu, active)) {
            if (!have) break;
            continue;
        }
        const ContractT<Real>& c = a.book.contracts[contract];
        Real* values = a.values + a.value_offset[contract];
#pragma unroll 1
        for (int r = 0; r < a.refill; ++r) {
            bool finished = false;
            Real value = Real(0);
            if (active) {
                if (bridged) {
                    finished = SOBOL ? bridge_unit_step<Real>(c, plan, s, sn) : bridge_unit_step<Real>(c, plan, s, pn);
                    if (finished) value = bridge_value(m, c, s);
                } else {
                    finished = SOBOL ? path_step<Real, MODEL, EXT>(m, c, plan, s, sn, value)
                                     : path_step<Real, MODEL, EXT>(m, c, plan, s, pn, value);
                }
                if (!finished && --guard == 0) {
                    finished = true;
                    value = xnan(Real());
                }
            }
            if (finished) {
                values[sample] = value;
                exec += s.executed;
                active = false;
            }
        }
    }
    if (exec) atomicAdd(a.executed + exec_contract, exec);
}

// Sums per-path values in a fixed order: one CTA per chunk of a contract's values,
// a fixed strided assignment and a fixed tree.
template <class Real>
__global__ void __launch_bounds__(256) reduce_values_kernel(const Real* values, const int4* chunks,
                                                            const int64_t* value_offset, TilePartial* out) {
    __shared__ double red[3][256];
    const int4 ch = chunks[blockIdx.x];
    const Real* v = values + value_offset[ch.x] + ch.y;
    double s0 = 0, s1 = 0, s2 = 0;
    for (int i = threadIdx.x; i < ch.z; i += blockDim.x) {
        const double x = double(v[i]);
        s0 += x;
        s1 += x * x;
        s2 += 1.0;
    }
    red[0][threadIdx.x] = s0;
    red[1][threadIdx.x] = s1;
    red[2][threadIdx.x] = s2;
    __syncthreads();
    for (int half = 128; half > 0; half >>= 1) {
        if (threadIdx.x < half)
            for (int k = 0; k < 3; ++k) red[k][threadIdx.x] += red[k][threadIdx.x + half];
        __syncthreads();
    }
    if (threadIdx.x == 0) out[blockIdx.x] = TilePartial{red[0][0], red[1][0], red[2][0], 0.0};
}

// Sums each contract's tile partials: one CTA per contract, a fixed strided assignment
// and a fixed shared-memory tree, so the order of additions never changes.
static __global__ void __launch_bounds__(256) reduce_tiles_kernel(const TilePartial* partials,
                                                                  const int* first_item,
                                                                  TilePartial* out) {
    __shared__ double red[4][256];
    const int c = blockIdx.x;
    double a0 = 0, a1 = 0, a2 = 0, a3 = 0;
    for (int i = first_item[c] + threadIdx.x; i < first_item[c + 1]; i += blockDim.x) {
        a0 += partials[i].sum;
        a1 += partials[i].sumsq;
        a2 += partials[i].count;
        a3 += partials[i].executed;
    }
    red[0][threadIdx.x] = a0;
    red[1][threadIdx.x] = a1;
    red[2][threadIdx.x] = a2;
    red[3][threadIdx.x] = a3;
    __syncthreads();
    for (int half = 128; half > 0; half >>= 1) {
        if (threadIdx.x < half)
            for (int k = 0; k < 4; ++k) red[k][threadIdx.x] += red[k][threadIdx.x + half];
        __syncthreads();
    }
    if (threadIdx.x == 0) out[c] = TilePartial{red[0][0], red[1][0], red[2][0], red[3][0]};
}

}  // namespace kgpu
