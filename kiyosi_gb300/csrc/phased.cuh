// Phase-major schedule of bridged autocallable books (FP32).
//
// A bridged path (bridge_payoffs, engines/monte_carlo/autocallable.rs:628-736) is a
// sequence of bridge intervals: the interval end is drawn first, then the daily bridge
// steps while knock-in is still undecided, then the interval end settles knock-in and
// the cash event.  The lane-refill kernel gives each lane its own path, so the lanes of
// a warp sit at different positions: every table read is a gather and every branch of
// the interval end is taken by some lane at every step; and because a surviving note
// runs 504 daily positions while the average path runs 80, the last paths of each lane
// leave most lanes idle.
//
// Here launch k advances every path still monitoring knock-in by exactly one interval.
// A warp takes 32 paths of one list, so its lanes walk the same grid positions: unit
// records, cash events and Sobol direction rows are broadcast reads and the loop over
// days is uniform.  Paths that finish write their payoff to
// values[value_offset[contract] + sample]; monitoring survivors are appended to the list
// of launch k + 1, one atomic per warp.  A knocked-in path draws only one normal per
// interval (its daily steps no longer matter), so it leaves the phase lists for a pool
// that one drain launch, after the last phase, runs to completion.  Once the monitoring
// paths fit in one wave of resident lanes, a launch runs them to completion as well and
// the remaining phase launches return at once.  The lists carry all the state a path
// holds between intervals, so the per-path payoffs are the lane-refill kernel's to the
// bit: the same arithmetic in the same order on the same normals.
#pragma once
#include "kernels.cuh"

namespace kgpu {

// Entry tag: bit 0 monitoring, bit 1 knocked in, bits 2-11 the next interval, bits
// 12-31 the contract.
constexpr int kPhaseMonitoring = 1;
constexpr int kPhaseKnockedIn = 2;
constexpr int kPhaseIntervalShift = 2;
constexpr int kPhaseMaxIntervals = 1024;
constexpr int kPhaseTagShift = 12;

// A path between two intervals.
template <class Real, bool SOBOL>
struct PhaseEntry;
template <class Real>
struct __align__(16) PhaseEntry<Real, true> {
    uint32_t sample;
    uint32_t tag;
    Real lr, cash;
};
template <class Real>
struct __align__(16) PhaseEntry<Real, false> {
    uint32_t sample;
    uint32_t tag;
    Real lr, cash;
    uint64_t state;  // PCG state at the interval's first normal (inc follows from the block)
    Real spare;
    uint32_t has_spare;
};

template <class Real, bool SOBOL>
struct PhaseArgs {
    DevBook<Real> book;
    int phase;
    int contract_count;
    int64_t total;                  // phase 0: every sample of every contract
    const int64_t* value_offset;    // [contract_count + 1]
    const int* dims;                // per contract: normals per sample (PCG positions)
    const PhaseEntry<Real, SOBOL>* in_monitoring;  // paths still monitoring knock-in
    const int* in_count;            // their number (phase > 0)
    PhaseEntry<Real, SOBOL>* out_monitoring;
    int* out_count;
    PhaseEntry<Real, SOBOL>* knocked;  // knocked-in paths, each with its next interval
    int* knocked_count;
    int drain;                      // this launch runs the knocked-in pool to completion
    Real* values;
    unsigned long long* executed;   // per contract: positions simulated
    uint64_t seed;
    SobolTables sobol;              // nibbles32 [dims][32], directions/shifts for the tails
    const uint32_t* high_t;         // [dims][blocks]: the high part of every block, by dimension
    int high_blocks;
    const volatile int* cancel;     // host-mapped cancellation word (may be null)
    int* aborted;
    int* finished;                  // phase + 1 of the launch that completed the monitoring paths
    int64_t complete_below;         // monitoring paths at or below which a launch completes them
};

// One path's state within a launch.
template <class Real>
struct PhaseLane {
    uint32_t sample;
    int contract;
    bool valid, monitoring, knocked_in;
    Real lr, cash;
};

// The normal of a Sobol word of dimension `d` (SobolSource32::normal after its loads).
__device__ __forceinline__ float phase_sobol_from_word(const SobolTables& t, uint32_t v, uint64_t gray, int d) {
    const bool upper = (v >> 31) != 0;
    const uint32_t k = upper ? ~v : v;
    if (k < (1u << 12)) {
        uint64_t x = t.shifts[d];
        for (uint64_t g = gray; g; g &= g - 1) x ^= t.directions[size_t(__ffsll(g) - 1) * t.dims + d];
        return sobol_normal(x, 0.0f);
    }
    return normal_from_tail32(k, upper);
}

// Advances the lanes of a warp by one bridge interval (`phase`, per lane) of their
// contracts, position by position as bridge_unit_step (path_engine.cuh) does.  Returns
// whether the lane's path finished; its payoff is then stored.
template <class Real, bool SOBOL>
__device__ __forceinline__ bool phase_interval(const PhaseArgs<Real, SOBOL>& a, int phase, PhaseLane<Real>& L,
                                               PcgSource<Real>& pn, int& executed) {
    constexpr unsigned kFull = 0xffffffffu;
    const ContractT<Real>& c = a.book.contracts[L.contract];
    const UnitT<Real>* units = a.book.units + c.step_offset;
    // The interval's first position and its begin unit (the interval end's diffusion and
    // drift, the end, the end's step flags).  Lanes without a path read contract 0's
    // first unit, which always exists.
    const int start = (L.valid && phase > 0) ? a.book.intervals[c.bridge_offset + phase - 1].end + 1 : 0;
    const UnitT<Real> u0 = units[start];
    const int end = u0.end;
    const uint32_t block = L.sample / kBlockSize;
    const uint64_t gray = uint64_t(L.sample) ^ (uint64_t(L.sample) >> 1);
    const uint32_t glo = uint32_t(gray & 0xF), ghi = uint32_t((gray >> 4) & 0xF) + 16;
    // The normal of dimension `d`: Sobol words from the dimension-major high table
    // (lanes of a warp read neighbouring words) and the nibble rows.
    auto normal_at = [&](int d) -> Real {
        if constexpr (SOBOL) {
            const uint32_t* row = a.sobol.nibbles32 + size_t(d) * 32;
            const uint32_t v = __ldg(a.high_t + size_t(d) * a.high_blocks + block) ^ __ldg(row + glo) ^ __ldg(row + ghi);
            return phase_sobol_from_word(a.sobol, v, gray, d);
        } else {
            return pn.normal();
        }
    };
    const Real level = c.knock_in;
    Real lr = L.lr, target = L.lr, minimum = xinf(Real());
    if (L.valid) {
        target = lr + xfma(u0.a, normal_at(start), u0.b);
        executed += 1;
    }
    // Daily bridge steps of the monitoring paths, until knock-in is decided.  `next`:
    // the lane's next undrawn position (PCG stream position).
    bool walking = L.valid && L.monitoring;
    int next = start + 1;
    for (int q = start + 1; __any_sync(kFull, walking && q <= end); ++q) {
        if (walking && q <= end) {
            const UnitT<Real> u = units[q];
            const Real z = normal_at(q);
            const Real daily = lr + xfma(u.b, target - lr, u.a * z);
            lr = daily;
            minimum = daily < minimum ? daily : minimum;
            executed += 1;
            next = q + 1;
            walking = !(minimum < level);
        }
    }
    // PCG: the interval's normals not drawn (knock-in decided, or not monitored) are
    // skipped, as SkippingPath::skip does; Sobol draws are positional.
    if (!SOBOL && L.valid) pn.skip(end + 1 - next);
    if (!L.valid) return false;
    // Interval end: knock-in, the cash event, the finish.
    lr = target;
    const int fl = u0.flags >> 8;
    const bool ki = L.monitoring && (minimum < level || ((fl & KGPU_STEP_KNOCK_IN) && lr < level));
    L.knocked_in = L.knocked_in || ki;
    L.monitoring = L.monitoring && !ki;
    L.lr = lr;
    bool hit = false;
    if (fl & KGPU_STEP_EVENT) {
        const EndT<Real> e = a.book.ends[c.step_offset + end];
        hit = (u0.flags & kUnitKnockOut) && lr >= e.knock_out;
        const bool coupon = lr >= e.coupon_barrier;
        L.cash += hit ? (coupon ? e.payment[3] : e.payment[2]) : (coupon ? e.payment[1] : e.payment[0]);
    }
    Real value;
    if (hit) {
        value = L.cash;
    } else if (end + 1 >= c.step_count) {
        const bool in = L.knocked_in ||
                        ((c.flags & KGPU_C_EXPIRY_KNOCK_IN) && (c.flags & KGPU_C_HAS_KNOCK_IN) && lr < level);
        value = L.cash + autocallable_terminal(c, spot_at(c.spot, lr), in) * c.final_discount;
    } else {
        return false;
    }
    a.values[a.value_offset[L.contract] + L.sample] = value;
    return true;
}

template <class Real, bool SOBOL>
__device__ __forceinline__ PhaseEntry<Real, SOBOL> phase_entry(const PhaseLane<Real>& L, int next,
                                                               const PcgSource<Real>& pn) {
    PhaseEntry<Real, SOBOL> e;
    e.sample = L.sample;
    e.tag = uint32_t(L.contract) << kPhaseTagShift | uint32_t(next) << kPhaseIntervalShift |
            (L.knocked_in ? kPhaseKnockedIn : 0) | (L.monitoring ? kPhaseMonitoring : 0);
    e.lr = L.lr;
    e.cash = L.cash;
    if constexpr (!SOBOL) {
        e.state = pn.g.state;
        e.spare = pn.spare;
        e.has_spare = pn.has_spare ? 1u : 0u;
    }
    return e;
}

// Launch `phase` advances the paths still monitoring knock-in by one interval; the
// drain launch (after the last phase) runs the knocked-in pool to completion.
template <class Real, bool SOBOL>
__global__ void __launch_bounds__(kThreads, 4) phased_kernel(PhaseArgs<Real, SOBOL> a) {
    using Entry = PhaseEntry<Real, SOBOL>;
    constexpr unsigned kFull = 0xffffffffu;
    // An earlier launch completed every monitoring path (`finished` holds its phase + 1).
    const int done = *(volatile int*)a.finished;
    if (!a.drain && done != 0 && done - 1 < a.phase) return;
    if (*(volatile int*)a.aborted) return;
    if (a.cancel && blockIdx.x == 0 && threadIdx.x == 0 && *a.cancel) atomicExch(a.aborted, 1);
    const int lane = threadIdx.x & 31;
    const unsigned below = lanemask_lt();
    const int64_t count = a.drain ? int64_t(*a.knocked_count) : a.phase == 0 ? a.total : int64_t(*a.in_count);
    // Few monitoring paths left: run them to completion in this launch, so the last
    // intervals pay no launch or list handoff.
    const bool complete = a.drain || count <= a.complete_below;
    if (!a.drain && complete && blockIdx.x == 0 && threadIdx.x == 0) *(volatile int*)a.finished = a.phase + 1;
    const int64_t chunks = (count + 31) / 32;
    const int64_t warps = int64_t(gridDim.x) * kWarps;
    for (int64_t ch = (int64_t(blockIdx.x) * kThreads + threadIdx.x) / 32; ch < chunks; ch += warps) {
        const int64_t idx = ch * 32 + lane;
        // The path's state at the start of its next interval.
        PhaseLane<Real> L;
        L.valid = idx < count;
        L.sample = 0;
        L.contract = 0;
        L.monitoring = L.knocked_in = false;
        L.lr = L.cash = Real(0);
        int phase = a.phase;
        PcgSource<Real> pn;
        if (L.valid) {
            if (!a.drain && a.phase == 0) {
                int lo = 0, hi = a.contract_count;  // contract with value_offset[c] <= idx
                while (hi - lo > 1) {
                    const int mid = (lo + hi) >> 1;
                    if (a.value_offset[mid] <= idx) lo = mid; else hi = mid;
                }
                L.contract = lo;
                L.sample = uint32_t(idx - a.value_offset[lo]);
                const ContractT<Real>& c0 = a.book.contracts[lo];
                L.knocked_in = (c0.flags & KGPU_C_KNOCKED_IN) != 0;
                L.monitoring = !L.knocked_in && (c0.flags & KGPU_C_HAS_KNOCK_IN);
                L.cash = c0.initial_cash;
                if (!SOBOL) pn.start(a.seed, L.sample, a.dims[lo]);
            } else {
                const Entry e = a.drain ? a.knocked[idx] : a.in_monitoring[idx];
                L.sample = e.sample;
                L.contract = int(e.tag >> kPhaseTagShift);
                L.monitoring = (e.tag & kPhaseMonitoring) != 0;
                L.knocked_in = (e.tag & kPhaseKnockedIn) != 0;
                phase = int((e.tag >> kPhaseIntervalShift) & (kPhaseMaxIntervals - 1));
                L.lr = e.lr;
                L.cash = e.cash;
                if constexpr (!SOBOL) {
                    pn.g.state = e.state;
                    pn.g.inc = ((uint64_t(L.sample) / kBlockSize) << 1) | 1;
                    pn.spare = e.spare;
                    pn.has_spare = e.has_spare != 0;
                }
            }
        }
        int executed = 0;
        bool finished = phase_interval<Real, SOBOL>(a, phase, L, pn, executed);
        if (complete) {
            while (__any_sync(kFull, L.valid && !finished)) {
                L.valid = L.valid && !finished;
                ++phase;
                finished = phase_interval<Real, SOBOL>(a, phase, L, pn, executed);
            }
        }
        // Positions simulated, summed per contract.
        const int lead = __shfl_sync(kFull, L.contract, 0);
        if (__all_sync(kFull, L.contract == lead)) {
            const unsigned total = __reduce_add_sync(kFull, unsigned(executed));
            if (lane == 0 && total) atomicAdd(a.executed + lead, (unsigned long long)total);
        } else if (executed) {
            atomicAdd(a.executed + L.contract, (unsigned long long)executed);
        }
        if (complete) continue;
        // Survivors: monitoring paths to the next phase's list, knocked-in paths to the
        // pool the drain launch completes.
        const bool keep = L.valid && !finished;
        const bool keep_m = keep && L.monitoring, keep_k = keep && !L.monitoring;
        const unsigned bm = __ballot_sync(kFull, keep_m), bk = __ballot_sync(kFull, keep_k);
        int base_m = 0, base_k = 0;
        if (lane == 0) {
            if (bm) base_m = atomicAdd(a.out_count, __popc(bm));
            if (bk) base_k = atomicAdd(a.knocked_count, __popc(bk));
        }
        base_m = __shfl_sync(kFull, base_m, 0);
        base_k = __shfl_sync(kFull, base_k, 0);
        if (keep_m) a.out_monitoring[base_m + __popc(bm & below)] = phase_entry<Real, SOBOL>(L, phase + 1, pn);
        if (keep_k) a.knocked[base_k + __popc(bk & below)] = phase_entry<Real, SOBOL>(L, phase + 1, pn);
    }
}

// The high part of every reference block, dimension-major: out[d * blocks + b].
static __global__ void sobol_high_table_t_kernel(SobolTables t, int blocks, uint32_t* out) {
    const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= int64_t(blocks) * t.dims) return;
    const int d = int(i / blocks), b = int(i % blocks);
    const uint64_t first = uint64_t(b) * kBlockSize;
    uint64_t g = (first ^ (first >> 1)) >> 8;
    uint32_t x = t.shifts32[d];
    for (; g; g &= g - 1) x ^= t.directions32[size_t(__ffsll(g) - 1 + 8) * t.dims + d];
    out[i] = x;
}

}  // namespace kgpu
