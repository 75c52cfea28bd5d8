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
// Here the book advances interval by interval.  While many paths still monitor
// knock-in, each interval is a grid-wide step: a warp takes 32 paths of the current
// monitoring list, so its lanes walk the same grid positions (unit records, cash events
// and Sobol direction rows are broadcast reads; the loop over days is uniform).  Paths
// that finish write their payoff to values[value_offset[contract] + sample]; monitoring
// survivors are appended to the next interval's list, one atomic per warp.  A
// knocked-in path draws one normal per interval (its daily steps no longer matter), so
// it leaves for a pool completed at the end.  Once the monitoring paths fit in one wave
// of resident lanes, each CTA runs a batch of them to completion, compacting the live
// paths after every interval so its warps stay full; the knocked-in pool is completed
// the same way.  The whole schedule is one cooperative launch with a grid barrier
// between the steps.  The lists carry all the state a path holds between intervals, so
// the per-path payoffs are the lane-refill kernel's to the bit: the same arithmetic in
// the same order on the same normals.
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
    int phases;                     // intervals of the longest contract
    int contract_count;
    int64_t total;                  // every sample of every contract
    const int64_t* value_offset;    // [contract_count + 1]
    const int* dims;                // per contract: normals per sample (PCG positions)
    PhaseEntry<Real, SOBOL>* lists;    // two generations of the monitoring list, total each
    PhaseEntry<Real, SOBOL>* knocked;  // knocked-in paths, each with its next interval
    int* counts;                    // [phases + 1] monitoring-list sizes, then the knocked-in
                                    // pool size, the barrier's arrivals and generation, and
                                    // the barrier failure flag
    Real* values;
    unsigned long long* executed;   // per contract: positions simulated
    uint64_t seed;
    SobolTables sobol;              // nibbles32 [dims][32], directions/shifts for the tails
    const uint32_t* high_t;         // [dims][blocks]: the high part of every block, by dimension
    int high_blocks;
    const volatile int* cancel;     // host-mapped cancellation word (may be null)
    int* aborted;
    int64_t complete_below;         // monitoring paths at or below which the CTAs complete them
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

// The normals of two Sobol words of dimensions d and d + 1 (phase_sobol_from_word for
// both, the central quantile piece evaluated as a packed pair).  An element not `need`ed
// may hold any word; it is neither rebuilt nor sent to the tail piece.
__device__ __forceinline__ float2 phase_sobol_pair(const SobolTables& t, uint32_t v0, uint32_t v1, bool need0,
                                                   bool need1, uint64_t gray, int d) {
    const bool up0 = (v0 >> 31) != 0, up1 = (v1 >> 31) != 0;
    const uint32_t k0 = up0 ? ~v0 : v0, k1 = up1 ? ~v1 : v1;
    const float2 tail = __ffma2_rn(make_float2(__uint2float_rn(k0), __uint2float_rn(k1)), make_float2(0x1p-32f, 0x1p-32f),
                                   make_float2(0x1p-33f, 0x1p-33f));
    float2 z = normal_from_tail_pair(tail, up0, up1, need0 && k0 >= (1u << 12), need1 && k1 >= (1u << 12));
    if (need0 && k0 < (1u << 12)) z.x = phase_sobol_from_word(t, v0, gray, d);
    if (need1 && k1 < (1u << 12)) z.y = phase_sobol_from_word(t, v1, gray, d + 1);
    return z;
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
    // Four positions per iteration: their normals are drawn together (two packed
    // quantile pairs for Sobol), then the bridge steps run in order; a path that decides
    // knock-in early leaves the later ones unused.
    bool walking = L.valid && L.monitoring;
    int next = start + 1;
    const UnitT<Real>* up = units + start + 1;
    size_t hi = size_t(start + 1) * a.high_blocks + block;  // Sobol: high table and nibble rows
    size_t ri = size_t(start + 1) * 32;
    const size_t hstep = size_t(4) * a.high_blocks;
    for (int q = start + 1; __any_sync(kFull, walking && q <= end); q += 4, up += 4, hi += hstep, ri += 128) {
        bool s[4];
        UnitT<Real> u[4];
        Real z[4];
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            s[j] = walking && q + j <= end;
            u[j] = UnitT<Real>{};
            z[j] = Real(0);
        }
        if constexpr (SOBOL) {
            const uint32_t* row = a.sobol.nibbles32 + ri;
            uint32_t w[4];
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                w[j] = 0;
                if (s[j]) {
                    u[j] = up[j];
                    w[j] = __ldg(a.high_t + hi + size_t(j) * a.high_blocks) ^ __ldg(row + 32 * j + glo) ^
                           __ldg(row + 32 * j + ghi);
                }
            }
            const float2 za = phase_sobol_pair(a.sobol, w[0], w[1], s[0], s[1], gray, q);
            const float2 zb = phase_sobol_pair(a.sobol, w[2], w[3], s[2], s[3], gray, q + 2);
            z[0] = za.x;
            z[1] = za.y;
            z[2] = zb.x;
            z[3] = zb.y;
        } else {
#pragma unroll
            for (int j = 0; j < 4; ++j)
                if (s[j]) {
                    u[j] = up[j];
                    z[j] = pn.normal();
                    next = q + j + 1;
                }
        }
#pragma unroll
        for (int j = 0; j < 4; ++j)
            if (s[j] && walking) {
                const Real daily = lr + xfma(u[j].b, target - lr, u[j].a * z[j]);
                lr = daily;
                minimum = daily < minimum ? daily : minimum;
                executed += 1;
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

// Loads path `idx` of a list (or, in the first interval, sample `idx` of the book) into
// a lane; returns the interval it runs next.
template <class Real, bool SOBOL>
__device__ __forceinline__ int phase_load(const PhaseArgs<Real, SOBOL>& a, const PhaseEntry<Real, SOBOL>* list,
                                          int64_t idx, PhaseLane<Real>& L, PcgSource<Real>& pn) {
    if (!list) {
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
        L.lr = Real(0);
        L.cash = c0.initial_cash;
        if (!SOBOL) pn.start(a.seed, L.sample, a.dims[lo]);
        return 0;
    }
    const PhaseEntry<Real, SOBOL> e = list[idx];
    L.sample = e.sample;
    L.contract = int(e.tag >> kPhaseTagShift);
    L.monitoring = (e.tag & kPhaseMonitoring) != 0;
    L.knocked_in = (e.tag & kPhaseKnockedIn) != 0;
    L.lr = e.lr;
    L.cash = e.cash;
    if constexpr (!SOBOL) {
        pn.g.state = e.state;
        pn.g.inc = ((uint64_t(L.sample) / kBlockSize) << 1) | 1;
        pn.spare = e.spare;
        pn.has_spare = e.has_spare != 0;
    }
    return int((e.tag >> kPhaseIntervalShift) & (kPhaseMaxIntervals - 1));
}

// Adds the positions a warp's lanes simulated to their contracts' counters.
__device__ __forceinline__ void phase_count(unsigned long long* counters, int contract, int executed, int lane) {
    constexpr unsigned kFull = 0xffffffffu;
    const int lead = __shfl_sync(kFull, contract, 0);
    if (__all_sync(kFull, contract == lead || executed == 0)) {
        const unsigned total = __reduce_add_sync(kFull, unsigned(executed));
        if (lane == 0 && total) atomicAdd(counters + lead, (unsigned long long)total);
    } else if (executed) {
        atomicAdd(counters + contract, (unsigned long long)executed);
    }
}

// Appends the flagged lanes of a warp to a list, one atomic per warp.
template <class Entry>
__device__ __forceinline__ void phase_append(Entry* list, int* count, bool keep, const Entry& e, int lane,
                                             unsigned below) {
    const unsigned b = __ballot_sync(0xffffffffu, keep);
    int base = 0;
    if (lane == 0 && b) base = atomicAdd(count, __popc(b));
    base = __shfl_sync(0xffffffffu, base, 0);
    if (keep) list[base + __popc(b & below)] = e;
}

// Grid-wide barrier of the cooperative launch.  The wait is bounded: after about two
// seconds it records a failure and returns false, and the kernel stops.
constexpr long long kPhaseBarrierCycles = 4000000000LL;

__device__ __forceinline__ bool phase_grid_sync(int* arrive, volatile int* generation, int* failed) {
    __shared__ int ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        const int g = *generation;
        __threadfence();
        if (atomicAdd(arrive, 1) == int(gridDim.x) - 1) {
            atomicExch(arrive, 0);
            __threadfence();
            atomicAdd((int*)generation, 1);
        } else {
            const long long t0 = clock64();
            while (*generation == g) {
                if (clock64() - t0 > kPhaseBarrierCycles) {
                    atomicExch(failed, 1);
                    break;
                }
                __nanosleep(64);
            }
        }
        __threadfence();
        ok = *(volatile int*)failed == 0;
    }
    __syncthreads();
    return ok != 0;  // the same answer for every thread of the CTA
}

// Runs paths of a list to completion, a CTA batch of kThreads paths at a time.  After
// every interval the batch's live paths are compacted to the front of the CTA through
// shared memory, so its warps stay full while the batch thins out.  A path that knocks
// in moves to the knocked-in pool.
template <class Real, bool SOBOL>
__device__ void phase_complete(const PhaseArgs<Real, SOBOL>& a, const PhaseEntry<Real, SOBOL>* list, int64_t count,
                               int first_phase, PhaseEntry<Real, SOBOL>* pool, int* warp_live) {
    constexpr unsigned kFull = 0xffffffffu;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const unsigned below = lanemask_lt();
    int* knocked_count = a.counts + a.phases + 1;
    for (int64_t base = int64_t(blockIdx.x) * kThreads; base < count; base += int64_t(gridDim.x) * kThreads) {
        PhaseLane<Real> L;
        PcgSource<Real> pn;
        L.valid = base + threadIdx.x < count;
        L.sample = 0;
        L.contract = 0;
        L.monitoring = L.knocked_in = false;
        L.lr = L.cash = Real(0);
        int phase = first_phase;
        if (L.valid) {
            const int p = phase_load<Real, SOBOL>(a, list, base + threadIdx.x, L, pn);
            if (list) phase = p;
        }
        bool alive = L.valid;
        for (;;) {
            // Compact the live paths to the front of the CTA.
            const unsigned b = __ballot_sync(kFull, alive);
            if (lane == 0) warp_live[warp] = __popc(b);
            __syncthreads();
            int offset = 0, live = 0;
            for (int w = 0; w < kWarps; ++w) {
                offset += w < warp ? warp_live[w] : 0;
                live += warp_live[w];
            }
            if (live == 0) break;
            if (alive) pool[offset + __popc(b & below)] = phase_entry<Real, SOBOL>(L, phase, pn);
            __syncthreads();
            L.valid = int(threadIdx.x) < live;
            if (L.valid) phase = phase_load<Real, SOBOL>(a, pool, threadIdx.x, L, pn);
            __syncthreads();
            bool finished = false;
            int executed = 0;
            if (warp * 32 < live) {
                finished = phase_interval<Real, SOBOL>(a, phase, L, pn, executed);
                phase_count(a.executed, L.contract, executed, lane);
                alive = L.valid && !finished;
                ++phase;
                const bool to_pool = alive && !L.monitoring;
                phase_append(a.knocked, knocked_count, to_pool, phase_entry<Real, SOBOL>(L, phase, pn), lane, below);
                alive = alive && !to_pool;
            } else {
                alive = false;
            }
        }
    }
}

// Runs the knocked-in pool to completion.  A knocked-in path only draws its interval
// ends, so the warp keeps its 32 paths to the end with no compaction: lanes whose path
// finished idle while the others take their remaining intervals (at most the contract's
// interval count).
template <class Real, bool SOBOL>
__device__ void phase_drain(const PhaseArgs<Real, SOBOL>& a, int64_t count) {
    constexpr unsigned kFull = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const int64_t warps = int64_t(gridDim.x) * kWarps;
    for (int64_t ch = (int64_t(blockIdx.x) * kThreads + threadIdx.x) / 32; ch * 32 < count; ch += warps) {
        const int64_t idx = ch * 32 + lane;
        PhaseLane<Real> L;
        PcgSource<Real> pn;
        L.valid = idx < count;
        L.sample = 0;
        L.contract = 0;
        L.monitoring = L.knocked_in = false;
        L.lr = L.cash = Real(0);
        int phase = 0;
        if (L.valid) phase = phase_load<Real, SOBOL>(a, a.knocked, idx, L, pn);
        bool alive = L.valid;
        int executed = 0;
        while (__any_sync(kFull, alive)) {
            L.valid = alive;
            const bool finished = phase_interval<Real, SOBOL>(a, phase, L, pn, executed);
            alive = alive && !finished;
            ++phase;
        }
        phase_count(a.executed, L.contract, executed, lane);
    }
}

// One cooperative launch prices the book.  While more paths monitor knock-in than fill
// one wave of resident lanes, every interval is a grid-wide step: each warp advances 32
// paths of the current monitoring list by one interval, appends the survivors to the
// next list (knocked-in ones to the pool), and a grid barrier ends the step.  Then the
// CTAs complete the remaining monitoring paths, and after one more barrier the
// knocked-in pool.
template <class Real, bool SOBOL>
__global__ void __launch_bounds__(kThreads, 4) phased_kernel(PhaseArgs<Real, SOBOL> a) {
    using Entry = PhaseEntry<Real, SOBOL>;
    __shared__ Entry pool[kThreads];
    __shared__ int warp_live[kWarps];
    const int lane = threadIdx.x & 31;
    const unsigned below = lanemask_lt();
    int* knocked_count = a.counts + a.phases + 1;
    int* arrive = a.counts + a.phases + 2;
    volatile int* generation = a.counts + a.phases + 3;
    int* failed = a.counts + a.phases + 4;
    int phase = 0;
    int64_t count = a.total;
    const int64_t warps = int64_t(gridDim.x) * kWarps;
    while (count > a.complete_below && phase < a.phases) {
        if (a.cancel && blockIdx.x == 0 && threadIdx.x == 0 && *a.cancel) atomicExch(a.aborted, 1);
        const Entry* in = phase == 0 ? nullptr : a.lists + size_t(phase % 2) * a.total;
        Entry* out = a.lists + size_t((phase + 1) % 2) * a.total;
        int* out_count = a.counts + phase + 1;
        const int64_t chunks = (count + 31) / 32;
        for (int64_t ch = (int64_t(blockIdx.x) * kThreads + threadIdx.x) / 32; ch < chunks; ch += warps) {
            const int64_t idx = ch * 32 + lane;
            PhaseLane<Real> L;
            PcgSource<Real> pn;
            L.valid = idx < count;
            L.sample = 0;
            L.contract = 0;
            L.monitoring = L.knocked_in = false;
            L.lr = L.cash = Real(0);
            if (L.valid) phase_load<Real, SOBOL>(a, in, idx, L, pn);
            int executed = 0;
            const bool finished = phase_interval<Real, SOBOL>(a, phase, L, pn, executed);
            phase_count(a.executed, L.contract, executed, lane);
            // Survivors: monitoring paths to the next list, knocked-in paths to the pool.
            const bool keep = L.valid && !finished;
            const Entry e = phase_entry<Real, SOBOL>(L, phase + 1, pn);
            phase_append(out, out_count, keep && L.monitoring, e, lane, below);
            phase_append(a.knocked, knocked_count, keep && !L.monitoring, e, lane, below);
        }
        // The cancellation word is read before the barrier, so after it every thread
        // sees the same value.
        if (!phase_grid_sync(arrive, generation, failed) || *(volatile int*)a.aborted) return;
        ++phase;
        count = *(volatile int*)(a.counts + phase);
    }
    phase_complete<Real, SOBOL>(a, phase == 0 ? nullptr : a.lists + size_t(phase % 2) * a.total, count, phase,
                                pool, warp_live);
    if (!phase_grid_sync(arrive, generation, failed)) return;
    phase_drain<Real, SOBOL>(a, *(volatile int*)knocked_count);
}

// The high part of every reference block, dimension-major: out[d * blocks + b] is the
// shift of dimension d XOR the directions of the gray-code bits >= 8 of block b's first
// point (those bits are the gray code of b).  Grid: (block tiles, dimensions).
static __global__ void sobol_high_table_t_kernel(SobolTables t, int blocks, uint32_t* out) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    const int d = blockIdx.y;
    if (b >= blocks) return;
    uint32_t g = uint32_t(b) ^ (uint32_t(b) >> 1);
    uint32_t x = t.shifts32[d];
    for (; g; g &= g - 1) x ^= t.directions32[size_t(__ffs(g) - 1 + 8) * t.dims + d];
    out[size_t(d) * blocks + b] = x;
}

}  // namespace kgpu
