// Plain and persistent Monte Carlo kernels (templates; instantiated per precision in
// kernels_fp64.cu, compiled with --fmad=false, and kernels_fp32.cu).
#pragma once
#include <cstdint>

#include "path_engine.cuh"

namespace kgpu {

constexpr int kThreads = 256;  // one CUDA block = one reference block of 256 samples
constexpr int kWarps = kThreads / 32;

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

// Sobol tables of one sequence: directions [column * dims + dim] and shifts [dim].
struct SobolTables {
    const uint64_t* directions;
    const uint64_t* shifts;
    int dims;
};

struct PlainArgs {
    DevBook book;
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

struct PersistentArgs {
    DevBook book;
    const int4* items;  // (contract, first sample, sample count, dims), grouped by contract
    const int* order;   // dispatch order of the items (longest contracts first)
    int item_count;
    int* queue;         // work-queue head
    uint64_t seed;
    SobolTables sobol;
    TilePartial* partials;
    const volatile int* cancel;  // host-mapped cancellation word (may be null)
    int* aborted;
};

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

template <class S, class Real>
struct Negated {
    S& s;
    __device__ __forceinline__ Real normal() { return -s.normal(); }
    __device__ __forceinline__ void skip(int n) { s.skip(n); }
};

// Runs one whole path to completion.
template <class Real, int MODEL, class Source>
__device__ __forceinline__ Real run_path(const DevModel<Real>& m, const kgpu_contract& c,
                                         const DevBook& b, Source& n, int& executed) {
    PathState<Real> s;
    path_init(s, c, m.v0);
    const kgpu_step* steps = b.steps + c.step_offset;
    const uint8_t* flags = b.flags + c.step_offset;
    const kgpu_event* events = b.events ? b.events + c.event_offset : nullptr;
    const kgpu_bridge_interval* intervals = b.intervals ? b.intervals + c.bridge_offset : nullptr;
    const kgpu_bridge_daily* daily = b.daily ? b.daily + c.step_offset : nullptr;
    Real value = Real(0);
    // Every path ends within step_count + bridge_count units of work.
    int guard = 2 * c.step_count + c.bridge_count + 2;
    while (!path_step<Real, MODEL>(m, c, steps, flags, events, intervals, daily, s, n, value)) {
        if (--guard == 0) {
            value = Real(__int_as_float(0x7fc00000));  // NaN: reported as a computation failure
            break;
        }
    }
    executed = s.executed;
    return value;
}

// Plain schedule: thread = sample, CUDA block = reference block; the block's moments are
// accumulated sequentially in sample order as sample_paths does (monte_carlo.rs:1778-1798).
template <class Real, int MODEL, bool SOBOL>
__global__ void __launch_bounds__(kThreads) plain_kernel(PlainArgs a, kgpu_model model,
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
    const kgpu_contract& c = a.book.contracts[a.contract];
    const int64_t sample = int64_t(block) * kBlockSize + threadIdx.x;
    double positive = 0.0, negative = 0.0;
    int executed = 0;
    if (sample < a.samples) {
        const bool paired = a.antithetic && sample < a.paths / 2;
        int e1 = 0, e2 = 0;
        if (SOBOL) {
            SobolSource<Real> n{high, a.sobol.directions, a.dims, 0, 0};
            n.start(uint64_t(sample));
            positive = double(run_path<Real, MODEL>(m, c, a.book, n, e1));
            if (paired) {
                n.start(uint64_t(sample));
                Negated<SobolSource<Real>, Real> neg{n};
                negative = double(run_path<Real, MODEL>(m, c, a.book, neg, e2));
            }
        } else {
            PcgSource<Real> n;
            n.start(a.seed, uint64_t(sample), a.dims);
            positive = double(run_path<Real, MODEL>(m, c, a.book, n, e1));
            if (paired) {
                n.start(a.seed, uint64_t(sample), a.dims);
                Negated<PcgSource<Real>, Real> neg{n};
                negative = double(run_path<Real, MODEL>(m, c, a.book, neg, e2));
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
static __global__ void merge_blocks_kernel(const BlockPartial* partials, int blocks, int variance,
                                    int statistics, int antithetic, BlockPartial* out) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    BlockPartial r;
    r.moments = Moments{0, 0, 0, 0};
    r.pairs = Moments{0, 0, 0, 0};
    r.sample = Moments{0, 0, 0, 0};
    r.executed = 0.0;
    for (int b = 0; b < blocks; ++b) {
        moments_merge(r.moments, partials[b].moments, variance);
        moments_merge(r.sample, partials[b].sample, true);
        if (statistics && antithetic) moments_merge(r.pairs, partials[b].pairs, true);
        r.executed += partials[b].executed;
    }
    *out = r;
}

__device__ __forceinline__ unsigned lanemask_lt() {
    unsigned m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

// Kahan-compensated single-precision running sum.
template <class Real>
struct Compensated {
    Real sum, carry;
    __device__ __forceinline__ void add(Real x) {
        Real y = x - carry;
        Real t = sum + y;
        carry = (t - sum) - y;
        sum = t;
    }
    __device__ __forceinline__ double value() const { return double(sum) - double(carry); }
};

// Persistent schedule: warps pull (contract, tile) items from a queue; inside an item,
// a lane whose path has finished starts the tile's next unstarted sample, so the warp
// stays full however unevenly its paths end (early knock-out, bridge skipping).
// Refill order is a deterministic function of the path lengths (warp-synchronous
// ballots), so results do not depend on scheduling.
template <class Real, int MODEL, bool SOBOL>
__global__ void __launch_bounds__(kThreads) persistent_kernel(PersistentArgs a, kgpu_model model,
                                                              const double* lv_dev) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    uint64_t* low = reinterpret_cast<uint64_t*>(smem_raw);                  // [8 * dims]
    uint64_t* highs = low + (SOBOL ? 8 * a.sobol.dims : 0);                 // [kWarps * dims]
    Real* lv = reinterpret_cast<Real*>(highs + (SOBOL ? kWarps * a.sobol.dims : 0));
    DevModel<Real> m;
    load_model(m, model, lv, lv_dev);
    if (SOBOL) {
        for (int i = threadIdx.x; i < 8 * a.sobol.dims; i += blockDim.x) low[i] = a.sobol.directions[i];
    }
    __syncthreads();
    const int warp = threadIdx.x >> 5;
    const int lane = threadIdx.x & 31;
    uint64_t* high = highs + (SOBOL ? warp * a.sobol.dims : 0);
    for (;;) {
        int item = 0;
        if (lane == 0) {
            int q = atomicAdd(a.queue, 1);
            if (a.cancel && *a.cancel) {
                atomicExch(a.aborted, 1);
                q = a.item_count;
            }
            item = q < a.item_count ? a.order[q] : -1;
        }
        item = __shfl_sync(0xffffffffu, item, 0);
        if (item < 0) break;
        const int4 w = a.items[item];
        const kgpu_contract& c = a.book.contracts[w.x];
        const int64_t begin = w.y, end = int64_t(w.y) + w.z;
        const int dims = w.w;
        if (SOBOL) {
            sobol_high(a.sobol, uint64_t(begin) / kBlockSize, high, lane, 32);
            __syncwarp();
        }
        const kgpu_step* steps = a.book.steps + c.step_offset;
        const uint8_t* flags = a.book.flags + c.step_offset;
        const kgpu_event* events = a.book.events ? a.book.events + c.event_offset : nullptr;
        const kgpu_bridge_interval* intervals =
            a.book.intervals ? a.book.intervals + c.bridge_offset : nullptr;
        const kgpu_bridge_daily* daily = a.book.daily ? a.book.daily + c.step_offset : nullptr;
        Compensated<Real> sum{0, 0}, sumsq{0, 0};
        int count = 0;
        int executed = 0;
        int64_t next = begin + 32;
        int64_t sample = begin + lane;
        bool active = sample < end;
        PathState<Real> s;
        PcgSource<Real> pn;
        SobolSource<Real> sn{high, low, dims, 0, 0};
        if (active) {
            path_init(s, c, m.v0);
            if (SOBOL)
                sn.start(uint64_t(sample));
            else
                pn.start(a.seed, uint64_t(sample), dims);
        }
        const int guard_limit = 2 * c.step_count + c.bridge_count + 2;
        int guard = guard_limit;
        while (__any_sync(0xffffffffu, active)) {
            bool finished = false;
            Real value = Real(0);
            if (active) {
                if (SOBOL)
                    finished = path_step<Real, MODEL>(m, c, steps, flags, events, intervals, daily, s,
                                                      sn, value);
                else
                    finished = path_step<Real, MODEL>(m, c, steps, flags, events, intervals, daily, s,
                                                      pn, value);
                if (!finished && --guard == 0) {
                    finished = true;
                    value = Real(__int_as_float(0x7fc00000));
                }
                if (finished) {
                    sum.add(value);
                    sumsq.add(value * value);
                    count += 1;
                    executed += s.executed;
                }
            }
            const unsigned done = __ballot_sync(0xffffffffu, finished);
            if (done) {
                if (finished) {
                    int64_t mine = next + __popc(done & lanemask_lt());
                    if (mine < end) {
                        sample = mine;
                        path_init(s, c, m.v0);
                        guard = guard_limit;
                        if (SOBOL)
                            sn.start(uint64_t(sample));
                        else
                            pn.start(a.seed, uint64_t(sample), dims);
                    } else {
                        active = false;
                    }
                }
                next += __popc(done);
            }
        }
        double t0 = sum.value(), t1 = sumsq.value(), t2 = double(count), t3 = double(executed);
        for (int off = 16; off > 0; off >>= 1) {
            t0 += __shfl_xor_sync(0xffffffffu, t0, off);
            t1 += __shfl_xor_sync(0xffffffffu, t1, off);
            t2 += __shfl_xor_sync(0xffffffffu, t2, off);
            t3 += __shfl_xor_sync(0xffffffffu, t3, off);
        }
        if (lane == 0) a.partials[item] = TilePartial{t0, t1, t2, t3};
        __syncwarp();
    }
}

// Sums each contract's tile partials in item order.
static __global__ void reduce_tiles_kernel(const TilePartial* partials, const int* first_item,
                                    int contracts, TilePartial* out) {
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= contracts) return;
    TilePartial r{0, 0, 0, 0};
    for (int i = first_item[c]; i < first_item[c + 1]; ++i) {
        r.sum += partials[i].sum;
        r.sumsq += partials[i].sumsq;
        r.count += partials[i].count;
        r.executed += partials[i].executed;
    }
    out[c] = r;
}

}  // namespace kgpu
