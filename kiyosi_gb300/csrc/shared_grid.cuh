// The lanes of one shared daily grid, path-major (engines/monte_carlo/autocallable/
// portfolio.rs:1275-1439).
//
// The reference walks one path per sample and lets every note of the group read it.
// That is the GB300 shape too: a thread simulates its path once, then fans out over
// every lane of the group.
//
// * Path phase. The path follows the base lane's interval plan: the interval end is
//   drawn first, then the bridged days, exactly as the per-lane bridge kernel draws them.
//   At each action date (a step where some lane pays or matures) the thread records, in
//   shared memory, the log return and the running minimum over the monitored days. The
//   layout is [date][thread], which is conflict-free.
// * Lane phase. Every lane walks its cash events on those records and settles at its
//   maturity. Knock-in is decided by the recorded minimum: the per-lane kernel stops
//   drawing a lane's days once the lane has knocked in, and the values it does draw are
//   the same, so the outcome is the same.
// * Reduction. Each CTA writes the lanes' sums and sums of squares. The merge kernel adds
//   the CTAs in a fixed order.
// * Grid. CTAs are (path tile) x (lane chunk): every chunk re-walks its tile's paths,
//   which is cheap next to the lanes, so that enough warps are resident to hide the
//   latency of the lane walk.
//
// Cost is paths x (grid steps + lane events), against paths x lanes x grid steps when
// each lane re-simulates the path.
#pragma once
#include "kernels.cuh"

namespace kgpu {

constexpr int kSharedThreads = 128;  // paths per CTA
constexpr int kSharedWarps = kSharedThreads / 32;

template <class Real>
struct SharedArgs {
    DevBook<Real> book;   // the lanes (compiled contracts, steps, events, plan)
    int lanes;
    int base;             // the lane whose grid and interval plan drive the path
    const int16_t* slot;  // [base steps]: the action-date record of each step, or -1
    int slots;
    int steps;            // base grid steps
    int dims;             // sampling dimensions per path
    int64_t samples;
    int64_t paths;
    int antithetic;       // pairs Z and -Z: sample s < paths / 2 walks both
    uint64_t seed;
    SobolTables sobol;
    double* partials;     // [lane][CTA][3]: sum, sum of squares, sum of squared pair means
    int ctas;
};

__host__ __device__ inline size_t shared_grid_smem_bytes(size_t real, int slots, int steps, bool sobol,
                                                         bool antithetic) {
    size_t records = (antithetic ? 4 : 2) * size_t(slots) * kSharedThreads * real;
    size_t sums = size_t(32) * kSharedWarps * 3 * sizeof(double);
    size_t table = (size_t(steps) * sizeof(int16_t) + 15) / 16 * 16;
    return records + sums + table + (sobol ? size_t(steps) * 8 : 0);
}

// PAIRS: antithetic pairs (a.antithetic), compiled apart so that single paths carry no
// pair bookkeeping.
template <class Real, bool SOBOL, bool PAIRS>
__global__ void __launch_bounds__(kSharedThreads) shared_grid_kernel(SharedArgs<Real> a) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const size_t plane = size_t(a.slots) * kSharedThreads;
    Real* lr = reinterpret_cast<Real*>(smem_raw);  // [slots][kSharedThreads]
    Real* mn = lr + plane;                         // [slots][kSharedThreads]
    Real* lr_neg = mn + plane;                     // the antithetic partner's records
    Real* mn_neg = lr_neg + plane;
    double* sums = reinterpret_cast<double*>(mn + (PAIRS ? 3 : 1) * plane);  // [32][warps][3]
    int16_t* slot = reinterpret_cast<int16_t*>(sums + 32 * kSharedWarps * 3);     // [steps]
    uint64_t* high = reinterpret_cast<uint64_t*>(
        reinterpret_cast<unsigned char*>(slot) + (size_t(a.steps) * sizeof(int16_t) + 15) / 16 * 16);
    const int tid = threadIdx.x, warp = tid >> 5, lane_id = tid & 31;
    for (int i = tid; i < a.steps; i += kSharedThreads) slot[i] = a.slot[i];
    const int64_t sample = int64_t(blockIdx.x) * kSharedThreads + tid;
    // A CTA's samples lie inside one reference block of 256 (kSharedThreads divides it).
    if (SOBOL) sobol_high(a.sobol, uint64_t(int64_t(blockIdx.x) * kSharedThreads / kBlockSize), high, tid,
                          kSharedThreads);
    __syncthreads();
    const bool active = sample < a.samples;
    const bool paired = PAIRS && active && sample < a.paths / 2;
    const ContractT<Real>& b = a.book.contracts[a.base];
    const PlanPtrs<Real> p = plan_of(a.book, b);
    if (active) {
        // bridge_payoffs' draw order: interval end, then the interval's days.
        auto walk = [&](auto& n, Real* lr, Real* mn) {
            Real x = Real(0), minimum = xinf(Real());
            int i = 0;
            for (int k = 0; k < b.bridge_count; ++k) {
                const IntervalT<Real> iv = p.intervals[k];
                const Real target = x + xfma(iv.diffusion, n.normal(), iv.drift);
                for (; i < iv.end; ++i) {
                    const DailyT<Real> d = p.daily[i];
                    x = x + xfma(d.weight, target - x, d.width * n.normal());
                    if (p.flags[i] & KGPU_STEP_KNOCK_IN) minimum = x < minimum ? x : minimum;
                }
                x = target;
                if (p.flags[iv.end] & KGPU_STEP_KNOCK_IN) minimum = x < minimum ? x : minimum;
                i = iv.end + 1;
                const int s = slot[iv.end];
                if (s >= 0) {
                    lr[size_t(s) * kSharedThreads + tid] = x;
                    mn[size_t(s) * kSharedThreads + tid] = minimum;
                }
            }
        };
        if (SOBOL) {
            SobolSource<Real> n{high, a.sobol.nibbles, a.dims, 0, 0, 0};
            n.start(uint64_t(sample));
            walk(n, lr, mn);
            if (paired) {
                n.start(uint64_t(sample));
                Negated<SobolSource<Real>, Real> neg{n};
                walk(neg, lr_neg, mn_neg);
            }
        } else {
            PcgSource<Real, true> n;
            n.start(a.seed, uint64_t(sample), a.dims);
            walk(n, lr, mn);
            if (paired) {
                n.start(a.seed, uint64_t(sample), a.dims);
                Negated<PcgSource<Real, true>, Real> neg{n};
                walk(neg, lr_neg, mn_neg);
            }
        }
    }
    // Lane phase over this CTA's chunk of lanes (blockIdx.y); each thread reads only its
    // own columns of the records.
    const int per_chunk = (a.lanes + int(gridDim.y) - 1) / int(gridDim.y);
    const int l_begin = int(blockIdx.y) * per_chunk;
    const int l_end = min(a.lanes, l_begin + per_chunk);
    // One lane's value on one path's records.
    auto settle = [&](const ContractT<Real>& c, const Real* my_lr, const Real* my_mn) {
        const EventT<Real>* ev = a.book.events ? a.book.events + c.event_offset : nullptr;
        Real cash = c.initial_cash;
        // A warp walks a lane's events until its last path knocks out, so the walk
        // runs to the end with the knocked-out paths masked: the loads of successive
        // events are independent and overlap.
        bool live = true;
#pragma unroll 4
        for (int e = 0; e < c.event_count; ++e) {
            const EventT<Real>& E = ev[e];
            const Real y = my_lr[size_t(slot[E.step]) * kSharedThreads];
            const bool hit = E.has_knock_out && y >= E.knock_out;
            const Real pay = E.payment[int(y >= E.coupon_barrier) | (int(hit) << 1)];
            if (live) cash += pay;
            live = live && !hit;
        }
        if (live) {
            const size_t m = size_t(slot[c.step_count - 1]) * kSharedThreads;
            const Real y = my_lr[m];
            const bool has = (c.flags & KGPU_C_HAS_KNOCK_IN) != 0;
            const bool ki = (c.flags & KGPU_C_KNOCKED_IN) || (has && my_mn[m] < c.knock_in) ||
                            ((c.flags & KGPU_C_EXPIRY_KNOCK_IN) && has && y < c.knock_in);
            cash += autocallable_terminal(c, spot_at(c.spot, y), ki) * c.final_discount;
        }
        return cash;
    };
    for (int l = l_begin; l < l_end; ++l) {
        Real v = Real(0), q = Real(0), r = Real(0);
        if (active) {
            const ContractT<Real>& c = a.book.contracts[l];
            const Real x = settle(c, lr + tid, mn + tid);
            v = x;
            q = x * x;
            if (paired) {
                const Real y = settle(c, lr_neg + tid, mn_neg + tid);
                const Real m = (x + y) / Real(2);
                v = x + y;
                q = q + y * y;
                r = m * m;
            }
        }
        // Warp sums in the kernel's precision, CTA sums in FP64.
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) {
            v += __shfl_down_sync(0xffffffffu, v, off);
            q += __shfl_down_sync(0xffffffffu, q, off);
            if (PAIRS) r += __shfl_down_sync(0xffffffffu, r, off);
        }
        const int j = l - l_begin;
        if (lane_id == 0) {
            double* slot_sums = sums + ((j & 31) * kSharedWarps + warp) * 3;
            slot_sums[0] = double(v);
            slot_sums[1] = double(q);
            slot_sums[2] = double(r);
        }
        if ((j & 31) == 31 || l == l_end - 1) {
            __syncthreads();
            const int first = l - (j & 31);
            if (tid <= l - first) {
                double t0 = 0.0, t1 = 0.0, t2 = 0.0;
#pragma unroll
                for (int w = 0; w < kSharedWarps; ++w) {
                    const double* u = sums + (tid * kSharedWarps + w) * 3;
                    t0 += u[0];
                    t1 += u[1];
                    t2 += u[2];
                }
                double* out = a.partials + (size_t(first + tid) * a.ctas + blockIdx.x) * 3;
                out[0] = t0;
                out[1] = t1;
                out[2] = t2;
            }
            __syncthreads();
        }
    }
}

// One warp per lane adds the CTAs' sums in a fixed order.
static __global__ void shared_merge_kernel(const double* partials, int ctas, int lanes, double* out) {
    const int l = blockIdx.x;
    if (l >= lanes) return;
    const double* row = partials + size_t(l) * ctas * 3;
    double s = 0.0, q = 0.0, r = 0.0;
    for (int i = threadIdx.x; i < ctas; i += 32) {
        s += row[3 * i];
        q += row[3 * i + 1];
        r += row[3 * i + 2];
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        s += __shfl_down_sync(0xffffffffu, s, off);
        q += __shfl_down_sync(0xffffffffu, q, off);
        r += __shfl_down_sync(0xffffffffu, r, off);
    }
    if (threadIdx.x == 0) {
        out[3 * l] = s;
        out[3 * l + 1] = q;
        out[3 * l + 2] = r;
    }
}

}  // namespace kgpu
