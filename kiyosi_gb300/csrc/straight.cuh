// Books whose paths take every grid step to the end -- arithmetic Asians on their fixings
// and vanilla paths, under any model -- in FP32 with pseudo-random sampling: one thread
// per path.
//
// The lane-refill kernel exists for books whose paths end at different steps (knock-outs,
// bridge skips): a warp pulls work items from a queue and refills finished lanes, and
// every unit of work goes through the payoff dispatch.  A path that never ends early
// needs none of that.  Here a thread walks one sample through the model step and the
// fixing rule of the lane-refill kernel's grid_step, on the same normals (path_samples
// over the model's transitions, engines/monte_carlo.rs:1498-1676), so each path's payoff
// is that kernel's; only the queue, the refills, the per-unit dispatch and the step's
// bookkeeping are gone.  The Heston Asian book (2^22 paths x 252 steps) is such a book.
#pragma once
#include "kernels.cuh"

namespace kgpu {

constexpr int kStraightThreads = 256;

struct StraightArgs {
    DevBook<float> book;
    int contract_count;
    int64_t total;                 // samples of the book
    const int64_t* value_offset;   // [contract_count + 1]: first slot of a contract's samples
    const int* dims;               // per contract: normals per sample (stream positions)
    uint64_t seed;
    float* values;                 // per-path payoffs
    unsigned long long* executed;  // per contract: grid steps simulated
    const volatile int* cancel;    // host-mapped cancellation word (may be null)
    int* aborted;
};

// Shared memory: the local-volatility surface (lv_values floats), as the persistent kernel
// stages it.
template <int MODEL>
__global__ void __launch_bounds__(kStraightThreads, 4)
    straight_path_kernel(StraightArgs a, kgpu_model model, const double* lv_dev) {
    constexpr unsigned kFull = 0xffffffffu;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    DevModel<float> m;
    load_model(m, model, reinterpret_cast<float*>(smem_raw), lv_dev);
    __syncthreads();
    if (a.cancel && threadIdx.x == 0 && *a.cancel) atomicExch(a.aborted, 1);
    const int lane = threadIdx.x & 31;
    const int64_t idx = int64_t(blockIdx.x) * kStraightThreads + threadIdx.x;
    const bool valid = idx < a.total;
    // The contract of sample idx: the last c with value_offset[c] <= idx.
    int contract = 0;
    if (valid) {
        int lo = 0, hi = a.contract_count - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) / 2;
            if (a.value_offset[mid] <= idx) lo = mid;
            else hi = mid - 1;
        }
        contract = lo;
    }
    int steps_done = 0;
    if (valid) {
        const ContractT<float>& c = a.book.contracts[contract];
        const int64_t sample = idx - a.value_offset[contract];
        const PlanPtrs<float> p = plan_of(a.book, c);
        PathState<float> s;
        path_init(s, c, m.v0);
        PcgSource<float> n;
        n.start(a.seed, uint64_t(sample), a.dims[contract]);
        // grid_step's model step and fixing rule, step by step to the last; a plan without
        // steps gives NaN there (no step ends the path) and here.
        const int steps = c.step_count;
        if (MODEL == KGPU_MODEL_HESTON && !n.has_spare) {
            // A Heston step takes both normals of one Box-Muller draw, so a path that
            // starts on a fresh draw starts every step on one: stating it lets the
            // compiler drop the spare's branches.
            for (int i = 0; i < steps; ++i) {
                n.has_spare = false;
                model_step<float, MODEL>(m, p.steps[i], s, n);
                fixing_rule(c, p.flags[i], s);
            }
        } else {
            for (int i = 0; i < steps; ++i) {
                model_step<float, MODEL>(m, p.steps[i], s, n);
                fixing_rule(c, p.flags[i], s);
            }
        }
        a.values[a.value_offset[contract] + sample] = steps > 0 ? fixing_value(c, s) : xnan(0.f);
        steps_done = steps;
    }
    // Simulated steps per contract, one atomic per warp when the warp's samples share one.
    const int head = __shfl_sync(kFull, contract, 0);
    if (__all_sync(kFull, contract == head || steps_done == 0)) {
        const unsigned total = __reduce_add_sync(kFull, unsigned(steps_done));
        if (lane == 0 && total) atomicAdd(a.executed + head, (unsigned long long)total);
    } else if (steps_done) {
        atomicAdd(a.executed + contract, (unsigned long long)steps_done);
    }
}

}  // namespace kgpu
