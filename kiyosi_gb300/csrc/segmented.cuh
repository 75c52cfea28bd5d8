// Books of BSM vanilla-path contracts in FP32 with pseudo-random sampling, each path walked
// in segments.
//
// A log-Euler path under BSM (path_samples over transition(), engines/monte_carlo.rs:
// 1498-1676,2123-2137) ends at the log return sum_i (drift_i + diffusion_i z_i): a step's
// increment depends on its own normal only.  So one path's steps split into kSegments
// contiguous segments that kSegments lanes of a warp walk at once, each from its own
// position of the path's PCG32 stream (the reference block's stream advanced to the
// segment's first normal, with the Box-Muller spare handled as PcgSource::start does), and
// a fixed shuffle tree adds the segment sums.  The normals are the sequential walk's; only
// the order of the FP32 additions differs.  A book of 2^16 paths then runs 2^19 threads,
// where the lane-refill kernel had 2^16 lanes and ran latency-bound at 12 warps per SM.
#pragma once
#include "path_engine.cuh"

namespace kgpu {

constexpr int kSegments = 8;
constexpr int kSegmentThreads = 256;

struct SegmentArgs {
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

// SEGMENTS lanes per path (kSegments; a template so that only the launching unit
// instantiates it).
template <int SEGMENTS>
__global__ void __launch_bounds__(kSegmentThreads) segmented_vanilla_kernel(SegmentArgs a) {
    constexpr unsigned kFull = 0xffffffffu;
    constexpr int kSegments = SEGMENTS;
    if (a.cancel && threadIdx.x == 0 && *a.cancel) atomicExch(a.aborted, 1);
    const int lane = threadIdx.x & 31;
    const int seg = lane % kSegments;
    const int64_t idx = (int64_t(blockIdx.x) * kSegmentThreads + threadIdx.x) / kSegments;
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
    const ContractT<float>& c = a.book.contracts[contract];
    const int64_t sample = valid ? idx - a.value_offset[contract] : 0;
    const int steps = valid ? c.step_count : 0;
    // Segments of an even number of steps, so that each starts a Box-Muller pair of the
    // sample's own normals whenever the sample's first normal does.
    const int per = (((steps + kSegments - 1) / kSegments) + 1) & ~1;
    const int first = min(steps, seg * per), last = min(steps, first + per);
    float part = 0.f;
    if (first < last) {
        PcgSource<float> n;
        const uint64_t pos = (uint64_t(sample) % kBlockSize) * uint64_t(a.dims[contract]) + uint64_t(first);
        n.g = pcg_new(a.seed, uint64_t(sample) / kBlockSize);
        pcg_advance(n.g, (pos / 2) * 4);
        n.has_spare = false;
        if (pos & 1) {
            float cs, sn;
            n.draw(cs, sn);
            n.spare = sn;
            n.has_spare = true;
        }
        const StepT<float>* st = a.book.steps + c.step_offset;
        for (int i = first; i < last; ++i) {
            const StepT<float> s = st[i];
            part = part + xfma(s.diffusion, n.normal(), s.drift);
        }
    }
    // Segment sums in a fixed tree; segment 0 ends with the path's log return.
#pragma unroll
    for (int off = kSegments / 2; off > 0; off >>= 1) {
        const float other = __shfl_down_sync(kFull, part, off, kSegments);
        if (seg < off) part = part + other;
    }
    const bool lead = valid && seg == 0;
    if (lead) {
        const float x = c.sign * (spot_at(c.spot, part) - c.strike);
        a.values[a.value_offset[contract] + sample] = (x > 0.f ? x : 0.f) * c.final_discount;
    }
    // Simulated steps per contract, one atomic per warp when the warp's samples share one.
    const int steps_done = lead ? steps : 0;
    const int head = __shfl_sync(kFull, contract, 0);
    if (__all_sync(kFull, contract == head || steps_done == 0)) {
        const unsigned total = __reduce_add_sync(kFull, unsigned(steps_done));
        if (lane == 0 && total) atomicAdd(a.executed + head, (unsigned long long)total);
    } else if (steps_done) {
        atomicAdd(a.executed + contract, (unsigned long long)steps_done);
    }
}

}  // namespace kgpu
