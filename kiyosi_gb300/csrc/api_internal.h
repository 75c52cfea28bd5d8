// Internal state of a kgpu_context.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/kgpu.h"

namespace kgpu {

// Grow-only device allocation owned by a context.
struct DeviceBuffer {
    void* ptr = nullptr;
    size_t bytes = 0;
    kgpu_status ensure(size_t n);
    void release();
};

void build_sobol(int dims, uint64_t seed, std::vector<uint64_t>& directions,
                 std::vector<uint64_t>& shifts);

// Records the calling thread's last error message (kgpu_last_error_message(NULL)).
void set_thread_error(const char* message);

// Reallocations of any DeviceBuffer so far: a captured launch sequence bakes in buffer
// addresses, so it is replayed only while this count is unchanged.
uint64_t alloc_generation();

struct BlockPartial;
// MonteCarloEstimate of one contract from its block-merged scaled moments.
void estimate_from_moments(const kgpu_contract& c, const kgpu_settings& s, int64_t paths,
                           const BlockPartial& p, kgpu_estimate* out);

}  // namespace kgpu

struct kgpu_context {
    int device = 0;
    int sm_count = 0;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev_start = nullptr, ev_stop = nullptr;
    std::mutex mu;
    std::string error;
    // book staging
    kgpu::DeviceBuffer contracts, steps, flags, events, intervals, daily, lv;
    // plain schedule (partials and merged sums also serve the shared-grid schedule)
    kgpu::DeviceBuffer partials, merged, shared_slots;
    // persistent schedule
    kgpu::DeviceBuffer items, order, first_item, tiles, tile_out, queue, values, value_offset, chunks, executed;
    // phase-major schedule: two generations of the monitoring list and the knocked-in
    // pool, the list sizes and completion flag, per-contract sampling dimensions
    kgpu::DeviceBuffer phase_lists, phase_counts, phase_dims;
    // the dimension-major Sobol high table of the cached sequence, for `sobol_high_t_blocks`
    // reference blocks (0: not built since the sequence was last rebuilt)
    kgpu::DeviceBuffer sobol_high_t;
    int64_t sobol_high_t_blocks = 0;
    // plan in the kernel's precision (contract table always, arrays for FP32)
    kgpu::DeviceBuffer ccontracts, csteps, cevents, cintervals, cdaily, cunits, cends;
    // Sobol sequence cache (one sequence per (seed, dims))
    kgpu::DeviceBuffer sobol_dirs, sobol_shifts, sobol_nibbles, sobol_dirs32, sobol_shifts32, sobol_nibbles32, sobol_high32;
    int sobol_dims = 0;
    uint64_t sobol_seed = 0;
    // LSMC
    kgpu::DeviceBuffer lsmc_store, lsmc_cash, lsmc_sums, lsmc_coef, lsmc_misc, mlp_params,
        mlp_scratch;
    // raw streams
    kgpu::DeviceBuffer stream_out;
    // polynomial LSMC: the captured launch sequence of the last problem and its key
    cudaGraphExec_t lsmc_exec = nullptr;
    std::vector<unsigned char> lsmc_key;
    cudaEvent_t lsmc_events[4] = {nullptr, nullptr, nullptr, nullptr};
    // The persistent schedules' launch sequence as a CUDA graph: captured on the second
    // of two consecutive calls with one key (the first one staged the sequence's metadata
    // on the device) and replayed while the calls keep that key.
    cudaGraphExec_t book_exec = nullptr;
    std::vector<unsigned char> book_key;       // key of book_exec
    std::vector<unsigned char> last_book_key;  // key of the previous direct call
    bool capturing = false;                    // a capture pass is recording
    bool capture_failed = false;               // the capture pass could not be completed
    int book_launches = 0;                     // launches the graph holds
    size_t book_path_events = 0;               // path-kernel event pairs it records
    int book_failed_slot = -1;                 // phase_counts word of a grid-barrier timeout
    int last_graph = 0;                        // the last call: 0 direct, 1 captured, 2 replayed
    // cancellation word mirrored into host-mapped memory for persistent kernels
    volatile int* cancel_host = nullptr;
    int* cancel_dev = nullptr;
    // instrumentation of the last call
    double last_kernel_ms = 0.0;
    double last_path_kernel_ms = 0.0;  // the path kernels alone (plain or persistent)
    int last_launches = 0;
    // Event pairs around each path-kernel launch of a call, grown on demand.
    std::vector<std::pair<cudaEvent_t, cudaEvent_t>> path_events;
    size_t path_events_used = 0;
    size_t h2d_bytes = 0;

    std::vector<kgpu::DeviceBuffer*> buffers() {
        return {&contracts, &steps,     &flags,     &events,   &intervals, &daily,     &lv,
                &partials,  &merged,    &shared_slots, &items,     &order,    &first_item, &tiles,    &tile_out,
                &queue,     &values,    &value_offset, &chunks, &executed, &phase_lists, &phase_counts, &phase_dims, &sobol_high_t, &sobol_dirs, &sobol_shifts, &sobol_nibbles, &sobol_dirs32, &sobol_shifts32, &sobol_nibbles32, &sobol_high32, &ccontracts, &csteps,
                &cevents,   &cintervals, &cdaily,      &cunits,     &cends,      &lsmc_store, &lsmc_cash, &lsmc_sums,
                &lsmc_coef, &lsmc_misc, &mlp_params, &mlp_scratch, &stream_out};
    }
};
