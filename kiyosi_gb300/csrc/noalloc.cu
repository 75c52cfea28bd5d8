// Pricing one contract without allocating device memory.
//
// Some callers cannot call cudaMalloc: a host application that reserves its whole
// device-memory budget up front and hands out slices itself, a plugin running inside
// such a host, or a latency-critical pricing loop that must never pay an allocation or
// risk an out-of-memory failure mid-session.  kgpu_price_contract_noalloc serves them:
// it runs the FP64 plain schedule (one thread per sample, reference blocks as CUDA
// blocks, block-ordered Welford merge) with all of its scratch -- the per-block moments,
// the merged moments and the compiled contract record -- in one file-scope device array
// of fixed size, which every GPU that loads this library holds until process exit.
#include <cuda_runtime.h>

#include <cstdio>
#include <mutex>

#include "../../include/kgpu.h"
#include "api_internal.h"
#include "launch.h"

namespace {

using kgpu::BlockPartial;
using kgpu::ContractT;

// At most this many reference blocks of 256 samples per call (4,194,304 samples).
constexpr int kNoAllocMaxBlocks = 16384;

struct NoAllocScratch {
    BlockPartial partials[kNoAllocMaxBlocks];
    BlockPartial merged;
    ContractT<double> contract;
};

// The scratch.  Its host-side name is only a stand-in: device code is handed the
// address cudaGetSymbolAddress returns for the current device.
static __device__ __align__(256) unsigned char g_noalloc_scratch[sizeof(NoAllocScratch)];

constexpr int kMaxDevices = 64;
std::mutex g_noalloc_mutex;
NoAllocScratch* g_noalloc_address[kMaxDevices] = {};

// Failures are reported through kgpu_last_error_message(NULL) (thread-local).
kgpu_status noalloc_fail(kgpu_status status, const char* message) {
    kgpu::set_thread_error(message);
    return status;
}

// Device address of the scratch on the current device, looked up by the first call on
// each device (with that device current) and kept; that first call belongs before any
// stream capture.
kgpu_status scratch_address(NoAllocScratch** out) {
    int device = 0;
    if (cudaGetDevice(&device) != cudaSuccess || device < 0 || device >= kMaxDevices)
        return noalloc_fail(KGPU_DEVICE_ERROR, "no usable current CUDA device");
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    if (!g_noalloc_address[device]) {
        void* ptr = nullptr;
        const cudaError_t rc = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
        if (rc != cudaSuccess || !ptr) return noalloc_fail(KGPU_DEVICE_ERROR, cudaGetErrorString(rc));
        g_noalloc_address[device] = static_cast<NoAllocScratch*>(ptr);
    }
    *out = g_noalloc_address[device];
    return KGPU_OK;
}

// The plan checks kgpu_price_book makes on host books, made here on the device book
// through fixed host stack buffers: every event step of an autocallable has an event
// record (the kernel reads one record per event step), and bridge intervals end in
// ascending order with the last one on the final step.
kgpu_status check_device_plan(const kgpu_book& book, const kgpu_contract& c, cudaStream_t st) {
    constexpr int kChunk = 4096;
    if (c.payoff == KGPU_PAYOFF_AUTOCALLABLE) {
        uint8_t flags[kChunk];
        int events = 0;
        for (int q = 0; q < c.step_count; q += kChunk) {
            const int n = c.step_count - q < kChunk ? c.step_count - q : kChunk;
            if (cudaMemcpyAsync(flags, book.step_flags + c.step_offset + q, size_t(n), cudaMemcpyDeviceToHost, st) !=
                    cudaSuccess ||
                cudaStreamSynchronize(st) != cudaSuccess)
                return noalloc_fail(KGPU_DEVICE_ERROR, "cannot read the step flags");
            for (int k = 0; k < n; ++k) events += (flags[k] & KGPU_STEP_EVENT) != 0;
        }
        if (events != c.event_count) return noalloc_fail(KGPU_INVALID_INPUT, "event steps and event records differ");
    }
    if (c.flags & KGPU_C_BRIDGE) {
        constexpr int kIntervals = kChunk / int(sizeof(kgpu_bridge_interval)) + 1;
        kgpu_bridge_interval intervals[kIntervals];
        int previous = -1;
        for (int q = 0; q < c.bridge_count; q += kIntervals) {
            const int n = c.bridge_count - q < kIntervals ? c.bridge_count - q : kIntervals;
            if (cudaMemcpyAsync(intervals, book.intervals + c.bridge_offset + q, sizeof(kgpu_bridge_interval) * n,
                                cudaMemcpyDeviceToHost, st) != cudaSuccess ||
                cudaStreamSynchronize(st) != cudaSuccess)
                return noalloc_fail(KGPU_DEVICE_ERROR, "cannot read the bridge intervals");
            for (int k = 0; k < n; ++k) {
                if (intervals[k].end <= previous || intervals[k].end >= c.step_count)
                    return noalloc_fail(KGPU_INVALID_INPUT, "bridge intervals end out of order");
                previous = intervals[k].end;
            }
        }
        if (previous != c.step_count - 1)
            return noalloc_fail(KGPU_INVALID_INPUT, "the last bridge interval must end the grid");
    }
    return KGPU_OK;
}

}  // namespace

extern "C" kgpu_status kgpu_price_contract_noalloc(const kgpu_model* model, const kgpu_book* device_book,
                                                   int32_t contract, const kgpu_settings* settings,
                                                   kgpu_estimate* out, void* stream) {
    kgpu::set_thread_error("");
    if (!model || !device_book || !settings || !out)
        return noalloc_fail(KGPU_INVALID_INPUT, "null argument");
    if (model->kind < KGPU_MODEL_BSM || model->kind > KGPU_MODEL_LOCAL_VOL)
        return noalloc_fail(KGPU_INVALID_INPUT, "unknown model");
    if (model->kind != KGPU_MODEL_BSM && model->kind != KGPU_MODEL_HESTON)
        return noalloc_fail(KGPU_UNSUPPORTED_OPERATION, "the no-allocation entry point prices BSM and Heston");
    if (settings->sampling != KGPU_SAMPLING_PSEUDO_RANDOM && settings->sampling != KGPU_SAMPLING_SOBOL)
        return noalloc_fail(KGPU_INVALID_INPUT, "unknown sampling");
    if (settings->sampling != KGPU_SAMPLING_PSEUDO_RANDOM)
        return noalloc_fail(KGPU_UNSUPPORTED_OPERATION, "the no-allocation entry point samples pseudo-random paths");
    if (settings->precision != KGPU_PRECISION_FP64 && settings->precision != KGPU_PRECISION_FP32)
        return noalloc_fail(KGPU_INVALID_INPUT, "unknown precision");
    if (settings->schedule < KGPU_SCHEDULE_PLAIN || settings->schedule > KGPU_SCHEDULE_LANE_REFILL)
        return noalloc_fail(KGPU_INVALID_INPUT, "unknown schedule");
    if (settings->precision != KGPU_PRECISION_FP64 || settings->schedule != KGPU_SCHEDULE_PLAIN)
        return noalloc_fail(KGPU_UNSUPPORTED_OPERATION,
                            "the no-allocation entry point runs the FP64 plain schedule only");
    if (contract < 0 || contract >= device_book->contract_count || !device_book->contracts)
        return noalloc_fail(KGPU_INVALID_INPUT, "contract index out of range");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    // The contract record, read from device memory into this stack frame.
    kgpu_contract c;
    if (cudaMemcpyAsync(&c, device_book->contracts + contract, sizeof c, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess)
        return noalloc_fail(KGPU_DEVICE_ERROR, "cannot read the contract record");
    const int64_t paths = c.path_count > 0 ? c.path_count : settings->path_count;
    if (paths < 1 || paths > 2147483647LL) return noalloc_fail(KGPU_INVALID_INPUT, "path_count must be positive");
    if (c.payoff < KGPU_PAYOFF_EUROPEAN || c.payoff > KGPU_PAYOFF_DIGITAL)
        return noalloc_fail(KGPU_INVALID_INPUT, "unknown payoff");
    if (!(c.spot > 0.0) || !std::isfinite(c.spot))
        return noalloc_fail(KGPU_INVALID_INPUT, "spot must be positive and finite");
    if ((c.flags & KGPU_C_BRIDGE) && model->kind != KGPU_MODEL_BSM)
        return noalloc_fail(KGPU_INVALID_INPUT, "a bridge plan needs BSM");
    if (c.step_count < 1 || c.step_offset < 0 || c.step_offset + c.step_count > device_book->step_total)
        return noalloc_fail(KGPU_INVALID_INPUT, "steps out of range");
    if (!device_book->steps || !device_book->step_flags)
        return noalloc_fail(KGPU_INVALID_INPUT, "steps missing");
    if (c.event_count < 0 || c.event_offset < 0 || c.event_offset + c.event_count > device_book->event_total)
        return noalloc_fail(KGPU_INVALID_INPUT, "events out of range");
    if (c.event_count > 0 && !device_book->events)
        return noalloc_fail(KGPU_INVALID_INPUT, "events missing");
    if ((c.flags & KGPU_C_BRIDGE) &&
        (!device_book->bridge_daily || !device_book->intervals || c.bridge_count < 1 || c.bridge_offset < 0 ||
         c.bridge_offset + c.bridge_count > device_book->interval_total))
        return noalloc_fail(KGPU_INVALID_INPUT, "invalid bridge plan");
    if (c.payoff == KGPU_PAYOFF_AUTOCALLABLE || (c.flags & KGPU_C_BRIDGE)) {
        const kgpu_status plan = check_device_plan(*device_book, c, st);
        if (plan != KGPU_OK) return plan;
    }
    const bool terminal = c.payoff == KGPU_PAYOFF_EUROPEAN || c.payoff == KGPU_PAYOFF_DIGITAL;
    const int step_dims = c.step_count * (model->kind == KGPU_MODEL_HESTON ? 2 : 1);
    if (c.dimensions < 0 || (c.dimensions > 0 && (terminal || c.dimensions < step_dims)))
        return noalloc_fail(KGPU_INVALID_INPUT, "dimensions must cover every step's normals");
    const int64_t samples = settings->antithetic ? (paths + 1) / 2 : paths;
    const int64_t blocks = (samples + 255) / 256;
    if (blocks > kNoAllocMaxBlocks)
        return noalloc_fail(KGPU_INVALID_INPUT,
                            "path count exceeds the no-allocation scratch limit of 4,194,304 samples");
    NoAllocScratch* scratch = nullptr;
    kgpu_status status = scratch_address(&scratch);
    if (status != KGPU_OK) return status;
    // Every field of the scratch is written before it is read (the compiled contract,
    // one partial per block, the merged moments), so nothing needs clearing.
    if (kgpu::launch_compile_contracts_fp64(device_book->contracts + contract, 1, &scratch->contract, st) !=
        cudaSuccess)
        return noalloc_fail(KGPU_DEVICE_ERROR, "contract compile launch failed");
    kgpu::PlainArgs<double> a;
    a.book.contracts = &scratch->contract;
    a.book.steps = reinterpret_cast<const kgpu::StepT<double>*>(device_book->steps);
    a.book.flags = device_book->step_flags;
    a.book.events = device_book->event_total ? reinterpret_cast<const kgpu::EventT<double>*>(device_book->events) : nullptr;
    a.book.intervals =
        device_book->interval_total ? reinterpret_cast<const kgpu::IntervalT<double>*>(device_book->intervals) : nullptr;
    a.book.daily = reinterpret_cast<const kgpu::DailyT<double>*>(device_book->bridge_daily);
    a.book.units = nullptr;
    a.book.ends = nullptr;
    a.contract = 0;
    a.dims = terminal ? 1 : c.dimensions > 0 ? c.dimensions : step_dims;
    a.paths = paths;
    a.samples = samples;
    a.seed = settings->seed;
    a.antithetic = settings->antithetic;
    a.statistics = !settings->antithetic || paths % 2 == 0;
    a.variance = a.statistics && !settings->antithetic;
    a.sobol = kgpu::SobolTables{nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, 0};
    a.partials = scratch->partials;
    const size_t smem = kgpu::plain_smem_bytes(KGPU_PRECISION_FP64, false, a.dims, 0);
    if (kgpu::launch_plain_fp64(model->kind, false, int(blocks), smem, st, a, *model, nullptr) != cudaSuccess)
        return noalloc_fail(KGPU_DEVICE_ERROR, "pricing kernel launch failed");
    kgpu::merge_blocks_kernel<<<1, kgpu::kMergeThreads, 0, st>>>(scratch->partials, int(blocks), a.variance, a.statistics,
                                                 settings->antithetic, &scratch->merged);
    if (cudaGetLastError() != cudaSuccess) return noalloc_fail(KGPU_DEVICE_ERROR, "merge kernel launch failed");
    BlockPartial merged;
    if (cudaMemcpyAsync(&merged, &scratch->merged, sizeof merged, cudaMemcpyDeviceToHost, st) != cudaSuccess)
        return noalloc_fail(KGPU_DEVICE_ERROR, "cannot read the merged moments");
    const cudaError_t rc = cudaStreamSynchronize(st);
    if (rc != cudaSuccess) return noalloc_fail(KGPU_DEVICE_ERROR, cudaGetErrorString(rc));
    kgpu_settings s = *settings;
    s.sampling = KGPU_SAMPLING_PSEUDO_RANDOM;
    kgpu::estimate_from_moments(c, s, paths, merged, out);
    const int grid = terminal ? 1 : c.step_count;
    out->path_steps = double(paths) * grid;
    out->executed_steps = merged.executed;
    if (!(out->price == out->price) || out->price - out->price != 0.0)
        return noalloc_fail(KGPU_COMPUTATION_FAILURE, "Monte Carlo produced a non-finite parameter, path or result");
    return KGPU_OK;
}
