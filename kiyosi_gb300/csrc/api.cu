// C ABI of libkiyosi_gpu.so (include/kgpu.h): contexts, device buffers, the two launch
// schedules and the estimates returned to the caller.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "../../include/kgpu.h"
#include "api_internal.h"
#include "launch.h"

namespace kgpu {

#include "joe_kuo_6_21201.inc"

// SobolSequence::new (engines/monte_carlo/sobol.rs:85-134): Joe-Kuo direction numbers,
// scrambled with a random lower-triangular binary matrix (LMS) and a digital shift, both
// drawn from Pcg32::new(seed, dimension).  Directions are stored [column * dims + dim].
void build_sobol(int dims, uint64_t seed, std::vector<uint64_t>& directions,
                 std::vector<uint64_t>& shifts) {
    const uint64_t mask = (uint64_t(1) << kSobolBits) - 1;
    directions.assign(size_t(dims) * kSobolBits, 0);
    shifts.assign(dims, 0);
    const uint32_t* record = kgpu_joe_kuo_table;
    for (int d = 0; d < dims; ++d) {
        uint64_t m[kSobolBits];
        if (d == 0) {
            for (int j = 0; j < kSobolBits; ++j) m[j] = uint64_t(1) << (kSobolBits - 1 - j);
        } else {
            const int s = int(record[0]);
            const uint32_t a = record[1];
            for (int j = 0; j < s; ++j) m[j] = uint64_t(record[2 + j]) << (kSobolBits - 1 - j);
            record += s + 2;
            for (int j = s; j < kSobolBits; ++j) {
                uint64_t v = m[j - s] ^ (m[j - s] >> s);
                for (int k = 1; k < s; ++k)
                    if ((a >> (s - 1 - k)) & 1) v ^= m[j - k];
                m[j] = v;
            }
        }
        Pcg g = pcg_new(seed, uint64_t(d));
        auto word64 = [&g]() {
            uint64_t hi = pcg_next(g);
            return (hi << 32) | uint64_t(pcg_next(g));
        };
        shifts[d] = word64() & mask;
        uint64_t rows[kSobolBits];
        for (int r = 0; r < kSobolBits; ++r) {
            const int bit = kSobolBits - 1 - r;
            rows[r] = (word64() & (mask << (bit + 1))) | (uint64_t(1) << bit);
        }
        for (int j = 0; j < kSobolBits; ++j) {
            uint64_t out = 0;
            for (int r = 0; r < kSobolBits; ++r)
                out |= uint64_t(__builtin_popcountll(m[j] & rows[r]) & 1) << (kSobolBits - 1 - r);
            directions[size_t(j) * dims + d] = out;
        }
    }
}

}  // namespace kgpu

using namespace kgpu;

static thread_local std::string g_thread_error;

static kgpu_status fail(kgpu_context* ctx, kgpu_status status, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    if (ctx)
        ctx->error = buf;
    else
        g_thread_error = buf;
    return status;
}

#define CUDA_TRY(ctx, expr)                                                                  \
    do {                                                                                     \
        cudaError_t _e = (expr);                                                             \
        if (_e != cudaSuccess)                                                               \
            return fail(ctx, KGPU_DEVICE_ERROR, "%s: %s", #expr, cudaGetErrorString(_e));    \
    } while (0)

kgpu_status DeviceBuffer::ensure(size_t n) {
    if (n <= bytes) return KGPU_OK;
    if (ptr) cudaFree(ptr);
    ptr = nullptr;
    bytes = 0;
    size_t want = std::max<size_t>(n, 256);
    if (cudaMalloc(&ptr, want) != cudaSuccess) {
        ptr = nullptr;
        return KGPU_DEVICE_ERROR;
    }
    bytes = want;
    return KGPU_OK;
}

void DeviceBuffer::release() {
    if (ptr) cudaFree(ptr);
    ptr = nullptr;
    bytes = 0;
}

static kgpu_status upload(kgpu_context* ctx, DeviceBuffer& buf, const void* src, size_t bytes) {
    if (bytes == 0) return KGPU_OK;
    if (buf.ensure(bytes) != KGPU_OK)
        return fail(ctx, KGPU_DEVICE_ERROR, "cudaMalloc of %zu bytes failed", bytes);
    CUDA_TRY(ctx, cudaMemcpyAsync(buf.ptr, src, bytes, cudaMemcpyHostToDevice, ctx->stream));
    ctx->h2d_bytes += bytes;
    return KGPU_OK;
}

extern "C" {

int32_t kgpu_abi_version(void) { return KGPU_ABI_VERSION; }

int32_t kgpu_device_count(void) {
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess) return 0;
    return n;
}

kgpu_status kgpu_context_create(int device, kgpu_context** out) {
    if (!out) return fail(nullptr, KGPU_INVALID_INPUT, "null output pointer");
    *out = nullptr;
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0)
        return fail(nullptr, KGPU_DEVICE_ERROR, "no CUDA device is available");
    if (device < 0 || device >= count)
        return fail(nullptr, KGPU_INVALID_INPUT, "device %d is out of range (%d devices)", device, count);
    if (cudaSetDevice(device) != cudaSuccess)
        return fail(nullptr, KGPU_DEVICE_ERROR, "cudaSetDevice(%d) failed", device);
    cudaDeviceProp prop;
    if (cudaGetDeviceProperties(&prop, device) != cudaSuccess)
        return fail(nullptr, KGPU_DEVICE_ERROR, "cudaGetDeviceProperties failed");
    if (prop.major < 10)
        return fail(nullptr, KGPU_DEVICE_ERROR, "device %d (sm_%d%d) is not a Blackwell GPU", device,
                    prop.major, prop.minor);
    kgpu_context* ctx = new kgpu_context();
    ctx->device = device;
    ctx->sm_count = prop.multiProcessorCount;
    if (cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreate(&ctx->ev_start) != cudaSuccess || cudaEventCreate(&ctx->ev_stop) != cudaSuccess ||
        cudaHostAlloc((void**)&ctx->cancel_host, sizeof(int), cudaHostAllocMapped) != cudaSuccess ||
        cudaHostGetDevicePointer((void**)&ctx->cancel_dev, (void*)ctx->cancel_host, 0) != cudaSuccess) {
        delete ctx;
        return fail(nullptr, KGPU_DEVICE_ERROR, "stream/event/pinned allocation failed");
    }
    *ctx->cancel_host = 0;
    *out = ctx;
    return KGPU_OK;
}

void kgpu_context_destroy(kgpu_context* ctx) {
    if (!ctx) return;
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->stream);
    for (DeviceBuffer* b : ctx->buffers()) b->release();
    if (ctx->cancel_host) cudaFreeHost((void*)ctx->cancel_host);
    cudaEventDestroy(ctx->ev_start);
    cudaEventDestroy(ctx->ev_stop);
    cudaStreamDestroy(ctx->stream);
    delete ctx;
}

const char* kgpu_last_error_message(const kgpu_context* ctx) {
    return ctx ? ctx->error.c_str() : g_thread_error.c_str();
}

double kgpu_context_last_kernel_ms(const kgpu_context* ctx) { return ctx ? ctx->last_kernel_ms : 0.0; }
int32_t kgpu_context_last_launches(const kgpu_context* ctx) { return ctx ? ctx->last_launches : 0; }

}  // extern "C"

// ------------------------------------------------------------------------------------
// Pricing
// ------------------------------------------------------------------------------------
namespace {

struct ContractInfo {
    int dims;
    int64_t paths;
    int64_t samples;
};

int model_normals_per_step(const kgpu_model* m) { return m->kind == KGPU_MODEL_HESTON ? 2 : 1; }

int dims_of(const kgpu_contract& c, const kgpu_model* m) {
    if (c.payoff == KGPU_PAYOFF_EUROPEAN || c.payoff == KGPU_PAYOFF_DIGITAL) return 1;
    return c.step_count * model_normals_per_step(m);
}

// MonteCarloEstimate::from_sampling and sampling_standard_error (monte_carlo.rs:939-963,
// 1435-1452), from merged scaled moments.
void estimate_from_moments(const kgpu_contract& c, const kgpu_settings& s, int64_t paths,
                           const BlockPartial& p, kgpu_estimate* out) {
    const bool sobol = s.sampling == KGPU_SAMPLING_SOBOL;
    const bool antithetic = s.antithetic != 0;
    const bool statistics = !sobol && (!antithetic || paths % 2 == 0);
    const double log_discount = c.payoff == KGPU_PAYOFF_EUROPEAN ? c.log_scale : 0.0;
    auto scaled = [](double scale, double weight, double log_d) {
        double value = scale * weight;
        double discount = std::exp(log_d);
        if (scale == 0.0 || weight == 0.0) return 0.0;
        if (std::isnormal(discount) && std::isnormal(value)) return value * discount;
        return std::copysign(std::exp(std::log(scale) + std::log(std::fabs(weight)) + log_d), weight);
    };
    out->price = scaled(p.moments.scale, p.moments.mean, log_discount);
    const Moments& u = antithetic ? p.pairs : p.moments;
    out->standard_error = 0.0;
    if (statistics && u.count >= 2.0) {
        double deviation = std::sqrt(std::max(u.m2, 0.0) / (u.count - 1.0) / u.count);
        double se = scaled(u.scale, deviation, log_discount);
        if (se == 0.0) {
            out->uncertainty_status = KGPU_UNCERTAINTY_ZERO_OBSERVED_VARIANCE;
        } else {
            out->standard_error = se;
            out->uncertainty_status = KGPU_UNCERTAINTY_AVAILABLE;
        }
    } else if (sobol) {
        out->uncertainty_status = KGPU_UNCERTAINTY_UNSUPPORTED_SAMPLING;
    } else if (antithetic && paths % 2 != 0) {
        out->uncertainty_status = KGPU_UNCERTAINTY_INCOMPLETE_ANTITHETIC_PAIR;
    } else {
        out->uncertainty_status = KGPU_UNCERTAINTY_INSUFFICIENT_OBSERVATIONS;
    }
    const Moments& v = p.sample;
    out->sample_error = v.count >= 2.0
                            ? scaled(v.scale, std::sqrt(std::max(v.m2, 0.0) / (v.count - 1.0) / v.count),
                                     log_discount)
                            : 0.0;
    out->seed = s.seed;
}

void estimate_from_sums(const kgpu_contract& c, const kgpu_settings& s, int64_t paths,
                        const TilePartial& t, kgpu_estimate* out) {
    const bool sobol = s.sampling == KGPU_SAMPLING_SOBOL;
    const double scale = c.payoff == KGPU_PAYOFF_EUROPEAN ? std::exp(c.log_scale) : 1.0;
    const double n = t.count;
    const double mean = n > 0 ? t.sum / n : 0.0;
    out->price = mean * scale;
    double se = 0.0;
    if (n >= 2) {
        double var = std::max(0.0, (t.sumsq - t.sum * mean) / (n - 1.0));
        se = std::sqrt(var / n) * scale;
    }
    out->sample_error = se;
    out->standard_error = 0.0;
    if (sobol) {
        out->uncertainty_status = KGPU_UNCERTAINTY_UNSUPPORTED_SAMPLING;
    } else if (n < 2) {
        out->uncertainty_status = KGPU_UNCERTAINTY_INSUFFICIENT_OBSERVATIONS;
    } else if (se == 0.0) {
        out->uncertainty_status = KGPU_UNCERTAINTY_ZERO_OBSERVED_VARIANCE;
    } else {
        out->standard_error = se;
        out->uncertainty_status = KGPU_UNCERTAINTY_AVAILABLE;
    }
    out->seed = s.seed;
    (void)paths;
}

bool is_pow2(int64_t x) { return x > 0 && (x & (x - 1)) == 0; }

}  // namespace

static kgpu_status ensure_sobol(kgpu_context* ctx, int dims, uint64_t seed, SobolTables* t) {
    if (dims < 1 || dims > 21201)
        return fail(ctx, KGPU_INVALID_INPUT, "Sobol dimension must be in 1..=21,201");
    if (!(ctx->sobol_dims == dims && ctx->sobol_seed == seed)) {
        std::vector<uint64_t> dirs, shifts;
        build_sobol(dims, seed, dirs, shifts);
        kgpu_status st = upload(ctx, ctx->sobol_dirs, dirs.data(), dirs.size() * 8);
        if (st != KGPU_OK) return st;
        st = upload(ctx, ctx->sobol_shifts, shifts.data(), shifts.size() * 8);
        if (st != KGPU_OK) return st;
        ctx->sobol_dims = dims;
        ctx->sobol_seed = seed;
    }
    t->directions = static_cast<const uint64_t*>(ctx->sobol_dirs.ptr);
    t->shifts = static_cast<const uint64_t*>(ctx->sobol_shifts.ptr);
    t->dims = dims;
    return KGPU_OK;
}

// Mirrors the caller's cancellation word into host-mapped memory the persistent kernel
// reads, while a launch is in flight.
struct CancelWatcher {
    std::atomic<bool> done{false};
    std::thread th;
    CancelWatcher(const volatile int32_t* src, volatile int* dst) {
        if (!src) return;
        th = std::thread([this, src, dst]() {
            while (!done.load()) {
                if (*src) *dst = 1;
                std::this_thread::sleep_for(std::chrono::microseconds(500));
            }
        });
    }
    ~CancelWatcher() {
        done = true;
        if (th.joinable()) th.join();
    }
};

static kgpu_status price_book_impl(kgpu_context* ctx, const kgpu_model* model, const kgpu_book* book,
                                   const kgpu_settings* settings, kgpu_estimate* out,
                                   const volatile int32_t* cancel, bool device_resident) {
    if (!ctx) return fail(nullptr, KGPU_INVALID_INPUT, "null context");
    std::lock_guard<std::mutex> lock(ctx->mu);
    ctx->error.clear();
    ctx->h2d_bytes = 0;
    ctx->last_launches = 0;
    if (!model || !book || !settings || !out) return fail(ctx, KGPU_INVALID_INPUT, "null argument");
    if (cudaSetDevice(ctx->device) != cudaSuccess)
        return fail(ctx, KGPU_DEVICE_ERROR, "cudaSetDevice(%d) failed", ctx->device);
    const int n = book->contract_count;
    if (n < 0) return fail(ctx, KGPU_INVALID_INPUT, "negative contract count");
    if (n == 0) return KGPU_OK;
    const kgpu_settings s = *settings;
    if (s.precision != KGPU_PRECISION_FP64 && s.precision != KGPU_PRECISION_FP32)
        return fail(ctx, KGPU_INVALID_INPUT, "unknown precision %d", s.precision);
    if (s.sampling != KGPU_SAMPLING_PSEUDO_RANDOM && s.sampling != KGPU_SAMPLING_SOBOL)
        return fail(ctx, KGPU_INVALID_INPUT, "unknown sampling %d", s.sampling);
    if (model->kind < KGPU_MODEL_BSM || model->kind > KGPU_MODEL_LOCAL_VOL)
        return fail(ctx, KGPU_INVALID_INPUT, "unknown model %d", model->kind);
    const bool sobol = s.sampling == KGPU_SAMPLING_SOBOL;
    const bool persistent = s.schedule == KGPU_SCHEDULE_PERSISTENT;
    if (persistent && s.antithetic)
        return fail(ctx, KGPU_UNSUPPORTED_OPERATION,
                    "the persistent schedule does not pair antithetic samples; use the plain schedule");
    // Validate contracts (MonteCarloSettings::validate, monte_carlo.rs:197-220).
    std::vector<ContractInfo> info(n);
    for (int i = 0; i < n; ++i) {
        const kgpu_contract& c = book->contracts[i];
        int64_t paths = c.path_count > 0 ? c.path_count : s.path_count;
        if (paths < 1 || paths > 2147483647LL)
            return fail(ctx, KGPU_INVALID_INPUT, "contract %d: path_count must be positive", i);
        if (sobol && !is_pow2(paths))
            return fail(ctx, KGPU_INVALID_INPUT, "path_count must be a power of two for Sobol sampling");
        if (c.payoff < KGPU_PAYOFF_EUROPEAN || c.payoff > KGPU_PAYOFF_DIGITAL)
            return fail(ctx, KGPU_INVALID_INPUT, "contract %d: unknown payoff %d", i, c.payoff);
        if (c.step_count < 1 || c.step_offset < 0 || c.step_offset + c.step_count > book->step_total)
            return fail(ctx, KGPU_INVALID_INPUT, "contract %d: steps out of range", i);
        if (c.event_count < 0 || c.event_offset < 0 || c.event_offset + c.event_count > book->event_total)
            return fail(ctx, KGPU_INVALID_INPUT, "contract %d: events out of range", i);
        if (c.flags & KGPU_C_BRIDGE) {
            if (model->kind != KGPU_MODEL_BSM || !book->bridge_daily || c.bridge_count < 1 ||
                c.bridge_offset < 0 || c.bridge_offset + c.bridge_count > book->interval_total)
                return fail(ctx, KGPU_INVALID_INPUT, "contract %d: invalid bridge plan", i);
        }
        if (c.payoff == KGPU_PAYOFF_AUTOCALLABLE || c.payoff == KGPU_PAYOFF_ACCUMULATOR) {
            // Every event flag must be backed by an event record.
            if (!device_resident) {
                int events = 0;
                for (int k = 0; k < c.step_count; ++k)
                    events += (book->step_flags[c.step_offset + k] & KGPU_STEP_EVENT) != 0;
                if (c.payoff == KGPU_PAYOFF_AUTOCALLABLE && events != c.event_count)
                    return fail(ctx, KGPU_INVALID_INPUT, "contract %d: %d event steps but %d events",
                                i, events, c.event_count);
            }
        }
        info[i].dims = dims_of(c, model);
        info[i].paths = paths;
        info[i].samples = s.antithetic ? (paths + 1) / 2 : paths;
    }
    kgpu_status st;
    // Stage the book.
    DevBook db;
    if (!device_resident) {
        if ((st = upload(ctx, ctx->steps, book->steps, size_t(book->step_total) * sizeof(kgpu_step))) ||
            (st = upload(ctx, ctx->flags, book->step_flags, size_t(book->step_total))) ||
            (st = upload(ctx, ctx->events, book->events, size_t(book->event_total) * sizeof(kgpu_event))) ||
            (st = upload(ctx, ctx->intervals, book->intervals,
                         size_t(book->interval_total) * sizeof(kgpu_bridge_interval))))
            return st;
        if (book->bridge_daily &&
            (st = upload(ctx, ctx->daily, book->bridge_daily, size_t(book->step_total) * sizeof(kgpu_bridge_daily))))
            return st;
        db.steps = static_cast<const kgpu_step*>(ctx->steps.ptr);
        db.flags = static_cast<const uint8_t*>(ctx->flags.ptr);
        db.events = book->event_total ? static_cast<const kgpu_event*>(ctx->events.ptr) : nullptr;
        db.intervals = book->interval_total ? static_cast<const kgpu_bridge_interval*>(ctx->intervals.ptr) : nullptr;
        db.daily = book->bridge_daily ? static_cast<const kgpu_bridge_daily*>(ctx->daily.ptr) : nullptr;
    } else {
        db.steps = book->steps;
        db.flags = book->step_flags;
        db.events = book->events;
        db.intervals = book->intervals;
        db.daily = book->bridge_daily;
    }
    if ((st = upload(ctx, ctx->contracts, book->contracts, size_t(n) * sizeof(kgpu_contract)))) return st;
    db.contracts = static_cast<const kgpu_contract*>(ctx->contracts.ptr);
    // Local volatility surface: [years since the first node][spots][values].
    int lv_values = 0;
    const double* lv_dev = nullptr;
    if (model->kind == KGPU_MODEL_LOCAL_VOL) {
        const int nt = model->lv_time_count, ns = model->lv_spot_count;
        if (nt < 2 || ns < 2 || !model->lv_times || !model->lv_spots || !model->lv_values)
            return fail(ctx, KGPU_INVALID_INPUT, "invalid local volatility surface");
        std::vector<double> lv(size_t(nt) + ns + size_t(nt) * ns);
        for (int i = 0; i < nt; ++i) lv[i] = model->lv_times[i] - model->lv_times[0];
        for (int i = 0; i < ns; ++i) lv[nt + i] = model->lv_spots[i];
        std::memcpy(&lv[nt + ns], model->lv_values, sizeof(double) * size_t(nt) * ns);
        lv_values = int(lv.size());
        if ((st = upload(ctx, ctx->lv, lv.data(), lv.size() * sizeof(double)))) return st;
        CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));  // `lv` is a stack vector
        lv_dev = static_cast<const double*>(ctx->lv.ptr);
    }
    *ctx->cancel_host = 0;
    int launches = 0;
    bool started = false;
    auto start_clock = [&]() -> kgpu_status {
        if (!started) {
            CUDA_TRY(ctx, cudaEventRecord(ctx->ev_start, ctx->stream));
            started = true;
        }
        return KGPU_OK;
    };
    if (!persistent) {
        // Plain schedule: one contract per launch.
        int64_t max_blocks = 0;
        for (int i = 0; i < n; ++i) max_blocks = std::max<int64_t>(max_blocks, (info[i].samples + 255) / 256);
        if ((st = ctx->partials.ensure(size_t(max_blocks) * sizeof(BlockPartial)) ? KGPU_DEVICE_ERROR : KGPU_OK) ||
            (st = ctx->merged.ensure(size_t(n) * sizeof(BlockPartial)) ? KGPU_DEVICE_ERROR : KGPU_OK))
            return fail(ctx, st, "cudaMalloc of partials failed");
        for (int i = 0; i < n; ++i) {
            if (cancel && *cancel) return fail(ctx, KGPU_INTERRUPTED, "cancelled");
            const ContractInfo& ci = info[i];
            PlainArgs a;
            a.book = db;
            a.contract = i;
            a.dims = ci.dims;
            a.paths = ci.paths;
            a.samples = ci.samples;
            a.seed = s.seed;
            a.antithetic = s.antithetic;
            a.statistics = !sobol && (!s.antithetic || ci.paths % 2 == 0);
            a.variance = a.statistics && !s.antithetic;
            a.sobol = SobolTables{nullptr, nullptr, 0};
            if (sobol && (st = ensure_sobol(ctx, ci.dims, s.seed, &a.sobol))) return st;
            a.partials = static_cast<BlockPartial*>(ctx->partials.ptr);
            const int blocks = int((ci.samples + 255) / 256);
            size_t smem = plain_smem_bytes(s.precision, sobol, ci.dims, lv_values);
            if (smem > 227 * 1024)
                return fail(ctx, KGPU_INVALID_INPUT, "dimension %d exceeds the plain kernel's shared memory",
                            ci.dims);
            if ((st = start_clock())) return st;
            CUDA_TRY(ctx, launch_plain(s.precision, model->kind, sobol, blocks, smem, ctx->stream, a, *model, lv_dev));
            const bool variance = a.variance;
            merge_blocks_kernel<<<1, 32, 0, ctx->stream>>>(a.partials, blocks, variance, a.statistics,
                                                            s.antithetic, static_cast<BlockPartial*>(ctx->merged.ptr) + i);
            CUDA_TRY(ctx, cudaGetLastError());
            launches += 2;
            if (cancel) CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
        }
        CUDA_TRY(ctx, cudaEventRecord(ctx->ev_stop, ctx->stream));
        std::vector<BlockPartial> merged(n);
        CUDA_TRY(ctx, cudaMemcpyAsync(merged.data(), ctx->merged.ptr, sizeof(BlockPartial) * n,
                                      cudaMemcpyDeviceToHost, ctx->stream));
        CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
        float ms = 0;
        cudaEventElapsedTime(&ms, ctx->ev_start, ctx->ev_stop);
        ctx->last_kernel_ms = ms;
        ctx->last_launches = launches;
        for (int i = 0; i < n; ++i) {
            const kgpu_contract& c = book->contracts[i];
            estimate_from_moments(c, s, info[i].paths, merged[i], &out[i]);
            int grid = (c.payoff == KGPU_PAYOFF_EUROPEAN || c.payoff == KGPU_PAYOFF_DIGITAL) ? 1 : c.step_count;
            out[i].path_steps = double(info[i].paths) * grid;
            out[i].executed_steps = merged[i].executed;
            if (!std::isfinite(out[i].price) || !std::isfinite(out[i].standard_error))
                return fail(ctx, KGPU_COMPUTATION_FAILURE,
                            "Monte Carlo produced a non-finite parameter, path or result (contract %d)", i);
        }
        return KGPU_OK;
    }
    // Persistent schedule: group contracts by sampling dimension for Sobol (one sequence
    // per launch); pseudo-random books run in a single launch.
    std::vector<int> group_of(n, 0);
    std::vector<int> group_dims;
    if (sobol) {
        for (int i = 0; i < n; ++i) {
            auto it = std::find(group_dims.begin(), group_dims.end(), info[i].dims);
            if (it == group_dims.end()) {
                group_of[i] = int(group_dims.size());
                group_dims.push_back(info[i].dims);
            } else {
                group_of[i] = int(it - group_dims.begin());
            }
        }
    } else {
        group_dims.push_back(0);
    }
    // Items grouped by contract (contract order), tile size per contract.
    std::vector<int4> items;
    std::vector<int> first_item(n + 1, 0);
    for (int i = 0; i < n; ++i) {
        first_item[i] = int(items.size());
        int64_t tile = sobol ? 256 : (s.tile_paths > 0 ? s.tile_paths : 1024);
        for (int64_t b = 0; b < info[i].samples; b += tile)
            items.push_back(make_int4(i, int(b), int(std::min<int64_t>(tile, info[i].samples - b)), info[i].dims));
    }
    first_item[n] = int(items.size());
    const int item_count = int(items.size());
    if ((st = upload(ctx, ctx->items, items.data(), items.size() * sizeof(int4))) ||
        (st = upload(ctx, ctx->first_item, first_item.data(), first_item.size() * sizeof(int))))
        return st;
    if (ctx->tiles.ensure(size_t(item_count) * sizeof(TilePartial)) ||
        ctx->tile_out.ensure(size_t(n) * sizeof(TilePartial)) || ctx->queue.ensure(sizeof(int) * 4))
        return fail(ctx, KGPU_DEVICE_ERROR, "cudaMalloc of tile partials failed");
    CancelWatcher watcher(cancel, ctx->cancel_host);
    std::vector<int> order;
    for (size_t g = 0; g < group_dims.size(); ++g) {
        // Dispatch order: most expensive contracts first.
        order.clear();
        std::vector<int> members;
        for (int i = 0; i < n; ++i)
            if (group_of[i] == int(g)) members.push_back(i);
        std::stable_sort(members.begin(), members.end(), [&](int x, int y) {
            return double(info[x].samples) * book->contracts[x].step_count >
                   double(info[y].samples) * book->contracts[y].step_count;
        });
        int max_dims = 0;
        for (int i : members) {
            for (int k = first_item[i]; k < first_item[i + 1]; ++k) order.push_back(k);
            max_dims = std::max(max_dims, info[i].dims);
        }
        if (order.empty()) continue;
        if (cancel && *cancel) return fail(ctx, KGPU_INTERRUPTED, "cancelled");
        if ((st = upload(ctx, ctx->order, order.data(), order.size() * sizeof(int)))) return st;
        PersistentArgs a;
        a.book = db;
        a.items = static_cast<const int4*>(ctx->items.ptr);
        a.order = static_cast<const int*>(ctx->order.ptr);
        a.item_count = int(order.size());
        a.queue = static_cast<int*>(ctx->queue.ptr);
        a.seed = s.seed;
        a.sobol = SobolTables{nullptr, nullptr, 0};
        if (sobol && (st = ensure_sobol(ctx, group_dims[g], s.seed, &a.sobol))) return st;
        a.partials = static_cast<TilePartial*>(ctx->tiles.ptr);
        a.cancel = cancel ? ctx->cancel_dev : nullptr;
        a.aborted = static_cast<int*>(ctx->queue.ptr) + 1;
        size_t smem = persistent_smem_bytes(s.precision, sobol, sobol ? group_dims[g] : 0, lv_values);
        if (smem > 227 * 1024)
            return fail(ctx, KGPU_UNSUPPORTED_OPERATION,
                        "Sobol dimension %d exceeds the persistent kernel's shared memory; use the plain schedule",
                        group_dims[g]);
        const int per_sm = persistent_blocks_per_sm(s.precision, model->kind, sobol, smem);
        const int blocks = std::max(1, std::min(ctx->sm_count * per_sm, (a.item_count + kWarps - 1) / kWarps));
        CUDA_TRY(ctx, cudaMemsetAsync(ctx->queue.ptr, 0, sizeof(int) * 2, ctx->stream));
        if ((st = start_clock())) return st;
        CUDA_TRY(ctx, launch_persistent(s.precision, model->kind, sobol, blocks, smem, ctx->stream, a,
                                        *model, lv_dev));
        launches += 1;
        if (group_dims.size() > 1) CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    }
    reduce_tiles_kernel<<<(n + 127) / 128, 128, 0, ctx->stream>>>(
        static_cast<const TilePartial*>(ctx->tiles.ptr), static_cast<const int*>(ctx->first_item.ptr), n,
        static_cast<TilePartial*>(ctx->tile_out.ptr));
    CUDA_TRY(ctx, cudaGetLastError());
    launches += 1;
    CUDA_TRY(ctx, cudaEventRecord(ctx->ev_stop, ctx->stream));
    std::vector<TilePartial> sums(n);
    int aborted = 0;
    CUDA_TRY(ctx, cudaMemcpyAsync(sums.data(), ctx->tile_out.ptr, sizeof(TilePartial) * n,
                                  cudaMemcpyDeviceToHost, ctx->stream));
    CUDA_TRY(ctx, cudaMemcpyAsync(&aborted, static_cast<int*>(ctx->queue.ptr) + 1, sizeof(int),
                                  cudaMemcpyDeviceToHost, ctx->stream));
    CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    float ms = 0;
    cudaEventElapsedTime(&ms, ctx->ev_start, ctx->ev_stop);
    ctx->last_kernel_ms = ms;
    ctx->last_launches = launches;
    if (aborted) return fail(ctx, KGPU_INTERRUPTED, "cancelled");
    for (int i = 0; i < n; ++i) {
        const kgpu_contract& c = book->contracts[i];
        estimate_from_sums(c, s, info[i].paths, sums[i], &out[i]);
        int grid = (c.payoff == KGPU_PAYOFF_EUROPEAN || c.payoff == KGPU_PAYOFF_DIGITAL) ? 1 : c.step_count;
        out[i].path_steps = double(info[i].paths) * grid;
        out[i].executed_steps = sums[i].executed;
        if (!std::isfinite(out[i].price) || !std::isfinite(out[i].standard_error))
            return fail(ctx, KGPU_COMPUTATION_FAILURE,
                        "Monte Carlo produced a non-finite parameter, path or result (contract %d)", i);
    }
    return KGPU_OK;
}

namespace kgpu {

size_t plain_smem_bytes(int precision, bool sobol, int dims, int lv_values) {
    size_t real = precision == KGPU_PRECISION_FP64 ? 8 : 4;
    return 2 * kThreads * 8 + kThreads * 4 + (sobol ? size_t(dims) * 8 : 0) + size_t(lv_values) * real + 16;
}

size_t persistent_smem_bytes(int precision, bool sobol, int dims, int lv_values) {
    size_t real = precision == KGPU_PRECISION_FP64 ? 8 : 4;
    return (sobol ? size_t(dims) * 8 * (8 + kWarps) : 0) + size_t(lv_values) * real + 16;
}

cudaError_t launch_plain_fp64(int, bool, int, size_t, cudaStream_t, const PlainArgs&, const kgpu_model&, const double*);
cudaError_t launch_plain_fp32(int, bool, int, size_t, cudaStream_t, const PlainArgs&, const kgpu_model&, const double*);
cudaError_t launch_persistent_fp64(int, bool, int, size_t, cudaStream_t, const PersistentArgs&, const kgpu_model&, const double*);
cudaError_t launch_persistent_fp32(int, bool, int, size_t, cudaStream_t, const PersistentArgs&, const kgpu_model&, const double*);
int persistent_occupancy_fp64(int, bool, size_t);
int persistent_occupancy_fp32(int, bool, size_t);
cudaError_t launch_pcg_normals_fp64(uint64_t, uint64_t, uint64_t, int64_t, double*, cudaStream_t);
cudaError_t launch_pcg_normals_fp32(uint64_t, uint64_t, uint64_t, int64_t, double*, cudaStream_t);
cudaError_t launch_sobol_points_fp64(const SobolTables&, int, uint64_t, int64_t, uint64_t*, double*, cudaStream_t);
cudaError_t launch_sobol_points_fp32(const SobolTables&, int, uint64_t, int64_t, uint64_t*, double*, cudaStream_t);

cudaError_t launch_plain(int precision, int model, bool sobol, int blocks, size_t smem, cudaStream_t stream,
                         const PlainArgs& a, const kgpu_model& m, const double* lv) {
    return precision == KGPU_PRECISION_FP64 ? launch_plain_fp64(model, sobol, blocks, smem, stream, a, m, lv)
                                            : launch_plain_fp32(model, sobol, blocks, smem, stream, a, m, lv);
}

cudaError_t launch_persistent(int precision, int model, bool sobol, int blocks, size_t smem,
                              cudaStream_t stream, const PersistentArgs& a, const kgpu_model& m,
                              const double* lv) {
    return precision == KGPU_PRECISION_FP64
               ? launch_persistent_fp64(model, sobol, blocks, smem, stream, a, m, lv)
               : launch_persistent_fp32(model, sobol, blocks, smem, stream, a, m, lv);
}

int persistent_blocks_per_sm(int precision, int model, bool sobol, size_t smem) {
    return precision == KGPU_PRECISION_FP64 ? persistent_occupancy_fp64(model, sobol, smem)
                                            : persistent_occupancy_fp32(model, sobol, smem);
}

__global__ void pcg_words_kernel(uint64_t seed, uint64_t stream_id, uint64_t first, int64_t count,
                                 uint32_t* out) {
    int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= count) return;
    Pcg g = pcg_new(seed, stream_id);
    pcg_advance(g, first + uint64_t(i));
    out[i] = pcg_next(g);
}

}  // namespace kgpu

extern "C" {

kgpu_status kgpu_price_book(kgpu_context* ctx, const kgpu_model* model, const kgpu_book* book,
                            const kgpu_settings* settings, kgpu_estimate* out,
                            const volatile int32_t* cancel_flag) {
    return price_book_impl(ctx, model, book, settings, out, cancel_flag, false);
}

kgpu_status kgpu_price_book_device(kgpu_context* ctx, const kgpu_model* model, const kgpu_book* device_book,
                                   const kgpu_settings* settings, kgpu_estimate* out) {
    return price_book_impl(ctx, model, device_book, settings, out, nullptr, true);
}

kgpu_status kgpu_pcg_words(kgpu_context* ctx, uint64_t seed, uint64_t stream, uint64_t first, int64_t count,
                           uint32_t* out) {
    if (!ctx || !out || count < 0) return fail(ctx, KGPU_INVALID_INPUT, "invalid arguments");
    std::lock_guard<std::mutex> lock(ctx->mu);
    if (count == 0) return KGPU_OK;
    if (ctx->stream_out.ensure(size_t(count) * 4)) return fail(ctx, KGPU_DEVICE_ERROR, "cudaMalloc failed");
    pcg_words_kernel<<<unsigned((count + 255) / 256), 256, 0, ctx->stream>>>(
        seed, stream, first, count, static_cast<uint32_t*>(ctx->stream_out.ptr));
    CUDA_TRY(ctx, cudaGetLastError());
    CUDA_TRY(ctx, cudaMemcpyAsync(out, ctx->stream_out.ptr, size_t(count) * 4, cudaMemcpyDeviceToHost, ctx->stream));
    CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    return KGPU_OK;
}

kgpu_status kgpu_pcg_normals(kgpu_context* ctx, uint64_t seed, uint64_t block, uint64_t first, int64_t count,
                             int32_t precision, double* out) {
    if (!ctx || !out || count < 0) return fail(ctx, KGPU_INVALID_INPUT, "invalid arguments");
    std::lock_guard<std::mutex> lock(ctx->mu);
    if (count == 0) return KGPU_OK;
    if (ctx->stream_out.ensure(size_t(count) * 8)) return fail(ctx, KGPU_DEVICE_ERROR, "cudaMalloc failed");
    double* d = static_cast<double*>(ctx->stream_out.ptr);
    CUDA_TRY(ctx, precision == KGPU_PRECISION_FP64 ? launch_pcg_normals_fp64(seed, block, first, count, d, ctx->stream)
                                                   : launch_pcg_normals_fp32(seed, block, first, count, d, ctx->stream));
    CUDA_TRY(ctx, cudaMemcpyAsync(out, d, size_t(count) * 8, cudaMemcpyDeviceToHost, ctx->stream));
    CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    return KGPU_OK;
}

kgpu_status kgpu_sobol_points(kgpu_context* ctx, uint64_t seed, int32_t dimensions, int32_t dimension,
                              uint64_t first, int64_t count, uint64_t* bits_out, double* normals_out,
                              int32_t precision) {
    if (!ctx || count < 0 || dimension < 0 || dimension >= dimensions)
        return fail(ctx, KGPU_INVALID_INPUT, "invalid arguments");
    std::lock_guard<std::mutex> lock(ctx->mu);
    if (count == 0) return KGPU_OK;
    SobolTables t;
    kgpu_status st = ensure_sobol(ctx, dimensions, seed, &t);
    if (st) return st;
    if (ctx->stream_out.ensure(size_t(count) * 16)) return fail(ctx, KGPU_DEVICE_ERROR, "cudaMalloc failed");
    uint64_t* bits = static_cast<uint64_t*>(ctx->stream_out.ptr);
    double* normals = reinterpret_cast<double*>(bits + count);
    CUDA_TRY(ctx, precision == KGPU_PRECISION_FP64
                      ? launch_sobol_points_fp64(t, dimension, first, count, bits, normals, ctx->stream)
                      : launch_sobol_points_fp32(t, dimension, first, count, bits, normals, ctx->stream));
    if (bits_out) CUDA_TRY(ctx, cudaMemcpyAsync(bits_out, bits, size_t(count) * 8, cudaMemcpyDeviceToHost, ctx->stream));
    if (normals_out)
        CUDA_TRY(ctx, cudaMemcpyAsync(normals_out, normals, size_t(count) * 8, cudaMemcpyDeviceToHost, ctx->stream));
    CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    return KGPU_OK;
}

}  // extern "C"
