// C ABI of libkiyosi_gpu.so (include/kgpu.h): contexts, device buffers, the two launch
// schedules and the estimates returned to the caller.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <thread>
#include <tuple>
#include <type_traits>
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
    // The arithmetic average's samples are residuals against the geometric control;
    // its exact mean is added back (ArithmeticGrid::sample, asian.rs:616-621).
    if (c.payoff == KGPU_PAYOFF_AVERAGE_ARITHMETIC && (c.flags & KGPU_C_AVERAGE_CONTROL))
        out->price += c.control_mean;
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

}  // namespace kgpu

using namespace kgpu;

static thread_local std::string g_thread_error;

namespace kgpu {
void set_thread_error(const char* message) { g_thread_error = message; }
}  // namespace kgpu

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

static std::atomic<uint64_t> g_alloc_generation{0};

uint64_t kgpu::alloc_generation() { return g_alloc_generation.load(); }

kgpu_status DeviceBuffer::ensure(size_t n) {
    if (n <= bytes) return KGPU_OK;
    g_alloc_generation.fetch_add(1);
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
    if (ptr) g_alloc_generation.fetch_add(1);
    if (ptr) cudaFree(ptr);
    ptr = nullptr;
    bytes = 0;
}

static kgpu_status upload(kgpu_context* ctx, DeviceBuffer& buf, const void* src, size_t bytes) {
    if (bytes == 0) return KGPU_OK;
    // A capture pass follows a direct call with the same key, which staged exactly these
    // bytes in the same buffer: nothing to copy (and a pageable copy cannot be captured).
    if (ctx->capturing) return buf.bytes >= bytes ? KGPU_OK : KGPU_DEVICE_ERROR;
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
    for (auto& e : ctx->path_events) {
        cudaEventDestroy(e.first);
        cudaEventDestroy(e.second);
    }
    if (ctx->lsmc_exec) cudaGraphExecDestroy(ctx->lsmc_exec);
    if (ctx->book_exec) cudaGraphExecDestroy(ctx->book_exec);
    for (cudaEvent_t e : ctx->lsmc_events)
        if (e) cudaEventDestroy(e);
    cudaStreamDestroy(ctx->stream);
    delete ctx;
}

const char* kgpu_last_error_message(const kgpu_context* ctx) {
    return ctx ? ctx->error.c_str() : g_thread_error.c_str();
}

double kgpu_context_last_kernel_ms(const kgpu_context* ctx) { return ctx ? ctx->last_kernel_ms : 0.0; }
double kgpu_context_last_path_kernel_ms(const kgpu_context* ctx) { return ctx ? ctx->last_path_kernel_ms : 0.0; }
int32_t kgpu_context_last_launches(const kgpu_context* ctx) { return ctx ? ctx->last_launches : 0; }
int32_t kgpu_context_last_graph(const kgpu_context* ctx) { return ctx ? ctx->last_graph : 0; }

}  // extern "C"

// ------------------------------------------------------------------------------------
// Pricing
// ------------------------------------------------------------------------------------
namespace {

// Records the start of one path-kernel launch; path_kernel_end records its end.
cudaError_t path_kernel_begin(kgpu_context* ctx) {
    if (ctx->path_events_used == ctx->path_events.size()) {
        std::pair<cudaEvent_t, cudaEvent_t> e{nullptr, nullptr};
        cudaError_t rc = cudaEventCreate(&e.first);
        if (rc == cudaSuccess) rc = cudaEventCreate(&e.second);
        if (rc != cudaSuccess) {
            if (e.first) cudaEventDestroy(e.first);
            return rc;
        }
        ctx->path_events.push_back(e);
    }
    // Inside a capture the record must be an external node of the graph, so that every
    // replay records the event; outside one the flag is refused.
    return cudaEventRecordWithFlags(ctx->path_events[ctx->path_events_used].first, ctx->stream,
                                    ctx->capturing ? cudaEventRecordExternal : cudaEventRecordDefault);
}

cudaError_t path_kernel_end(kgpu_context* ctx) {
    return cudaEventRecordWithFlags(ctx->path_events[ctx->path_events_used++].second, ctx->stream,
                                    ctx->capturing ? cudaEventRecordExternal : cudaEventRecordDefault);
}

// Sum of the recorded path-kernel times; call after the stream has been synchronised.
double path_kernel_ms(kgpu_context* ctx) {
    double total = 0.0;
    for (size_t i = 0; i < ctx->path_events_used; ++i) {
        float ms = 0.0f;
        if (cudaEventElapsedTime(&ms, ctx->path_events[i].first, ctx->path_events[i].second) == cudaSuccess)
            total += ms;
    }
    return total;
}

struct ContractInfo {
    int dims;
    int64_t paths;
    int64_t samples;
};

int model_normals_per_step(const kgpu_model* m) { return m->kind == KGPU_MODEL_HESTON ? 2 : 1; }

// Payoffs sampled with one terminal draw per path (no grid).
bool terminal_payoff(const kgpu_contract& c) {
    return c.payoff == KGPU_PAYOFF_EUROPEAN || c.payoff == KGPU_PAYOFF_DIGITAL || c.payoff == KGPU_PAYOFF_BARRIER ||
           c.payoff == KGPU_PAYOFF_AVERAGE_GEOMETRIC || c.payoff == KGPU_PAYOFF_DOUBLE_BARRIER;
}

// FP32 plans are converted from the FP64 plan field by field.  A finite nonzero value
// below 2^-100 or above 2^120 in magnitude would underflow, or leave no headroom for
// the products the kernels form, in single precision (a diffusion of 1e-200, a daily
// quantity of 1e200); such plans are priced in FP64 or not at all.
bool fp32_value(double v) {
    const double a = std::fabs(v);
    return v == 0.0 || !std::isfinite(v) || (a >= 0x1p-100 && a <= 0x1p120);
}

// Whether FP32 kernels can carry contract c of a host book (every double field of the
// contract, its steps, events, bridge records and the model).
// Checks of a host book over ranges of its step, flag, bridge-weight and interval arrays,
// each computed once per distinct range: contracts that share a segment (the lanes of a
// shared daily grid) share the result.
struct RangeChecks {
    const kgpu_book* b;
    std::map<std::tuple<int64_t, int, bool>, bool> steps_fp32;
    std::map<std::pair<int, int>, bool> intervals_fp32;
    std::map<std::pair<int64_t, int>, int> event_steps;

    bool steps_ok(const kgpu_contract& c) {
        const bool bridged = b->bridge_daily && (c.flags & KGPU_C_BRIDGE);
        const auto key = std::make_tuple(c.step_offset, c.step_count, bridged);
        auto hit = steps_fp32.find(key);
        if (hit != steps_fp32.end()) return hit->second;
        bool ok = true;
        for (int64_t q = c.step_offset; ok && q < c.step_offset + c.step_count; ++q) {
            const kgpu_step& st = b->steps[q];
            ok = fp32_value(st.drift) && fp32_value(st.diffusion) && fp32_value(st.discount) &&
                 (!bridged || (fp32_value(b->bridge_daily[q].weight) && fp32_value(b->bridge_daily[q].width)));
        }
        steps_fp32.emplace(key, ok);
        return ok;
    }
    bool intervals_ok(const kgpu_contract& c) {
        const auto key = std::make_pair(c.bridge_offset, c.bridge_count);
        auto hit = intervals_fp32.find(key);
        if (hit != intervals_fp32.end()) return hit->second;
        bool ok = true;
        for (int q = c.bridge_offset; ok && q < c.bridge_offset + c.bridge_count; ++q)
            ok = fp32_value(b->intervals[q].drift) && fp32_value(b->intervals[q].diffusion);
        intervals_fp32.emplace(key, ok);
        return ok;
    }
    // Steps flagged KGPU_STEP_EVENT in the contract's range.
    int events(const kgpu_contract& c) {
        const auto key = std::make_pair(c.step_offset, c.step_count);
        auto hit = event_steps.find(key);
        if (hit != event_steps.end()) return hit->second;
        int n = 0;
        for (int q = 0; q < c.step_count; ++q) n += (b->step_flags[c.step_offset + q] & KGPU_STEP_EVENT) != 0;
        event_steps.emplace(key, n);
        return n;
    }
};

bool fp32_representable(const kgpu_model* m, const kgpu_book* b, const kgpu_contract& c, RangeChecks& ranges) {
    const double* first = &c.strike;
    const double* last = &c.greek_log_weight;
    for (const double* v = first; v <= last; ++v)
        if (!fp32_value(*v)) return false;
    for (double v : {m->spot, m->rate, m->dividend, m->volatility, m->v0, m->kappa, m->theta, m->xi, m->rho})
        if (!fp32_value(v)) return false;
    if (!ranges.steps_ok(c)) return false;
    for (int q = c.event_offset; q < c.event_offset + c.event_count; ++q) {
        const kgpu_event& e = b->events[q];
        if (!fp32_value(e.knock_out) || !fp32_value(e.coupon_barrier)) return false;
        for (double v : e.payment)
            if (!fp32_value(v)) return false;
    }
    if ((c.flags & KGPU_C_BRIDGE) && !ranges.intervals_ok(c)) return false;
    return true;
}

int dims_of(const kgpu_contract& c, const kgpu_model* m) {
    if (terminal_payoff(c)) return 1;
    if (c.dimensions > 0) return c.dimensions;
    return c.step_count * model_normals_per_step(m);
}

void estimate_from_sums(const kgpu_contract& c, const kgpu_settings& s, int64_t paths,
                        const TilePartial& t, kgpu_estimate* out) {
    const bool sobol = s.sampling == KGPU_SAMPLING_SOBOL;
    const double scale = c.payoff == KGPU_PAYOFF_EUROPEAN ? std::exp(c.log_scale) : 1.0;
    const double n = t.count;
    const double mean = n > 0 ? t.sum / n : 0.0;
    out->price = mean * scale;
    if (c.payoff == KGPU_PAYOFF_AVERAGE_ARITHMETIC && (c.flags & KGPU_C_AVERAGE_CONTROL))
        out->price += c.control_mean;
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

// Samples per persistent work item.  FP64 Sobol items are one reference block (they
// share the block's high part in shared memory); FP32 Sobol items may be any divisor
// of 256 (every lane reads its own block's row of the high table).
int64_t persistent_tile(bool sobol, int requested, int precision, int64_t book_samples, int sm_count) {
    if (sobol) {
        if (precision == KGPU_PRECISION_FP64) return 256;
        return (requested > 0 && requested <= 256 && 256 % requested == 0) ? requested : 64;
    }
    if (requested > 0) return requested;
    // 128-path items (four paths per lane), halved down to one path per lane while the
    // book has fewer than 128 items per SM: the grid holds 32 warps per SM, and items
    // several times that keep every warp busy to the end (measured: the 2^22-path Heston
    // Asian book in 1024-path items left 16% of the warps without an item).
    int64_t tile = 128;
    while (tile > 32 && book_samples < tile * 128 * int64_t(sm_count)) tile >>= 1;
    return tile;
}

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
        if (ctx->sobol_nibbles.ensure(size_t(dims) * 32 * 8) || ctx->sobol_dirs32.ensure(size_t(dims) * 52 * 4) ||
            ctx->sobol_shifts32.ensure(size_t(dims) * 4) || ctx->sobol_nibbles32.ensure(size_t(dims) * 32 * 4))
            return fail(ctx, KGPU_DEVICE_ERROR, "cudaMalloc of Sobol tables failed");
        sobol_nibbles_kernel<<<(dims * 32 + 255) / 256, 256, 0, ctx->stream>>>(
            static_cast<const uint64_t*>(ctx->sobol_dirs.ptr), dims, static_cast<uint64_t*>(ctx->sobol_nibbles.ptr));
        CUDA_TRY(ctx, cudaGetLastError());
        auto top32 = [&](const DeviceBuffer& in, DeviceBuffer& out, int64_t n) {
            sobol_top32_kernel<<<unsigned((n + 255) / 256), 256, 0, ctx->stream>>>(
                static_cast<const uint64_t*>(in.ptr), n, static_cast<uint32_t*>(out.ptr));
        };
        top32(ctx->sobol_dirs, ctx->sobol_dirs32, int64_t(dims) * 52);
        top32(ctx->sobol_shifts, ctx->sobol_shifts32, dims);
        top32(ctx->sobol_nibbles, ctx->sobol_nibbles32, int64_t(dims) * 32);
        CUDA_TRY(ctx, cudaGetLastError());
        // `dirs` and `shifts` are host vectors freed on return.
        CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
        ctx->sobol_dims = dims;
        ctx->sobol_seed = seed;
        ctx->sobol_high_t_blocks = 0;
    }
    t->directions = static_cast<const uint64_t*>(ctx->sobol_dirs.ptr);
    t->shifts = static_cast<const uint64_t*>(ctx->sobol_shifts.ptr);
    t->nibbles = static_cast<const uint64_t*>(ctx->sobol_nibbles.ptr);
    t->directions32 = static_cast<const uint32_t*>(ctx->sobol_dirs32.ptr);
    t->shifts32 = static_cast<const uint32_t*>(ctx->sobol_shifts32.ptr);
    t->nibbles32 = static_cast<const uint32_t*>(ctx->sobol_nibbles32.ptr);
    t->high32 = static_cast<const uint32_t*>(ctx->sobol_high32.ptr);
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

namespace {

// Everything a precision-specific runner needs about the staged call.
struct Call {
    kgpu_context* ctx;
    const kgpu_model* model;
    const kgpu_book* book;
    kgpu_settings s;
    kgpu_estimate* out;
    const volatile int32_t* cancel;
    std::vector<ContractInfo> info;
    RawBook raw;
    const double* lv_dev;
    int lv_values;
    bool sobol;
};

template <class Real>
struct PrecisionOps;
template <>
struct PrecisionOps<double> {
    static constexpr int precision = KGPU_PRECISION_FP64;
    static cudaError_t plain(int m, bool so, int b, size_t sm, cudaStream_t st, const PlainArgs<double>& a,
                             const kgpu_model& mo, const double* lv) {
        return launch_plain_fp64(m, so, b, sm, st, a, mo, lv);
    }
    static cudaError_t persistent(int m, bool so, bool ext, int b, size_t sm, cudaStream_t st,
                                  const PersistentArgs<double>& a, const kgpu_model& mo, const double* lv) {
        return launch_persistent_fp64(m, so, ext, b, sm, st, a, mo, lv);
    }
    static int occupancy(int m, bool so, bool ext, size_t sm) { return persistent_occupancy_fp64(m, so, ext, sm); }
    static cudaError_t contracts(const kgpu_contract* in, int n, ContractT<double>* out, cudaStream_t st) {
        return launch_compile_contracts_fp64(in, n, out, st);
    }
    static cudaError_t units(const kgpu_contract* c, int n, const kgpu_bridge_interval* iv,
                             const kgpu_bridge_daily* d, const uint8_t* f, const kgpu_event* e,
                             UnitT<double>* out, EndT<double>* ends, cudaStream_t st) {
        return launch_compile_units_fp64(c, n, iv, d, f, e, out, ends, st);
    }
};
template <>
struct PrecisionOps<float> {
    static constexpr int precision = KGPU_PRECISION_FP32;
    static cudaError_t plain(int m, bool so, int b, size_t sm, cudaStream_t st, const PlainArgs<float>& a,
                             const kgpu_model& mo, const double* lv) {
        return launch_plain_fp32(m, so, b, sm, st, a, mo, lv);
    }
    static cudaError_t persistent(int m, bool so, bool ext, int b, size_t sm, cudaStream_t st,
                                  const PersistentArgs<float>& a, const kgpu_model& mo, const double* lv) {
        return launch_persistent_fp32(m, so, ext, b, sm, st, a, mo, lv);
    }
    static int occupancy(int m, bool so, bool ext, size_t sm) { return persistent_occupancy_fp32(m, so, ext, sm); }
    static cudaError_t contracts(const kgpu_contract* in, int n, ContractT<float>* out, cudaStream_t st) {
        return launch_compile_contracts_fp32(in, n, out, st);
    }
    static cudaError_t units(const kgpu_contract* c, int n, const kgpu_bridge_interval* iv,
                             const kgpu_bridge_daily* d, const uint8_t* f, const kgpu_event* e,
                             UnitT<float>* out, EndT<float>* ends, cudaStream_t st) {
        return launch_compile_units_fp32(c, n, iv, d, f, e, out, ends, st);
    }
};

// The plan in the kernel's precision: FP64 reads the caller's arrays, FP32 converts them.
template <class Real>
kgpu_status compile_book(Call& k, DevBook<Real>* db);

template <>
kgpu_status compile_book<double>(Call& k, DevBook<double>* db) {
    kgpu_context* ctx = k.ctx;
    const int n = k.raw.contract_count;
    if (ctx->ccontracts.ensure(size_t(n) * sizeof(ContractT<double>)))
        return fail(ctx, KGPU_DEVICE_ERROR, "cudaMalloc of the contract table failed");
    CUDA_TRY(ctx, launch_compile_contracts_fp64(k.raw.contracts, n,
                                                static_cast<ContractT<double>*>(ctx->ccontracts.ptr), ctx->stream));
    db->contracts = static_cast<const ContractT<double>*>(ctx->ccontracts.ptr);
    db->steps = reinterpret_cast<const StepT<double>*>(k.raw.steps);
    db->flags = k.raw.flags;
    db->events = reinterpret_cast<const EventT<double>*>(k.raw.events);
    db->intervals = reinterpret_cast<const IntervalT<double>*>(k.raw.intervals);
    db->daily = reinterpret_cast<const DailyT<double>*>(k.raw.daily);
    db->units = nullptr;
    db->ends = nullptr;
    return KGPU_OK;
}

template <>
kgpu_status compile_book<float>(Call& k, DevBook<float>* db) {
    kgpu_context* ctx = k.ctx;
    const RawBook& r = k.raw;
    const int n = r.contract_count;
    if (ctx->ccontracts.ensure(size_t(n) * sizeof(ContractT<float>)) ||
        ctx->csteps.ensure(size_t(r.step_total) * sizeof(StepT<float>)) ||
        ctx->cevents.ensure(size_t(r.event_total) * sizeof(EventT<float>) + 16) ||
        ctx->cintervals.ensure(size_t(r.interval_total) * sizeof(IntervalT<float>) + 16) ||
        ctx->cdaily.ensure((r.daily ? size_t(r.step_total) : 1) * sizeof(DailyT<float>)))
        return fail(ctx, KGPU_DEVICE_ERROR, "cudaMalloc of the single-precision plan failed");
    CUDA_TRY(ctx, launch_compile_contracts_fp32(r.contracts, n,
                                                static_cast<ContractT<float>*>(ctx->ccontracts.ptr), ctx->stream));
    CUDA_TRY(ctx, launch_compile_arrays_fp32(r, static_cast<StepT<float>*>(ctx->csteps.ptr),
                                             static_cast<EventT<float>*>(ctx->cevents.ptr),
                                             static_cast<IntervalT<float>*>(ctx->cintervals.ptr),
                                             static_cast<DailyT<float>*>(ctx->cdaily.ptr), ctx->stream));
    db->contracts = static_cast<const ContractT<float>*>(ctx->ccontracts.ptr);
    db->steps = static_cast<const StepT<float>*>(ctx->csteps.ptr);
    db->flags = r.flags;
    db->events = r.events ? static_cast<const EventT<float>*>(ctx->cevents.ptr) : nullptr;
    db->intervals = r.intervals ? static_cast<const IntervalT<float>*>(ctx->cintervals.ptr) : nullptr;
    db->daily = r.daily ? static_cast<const DailyT<float>*>(ctx->cdaily.ptr) : nullptr;
    db->units = nullptr;
    db->ends = nullptr;
    return KGPU_OK;
}

template <class Real>
kgpu_status run_plain(Call& k, const DevBook<Real>& db, int& launches) {
    kgpu_context* ctx = k.ctx;
    const kgpu_settings& s = k.s;
    const int n = k.raw.contract_count;
    int64_t max_blocks = 0;
    for (int i = 0; i < n; ++i) max_blocks = std::max<int64_t>(max_blocks, (k.info[i].samples + 255) / 256);
    if (ctx->partials.ensure(size_t(max_blocks) * sizeof(BlockPartial)) ||
        ctx->merged.ensure(size_t(n) * sizeof(BlockPartial)))
        return fail(ctx, KGPU_DEVICE_ERROR, "cudaMalloc of partials failed");
    for (int i = 0; i < n; ++i) {
        if (k.cancel && *k.cancel) return fail(ctx, KGPU_INTERRUPTED, "cancelled");
        const ContractInfo& ci = k.info[i];
        PlainArgs<Real> a;
        a.book = db;
        a.contract = i;
        a.dims = ci.dims;
        a.paths = ci.paths;
        a.samples = ci.samples;
        a.seed = s.seed;
        a.antithetic = s.antithetic;
        a.statistics = !k.sobol && (!s.antithetic || ci.paths % 2 == 0);
        a.variance = a.statistics && !s.antithetic;
        a.sobol = SobolTables{nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, 0};
        kgpu_status st;
        if (k.sobol && (st = ensure_sobol(ctx, ci.dims, s.seed, &a.sobol))) return st;
        a.partials = static_cast<BlockPartial*>(ctx->partials.ptr);
        const int blocks = int((ci.samples + 255) / 256);
        size_t smem = plain_smem_bytes(PrecisionOps<Real>::precision, k.sobol, ci.dims, k.lv_values);
        if (smem > 227 * 1024)
            return fail(ctx, KGPU_INVALID_INPUT, "dimension %d exceeds the plain kernel's shared memory", ci.dims);
        CUDA_TRY(ctx, path_kernel_begin(ctx));
        CUDA_TRY(ctx, PrecisionOps<Real>::plain(k.model->kind, k.sobol, blocks, smem, ctx->stream, a, *k.model,
                                                k.lv_dev));
        CUDA_TRY(ctx, path_kernel_end(ctx));
        merge_blocks_kernel<<<1, kMergeThreads, 0, ctx->stream>>>(a.partials, blocks, a.variance, a.statistics, s.antithetic,
                                                        static_cast<BlockPartial*>(ctx->merged.ptr) + i);
        CUDA_TRY(ctx, cudaGetLastError());
        launches += 2;
        if (k.cancel) CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    }
    CUDA_TRY(ctx, cudaEventRecord(ctx->ev_stop, ctx->stream));
    std::vector<BlockPartial> merged(n);
    CUDA_TRY(ctx, cudaMemcpyAsync(merged.data(), ctx->merged.ptr, sizeof(BlockPartial) * n, cudaMemcpyDeviceToHost,
                                  ctx->stream));
    CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    for (int i = 0; i < n; ++i) {
        const kgpu_contract& c = k.book->contracts[i];
        estimate_from_moments(c, s, k.info[i].paths, merged[i], &k.out[i]);
        int grid = terminal_payoff(c) ? 1 : c.step_count;
        k.out[i].path_steps = double(k.info[i].paths) * grid;
        k.out[i].executed_steps = merged[i].executed;
        if (!std::isfinite(k.out[i].price) || !std::isfinite(k.out[i].standard_error))
            return fail(ctx, KGPU_COMPUTATION_FAILURE,
                        "Monte Carlo produced a non-finite parameter, path or result (contract %d)", i);
    }
    return KGPU_OK;
}

// Whether a book needs the persistent kernel's extended payoff set.
bool extended_payoffs(const kgpu_book& b) {
    for (int i = 0; i < b.contract_count; ++i) {
        const int p = b.contracts[i].payoff;
        if (p == KGPU_PAYOFF_BARRIER_DISCRETE || p == KGPU_PAYOFF_AVERAGE_ARITHMETIC ||
            p == KGPU_PAYOFF_AVERAGE_GEOMETRIC || p == KGPU_PAYOFF_DOUBLE_BARRIER)
            return true;
    }
    return false;
}

// Per-path value slots of every contract, the reduction chunks over them and the
// per-contract counters of simulated positions, staged for a persistent or phased launch.
template <class Real>
kgpu_status stage_values(Call& k, int* chunk_count) {
    kgpu_context* ctx = k.ctx;
    const int n = k.raw.contract_count;
    std::vector<int64_t> value_offset(n + 1, 0);
    for (int i = 0; i < n; ++i) value_offset[i + 1] = value_offset[i] + k.info[i].samples;
    // Reduction chunks of each contract's per-path values (four per thread of a CTA).
    const int64_t chunk = 1024;
    std::vector<int4> chunks;
    std::vector<int> first_chunk(n + 1, 0);
    for (int i = 0; i < n; ++i) {
        first_chunk[i] = int(chunks.size());
        for (int64_t b = 0; b < k.info[i].samples; b += chunk)
            chunks.push_back(make_int4(i, int(b), int(std::min<int64_t>(chunk, k.info[i].samples - b)), 0));
    }
    first_chunk[n] = int(chunks.size());
    kgpu_status st;
    if ((st = upload(ctx, ctx->value_offset, value_offset.data(), value_offset.size() * sizeof(int64_t))) ||
        (st = upload(ctx, ctx->chunks, chunks.data(), chunks.size() * sizeof(int4))) ||
        (st = upload(ctx, ctx->first_item, first_chunk.data(), first_chunk.size() * sizeof(int))))
        return st;
    if (ctx->values.ensure(size_t(value_offset[n]) * sizeof(Real)) ||
        ctx->tiles.ensure(chunks.size() * sizeof(TilePartial)) || ctx->tile_out.ensure(size_t(n) * sizeof(TilePartial)) ||
        ctx->executed.ensure(size_t(n) * sizeof(unsigned long long)) || ctx->queue.ensure(sizeof(int) * 4))
        return fail(ctx, KGPU_DEVICE_ERROR, "cudaMalloc of path values failed");
    CUDA_TRY(ctx, cudaMemsetAsync(static_cast<int*>(ctx->queue.ptr) + 1, 0, sizeof(int), ctx->stream));
    CUDA_TRY(ctx, cudaMemsetAsync(ctx->executed.ptr, 0, size_t(n) * sizeof(unsigned long long), ctx->stream));
    *chunk_count = int(chunks.size());
    return KGPU_OK;
}

// Sums the per-path values in a fixed order, reads the sums, the simulated positions and
// the cancellation state back, and forms the estimates.
// Ends a capture pass: instantiates the recorded launch sequence and launches it (none of
// it has run yet).  On failure the call is repeated without capture (run_book).
kgpu_status end_book_capture(kgpu_context* ctx) {
    cudaGraph_t graph = nullptr;
    ctx->capturing = false;
    const bool recorded = cudaStreamEndCapture(ctx->stream, &graph) == cudaSuccess && graph;
    cudaGraphExec_t exec = nullptr;
    if (recorded && cudaGraphInstantiate(&exec, graph, 0) != cudaSuccess) exec = nullptr;
    if (graph) cudaGraphDestroy(graph);
    if (exec && cudaGraphLaunch(exec, ctx->stream) != cudaSuccess) {
        cudaGraphExecDestroy(exec);
        exec = nullptr;
    }
    if (!exec) {
        cudaGetLastError();
        ctx->capture_failed = true;
        return fail(ctx, KGPU_DEVICE_ERROR, "the launch sequence could not be captured");
    }
    ctx->book_exec = exec;
    return KGPU_OK;
}

// Reads back a persistent or phase-major call's per-contract sums and counters, its
// cancellation word and, for the phase-major kernel, its grid-barrier failure word
// (phase_counts[failed_slot]), and turns the sums into estimates.
template <class Real>
kgpu_status collect_values(Call& k, int failed_slot) {
    kgpu_context* ctx = k.ctx;
    const kgpu_settings& s = k.s;
    const int n = k.raw.contract_count;
    CUDA_TRY(ctx, cudaEventRecord(ctx->ev_stop, ctx->stream));
    std::vector<TilePartial> sums(n);
    std::vector<unsigned long long> executed(n);
    int aborted = 0, failed = 0;
    CUDA_TRY(ctx, cudaMemcpyAsync(sums.data(), ctx->tile_out.ptr, sizeof(TilePartial) * n, cudaMemcpyDeviceToHost,
                                  ctx->stream));
    CUDA_TRY(ctx, cudaMemcpyAsync(executed.data(), ctx->executed.ptr, sizeof(unsigned long long) * n,
                                  cudaMemcpyDeviceToHost, ctx->stream));
    CUDA_TRY(ctx, cudaMemcpyAsync(&aborted, static_cast<int*>(ctx->queue.ptr) + 1, sizeof(int),
                                  cudaMemcpyDeviceToHost, ctx->stream));
    if (failed_slot >= 0)
        CUDA_TRY(ctx, cudaMemcpyAsync(&failed, static_cast<int*>(ctx->phase_counts.ptr) + failed_slot, sizeof(int),
                                      cudaMemcpyDeviceToHost, ctx->stream));
    CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    if (aborted) return fail(ctx, KGPU_INTERRUPTED, "cancelled");
    for (int i = 0; i < n; ++i) {
        const kgpu_contract& c = k.book->contracts[i];
        sums[i].executed = double(executed[i]);
        estimate_from_sums(c, s, k.info[i].paths, sums[i], &k.out[i]);
        int grid = terminal_payoff(c) ? 1 : c.step_count;
        k.out[i].path_steps = double(k.info[i].paths) * grid;
        k.out[i].executed_steps = sums[i].executed;
        if (!std::isfinite(k.out[i].price) || !std::isfinite(k.out[i].standard_error))
            return fail(ctx, KGPU_COMPUTATION_FAILURE,
                        "Monte Carlo produced a non-finite parameter, path or result (contract %d)", i);
    }
    if (failed) return fail(ctx, KGPU_DEVICE_ERROR, "the phase-major kernel's grid barrier timed out");
    return KGPU_OK;
}

// Reduces the per-path values in a fixed order, ends a capture pass, then collects.
template <class Real>
kgpu_status finish_values(Call& k, int chunk_count, int& launches, int failed_slot = -1) {
    kgpu_context* ctx = k.ctx;
    const int n = k.raw.contract_count;
    reduce_values_kernel<Real><<<chunk_count, 256, 0, ctx->stream>>>(
        static_cast<const Real*>(ctx->values.ptr), static_cast<const int4*>(ctx->chunks.ptr),
        static_cast<const int64_t*>(ctx->value_offset.ptr), static_cast<TilePartial*>(ctx->tiles.ptr));
    CUDA_TRY(ctx, cudaGetLastError());
    reduce_tiles_kernel<<<n, 256, 0, ctx->stream>>>(static_cast<const TilePartial*>(ctx->tiles.ptr),
                                                     static_cast<const int*>(ctx->first_item.ptr),
                                                     static_cast<TilePartial*>(ctx->tile_out.ptr));
    CUDA_TRY(ctx, cudaGetLastError());
    launches += 2;
    ctx->book_failed_slot = failed_slot;
    if (ctx->capturing) {
        kgpu_status st = end_book_capture(ctx);
        if (st != KGPU_OK) return st;
    }
    return collect_values<Real>(k, failed_slot);
}

// Books the segmented kernel takes: FP32 on the persistent schedule (the lane-refill
// schedule asked for by name keeps its kernel), BSM, pseudo-random, every contract a
// vanilla path reporting its payoff.
bool segmented_eligible(const Call& k) {
    if (k.s.precision != KGPU_PRECISION_FP32 || k.s.schedule != KGPU_SCHEDULE_PERSISTENT ||
        k.model->kind != KGPU_MODEL_BSM || k.sobol || k.s.antithetic)
        return false;
    for (int i = 0; i < k.book->contract_count; ++i) {
        const kgpu_contract& c = k.book->contracts[i];
        if (c.payoff != KGPU_PAYOFF_VANILLA_PATH || (c.flags & (KGPU_C_OUTPUT_DELTA | KGPU_C_OUTPUT_GAMMA)))
            return false;
    }
    return true;
}

// A vanilla-path book on the segmented kernel: per-path payoffs, then the same fixed-order
// reduction as the persistent kernels.
kgpu_status run_segmented(Call& k, const DevBook<float>& db, int& launches) {
    kgpu_context* ctx = k.ctx;
    const int n = k.raw.contract_count;
    kgpu_status st;
    int chunk_count = 0;
    if ((st = stage_values<float>(k, &chunk_count))) return st;
    std::vector<int> dims(n);
    int64_t total = 0;
    for (int i = 0; i < n; ++i) {
        dims[i] = k.info[i].dims;
        total += k.info[i].samples;
    }
    if ((st = upload(ctx, ctx->phase_dims, dims.data(), dims.size() * sizeof(int)))) return st;
    SegmentArgs a;
    a.book = db;
    a.contract_count = n;
    a.total = total;
    a.value_offset = static_cast<const int64_t*>(ctx->value_offset.ptr);
    a.dims = static_cast<const int*>(ctx->phase_dims.ptr);
    a.seed = k.s.seed;
    a.values = static_cast<float*>(ctx->values.ptr);
    a.executed = static_cast<unsigned long long*>(ctx->executed.ptr);
    a.cancel = k.cancel ? ctx->cancel_dev : nullptr;
    a.aborted = static_cast<int*>(ctx->queue.ptr) + 1;
    CancelWatcher watcher(k.cancel, ctx->cancel_host);
    CUDA_TRY(ctx, path_kernel_begin(ctx));
    CUDA_TRY(ctx, launch_segmented_fp32(total, ctx->stream, a));
    CUDA_TRY(ctx, path_kernel_end(ctx));
    launches += 1;
    return finish_values<float>(k, chunk_count, launches);
}

// Books the straight kernel takes: FP32 on the persistent schedule, pseudo-random, every
// contract a path that takes every grid step (an Asian on fixings or a vanilla path)
// reporting its payoff, under any model.
bool straight_eligible(const Call& k) {
    if (k.s.precision != KGPU_PRECISION_FP32 || k.s.schedule != KGPU_SCHEDULE_PERSISTENT || k.sobol ||
        k.s.antithetic)
        return false;
    for (int i = 0; i < k.book->contract_count; ++i) {
        const kgpu_contract& c = k.book->contracts[i];
        if ((c.payoff != KGPU_PAYOFF_ASIAN && c.payoff != KGPU_PAYOFF_VANILLA_PATH) ||
            (c.flags & (KGPU_C_OUTPUT_DELTA | KGPU_C_OUTPUT_GAMMA)))
            return false;
    }
    return true;
}

// Such a book on the straight kernel: per-path payoffs, then the same fixed-order
// reduction as the persistent kernels.
kgpu_status run_straight(Call& k, const DevBook<float>& db, int& launches) {
    kgpu_context* ctx = k.ctx;
    const int n = k.raw.contract_count;
    kgpu_status st;
    int chunk_count = 0;
    if ((st = stage_values<float>(k, &chunk_count))) return st;
    std::vector<int> dims(n);
    int64_t total = 0;
    for (int i = 0; i < n; ++i) {
        dims[i] = k.info[i].dims;
        total += k.info[i].samples;
    }
    if ((st = upload(ctx, ctx->phase_dims, dims.data(), dims.size() * sizeof(int)))) return st;
    StraightArgs a;
    a.book = db;
    a.contract_count = n;
    a.total = total;
    a.value_offset = static_cast<const int64_t*>(ctx->value_offset.ptr);
    a.dims = static_cast<const int*>(ctx->phase_dims.ptr);
    a.seed = k.s.seed;
    a.values = static_cast<float*>(ctx->values.ptr);
    a.executed = static_cast<unsigned long long*>(ctx->executed.ptr);
    a.cancel = k.cancel ? ctx->cancel_dev : nullptr;
    a.aborted = static_cast<int*>(ctx->queue.ptr) + 1;
    const size_t smem = size_t(k.lv_values) * sizeof(float) + 16;
    if (smem > 227 * 1024)
        return fail(ctx, KGPU_UNSUPPORTED_OPERATION, "the local-volatility surface exceeds shared memory");
    CancelWatcher watcher(k.cancel, ctx->cancel_host);
    CUDA_TRY(ctx, path_kernel_begin(ctx));
    CUDA_TRY(ctx, launch_straight_fp32(k.model->kind, total, smem, ctx->stream, a, *k.model, k.lv_dev));
    CUDA_TRY(ctx, path_kernel_end(ctx));
    launches += 1;
    return finish_values<float>(k, chunk_count, launches);
}

template <class Real>
kgpu_status run_persistent(Call& k, DevBook<Real> db, int& launches) {
    if constexpr (std::is_same<Real, float>::value) {
        if (segmented_eligible(k)) return run_segmented(k, db, launches);
        if (straight_eligible(k)) return run_straight(k, db, launches);
    }
    const bool ext = extended_payoffs(*k.book);
    kgpu_context* ctx = k.ctx;
    const kgpu_settings& s = k.s;
    const int n = k.raw.contract_count;
    // Bridged contracts run on per-position units compiled from their bridge plans.
    bool bridged = false;
    for (int i = 0; i < n; ++i) bridged |= (k.book->contracts[i].flags & KGPU_C_BRIDGE) != 0;
    if (bridged) {
        if (ctx->cunits.ensure(size_t(k.raw.step_total) * sizeof(UnitT<Real>)) ||
            ctx->cends.ensure(size_t(k.raw.step_total) * sizeof(EndT<Real>)))
            return fail(ctx, KGPU_DEVICE_ERROR, "cudaMalloc of bridge units failed");
        CUDA_TRY(ctx, PrecisionOps<Real>::units(k.raw.contracts, n, k.raw.intervals, k.raw.daily, k.raw.flags,
                                                k.raw.events, static_cast<UnitT<Real>*>(ctx->cunits.ptr),
                                                static_cast<EndT<Real>*>(ctx->cends.ptr), ctx->stream));
        db.units = static_cast<const UnitT<Real>*>(ctx->cunits.ptr);
        db.ends = static_cast<const EndT<Real>*>(ctx->cends.ptr);
        launches += 1;
    }
    // Sobol books run one launch per sampling dimension (one sequence per launch);
    // pseudo-random books run in a single launch.
    std::vector<int> group_of(n, 0);
    std::vector<int> group_dims;
    if (k.sobol) {
        for (int i = 0; i < n; ++i) {
            auto it = std::find(group_dims.begin(), group_dims.end(), k.info[i].dims);
            if (it == group_dims.end()) {
                group_of[i] = int(group_dims.size());
                group_dims.push_back(k.info[i].dims);
            } else {
                group_of[i] = int(it - group_dims.begin());
            }
        }
    } else {
        group_dims.push_back(0);
    }
    // Work items grouped by contract, in contract order.  Sobol tiles are one reference
    // block (they share the block's high gray-code bits).
    std::vector<int4> items;
    int64_t book_samples = 0;
    for (int i = 0; i < n; ++i) book_samples += k.info[i].samples;
    for (int i = 0; i < n; ++i) {
        int64_t tile = persistent_tile(k.sobol, s.tile_paths, s.precision, book_samples, ctx->sm_count);
        for (int64_t b = 0; b < k.info[i].samples; b += tile)
            items.push_back(make_int4(i, int(b), int(std::min<int64_t>(tile, k.info[i].samples - b)), k.info[i].dims));
    }
    const int item_count = int(items.size());
    kgpu_status st;
    if ((st = upload(ctx, ctx->items, items.data(), items.size() * sizeof(int4)))) return st;
    int chunk_count = 0;
    if ((st = stage_values<Real>(k, &chunk_count))) return st;
    CancelWatcher watcher(k.cancel, ctx->cancel_host);
    std::vector<int> order;
    std::vector<int> first_item(n + 1, 0);
    {
        int q = 0;
        for (int i = 0; i < n; ++i) {
            first_item[i] = q;
            const int64_t tile = persistent_tile(k.sobol, s.tile_paths, s.precision, book_samples, ctx->sm_count);
            q += int((k.info[i].samples + tile - 1) / tile);
        }
        first_item[n] = q;
    }
    for (size_t g = 0; g < group_dims.size(); ++g) {
        order.clear();
        std::vector<int> members;
        for (int i = 0; i < n; ++i)
            if (group_of[i] == int(g)) members.push_back(i);
        // Dispatch order: most expensive contracts first.
        std::stable_sort(members.begin(), members.end(), [&](int x, int y) {
            return double(k.info[x].samples) * k.book->contracts[x].step_count >
                   double(k.info[y].samples) * k.book->contracts[y].step_count;
        });
        for (int i : members)
            for (int q = first_item[i]; q < first_item[i + 1]; ++q) order.push_back(q);
        if (order.empty()) continue;
        if (k.cancel && *k.cancel) return fail(ctx, KGPU_INTERRUPTED, "cancelled");
        if ((st = upload(ctx, ctx->order, order.data(), order.size() * sizeof(int)))) return st;
        PersistentArgs<Real> a;
        a.book = db;
        a.items = static_cast<const int4*>(ctx->items.ptr);
        a.order = static_cast<const int*>(ctx->order.ptr);
        a.item_count = int(order.size());
        a.queue = static_cast<int*>(ctx->queue.ptr);
        a.seed = s.seed;
        a.sobol = SobolTables{nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, 0};
        if (k.sobol && (st = ensure_sobol(ctx, group_dims[g], s.seed, &a.sobol))) return st;
        if (k.sobol) {
            // High parts of every reference block the group's contracts use.
            int64_t blocks = 1;
            for (int i : members) blocks = std::max<int64_t>(blocks, (k.info[i].samples + 255) / 256);
            if (ctx->sobol_high32.ensure(size_t(blocks) * group_dims[g] * 4))
                return fail(ctx, KGPU_DEVICE_ERROR, "cudaMalloc of the Sobol high table failed");
            a.sobol.high32 = static_cast<const uint32_t*>(ctx->sobol_high32.ptr);
            const int64_t total = blocks * group_dims[g];
            sobol_high_table_kernel<<<unsigned((total + 255) / 256), 256, 0, ctx->stream>>>(
                a.sobol, int(blocks), static_cast<uint32_t*>(ctx->sobol_high32.ptr));
            CUDA_TRY(ctx, cudaGetLastError());
            launches += 1;
        }
        a.values = static_cast<Real*>(ctx->values.ptr);
        a.value_offset = static_cast<const int64_t*>(ctx->value_offset.ptr);
        a.executed = static_cast<unsigned long long*>(ctx->executed.ptr);
        a.cancel = k.cancel ? ctx->cancel_dev : nullptr;
        a.aborted = static_cast<int*>(ctx->queue.ptr) + 1;
        a.refill = s.refill > 0 ? s.refill : kRefill;
        size_t smem = persistent_smem_bytes(PrecisionOps<Real>::precision, k.sobol, k.sobol ? group_dims[g] : 0,
                                            k.lv_values);
        if (smem > 227 * 1024)
            return fail(ctx, KGPU_UNSUPPORTED_OPERATION,
                        "Sobol dimension %d exceeds the persistent kernel's shared memory; use the plain schedule",
                        group_dims[g]);
        int per_sm = PrecisionOps<Real>::occupancy(k.model->kind, k.sobol, ext, smem);
        if (s.ctas_per_sm > 0) per_sm = std::min(per_sm, s.ctas_per_sm);
        const int blocks = std::max(1, std::min(ctx->sm_count * per_sm, (a.item_count + kWarps - 1) / kWarps));
        CUDA_TRY(ctx, cudaMemsetAsync(ctx->queue.ptr, 0, sizeof(int), ctx->stream));
        CUDA_TRY(ctx, path_kernel_begin(ctx));
        CUDA_TRY(ctx, PrecisionOps<Real>::persistent(k.model->kind, k.sobol, ext, blocks, smem, ctx->stream, a,
                                                     *k.model, k.lv_dev));
        CUDA_TRY(ctx, path_kernel_end(ctx));
        launches += 1;
        // `order` is reused by the next group: wait for this launch's upload to be consumed.
        if (group_dims.size() > 1) CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    }
    return finish_values<Real>(k, chunk_count, launches);
}

// Phase-major schedule (phased.cuh) of books whose every contract is a bridged
// autocallable: FP32, BSM, the persistent schedule, one Sobol dimension count.
bool phased_eligible(const Call& k) {
    if (k.s.precision != KGPU_PRECISION_FP32 || k.s.schedule != KGPU_SCHEDULE_PERSISTENT ||
        k.model->kind != KGPU_MODEL_BSM || k.s.antithetic)
        return false;
    const kgpu_book& b = *k.book;
    if (b.contract_count >= (1 << (32 - kPhaseTagShift))) return false;
    int64_t total = 0;
    for (int i = 0; i < b.contract_count; ++i) {
        const kgpu_contract& c = b.contracts[i];
        if (c.payoff != KGPU_PAYOFF_AUTOCALLABLE || !(c.flags & KGPU_C_BRIDGE) || c.bridge_count < 1 ||
            c.bridge_count >= kPhaseMaxIntervals)
            return false;
        if (k.sobol && k.info[i].dims != k.info[0].dims) return false;
        total += k.info[i].samples;
    }
    // Two generations of the monitoring list and the knocked-in pool.
    const int64_t entry = k.sobol ? 16 : 32;
    return total < (int64_t(1) << 31) && total * entry * 3 <= (int64_t(16) << 30);
}

template <class Real, bool SOBOL>
kgpu_status run_phased_impl(Call& k, DevBook<Real> db, int& launches) {
    kgpu_context* ctx = k.ctx;
    const kgpu_settings& s = k.s;
    const int n = k.raw.contract_count;
    using Entry = PhaseEntry<Real, SOBOL>;
    if (ctx->cunits.ensure(size_t(k.raw.step_total) * sizeof(UnitT<Real>)) ||
        ctx->cends.ensure(size_t(k.raw.step_total) * sizeof(EndT<Real>)))
        return fail(ctx, KGPU_DEVICE_ERROR, "cudaMalloc of bridge units failed");
    CUDA_TRY(ctx, PrecisionOps<Real>::units(k.raw.contracts, n, k.raw.intervals, k.raw.daily, k.raw.flags, k.raw.events,
                                            static_cast<UnitT<Real>*>(ctx->cunits.ptr),
                                            static_cast<EndT<Real>*>(ctx->cends.ptr), ctx->stream));
    db.units = static_cast<const UnitT<Real>*>(ctx->cunits.ptr);
    db.ends = static_cast<const EndT<Real>*>(ctx->cends.ptr);
    launches += 1;
    kgpu_status st;
    int chunk_count = 0;
    if ((st = stage_values<Real>(k, &chunk_count))) return st;
    int64_t total = 0;
    int phases = 0;
    std::vector<int> dims(n);
    for (int i = 0; i < n; ++i) {
        total += k.info[i].samples;
        phases = std::max(phases, k.book->contracts[i].bridge_count);
        dims[i] = k.info[i].dims;
    }
    if ((st = upload(ctx, ctx->phase_dims, dims.data(), dims.size() * sizeof(int)))) return st;
    // Monitoring-list sizes of every generation, the knocked-in pool size and the grid
    // barrier's words.
    const size_t count_bytes = (size_t(phases + 1) + 4) * sizeof(int);
    if (ctx->phase_lists.ensure(3 * size_t(total) * sizeof(Entry) + 16) || ctx->phase_counts.ensure(count_bytes))
        return fail(ctx, KGPU_DEVICE_ERROR, "cudaMalloc of the phase lists failed");
    CUDA_TRY(ctx, cudaMemsetAsync(ctx->phase_counts.ptr, 0, count_bytes, ctx->stream));
    PhaseArgs<Real, SOBOL> a;
    a.book = db;
    a.phases = phases;
    a.contract_count = n;
    a.total = total;
    a.value_offset = static_cast<const int64_t*>(ctx->value_offset.ptr);
    a.dims = static_cast<const int*>(ctx->phase_dims.ptr);
    a.values = static_cast<Real*>(ctx->values.ptr);
    a.executed = static_cast<unsigned long long*>(ctx->executed.ptr);
    a.seed = s.seed;
    a.sobol = SobolTables{nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, 0};
    a.high_t = nullptr;
    a.high_blocks = 0;
    if (SOBOL) {
        if ((st = ensure_sobol(ctx, k.info[0].dims, s.seed, &a.sobol))) return st;
        int64_t blocks = 1;
        for (int i = 0; i < n; ++i) blocks = std::max<int64_t>(blocks, (k.info[i].samples + 255) / 256);
        // Like the sequence's other tables, the high table depends on the seed and the
        // dimension count only: it is kept for later calls and rebuilt when they need
        // more blocks or another sequence.
        if (ctx->sobol_high_t_blocks < blocks) {
            if (ctx->sobol_high_t.ensure(size_t(blocks) * k.info[0].dims * 4))
                return fail(ctx, KGPU_DEVICE_ERROR, "cudaMalloc of the Sobol high table failed");
            CUDA_TRY(ctx, launch_sobol_high_t(a.sobol, int(blocks), static_cast<uint32_t*>(ctx->sobol_high_t.ptr),
                                              ctx->stream));
            ctx->sobol_high_t_blocks = blocks;
            launches += 1;
        }
        a.high_t = static_cast<const uint32_t*>(ctx->sobol_high_t.ptr);
        a.high_blocks = int(ctx->sobol_high_t_blocks);
    }
    a.cancel = k.cancel ? ctx->cancel_dev : nullptr;
    a.aborted = static_cast<int*>(ctx->queue.ptr) + 1;
    Entry* lists = static_cast<Entry*>(ctx->phase_lists.ptr);
    a.lists = lists;
    a.knocked = lists + 2 * size_t(total);
    a.counts = static_cast<int*>(ctx->phase_counts.ptr);
    // Every CTA of the cooperative launch is resident at once; monitoring paths that fit
    // in that wave of lanes are completed CTA by CTA.
    const int per_sm = phased_occupancy_fp32(SOBOL);
    const int grid = std::max(1, ctx->sm_count * per_sm);
    a.complete_below = int64_t(grid) * kThreads;
    CancelWatcher watcher(k.cancel, ctx->cancel_host);
    CUDA_TRY(ctx, path_kernel_begin(ctx));
    CUDA_TRY(ctx, launch_phased_fp32(grid, ctx->stream, a));
    launches += 1;
    CUDA_TRY(ctx, path_kernel_end(ctx));
    // phase_counts[phases + 4] is the grid barrier's failure word, read with the sums
    return finish_values<Real>(k, chunk_count, launches, phases + 4);
}

template <class Real>
kgpu_status run_phased(Call& k, DevBook<Real> db, int& launches) {
    if constexpr (std::is_same<Real, float>::value)
        return k.sobol ? run_phased_impl<Real, true>(k, db, launches) : run_phased_impl<Real, false>(k, db, launches);
    else
        return fail(k.ctx, KGPU_UNSUPPORTED_OPERATION, "the phase-major schedule runs in FP32");
}

// KGPU_SCHEDULE_SHARED_GRID: the lanes of one shared daily grid on one path per sample
// (portfolio.rs:1275-1439), path-major.  plan_shared checks the lanes on the host (before
// the call's timed region) and numbers the action dates; run_shared launches.
struct SharedPlan {
    int base = 0;
    int slots = 0;
    std::vector<int16_t> slot;
};

kgpu_status plan_shared(Call& k, SharedPlan* plan) {
    kgpu_context* ctx = k.ctx;
    const kgpu_book& b = *k.book;
    const int n = b.contract_count;
    int base = 0;
    for (int i = 0; i < n; ++i)
        if (b.contracts[i].step_count >= b.contracts[base].step_count) base = i;
    const kgpu_contract& bc = b.contracts[base];
    const int steps = bc.step_count;
    std::vector<char> ends(steps, 0);
    for (int q = 0; q < bc.bridge_count; ++q) ends[b.intervals[bc.bridge_offset + q].end] = 1;
    std::vector<int16_t> slot(steps, -1);
    int slots = 0;
    std::map<std::tuple<int64_t, int, int, int>, bool> prefixes;
    auto take = [&](int step) {
        if (step < 0 || step >= steps || !ends[step]) return false;
        if (slot[step] < 0) slot[step] = int16_t(slots++);
        return slots < 32768;
    };
    for (int i = 0; i < n; ++i) {
        const kgpu_contract& c = b.contracts[i];
        if (c.payoff != KGPU_PAYOFF_AUTOCALLABLE || !(c.flags & KGPU_C_BRIDGE))
            return fail(ctx, KGPU_UNSUPPORTED_OPERATION, "lane %d: shared-grid lanes are bridged autocallables", i);
        if (k.info[i].dims != k.info[base].dims || k.info[i].paths != k.info[base].paths)
            return fail(ctx, KGPU_INVALID_INPUT, "lane %d: lanes share their sampling dimensions and path count", i);
        // Lanes that share a segment (or the base's own arrays) are compared once.
        const auto seg = std::make_tuple(c.step_offset, c.step_count, c.bridge_offset, c.bridge_count);
        auto known = prefixes.find(seg);
        bool prefix;
        if (known != prefixes.end()) {
            prefix = known->second;
        } else {
            const bool same_steps = c.step_offset == bc.step_offset;
            prefix = c.bridge_count <= bc.bridge_count &&
                     (same_steps || (std::memcmp(b.steps + c.step_offset, b.steps + bc.step_offset,
                                                 sizeof(kgpu_step) * size_t(c.step_count)) == 0 &&
                                     std::memcmp(b.bridge_daily + c.step_offset, b.bridge_daily + bc.step_offset,
                                                 sizeof(kgpu_bridge_daily) * size_t(c.step_count)) == 0)) &&
                     (c.bridge_offset == bc.bridge_offset ||
                      std::memcmp(b.intervals + c.bridge_offset, b.intervals + bc.bridge_offset,
                                  sizeof(kgpu_bridge_interval) * size_t(c.bridge_count)) == 0);
            for (int q = 0; prefix && !same_steps && q < c.step_count; ++q)
                prefix = ((b.step_flags[c.step_offset + q] ^ b.step_flags[bc.step_offset + q]) & KGPU_STEP_KNOCK_IN) == 0;
            prefixes.emplace(seg, prefix);
        }
        if (!prefix) return fail(ctx, KGPU_INVALID_INPUT, "lane %d: the grid is not a prefix of the longest lane's", i);
        for (int e = 0; e < c.event_count; ++e)
            if (!take(b.events[c.event_offset + e].step))
                return fail(ctx, KGPU_INVALID_INPUT, "lane %d: event %d is not on an interval end", i, e);
        if (!take(c.step_count - 1)) return fail(ctx, KGPU_INVALID_INPUT, "lane %d: maturity is not an interval end", i);
    }
    plan->base = base;
    plan->slots = slots;
    plan->slot = std::move(slot);
    return KGPU_OK;
}

template <class Real>
kgpu_status run_shared(Call& k, const DevBook<Real>& db, const SharedPlan& plan, int& launches) {
    kgpu_context* ctx = k.ctx;
    const kgpu_book& b = *k.book;
    const kgpu_settings& s = k.s;
    const int n = b.contract_count;
    const int base = plan.base, slots = plan.slots;
    const std::vector<int16_t>& slot = plan.slot;
    const int steps = b.contracts[base].step_count;
    const size_t smem = shared_grid_smem_bytes(sizeof(Real), slots, steps, k.sobol, s.antithetic != 0);
    if (smem > 227 * 1024)
        return fail(ctx, KGPU_UNSUPPORTED_OPERATION, "%d action dates exceed the shared-grid kernel's shared memory",
                    slots);
    const int64_t samples = k.info[base].samples;
    const int ctas = int((samples + kSharedThreads - 1) / kSharedThreads);
    kgpu_status st;
    if ((st = upload(ctx, ctx->shared_slots, slot.data(), slot.size() * sizeof(int16_t)))) return st;
    if (ctx->partials.ensure(size_t(n) * ctas * 3 * sizeof(double)) || ctx->merged.ensure(size_t(n) * 3 * sizeof(double)))
        return fail(ctx, KGPU_DEVICE_ERROR, "cudaMalloc of the shared-grid sums failed");
    SharedArgs<Real> a;
    a.book = db;
    a.lanes = n;
    a.base = base;
    a.slot = static_cast<const int16_t*>(ctx->shared_slots.ptr);
    a.slots = slots;
    a.steps = steps;
    a.dims = k.info[base].dims;
    a.samples = samples;
    a.paths = k.info[base].paths;
    a.antithetic = s.antithetic != 0;
    a.seed = s.seed;
    a.sobol = SobolTables{nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, 0};
    if (k.sobol && (st = ensure_sobol(ctx, a.dims, s.seed, &a.sobol))) return st;
    a.partials = static_cast<double*>(ctx->partials.ptr);
    a.ctas = ctas;
    CUDA_TRY(ctx, path_kernel_begin(ctx));
    // Lane chunks: enough CTAs for about four waves of resident CTAs, each chunk at
    // least 16 lanes.
    const int resident = (std::is_same<Real, double>::value ? shared_grid_occupancy_fp64(k.sobol, smem)
                                                            : shared_grid_occupancy_fp32(k.sobol, smem)) *
                         ctx->sm_count;
    const int chunks = int(std::max<int64_t>(
        1, std::min<int64_t>({(n + 15) / 16, (4LL * resident + ctas - 1) / ctas, int64_t(65535)})));
    cudaError_t launched;
    if constexpr (std::is_same<Real, double>::value)
        launched = launch_shared_grid_fp64(k.sobol, ctas, chunks, smem, ctx->stream, a);
    else
        launched = launch_shared_grid_fp32(k.sobol, ctas, chunks, smem, ctx->stream, a);
    CUDA_TRY(ctx, launched);
    CUDA_TRY(ctx, path_kernel_end(ctx));
    CUDA_TRY(ctx, launch_shared_merge(a.partials, ctas, n, static_cast<double*>(ctx->merged.ptr), ctx->stream));
    launches += 2;
    CUDA_TRY(ctx, cudaEventRecord(ctx->ev_stop, ctx->stream));
    std::vector<double> merged(size_t(n) * 3);
    CUDA_TRY(ctx, cudaMemcpyAsync(merged.data(), ctx->merged.ptr, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost,
                                  ctx->stream));
    CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    for (int i = 0; i < n; ++i) {
        const kgpu_contract& c = b.contracts[i];
        const int64_t paths = k.info[i].paths;
        const double path_steps = double(paths) * c.step_count;
        const double sum = merged[3 * i], sumsq = merged[3 * i + 1], pairsq = merged[3 * i + 2];
        TilePartial t{sum, sumsq, double(paths), path_steps};
        estimate_from_sums(c, s, paths, t, &k.out[i]);
        if (s.antithetic && !k.sobol) {
            // sampling_standard_error over the pair means (monte_carlo.rs:1435-1452).
            kgpu_estimate& e = k.out[i];
            e.standard_error = 0.0;
            const double pairs = double(paths / 2);
            if (paths % 2 != 0) {
                e.uncertainty_status = KGPU_UNCERTAINTY_INCOMPLETE_ANTITHETIC_PAIR;
            } else if (pairs < 2) {
                e.uncertainty_status = KGPU_UNCERTAINTY_INSUFFICIENT_OBSERVATIONS;
            } else {
                const double mean = 0.5 * sum / pairs;
                const double var = std::max(0.0, (pairsq - 0.5 * sum * mean) / (pairs - 1.0));
                e.standard_error = std::sqrt(var / pairs);
                e.uncertainty_status = e.standard_error == 0.0 ? KGPU_UNCERTAINTY_ZERO_OBSERVED_VARIANCE
                                                               : KGPU_UNCERTAINTY_AVAILABLE;
            }
        }
        k.out[i].path_steps = path_steps;
        k.out[i].executed_steps = path_steps;
        if (!std::isfinite(k.out[i].price) || !std::isfinite(k.out[i].sample_error))
            return fail(ctx, KGPU_COMPUTATION_FAILURE,
                        "Monte Carlo produced a non-finite parameter, path or result (lane %d)", i);
    }
    return KGPU_OK;
}

// Key of a persistent call's launch sequence: everything its launches and its staged
// metadata derive from -- the model's scalars, the settings, the book's device arrays and
// sizes, the host contract table, whether a cancellation word is watched, the cached
// Sobol sequence and the device buffers' addresses (through their reallocation count).
std::vector<unsigned char> book_call_key(const Call& k) {
    std::vector<unsigned char> key;
    auto put = [&key](const void* p, size_t n) {
        const unsigned char* b = static_cast<const unsigned char*>(p);
        key.insert(key.end(), b, b + n);
    };
    kgpu_model m = *k.model;
    m.lv_times = m.lv_spots = m.lv_values = nullptr;
    put(&m, sizeof(m));
    put(&k.s, sizeof(k.s));
    const RawBook& r = k.raw;
    const void* ptrs[] = {r.contracts, r.steps, r.flags, r.events, r.intervals, r.daily, k.lv_dev};
    put(ptrs, sizeof(ptrs));
    const int64_t sizes[] = {r.contract_count,
                             r.step_total,
                             r.event_total,
                             r.interval_total,
                             k.lv_values,
                             k.cancel ? 1 : 0,
                             k.ctx->sobol_dims,
                             int64_t(k.ctx->sobol_seed),
                             k.ctx->sobol_high_t_blocks,
                             int64_t(kgpu::alloc_generation())};
    put(sizes, sizeof(sizes));
    put(k.book->contracts, sizeof(kgpu_contract) * size_t(r.contract_count));
    return key;
}

// A call whose key equals the captured sequence's: launch the graph and collect.
template <class Real>
kgpu_status replay_book(Call& k) {
    kgpu_context* ctx = k.ctx;
    ctx->last_path_kernel_ms = 0.0;
    if (k.cancel && *k.cancel) return fail(ctx, KGPU_INTERRUPTED, "cancelled");
    CUDA_TRY(ctx, cudaEventRecord(ctx->ev_start, ctx->stream));
    kgpu_status st;
    {
        CancelWatcher watcher(k.cancel, ctx->cancel_host);
        CUDA_TRY(ctx, cudaGraphLaunch(ctx->book_exec, ctx->stream));
        ctx->path_events_used = ctx->book_path_events;
        st = collect_values<Real>(k, ctx->book_failed_slot);
    }
    float ms = 0;
    if (cudaEventElapsedTime(&ms, ctx->ev_start, ctx->ev_stop) == cudaSuccess) ctx->last_kernel_ms = ms;
    if (st == KGPU_OK) ctx->last_path_kernel_ms = path_kernel_ms(ctx);
    cudaGetLastError();
    ctx->last_launches = ctx->book_launches;
    return st;
}

template <class Real>
kgpu_status run_direct(Call& k, const SharedPlan& shared, bool capture);

// Prices a staged book.  The persistent schedules' launch sequence runs as a CUDA graph:
// the first call with a key runs directly and stages the sequence's metadata on the
// device; an identical second call captures the sequence (its uploads would copy the same
// bytes into the same buffers, so they are skipped) and launches the graph; later
// identical calls replay it.  Any other call on the context drops the graph.  Lane-refill
// Sobol books of several dimension counts (one launch per count, synchronised in between)
// run directly.
template <class Real>
kgpu_status run_book(Call& k) {
    kgpu_context* ctx = k.ctx;
    SharedPlan shared;
    if (k.s.schedule == KGPU_SCHEDULE_SHARED_GRID) {
        kgpu_status planned = plan_shared(k, &shared);
        if (planned) return planned;
    }
    bool graphable = k.s.schedule == KGPU_SCHEDULE_PERSISTENT || k.s.schedule == KGPU_SCHEDULE_LANE_REFILL;
    if (graphable && k.sobol && !(k.s.schedule == KGPU_SCHEDULE_PERSISTENT && phased_eligible(k)))
        for (const ContractInfo& ci : k.info) graphable = graphable && ci.dims == k.info[0].dims;
    std::vector<unsigned char> key;
    if (graphable) key = book_call_key(k);
    ctx->last_graph = 0;
    if (graphable && ctx->book_exec && ctx->book_key == key) {
        ctx->last_graph = 2;
        return replay_book<Real>(k);
    }
    if (ctx->book_exec) cudaGraphExecDestroy(ctx->book_exec);
    ctx->book_exec = nullptr;
    ctx->book_key.clear();
    const bool capture = graphable && ctx->last_book_key == key;
    ctx->last_book_key = key;
    ctx->capture_failed = false;
    kgpu_status st = run_direct<Real>(k, shared, capture);
    if (capture && (ctx->capturing || ctx->capture_failed)) {
        // The sequence could not be captured (an error inside the pass, or a refused
        // capture): nothing of it ran.  Repeat the call directly.
        if (ctx->capturing) {
            cudaGraph_t g = nullptr;
            cudaStreamEndCapture(ctx->stream, &g);
            if (g) cudaGraphDestroy(g);
            ctx->capturing = false;
        }
        cudaGetLastError();
        ctx->error.clear();
        ctx->capture_failed = false;
        ctx->last_book_key.clear();
        if (ctx->book_exec) cudaGraphExecDestroy(ctx->book_exec);
        ctx->book_exec = nullptr;
        st = run_direct<Real>(k, shared, false);
    } else if (capture && ctx->book_exec) {
        if (st == KGPU_OK) {
            ctx->book_key = key;
            ctx->book_launches = ctx->last_launches;
            ctx->book_path_events = ctx->path_events_used;
            ctx->last_graph = 1;
        } else {
            cudaGraphExecDestroy(ctx->book_exec);
            ctx->book_exec = nullptr;
        }
    }
    return st;
}

template <class Real>
kgpu_status run_direct(Call& k, const SharedPlan& shared, bool capture) {
    kgpu_context* ctx = k.ctx;
    CUDA_TRY(ctx, cudaEventRecord(ctx->ev_start, ctx->stream));
    ctx->path_events_used = 0;
    ctx->last_path_kernel_ms = 0.0;
    if (capture) {
        if (cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal) == cudaSuccess)
            ctx->capturing = true;
        else
            ctx->capture_failed = true;  // run_book repeats the call directly
        if (!ctx->capturing) return KGPU_DEVICE_ERROR;
    }
    DevBook<Real> db;
    kgpu_status st = compile_book<Real>(k, &db);
    if (st) return st;
    int launches = std::is_same<Real, float>::value ? 2 : 1;
    st = k.s.schedule == KGPU_SCHEDULE_PERSISTENT    ? (phased_eligible(k) ? run_phased<Real>(k, db, launches)
                                                                           : run_persistent<Real>(k, db, launches))
         : k.s.schedule == KGPU_SCHEDULE_LANE_REFILL ? run_persistent<Real>(k, db, launches)
         : k.s.schedule == KGPU_SCHEDULE_SHARED_GRID ? run_shared<Real>(k, db, shared, launches)
                                                     : run_plain<Real>(k, db, launches);
    float ms = 0;
    if (cudaEventElapsedTime(&ms, ctx->ev_start, ctx->ev_stop) == cudaSuccess) ctx->last_kernel_ms = ms;
    if (st == KGPU_OK) ctx->last_path_kernel_ms = path_kernel_ms(ctx);
    cudaGetLastError();  // a refused timing query must not surface in the next call
    ctx->last_launches = launches;
    return st;
}

}  // namespace

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
    Call k;
    k.ctx = ctx;
    k.model = model;
    k.book = book;
    k.s = *settings;
    k.out = out;
    k.cancel = cancel;
    const kgpu_settings& s = k.s;
    if (s.precision != KGPU_PRECISION_FP64 && s.precision != KGPU_PRECISION_FP32)
        return fail(ctx, KGPU_INVALID_INPUT, "unknown precision %d", s.precision);
    if (s.sampling != KGPU_SAMPLING_PSEUDO_RANDOM && s.sampling != KGPU_SAMPLING_SOBOL)
        return fail(ctx, KGPU_INVALID_INPUT, "unknown sampling %d", s.sampling);
    if (model->kind < KGPU_MODEL_BSM || model->kind > KGPU_MODEL_LOCAL_VOL)
        return fail(ctx, KGPU_INVALID_INPUT, "unknown model %d", model->kind);
    k.sobol = s.sampling == KGPU_SAMPLING_SOBOL;
    const bool persistent = s.schedule == KGPU_SCHEDULE_PERSISTENT || s.schedule == KGPU_SCHEDULE_LANE_REFILL;
    if (s.schedule < KGPU_SCHEDULE_PLAIN || s.schedule > KGPU_SCHEDULE_LANE_REFILL)
        return fail(ctx, KGPU_INVALID_INPUT, "unknown schedule %d", s.schedule);
    if (persistent && s.antithetic)
        return fail(ctx, KGPU_UNSUPPORTED_OPERATION,
                    "the persistent schedule does not pair antithetic samples; use the plain schedule");
    if (s.schedule == KGPU_SCHEDULE_SHARED_GRID && (device_resident || model->kind != KGPU_MODEL_BSM))
        return fail(ctx, KGPU_UNSUPPORTED_OPERATION, "the shared-grid schedule takes host books under BSM");
    // Validate contracts (MonteCarloSettings::validate, monte_carlo.rs:197-220).
    k.info.resize(n);
    RangeChecks ranges{book, {}, {}, {}};
    for (int i = 0; i < n; ++i) {
        const kgpu_contract& c = book->contracts[i];
        int64_t paths = c.path_count > 0 ? c.path_count : s.path_count;
        if (paths < 1 || paths > 2147483647LL)
            return fail(ctx, KGPU_INVALID_INPUT, "contract %d: path_count must be positive", i);
        if (k.sobol && !is_pow2(paths))
            return fail(ctx, KGPU_INVALID_INPUT, "path_count must be a power of two for Sobol sampling");
        if (c.payoff < KGPU_PAYOFF_EUROPEAN || c.payoff > KGPU_PAYOFF_DOUBLE_BARRIER)
            return fail(ctx, KGPU_INVALID_INPUT, "contract %d: unknown payoff %d", i, c.payoff);
        if (!(c.spot > 0.0) || !std::isfinite(c.spot))
            return fail(ctx, KGPU_INVALID_INPUT, "contract %d: spot must be positive and finite", i);
        if ((c.payoff == KGPU_PAYOFF_BARRIER || c.payoff == KGPU_PAYOFF_DOUBLE_BARRIER) &&
            (model->kind != KGPU_MODEL_BSM || !(c.diffusion > 0.0)))
            return fail(ctx, KGPU_UNSUPPORTED_OPERATION, "contract %d: the Monte Carlo barrier needs BSM volatility", i);
        if ((c.payoff == KGPU_PAYOFF_AVERAGE_ARITHMETIC || c.payoff == KGPU_PAYOFF_AVERAGE_GEOMETRIC) &&
            model->kind != KGPU_MODEL_BSM)
            return fail(ctx, KGPU_UNSUPPORTED_OPERATION, "contract %d: average-price sampling needs BSM", i);
        if (c.payoff == KGPU_PAYOFF_BARRIER_DISCRETE &&
            (model->kind != KGPU_MODEL_BSM || c.event_count != c.step_count || !book->events))
            return fail(ctx, KGPU_INVALID_INPUT,
                        "contract %d: a scheduled barrier needs BSM and one event record per date", i);
        if (c.step_count < 1 || c.step_offset < 0 || c.step_offset + c.step_count > book->step_total)
            return fail(ctx, KGPU_INVALID_INPUT, "contract %d: steps out of range", i);
        if (c.event_count < 0 || c.event_offset < 0 || c.event_offset + c.event_count > book->event_total)
            return fail(ctx, KGPU_INVALID_INPUT, "contract %d: events out of range", i);
        if (c.event_count > 0 && !book->events)
            return fail(ctx, KGPU_INVALID_INPUT, "contract %d: events missing", i);
        if (c.dimensions < 0 ||
            (c.dimensions > 0 && (terminal_payoff(c) || c.dimensions < c.step_count * model_normals_per_step(model))))
            return fail(ctx, KGPU_INVALID_INPUT, "contract %d: dimensions must cover every step's normals", i);
        if (c.flags & KGPU_C_BRIDGE) {
            if (model->kind != KGPU_MODEL_BSM || !book->bridge_daily || !book->intervals || c.bridge_count < 1 ||
                c.bridge_offset < 0 || c.bridge_offset + c.bridge_count > book->interval_total)
                return fail(ctx, KGPU_INVALID_INPUT, "contract %d: invalid bridge plan", i);
            if (!device_resident) {
                // Interval ends ascend strictly and the last one is the final step.
                int previous = -1;
                for (int q = 0; q < c.bridge_count; ++q) {
                    const int end = book->intervals[c.bridge_offset + q].end;
                    if (end <= previous || end >= c.step_count)
                        return fail(ctx, KGPU_INVALID_INPUT, "contract %d: bridge interval %d ends out of order", i, q);
                    previous = end;
                }
                if (previous != c.step_count - 1)
                    return fail(ctx, KGPU_INVALID_INPUT, "contract %d: the last bridge interval must end the grid", i);
            }
        }
        if (!device_resident && c.payoff == KGPU_PAYOFF_AUTOCALLABLE) {
            // Every event step must be backed by an event record.
            const int events = ranges.events(c);
            if (events != c.event_count)
                return fail(ctx, KGPU_INVALID_INPUT, "contract %d: %d event steps but %d events", i, events,
                            c.event_count);
        }
        if (s.precision == KGPU_PRECISION_FP32 && !device_resident && !fp32_representable(model, book, c, ranges))
            return fail(ctx, KGPU_UNSUPPORTED_OPERATION,
                        "contract %d: FP32 cannot carry this plan (a nonzero value below 2^-100 or above "
                        "2^120 in magnitude); price it in FP64",
                        i);
        k.info[i].dims = dims_of(c, model);
        k.info[i].paths = paths;
        k.info[i].samples = s.antithetic ? (paths + 1) / 2 : paths;
    }
    kgpu_status st;
    // Stage the book.
    RawBook& r = k.raw;
    r.contract_count = n;
    r.step_total = book->step_total;
    r.event_total = book->event_total;
    r.interval_total = book->interval_total;
    if (!device_resident) {
        if ((st = upload(ctx, ctx->steps, book->steps, size_t(book->step_total) * sizeof(kgpu_step))) ||
            (st = upload(ctx, ctx->flags, book->step_flags, size_t(book->step_total))) ||
            (st = upload(ctx, ctx->events, book->events, size_t(book->event_total) * sizeof(kgpu_event))) ||
            (st = upload(ctx, ctx->intervals, book->intervals, size_t(book->interval_total) * sizeof(kgpu_bridge_interval))))
            return st;
        if (book->bridge_daily &&
            (st = upload(ctx, ctx->daily, book->bridge_daily, size_t(book->step_total) * sizeof(kgpu_bridge_daily))))
            return st;
        r.steps = static_cast<const kgpu_step*>(ctx->steps.ptr);
        r.flags = static_cast<const uint8_t*>(ctx->flags.ptr);
        r.events = book->event_total ? static_cast<const kgpu_event*>(ctx->events.ptr) : nullptr;
        r.intervals = book->interval_total ? static_cast<const kgpu_bridge_interval*>(ctx->intervals.ptr) : nullptr;
        r.daily = book->bridge_daily ? static_cast<const kgpu_bridge_daily*>(ctx->daily.ptr) : nullptr;
    } else {
        r.steps = book->steps;
        r.flags = book->step_flags;
        r.events = book->event_total ? book->events : nullptr;
        r.intervals = book->interval_total ? book->intervals : nullptr;
        r.daily = book->bridge_daily;
    }
    if ((st = upload(ctx, ctx->contracts, book->contracts, size_t(n) * sizeof(kgpu_contract)))) return st;
    r.contracts = static_cast<const kgpu_contract*>(ctx->contracts.ptr);
    // Local volatility surface: [years since the first node][spots][values].
    k.lv_values = 0;
    k.lv_dev = nullptr;
    if (model->kind == KGPU_MODEL_LOCAL_VOL) {
        const int nt = model->lv_time_count, ns = model->lv_spot_count;
        if (nt < 2 || ns < 2 || !model->lv_times || !model->lv_spots || !model->lv_values)
            return fail(ctx, KGPU_INVALID_INPUT, "invalid local volatility surface");
        std::vector<double> lv(size_t(nt) + ns + size_t(nt) * ns);
        for (int i = 0; i < nt; ++i) lv[i] = model->lv_times[i] - model->lv_times[0];
        for (int i = 0; i < ns; ++i) lv[nt + i] = model->lv_spots[i];
        std::memcpy(&lv[nt + ns], model->lv_values, sizeof(double) * size_t(nt) * ns);
        k.lv_values = int(lv.size());
        if ((st = upload(ctx, ctx->lv, lv.data(), lv.size() * sizeof(double)))) return st;
        CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));  // `lv` is a host vector
        k.lv_dev = static_cast<const double*>(ctx->lv.ptr);
    }
    *ctx->cancel_host = 0;
    return s.precision == KGPU_PRECISION_FP64 ? run_book<double>(k) : run_book<float>(k);
}

namespace kgpu {

size_t plain_smem_bytes(int precision, bool sobol, int dims, int lv_values) {
    size_t real = precision == KGPU_PRECISION_FP64 ? 8 : 4;
    return 2 * kThreads * 8 + kThreads * 4 + (sobol ? size_t(dims) * 8 : 0) + size_t(lv_values) * real + 16;
}

size_t persistent_smem_bytes(int precision, bool sobol, int dims, int lv_values) {
    size_t real = precision == KGPU_PRECISION_FP64 ? 8 : 4;
    // FP64 Sobol keeps a per-warp shared copy of the item's high part; FP32 reads a table.
    return (sobol && precision == KGPU_PRECISION_FP64 ? size_t(dims) * 8 * kWarps : 0) +
           size_t(lv_values) * real + 16;
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
