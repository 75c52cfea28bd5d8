// Instantiation body shared by kernels_fp64.cu and kernels_fp32.cu; REAL and PRECISION
// are defined by the including translation unit.
#include "launch.h"
#include "phased.cuh"
#include "segmented.cuh"
#include "shared_grid.cuh"
#include "straight.cuh"

namespace kgpu {

template <int MODEL, bool SOBOL>
static cudaError_t plain_one(int blocks, size_t smem, cudaStream_t s, const PlainArgs<REAL>& a,
                             const kgpu_model& m, const double* lv) {
    auto k = plain_kernel<REAL, MODEL, SOBOL>;
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
    if (e != cudaSuccess) return e;
    k<<<blocks, kThreads, smem, s>>>(a, m, lv);
    return cudaGetLastError();
}

template <int MODEL, bool SOBOL, bool EXT>
static cudaError_t persistent_one(int blocks, size_t smem, cudaStream_t s,
                                  const PersistentArgs<REAL>& a, const kgpu_model& m, const double* lv) {
    auto k = persistent_kernel<REAL, MODEL, SOBOL, EXT>;
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
    if (e != cudaSuccess) return e;
    k<<<blocks, kThreads, smem, s>>>(a, m, lv);
    return cudaGetLastError();
}

template <int MODEL, bool SOBOL, bool EXT>
static int occupancy_one(size_t smem) {
    auto k = persistent_kernel<REAL, MODEL, SOBOL, EXT>;
    if (cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)) != cudaSuccess)
        return 1;
    int n = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k, kThreads, smem) != cudaSuccess) return 1;
    return n > 0 ? n : 1;
}

#define KGPU_DISPATCH(FN, ...)                                                         \
    switch (model * 2 + int(sobol)) {                                                  \
        case 0: return FN<KGPU_MODEL_BSM, false>(__VA_ARGS__);                         \
        case 1: return FN<KGPU_MODEL_BSM, true>(__VA_ARGS__);                          \
        case 2: return FN<KGPU_MODEL_HESTON, false>(__VA_ARGS__);                      \
        case 3: return FN<KGPU_MODEL_HESTON, true>(__VA_ARGS__);                       \
        case 4: return FN<KGPU_MODEL_LOCAL_VOL, false>(__VA_ARGS__);                   \
        default: return FN<KGPU_MODEL_LOCAL_VOL, true>(__VA_ARGS__);                   \
    }

// The extended payoffs are BSM-only: other models use the core instantiation.
#define KGPU_DISPATCH_EXT(FN, ...)                                                     \
    switch (model * 2 + int(sobol)) {                                                  \
        case 0: return ext ? FN<KGPU_MODEL_BSM, false, true>(__VA_ARGS__)              \
                           : FN<KGPU_MODEL_BSM, false, false>(__VA_ARGS__);            \
        case 1: return ext ? FN<KGPU_MODEL_BSM, true, true>(__VA_ARGS__)               \
                           : FN<KGPU_MODEL_BSM, true, false>(__VA_ARGS__);             \
        case 2: return FN<KGPU_MODEL_HESTON, false, false>(__VA_ARGS__);               \
        case 3: return FN<KGPU_MODEL_HESTON, true, false>(__VA_ARGS__);                \
        case 4: return FN<KGPU_MODEL_LOCAL_VOL, false, false>(__VA_ARGS__);            \
        default: return FN<KGPU_MODEL_LOCAL_VOL, true, false>(__VA_ARGS__);            \
    }

#define KGPU_CAT2(a, b) a##b
#define KGPU_CAT(a, b) KGPU_CAT2(a, b)

cudaError_t KGPU_CAT(launch_plain_, PRECISION)(int model, bool sobol, int blocks, size_t smem,
                                               cudaStream_t s, const PlainArgs<REAL>& a,
                                               const kgpu_model& m, const double* lv) {
    KGPU_DISPATCH(plain_one, blocks, smem, s, a, m, lv)
}

cudaError_t KGPU_CAT(launch_persistent_, PRECISION)(int model, bool sobol, bool ext, int blocks, size_t smem,
                                                    cudaStream_t s, const PersistentArgs<REAL>& a,
                                                    const kgpu_model& m, const double* lv) {
    KGPU_DISPATCH_EXT(persistent_one, blocks, smem, s, a, m, lv)
}

int KGPU_CAT(persistent_occupancy_, PRECISION)(int model, bool sobol, bool ext, size_t smem) {
    KGPU_DISPATCH_EXT(occupancy_one, smem)
}

cudaError_t KGPU_CAT(launch_compile_contracts_, PRECISION)(const kgpu_contract* in, int n,
                                                           ContractT<REAL>* out, cudaStream_t s) {
    compile_contracts_kernel<REAL><<<(n + 255) / 256, 256, 0, s>>>(in, n, out);
    return cudaGetLastError();
}

cudaError_t KGPU_CAT(launch_compile_units_, PRECISION)(const kgpu_contract* contracts, int n,
                                                       const kgpu_bridge_interval* intervals,
                                                       const kgpu_bridge_daily* daily, const uint8_t* flags,
                                                       const kgpu_event* events, UnitT<REAL>* units,
                                                       EndT<REAL>* ends, cudaStream_t s) {
    compile_units_kernel<REAL><<<n, 256, 0, s>>>(contracts, intervals, daily, flags, events, units, ends);
    return cudaGetLastError();
}

// Normals first..first+count of block `block`, one thread per Box-Muller pair.
static __global__ void pcg_normals_kernel(uint64_t seed, uint64_t block, uint64_t first, int64_t count,
                                   double* out) {
    int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= count) return;
    uint64_t index = first + uint64_t(i);
    Pcg g = pcg_new(seed, block);
    pcg_advance(g, (index / 2) * 4);
    uint64_t b1 = pcg_bits52(g), b2 = pcg_bits52(g);
    REAL c, s;
    box_muller(b1, b2, &c, &s);
    out[i] = double((index & 1) ? s : c);
}

static __global__ void sobol_points_kernel(SobolTables t, int dim, uint64_t first, int64_t count,
                                    uint64_t* bits, double* normals) {
    int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= count) return;
    uint64_t index = first + uint64_t(i);
    uint64_t x = t.shifts[dim];
    uint64_t g = index ^ (index >> 1);
    while (g) {
        x ^= t.directions[size_t(__ffsll(g) - 1) * t.dims + dim];
        g &= g - 1;
    }
    if (bits) bits[i] = x;
    if (normals) normals[i] = double(sobol_normal(x, REAL()));
}

#if KGPU_FP32_UNIT
// A cooperative launch: every CTA is resident at once (the kernel's grid barrier needs
// it); the runtime refuses a grid larger than the device can hold.
template <bool SOBOL>
static cudaError_t phased_one(int blocks, cudaStream_t s, const PhaseArgs<float, SOBOL>& a) {
    PhaseArgs<float, SOBOL> args = a;
    void* params[] = {&args};
    return cudaLaunchCooperativeKernel((const void*)phased_kernel<float, SOBOL>, dim3(blocks), dim3(kThreads), params,
                                       0, s);
}

cudaError_t launch_phased_fp32(int blocks, cudaStream_t s, const PhaseArgs<float, true>& a) {
    return phased_one<true>(blocks, s, a);
}

cudaError_t launch_phased_fp32(int blocks, cudaStream_t s, const PhaseArgs<float, false>& a) {
    return phased_one<false>(blocks, s, a);
}

int phased_occupancy_fp32(bool sobol) {
    int n = 0;
    const cudaError_t e = sobol ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, phased_kernel<float, true>, kThreads, 0)
                                : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, phased_kernel<float, false>, kThreads, 0);
    return e == cudaSuccess && n > 0 ? n : 1;
}

cudaError_t launch_segmented_fp32(int64_t total, cudaStream_t s, const SegmentArgs& a) {
    if (total <= 0) return cudaSuccess;
    const int64_t threads = total * kSegments;
    segmented_vanilla_kernel<kSegments>
        <<<unsigned((threads + kSegmentThreads - 1) / kSegmentThreads), kSegmentThreads, 0, s>>>(a);
    return cudaGetLastError();
}

template <int MODEL>
static cudaError_t straight_one(int64_t total, size_t smem, cudaStream_t s, const StraightArgs& a,
                                const kgpu_model& m, const double* lv) {
    auto k = straight_path_kernel<MODEL>;
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
    if (e != cudaSuccess) return e;
    k<<<unsigned((total + kStraightThreads - 1) / kStraightThreads), kStraightThreads, smem, s>>>(a, m, lv);
    return cudaGetLastError();
}

cudaError_t launch_straight_fp32(int model, int64_t total, size_t smem, cudaStream_t s, const StraightArgs& a,
                                 const kgpu_model& m, const double* lv) {
    if (total <= 0) return cudaSuccess;
    switch (model) {
        case KGPU_MODEL_BSM: return straight_one<KGPU_MODEL_BSM>(total, smem, s, a, m, lv);
        case KGPU_MODEL_HESTON: return straight_one<KGPU_MODEL_HESTON>(total, smem, s, a, m, lv);
        default: return straight_one<KGPU_MODEL_LOCAL_VOL>(total, smem, s, a, m, lv);
    }
}

cudaError_t launch_sobol_high_t(const SobolTables& t, int blocks, uint32_t* out, cudaStream_t s) {
    if (blocks <= 0 || t.dims <= 0) return cudaSuccess;
    sobol_high_table_t_kernel<<<dim3(unsigned((blocks + 255) / 256), unsigned(t.dims)), 256, 0, s>>>(t, blocks, out);
    return cudaGetLastError();
}

cudaError_t launch_compile_arrays_fp32(const RawBook& b, StepT<float>* steps, EventT<float>* events,
                                       IntervalT<float>* intervals, DailyT<float>* daily,
                                       cudaStream_t s) {
    compile_arrays_fp32_kernel<<<1024, 256, 0, s>>>(b, steps, events, intervals, daily);
    return cudaGetLastError();
}
#endif

cudaError_t KGPU_CAT(launch_pcg_normals_, PRECISION)(uint64_t seed, uint64_t block, uint64_t first,
                                                     int64_t count, double* out, cudaStream_t s) {
    if (count <= 0) return cudaSuccess;
    pcg_normals_kernel<<<unsigned((count + 255) / 256), 256, 0, s>>>(seed, block, first, count, out);
    return cudaGetLastError();
}

cudaError_t KGPU_CAT(launch_sobol_points_, PRECISION)(const SobolTables& t, int dim, uint64_t first,
                                                      int64_t count, uint64_t* bits,
                                                      double* normals, cudaStream_t s) {
    if (count <= 0) return cudaSuccess;
    sobol_points_kernel<<<unsigned((count + 255) / 256), 256, 0, s>>>(t, dim, first, count, bits,
                                                                      normals);
    return cudaGetLastError();
}

template <bool SOBOL, bool PAIRS>
static cudaError_t shared_one(int ctas, int chunks, size_t smem, cudaStream_t s, const SharedArgs<REAL>& a) {
    auto k = shared_grid_kernel<REAL, SOBOL, PAIRS>;
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
    if (e != cudaSuccess) return e;
    k<<<dim3(unsigned(ctas), unsigned(chunks)), kSharedThreads, smem, s>>>(a);
    return cudaGetLastError();
}

cudaError_t KGPU_CAT(launch_shared_grid_, PRECISION)(bool sobol, int ctas, int chunks, size_t smem,
                                                     cudaStream_t s, const SharedArgs<REAL>& a) {
    if (a.antithetic)
        return sobol ? shared_one<true, true>(ctas, chunks, smem, s, a) : shared_one<false, true>(ctas, chunks, smem, s, a);
    return sobol ? shared_one<true, false>(ctas, chunks, smem, s, a) : shared_one<false, false>(ctas, chunks, smem, s, a);
}

int KGPU_CAT(shared_grid_occupancy_, PRECISION)(bool sobol, size_t smem) {
    auto k = sobol ? shared_grid_kernel<REAL, true, false> : shared_grid_kernel<REAL, false, false>;
    if (cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)) != cudaSuccess) return 1;
    int n = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k, kSharedThreads, smem) != cudaSuccess) return 1;
    return n > 0 ? n : 1;
}

#if !KGPU_FP32_UNIT
cudaError_t launch_shared_merge(const double* partials, int ctas, int lanes, double* out, cudaStream_t s) {
    shared_merge_kernel<<<lanes, 32, 0, s>>>(partials, ctas, lanes, out);
    return cudaGetLastError();
}
#endif

}  // namespace kgpu
