// Host-side launchers of the precision-specific kernel translation units.
#pragma once
#include <cuda_runtime.h>

#include "kernels.cuh"
#include "phased.cuh"
#include "segmented.cuh"
#include "straight.cuh"
#include "shared_grid.cuh"

namespace kgpu {

// Shared-memory bytes of the kernels for `dims` Sobol dimensions and a surface.
size_t plain_smem_bytes(int precision, bool sobol, int dims, int lv_values);
size_t persistent_smem_bytes(int precision, bool sobol, int dims, int lv_values);

cudaError_t launch_plain_fp64(int model, bool sobol, int blocks, size_t smem, cudaStream_t s,
                              const PlainArgs<double>& a, const kgpu_model& m, const double* lv);
cudaError_t launch_plain_fp32(int model, bool sobol, int blocks, size_t smem, cudaStream_t s,
                              const PlainArgs<float>& a, const kgpu_model& m, const double* lv);
// `ext`: the book holds a payoff of the extended set (scheduled barriers, continuous
// averages), which runs in its own instantiation so the core kernels keep their
// register allocation.
cudaError_t launch_persistent_fp64(int model, bool sobol, bool ext, int blocks, size_t smem, cudaStream_t s,
                                   const PersistentArgs<double>& a, const kgpu_model& m,
                                   const double* lv);
cudaError_t launch_persistent_fp32(int model, bool sobol, bool ext, int blocks, size_t smem, cudaStream_t s,
                                   const PersistentArgs<float>& a, const kgpu_model& m,
                                   const double* lv);
int persistent_occupancy_fp64(int model, bool sobol, bool ext, size_t smem);
int persistent_occupancy_fp32(int model, bool sobol, bool ext, size_t smem);
cudaError_t launch_compile_contracts_fp64(const kgpu_contract* in, int n, ContractT<double>* out,
                                          cudaStream_t s);
cudaError_t launch_compile_contracts_fp32(const kgpu_contract* in, int n, ContractT<float>* out,
                                          cudaStream_t s);
cudaError_t launch_compile_units_fp64(const kgpu_contract* contracts, int n,
                                      const kgpu_bridge_interval* intervals,
                                      const kgpu_bridge_daily* daily, const uint8_t* flags,
                                      const kgpu_event* events, UnitT<double>* units,
                                      EndT<double>* ends, cudaStream_t s);
cudaError_t launch_compile_units_fp32(const kgpu_contract* contracts, int n,
                                      const kgpu_bridge_interval* intervals,
                                      const kgpu_bridge_daily* daily, const uint8_t* flags,
                                      const kgpu_event* events, UnitT<float>* units,
                                      EndT<float>* ends, cudaStream_t s);
cudaError_t launch_compile_arrays_fp32(const RawBook& b, StepT<float>* steps, EventT<float>* events,
                                       IntervalT<float>* intervals, DailyT<float>* daily,
                                       cudaStream_t s);

// Phase-major schedule of bridged autocallable books (FP32): one launch per bridge
// interval and a final drain launch; the dimension-major Sobol high table it reads.
cudaError_t launch_phased_fp32(int blocks, cudaStream_t s, const PhaseArgs<float, true>& a);
cudaError_t launch_phased_fp32(int blocks, cudaStream_t s, const PhaseArgs<float, false>& a);
int phased_occupancy_fp32(bool sobol);

// Books of BSM vanilla-path contracts, FP32, pseudo-random: kSegments lanes per path.
cudaError_t launch_segmented_fp32(int64_t total, cudaStream_t s, const SegmentArgs& a);

// Books of paths that take every grid step (Asians on fixings, vanilla paths), FP32,
// pseudo-random: one thread per path.  `smem`: the local-volatility surface.
cudaError_t launch_straight_fp32(int model, int64_t total, size_t smem, cudaStream_t s, const StraightArgs& a,
                                 const kgpu_model& m, const double* lv);
cudaError_t launch_sobol_high_t(const SobolTables& t, int blocks, uint32_t* out, cudaStream_t s);

// The lanes of one shared daily grid, path-major, and the merge of their CTA sums.
// `ctas` path tiles x `chunks` lane chunks.
cudaError_t launch_shared_grid_fp64(bool sobol, int ctas, int chunks, size_t smem, cudaStream_t s,
                                    const SharedArgs<double>& a);
cudaError_t launch_shared_grid_fp32(bool sobol, int ctas, int chunks, size_t smem, cudaStream_t s,
                                    const SharedArgs<float>& a);
int shared_grid_occupancy_fp64(bool sobol, size_t smem);
int shared_grid_occupancy_fp32(bool sobol, size_t smem);
cudaError_t launch_shared_merge(const double* partials, int ctas, int lanes, double* out, cudaStream_t s);

// Raw streams (kgpu_pcg_words, kgpu_pcg_normals, kgpu_sobol_points).
cudaError_t launch_pcg_normals_fp64(uint64_t seed, uint64_t block, uint64_t first, int64_t count,
                                    double* out, cudaStream_t s);
cudaError_t launch_pcg_normals_fp32(uint64_t seed, uint64_t block, uint64_t first, int64_t count,
                                    double* out, cudaStream_t s);
cudaError_t launch_sobol_points_fp64(const SobolTables& t, int dim, uint64_t first, int64_t count,
                                     uint64_t* bits, double* normals, cudaStream_t s);
cudaError_t launch_sobol_points_fp32(const SobolTables& t, int dim, uint64_t first, int64_t count,
                                     uint64_t* bits, double* normals, cudaStream_t s);

}  // namespace kgpu
