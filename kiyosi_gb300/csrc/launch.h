// Host-side launchers of the precision-specific kernel translation units.
#pragma once
#include <cuda_runtime.h>

#include "kernels.cuh"

namespace kgpu {

// Shared-memory bytes of the plain kernel for `dims` Sobol dimensions and a surface.
size_t plain_smem_bytes(int precision, bool sobol, int dims, int lv_values);
size_t persistent_smem_bytes(int precision, bool sobol, int dims, int lv_values);

cudaError_t launch_plain(int precision, int model, bool sobol, int blocks, size_t smem,
                         cudaStream_t stream, const PlainArgs& a, const kgpu_model& m,
                         const double* lv_dev);
cudaError_t launch_persistent(int precision, int model, bool sobol, int blocks, size_t smem,
                              cudaStream_t stream, const PersistentArgs& a, const kgpu_model& m,
                              const double* lv_dev);
// Resident CTAs per SM of the persistent kernel at `smem` bytes.
int persistent_blocks_per_sm(int precision, int model, bool sobol, size_t smem);

// Raw streams (kgpu_pcg_words, kgpu_pcg_normals, kgpu_sobol_points).
cudaError_t launch_pcg_words(uint64_t seed, uint64_t stream_id, uint64_t first, int64_t count,
                             uint32_t* out, cudaStream_t stream);
cudaError_t launch_pcg_normals(int precision, uint64_t seed, uint64_t block, uint64_t first,
                               int64_t count, double* out, cudaStream_t stream);
cudaError_t launch_sobol_points(int precision, const SobolTables& t, int dim, uint64_t first,
                                int64_t count, uint64_t* bits, double* normals,
                                cudaStream_t stream);

}  // namespace kgpu
