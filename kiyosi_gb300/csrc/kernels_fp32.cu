// FP32 kernels: single-precision path arithmetic on the reference's integer streams.
#define REAL float
#define PRECISION fp32
#define KGPU_FP32_UNIT 1
#include "kernels_impl.cuh"
