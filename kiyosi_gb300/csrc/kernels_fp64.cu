// FP64 kernels.  Compiled with --fmad=false so that every product and sum is rounded
// separately, as in the Rust reference; fma() appears exactly where it calls mul_add.
#define REAL double
#define PRECISION fp64
#define KGPU_FP32_UNIT 0
#include "kernels_impl.cuh"
