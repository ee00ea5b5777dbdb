// qdg_step_f32_2.cu -- instantiations of the persistent Chebyshev step kernel
// (qdg_step.cuh) for the FP32 bulk (mixed form) of two-dimensional grids.  One translation unit per bulk type and grid
// rank keeps the library build parallel.
#include "qdg_step.cuh"

namespace qdg {

void *step_kernel_f32_2(int S) { return step_kernel_for<float, float, 2, 2>(S); }

}  // namespace qdg
