// qdg_step_f32_34.cu -- instantiations of the persistent Chebyshev step kernel
// (qdg_step.cuh) for the FP32 bulk (mixed form) of three- and four-dimensional grids.  One translation unit per bulk type and grid
// rank keeps the library build parallel.
#include "qdg_step.cuh"

namespace qdg {

void *step_kernel_f32_34(int S, int nd) {
  return nd == 3 ? step_kernel_for<float, float, 3, 2>(S) : step_kernel_for<float, float, 4, 2>(S);
}

}  // namespace qdg
