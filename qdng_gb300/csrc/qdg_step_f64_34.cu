// qdg_step_f64_34.cu -- instantiations of the persistent Chebyshev step kernel
// (qdg_step.cuh) for binary64 three- and four-dimensional grids.  One translation unit per bulk type and grid
// rank keeps the library build parallel.
#include "qdg_step.cuh"

namespace qdg {

void *step_kernel_f64_34(int S, int nd) {
  return nd == 3 ? step_kernel_for<double, double, 3, 1>(S) : step_kernel_for<double, double, 4, 1>(S);
}

}  // namespace qdg
