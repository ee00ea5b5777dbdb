// qdg_step_f64_2.cu -- instantiations of the persistent Chebyshev step kernel
// (qdg_step.cuh) for binary64 two-dimensional grids.  One translation unit per bulk type and grid
// rank keeps the library build parallel.
#include "qdg_step.cuh"

namespace qdg {

void *step_kernel_f64_2(int S) { return step_kernel_for<double, double, 2, 1>(S); }

}  // namespace qdg
