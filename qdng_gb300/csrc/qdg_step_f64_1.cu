// qdg_step_f64_1.cu -- instantiations of the persistent Chebyshev step kernel
// (qdg_step.cuh) for binary64 one-dimensional grids.  One translation unit per bulk type and grid
// rank keeps the library build parallel.
#include "qdg_step.cuh"

namespace qdg {

void *step_kernel_f64_1(int S) { return step_kernel_for<double, double, 1, 1>(S); }

}  // namespace qdg
