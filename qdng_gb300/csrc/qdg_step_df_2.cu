// qdg_step_df_2.cu -- instantiations of the persistent Chebyshev step kernel
// (qdg_step.cuh) for the double-float bulk (DF64 form) of two-dimensional grids.  One translation unit per bulk type and grid
// rank keeps the library build parallel.
#include "qdg_step.cuh"

namespace qdg {

void *step_kernel_df_2(int S) { return step_kernel_for<double, dfl, 2, 1>(S); }

}  // namespace qdg
