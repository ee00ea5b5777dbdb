// qdg_step_df_34.cu -- instantiations of the persistent Chebyshev step kernel
// (qdg_step.cuh) for the double-float bulk (DF64 form) of three- and four-dimensional grids.  One translation unit per bulk type and grid
// rank keeps the library build parallel.
#include "qdg_step.cuh"

namespace qdg {

void *step_kernel_df_34(int S, int nd) {
  return nd == 3 ? step_kernel_for<double, dfl, 3, 1>(S) : step_kernel_for<double, dfl, 4, 1>(S);
}

}  // namespace qdg
