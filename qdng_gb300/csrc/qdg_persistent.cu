// qdg_persistent.cu -- launch of the persistent Chebyshev step kernel.
//
// The kernel itself is qdg_step.cuh; its instantiations live in one
// translation unit per bulk type and grid rank (qdg_step_*.cu).  This file
// picks the instantiation of a plan (bulk type, states, grid rank) and
// launches it cooperatively, so every block is resident and the kernel's
// grid barriers are legal.
#include <cuda_runtime.h>

#include "qdg_kernels.cuh"

namespace qdg {

void *step_kernel_f64_1(int S);
void *step_kernel_f64_2(int S);
void *step_kernel_f64_34(int S, int nd);
void *step_kernel_df_2(int S);
void *step_kernel_df_34(int S, int nd);
void *step_kernel_f32_1(int S);
void *step_kernel_f32_2(int S);
void *step_kernel_f32_34(int S, int nd);

static void *step_ptr(int bulk, int S, int nd) {
  if (bulk == BULK_F32) return nd == 1 ? step_kernel_f32_1(S) : nd == 2 ? step_kernel_f32_2(S) : step_kernel_f32_34(S, nd);
  // one-dimensional grids compute in binary64 in both FP64 forms
  if (nd == 1) return step_kernel_f64_1(S);
  if (bulk == BULK_DF64) return nd == 2 ? step_kernel_df_2(S) : step_kernel_df_34(S, nd);
  return nd == 2 ? step_kernel_f64_2(S) : step_kernel_f64_34(S, nd);
}

int cheby_step_max_blocks(int bulk, int S, int nd, int block, size_t smem) {
  void *k = step_ptr(bulk, S, nd);
  if (smem > 48 * 1024 && cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
    return 0;
  int nb = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k, block, smem) != cudaSuccess) return 0;
  return nb;
}

template <typename T>
cudaError_t launch_cheby_step(const StepArgs<T> &a, int grid, int block, size_t smem, cudaStream_t st) {
  void *k = step_ptr(a.bulk, a.S, a.nd);
  if (smem > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
  }
  void *args[] = {(void *)&a};
  add_launches(1);
  return cudaLaunchCooperativeKernel(k, dim3(grid), dim3(block), args, smem, st);
}

template cudaError_t launch_cheby_step<double>(const StepArgs<double> &, int, int, size_t, cudaStream_t);
template cudaError_t launch_cheby_step<float>(const StepArgs<float> &, int, int, size_t, cudaStream_t);

}  // namespace qdg
