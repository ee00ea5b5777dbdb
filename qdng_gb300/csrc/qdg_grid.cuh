// qdg_grid.cuh -- grid-wide synchronisation of the persistent step kernels.
//
// A cooperative launch keeps every block resident, so blocks can wait for
// one another.  Every wait is bounded: a block that polls a barrier more than
// kBarrierSpinLimit times raises the error flag and leaves, and every block
// that sees the flag leaves too; the host turns the flag into QDG_ETIMEOUT.
#pragma once

#include <cuda_runtime.h>

#include "qdg_kernels.cuh"

namespace qdg {

__device__ __forceinline__ unsigned int ld_acquire_u32(const unsigned int *p) {
  unsigned int v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

// Sense-free generation barrier over all blocks of the grid.  Returns false
// when any block gave up waiting (then every block leaves the step).
__device__ __forceinline__ bool grid_sync(GridBarrier *b) {
  __shared__ int ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    const unsigned int g = ld_acquire_u32(&b->gen);
    __threadfence();
    const unsigned int arrived = atomicAdd(&b->count, 1u);
    if (arrived == gridDim.x - 1) {
      atomicExch(&b->count, 0u);
      __threadfence();
      atomicAdd(&b->gen, 1u);
    } else {
      unsigned int spins = 0;
      while (ld_acquire_u32(&b->gen) == g) {
        if (++spins > kBarrierSpinLimit) {
          atomicExch(&b->err, 1);
          break;
        }
        if (spins > (1u << 14)) __nanosleep(64);  // tight spin first (a term is ~10-100 us), back off later
      }
    }
    __threadfence();
    ok = *(volatile int *)&b->err == 0;
  }
  __syncthreads();
  return ok != 0;
}

__device__ __forceinline__ unsigned long long gtimer() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Sum of the per-block partials by the first warp, in the same fixed order
// in every block (strided lane sums, then a shuffle tree), so every block
// takes the same series-cut decision; valid on thread 0, no block barrier.
__device__ __forceinline__ double sum_partials(const double *partials, double *) {
  double v = 0.0;
  if (threadIdx.x < 32) {
    for (int i = threadIdx.x; i < (int)gridDim.x; i += 32) v += __ldcg(partials + i);
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  }
  return v;
}

}  // namespace qdg
