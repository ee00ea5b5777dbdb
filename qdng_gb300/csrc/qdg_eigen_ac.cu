// qdg_eigen_ac.cu -- the device parts of ProgEigen::AutoCorrEF
// (src/ProgEigen.cpp:414-600): the autocorrelation of a stored propagation
// and the Fourier integration of the stored wave functions at the energies of
// the spectrum's peaks.
//
// The propagation psi_0 .. psi_{M-1} stays in HBM as an M x n array (the
// reference keeps it in a WFBuffer); both kernels read it once.
#include <cuda_runtime.h>

#include <algorithm>

#include "qdg_kernels.cuh"

namespace qdg {

// a_s = sum_p conj(psi_s(p)) psi_0(p), one block per step, a fixed
// summation order (thread-strided sums, then the block's shuffle tree)
__global__ void __launch_bounds__(256) step_overlaps_kernel(const cplx<double> *T, long long n, int M,
                                                            cplx<double> *out) {
  __shared__ double red[32];
  for (int s = blockIdx.x; s < M; s += gridDim.x) {
    const cplx<double> *x = T + (long long)s * n;
    double re = 0.0, im = 0.0;
    for (long long p = threadIdx.x; p < n; p += blockDim.x) {
      const cplx<double> a = x[p], b = T[p];
      re = fma(a.re, b.re, fma(a.im, b.im, re));
      im = fma(a.re, b.im, fma(-a.im, b.re, im));
    }
    const double tr = block_sum(re, red);
    __syncthreads();
    const double ti = block_sum(im, red);
    if (threadIdx.x == 0) out[s] = cplx<double>{tr, ti};
    __syncthreads();
  }
}

// out_k(p) = psi_0(p) + sum_{s >= 1} c_k(s) psi_s(p), s ascending as the
// reference accumulates (ProgEigen.cpp:575-579); c_k(s) = exp(i E_k s dt)
__global__ void __launch_bounds__(256) integrate_steps_kernel(const cplx<double> *T, long long n, int M,
                                                              const cplx<double> *C, int K, cplx<double> *out) {
  const long long total = (long long)K * n;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
       i += (long long)gridDim.x * blockDim.x) {
    const int k = (int)(i / n);
    const long long p = i - (long long)k * n;
    const cplx<double> *c = C + (long long)k * M;
    cplx<double> acc = T[p];
    for (int s = 1; s < M; ++s) acc = acc + cmul(T[(long long)s * n + p], c[s]);
    out[i] = acc;
  }
}

cudaError_t launch_step_overlaps(const cplx<double> *T, long long n, int M, cplx<double> *out, int sm_count,
                                 cudaStream_t st) {
  const int grid = std::max(1, std::min(M, 4 * sm_count));
  add_launches(1);
  step_overlaps_kernel<<<grid, 256, 0, st>>>(T, n, M, out);
  return cudaGetLastError();
}

cudaError_t launch_integrate_steps(const cplx<double> *T, long long n, int M, const cplx<double> *C, int K,
                                   cplx<double> *out, int sm_count, cudaStream_t st) {
  const long long items = ((long long)K * n + 255) / 256;
  const int grid = (int)std::max<long long>(1, std::min<long long>(items, 8LL * sm_count));
  add_launches(1);
  integrate_steps_kernel<<<grid, 256, 0, st>>>(T, n, M, C, K, out);
  return cudaGetLastError();
}

}  // namespace qdg
