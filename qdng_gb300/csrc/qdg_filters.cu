// qdg_filters.cu -- expectation values of QDng's filter operators
// (FiltersList expec / expeconly, src/FiltersList.cpp:289-308).
//
// ProgPropa renormalises every filter value by <psi|psi> (ProgPropa.cpp:260,
// 276), so each function returns Re <psi|O|psi> / <psi|psi>; the volume
// element cancels and the sums run over the raw grid values.
//
// * point operators (OGridPosition, a potential grid, OGobbler without nip):
//   sum_p w(p) |psi(p)|^2, the weight from a grid or the coordinate;
// * operators diagonal in k along one dimension (GridMomentum = OGridNabla
//   with momentum, the kinetic energy of OGridNablaSq): by Parseval,
//   Re <psi|IFFT m FFT|psi> = sum over the lines of that dimension of
//   sum_k m(k) |FFT psi (k)|^2, with m holding the 1/N of the unnormalised
//   transform pair; each block transforms whole lines in shared memory;
// * OProjection: sum_k |<phi_k|psi>|^2 with the plan's scalar products.
//
// All arithmetic is binary64 in every precision form (the twiddles and the
// weights are uploaded as binary64 tables for the call), and the per-block
// partial sums are added on the host in block order.
#include <cuda_runtime.h>
#include <math.h>

#include "qdg_kernels.cuh"

namespace qdg {

__global__ void __launch_bounds__(256) point_expec_kernel(PointExpecArgs a) {
  __shared__ double red[32];
  double ws = 0.0, ns = 0.0;
  const long long total = a.npts * a.S;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
       i += (long long)gridDim.x * blockDim.x) {
    const long long p = i % a.npts;
    const double m = cabs2(a.psi[i]);
    double w;
    if (a.grid) {
      w = a.grid[p];
    } else {
      w = 0.0;
      for (int d = 0; d < a.nd; ++d) {
        if (a.dim >= 0 && d != a.dim) continue;
        const long long id = (p / a.stride[d]) % a.n[d];
        w += (a.xmin[d] + a.dx[d] * (double)id) * a.scale;
      }
    }
    ws = fma(w, m, ws);
    ns += m;
  }
  const double tw = block_sum(ws, red);
  __syncthreads();
  const double tn = block_sum(ns, red);
  if (threadIdx.x == 0) {
    a.partials[2 * blockIdx.x] = tw;
    a.partials[2 * blockIdx.x + 1] = tn;
  }
}

__global__ void __launch_bounds__(256) spectral_expec_kernel(SpecExpecArgs a) {
  extern __shared__ __align__(16) unsigned char smraw[];
  __shared__ double red[32];
  const int N = a.N, LS = lstride(N);
  cplx<double> *tws = reinterpret_cast<cplx<double> *>(smraw);
  cplx<double> *bb[2] = {tws + N, tws + N + LS};
  for (int i = threadIdx.x; i < N; i += blockDim.x) tws[i] = a.tw[i];
  auto twf = [tws](int m) { return tws[m]; };
  const long long nl = a.npts / N;
  double acc = 0.0;
  for (long long L = blockIdx.x; L < nl * a.S; L += gridDim.x) {
    const long long s = L / nl, l = L - s * nl;
    const long long base = s * a.npts + (l % a.es) + (l / a.es) * a.es * N;
    __syncthreads();
    for (int j = threadIdx.x; j < N; j += blockDim.x) bb[0][lpos(j)] = a.psi[base + (long long)j * a.es];
    __syncthreads();
    int cur = 0, Ns = 1;
    for (int st = 0; st < a.rp.nstages; ++st) {
      cplx<double> *dst = bb[cur ^ 1];
      stage_s_any<double, -1, true>(a.rp.radix[st], bb[cur], [dst](int, int i, cplx<double> v) { dst[lpos(i)] = v; }, N, 1,
                              Ns, false, twf);
      __syncthreads();
      cur ^= 1;
      Ns *= a.rp.radix[st];
    }
    const double *w = a.w + s * N;
    for (int j = threadIdx.x; j < N; j += blockDim.x) acc = fma(w[j], cabs2(bb[cur][lpos(j)]), acc);
  }
  const double t = block_sum(acc, red);
  if (threadIdx.x == 0) a.partials[blockIdx.x] = t;
}

size_t spectral_expec_smem(int N) { return sizeof(cplx<double>) * ((size_t)N + 2 * (size_t)lstride(N)); }

cudaError_t launch_point_expec(const PointExpecArgs &a, int grid, cudaStream_t st) {
  add_launches(1);
  point_expec_kernel<<<grid, 256, 0, st>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_spectral_expec(const SpecExpecArgs &a, int grid, cudaStream_t st) {
  const size_t smem = spectral_expec_smem(a.N);
  if (smem > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(spectral_expec_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
  }
  add_launches(1);
  spectral_expec_kernel<<<grid, 256, smem, st>>>(a);
  return cudaGetLastError();
}

}  // namespace qdg
