// qdg_fdkin.cu -- the kinetic operators that are not diagonal in k:
//
// * OGridNablaSq with method="HOFD" (Diff.cpp:203-218 -> HOFD::Diff over all
//   dimensions, src/qdlib/HOFD.h:124-176), and OGridHOFD (HOFD::Diff along
//   each dimension, HOFD.h:188-211, 372-433): a central finite-difference
//   stencil, one thread per point and state, neighbours read through L1/L2
//   (a few hundred bytes per point at order 8);
// * OGridGMat (src/qdlib/OGridGMat.cpp:313-386): -1/2 sum_ij d/dx_j G_ij d/dx_i
//   with FFT first derivatives, as two launches of shared-memory line passes
//   (the kinetic pass's tiles and transforms).  The reference adds one
//   derivative per element (i, j); the sum over i is taken before the
//   derivative along j here (the derivative is linear), which leaves nd + nd
//   line passes instead of nd + nd^2.
#include <cuda_runtime.h>

#include "qdg_kernels.cuh"

namespace qdg {

// QDng's neighbour rule for point i along a dimension of stride lo and size
// N (HOFD.h:151-169), lrep = i / N:
//   above: i + k lo while (i + k lo) / N == lrep, weight cf[o2 - k];
//   below: (N + i - k lo) mod N while (N + k lo) / N == lrep + 1;
//   pbc:   (i + k lo) mod N and (N + i - k lo) mod N for every k.
// On one dimension: neighbours above the grid are dropped and those below it
// wrap to its top end.  Each index formed is inside [0, npts): above, the
// loop condition keeps it below (lrep + 1) N <= npts; below, it implies
// k lo < (lrep + 1) N <= N + i, so N + i - k lo > 0; pbc is one-dimensional,
// where k <= o2 < N.
template <typename T>
__global__ void __launch_bounds__(256) fd_kinetic_kernel(FdArgs<T> a) {
  __shared__ double cf[kMaxFdHalf + 1];
  __shared__ double h[kMaxStates][4];
  if (a.done != nullptr && *a.done) return;
  for (int k = threadIdx.x; k <= a.o2; k += blockDim.x) cf[k] = a.cf[k];
  for (int k = threadIdx.x; k < kMaxStates * 4; k += blockDim.x) h[k / 4][k % 4] = a.h[k / 4][k % 4];
  __syncthreads();
  const cplx<T> *phi = a.dyn ? a.bufs[(a.cs->i + 1) & 1] : a.phi;
  const long long npts = a.npts;
  const long long total = npts * a.S;
  const int o2 = a.o2;
  for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < total;
       g += (long long)gridDim.x * blockDim.x) {
    const int s = (int)(g / npts);
    const long long i = g - (long long)s * npts;
    const cplx<T> *x = phi + (long long)s * npts;
    cplx<T> D = mk<T>(0, 0);
    for (int d = 0; d < a.nd; ++d) {
      const double hd = h[s][d];
      if (hd == 0.0) continue;
      const long long N = a.n[d], lo = a.lo[d];
      cplx<T> v = cmulr(ld(x + i), (T)cf[o2]);
      if (a.mode == 1) {
        // the point's coordinate along d; neighbours past the ends are zero or wrap
        const long long c = (i / lo) % N;
        for (int k = 1; k <= o2; ++k) {
          cplx<T> lw = mk<T>(0, 0), up = mk<T>(0, 0);
          if (c - k >= 0) lw = ld(x + i - k * lo);
          else if (a.pbc) lw = ld(x + i + (N - k) * lo);
          if (c + k < N) up = ld(x + i + k * lo);
          else if (a.pbc) up = ld(x + i + (k - N) * lo);
          v = v + cmulr(lw + cmulr(up, (T)a.df), (T)cf[o2 - k]);
        }
        D = D + cmulr(v, (T)hd);
        continue;
      }
      const long long lrep = i / N;
      if (a.pbc) {
        long long step = lo;
        for (int j = o2 - 1; j >= 0; --j) {
          v = v + cmulr(ld(x + (i + step) % N), (T)cf[j]);
          v = v + cmulr(ld(x + (N + i - step) % N), (T)cf[j]);
          step += lo;
        }
      } else {
        long long step = i + lo;
        for (int j = o2 - 1; j >= 0 && step / N == lrep; --j) {
          v = v + cmulr(ld(x + step), (T)cf[j]);
          step += lo;
        }
        step = i - lo;
        for (int j = o2 - 1; j >= 0 && (N + i - step) / N == lrep + 1; --j) {
          v = v + cmulr(ld(x + (N + step) % N), (T)cf[j]);
          step -= lo;
        }
      }
      D = D + cmulr(v, (T)hd);
    }
    st(a.out + g, D);
  }
}

// Work items (dimension, line tile, state) as in the kinetic pass.  Pass 0
// loads phi; pass 1 loads sum_i G_ij D_i at every point of the tile (G_ij
// from the lower triangle) and stores zeros for states without a G-matrix.
// The multiplier of line index q is i q kmul (Kspace::Init1Dddx order,
// src/qdlib/Kspace.cpp:64-88: the Nyquist index of an even line negative).
template <typename T>
__global__ void __launch_bounds__(256) gmat_pass_kernel(GmatArgs<T> a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  if (a.done != nullptr && *a.done) return;
  const cplx<T> *phi = a.dyn ? a.bufs[(a.cs->i + 1) & 1] : a.phi;
  const long long nitems = a.item_start[a.nd];
  const long long npts = a.npts;
  int cur_dim = -1;
  cplx<T> *tws = reinterpret_cast<cplx<T> *>(smem_raw);
  for (long long item = blockIdx.x; item < nitems; item += gridDim.x) {
    int d = 0;
    while (item >= a.item_start[d + 1]) ++d;
    const DimPass<T> &g = a.dp[d];
    const int N = g.N, TW = g.TW;
    const int LS = lstride(N);
    cplx<T> *b0 = tws + N;
    cplx<T> *b1 = b0 + line_buf_elems(N, TW);
    if (d != cur_dim) {
      __syncthreads();
      for (int i = threadIdx.x; i < N; i += blockDim.x) tws[i] = g.tw[i];
      cur_dim = d;
    }
    const long long local = item - a.item_start[d];
    const long long tile = local / a.S;
    const int s = (int)(local - tile * a.S);
    const long long hi = tile / g.tiles_per_hi;
    const long long base = hi * g.hi_stride + (tile - hi * g.tiles_per_hi) * TW;
    const int tileN = TW * N;
    const long long so = (long long)s * npts;
    if (a.gbase[s] < 0) {  // no G-matrix on this state (uniform over the block)
      if (a.pass == 1)
        for (int idx = threadIdx.x; idx < tileN; idx += blockDim.x) {
          int w, i;
          tile_coord(idx, TW, N, g.es, w, i);
          st(a.P[d] + so + base + (long long)w * g.ls + (long long)i * g.es, mk<T>(0, 0));
        }
      continue;
    }
    __syncthreads();
    for (int idx = threadIdx.x; idx < tileN; idx += blockDim.x) {
      int w, i;
      tile_coord(idx, TW, N, g.es, w, i);
      const long long p = base + (long long)w * g.ls + (long long)i * g.es;
      cplx<T> v;
      if (a.pass == 0) {
        v = ld(phi + so + p);
      } else {
        v = mk<T>(0, 0);
        for (int k = 0; k < a.nd; ++k) {
          const int r = k > d ? k : d, c = k > d ? d : k;
          const int e = r * (r + 1) / 2 + c;
          if (!((a.gmask[s] >> e) & 1u)) continue;
          v = v + cmulr(ld(a.D[k] + so + p), a.grids[(a.gbase[s] + e) * npts + p]);
        }
      }
      b0[lidx(w, i, LS)] = v;
    }
    __syncthreads();
    const int cur = fft_lines<T>(b0, b1, g.rp, TW, tws, -1);
    cplx<T> *bc = cur ? b1 : b0;
    const double km = a.kmul[d];
    for (int idx = threadIdx.x; idx < tileN; idx += blockDim.x) {
      const int w = idx / N, i = idx - w * N;
      const int q = i < (N + 1) / 2 ? i : i - N;
      const T m = (T)(km * (double)q);
      const int x = lidx(w, i, LS);
      const cplx<T> v = bc[x];
      bc[x] = mk<T>(-v.im * m, v.re * m);
    }
    __syncthreads();
    const int cur2 = fft_lines<T>(bc, cur ? b0 : b1, g.rp, TW, tws, +1);
    const cplx<T> *res = cur2 ? (cur ? b0 : b1) : bc;
    cplx<T> *dst = (a.pass == 0 ? a.D[d] : a.P[d]) + so;
    for (int idx = threadIdx.x; idx < tileN; idx += blockDim.x) {
      int w, i;
      tile_coord(idx, TW, N, g.es, w, i);
      st(dst + base + (long long)w * g.ls + (long long)i * g.es, res[lidx(w, i, LS)]);
    }
    __syncthreads();
  }
}

template <typename T>
cudaError_t launch_fd_kinetic(const FdArgs<T> &a, int grid, cudaStream_t st) {
  add_launches(1);
  fd_kinetic_kernel<T><<<grid, 256, 0, st>>>(a);
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch_gmat_pass(const GmatArgs<T> &a, int grid, int block, size_t smem, cudaStream_t st) {
  void *k = (void *)gmat_pass_kernel<T>;
  if (smem > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
  }
  void *args[] = {(void *)&a};
  add_launches(1);
  return cudaLaunchKernel(k, dim3(grid), dim3(block), args, smem, st);
}

template <typename T>
int gmat_max_blocks(int block, size_t smem) {
  void *k = (void *)gmat_pass_kernel<T>;
  if (smem > 48 * 1024) cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  int nb = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k, block, smem) != cudaSuccess) return 1;
  return nb > 0 ? nb : 1;
}

template cudaError_t launch_fd_kinetic<double>(const FdArgs<double> &, int, cudaStream_t);
template cudaError_t launch_fd_kinetic<float>(const FdArgs<float> &, int, cudaStream_t);
template cudaError_t launch_gmat_pass<double>(const GmatArgs<double> &, int, int, size_t, cudaStream_t);
template cudaError_t launch_gmat_pass<float>(const GmatArgs<float> &, int, int, size_t, cudaStream_t);
template int gmat_max_blocks<double>(int, size_t);
template int gmat_max_blocks<float>(int, size_t);

}  // namespace qdg
