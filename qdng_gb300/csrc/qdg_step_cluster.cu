// qdg_step_cluster.cu -- the Chebyshev step of a single one-dimensional line
// on a thread-block cluster.
//
// One line of N points (the 1-D Morse benchmark: N = 1024) is too little
// work for one SM to finish a term quickly, and every term depends on the
// previous one, so the line is split over the C = 8 blocks of a cluster.
// Block c owns the points n = c + C m (m < M = N/C) of phi_{n-1},
// phi_{n-2}, psi and the potential for the whole step, in its shared
// memory.  The kinetic part uses the N = C x M factorisation of the DFT:
//
//   forward:  Y_c[k2]  = W_N^{c k2} sum_m x[c + C m] W_M^{m k2}      (local)
//   exchange: block j takes k2 in [j M/C, (j+1) M/C) and forms, per k2,
//             Z[c][k2] = IDFT_C( T(M k1 + k2) DFT_C( Y_.[k2] ) )[c]
//             reading Y_c[k2] from every block's shared memory (DSMEM)
//   inverse:  (T x)[c + C m] = sum_k2 W_M^{-m k2} W_N^{-c k2} Z[c][k2]
//             with Z[c][.] read back from the blocks that formed it.
//
// T already carries the series factor f and 1/N (the pre-scaled form of
// the step kernels), and the point work is that of the other step kernels:
// phi_n = (i) (T' + V') phi_{n-1} - f offset phi_{n-1} +- phi_{n-2}, psi +=
// a_n phi_n, norm of psi.  Two cluster barriers per term: one before the
// exchange (Y written), one before the inverse gathers (Z written); the
// norm partials of a term are read after the next term's first barrier,
// and every block sums them in the same order, so all blocks take the
// reference's series cut (OCheby.cpp:178-182, 285-289) in the same term.
// Cluster barriers are hardware barriers among co-scheduled blocks; every
// block runs the same sequence of them.
#include <cooperative_groups.h>
#include <cuda_runtime.h>
#include <math.h>

#include "qdg_kernels.cuh"

namespace cg = cooperative_groups;

namespace qdg {

template <typename T>
struct ClusterSmem {
  cplx<T> *phm1, *phm2, *buf0, *buf1, *Y, *Z, *twM;
  cplx<double> *psi;
  T *V;
  double *part;
};

template <typename T>
__device__ __forceinline__ cplx<T> soffadd(cplx<T> h, cplx<T> x, T hi, T lo) {
  return mk(fma(hi, x.re, fma(lo, x.re, h.re)), fma(hi, x.im, fma(lo, x.im, h.im)));
}

// T' x for the cluster's line: x in sm.phm1 (block c holds x[c + C m]),
// result into sm.buf0 at lpos(m) (natural order m).  Leaves a cluster
// barrier behind the exchange; the caller reads the previous term's
// partials after the first one (before the exchange).
template <typename T, int C>
__device__ void kinetic_cluster(const ClusterStepArgs<T> &a, const ClusterSmem<T> &sm, cg::cluster_group &cl,
                                const cplx<T> *x, int c) {
  const int M = a.M, N = a.N;
  auto twf = [&sm](int m) { return sm.twM[m]; };
  // local forward transform of x[c + C m] (m = 0..M-1): buf0 -> ... -> Y
  for (int m = threadIdx.x; m < M; m += blockDim.x) sm.buf0[lpos(m)] = x[m];
  __syncthreads();
  cplx<T> *bb[2] = {sm.buf0, sm.buf1};
  int cur = 0, Ns = 1;
  for (int s = 0; s < a.rp.nstages; ++s) {
    cplx<T> *dst = bb[cur ^ 1];
    const bool last = s + 1 == a.rp.nstages;
    const int ns = Ns;
    if (!last) {
      stage_s_any<T, -1>(a.rp.radix[s], bb[cur], [dst](int, int i, cplx<T> v) { dst[lpos(i)] = v; }, M, 1, ns,
                         false, twf);
    } else {
      // the twiddle W_N^{c k2} on the way out
      const cplx<T> *twN = a.twN;
      cplx<T> *Y = sm.Y;
      stage_s_any<T, -1>(a.rp.radix[s], bb[cur],
                         [Y, twN, c, N](int, int k2, cplx<T> v) {
                           Y[k2] = twmul<-1>(v, twN[(long long)c * k2 % N]);
                         },
                         M, 1, ns, false, twf);
    }
    __syncthreads();
    cur ^= 1;
    Ns *= a.rp.radix[s];
  }
  cl.sync();  // every block's Y is complete
}

// The exchange: for the k2 this block owns, Z[c'][k2] = IDFT_C(T' DFT_C(Y_.[k2]))[c'].
template <typename T, int C>
__device__ void exchange_cluster(const ClusterStepArgs<T> &a, const ClusterSmem<T> &sm, cg::cluster_group &cl,
                                 int c) {
  const int M = a.M, KB = M / C;
  for (int j = threadIdx.x; j < KB; j += blockDim.x) {
    const int k2 = c * KB + j;
    cplx<T> v[C];
#pragma unroll
    for (int r = 0; r < C; ++r) v[r] = cl.map_shared_rank(sm.Y, r)[k2];
    dft8s<-1>(v);  // v[k1] = X[M k1 + k2]
#pragma unroll
    for (int k1 = 0; k1 < C; ++k1) {
      // the table holds f kfac min(k, N - k)^2 at k = M k1 + k2
      v[k1] = cmulr(v[k1], __ldg(a.ktab + M * k1 + k2));
    }
    dft8s<1>(v);  // v[c'] = Z[c'][k2]
#pragma unroll
    for (int r = 0; r < C; ++r) sm.Z[r * KB + j] = v[r];
  }
  cl.sync();  // every block's Z is complete
}

// The inverse: gather Z[c][k2] for all k2, twiddle W_N^{-c k2}, inverse
// M-point transform; T'x[c + C m] ends in the buffer returned.
template <typename T, int C>
__device__ cplx<T> *inverse_cluster(const ClusterStepArgs<T> &a, const ClusterSmem<T> &sm, cg::cluster_group &cl,
                                    int c) {
  const int M = a.M, N = a.N, KB = M / C;
  for (int k2 = threadIdx.x; k2 < M; k2 += blockDim.x) {
    const cplx<T> z = cl.map_shared_rank(sm.Z, k2 / KB)[c * KB + (k2 % KB)];
    sm.buf0[lpos(k2)] = twmul<1>(z, a.twN[(long long)c * k2 % N]);
  }
  __syncthreads();
  auto twf = [&sm](int m) { return sm.twM[m]; };
  cplx<T> *bb[2] = {sm.buf0, sm.buf1};
  int cur = 0, Ns = 1;
  for (int s = 0; s < a.rp.nstages; ++s) {
    cplx<T> *dst = bb[cur ^ 1];
    stage_s_any<T, 1>(a.rp.radix[s], bb[cur], [dst](int, int i, cplx<T> v) { dst[lpos(i)] = v; }, M, 1, Ns, false,
                      twf);
    __syncthreads();
    cur ^= 1;
    Ns *= a.rp.radix[s];
  }
  return bb[cur];
}

template <typename T, int C>
__global__ void __launch_bounds__(256, 1) cheby_step_cluster_kernel(ClusterStepArgs<T> a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ double red[32];
  __shared__ double tot_s;
  cg::cluster_group cl = cg::this_cluster();
  const int c = (int)cl.block_rank();
  const int M = a.M;
  const int LS = lstride(M);
  ClusterSmem<T> sm;
  cplx<T> *p = reinterpret_cast<cplx<T> *>(smem_raw);
  sm.phm1 = p; p += M;
  sm.phm2 = p; p += M;
  sm.buf0 = p; p += LS;
  sm.buf1 = p; p += LS;
  sm.Y = p; p += M;
  sm.Z = p; p += M;
  sm.twM = p; p += M;
  sm.psi = reinterpret_cast<cplx<double> *>(p);
  sm.V = reinterpret_cast<T *>(sm.psi + M);
  __shared__ double part[8];
  sm.part = part;

  // the block's points: psi, phi_0 = psi, the scaled potential f V, twiddles of M
  for (int m = threadIdx.x; m < M; m += blockDim.x) {
    const long long n = c + (long long)C * m;
    const cplx<double> ps = ld(a.psi + n);
    sm.psi[m] = ps;
    sm.phm1[m] = ccast<T>(ps);
    sm.V[m] = a.V[n];
    sm.twM[m] = a.twN[(long long)m * C];
  }
  const T soh = (T)a.soff_hi, sol = (T)(((double)a.soff_hi - (double)(T)a.soff_hi) + a.soff_lo);
  __syncthreads();

  double norm0 = 0.0, last = 0.0, norm_last = 0.0;
  bool done = false;
  int status = 0, used = 2;
  // term i = 1 is the first (phi_1 = fac/2 (H - E) phi_0), then phi_i
  for (int i = 1; i < a.order; ++i) {
    const bool first = i == 1;
    kinetic_cluster<T, C>(a, sm, cl, sm.phm1, c);
    if (!first) {
      // the previous term's norm: every block sums the partials in block
      // order, so every block takes the same decision here
      if (threadIdx.x == 0) {
        double t = 0.0;
        for (int r = 0; r < C; ++r) t += cl.map_shared_rank(sm.part, r)[0];
        tot_s = t;
      }
      __syncthreads();
      const double tot = tot_s;
      if (i == 2) {
        norm0 = last = tot;  // raw norm of psi before the step
        if (!isfinite(norm0)) { done = true; status = 2; }
      } else {
        used = i;
        if (!isfinite(tot)) { done = true; status = 2; }
        else if (!a.imag) {
          // OCheby.cpp:179-182 (mixed precision: change against the previous term)
          const double ref = a.diff ? last : norm0;
          if (fabs(ref - tot) / norm0 < a.prec && a.offim0) done = true;
        } else {
          // OCheby.cpp:286-289
          if (fabs(tot - norm_last) / norm_last < a.prec) done = true;
          norm_last = tot;
        }
        last = tot;
      }
      if (done) break;
    }
    exchange_cluster<T, C>(a, sm, cl, c);
    const cplx<T> *tx = inverse_cluster<T, C>(a, sm, cl, c);
    // point work on the block's points
    const double ai = a.a[i];
    double acc = 0.0;
    for (int m = threadIdx.x; m < M; m += blockDim.x) {
      const cplx<T> x = sm.phm1[m];
      cplx<T> h = tx[lpos(m)];
      h.re = fma(x.re, sm.V[m], h.re);
      h.im = fma(x.im, sm.V[m], h.im);
      h = soffadd(h, x, soh, sol);
      cplx<T> bf = a.rt ? mk(-h.im, h.re) : h;
      cplx<double> ps = sm.psi[m];
      if (first) {
        bf = cmulr(bf, (T)0.5);
        acc += cabs2(ps);
        sm.phm2[m] = x;   // phi_0 becomes phi_{i-2} of the next term
        sm.phm1[m] = bf;  // phi_1
        ps = mk(fma((double)bf.re, ai, ps.re * a.a[0]), fma((double)bf.im, ai, ps.im * a.a[0]));
      } else {
        const cplx<T> km2 = sm.phm2[m];
        const cplx<T> k2 = a.imag ? bf - km2 : bf + km2;
        sm.phm2[m] = x;
        sm.phm1[m] = k2;
        ps.re = fma(ai, (double)k2.re, ps.re);
        ps.im = fma(ai, (double)k2.im, ps.im);
        acc = fma(ps.re, ps.re, fma(ps.im, ps.im, acc));
      }
      sm.psi[m] = ps;
    }
    const double t = block_sum(acc, red);
    if (threadIdx.x == 0) sm.part[0] = t;
    __syncthreads();
    if (i + 1 == a.order) used = a.order;  // series exhausted
  }
  // no block leaves while another may still read its shared memory
  cl.sync();
  // common phase exp(c0 offset) of all coefficients, then psi back to HBM
  for (int m = threadIdx.x; m < M; m += blockDim.x) {
    const long long n = c + (long long)C * m;
    st(a.psi_out + n, cmul(sm.psi[m], a.ph));
  }
  if (c == 0 && threadIdx.x == 0) {
    a.cs->terms = used;
    a.cs->total += used;
    a.cs->status = status;
    a.cs->norm0 = norm0;
  }
}

template <typename T>
size_t cluster_step_smem(int M) {
  const size_t LS = (size_t)lstride(M);
  return sizeof(cplx<T>) * (5 * (size_t)M + 2 * LS) + sizeof(cplx<double>) * M + sizeof(T) * M + 64;
}

template <typename T>
cudaError_t launch_cheby_step_cluster(const ClusterStepArgs<T> &a, cudaStream_t st) {
  void *k = (void *)cheby_step_cluster_kernel<T, 8>;
  const size_t smem = cluster_step_smem<T>(a.M);
  if (smem > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
  }
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(8);
  cfg.blockDim = dim3(256);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = 8;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  add_launches(1);
  return cudaLaunchKernelEx(&cfg, cheby_step_cluster_kernel<T, 8>, a);
}

template cudaError_t launch_cheby_step_cluster<double>(const ClusterStepArgs<double> &, cudaStream_t);
template cudaError_t launch_cheby_step_cluster<float>(const ClusterStepArgs<float> &, cudaStream_t);
template size_t cluster_step_smem<double>(int);
template size_t cluster_step_smem<float>(int);

}  // namespace qdg
