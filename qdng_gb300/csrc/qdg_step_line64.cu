// qdg_step_line64.cu -- the binary64 Chebyshev step of one one-dimensional
// line on a thread-block cluster, one real component per thread.
//
// On GB300 a binary64 warp instruction occupies the SM sub-partition's FP64
// pipe for the same time whether 1 or 32 of its lanes are active, so a
// term's latency is the number of FP64 warp instructions that the busiest
// sub-partition issues.  This kernel therefore spreads every phase of a term
// over all lanes of C blocks (C = 16, or 8 where a cluster of 16 cannot be
// scheduled), 2M threads per block for the M = N / C points of the block:
//
//  * FFT stages are radix-2 Stockham stages in which each thread forms ONE
//    real component of ONE butterfly output: y = a +- w b costs two fused
//    multiply-adds, y.re = a.re + (+-w.re) b.re + (-+w.im) b.im (or the
//    imaginary analogue), with the signed twiddle parts held in registers
//    for the whole step.  The first two stages of every transform have
//    twiddles 1 and -i and cost one instruction.
//  * The point work (potential, offset, recurrence, psi update, norm) runs
//    one thread per component of a point; phi_{n-1}, phi_{n-2} and psi stay
//    in registers for the whole step.
//
// The N = C x M factorisation of the DFT (Bailey's four-step form) splits a
// transform into local M-point transforms and C-point transforms across the
// cluster (block c holds the points n = c + C m):
//
//   forward:  Y_c[k2] = sum_m x[c + C m] W_M^{m k2}                  (local)
//   columns:  block q owns k2 in [q B, q B + B), B = M / C; it gathers
//             Y_c[k2] W_N^{c k2} from every block's shared memory, forms
//             the C-point DFT over c (k = k2 + M k1), multiplies by the
//             kinetic table T(k) and takes the inverse C-point DFT -> Z
//   inverse:  block c gathers Z[c][k2] W_N^{-c k2} from the owners and
//             takes the inverse M-point transform: (T x)[c + C m].
//
// T carries the series factor f and 1/N, the potential the factor f, and the
// energy offset enters as -f offset in value and residual (the pre-scaled
// form of the other step kernels).  Two cluster barriers per term; the norm
// partials of a term (one per warp) are read by warp 0 of every block after
// the next term's first cluster barrier and summed in the same order in
// every block, so all blocks take the reference's series cut
// (OCheby.cpp:178-182, 285-289) in the same term.
#include <cooperative_groups.h>
#include <cuda_runtime.h>
#include <math.h>

#include "qdg_kernels.cuh"

namespace cg = cooperative_groups;

namespace qdg {

namespace {

constexpr unsigned kFull = 0xffffffffu;

// Per-thread constants of one radix-2 stage: write index and the folded
// twiddle factors of the forward direction (the inverse negates Q).
struct Stage2 {
  int io;
  double P, Q;
};

// Stage constants for transforms of length L = 2^LL, nb interleaved
// transforms (element e of transform b at e * nb + b), stage s
// (Ns = 2^s).  comp = out * 2 + part: out 0/1 = a + w b / a - w b,
// part 0/1 = real/imaginary component.
__device__ __forceinline__ Stage2 stage_consts(int s, int rest, int comp, int nb, int N,
                                               const cplx<double> *twN) {
  const int out = comp >> 1, part = comp & 1;
  const int b = rest % nb, j = rest / nb;
  const int Ns = 1 << s;
  const int k = j & (Ns - 1);
  // exp(-2 pi i k / (2 Ns)); exactly 1 and -i in the first two stages
  cplx<double> w = twN[(long long)k * (N >> (s + 1))];
  if (s == 0 || k == 0) w = cplx<double>{1.0, 0.0};
  else if (s == 1) w = cplx<double>{0.0, -1.0};
  const double sg = out ? -1.0 : 1.0;
  Stage2 st;
  st.io = ((((j >> s) << (s + 1)) + k + out * Ns) * nb) + b;
  st.P = sg * w.re;
  st.Q = part ? sg * w.im : -sg * w.im;
  return st;
}

// One stage: X, Y are the real planes (imaginary plane at + PL).  The
// thread reads a (own component) at rest, b (both components) at rest +
// M/2 and writes its component at st.io.  SIGN -1 forward, +1 inverse.
// Stage 0 has w = 1 (Q = 0); stage 1 has w in {1, -i}: either P or Q is
// zero, and the thread reads only the component it needs.
template <int SIGN, int KIND>
__device__ __forceinline__ double stage_val(const double *X, int op, int oq, int ia, int ib, const Stage2 &st) {
  const double a = X[op + ia];
  if constexpr (KIND == 0) {
    return fma(st.P, X[op + ib], a);
  } else if constexpr (KIND == 1) {
    // P != 0 (w = 1): b's own component; else Q != 0 (w = -i): the other one
    if (st.P != 0.0) return fma(st.P, X[op + ib], a);
    return fma(SIGN < 0 ? st.Q : -st.Q, X[oq + ib], a);
  } else {
    return fma(st.P, X[op + ib], fma(SIGN < 0 ? st.Q : -st.Q, X[oq + ib], a));
  }
}

}  // namespace

template <int LM, int LC>
__global__ void __launch_bounds__(2 << LM, 1) cheby_line64_kernel(ClusterStepArgs<double> a) {
  constexpr int M = 1 << LM, C = 1 << LC, NB = M / C, NT = 2 * M, NW = NT / 32;
  constexpr int PL = M + 8;  // plane stride: the imaginary plane starts 64 bytes off the real one's banks
  constexpr int NP = C * NW;  // norm partials per term (one per warp of every block)
  static_assert(NB >= 1 && NP >= 32 && NT <= 1024, "line split out of range");
  extern __shared__ __align__(16) double smd[];
  double *F0 = smd, *F1 = smd + 2 * PL, *Yb = smd + 4 * PL, *Zb = smd + 6 * PL, *wpart = smd + 8 * PL;
  __shared__ int flag_s;
  cg::cluster_group cl = cg::this_cluster();
  const int c = (int)cl.block_rank();
  const int N = a.N;
  const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
  const cplx<double> *twN = a.twN;

  // FFT-stage role: butterfly rest, output component comp
  const int rest = t >> 2, comp = t & 3, fpart = comp & 1;
  const int op = fpart * PL, oq = (1 - fpart) * PL;
  const int ia = rest, ib = rest + M / 2;
  Stage2 sl[LM], sc[LC];
#pragma unroll
  for (int s = 0; s < LM; ++s) sl[s] = stage_consts(s, rest, comp, 1, N, twN);
#pragma unroll
  for (int s = 0; s < LC; ++s) sc[s] = stage_consts(s, rest, comp, NB, N, twN);
  // the kinetic factor of this thread's output of the last forward column stage
  double kt;
  {
    const int e = sc[LC - 1].io, k1 = e / NB, kk = e % NB;
    kt = a.ktab[(long long)M * k1 + c * NB + kk];
  }

  // point role: point e = t / 2 (m in the local transforms), component part
  const int e = t >> 1, part = t & 1;
  // column gather: Y_r[k2] W_N^{r k2}, r = e / NB, k2 = c NB + e % NB
  double G1, G2;
  const double *Yr;
  {
    const int r = e / NB, k2 = c * NB + e % NB;
    const cplx<double> w = twN[((long long)r * k2) % N];
    G1 = part ? w.im : w.re;
    G2 = part ? w.re : -w.im;
    Yr = cl.map_shared_rank(Yb, r) + k2;
  }
  // inverse gather: Z_q[c NB + k2 % NB] W_N^{-c k2}, q = k2 / NB, k2 = e
  double H1, H2;
  const double *Zq;
  {
    const int q = e / NB, kk = e % NB;
    const cplx<double> w = twN[((long long)c * e) % N];
    H1 = w.re;
    H2 = part ? -w.im : w.im;
    Zq = cl.map_shared_rank(Zb, q) + c * NB + kk;
  }

  // the step's state of this thread's component of point n = c + C e
  const long long n = c + (long long)C * e;
  const double *psin = reinterpret_cast<const double *>(a.psi);
  double ps = psin[2 * n + part];
  double xo = ps, xp = psin[2 * n + 1 - part], km2 = 0.0;
  const double V = a.V[n];
  const double soh = a.soff_hi, sol = a.soff_lo;
  const int rt = a.rt;
  const int pq = rt ? 1 - part : part;  // component of H x this thread's bf takes
  const bool neg = rt && part == 0;  // bf = i h: bf.re = -h.im

  // warp 0: the cluster's partials, NP / 32 per lane in (rank, warp) order
  const double *pp[NP / 32];
#pragma unroll
  for (int u = 0; u < NP / 32; ++u) {
    const int g = lane + 32 * u;
    pp[u] = cl.map_shared_rank(wpart, g / NW) + (g % NW);
  }

  double norm0 = 0.0, last = 0.0, norm_last = 0.0;
  int status = 0, used = 2;
  for (int i = 1; i < a.order; ++i) {
    const bool first = i == 1;
    // phi_{i-1} into the forward transform
    F0[part * PL + e] = xo;
    __syncthreads();
    // local forward M-point transform: F0 -> F1 -> ... -> Yb
#pragma unroll
    for (int s = 0; s < LM; ++s) {
      const double *X = (s & 1) ? F1 : F0;
      double *Y = (s == LM - 1) ? Yb : ((s & 1) ? F0 : F1);
      const int kind = s == 0 ? 0 : s == 1 ? 1 : 2;
      double v;
      if (kind == 0) v = stage_val<-1, 0>(X, op, oq, ia, ib, sl[s]);
      else if (kind == 1) v = stage_val<-1, 1>(X, op, oq, ia, ib, sl[s]);
      else v = stage_val<-1, 2>(X, op, oq, ia, ib, sl[s]);
      Y[op + sl[s].io] = v;
      if (s < LM - 1) __syncthreads();
    }
    cl.sync();  // every block's Y is complete; the previous term's partials too

    if (!first && warp == 0) {
      double tsum = 0.0;
#pragma unroll
      for (int u = 0; u < NP / 32; ++u) tsum += *pp[u];
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) tsum += __shfl_down_sync(kFull, tsum, o);
      if (lane == 0) {
        bool done = false;
        if (i == 2) {
          norm0 = last = tsum;  // raw norm of psi before the step
          if (!isfinite(norm0)) { done = true; status = 2; }
        } else {
          used = i;
          if (!isfinite(tsum)) { done = true; status = 2; }
          else if (!a.imag) {
            // OCheby.cpp:179-182
            const double ref = a.diff ? last : norm0;
            if (fabs(ref - tsum) / norm0 < a.prec && a.offim0) done = true;
          } else {
            // OCheby.cpp:286-289
            if (fabs(tsum - norm_last) / norm_last < a.prec) done = true;
            norm_last = tsum;
          }
          last = tsum;
        }
        flag_s = done ? 1 : 0;
      }
    }
    // column gather with the twiddle W_N^{r k2}
    {
      const double yre = Yr[0], yim = Yr[PL];
      F0[part * PL + e] = fma(yre, G1, yim * G2);
    }
    __syncthreads();
    if (!first && flag_s) break;
    // forward C-point transforms over the blocks, kinetic factor, inverse ones
    int cur = 0;
#pragma unroll
    for (int s = 0; s < LC; ++s) {
      const double *X = cur ? F1 : F0;
      double *Y = cur ? F0 : F1;
      const int kind = s == 0 ? 0 : s == 1 ? 1 : 2;
      double v;
      if (kind == 0) v = stage_val<-1, 0>(X, op, oq, ia, ib, sc[s]);
      else if (kind == 1) v = stage_val<-1, 1>(X, op, oq, ia, ib, sc[s]);
      else v = stage_val<-1, 2>(X, op, oq, ia, ib, sc[s]);
      if (s == LC - 1) v *= kt;
      Y[op + sc[s].io] = v;
      __syncthreads();
      cur ^= 1;
    }
#pragma unroll
    for (int s = 0; s < LC; ++s) {
      const double *X = cur ? F1 : F0;
      double *Y = (s == LC - 1) ? Zb : (cur ? F0 : F1);
      const int kind = s == 0 ? 0 : s == 1 ? 1 : 2;
      double v;
      if (kind == 0) v = stage_val<1, 0>(X, op, oq, ia, ib, sc[s]);
      else if (kind == 1) v = stage_val<1, 1>(X, op, oq, ia, ib, sc[s]);
      else v = stage_val<1, 2>(X, op, oq, ia, ib, sc[s]);
      Y[op + sc[s].io] = v;
      if (s < LC - 1) __syncthreads();
      cur ^= 1;
    }
    cl.sync();  // every block's Z is complete
    // inverse gather with the twiddle W_N^{-c k2}
    {
      const double zre = Zq[0], zim = Zq[PL];
      F0[part * PL + e] = fma(part ? zim : zre, H1, (part ? zre : zim) * H2);
    }
    __syncthreads();
    // local inverse M-point transform: F0 -> F1 -> ...
#pragma unroll
    for (int s = 0; s < LM; ++s) {
      const double *X = (s & 1) ? F1 : F0;
      double *Y = (s & 1) ? F0 : F1;
      const int kind = s == 0 ? 0 : s == 1 ? 1 : 2;
      double v;
      if (kind == 0) v = stage_val<1, 0>(X, op, oq, ia, ib, sl[s]);
      else if (kind == 1) v = stage_val<1, 1>(X, op, oq, ia, ib, sl[s]);
      else v = stage_val<1, 2>(X, op, oq, ia, ib, sl[s]);
      Y[op + sl[s].io] = v;
      __syncthreads();
    }
    const double *TX = (LM & 1) ? F1 : F0;
    // point work: H' x = T' x + V' x - f offset x (value and residual)
    const double xq = rt ? xp : xo;
    double h = fma(xq, V, TX[pq * PL + e]);
    h = fma(soh, xq, fma(sol, xq, h));
    double bf = neg ? -h : h;
    const double ai = a.a[i];
    double acc;
    if (first) {
      bf *= 0.5;
      acc = ps * ps;
      km2 = xo;
      xo = bf;
      ps = fma(bf, ai, ps * a.a[0]);
    } else {
      const double k2 = a.imag ? bf - km2 : bf + km2;
      km2 = xo;
      xo = k2;
      ps = fma(ai, k2, ps);
      acc = ps * ps;
    }
    xp = __shfl_xor_sync(kFull, xo, 1);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(kFull, acc, o);
    if (lane == 0) wpart[warp] = acc;
    if (i + 1 == a.order) used = a.order;  // series exhausted
  }
  // no block leaves while another may still read its shared memory
  cl.sync();
  // common phase exp(c0 offset) of all coefficients, psi back to memory
  {
    const double pr = __shfl_xor_sync(kFull, ps, 1);
    const double re = part ? pr : ps, im = part ? ps : pr;
    const cplx<double> ph = a.ph;
    double *pout = reinterpret_cast<double *>(a.psi_out);
    pout[2 * n + part] = part ? fma(re, ph.im, im * ph.re) : fma(re, ph.re, -im * ph.im);
  }
  if (c == 0 && t == 0) {
    a.cs->terms = used;
    a.cs->total += used;
    a.cs->status = status;
    a.cs->norm0 = norm0;
  }
}

namespace {

template <int LM, int LC>
void *line64_ptr() { return (void *)cheby_line64_kernel<LM, LC>; }

void *line64_kernel(int M, int C) {
  if (C == 16) return M == 32 ? line64_ptr<5, 4>() : M == 64 ? line64_ptr<6, 4>() : M == 128 ? line64_ptr<7, 4>() : nullptr;
  if (C == 8) return M == 64 ? line64_ptr<6, 3>() : M == 128 ? line64_ptr<7, 3>() : nullptr;
  return nullptr;
}

size_t line64_smem(int M) { return sizeof(double) * (8 * (size_t)(M + 8) + 64); }

cudaLaunchConfig_t line64_config(void *k, int M, int C, cudaStream_t st, cudaLaunchAttribute *attr) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(C);
  cfg.blockDim = dim3(2 * M);
  cfg.dynamicSmemBytes = line64_smem(M);
  cfg.stream = st;
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = C;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  (void)k;
  return cfg;
}

}  // namespace

// The cluster size for an N-point line: 16 where the device schedules a
// cluster of 16 of these blocks, else 8; 0 when N has no split here.
int line64_cluster_size(int N) {
  for (int C : {16, 8}) {
    if (N % C != 0) continue;
    const int M = N / C;
    void *k = line64_kernel(M, C);
    if (!k) continue;
    if (C > 8 && cudaFuncSetAttribute(k, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) != cudaSuccess) {
      cudaGetLastError();
      continue;
    }
    cudaLaunchAttribute attr[1];
    cudaLaunchConfig_t cfg = line64_config(k, M, C, 0, attr);
    int nc = 0;
    if (cudaOccupancyMaxActiveClusters(&nc, k, &cfg) != cudaSuccess) {
      cudaGetLastError();
      continue;
    }
    if (nc > 0) return C;
  }
  return 0;
}

cudaError_t launch_cheby_line64(const ClusterStepArgs<double> &a, int C, cudaStream_t st) {
  const int M = a.N / C;
  void *k = line64_kernel(M, C);
  if (!k || M * C != a.N) return cudaErrorInvalidValue;
  if (C > 8) {
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
    if (e != cudaSuccess) return e;
  }
  cudaLaunchAttribute attr[1];
  cudaLaunchConfig_t cfg = line64_config(k, M, C, st, attr);
  void *args[] = {(void *)&a};
  add_launches(1);
  return cudaLaunchKernelExC(&cfg, k, args);
}

}  // namespace qdg
