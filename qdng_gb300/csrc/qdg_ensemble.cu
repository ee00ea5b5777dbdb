// qdg_ensemble.cu -- many independent wavepackets in one persistent launch.
//
// Each member is a single-state grid Hamiltonian Sum(GridNablaSq, GridPotential,
// GridDipole x laser) on its own 1-D or 2-D grid (QDng's TGPL-IR-Pulse-Cheby
// shape), propagated with the Chebyshev series of OCheby
// (src/qdlib/OCheby.cpp:92-198) with its own order, scaling and offset.
// Members are taken by blocks from a device work queue in descending cost
// (largest first: list scheduling in LPT order), and one block runs a whole
// member for all requested steps: every synchronisation is a block barrier,
// so the launch has no grid-wide waits at all.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <complex>
#include <cstring>
#include <map>
#include <numeric>
#include <string>
#include <vector>

#include "../../include/qdg.h"
#include "qdg_host.h"
#include "qdg_kernels.cuh"

namespace qdg {

// The point work of a term: (h - offset x) times the series factor, with
// the offset and the factor each carried as a rounded value plus its
// rounding residual.  Binary64 needs the residual of the factor only (the
// product offset x is rounded per point); FP32 needs both.  Multiplying
// every point by a rounded constant would scale or shift the series
// argument coherently: a phase error that grows with every time step.
template <typename T>
struct SeriesK {
  cplx<T> oh, ol, fh, fl;
  __device__ __forceinline__ cplx<T> operator()(cplx<T> h, cplx<T> x) const {
    cplx<T> hm;
    if constexpr (sizeof(T) == sizeof(double)) {
      hm = h - cmul(oh, x);
    } else {
      hm.re = fma(-oh.re, x.re, fma(oh.im, x.im, fma(-ol.re, x.re, fma(ol.im, x.im, h.re))));
      hm.im = fma(-oh.re, x.im, fma(-oh.im, x.re, fma(-ol.re, x.im, fma(-ol.im, x.re, h.im))));
    }
    const T sre = hm.re * fl.re - hm.im * fl.im, sim = hm.re * fl.im + hm.im * fl.re;
    return mk<T>(fma(hm.re, fh.re, fma(-hm.im, fh.im, sre)), fma(hm.re, fh.im, fma(hm.im, fh.re, sim)));
  }
};
template <typename T>
__device__ __forceinline__ SeriesK<T> series_k(cplx<double> off, cplx<double> fac, cplx<double> lo) {
  SeriesK<T> k;
  k.oh = ccast<T>(off);
  k.ol = mk<T>((T)(off.re - (double)k.oh.re), (T)(off.im - (double)k.oh.im));
  k.fh = ccast<T>(fac);
  k.fl = mk<T>((T)((fac.re - (double)k.fh.re) + lo.re), (T)((fac.im - (double)k.fh.im) + lo.im));
  return k;
}

struct EnsMember {
  int nd;
  int n[2];
  long long npts;
  long long off;          // first point in the concatenated arrays
  long long tw_off[2];    // twiddles of each dimension (complex elements)
  long long kt_off[2];    // kinetic multipliers of each dimension
  RadixPlan rp[2];
  int lmax[2];            // lines per batch
  int order;
  long long coef_off;     // series coefficients a_i
  cplx<double> offset, fac1, fac, ph;
  cplx<double> fac1_lo, fac_lo;  // rounding residuals of fac1, fac (exact factor = fac + fac_lo)
  double prec;
  long long laser_off;    // -1: no field
  int laser_nt;
  int has_dipole;
  int fast;               // 1-D member kept in shared memory for the whole step
  double kf;              // k^2 multiplier of dimension 0: dk^2 / (2 m) / N
};

// psi of the mixed form as an unevaluated sum hi + lo of two FP32 numbers
struct dfloat { float hi, lo; };

template <typename T>
struct EnsArgs {
  const EnsMember *m;
  const int *order;       // work order (member indices)
  int n;
  int *queue;
  cplx<double> *psi;
  cplx<T> *buf0, *buf1;   // phi_{i-1}, phi_{i-2} (in/out)
  cplx<T> *P0, *P1;       // T_d phi per dimension
  const T *V, *mu;
  const double *lasers;
  const double *coef;
  const cplx<T> *tw;
  const T *ktab;
  long long step0;
  int nsteps;
  int diff;               // mixed precision: differential series cut
  long long *terms;       // per member, accumulated
  int *status;            // per member: 2 = non-finite norm
  dfloat *dfr, *dfi;      // mixed form: psi in double-float during a step (members off the resident path)
  unsigned long long *tl; // per member: start, end (GPU clock, ns) and block of the last run
  int block0;             // number of this launch's first block in the timeline
};

__device__ __forceinline__ unsigned long long ens_clock() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// T_d phi for every dimension of member m: lines in batches of lmax[d].
template <typename T>
__device__ void ens_kinetic(const EnsArgs<T> &a, const EnsMember &m, const cplx<T> *phi, cplx<T> *smem) {
  __shared__ long long lb[64];
  for (int d = 0; d < m.nd; ++d) {
    const int N = m.n[d];
    const long long stride = d == 0 ? 1 : m.n[0];
    const long long nl = m.npts / N;
    const cplx<T> *tw = a.tw + m.tw_off[d];
    const T *kt = a.ktab + m.kt_off[d];
    cplx<T> *dst = (d == 0 ? a.P0 : a.P1) + m.off;
    const int LS = lstride(N);
    cplx<T> *tws = smem;
    cplx<T> *b0 = tws + N;
    cplx<T> *b1 = b0 + line_buf_elems(N, m.lmax[d]);
    __syncthreads();
    for (int i = threadIdx.x; i < N; i += blockDim.x) tws[i] = tw[i];
    for (long long l0 = 0; l0 < nl; l0 += m.lmax[d]) {
      const int L = (int)min((long long)m.lmax[d], nl - l0);
      __syncthreads();
      if (threadIdx.x < L) {
        const long long line = l0 + threadIdx.x;
        lb[threadIdx.x] = (line % stride) + (line / stride) * stride * N;
      }
      __syncthreads();
      const int tot = L * N;
      for (int idx = threadIdx.x; idx < tot; idx += blockDim.x) {
        int w, i;
        if (stride == 1) { w = idx / N; i = idx - w * N; }
        else { i = idx / L; w = idx - i * L; }
        b0[lidx(w, i, LS)] = ld(phi + m.off + lb[w] + (long long)i * stride);
      }
      __syncthreads();
      const int cur = fft_lines<T>(b0, b1, m.rp[d], L, tws, -1);
      cplx<T> *bc = cur ? b1 : b0;
      for (int w = 0; w < L; ++w)
        for (int i = threadIdx.x; i < N; i += blockDim.x) {
          const int x = lidx(w, i, LS);
          bc[x] = cmulr(bc[x], kt[i]);
        }
      __syncthreads();
      const int cur2 = fft_lines<T>(bc, cur ? b0 : b1, m.rp[d], L, tws, +1);
      const cplx<T> *res = cur2 ? (cur ? b0 : b1) : bc;
      for (int idx = threadIdx.x; idx < tot; idx += blockDim.x) {
        int w, i;
        if (stride == 1) { w = idx / N; i = idx - w * N; }
        else { i = idx / L; w = idx - i * L; }
        st(dst + lb[w] + (long long)i * stride, res[lidx(w, i, LS)]);
      }
    }
  }
  __syncthreads();
}

// Point work of one term; returns the block's partial norm.
template <typename T, bool FIRST>
__device__ double ens_points(const EnsArgs<T> &a, const EnsMember &m, const cplx<T> *phi, cplx<T> *kout,
                             double ai, T field) {
  double acc = 0.0;
  const SeriesK<T> sk = series_k<T>(m.offset, FIRST ? m.fac1 : m.fac, FIRST ? m.fac1_lo : m.fac_lo);
  for (long long p = threadIdx.x; p < m.npts; p += blockDim.x) {
    const long long g = m.off + p;
    const cplx<T> x = ld(phi + g);
    cplx<T> h = ld(a.P0 + g);
    if (m.nd > 1) h = h + ld(a.P1 + g);
    T v = a.V[g];
    if (m.has_dipole) v = v + field * a.mu[g];
    h = h + cmulr(x, v);
    const cplx<T> bf = sk(h, x);
    if (FIRST) {
      const cplx<double> ps = ld(a.psi + g);
      acc += cabs2(ps);
      st(kout + g, bf);
      const cplx<double> b = ccast<double>(bf);
      const double a0 = a.coef[m.coef_off], a1 = a.coef[m.coef_off + 1];
      st(a.psi + g, mk(ps.re * a0 + b.re * a1, ps.im * a0 + b.im * a1));
    } else {
      const cplx<T> k2 = bf + ld(kout + g);
      st(kout + g, k2);
      cplx<double> ps = ld(a.psi + g);
      ps.re += ai * (double)k2.re;
      ps.im += ai * (double)k2.im;
      st(a.psi + g, ps);
      acc += cabs2(ps);
    }
  }
  return acc;
}

// Shared memory of the resident 1-D path for a line of N points: psi
// (FP64 or double-float), phi_{i-1}, phi_{i-2}, the two FFT buffers (padded
// line layout), the twiddles as two tables (w^m = W[m / 64] w[m % 64]) and
// V - mu E.
__host__ __device__ inline int ens_tw_hi(int N) { return (N + 63) / 64; }
template <typename T>
__host__ __device__ inline size_t ens_fast_smem(int N) {
  return (size_t)N * (sizeof(cplx<double>) + 2 * sizeof(cplx<T>) + sizeof(T)) +
         (2 * line_buf_elems(N, 1) + 64 + ens_tw_hi(N)) * sizeof(cplx<T>);
}

// Fills the two twiddle tables from the N-entry table tw of the line.
template <typename T>
__device__ __forceinline__ void ens_load_twiddles(const cplx<T> *__restrict__ tw, int N, cplx<T> *twl, cplx<T> *twh) {
  for (int i = threadIdx.x; i < 64; i += blockDim.x) twl[i] = tw[i < N ? i : 0];
  for (int j = threadIdx.x; j < ens_tw_hi(N); j += blockDim.x) twh[j] = tw[64 * j];
}

// One step of a 1-D member that lives in shared memory for the whole step.
// Per term: the forward FFT reads phi_{i-1} directly, the k^2 multiply is
// fused into the loads of the first inverse stage and the point update
// (H phi, the recurrence, the psi accumulation and the norm) into the stores
// of the last inverse stage, so a term costs 2 x stages block barriers.
template <typename T>
__device__ void ens_step_1d(const EnsArgs<T> &a, const EnsMember &m, T field, unsigned char *smem_raw,
                            double *red, long long &terms, int &status) {
  const int N = m.n[0];
  cplx<double> *ps = reinterpret_cast<cplx<double> *>(smem_raw);
  cplx<T> *cur = reinterpret_cast<cplx<T> *>(ps + N);
  cplx<T> *prev = cur + N;
  cplx<T> *f0 = prev + N;
  cplx<T> *f1 = f0 + line_buf_elems(N, 1);
  cplx<T> *twl = f1 + line_buf_elems(N, 1);
  cplx<T> *twh = twl + 64;
  T *Vs = reinterpret_cast<T *>(twh + ens_tw_hi(N));
  ens_load_twiddles<T>(a.tw + m.tw_off[0], N, twl, twh);
  auto tw = [&](int q) { return cmul(twh[q >> 6], twl[q & 63]); };
  const T kfT = (T)m.kf;
  cplx<double> *__restrict__ gpsi = a.psi + m.off;
  for (int i = threadIdx.x; i < N; i += blockDim.x) {
    T v = a.V[m.off + i];
    if (m.has_dipole) v = v + field * a.mu[m.off + i];
    Vs[i] = v;
    const cplx<double> p = ld(gpsi + i);
    ps[i] = p;
    cur[i] = ccast<T>(p);
  }
  __syncthreads();
  const RadixPlan &rp = m.rp[0];
  const int nw = (blockDim.x + 31) >> 5;
  double norm0 = 0.0, last = 0.0;
  bool done = false;
  int used = 2;
  for (int it = 1; it < m.order && !done; ++it) {
    const bool first = it == 1;
    // forward transform of phi_{i-1}: cur -> f0 -> f1 -> ...
    int Ns = 1;
    cplx<T> *dst = f0;
    const cplx<T> *src = cur;
    for (int s = 0; s < rp.nstages; ++s) {
      const bool from_cur = s == 0;  // phi_{i-1} is stored unpadded
      stage_any<T>(rp.radix[s], [&](int i) { return from_cur ? src[i] : src[lpos(i)]; },
                   [&](int i, const cplx<T> &v) { dst[lpos(i)] = v; }, N, 1, Ns, tw, -1);
      __syncthreads();
      Ns *= rp.radix[s];
      src = dst;
      dst = dst == f0 ? f1 : f0;
    }
    // inverse transform; the last stage finishes the term point by point
    const SeriesK<T> sk = series_k<T>(m.offset, first ? m.fac1 : m.fac, first ? m.fac1_lo : m.fac_lo);
    const double ai = a.coef[m.coef_off + it];
    const double a0 = a.coef[m.coef_off];
    double acc = 0.0;
    auto point = [&](int i, const cplx<T> &tk) {
      const cplx<T> x = cur[i];
      const cplx<T> h = tk + cmulr(x, Vs[i]);
      const cplx<T> bf = sk(h, x);
      cplx<double> p = ps[i];
      if (first) {
        acc += cabs2(p);
        prev[i] = bf;  // phi_1
        const cplx<double> b = ccast<double>(bf);
        p = mk(p.re * a0 + b.re * ai, p.im * a0 + b.im * ai);
      } else {
        const cplx<T> k2 = bf + prev[i];
        prev[i] = k2;  // phi_i over phi_{i-2}
        p.re += ai * (double)k2.re;
        p.im += ai * (double)k2.im;
        acc += cabs2(p);
      }
      ps[i] = p;
    };
    Ns = 1;
    for (int s = 0; s < rp.nstages; ++s) {
      const bool ks = s == 0, ls = s == rp.nstages - 1;
      auto load = [&](int i) {
        if (!ks) return src[lpos(i)];
        const int q = min(i, N - i);
        return cmulr(src[lpos(i)], kfT * (T)(q * q));
      };
      if (ls) {
        stage_any<T>(rp.radix[s], load, point, N, 1, Ns, tw, +1);
      } else {
        stage_any<T>(rp.radix[s], load, [&](int i, const cplx<T> &v) { dst[lpos(i)] = v; }, N, 1, Ns, tw, +1);
        __syncthreads();
      }
      Ns *= rp.radix[s];
      src = dst;
      dst = dst == f0 ? f1 : f0;
    }
    // deterministic block reduction: every thread sums the warp totals in order
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
    __syncthreads();
    double tot = 0.0;
    for (int w = 0; w < nw; ++w) tot += red[w];
    // phi_{i-1} <- phi_i (prev), phi_{i-2} <- phi_{i-1} (cur)
    cplx<T> *tmp = cur;
    cur = prev;
    prev = tmp;
    if (first) {
      norm0 = last = tot;
      if (!isfinite(norm0)) { done = true; status = 2; }
      continue;
    }
    used = it + 1;
    if (!isfinite(tot)) { done = true; status = 2; }
    else {
      const double ref = a.diff ? last : norm0;
      if (fabs(ref - tot) / norm0 < m.prec && m.offset.im == 0.0) done = true;  // OCheby.cpp:179-182
    }
    last = tot;
  }
  for (int i = threadIdx.x; i < N; i += blockDim.x) st(gpsi + i, cmul(ps[i], m.ph));
  __syncthreads();
  terms += used;
}

// ---- double-float accumulation (mixed precision) --------------------------
// GB300 runs FP64 at 1/64 of the FP32 rate, and in the resident path the
// FP64 psi update and norm were ~40% of a term (ncu, one 4096-point member).
// The mixed form therefore accumulates psi as an unevaluated sum hi + lo of
// two FP32 numbers (error-free transformations of Dekker and Knuth; about
// 48 significant bits, far below the FP32 error of the phi_n) and tracks
// the series cut through the norm change of each term.  The explicit
// round-to-nearest intrinsics keep the compiler from contracting the
// transformations into FMAs.
__device__ __forceinline__ dfloat df_split(double x) {
  dfloat r;
  r.hi = (float)x;
  r.lo = (float)(x - (double)r.hi);
  return r;
}

// v += (ah + al) * x, with ah + al a split FP64 coefficient
__device__ __forceinline__ void df_axpy(dfloat &v, float ah, float al, float x) {
  const float p = __fmul_rn(ah, x);
  const float e = fmaf(al, x, fmaf(ah, x, -p));       // exact low part of ah x, plus al x
  const float s = __fadd_rn(v.hi, p);                  // two-sum of v.hi and p
  const float bb = __fsub_rn(s, v.hi);
  const float se = __fadd_rn(__fsub_rn(v.hi, __fsub_rn(s, bb)), __fsub_rn(p, bb));
  const float lo = __fadd_rn(v.lo, __fadd_rn(se, e));
  const float h2 = __fadd_rn(s, lo);                    // renormalise
  v.lo = __fsub_rn(lo, __fsub_rn(h2, s));
  v.hi = h2;
}

// One step of a 1-D member in shared memory, mixed form: as ens_step_1d with
// psi in double-float.  The cut uses the norm change of term i,
// 2 Re<psi|a_i phi_i> + |a_i phi_i|^2 (summed in FP32 per thread, FP64 across
// the block), which is what |psi|^2 - previous |psi|^2 measures; the
// reference's first comparison (term 2 against the norm before the step)
// becomes the change of term 2, which differs only for series that have
// converged by term 2.
__device__ void ens_step_1d_df(const EnsArgs<float> &a, const EnsMember &m, float field, unsigned char *smem_raw,
                               double *red, long long &terms, int &status) {
  typedef float T;
  const int N = m.n[0];
  dfloat *pre = reinterpret_cast<dfloat *>(smem_raw);   // psi real part
  dfloat *pim = pre + N;                                 // psi imaginary part
  cplx<T> *cur = reinterpret_cast<cplx<T> *>(pim + N);
  cplx<T> *prev = cur + N;
  cplx<T> *f0 = prev + N;
  cplx<T> *f1 = f0 + line_buf_elems(N, 1);
  cplx<T> *twl = f1 + line_buf_elems(N, 1);
  cplx<T> *twh = twl + 64;
  T *Vs = reinterpret_cast<T *>(twh + ens_tw_hi(N));
  ens_load_twiddles<T>(a.tw + m.tw_off[0], N, twl, twh);
  auto tw = [&](int q) { return cmul(twh[q >> 6], twl[q & 63]); };
  const T kfT = (T)m.kf;
  cplx<double> *__restrict__ gpsi = a.psi + m.off;
  double n0 = 0.0;
  for (int i = threadIdx.x; i < N; i += blockDim.x) {
    T v = a.V[m.off + i];
    if (m.has_dipole) v = v + field * a.mu[m.off + i];
    Vs[i] = v;
    const cplx<double> p = ld(gpsi + i);
    pre[i] = df_split(p.re);
    pim[i] = df_split(p.im);
    cur[i] = ccast<T>(p);
    n0 += cabs2(p);
  }
  const int nw = (blockDim.x + 31) >> 5;
  for (int o = 16; o > 0; o >>= 1) n0 += __shfl_down_sync(0xffffffffu, n0, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = n0;
  __syncthreads();
  double norm0 = 0.0;
  for (int w = 0; w < nw; ++w) norm0 += red[w];
  if (!isfinite(norm0)) status = 2;
  const RadixPlan &rp = m.rp[0];
  bool done = !isfinite(norm0);
  int used = 2;
  for (int it = 1; it < m.order && !done; ++it) {
    const bool first = it == 1;
    int Ns = 1;
    cplx<T> *dst = f0;
    const cplx<T> *src = cur;
    for (int s = 0; s < rp.nstages; ++s) {
      const bool from_cur = s == 0;
      stage_any<T>(rp.radix[s], [&](int i) { return from_cur ? src[i] : src[lpos(i)]; },
                   [&](int i, const cplx<T> &v) { dst[lpos(i)] = v; }, N, 1, Ns, tw, -1);
      __syncthreads();
      Ns *= rp.radix[s];
      src = dst;
      dst = dst == f0 ? f1 : f0;
    }
    const SeriesK<T> sk = series_k<T>(m.offset, first ? m.fac1 : m.fac, first ? m.fac1_lo : m.fac_lo);
    const double ai = a.coef[m.coef_off + it];
    const float ai_h = (float)ai, ai_l = (float)(ai - (double)ai_h);
    const double a0 = a.coef[m.coef_off];
    const float a0_h = (float)a0, a0_l = (float)(a0 - (double)a0_h);
    float dn = 0.0f;  // this thread's share of the norm change
    auto point = [&](int i, const cplx<T> &tk) {
      const cplx<T> x = cur[i];
      const cplx<T> h = tk + cmulr(x, Vs[i]);
      const cplx<T> bf = sk(h, x);
      dfloat pr = pre[i], pi = pim[i];
      if (first) {
        prev[i] = bf;  // phi_1
        // psi = a0 psi + a1 phi_1
        dfloat qr = {0.0f, 0.0f}, qi = {0.0f, 0.0f};
        df_axpy(qr, a0_h, a0_l, pr.hi);
        df_axpy(qr, a0_h, a0_l, pr.lo);
        df_axpy(qi, a0_h, a0_l, pi.hi);
        df_axpy(qi, a0_h, a0_l, pi.lo);
        df_axpy(qr, ai_h, ai_l, bf.re);
        df_axpy(qi, ai_h, ai_l, bf.im);
        pr = qr;
        pi = qi;
      } else {
        const cplx<T> k2 = bf + prev[i];
        prev[i] = k2;  // phi_i over phi_{i-2}
        const float tr = ai_h * k2.re, ti = ai_h * k2.im;
        dn = fmaf(2.0f * pr.hi + tr, tr, fmaf(2.0f * pi.hi + ti, ti, dn));
        df_axpy(pr, ai_h, ai_l, k2.re);
        df_axpy(pi, ai_h, ai_l, k2.im);
      }
      pre[i] = pr;
      pim[i] = pi;
    };
    Ns = 1;
    for (int s = 0; s < rp.nstages; ++s) {
      const bool ks = s == 0, ls = s == rp.nstages - 1;
      auto load = [&](int i) {
        if (!ks) return src[lpos(i)];
        const int q = min(i, N - i);
        return cmulr(src[lpos(i)], kfT * (T)(q * q));
      };
      if (ls) {
        stage_any<T>(rp.radix[s], load, point, N, 1, Ns, tw, +1);
      } else {
        stage_any<T>(rp.radix[s], load, [&](int i, const cplx<T> &v) { dst[lpos(i)] = v; }, N, 1, Ns, tw, +1);
        __syncthreads();
      }
      Ns *= rp.radix[s];
      src = dst;
      dst = dst == f0 ? f1 : f0;
    }
    double acc = (double)dn;
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
    __syncthreads();
    double delta = 0.0;
    for (int w = 0; w < nw; ++w) delta += red[w];
    cplx<T> *tmp = cur;
    cur = prev;
    prev = tmp;
    if (first) continue;
    used = it + 1;
    if (!isfinite(delta)) { done = true; status = 2; }
    else if (fabs(delta) / norm0 < m.prec && m.offset.im == 0.0) done = true;  // OCheby.cpp:179-182
  }
  for (int i = threadIdx.x; i < N; i += blockDim.x) {
    const cplx<double> p = mk((double)pre[i].hi + (double)pre[i].lo, (double)pim[i].hi + (double)pim[i].lo);
    st(gpsi + i, cmul(p, m.ph));
  }
  __syncthreads();
  terms += used;
}

// Sum over the block of one double per thread, returned to every thread.
__device__ __forceinline__ double block_sum_all(double v, double *red) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  __syncthreads();
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  double t = 0.0;
  const int nw = (blockDim.x + 31) >> 5;
  for (int w = 0; w < nw; ++w) t += red[w];
  return t;
}

// Point work of one term for members off the resident path, mixed form:
// psi in double-float (global), the norm change of the term per thread.
template <bool FIRST>
__device__ float ens_points_df(const EnsArgs<float> &a, const EnsMember &m, const cplx<float> *phi,
                               cplx<float> *kout, float a0h, float a0l, float aih, float ail, float field) {
  typedef float T;
  float dn = 0.0f;
  const SeriesK<T> sk = series_k<T>(m.offset, FIRST ? m.fac1 : m.fac, FIRST ? m.fac1_lo : m.fac_lo);
  for (long long p = threadIdx.x; p < m.npts; p += blockDim.x) {
    const long long g = m.off + p;
    const cplx<T> x = ld(phi + g);
    cplx<T> h = ld(a.P0 + g);
    if (m.nd > 1) h = h + ld(a.P1 + g);
    T v = a.V[g];
    if (m.has_dipole) v = v + field * a.mu[g];
    h = h + cmulr(x, v);
    const cplx<T> bf = sk(h, x);
    dfloat pr = a.dfr[g], pi = a.dfi[g];
    if (FIRST) {
      st(kout + g, bf);
      dfloat qr = {0.0f, 0.0f}, qi = {0.0f, 0.0f};
      df_axpy(qr, a0h, a0l, pr.hi);
      df_axpy(qr, a0h, a0l, pr.lo);
      df_axpy(qi, a0h, a0l, pi.hi);
      df_axpy(qi, a0h, a0l, pi.lo);
      df_axpy(qr, aih, ail, bf.re);
      df_axpy(qi, aih, ail, bf.im);
      pr = qr;
      pi = qi;
    } else {
      const cplx<T> k2 = bf + ld(kout + g);
      st(kout + g, k2);
      const float tr = aih * k2.re, ti = aih * k2.im;
      dn = fmaf(2.0f * pr.hi + tr, tr, fmaf(2.0f * pi.hi + ti, ti, dn));
      df_axpy(pr, aih, ail, k2.re);
      df_axpy(pi, aih, ail, k2.im);
    }
    a.dfr[g] = pr;
    a.dfi[g] = pi;
  }
  return dn;
}

// One step of a member off the resident path, mixed form (see ens_step_1d_df
// for the series cut).
__device__ void ens_step_df(const EnsArgs<float> &a, const EnsMember &m, float field, cplx<float> *smem,
                            double *red, long long &terms, int &status) {
  cplx<double> *__restrict__ psi = a.psi + m.off;
  double n0 = 0.0;
  for (long long p = threadIdx.x; p < m.npts; p += blockDim.x) {
    const cplx<double> ps = ld(psi + p);
    a.dfr[m.off + p] = df_split(ps.re);
    a.dfi[m.off + p] = df_split(ps.im);
    st(a.buf0 + m.off + p, ccast<float>(ps));
    n0 += cabs2(ps);
  }
  const double norm0 = block_sum_all(n0, red);
  bool done = !isfinite(norm0);
  if (done) status = 2;
  const double a0 = a.coef[m.coef_off], a1 = a.coef[m.coef_off + 1];
  const float a0h = (float)a0, a0l = (float)(a0 - (double)a0h);
  const float a1h = (float)a1, a1l = (float)(a1 - (double)a1h);
  int used = 2;
  if (!done) {
    ens_kinetic<float>(a, m, a.buf0, smem);
    ens_points_df<true>(a, m, a.buf0, a.buf1, a0h, a0l, a1h, a1l, field);
  }
  // phi_{i-1} in buf[(i+1)&1], phi_{i-2} in buf[i&1] (overwritten by phi_i)
  for (int i = 2; i < m.order && !done; ++i) {
    cplx<float> *phi = (i & 1) ? a.buf0 : a.buf1;
    cplx<float> *kout = (i & 1) ? a.buf1 : a.buf0;
    ens_kinetic<float>(a, m, phi, smem);
    const double ai = a.coef[m.coef_off + i];
    const float aih = (float)ai, ail = (float)(ai - (double)aih);
    const double delta = block_sum_all((double)ens_points_df<false>(a, m, phi, kout, 0.f, 0.f, aih, ail, field), red);
    used = i + 1;
    if (!isfinite(delta)) { done = true; status = 2; }
    else if (fabs(delta) / norm0 < m.prec && m.offset.im == 0.0) done = true;  // OCheby.cpp:179-182
  }
  __syncthreads();
  for (long long p = threadIdx.x; p < m.npts; p += blockDim.x) {
    const dfloat pr = a.dfr[m.off + p], pi = a.dfi[m.off + p];
    st(psi + p, cmul(mk((double)pr.hi + (double)pr.lo, (double)pi.hi + (double)pi.lo), m.ph));
  }
  __syncthreads();
  terms += used;
}

// Threads per block.  Members on the resident 1-D path run 256 threads (a
// 4096-point line is 256 radix-16 items per stage; 512 threads measured 40%
// slower there).  The FP32 form's line-batch members wait on shared memory
// and block barriers and run 25% faster with 512 threads, so the mixed
// ensemble runs them in a second launch beside the first.  The binary64 form
// is bound by its FP64 work and keeps 256 threads with more registers each.
template <typename T>
struct EnsBlock {
  static constexpr int threads = 256;
  static constexpr int wide = sizeof(T) == sizeof(float) ? 512 : 256;
};

template <typename T>
__global__ void __launch_bounds__(EnsBlock<T>::wide) ensemble_kernel(EnsArgs<T> a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ double red[32];
  __shared__ double tot_s;
  __shared__ int cur;
  cplx<T> *smem = reinterpret_cast<cplx<T> *>(smem_raw);
  for (;;) {
    __syncthreads();
    if (threadIdx.x == 0) cur = atomicAdd(a.queue, 1);
    __syncthreads();
    if (cur >= a.n) return;
    const int mi = a.order[cur];
    const EnsMember m = a.m[mi];
    if (threadIdx.x == 0) { a.tl[3 * mi] = ens_clock(); a.tl[3 * mi + 2] = a.block0 + blockIdx.x; }
    long long terms = 0;
    int status = 0;
    for (int k = 0; k < a.nsteps; ++k) {
      const long long step = a.step0 + k;
      // E(step) of Laser::Get (src/qdlib/Laser.cpp:125-128); the dipole term is -mu E
      T field = (T)0;
      if (m.has_dipole && step >= 0 && step < m.laser_nt) field = (T)(-a.lasers[m.laser_off + step]);
      if (m.nd == 1 && m.fast) {
        if constexpr (sizeof(T) == sizeof(float)) ens_step_1d_df(a, m, field, smem_raw, red, terms, status);
        else ens_step_1d<T>(a, m, field, smem_raw, red, terms, status);
        continue;
      }
      if constexpr (sizeof(T) == sizeof(float)) {
        ens_step_df(a, m, field, smem, red, terms, status);
        continue;
      }
      for (long long p = threadIdx.x; p < m.npts; p += blockDim.x)
        st(a.buf0 + m.off + p, ccast<T>(ld(a.psi + m.off + p)));
      ens_kinetic<T>(a, m, a.buf0, smem);
      double t = block_sum(ens_points<T, true>(a, m, a.buf0, a.buf1, 0.0, field), red);
      if (threadIdx.x == 0) tot_s = t;
      __syncthreads();
      const double norm0 = tot_s;
      double last = norm0;
      bool done = !isfinite(norm0);
      if (done) status = 2;
      int used = 2;
      // phi_{i-1} in buf[(i+1)&1], phi_{i-2} in buf[i&1] (overwritten by phi_i)
      for (int i = 2; i < m.order && !done; ++i) {
        cplx<T> *phi = (i & 1) ? a.buf0 : a.buf1;
        cplx<T> *kout = (i & 1) ? a.buf1 : a.buf0;
        ens_kinetic<T>(a, m, phi, smem);
        t = block_sum(ens_points<T, false>(a, m, phi, kout, a.coef[m.coef_off + i], field), red);
        if (threadIdx.x == 0) tot_s = t;
        __syncthreads();
        const double tot = tot_s;
        used = i + 1;
        if (!isfinite(tot)) { done = true; status = 2; }
        else {
          const double ref = a.diff ? last : norm0;
          if (fabs(ref - tot) / norm0 < m.prec && m.offset.im == 0.0) done = true;  // OCheby.cpp:179-182
        }
        last = tot;
      }
      for (long long p = threadIdx.x; p < m.npts; p += blockDim.x)
        st(a.psi + m.off + p, cmul(ld(a.psi + m.off + p), m.ph));
      terms += used;
    }
    if (threadIdx.x == 0) {
      a.terms[mi] += terms;
      if (status) a.status[mi] = status;
      a.tl[3 * mi + 1] = ens_clock();
    }
  }
}

template <typename T>
static int ensemble_occupancy(size_t smem, int threads) {
  void *k = (void *)ensemble_kernel<T>;
  if (smem > 48 * 1024 && cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
    return 0;
  int nb = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k, threads, smem) != cudaSuccess) return 0;
  return nb;
}

}  // namespace qdg

using qdg::cplx;
typedef std::complex<double> cd;

struct qdg_ensemble {
  int n = 0;
  int precision = QDG_PREC_MIXED;
  size_t csize = 8;
  double dt = 0;
  std::vector<qdg::EnsMember> hm;
  std::vector<int> order;
  long long total_pts = 0;
  // device
  qdg::EnsMember *d_m = nullptr;
  int *d_order = nullptr, *d_queue = nullptr, *d_status = nullptr;
  long long *d_terms = nullptr;
  cplx<double> *d_psi = nullptr;
  void *d_buf0 = nullptr, *d_buf1 = nullptr, *d_P0 = nullptr, *d_P1 = nullptr;
  void *d_dfr = nullptr, *d_dfi = nullptr;  // mixed form: double-float psi of a step
  unsigned long long *d_tl = nullptr;       // per member start, end, block of the last run
  void *d_V = nullptr, *d_mu = nullptr, *d_tw = nullptr, *d_kt = nullptr;
  double *d_lasers = nullptr, *d_coef = nullptr;
  size_t smem = 0;
  int grid = 1;
  // mixed form: order[0, nA) are the resident 1-D members (launch A, 256
  // threads, `grid` blocks), order[nA, n) the others (launch B beside it on
  // stream2, wide blocks, gridB blocks); otherwise one launch over all
  int nA = 0, gridB = 0;
  cudaStream_t stream = nullptr, stream2 = nullptr;
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
};

namespace {

qdg_status efail(qdg_status s, const std::string &m) {
  qdg::set_last_error(m);
  return s;
}

#define ECK(...)                                                                          \
  do {                                                                                    \
    cudaError_t e_ = (__VA_ARGS__);                                                       \
    if (e_ != cudaSuccess) return efail(QDG_ECUDA, std::string(#__VA_ARGS__) + ": " + cudaGetErrorString(e_)); \
  } while (0)

void parse_kv(const char *s, std::map<std::string, std::string> &out) {
  if (!s) return;
  std::string str(s);
  for (char &c : str)
    if (c == ';' || c == ',' || c == '\t' || c == '\n') c = ' ';
  size_t i = 0;
  while (i < str.size()) {
    while (i < str.size() && str[i] == ' ') ++i;
    size_t j = i;
    while (j < str.size() && str[j] != ' ') ++j;
    const std::string kv = str.substr(i, j - i);
    const size_t eq = kv.find('=');
    if (eq != std::string::npos) out[kv.substr(0, eq)] = kv.substr(eq + 1);
    i = j;
  }
}

template <typename T>
qdg_status upload_vec(void **dst, const std::vector<T> &v) {
  ECK(cudaMalloc(dst, sizeof(T) * std::max<size_t>(1, v.size())));
  if (!v.empty()) ECK(cudaMemcpy(*dst, v.data(), sizeof(T) * v.size(), cudaMemcpyHostToDevice));
  return QDG_OK;
}

void free_ensemble(qdg_ensemble *e) {
  void *ps[] = {e->d_m, e->d_order, e->d_queue, e->d_status, e->d_terms, e->d_psi, e->d_buf0, e->d_buf1, e->d_P0,
                e->d_P1, e->d_V, e->d_mu, e->d_tw, e->d_kt, e->d_lasers, e->d_coef, e->d_dfr, e->d_dfi, e->d_tl};
  for (void *p : ps)
    if (p) cudaFree(p);
  if (e->stream) cudaStreamDestroy(e->stream);
  if (e->stream2) cudaStreamDestroy(e->stream2);
  if (e->ev_fork) cudaEventDestroy(e->ev_fork);
  if (e->ev_join) cudaEventDestroy(e->ev_join);
  delete e;
}

// Time per point and term of a member off the resident path relative to one
// on it (one block each, measured on GB300 over the workload's sizes).
constexpr double kOffResidentCost = 2.0;
// Time per point and term of a line-batch member in a wide (512-thread)
// block relative to a resident member, for the split of the SMs between the
// two launches of the mixed form (measured on GB300 over the workload's
// sizes: 0.26-0.41 ns per point, log2 point and term resident, 0.33-0.41 in
// wide blocks).
constexpr double kOffResidentWideCost = 1.1;

template <typename T>
qdg_status build(qdg_ensemble *e, const qdg_ensemble_member *mem, const std::map<std::string, std::string> &params) {
  const int n = e->n;
  std::vector<T> V, mu, kt;
  std::vector<cplx<T>> tw;
  std::vector<double> lasers, coef;
  std::map<int, long long> tw_at;  // twiddle table of each line length
  std::vector<double> cost(n);
  long long off = 0;
  size_t smem = 0;
  const cd c0 = cd(0, -e->dt);  // forward real-time exponent (OPropagator.h:62-77)
  for (int k = 0; k < n; ++k) {
    const qdg_ensemble_member &x = mem[k];
    qdg::EnsMember m;
    memset(&m, 0, sizeof(m));
    if (x.grid.ndims < 1 || x.grid.ndims > 2) return efail(QDG_EUNSUPPORTED, "ensemble members are 1-D or 2-D grids");
    if (!x.potential) return efail(QDG_EINVAL, "ensemble member without a potential");
    m.nd = x.grid.ndims;
    m.npts = 1;
    bool generic = false;  // a line length with a prime factor above 5
    double dx[2], dk[2], Tmax = 0;
    for (int d = 0; d < m.nd; ++d) {
      const int N = x.grid.n[d];
      if (N < 2 || !(x.grid.xmax[d] > x.grid.xmin[d])) return efail(QDG_EINVAL, "invalid member grid");
      if (!(x.mass[d] > 0)) return efail(QDG_EINVAL, "Zero mass defined");
      if (!qdg::schedule_radix(qdg::SCHED_ENSEMBLE, N, e->precision, m.rp[d])) {
        // other prime factors: direct-DFT stages, which the line-batch path
        // (fft_lines) takes; such members stay off the resident 1-D path
        if (!qdg::any_radix(N, m.rp[d])) return efail(QDG_EUNSUPPORTED, "grid size has more than 16 prime factors");
        generic = true;
      }
      m.n[d] = N;
      m.npts *= N;
      dx[d] = (x.grid.xmax[d] - x.grid.xmin[d]) / double(N - 1);
      dk[d] = (2 * M_PI) / (x.grid.xmax[d] - x.grid.xmin[d] + dx[d]);
      Tmax += 1 / (x.mass[d] * dx[d] * dx[d]);
      if (!tw_at.count(N)) {
        tw_at[N] = (long long)tw.size();
        const long double pi = 3.141592653589793238462643383279502884L;
        for (int i = 0; i < N; ++i) {
          const long double ang = -2.0L * pi * i / N;
          cplx<T> c;
          c.re = (T)cosl(ang);
          c.im = (T)sinl(ang);
          tw.push_back(c);
        }
      }
      m.tw_off[d] = tw_at[N];
      m.kt_off[d] = (long long)kt.size();
      const double kf = dk[d] * dk[d] / (2.0 * x.mass[d]) / N;
      if (d == 0) m.kf = kf;
      for (int i = 0; i < N; ++i) {
        const double q = std::min(i, N - i);
        kt.push_back((T)(kf * q * q));
      }
      m.lmax[d] = (int)std::max(1, std::min(64, 4096 / N));
      smem = std::max(smem, ((size_t)N + 2 * qdg::line_buf_elems(N, m.lmax[d])) * sizeof(cplx<T>));
    }
    if (m.nd == 1 && !generic) {
      const size_t fsm = qdg::ens_fast_smem<T>(m.n[0]);
      if (fsm <= 216 * 1024) {
        m.fast = 1;
        smem = std::max(smem, fsm);
      }
    }
    m.off = off;
    off += m.npts;
    const double vmax = *std::max_element(x.potential, x.potential + m.npts);
    const double vmin = *std::min_element(x.potential, x.potential + m.npts);
    for (long long i = 0; i < m.npts; ++i) V.push_back((T)x.potential[i]);
    // OSum::Emax/Emin over (GridNablaSq, GridPotential, GridDipole)
    cd emax = Tmax * (M_PI * M_PI / 2) + vmax, emin = vmin;
    m.has_dipole = x.dipole && x.laser && x.laser_nt > 0;
    if (m.has_dipole) {
      const double mmax = *std::max_element(x.dipole, x.dipole + m.npts);
      const double lmax = *std::max_element(x.laser, x.laser + x.laser_nt);
      emax += mmax * lmax;  // OGridDipole::Emax (OGridDipole.cpp:36-39)
      for (long long i = 0; i < m.npts; ++i) mu.push_back((T)x.dipole[i]);
      m.laser_off = (long long)lasers.size();
      m.laser_nt = x.laser_nt;
      lasers.insert(lasers.end(), x.laser, x.laser + x.laser_nt);
    } else {
      for (long long i = 0; i < m.npts; ++i) mu.push_back((T)0);
      m.laser_off = -1;
    }
    qdg::host::ChebySeries cs;
    const std::string err = qdg::host::cheby_series(emax, emin, e->dt, c0, false, params, cs);
    if (!err.empty()) return efail(QDG_EINVAL, err);
    m.order = cs.order;
    m.coef_off = (long long)coef.size();
    coef.insert(coef.end(), cs.coeff.begin(), cs.coeff.end());
    const cd ex = c0 / e->dt;
    m.offset.re = cs.offset.real(); m.offset.im = cs.offset.imag();
    const cd f1 = ex / cs.scaling, f = 2.0 * ex / cs.scaling, ph = std::exp(c0 * cs.offset);
    m.fac1.re = f1.real(); m.fac1.im = f1.imag();
    m.fac.re = f.real(); m.fac.im = f.imag();
    {  // residuals of the rounded factors, from a long double evaluation
      const std::complex<long double> exl((long double)c0.real() / e->dt, (long double)c0.imag() / e->dt);
      const std::complex<long double> l1 = exl / (long double)cs.scaling, l2 = 2.0L * exl / (long double)cs.scaling;
      m.fac1_lo.re = (double)(l1.real() - (long double)m.fac1.re); m.fac1_lo.im = (double)(l1.imag() - (long double)m.fac1.im);
      m.fac_lo.re = (double)(l2.real() - (long double)m.fac.re); m.fac_lo.im = (double)(l2.imag() - (long double)m.fac.im);
    }
    m.ph.re = ph.real(); m.ph.im = ph.imag();
    m.prec = cs.prec;
    // LPT cost: the series needs about R = scaling dt terms (J_n(R) is
    // negligible beyond R + O(R^{1/3})), each about npts log npts of work;
    // members off the resident path run slower per point (global memory)
    const double R = cs.scaling * e->dt;
    const double est = std::min<double>(cs.order, R + 4.0 * std::cbrt(R) + 10.0);
    cost[k] = (double)m.npts * std::log2((double)m.npts + 1) * est * (m.fast ? 1.0 : kOffResidentCost);
    e->hm.push_back(m);
  }
  e->total_pts = off;
  // largest first (LPT order for the dynamic queue)
  e->order.resize(n);
  std::iota(e->order.begin(), e->order.end(), 0);
  std::stable_sort(e->order.begin(), e->order.end(), [&](int a, int b) { return cost[a] > cost[b]; });
  if (smem > 227 * 1024) return efail(QDG_EUNSUPPORTED, "member line too long for the shared-memory FFT");
  e->smem = smem;
  qdg_status s;
  if ((s = upload_vec(reinterpret_cast<void **>(&e->d_m), e->hm)) != QDG_OK) return s;
  if ((s = upload_vec(reinterpret_cast<void **>(&e->d_order), e->order)) != QDG_OK) return s;
  if ((s = upload_vec(&e->d_V, V)) != QDG_OK) return s;
  if ((s = upload_vec(&e->d_mu, mu)) != QDG_OK) return s;
  if ((s = upload_vec(&e->d_tw, tw)) != QDG_OK) return s;
  if ((s = upload_vec(&e->d_kt, kt)) != QDG_OK) return s;
  if ((s = upload_vec(reinterpret_cast<void **>(&e->d_lasers), lasers)) != QDG_OK) return s;
  if ((s = upload_vec(reinterpret_cast<void **>(&e->d_coef), coef)) != QDG_OK) return s;
  const size_t pts = (size_t)std::max<long long>(1, off);
  ECK(cudaMalloc(&e->d_psi, sizeof(cplx<double>) * pts));
  ECK(cudaMemset(e->d_psi, 0, sizeof(cplx<double>) * pts));
  ECK(cudaMalloc(&e->d_buf0, sizeof(cplx<T>) * pts));
  ECK(cudaMalloc(&e->d_buf1, sizeof(cplx<T>) * pts));
  if (sizeof(T) == sizeof(float)) {
    ECK(cudaMalloc(&e->d_dfr, sizeof(qdg::dfloat) * pts));
    ECK(cudaMalloc(&e->d_dfi, sizeof(qdg::dfloat) * pts));
  }
  ECK(cudaMalloc(&e->d_P0, sizeof(cplx<T>) * pts));
  ECK(cudaMalloc(&e->d_P1, sizeof(cplx<T>) * pts));
  ECK(cudaMalloc(&e->d_queue, 2 * sizeof(int)));
  ECK(cudaMalloc(&e->d_status, sizeof(int) * n));
  ECK(cudaMemset(e->d_status, 0, sizeof(int) * n));
  ECK(cudaMalloc(&e->d_terms, sizeof(long long) * n));
  ECK(cudaMalloc(&e->d_tl, sizeof(unsigned long long) * 3 * n));
  ECK(cudaMemset(e->d_tl, 0, sizeof(unsigned long long) * 3 * n));
  ECK(cudaMemset(e->d_terms, 0, sizeof(long long) * n));
  const int occ = qdg::ensemble_occupancy<T>(smem, qdg::EnsBlock<T>::threads);
  if (occ <= 0) return efail(QDG_EUNSUPPORTED, "ensemble kernel cannot be resident");
  int dev = 0, sms = 1;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  e->grid = std::max(1, std::min(n, occ * sms));
  e->nA = n;
  ECK(cudaStreamCreateWithFlags(&e->stream, cudaStreamNonBlocking));
  if (qdg::EnsBlock<T>::wide != qdg::EnsBlock<T>::threads) {
    // resident 1-D members first, then the others, each group in LPT order
    std::vector<int> grouped = e->order;
    const auto mid = std::stable_partition(grouped.begin(), grouped.end(), [&](int i) { return e->hm[i].fast != 0; });
    const int nA = (int)(mid - grouped.begin());
    const int occB = qdg::ensemble_occupancy<T>(smem, qdg::EnsBlock<T>::wide);
    // Two launches only where every block holds an SM alone (then the blocks
    // of the two launches cannot crowd each other out of SMs), with the SMs
    // split so that the groups' estimated loads per block match.
    if (nA > 0 && nA < n && occ == 1 && occB == 1 && sms > 1) {
      double costA = 0, costB = 0;
      for (int j = 0; j < n; ++j) {
        const int i = grouped[j];
        if (j < nA) costA += cost[i];
        else costB += cost[i] / kOffResidentCost * kOffResidentWideCost;
      }
      int best = 1;
      double best_t = 0;
      for (int g = 1; g < sms; ++g) {
        const double t = std::max(costA / g, costB / (sms - g));
        if (g == 1 || t < best_t) { best = g; best_t = t; }
      }
      e->order = grouped;
      e->nA = nA;
      e->grid = std::min(nA, best);
      e->gridB = std::min(n - nA, sms - best);
      ECK(cudaStreamCreateWithFlags(&e->stream2, cudaStreamNonBlocking));
      ECK(cudaEventCreateWithFlags(&e->ev_fork, cudaEventDisableTiming));
      ECK(cudaEventCreateWithFlags(&e->ev_join, cudaEventDisableTiming));
    } else if (nA == 0 && occB > 0) {  // line-batch members only: one wide launch
      e->nA = 0;
      e->gridB = std::max(1, std::min(n, occB * sms));
    }
    ECK(cudaMemcpy(e->d_order, e->order.data(), sizeof(int) * n, cudaMemcpyHostToDevice));
  }
  return QDG_OK;
}

template <typename T>
qdg_status run(qdg_ensemble *e, long long step0, int nsteps) {
  qdg::EnsArgs<T> a;
  memset(&a, 0, sizeof(a));
  a.m = e->d_m;
  a.order = e->d_order;
  a.n = e->n;
  a.queue = e->d_queue;
  a.psi = e->d_psi;
  a.buf0 = reinterpret_cast<cplx<T> *>(e->d_buf0);
  a.buf1 = reinterpret_cast<cplx<T> *>(e->d_buf1);
  a.P0 = reinterpret_cast<cplx<T> *>(e->d_P0);
  a.P1 = reinterpret_cast<cplx<T> *>(e->d_P1);
  a.V = reinterpret_cast<const T *>(e->d_V);
  a.mu = reinterpret_cast<const T *>(e->d_mu);
  a.lasers = e->d_lasers;
  a.coef = e->d_coef;
  a.tw = reinterpret_cast<const cplx<T> *>(e->d_tw);
  a.ktab = reinterpret_cast<const T *>(e->d_kt);
  a.step0 = step0;
  a.nsteps = nsteps;
  a.diff = e->precision == QDG_PREC_MIXED ? 1 : 0;
  a.terms = e->d_terms;
  a.status = e->d_status;
  a.dfr = reinterpret_cast<qdg::dfloat *>(e->d_dfr);
  a.tl = e->d_tl;
  a.dfi = reinterpret_cast<qdg::dfloat *>(e->d_dfi);
  ECK(cudaMemsetAsync(e->d_queue, 0, 2 * sizeof(int), e->stream));
  void *k = (void *)qdg::ensemble_kernel<T>;
  if (e->smem > 48 * 1024) ECK(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)e->smem));
  void *args[] = {(void *)&a};
  const bool two = e->nA > 0 && e->nA < e->n;
  if (e->nA < e->n) {
    // launch B (members off the resident path, wide blocks); issued first so
    // that its blocks take their SMs before launch A's
    cudaStream_t sb = two ? e->stream2 : e->stream;
    if (two) {
      ECK(cudaEventRecord(e->ev_fork, e->stream));
      ECK(cudaStreamWaitEvent(sb, e->ev_fork, 0));
    }
    a.order = e->d_order + e->nA;
    a.n = e->n - e->nA;
    a.queue = e->d_queue + 1;
    a.block0 = two ? e->grid : 0;
    qdg::add_launches(1);
    ECK(cudaLaunchKernel(k, dim3(e->gridB), dim3(qdg::EnsBlock<T>::wide), args, e->smem, sb));
    if (two) ECK(cudaEventRecord(e->ev_join, sb));
  }
  if (e->nA > 0) {
    a.order = e->d_order;
    a.n = e->nA;
    a.queue = e->d_queue;
    a.block0 = 0;
    qdg::add_launches(1);
    ECK(cudaLaunchKernel(k, dim3(e->grid), dim3(qdg::EnsBlock<T>::threads), args, e->smem, e->stream));
  }
  if (two) ECK(cudaStreamWaitEvent(e->stream, e->ev_join, 0));
  return QDG_OK;
}

}  // namespace

extern "C" {

qdg_status qdg_ensemble_create(const qdg_ensemble_member *members, int32_t n, double dt, const char *params,
                               int32_t precision, qdg_ensemble **out) {
  if (!members || n < 1 || !out) return efail(QDG_EINVAL, "bad arguments");
  if (!(dt > 0)) return efail(QDG_EINVAL, "No time step defined");
  if (precision != QDG_PREC_FP64 && precision != QDG_PREC_MIXED) return efail(QDG_EINVAL, "unknown precision");
  *out = nullptr;
  qdg_ensemble *e = new qdg_ensemble();
  e->n = n;
  e->precision = precision;
  e->csize = precision == QDG_PREC_FP64 ? 16 : 8;
  e->dt = dt;
  std::map<std::string, std::string> kv;
  parse_kv(params, kv);
  const qdg_status s = precision == QDG_PREC_FP64 ? build<double>(e, members, kv) : build<float>(e, members, kv);
  if (s != QDG_OK) {
    free_ensemble(e);
    return s;
  }
  *out = e;
  return QDG_OK;
}

qdg_status qdg_ensemble_destroy(qdg_ensemble *e) {
  if (!e) return QDG_OK;
  if (e->stream) cudaStreamSynchronize(e->stream);
  free_ensemble(e);
  return QDG_OK;
}

qdg_status qdg_ensemble_upload(qdg_ensemble *e, const double *psi) {
  if (!e || !psi) return efail(QDG_EINVAL, "null argument");
  ECK(cudaMemcpyAsync(e->d_psi, psi, sizeof(cplx<double>) * e->total_pts, cudaMemcpyHostToDevice, e->stream));
  ECK(cudaStreamSynchronize(e->stream));
  return QDG_OK;
}

qdg_status qdg_ensemble_download(const qdg_ensemble *e, double *psi) {
  if (!e || !psi) return efail(QDG_EINVAL, "null argument");
  ECK(cudaMemcpyAsync(psi, e->d_psi, sizeof(cplx<double>) * e->total_pts, cudaMemcpyDeviceToHost, e->stream));
  ECK(cudaStreamSynchronize(e->stream));
  return QDG_OK;
}

qdg_status qdg_ensemble_run(qdg_ensemble *e, int64_t step0, int32_t nsteps, int64_t *terms_total) {
  if (!e || nsteps < 0) return efail(QDG_EINVAL, "bad arguments");
  std::vector<long long> before(e->n), after(e->n);
  ECK(cudaMemcpy(before.data(), e->d_terms, sizeof(long long) * e->n, cudaMemcpyDeviceToHost));
  const qdg_status s = e->precision == QDG_PREC_FP64 ? run<double>(e, step0, nsteps) : run<float>(e, step0, nsteps);
  if (s != QDG_OK) return s;
  ECK(cudaStreamSynchronize(e->stream));
  ECK(cudaMemcpy(after.data(), e->d_terms, sizeof(long long) * e->n, cudaMemcpyDeviceToHost));
  std::vector<int> st(e->n);
  ECK(cudaMemcpy(st.data(), e->d_status, sizeof(int) * e->n, cudaMemcpyDeviceToHost));
  long long tot = 0;
  for (int i = 0; i < e->n; ++i) tot += after[i] - before[i];
  if (terms_total) *terms_total = tot;
  for (int i = 0; i < e->n; ++i)
    if (st[i]) return efail(QDG_ENONFINITE, "Norm is not a number (ensemble member " + std::to_string(i) + ")");
  return QDG_OK;
}

qdg_status qdg_ensemble_timeline(const qdg_ensemble *e, int64_t *start_end, int32_t *block) {
  if (!e || !start_end) return efail(QDG_EINVAL, "null argument");
  std::vector<unsigned long long> t(3 * (size_t)e->n);
  ECK(cudaMemcpy(t.data(), e->d_tl, sizeof(unsigned long long) * t.size(), cudaMemcpyDeviceToHost));
  unsigned long long t0 = ~0ULL;
  for (int i = 0; i < e->n; ++i) t0 = std::min(t0, t[3 * i]);
  for (int i = 0; i < e->n; ++i) {
    start_end[2 * i] = (int64_t)(t[3 * i] - t0);
    start_end[2 * i + 1] = (int64_t)(t[3 * i + 1] - t0);
    if (block) block[i] = (int32_t)t[3 * i + 2];
  }
  return QDG_OK;
}

qdg_status qdg_ensemble_member_info(const qdg_ensemble *e, int32_t i, qdg_prop_info *info) {
  if (!e || !info || i < 0 || i >= e->n) return efail(QDG_EINVAL, "bad arguments");
  const qdg::EnsMember &m = e->hm[i];
  info->kind = 1;
  info->order = m.order;
  info->scaling = std::abs(cd(0, -e->dt) / e->dt) / std::abs(cd(m.fac1.re, m.fac1.im));
  info->offset_re = m.offset.re;
  info->offset_im = m.offset.im;
  info->exponent_re = 0;
  info->exponent_im = -e->dt;
  return QDG_OK;
}

}  // extern "C"
