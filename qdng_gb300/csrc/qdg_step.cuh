// qdg_step.cuh -- one Chebyshev time step as one persistent kernel.
//
// The step of OCheby::real_time_step / imag_time_step
// (src/qdlib/OCheby.cpp:92-297) is a chain of up to `order` dependent
// Hamiltonian applications, each far shorter than a kernel launch on a
// 256x256 grid.  Here every block of a cooperative launch (all blocks
// resident by construction) walks the whole series:
//
//   psi -> phi_0;                                         grid barrier
//   term 1: T_d phi_0 for every d (FFT line items);       grid barrier
//           H phi_0, phi_1, psi = a_0 psi + a_1 phi_1;    grid barrier + norm sum
//   term i: T_d phi_{i-1} ...;                            grid barrier
//           phi_i = 2 X (H - E) phi_{i-1} +- phi_{i-2}, psi += a_i phi_i,
//           norm of psi;                                  grid barrier + norm sum
//   ... until the reference's norm cut; psi *= exp(c0 offset).
//
// Every block sums the per-block norms in the same order, so all blocks
// take the same decision without another barrier.  The coefficients a_i are
// real (2 J_i or 2 I_i); the common phase exp(c0 offset) that the reference
// folds into each of them (OCheby.cpp:107,122) is applied once at the end.
// One-dimensional grids fuse the FFT and the point work of a line (a block
// owns its lines for the whole step), leaving one barrier per term.
// Grid barriers spin with an iteration limit; on timeout a flag is raised
// and the kernel returns (the host reports QDG_ETIMEOUT).
//
// Template parameters: T is the storage type of the plan (double, or float
// for the mixed form); FT the arithmetic type of phi, T_d phi, the potential
// values and the FFTs of multi-dimensional grids: double (binary64, the
// drop-in form), dfl (double-float, the DF64 form) or float (mixed).  psi,
// the coefficients and all reductions are binary64 in every form.  This
// header is included by one translation unit per (T, FT, grid rank), which
// keeps the build parallel.
#pragma once

#include <cuda_runtime.h>
#include <math.h>

#include <type_traits>

#include "qdg_grid.cuh"
#include "qdg_kernels.cuh"

namespace qdg {

// ---- one phase per term on grids of two or more dimensions -----------------
// Phase i+1 computes phi_i point-wise while loading the lines of its kinetic
// transforms (H phi_{i-1} = sum_d T_d phi_{i-1} + W phi_{i-1} from the
// previous phase's P), so a term needs one grid barrier.  The lines along
// dimension 0 (rows) cover every point of a state exactly once: their loaders
// also store phi_i and update psi and its norm.  The other dimensions
// recompute phi_i for their own points.
enum PhaseKind { PK_START = 0, PK_FIRST = 1, PK_TERM = 2, PK_LAST = 3 };

template <typename T, typename FT>
__device__ __forceinline__ const cplx<FT> *step_twiddles(const DimPass<T> &g) {
  if constexpr (std::is_same<FT, dfl>::value) return g.twdf;
  else return reinterpret_cast<const cplx<FT> *>(g.tw);
}
template <typename T, typename FT>
__device__ __forceinline__ FT step_kmul(const DimPass<T> &g, long long i) {
  if constexpr (std::is_same<FT, dfl>::value) return g.ktdf[i];
  else return __ldg(reinterpret_cast<const FT *>(g.ktab) + i);
}
template <typename T, typename FT>
__device__ __forceinline__ const FT *step_grids(const StepArgs<T> &a) {
  if constexpr (std::is_same<FT, dfl>::value) return a.gdf;
  else return reinterpret_cast<const FT *>(a.grids);
}

// -f offset as the bulk type: binary64 and FP32 keep the rounded value and
// its residual (part 1), double-float carries both in one number (part 1 is
// zero).
template <typename B>
__device__ __forceinline__ B soff_part(double hi, double lo, int part) {
  if constexpr (std::is_same<B, double>::value) return part == 0 ? hi : lo;
  else if constexpr (std::is_same<B, dfl>::value) {
    if (part) return dfl(0.0f, 0.0f);
    const float h = __double2float_rn(hi);
    return dfl(h, __double2float_rn((hi - (double)h) + lo));
  } else {
    const float h = __double2float_rn(hi);
    return part == 0 ? h : __double2float_rn((hi - (double)h) + lo);
  }
}
// h + (hi + lo) x, the residual first so that the rounded hi does not act
// coherently on every point.
template <typename B>
__device__ __forceinline__ cplx<B> add_soff(cplx<B> h, cplx<B> x, B hi, B lo) {
  if constexpr (std::is_same<B, dfl>::value) return mk(fma_b(hi, x.re, h.re), fma_b(hi, x.im, h.im));
  else return mk(fma(hi, x.re, fma(lo, x.re, h.re)), fma(hi, x.im, fma(lo, x.im, h.im)));
}

// The potential-matrix row of each state as the point work reads it: entry
// columns, grids and field coefficients (1 for static potentials).  Filled
// once per launch (the coefficients are those of the step) so that a batch
// of lines starts without a chain of dependent global loads.
template <typename B>
struct RowCache {
  int ne[kMaxStates];
  int col[kMaxStates][kMaxRowEntries];
  int gid[kMaxStates][kMaxRowEntries];
  B coef[kMaxStates][kMaxRowEntries];
  int nim[kMaxStates][kMaxRowEntries];  // entry acts as -i coef grid (negative imaginary potential)
  int unit[kMaxStates];  // only static potentials (coefficient 1) in the row
};
template <typename T, typename B>
__device__ void fill_rows(const StepArgs<T> &a, RowCache<B> &rc) {
  const bool scaled = a.scaled != 0;
  const Couplings *__restrict__ cpx = scaled ? a.scp : a.cp;
  for (int s = threadIdx.x; s < a.S && s < kMaxStates; s += blockDim.x) {
    const int e0 = cpx->rs[s];
    const int ne = min(cpx->rs[s + 1] - e0, kMaxRowEntries);
    rc.ne[s] = ne;
    int unit = 1;
    for (int k = 0; k < kMaxRowEntries; ++k) {
      rc.col[s][k] = k < ne ? cpx->col[e0 + k] : 0;
      rc.gid[s][k] = k < ne ? cpx->gid[e0 + k] : 0;
      rc.nim[s][k] = (k < ne && !scaled) ? cpx->nim[e0 + k] : 0;
      // the field coefficient of the entry (scaled entries name the plan entry, -1: static)
      const int ci = k >= ne ? -1 : scaled ? cpx->lid[e0 + k] : e0 + k;
      const double c = ci >= 0 ? a.coef[ci] : (k < ne ? 1.0 : 0.0);
      rc.coef[s][k] = d2b<B>(c);
      if (k < ne && c != 1.0) unit = 0;
    }
    rc.unit[s] = unit;
  }
}

// Kinetic transforms of phi_i (computed on load) for every dimension;
// results go to Pnext.  PK_LAST only finishes phi_i and psi (row lines).
// Loads of UNR points per thread are issued before any use or store, so the
// latency of the L2 round trips overlaps.
template <typename T, typename FT, int ND, int SM>
__device__ void phase_fused(const StepArgs<T> &a, int kind, const cplx<T> *__restrict__ phim1,
                            const cplx<T> *__restrict__ phim2, cplx<T> *__restrict__ phout,
                            cplx<T> *const *Pprev, cplx<T> *const *Pnext, double coeff_i, double &acc,
                            cplx<T> *smem, int &cur_n, const RowCache<FT> &rc, const long long *bs,
                            long long lo, long long hi, unsigned long long *tp = nullptr) {
  typedef FT B;
  const bool tr = tp != nullptr && threadIdx.x == 0;
  const cplx<B> *phim1b = reinterpret_cast<const cplx<B> *>(phim1);
  const cplx<B> *phim2b = reinterpret_cast<const cplx<B> *>(phim2);
  cplx<B> *phoutb = reinterpret_cast<cplx<B> *>(phout);
  // points gathered per thread and iteration (loads in flight); the binary64
  // bulk is bound by its arithmetic and takes more to keep the FP64 pipe fed
  constexpr int UNR = SM > 2 ? 1 : std::is_same<FT, double>::value ? 3 : 2;
  constexpr int RE = kMaxRowEntries;
  const long long npts = a.npts;
  // this block's lines of the phase: from the table bs, or an even split of [lo, hi)
  const long long G = gridDim.x;
  const long long end = bs ? bs[blockIdx.x + 1] : lo + (hi - lo) * (blockIdx.x + 1) / G;
  long long l = bs ? bs[blockIdx.x] : lo + (hi - lo) * blockIdx.x / G;
  // cur_n: the line length whose twiddles the shared table holds (the
  // table depends on N only); it lives in the caller across terms, so a
  // block that keeps its line length loads it once per step
  // asynchronous staging of the gather's operands (binary64 and double-float
  // bulk, one or two states): kStageDepth slots of one point per thread in
  // front of the twiddle table; per slot the kinetic parts, phi_{i-1} of
  // every state and phi_{i-2} (16 bytes each), the potential values (8
  // bytes) and psi (16 bytes), each as an array over the 256 threads
  constexpr bool kStaged = step_staged(sizeof(cplx<FT>), SM);
  constexpr int kVgOff = (ND + SM + 1) * 256 * 16;
  constexpr int kPsOff = kVgOff + kMaxRowEntries * 256 * 8;
  constexpr int kSlotBytes = kPsOff + 256 * 16;
  static_assert(!kStaged || kStageDepth * kSlotBytes == step_stage_bytes_c(ND, SM), "staging layout");
  cplx<FT> *tws = reinterpret_cast<cplx<FT> *>(reinterpret_cast<unsigned char *>(smem) +
                                               (kStaged ? kStageDepth * kSlotBytes : 0));
  __shared__ long long lbase[kMaxBatchLines];
  const cplx<B> off = {d2b<B>(a.offset.re), d2b<B>(a.offset.im)};
  const cplx<double> facd = kind == PK_FIRST ? a.fac1 : a.fac;
  const cplx<B> fac = {d2b<B>(facd.re), d2b<B>(facd.im)};
  const bool off_real = a.offset.im == 0.0;
  const bool fac_imag = facd.re == 0.0;
  // pre-scaled point work: H' = f (H - offset) from the scaled tables, then
  // phi_i = (i) H' phi_{i-1} +- phi_{i-2}; otherwise the factor and the offset
  // are applied per point
  const bool scaled = a.scaled != 0;
  const bool srt = a.scaled_rt != 0;
  const B *__restrict__ grids = scaled ? reinterpret_cast<const B *>(a.sgrids) : step_grids<T, FT>(a);
  const B soh = soff_part<B>(a.soff_hi, a.soff_lo, 0), sol = soff_part<B>(a.soff_hi, a.soff_lo, 1);
  const B rsg = d2b<B>(a.imag ? -1.0 : 1.0);  // sign of phi_{i-2} in the recurrence
  while (l < end) {
    int d = 0;
    while (l >= a.line_start[d + 1]) ++d;
    const DimPass<T> &g = a.dp[d];
    const int N = g.N;
    const long long stride = g.ls == 1 ? (long long)g.es : 1;
    // the divisions in 32 bits while the grid has fewer than 2^31 points
    const bool i32 = npts < (1LL << 31);
    const long long nl = i32 ? (long long)((unsigned)npts / (unsigned)N) : npts / N;
    const long long local = l - a.line_start[d];
    const int s = i32 ? (int)((unsigned)local / (unsigned)nl) : (int)(local / nl);
    const long long l0 = local - (long long)s * nl;
    long long cnt = end - l;
    if (cnt > nl - l0) cnt = nl - l0;
    if (cnt > a.lmax[d]) cnt = a.lmax[d];
    const int L = (int)cnt;
    l += cnt;
    const bool owner = d == 0;
    if (kind == PK_LAST && !owner) continue;
    const int LS = lstride(N);
    cplx<FT> *b0 = tws + N;
    cplx<FT> *b1 = b0 + line_buf_elems(N, a.lmax[d]);
    __syncthreads();
    if (N != cur_n && kind != PK_LAST) {
      const cplx<FT> *twg = step_twiddles<T, FT>(g);
      for (int i = threadIdx.x; i < N; i += blockDim.x) tws[i] = twg[i];
      cur_n = N;
    }
    // first point of each line of the batch
    if (threadIdx.x < L) {
      const long long line = l0 + threadIdx.x;
      if (i32) {
        const unsigned q = (unsigned)line / (unsigned)stride;
        lbase[threadIdx.x] = (long long)((unsigned)line - q * (unsigned)stride) + (long long)q * stride * N;
      } else {
        lbase[threadIdx.x] = (line % stride) + (line / stride) * stride * N;
      }
    }
    __syncthreads();
    const int istr = (int)stride;  // element stride of a line (< 2^31 points per dimension block)
    // potential-matrix entries of row s
    const int ne = rc.ne[s];
    int ecol[RE], egid[RE], enim[RE];
    B ecoef[RE];
#pragma unroll
    for (int k = 0; k < RE; ++k) {
      ecol[k] = rc.col[s][k];
      egid[k] = rc.gid[s][k];
      ecoef[k] = rc.coef[s][k];
      enim[k] = rc.nim[s][k];
    }
    const bool unit_coef = rc.unit[s] != 0;
    const long long so = (long long)s * npts;
    const int tot = L * N;
    unsigned long long tg0 = tr ? gtimer() : 0;
    // the point of item idx of the batch: its offset and its shared-memory slot
    auto locate = [&](int idx, long long &p, int &sx) {
      int w, i;
      if (istr == 1) { w = idx / N; i = idx - w * N; }
      else { i = idx / L; w = idx - i * L; }
      sx = lidx(w, i, LS);
      p = lbase[w] + (long long)i * istr;
    };
    // phi_i at point p from its loaded operands (H phi_{i-1} = h + the
    // potential matrix, the offset, the recurrence); the row owner stores
    // phi_i, updates psi and its norm; the FFT input goes to slot sx
    auto finish = [&](long long p, int sx, cplx<B> h, const cplx<B> *pm, const B *vg, cplx<B> km2,
                      cplx<double> ps) {
      cplx<B> v = h;
      if (kind != PK_START) {
        cplx<B> self = pm[0];
#pragma unroll
        for (int j = 1; j < SM; ++j)
          if (j == s) self = pm[j];
#pragma unroll
        for (int k = 0; k < RE; ++k) {
          if (k < ne) {
            cplx<B> x = pm[0];
#pragma unroll
            for (int j = 1; j < SM; ++j)
              if (j == ecol[k]) x = pm[j];
            x = nim_operand(x, enim[k]);
            const B vv = unit_coef ? vg[k] : ecoef[k] * vg[k];
            h.re = fma_b(x.re, vv, h.re);
            h.im = fma_b(x.im, vv, h.im);
          }
        }
        cplx<B> bf;
        if (scaled) {
          h = add_soff(h, self, soh, sol);
          bf = srt ? mk(-h.im, h.re) : h;
          if (kind == PK_FIRST) bf = cmulr(bf, d2b<B>(0.5));
        } else {
          // (h - offset phi) * factor; a real offset and a purely imaginary
          // factor (real-time propagation) need half the multiplications
          cplx<B> hm;
          if (off_real) {
            hm.re = fma_b(-off.re, self.re, h.re);
            hm.im = fma_b(-off.re, self.im, h.im);
          } else {
            hm = h - cmul(off, self);
          }
          bf = fac_imag ? mk(-fac.im * hm.im, fac.im * hm.re) : cmul(hm, fac);
        }
        const long long gidx = so + p;
        if (kind == PK_FIRST) {
          v = bf;
          if (owner) {
            acc += cabs2(ps);
            st(phoutb + gidx, bf);
            const cplx<double> b = {b2d(bf.re), b2d(bf.im)};
            st(a.psi + gidx, mk(fma(b.re, a.a[1], ps.re * a.a[0]), fma(b.im, a.a[1], ps.im * a.a[0])));
          }
        } else {
          // bf +- km2: one exact fused multiply-add by the sign (no select
          // between two computed sums); double-float keeps its additions
          cplx<B> k2;
          if constexpr (std::is_same<B, dfl>::value) k2 = a.imag ? bf - km2 : bf + km2;
          else k2 = cplx<B>{fma_b(rsg, km2.re, bf.re), fma_b(rsg, km2.im, bf.im)};
          v = k2;
          if (owner) {
            st(phoutb + gidx, k2);
            ps.re = fma(coeff_i, b2d(k2.re), ps.re);
            ps.im = fma(coeff_i, b2d(k2.im), ps.im);
            st(a.psi + gidx, ps);
            acc = fma(ps.re, ps.re, fma(ps.im, ps.im, acc));
          }
        }
      }
      if (kind != PK_LAST) b0[sx] = v;
    };
    if constexpr (kStaged) {
      // operands staged in shared memory by asynchronous copies, kStageDepth
      // chunks of one point per thread in flight: the loads of the next
      // chunks overlap the arithmetic of this one.  Each thread reads only
      // what it copied itself, so no block barrier is needed between chunks.
      unsigned char *stage = reinterpret_cast<unsigned char *>(smem);
      const int t = threadIdx.x;
      const int nch = (tot + 255) >> 8;
      auto issue = [&](int ch) {
        const int idx = (ch << 8) + t;
        if (ch < nch && idx < tot) {
          long long p;
          int sx;
          locate(idx, p, sx);
          unsigned char *sl = stage + (size_t)(ch % kStageDepth) * kSlotBytes;
          if (kind == PK_START) {
            cp_async16(sl + t * 16, phim1b + so + p);
          } else {
#pragma unroll
            for (int dd = 0; dd < ND; ++dd)
              cp_async16(sl + (dd * 256 + t) * 16, reinterpret_cast<const cplx<B> *>(Pprev[dd]) + so + p);
#pragma unroll
            for (int j = 0; j < SM; ++j)
              if (j < a.S) cp_async16(sl + ((ND + j) * 256 + t) * 16, phim1b + (long long)j * npts + p);
            if (kind != PK_FIRST) cp_async16(sl + ((ND + SM) * 256 + t) * 16, phim2b + so + p);
#pragma unroll
            for (int k = 0; k < RE; ++k)
              if (k < ne) cp_async8(sl + kVgOff + (k * 256 + t) * 8, grids + (long long)egid[k] * npts + p);
            if (owner) cp_async16(sl + kPsOff + t * 16, a.psi + so + p);
          }
        }
        cp_async_commit();
      };
#pragma unroll
      for (int c = 0; c < kStageDepth - 1; ++c) issue(c);
      for (int ch = 0; ch < nch; ++ch) {
        issue(ch + kStageDepth - 1);
        cp_async_wait<kStageDepth - 1>();
        const int idx = (ch << 8) + t;
        if (idx >= tot) continue;
        long long p;
        int sx;
        locate(idx, p, sx);
        const unsigned char *sl = stage + (size_t)(ch % kStageDepth) * kSlotBytes;
        const cplx<B> *cb = reinterpret_cast<const cplx<B> *>(sl);
        if (kind == PK_START) {
          finish(p, sx, cb[t], nullptr, nullptr, cplx<B>{}, cplx<double>{});
          continue;
        }
        cplx<B> h = cb[t];
#pragma unroll
        for (int dd = 1; dd < ND; ++dd) h = h + cb[dd * 256 + t];
        cplx<B> pm[SM];
#pragma unroll
        for (int j = 0; j < SM; ++j) pm[j] = j < a.S ? cb[(ND + j) * 256 + t] : cplx<B>{};
        const cplx<B> km2 = kind != PK_FIRST ? cb[(ND + SM) * 256 + t] : cplx<B>{};
        B vg[RE];
        const B *vb = reinterpret_cast<const B *>(sl + kVgOff);
#pragma unroll
        for (int k = 0; k < RE; ++k) vg[k] = k < ne ? vb[k * 256 + t] : B(0);
        const cplx<double> ps = owner ? reinterpret_cast<const cplx<double> *>(sl + kPsOff)[t] : cplx<double>{};
        finish(p, sx, h, pm, vg, km2, ps);
      }
      cp_async_wait<0>();
    } else {
    for (int base = threadIdx.x; base < tot; base += UNR * blockDim.x) {
      long long pp[UNR];
      int sidx[UNR];
      // ---- gather
      cplx<B> hP[UNR], pm[UNR][SM], km2[UNR];
      B vg[UNR][RE];
      cplx<double> ps[UNR];
#pragma unroll
      for (int u = 0; u < UNR; ++u) {
        const int idx = base + u * blockDim.x;
        const bool ok = idx < tot;
        sidx[u] = -1;
        pp[u] = 0;
        if (!ok) continue;
        locate(idx, pp[u], sidx[u]);
        const long long p = pp[u];
        if (kind == PK_START) { hP[u] = ldcg(phim1b + so + p); continue; }
        cplx<B> h = ldcg(reinterpret_cast<const cplx<B> *>(Pprev[0]) + so + p);
#pragma unroll
        for (int dd = 1; dd < ND; ++dd) h = h + ldcg(reinterpret_cast<const cplx<B> *>(Pprev[dd]) + so + p);
        hP[u] = h;
#pragma unroll
        for (int j = 0; j < SM; ++j)
          if (j < a.S) pm[u][j] = ldcg(phim1b + (long long)j * npts + p);
#pragma unroll
        for (int k = 0; k < RE; ++k) vg[u][k] = k < ne ? ldg_b(grids + (long long)egid[k] * npts + p) : B(0);
        if (kind != PK_FIRST) km2[u] = ldcg(phim2b + so + p);
        if (owner) ps[u] = ldcg(a.psi + so + p);
      }
      // ---- compute and scatter
#pragma unroll
      for (int u = 0; u < UNR; ++u) {
        if (sidx[u] < 0) continue;
        finish(pp[u], sidx[u], hP[u], pm[u], vg[u], km2[u], ps[u]);
      }
    }
    }
    if (kind == PK_LAST) continue;
    __syncthreads();
    unsigned long long tg1 = tr ? gtimer() : 0;
    // T_d phi_i: forward FFT, k^2 multiply in the last forward stage, inverse
    // FFT whose last stage stores straight into Pnext[d] (lines fastest for
    // the strided dimensions, so the stores coalesce)
    const long long ks = (long long)s * N;
    const long long *lb = lbase;
    cplx<B> *dst = reinterpret_cast<cplx<B> *>(Pnext[d]) + so;
    kinetic_lines<FT>(
        b0, b1, g.rp, L, tws, [&g, ks](int, int i, cplx<FT> x) { return cmulr(x, step_kmul<T, FT>(g, ks + i)); },
        [dst, lb, istr](int w, int i, cplx<FT> x) { st(dst + lb[w] + (long long)i * istr, x); }, istr != 1);
    if (tr) {
      const unsigned long long tg2 = gtimer();
      tp[0] += tg1 - tg0; tp[1] += tg2 - tg1;
    }
  }
  __syncthreads();
}

// Point work of one term at point p for all states: H phi from the kinetic
// parts h[] and the potential matrix, then the recurrence.  Pre-scaled: h[]
// is already f T phi, the scaled entries carry f V, and -f offset is added
// as a value plus its residual, so no rounded constant multiplies every
// point coherently (that would scale or shift the series argument: a phase
// error growing with every step).
template <typename T, int SM, bool FIRST>
__device__ __forceinline__ void point_term(const StepArgs<T> &a, long long p, const cplx<T> *ph, cplx<T> *h,
                                           cplx<T> *kout, double coeff_i, int S, double &acc) {
  const bool scaled = a.scaled != 0;
  const Couplings *cpx = scaled ? a.scp : a.cp;
  const T *grids = scaled ? reinterpret_cast<const T *>(a.sgrids) : a.grids;
  const int ne = cpx->ne;
  for (int e = 0; e < ne; ++e) {
    const int r = cpx->row[e], c = cpx->col[e];
    const int ci = scaled ? cpx->lid[e] : e;
    const T gv = grids[(long long)cpx->gid[e] * a.npts + p];
    const T v = ci >= 0 ? (T)(a.coef[ci]) * gv : gv;
    const int nim = scaled ? 0 : cpx->nim[e];
#pragma unroll
    for (int s = 0; s < SM; ++s)
      if (s == r) {
#pragma unroll
        for (int q = 0; q < SM; ++q)
          if (q == c) h[s] = h[s] + cmulr(nim_operand(ph[q], nim), v);
      }
  }
  const cplx<T> off = ccast<T>(a.offset);
#pragma unroll
  for (int s = 0; s < SM; ++s) {
    if (s >= S) break;
    const long long g = (long long)s * a.npts + p;
    if (scaled) {
      const cplx<T> hs = add_soff<T>(h[s], ph[s], soff_part<T>(a.soff_hi, a.soff_lo, 0),
                                     soff_part<T>(a.soff_hi, a.soff_lo, 1));
      cplx<T> bf = a.scaled_rt ? mk(-hs.im, hs.re) : hs;
      if (FIRST) {
        bf = cmulr(bf, (T)0.5);
        const cplx<double> ps = ldcg(a.psi + g);
        acc += cabs2(ps);
        st(kout + g, bf);
        const cplx<double> b = ccast<double>(bf);
        st(a.psi + g, mk(ps.re * a.a[0] + b.re * a.a[1], ps.im * a.a[0] + b.im * a.a[1]));
      } else {
        const cplx<T> km2 = ldcg(kout + g);
        const cplx<T> k2 = a.imag ? bf - km2 : bf + km2;
        st(kout + g, k2);
        cplx<double> ps = ldcg(a.psi + g);
        ps.re += coeff_i * (double)k2.re;
        ps.im += coeff_i * (double)k2.im;
        st(a.psi + g, ps);
        acc += cabs2(ps);
      }
      continue;
    }
    if (FIRST) {
      const cplx<T> bf = cmul(h[s] - cmul(off, ph[s]), ccast<T>(a.fac1));
      const cplx<double> ps = ldcg(a.psi + g);
      acc += cabs2(ps);
      st(kout + g, bf);
      const cplx<double> b = ccast<double>(bf);
      st(a.psi + g, mk(ps.re * a.a[0] + b.re * a.a[1], ps.im * a.a[0] + b.im * a.a[1]));
    } else {
      const cplx<T> bf = cmul(h[s] - cmul(off, ph[s]), ccast<T>(a.fac));
      const cplx<T> km2 = ldcg(kout + g);
      const cplx<T> k2 = a.imag ? bf - km2 : bf + km2;
      st(kout + g, k2);
      cplx<double> ps = ldcg(a.psi + g);
      ps.re += coeff_i * (double)k2.re;
      ps.im += coeff_i * (double)k2.im;
      st(a.psi + g, ps);
      acc += cabs2(ps);
    }
  }
}

// One-dimensional grid: FFT, k^2, inverse FFT and point work of a tile of
// lines for all states in one block.
template <typename T, int SS, bool FIRST>
__device__ void phase_lines(const StepArgs<T> &a, const cplx<T> *phi, cplx<T> *kout, double coeff_i, double &acc,
                            cplx<T> *smem) {
  constexpr int SM = (SS > 0) ? SS : kMaxStates;
  const int S = (SS > 0) ? SS : a.S;
  const DimPass<T> &g = a.dp[0];
  const int N = g.N, TW = a.TW1;
  const int L = TW * S;
  const int LS = lstride(N);
  cplx<T> *tws = smem;
  cplx<T> *b0 = tws + N;
  cplx<T> *b1 = b0 + line_buf_elems(N, L);
  const long long ntiles = a.npts / ((long long)N * TW);
  for (long long tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const long long base = tile * TW * N;
    __syncthreads();
    for (int i = threadIdx.x; i < N; i += blockDim.x) tws[i] = g.tw[i];
    for (int idx = threadIdx.x; idx < L * N; idx += blockDim.x) {
      const int l = idx / N, i = idx - l * N;
      const int s = l / TW, w = l - s * TW;
      b0[lidx(l, i, LS)] = ldcg(phi + (long long)s * a.npts + base + (long long)w * N + i);
    }
    __syncthreads();
    // an even number of stages: the inverse FFT's last stage writes b0
    const T *kt = g.ktab;
    kinetic_lines<T>(
        b0, b1, g.rp, L, tws, [kt, N, TW](int l, int i, cplx<T> x) { return cmulr(x, __ldg(kt + (l / TW) * N + i)); },
        [b0, LS](int l, int i, cplx<T> x) { b0[lidx(l, i, LS)] = x; }, false);
    __syncthreads();
    for (int idx = threadIdx.x; idx < TW * N; idx += blockDim.x) {
      const int w = idx / N, i = idx - w * N;
      const long long p = base + (long long)w * N + i;
      cplx<T> ph[SM], h[SM];
#pragma unroll
      for (int s = 0; s < SM; ++s)
        if (s < S) {
          ph[s] = ldcg(phi + (long long)s * a.npts + p);
          h[s] = b0[lidx(s * TW + w, i, LS)];
        }
      point_term<T, SM, FIRST>(a, p, ph, h, kout, coeff_i, S, acc);
    }
  }
  __syncthreads();
}

// The series cut of the reference after a term's norm sum (identical in
// every block).  Returns true when the series stops.
__device__ __forceinline__ bool step_cut(const double tot, const double norm0, double &last, double &norm_last,
                                         int imag, int diff, double prec, int offim0, int &status) {
  bool done = false;
  if (!isfinite(tot)) { done = true; status = 2; }
  else if (!imag) {
    // OCheby.cpp:179-182 (mixed precision: change against the previous term)
    const double ref = diff ? last : norm0;
    if (fabs(ref - tot) / norm0 < prec && offim0) done = true;
  } else {
    // OCheby.cpp:286-289
    if (fabs(tot - norm_last) / norm_last < prec) done = true;
    norm_last = tot;
  }
  last = tot;
  return done;
}

// OCC: minimum resident blocks per SM the compiler must allow for (register
// cap).  The FP32 kernel is latency bound and needs the warps; the binary64
// and double-float ones are bound by their arithmetic and take all registers.
template <typename T, typename FT, int SS, int ND, int OCC>
__global__ void __launch_bounds__(256, OCC) cheby_step_kernel(StepArgs<T> a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ double red[32];
  __shared__ double tot_s;
  __shared__ bool done_s;  // the series cut of the term, decided by thread 0
  constexpr int SM = (SS > 0) ? SS : kMaxStates;
  cplx<T> *smem = reinterpret_cast<cplx<T> *>(smem_raw);
  const long long n = a.npts * a.S;
  const long long gtid = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  const long long gstride = (long long)gridDim.x * blockDim.x;
  const bool tr = a.trace && blockIdx.x == (unsigned)(a.trace - 1) && threadIdx.x == 0;
  unsigned long long tp[4] = {0, 0, 0, 0};
  unsigned long long *tpi = tp;  // gather, FFT + multiply + store (inside the phase), -, barrier

  // phi_0 = psi (OCheby: ket0->FastCopy(*Psi)), in the bulk type of the phases
  for (long long i = gtid; i < n; i += gstride) {
    const cplx<double> p = ld(a.psi + i);
    if constexpr (ND == 1) st(a.buf[0] + i, ccast<T>(p));
    else st(reinterpret_cast<cplx<FT> *>(a.buf[0]) + i, cplx<FT>{d2b<FT>(p.re), d2b<FT>(p.im)});
  }
  if (!grid_sync(a.bar)) return;

  double acc = 0.0, t;
  double norm0 = 0.0, last = 0.0, norm_last = 0.0;
  bool done = false;
  int status = 0, used = 2;

  if constexpr (ND == 1) {
    // first two terms; the reduction gives the raw norm of psi before the step
    phase_lines<T, SS, true>(a, a.buf[0], a.buf[1], 0.0, acc, smem);
    t = block_sum(acc, red);
    if (threadIdx.x == 0) a.partials[blockIdx.x] = t;
    if (!grid_sync(a.bar)) return;
    t = sum_partials(a.partials, red);
    if (threadIdx.x == 0) tot_s = t;
    __syncthreads();
    norm0 = last = tot_s;
    done = !isfinite(norm0);
    if (done) status = 2;
    for (int i = 2; i < a.order && !done; ++i) {
      const cplx<T> *phi = a.buf[(i + 1) & 1];
      cplx<T> *kout = a.buf[i & 1];
      acc = 0.0;
      phase_lines<T, SS, false>(a, phi, kout, a.a[i], acc, smem);
      t = block_sum(acc, red);
      if (threadIdx.x == 0) a.partials[blockIdx.x] = t;
      if (!grid_sync(a.bar)) return;
      t = sum_partials(a.partials, red);
      // the cut in one thread (its binary64 division costs every warp that
      // runs it a chain of FP64 pipe slots), the decision broadcast
      if (threadIdx.x == 0) {
        tot_s = t;
        done_s = step_cut(t, norm0, last, norm_last, a.imag, a.diff, a.prec, a.offim0, status);
      }
      __syncthreads();
      used = i + 1;
      done = done_s;
    }
  } else {
    int tw_n = -1;  // line length of the twiddles held in shared memory
    // raw storage: the double-float coefficient type has constructors
    __shared__ __align__(16) unsigned char rows_raw[sizeof(RowCache<FT>)];
    RowCache<FT> &rows = *reinterpret_cast<RowCache<FT> *>(rows_raw);
    fill_rows(a, rows);
    __syncthreads();
    const long long all = a.line_start[ND];
    // the lines of a term: all of them in one phase, or dimension 0 (phase A)
    // and then the others (phase B) for grids of three or more dimensions
    const bool two = a.two_phase != 0;
    const long long *bsA = two ? a.bstartA : a.bstart;
    const long long hiA = two ? a.line_start[1] : all;
    // phase B: T_d phi_i for d >= 1 from the stored phi_i
    auto phase_b = [&](const cplx<T> *phi_i, cplx<T> *const *Pnext) -> bool {
      double dummy = 0.0;
      phase_fused<T, FT, ND, SM>(a, PK_START, phi_i, nullptr, nullptr, nullptr, Pnext, 0.0, dummy, smem, tw_n, rows,
                                 a.bstartB, a.line_start[1], all);
      return grid_sync(a.bar);
    };
    // phase 1: T_d phi_0 -> P[1] (all dimensions)
    phase_fused<T, FT, ND, SM>(a, PK_START, a.buf[0], nullptr, nullptr, nullptr, a.Pn[1], 0.0, acc, smem, tw_n, rows,
                               a.bstart, 0, all);
    if (!grid_sync(a.bar)) return;
    // phase 2: phi_1 (+ psi = a0 psi + a1 phi_1, raw norm of psi) and T_d phi_1 -> P[0]
    acc = 0.0;
    const int kind1 = a.order > 2 ? PK_FIRST : PK_LAST;
    phase_fused<T, FT, ND, SM>(a, kind1, a.buf[0], nullptr, a.buf[1], a.Pn[1], a.Pn[0], 0.0, acc, smem, tw_n, rows,
                               bsA, 0, hiA);
    t = block_sum(acc, red);
    if (threadIdx.x == 0) a.partials[blockIdx.x] = t;
    if (!grid_sync(a.bar)) return;
    t = sum_partials(a.partials, red);
    if (threadIdx.x == 0) tot_s = t;
    __syncthreads();
    norm0 = last = tot_s;
    done = !isfinite(norm0);
    if (done) status = 2;
    if (two && !done && kind1 != PK_LAST && !phase_b(a.buf[1], a.Pn[0])) return;
    // phase i+1: phi_i from P[i&1], phi_{i-1} = buf[(i-1)%3], phi_{i-2} = buf[(i-2)%3] -> buf[i%3]
    for (int i = 2; i < a.order && !done; ++i) {
      const unsigned long long t0 = tr ? gtimer() : 0;
      acc = 0.0;
      const int kind = (i + 1 < a.order) ? PK_TERM : PK_LAST;
      phase_fused<T, FT, ND, SM>(a, kind, a.buf[(i - 1) % 3], a.buf[(i - 2) % 3], a.buf[i % 3], a.Pn[i & 1],
                                 a.Pn[(i + 1) & 1], a.a[i], acc, smem, tw_n, rows, bsA, 0, hiA,
                                 tr ? tpi : nullptr);
      const unsigned long long t1 = tr ? gtimer() : 0;
      t = block_sum(acc, red);
      if (threadIdx.x == 0) a.partials[blockIdx.x] = t;
      if (!grid_sync(a.bar)) return;
      if (tr) tp[3] += gtimer() - t1;
      t = sum_partials(a.partials, red);
      if (threadIdx.x == 0) {
        tot_s = t;
        done_s = step_cut(t, norm0, last, norm_last, a.imag, a.diff, a.prec, a.offim0, status);
      }
      __syncthreads();
      used = i + 1;
      done = done_s;
      if (two && !done && kind != PK_LAST && !phase_b(a.buf[i % 3], a.Pn[(i + 1) & 1])) return;
      if (tr) tp[2] += gtimer() - t0;  // the whole term
    }
  }

  // common phase exp(c0 offset) of all coefficients
  for (long long i = gtid; i < n; i += gstride) st(a.psi + i, cmul(ldcg(a.psi + i), a.ph));
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    a.cs->terms = used;
    a.cs->total += used;
    a.cs->status = status;
    a.cs->norm0 = norm0;
  }
  if (tr)
    for (int k = 0; k < 4; ++k) a.cs->t_phase[k] += tp[k];
}

// Kernel entry for S states (1, 2, or any up to kMaxStates) of one bulk type
// and grid rank.
template <typename T, typename FT, int ND, int OCC>
void *step_kernel_for(int S) {
  return S == 1 ? (void *)cheby_step_kernel<T, FT, 1, ND, OCC>
                : S == 2 ? (void *)cheby_step_kernel<T, FT, 2, ND, OCC> : (void *)cheby_step_kernel<T, FT, 0, ND, OCC>;
}

}  // namespace qdg
