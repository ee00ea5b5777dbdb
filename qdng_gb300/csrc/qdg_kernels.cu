// qdg_kernels.cu -- sm_103a kernels of the propagation engine.
//
// The hot kernel is the line pass: a block loads a tile of grid lines along
// one dimension for one or all electronic states, runs the unnormalised FFT
// in shared memory, multiplies by the k-space kinetic factor, transforms
// back, and finishes with an epilogue.  A Hamiltonian application over a
// D-dimensional grid is D passes (the kinetic operator is separable:
// T = sum_d T_d, T_d = IFFT_d k_d^2/(2m_d) FFT_d / N_d, which equals
// QDng's IFFT_nd [sum_d k_d^2/(2m_d)] FFT_nd / N of Diff::DnDxn,
// src/qdlib/Diff.cpp:203-218).  The last pass adds the potential matrix and,
// for the Chebyshev propagator, runs the three-term recurrence, the psi
// accumulation and the norm reduction in the same sweep
// (src/qdlib/OCheby.cpp:92-198, 200-297).
#include <cuda_runtime.h>
#include <math.h>

#include <atomic>

#include "qdg_kernels.cuh"

namespace qdg {

static std::atomic<long long> g_launches{0};
long long launch_counter() { return g_launches.load(); }
void add_launches(long long n) { g_launches.fetch_add(n); }
#define COUNT_LAUNCH() g_launches.fetch_add(1)

__device__ __forceinline__ cplx<double> dmul(cplx<double> a, cplx<double> b) { return cmul(a, b); }

// x (hi + lo) for a factor carried beyond binary64 (lo: the rounding residual
// of hi): the small part is added inside the fused products, so the result is
// not scaled by hi's rounding.  Multiplying every term of a Chebyshev series
// by the rounded factor 2 exp/scaling would scale the series argument by
// (1 + d), a phase error that grows with every time step.
__device__ __forceinline__ cplx<double> dmul2(cplx<double> x, cplx<double> hi, cplx<double> lo) {
  const double sre = x.re * lo.re - x.im * lo.im, sim = x.re * lo.im + x.im * lo.re;
  return mk(fma(x.re, hi.re, fma(-x.im, hi.im, sre)), fma(x.re, hi.im, fma(x.im, hi.re, sim)));
}


// Block-level end of a Chebyshev term: store this block's norm partial, and
// let the last block to arrive sum all partials in block order and apply the
// reference's series cut.  No block waits for another (threadfence
// reduction: the last arriving block does the work).
__device__ void cheby_term_finish(double acc, double *red, double *partials, const ChebyCut &cut, int term) {
  __shared__ int am_last;
  const double t = block_sum(acc, red);
  if (threadIdx.x == 0) {
    partials[blockIdx.x] = t;
    __threadfence();
    const unsigned int prev = atomicAdd(&cut.cs->arrive, 1u);
    am_last = (prev == gridDim.x - 1) ? 1 : 0;
  }
  __syncthreads();
  if (!am_last) return;
  __threadfence();
  double v = 0.0;
  for (int i = threadIdx.x; i < (int)gridDim.x; i += blockDim.x) v += __ldcg(partials + i);
  const double tot = block_sum(v, red);
  if (threadIdx.x != 0) return;
  ChebyState *cs = cut.cs;
  cs->arrive = 0;
  if (!isfinite(tot)) {
    cs->status = 2; cs->done = 1; cs->terms = cut.first ? 2 : term + 1;
  } else if (cut.first) {
    cs->norm0 = tot;
    cs->acc_last = tot;
  } else if (!cut.imag) {
    const double ref = cut.diff ? cs->acc_last : cs->norm0;
    const double nconv = fabs(ref - tot) / cs->norm0;
    if (nconv < cut.prec && cut.offim0) { cs->done = 1; cs->terms = term + 1; }
    cs->acc_last = tot;
  } else {
    if (fabs(tot - cs->norm_last) / cs->norm_last < cut.prec) { cs->done = 1; cs->terms = term + 1; }
    cs->norm_last = tot;
  }
  if (cut.use_cond) {
    const int next = cut.first ? 2 : term + 1;
    if (cs->done || next >= cut.order) cudaGraphSetConditional(cut.cond, 0u);
    else cs->i = next;
  }
}

template <typename T, int MODE, int SS>
__global__ void __launch_bounds__(256) linepass_kernel(PassArgs<T> a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ double red[32];
  if (a.done != nullptr && *a.done) return;  // Chebyshev series already converged

  const int N = a.N;
  const int TW = a.TW;
  const int nsub = a.nsub;
  const int L = TW * nsub;
  const int LS = lstride(N);
  cplx<T> *tws = reinterpret_cast<cplx<T> *>(smem_raw);
  cplx<T> *b0 = tws + N;
  cplx<T> *b1 = b0 + line_buf_elems(N, L);
  for (int i = threadIdx.x; i < N; i += blockDim.x) tws[i] = a.tw[i];
  __syncthreads();

  double acc = 0.0;
  const int nsplit = a.S / nsub;
  const long long nitems = a.ntiles * nsplit;
  const long long npts = a.npts;
  const int S = (SS > 0) ? SS : a.S;
  int term = a.cut.term;
  const cplx<T> *phi = a.phi;
  cplx<T> *kout = a.k0;
  cplx<double> coeff = a.coeff;
  if (a.cut.dyn) {
    term = a.cut.cs->i;
    phi = a.bufs[(term + 1) & 1];
    kout = const_cast<cplx<T> *>(a.bufs[term & 1]);
    coeff = a.cut.coeffs[term];
  }

  for (long long item = blockIdx.x; item < nitems; item += gridDim.x) {
    const long long tile = item / nsplit;
    const int s0 = (int)(item - tile * nsplit) * nsub;
    const long long hi = tile / a.tiles_per_hi;
    const long long base = hi * a.hi_stride + (tile - hi * a.tiles_per_hi) * TW;

    // load the tile: smem line (sl*TW + w), element i
    const int tileN = TW * N;
    for (int idx = threadIdx.x; idx < nsub * tileN; idx += blockDim.x) {
      const int sl = idx / tileN;
      int w, i;
      tile_coord(idx - sl * tileN, TW, N, a.es, w, i);
      const long long p = base + (long long)w * a.ls + (long long)i * a.es;
      b0[lidx(sl * TW + w, i, LS)] = ld(phi + (long long)(s0 + sl) * npts + p);
    }
    __syncthreads();

    int cur = fft_lines<T>(b0, b1, a.rp, L, tws, -1);
    cplx<T> *bc = cur ? b1 : b0;
    for (int idx = threadIdx.x; idx < L * N; idx += blockDim.x) {
      const int l = idx / N;
      const int i = idx - l * N;
      const int s = s0 + l / TW;
      const int x = lidx(l, i, LS);
      if (MODE == PM_GSPO_KIN) {
        bc[x] = cmul(bc[x], a.gtab[(long long)s * N + i]);
      } else {
        const int kq = min(i, N - i);
        const T f = (T)(a.kfac[s] * (double)kq * (double)kq);
        bc[x] = cmulr(bc[x], f);
      }
    }
    __syncthreads();
    int cur2 = fft_lines<T>(bc, cur ? b0 : b1, a.rp, L, tws, +1);
    // fft_lines returns the index relative to its own (bc, other) pair
    cplx<T> *res = cur2 ? (cur ? b0 : b1) : bc;

    if (MODE == PM_KIN_FIRST || MODE == PM_KIN_ACC || MODE == PM_GSPO_KIN) {
      for (int idx = threadIdx.x; idx < nsub * tileN; idx += blockDim.x) {
        const int sl = idx / tileN;
        int w, i;
        tile_coord(idx - sl * tileN, TW, N, a.es, w, i);
        const long long p = base + (long long)w * a.ls + (long long)i * a.es;
        const long long g = (long long)(s0 + sl) * npts + p;
        cplx<T> v = res[lidx(sl * TW + w, i, LS)];
        if (MODE == PM_KIN_FIRST) st(a.P + g, v);
        else if (MODE == PM_KIN_ACC) st(a.P + g, ld(a.P + g) + v);
        else st(a.out + g, v);
      }
    } else {
      // coupled epilogue: every point of the tile for all S states
      for (int idx = threadIdx.x; idx < tileN; idx += blockDim.x) {
        int w, i;
        tile_coord(idx, TW, N, a.es, w, i);
        const long long p = base + (long long)w * a.ls + (long long)i * a.es;
        cplx<T> ph[(SS > 0) ? SS : kMaxStates];
        cplx<T> h[(SS > 0) ? SS : kMaxStates];
#pragma unroll
        for (int s = 0; s < ((SS > 0) ? SS : kMaxStates); ++s) {
          if (s < S) {
            ph[s] = ld(phi + (long long)s * npts + p);
            h[s] = res[lidx(s * TW + w, i, LS)];
            if (a.multi_pass) h[s] = h[s] + ld(a.P + (long long)s * npts + p);
          }
        }
        const int ne = a.cp->ne;
        for (int e = 0; e < ne; ++e) {
          const int r = a.cp->row[e], c = a.cp->col[e];
          const T v = (T)(a.coef[e]) * a.grids[(long long)a.cp->gid[e] * npts + p];
          const int nim = a.cp->nim[e];
#pragma unroll
          for (int s = 0; s < ((SS > 0) ? SS : kMaxStates); ++s)
            if (s == r) {
#pragma unroll
              for (int q = 0; q < ((SS > 0) ? SS : kMaxStates); ++q)
                if (q == c) h[s] = h[s] + cmulr(nim_operand(ph[q], nim), v);
            }
        }
#pragma unroll
        for (int s = 0; s < ((SS > 0) ? SS : kMaxStates); ++s) {
          if (s >= S) break;
          const long long g = (long long)s * npts + p;
          if (MODE == PM_HAPPLY) {
            st(a.out + g, h[s]);
          } else {
            const cplx<double> hd = ccast<double>(h[s]);
            const cplx<double> pd = ccast<double>(ph[s]);
            const cplx<double> bf = dmul2(hd - dmul(a.offset, pd), a.fac, a.fac_lo);
            if (MODE == PM_CHEBY_FIRST) {
              const cplx<double> ps = ld(a.psi + g);
              acc += cabs2(ps);
              st(kout + g, ccast<T>(bf));                      // phi_1
              st(a.psi + g, dmul(ps, a.c0p) + dmul(bf, a.c1p)); // psi*c0 + phi_1*c1
            } else {
              const cplx<double> km2 = ccast<double>(ld(kout + g));
              const cplx<double> k2 = a.imag ? bf - km2 : bf + km2;
              st(kout + g, ccast<T>(k2));
              const cplx<double> ps = ld(a.psi + g) + dmul(k2, coeff);
              st(a.psi + g, ps);
              acc += cabs2(ps);
            }
          }
        }
      }
    }
    __syncthreads();
  }
  if (MODE == PM_CHEBY_FIRST || MODE == PM_CHEBY_TERM) cheby_term_finish(acc, red, a.partials, a.cut, term);
}

// ------------------------------------------------ all-dimension kinetic pass
// Work items are (dimension, line tile, state); each computes T_d phi on its
// lines with the shared-memory FFT and stores it to P_d.
template <typename T>
__global__ void __launch_bounds__(256) kin_all_kernel(KinArgs<T> a) {
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
    const cplx<T> *src = phi + (long long)s * npts;
    for (int idx = threadIdx.x; idx < tileN; idx += blockDim.x) {
      int w, i;
      tile_coord(idx, TW, N, g.es, w, i);
      b0[lidx(w, i, LS)] = ld(src + base + (long long)w * g.ls + (long long)i * g.es);
    }
    __syncthreads();
    const int cur = fft_lines<T>(b0, b1, g.rp, TW, tws, -1);
    cplx<T> *bc = cur ? b1 : b0;
    const double kf = g.kfac[s];
    for (int idx = threadIdx.x; idx < tileN; idx += blockDim.x) {
      const int w = idx / N, i = idx - w * N;
      const int kq = min(i, N - i);
      const int x = lidx(w, i, LS);
      bc[x] = cmulr(bc[x], (T)(kf * (double)kq * (double)kq));
    }
    __syncthreads();
    const int cur2 = fft_lines<T>(bc, cur ? b0 : b1, g.rp, TW, tws, +1);
    const cplx<T> *res = cur2 ? (cur ? b0 : b1) : bc;
    cplx<T> *dst = g.P + (long long)s * npts;
    for (int idx = threadIdx.x; idx < tileN; idx += blockDim.x) {
      int w, i;
      tile_coord(idx, TW, N, g.es, w, i);
      st(dst + base + (long long)w * g.ls + (long long)i * g.es, res[lidx(w, i, LS)]);
    }
    __syncthreads();
  }
}

// ------------------------------------ short binary64 lines, radix 2
// A block takes L lines of one dimension and state, N/2 threads per line.
// Stockham radix-2 stage with Ns: for j < N/2, k = j mod Ns, a = x[j],
// b = x[j + N/2], w = exp(-+2 pi i k / (2 Ns)): outputs (j / Ns) 2 Ns + k
// = a + w b and that + Ns = a - w b.  Thread (l, j) computes butterfly j of
// line l (w b once, eight binary64 instructions); a binary64 warp
// instruction holds its sub-partition's FP64 unit for ~70-80 cycles, so
// the lines are kept short per block (L = 1 from 128 points on) and a
// transform costs log2 N such stages instead of a radix-8/16 item's chain.
__global__ void __launch_bounds__(512) kin_r2_kernel(KinR2Args a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  if (a.done != nullptr && *a.done) return;
  const cplx<double> *phi = a.dyn ? a.bufs[(a.cs->i + 1) & 1] : a.phi;
  int d = 0;
  while ((long long)blockIdx.x >= a.item_start[d + 1]) ++d;
  const int N = a.N[d], L = a.L[d], lg = a.lgN[d], half = N >> 1;
  const long long local = (long long)blockIdx.x - a.item_start[d];
  const int s = (int)(local / a.groups[d]);
  const long long g = local - (long long)s * a.groups[d];
  const long long str = a.stride[d];
  const long long so = (long long)s * a.npts;
  const cplx<double> *tw = a.tw[d];
  cplx<double> *b0 = reinterpret_cast<cplx<double> *>(smem_raw);
  cplx<double> *b1 = b0 + L * N;
  // line g L + l: dimension 0 lines are contiguous; others are (lo, hi) with
  // lo = line mod stride fastest, so consecutive lines are adjacent in memory
  auto addr = [&](int l, int i) -> long long {
    const long long line = g * L + l;
    if (d == 0) return so + line * N + i;
    const long long hi = line / str, lo = line - hi * str;
    return so + hi * str * N + lo + (long long)i * str;
  };
  const int T = L * N;
  for (int idx = threadIdx.x; idx < T; idx += blockDim.x) {
    int l, i;
    if (d == 0) { l = idx / N; i = idx - l * N; } else { i = idx / L; l = idx - i * L; }
    b0[l * N + i] = ld(phi + addr(l, i));
  }
  __syncthreads();
  const int t = threadIdx.x;
  const bool act = t < L * half;
  const int l = t >> (lg - 1), j = t & (half - 1);
  cplx<double> *in = b0, *out = b1;
  for (int dir = 0; dir < 2; ++dir) {  // forward, then backward (conjugate twiddles)
    for (int Ns = 1, ls = 0; Ns < N; Ns <<= 1, ++ls) {
      if (act) {
        const int k = j & (Ns - 1);
        const cplx<double> x = in[l * N + j], y = in[l * N + j + half];
        const cplx<double> w0 = tw[k << (lg - 1 - ls)];
        const double wr = w0.re, wi = dir == 0 ? w0.im : -w0.im;
        const double pr = fma(wr, y.re, -wi * y.im), pi = fma(wr, y.im, wi * y.re);
        const int dst = l * N + ((j - k) << 1) + k;
        out[dst] = cplx<double>{x.re + pr, x.im + pi};
        out[dst + Ns] = cplx<double>{x.re - pr, x.im - pi};
      }
      __syncthreads();
      cplx<double> *tmp = in;
      in = out;
      out = tmp;
    }
    if (dir == 0) {
      // k^2 / (2 m) / N at k-index q = min(i, N - i), the kinetic pass's multiplier
      for (int idx = threadIdx.x; idx < T; idx += blockDim.x) {
        const int ll = idx / N, o = idx - ll * N;
        const int q = o < N - o ? o : N - o;
        const double m = a.kfac[d][s] * (double)q * (double)q;
        in[idx] = cplx<double>{in[idx].re * m, in[idx].im * m};
      }
      __syncthreads();
    }
  }
  for (int idx = threadIdx.x; idx < T; idx += blockDim.x) {
    int ll, i;
    if (d == 0) { ll = idx / N; i = idx - ll * N; } else { i = idx / L; ll = idx - i * L; }
    st(a.P[d] + addr(ll, i), in[ll * N + i]);
  }
}

cudaError_t launch_kin_r2(const KinR2Args &a, cudaStream_t st) {
  size_t smem = 0;
  for (int d = 0; d < a.nd; ++d) smem = std::max(smem, 2 * (size_t)a.L[d] * a.N[d] * sizeof(cplx<double>));
  if (smem > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(kin_r2_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
  }
  kin_r2_kernel<<<(unsigned)a.item_start[a.nd], a.threads, smem, st>>>(a);
  COUNT_LAUNCH();
  return cudaGetLastError();
}

// ---------------------------------------------------------------- NAC pass
// A tile of TW lines along d: phi lines and f phi lines are transformed
// together (2 TW lines), multiplied by i k c / N, transformed back, and the
// row state's T_0 phi gets f * (first half) + (second half).  Every point
// belongs to one line of one tile, so the read-modify-write is race free;
// the elements and dimensions of one H application are separate launches.
template <typename T>
__global__ void __launch_bounds__(256) nac_kernel(NacArgs<T> a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  if (a.done != nullptr && *a.done) return;
  const cplx<T> *phi = (a.dyn ? a.bufs[(a.cs->i + 1) & 1] : a.phi) + (long long)a.col * a.npts;
  const int N = a.N, TW = a.TW;
  const int LS = lstride(N);
  cplx<T> *tws = reinterpret_cast<cplx<T> *>(smem_raw);
  cplx<T> *b0 = tws + N;
  cplx<T> *b1 = b0 + line_buf_elems(N, 2 * TW);
  for (int i = threadIdx.x; i < N; i += blockDim.x) tws[i] = a.tw[i];
  const int tileN = TW * N;
  for (long long tile = blockIdx.x; tile < a.ntiles; tile += gridDim.x) {
    const long long hi = tile / a.tiles_per_hi;
    const long long base = hi * a.hi_stride + (tile - hi * a.tiles_per_hi) * TW;
    __syncthreads();
    for (int idx = threadIdx.x; idx < tileN; idx += blockDim.x) {
      int w, i;
      tile_coord(idx, TW, N, a.es, w, i);
      const long long g = base + (long long)w * a.ls + (long long)i * a.es;
      const cplx<T> x = ld(phi + g);
      b0[lidx(w, i, LS)] = x;
      b0[lidx(TW + w, i, LS)] = cmulr(x, a.f[g]);
    }
    __syncthreads();
    const int cur = fft_lines<T>(b0, b1, a.rp, 2 * TW, tws, -1);
    cplx<T> *bc = cur ? b1 : b0;
    for (int idx = threadIdx.x; idx < 2 * tileN; idx += blockDim.x) {
      const int l = idx / N, i = idx - l * N;
      const int q = i < (N + 1) / 2 ? i : i - N;  // Kspace::Init1Dddx order, Nyquist negative
      const T m = (T)(a.kfac * (double)q);
      const int x = lidx(l, i, LS);
      const cplx<T> v = bc[x];
      bc[x] = mk(-v.im * m, v.re * m);
    }
    __syncthreads();
    const int cur2 = fft_lines<T>(bc, cur ? b0 : b1, a.rp, 2 * TW, tws, +1);
    const cplx<T> *res = cur2 ? (cur ? b0 : b1) : bc;
    for (int idx = threadIdx.x; idx < tileN; idx += blockDim.x) {
      int w, i;
      tile_coord(idx, TW, N, a.es, w, i);
      const long long g = base + (long long)w * a.ls + (long long)i * a.es;
      const cplx<T> add = cmulr(res[lidx(w, i, LS)], a.f[g]) + res[lidx(TW + w, i, LS)];
      st(a.out + g, ld(a.out + g) + add);
    }
  }
}

template <typename T>
cudaError_t launch_nac(const NacArgs<T> &a, int grid, int block, size_t smem, cudaStream_t st) {
  void *k = (void *)nac_kernel<T>;
  if (smem > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
  }
  void *args[] = {(void *)&a};
  COUNT_LAUNCH();
  return cudaLaunchKernel(k, dim3(grid), dim3(block), args, smem, st);
}

template <typename T>
int nac_max_blocks(int block, size_t smem) {
  void *k = (void *)nac_kernel<T>;
  if (smem > 48 * 1024) cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  int nb = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k, block, smem) != cudaSuccess) return 1;
  return nb > 0 ? nb : 1;
}

template cudaError_t launch_nac<double>(const NacArgs<double> &, int, int, size_t, cudaStream_t);
template cudaError_t launch_nac<float>(const NacArgs<float> &, int, int, size_t, cudaStream_t);
template int nac_max_blocks<double>(int, size_t);
template int nac_max_blocks<float>(int, size_t);

// ------------------------------------------------------------ combine pass
template <typename T, int MODE, int SS>
__global__ void __launch_bounds__(256) combine_kernel(CombArgs<T> a) {
  __shared__ double red[32];
  if (a.cut.cs != nullptr && a.cut.cs->done) return;
  const long long npts = a.npts;
  const int S = (SS > 0) ? SS : a.S;
  constexpr int SM = (SS > 0) ? SS : kMaxStates;
  double acc = 0.0;
  int term = a.cut.term;
  const cplx<T> *phi = a.phi;
  cplx<T> *kout = a.k0;
  cplx<double> coeff = a.coeff;
  if (a.cut.dyn) {
    term = a.cut.cs->i;
    phi = a.bufs[(term + 1) & 1];
    kout = const_cast<cplx<T> *>(a.bufs[term & 1]);
    coeff = a.cut.coeffs[term];
  }
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < npts; p += (long long)gridDim.x * blockDim.x) {
    cplx<T> ph[SM], h[SM];
#pragma unroll
    for (int s = 0; s < SM; ++s) {
      if (s < S) {
        const long long g = (long long)s * npts + p;
        ph[s] = ld(phi + g);
        cplx<T> v = ld(a.P[0] + g);
        for (int d = 1; d < a.nd; ++d) v = v + ld(a.P[d] + g);
        h[s] = v;
      }
    }
    const int ne = a.cp->ne;
    for (int e = 0; e < ne; ++e) {
      const int r = a.cp->row[e], c = a.cp->col[e];
      const T v = (T)(a.coef[e]) * a.grids[(long long)a.cp->gid[e] * npts + p];
      const int nim = a.cp->nim[e];
#pragma unroll
      for (int s = 0; s < SM; ++s)
        if (s == r) {
#pragma unroll
          for (int q = 0; q < SM; ++q)
            if (q == c) h[s] = h[s] + cmulr(nim_operand(ph[q], nim), v);
        }
    }
#pragma unroll
    for (int s = 0; s < SM; ++s) {
      if (s >= S) break;
      const long long g = (long long)s * npts + p;
      if (MODE == PM_HAPPLY) {
        st(a.out + g, h[s]);
      } else {
        const cplx<double> bf = dmul2(ccast<double>(h[s]) - dmul(a.offset, ccast<double>(ph[s])), a.fac, a.fac_lo);
        if (MODE == PM_CHEBY_FIRST) {
          const cplx<double> ps = ld(a.psi + g);
          acc += cabs2(ps);
          st(kout + g, ccast<T>(bf));
          st(a.psi + g, dmul(ps, a.c0p) + dmul(bf, a.c1p));
        } else {
          const cplx<double> km2 = ccast<double>(ld(kout + g));
          const cplx<double> k2 = a.imag ? bf - km2 : bf + km2;
          st(kout + g, ccast<T>(k2));
          const cplx<double> ps = ld(a.psi + g) + dmul(k2, coeff);
          st(a.psi + g, ps);
          acc += cabs2(ps);
        }
      }
    }
  }
  if (MODE == PM_CHEBY_FIRST || MODE == PM_CHEBY_TERM) cheby_term_finish(acc, red, a.partials, a.cut, term);
}

template <typename T>
cudaError_t launch_kin_all(const KinArgs<T> &a, int grid, int block, size_t smem, cudaStream_t st) {
  void *k = (void *)kin_all_kernel<T>;
  if (smem > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
  }
  void *args[] = {(void *)&a};
  COUNT_LAUNCH();
  return cudaLaunchKernel(k, dim3(grid), dim3(block), args, smem, st);
}

template <typename T>
int kin_all_max_blocks(int block, size_t smem) {
  void *k = (void *)kin_all_kernel<T>;
  if (smem > 48 * 1024) cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  int nb = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k, block, smem) != cudaSuccess) return 1;
  return nb > 0 ? nb : 1;
}

template <typename T, int MODE>
static void *comb_ptr(int S) {
  return S == 1 ? (void *)combine_kernel<T, MODE, 1> : S == 2 ? (void *)combine_kernel<T, MODE, 2>
                                                              : (void *)combine_kernel<T, MODE, 0>;
}

template <typename T>
cudaError_t launch_combine(int mode, const CombArgs<T> &a, int grid, int block, cudaStream_t st) {
  void *k = mode == PM_HAPPLY ? comb_ptr<T, PM_HAPPLY>(a.S)
            : mode == PM_CHEBY_FIRST ? comb_ptr<T, PM_CHEBY_FIRST>(a.S) : comb_ptr<T, PM_CHEBY_TERM>(a.S);
  void *args[] = {(void *)&a};
  COUNT_LAUNCH();
  return cudaLaunchKernel(k, dim3(grid), dim3(block), args, 0, st);
}

template cudaError_t launch_kin_all<double>(const KinArgs<double> &, int, int, size_t, cudaStream_t);
template cudaError_t launch_kin_all<float>(const KinArgs<float> &, int, int, size_t, cudaStream_t);
template int kin_all_max_blocks<double>(int, size_t);
template int kin_all_max_blocks<float>(int, size_t);
template cudaError_t launch_combine<double>(int, const CombArgs<double> &, int, int, cudaStream_t);
template cudaError_t launch_combine<float>(int, const CombArgs<float> &, int, int, cudaStream_t);

template <typename T, int MODE, int SS>
static void *kernel_ptr() { return (void *)linepass_kernel<T, MODE, SS>; }

template <typename T>
static void *select_kernel(int mode, int S) {
  switch (mode) {
    case PM_KIN_FIRST: return kernel_ptr<T, PM_KIN_FIRST, 1>();
    case PM_KIN_ACC: return kernel_ptr<T, PM_KIN_ACC, 1>();
    case PM_GSPO_KIN: return kernel_ptr<T, PM_GSPO_KIN, 1>();
    case PM_HAPPLY:
      return S == 1 ? kernel_ptr<T, PM_HAPPLY, 1>() : S == 2 ? kernel_ptr<T, PM_HAPPLY, 2>() : kernel_ptr<T, PM_HAPPLY, 0>();
    case PM_CHEBY_FIRST:
      return S == 1 ? kernel_ptr<T, PM_CHEBY_FIRST, 1>() : S == 2 ? kernel_ptr<T, PM_CHEBY_FIRST, 2>()
                                                                  : kernel_ptr<T, PM_CHEBY_FIRST, 0>();
    case PM_CHEBY_TERM:
      return S == 1 ? kernel_ptr<T, PM_CHEBY_TERM, 1>() : S == 2 ? kernel_ptr<T, PM_CHEBY_TERM, 2>()
                                                                 : kernel_ptr<T, PM_CHEBY_TERM, 0>();
  }
  return nullptr;
}

template <typename T>
cudaError_t launch_pass(int mode, const PassArgs<T> &a, int grid, int block, size_t smem, cudaStream_t st) {
  void *k = select_kernel<T>(mode, a.S);
  if (!k) return cudaErrorInvalidValue;
  if (smem > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
  }
  void *args[] = {(void *)&a};
  COUNT_LAUNCH();
  return cudaLaunchKernel(k, dim3(grid), dim3(block), args, smem, st);
}

template <typename T>
int pass_max_blocks(int mode, int S, int block, size_t smem) {
  void *k = select_kernel<T>(mode, S);
  if (smem > 48 * 1024) cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  int nb = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k, block, smem) != cudaSuccess) return 1;
  return nb > 0 ? nb : 1;
}

template cudaError_t launch_pass<double>(int, const PassArgs<double> &, int, int, size_t, cudaStream_t);
template cudaError_t launch_pass<float>(int, const PassArgs<float> &, int, int, size_t, cudaStream_t);
template int pass_max_blocks<double>(int, int, int, size_t);
template int pass_max_blocks<float>(int, int, int, size_t);

// ---------------------------------------------------------------- control
__global__ void cheby_begin_kernel(ChebyState *cs, int order, unsigned long long cond, int use_cond) {
  cs->norm0 = 0; cs->norm_last = 0; cs->done = 0; cs->terms = order; cs->status = 0; cs->arrive = 0;
  cs->i = 2; cs->acc_last = 0;
  if (use_cond) cudaGraphSetConditional(cond, order > 2 ? 1u : 0u);
}

// Sums the per-block norms in a fixed order and applies the reference's
// series cut (OCheby.cpp:178-182 real time, 285-289 imaginary time).
__global__ void cheby_finalize_kernel(ChebyState *cs, const double *partials, int nparts, int first, int term,
                                      int order, double prec, int imag, int offim0) {
  __shared__ double red[32];
  if (cs->done) return;
  double v = 0;
  for (int i = threadIdx.x; i < nparts; i += blockDim.x) v += partials[i];
  const double tot = block_sum(v, red);
  if (threadIdx.x != 0) return;
  if (!isfinite(tot)) { cs->status = 2; cs->done = 1; cs->terms = first ? 2 : term + 1; return; }
  if (first) { cs->norm0 = tot; return; }
  if (!imag) {
    const double nconv = fabs(cs->norm0 - tot) / cs->norm0;
    if (nconv < prec && offim0) { cs->done = 1; cs->terms = term + 1; }
  } else {
    if (fabs(tot - cs->norm_last) / cs->norm_last < prec) { cs->done = 1; cs->terms = term + 1; }
    cs->norm_last = tot;
  }
}

cudaError_t launch_cheby_begin(ChebyState *cs, int order, unsigned long long cond, int use_cond, cudaStream_t st) {
  cheby_begin_kernel<<<1, 1, 0, st>>>(cs, order, cond, use_cond);
  COUNT_LAUNCH();
  return cudaGetLastError();
}

__global__ void cheby_end_kernel(ChebyState *cs) { cs->total += cs->terms; }

cudaError_t launch_cheby_end(ChebyState *cs, cudaStream_t st) {
  cheby_end_kernel<<<1, 1, 0, st>>>(cs);
  COUNT_LAUNCH();
  return cudaGetLastError();
}

cudaError_t launch_cheby_finalize(ChebyState *cs, const double *partials, int nparts, int first, int term,
                                  int order, double prec, int imag, int offim0, cudaStream_t st) {
  cheby_finalize_kernel<<<1, 256, 0, st>>>(cs, partials, nparts, first, term, order, prec, imag, offim0);
  COUNT_LAUNCH();
  return cudaGetLastError();
}

__global__ void set_coefs_kernel(double *coef, const Couplings *cp, const double *lasers, int nt, long long step) {
  for (int e = threadIdx.x; e < cp->ne; e += blockDim.x) {
    const int l = cp->lid[e];
    double v = 1.0;
    if (l >= 0) v = (step >= 0 && step < nt) ? -lasers[(long long)l * nt + step] : 0.0;
    coef[e] = v;
  }
}

cudaError_t launch_set_coefs(double *coef, const Couplings *cp, const double *lasers, int laser_nt, long long step,
                             cudaStream_t st) {
  set_coefs_kernel<<<1, 64, 0, st>>>(coef, cp, lasers, laser_nt, step);
  COUNT_LAUNCH();
  return cudaGetLastError();
}

// ------------------------------------------------------------ elementwise
template <typename T>
__global__ void convert_kernel(cplx<T> *dst, const cplx<double> *src, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    st(dst + i, ccast<T>(ld(src + i)));
}
template <typename T>
__global__ void widen_kernel(cplx<double> *dst, const cplx<T> *src, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    st(dst + i, ccast<double>(ld(src + i)));
}

static int ew_grid(long long n) {
  long long g = (n + 255) / 256;
  return (int)(g > 4096 ? 4096 : (g < 1 ? 1 : g));
}

template <typename T>
cudaError_t launch_convert(cplx<T> *dst, const cplx<double> *src, long long n, cudaStream_t st) {
  convert_kernel<T><<<ew_grid(n), 256, 0, st>>>(dst, src, n);
  COUNT_LAUNCH();
  return cudaGetLastError();
}
template <typename T>
cudaError_t launch_widen(cplx<double> *dst, const cplx<T> *src, long long n, cudaStream_t st) {
  widen_kernel<T><<<ew_grid(n), 256, 0, st>>>(dst, src, n);
  COUNT_LAUNCH();
  return cudaGetLastError();
}
template cudaError_t launch_convert<double>(cplx<double> *, const cplx<double> *, long long, cudaStream_t);
template cudaError_t launch_convert<float>(cplx<float> *, const cplx<double> *, long long, cudaStream_t);
template cudaError_t launch_widen<double>(cplx<double> *, const cplx<double> *, long long, cudaStream_t);
template cudaError_t launch_widen<float>(cplx<double> *, const cplx<float> *, long long, cudaStream_t);

template <typename T>
__global__ void lincomb_kernel(cplx<T> *y, const cplx<T> *x, cplx<double> a, cplx<double> b, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    cplx<double> yv = ccast<double>(ld(y + i));
    cplx<double> r = dmul(yv, a);
    if (x) r = r + dmul(ccast<double>(ld(x + i)), b);
    st(y + i, ccast<T>(r));
  }
}
template <typename T>
cudaError_t launch_lincomb(cplx<T> *y, const cplx<T> *x, cplx<double> a, cplx<double> b, long long n,
                           cudaStream_t st) {
  lincomb_kernel<T><<<ew_grid(n), 256, 0, st>>>(y, x, a, b, n);
  COUNT_LAUNCH();
  return cudaGetLastError();
}
template cudaError_t launch_lincomb<double>(cplx<double> *, const cplx<double> *, cplx<double>, cplx<double>,
                                            long long, cudaStream_t);
template cudaError_t launch_lincomb<float>(cplx<float> *, const cplx<float> *, cplx<double>, cplx<double>,
                                           long long, cudaStream_t);

// Block sums of two values (the real and imaginary part of a dot product)
// in a fixed order: a shuffle tree within each warp, then the warp sums by
// another shuffle tree, the real parts in warp 0 and the imaginary parts in
// warp 1 (two sub-partitions: a binary64 add occupies one for ~70-80
// cycles, so dependent chains are kept short).  Valid on thread 0.
__device__ __forceinline__ void block_sum2(double &re, double &im, double *red) {
  for (int o = 16; o > 0; o >>= 1) {
    re += __shfl_down_sync(0xffffffffu, re, o);
    im += __shfl_down_sync(0xffffffffu, im, o);
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
  __syncthreads();
  if (lane == 0) { red[warp] = re; red[32 + warp] = im; }
  __syncthreads();
  if (warp < 2) {
    double v = lane < nw ? red[32 * warp + lane] : 0.0;
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if (lane == 0) red[64 + warp] = v;
  }
  __syncthreads();
  re = red[64];
  im = red[65];
}

// Per-state sum conj(a) b, FP64 accumulation, fixed reduction order.
template <typename T, typename U>
__device__ __forceinline__ void dots_body(const cplx<T> *a, const cplx<U> *b, int S, long long npts,
                                          double *partials) {
  __shared__ double red[66];
  for (int s = 0; s < S; ++s) {
    double re = 0, im = 0;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < npts;
         i += (long long)gridDim.x * blockDim.x) {
      const cplx<double> x = ccast<double>(ld(a + s * npts + i));
      const cplx<double> y = ccast<double>(ld(b + s * npts + i));
      re += x.re * y.re + x.im * y.im;
      im += x.re * y.im - x.im * y.re;
    }
    block_sum2(re, im, red);
    if (threadIdx.x == 0) {
      partials[((long long)blockIdx.x * S + s) * 2 + 0] = re;
      partials[((long long)blockIdx.x * S + s) * 2 + 1] = im;
    }
    __syncthreads();  // red[] is reused by the next state
  }
}
template <typename T, typename U>
__global__ void dots_kernel(const cplx<T> *a, const cplx<U> *b, int S, long long npts, double *partials,
                            const int *done) {
  if (done != nullptr && *done) return;
  dots_body<T, U>(a, b, S, npts, partials);
}
template <typename T, typename U>
cudaError_t launch_dots(const cplx<T> *a, const cplx<U> *b, int S, long long npts, double *partials, int grid,
                        cudaStream_t st) {
  dots_kernel<T, U><<<grid, 256, 0, st>>>(a, b, S, npts, partials, nullptr);
  COUNT_LAUNCH();
  return cudaGetLastError();
}

// Per-state sums of the block partials (layout [block][state][re, im]):
// one warp per state and component, lane l adding blocks l, l + 32, ... in
// that order, then a shuffle tree; the warps run on different
// sub-partitions side by side (a serial sum in one thread would take one
// dependent binary64 add, ~80 cycles of the FP64 pipe, per partial).  A
// fixed order, the same in every launch; the sums are valid in thread 0.
// Every thread of the block calls this.
__device__ __forceinline__ void sum_partials(const double *partials, int grid, int S, double *re, double *im) {
  __shared__ double out[2 * kMaxStates];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int k = warp; k < 2 * S; k += nw) {
    const int st = k >> 1, c = k & 1;
    double v = 0.0;
    for (int b = lane; b < grid; b += 32) v += __ldcg(partials + ((long long)b * S + st) * 2 + c);
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if (lane == 0) out[k] = v;
  }
  __syncthreads();
  if (threadIdx.x == 0)
    for (int st = 0; st < S; ++st) {
      re[st] = out[2 * st];
      im[st] = out[2 * st + 1];
    }
  __syncthreads();
}

// Partial sums -> scalar (sum_partials' fixed order; states weighted, then
// added in order).
__device__ void ks_finish_body(const double *partials, const KsFinish &f, double *ks, int *done) {
  // the error estimate's factors beta_i / i and dt^(it-2) do not depend on
  // this dot product: warps 1 and 2 compute them while the partials are
  // summed (one FP64 division or pow is a long chain of pipe slots)
  __shared__ double q[kMaxKrylov];
  __shared__ double pw;
  const bool est = f.mode == KS_BETA && f.it >= 2;
  if (est) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (warp == 1)
      for (int i = 1 + lane; i < f.it - 2; i += 32) q[i] = ks[f.order + i] / double(i);
    if (warp == 2 && lane == 0) pw = pow(f.dt, (double)(f.it - 2));
  }
  double re[kMaxStates], im[kMaxStates];
  sum_partials(partials, f.grid, f.S, re, im);
  if (threadIdx.x != 0) return;
  double tr = 0.0;
  for (int s = 0; s < f.S; ++s) tr += re[s] * f.w;
  if (f.mode == KS_ALPHA) {
    ks[f.slot] = tr;
    return;
  }
  const double v = sqrt(tr);
  ks[f.slot] = v;
  if (f.mode != KS_BETA || f.it < 2) return;
  // OSIL::BuildLZB error estimate (src/qdlib/OSIL.cpp:106-112), tested after the iteration
  const double *beta = ks + f.order;
  double err = pw * beta[0];
  for (int i = 1; i < f.it - 2; ++i) err *= q[i];
  err = fabs(err);
  if (err < f.tol * ks[2 * f.order]) {  // ks[2 order] = |psi|
    done[1] = 1;                          // stop after this iteration's normalisation
    ks[2 * f.order + 1] = (double)(f.it + 1);
  }
}

__device__ void ka_finish_body(const double *partials, const KaArgs &a, int op, int j, int col, double *ks, int *ia,
                               int *done) {
  // KA_NORM: the error estimate's divisions H[i+1][i] / i and dt^(it-2) in
  // warps 1 and 2 while the partials are summed (they use earlier entries)
  __shared__ double qr[kMaxKrylov], qi[kMaxKrylov];
  __shared__ double pw;
  if (op == KA_NORM) {
    const int it = col + 1, m = a.m;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (warp == 1)
      for (int i = 1 + lane; i < it - 2; i += 32) {
        qr[i] = ks[2 * ((i + 1) * m + i)] / double(i);
        qi[i] = ks[2 * ((i + 1) * m + i) + 1] / double(i);
      }
    if (warp == 2 && lane == 0) pw = pow(a.dt, (double)(it - 2));
  }
  double re[kMaxStates], im[kMaxStates];
  sum_partials(partials, a.grid, a.S, re, im);
  if (threadIdx.x != 0) return;
  double tr = 0.0, ti = 0.0;
  for (int s = 0; s < a.S; ++s) { tr += re[s] * a.w; ti += im[s] * a.w; }
  const int m = a.m;
  double *H = ks;
  if (op == KA_PSN) { ks[2 * m * m] = sqrt(tr); return; }
  if (op == KA_H) { H[2 * (j * m + col)] = tr; H[2 * (j * m + col) + 1] = ti; return; }
  if (op == KA_LAST) {
    const int c = ia[0] - 1;
    H[2 * (j * m + c)] = tr; H[2 * (j * m + c) + 1] = ti;
    return;
  }
  // KA_NORM for iteration it = col + 1 (OArnoldi::BuildLZB, src/qdlib/OArnoldi.cpp:111-136)
  const int it = col + 1;
  const double nrm = sqrt(tr);
  if (nrm < 1e-11) {  // ARNOLDI_UNDERRUN (OArnoldi.h:12): stop before this vector
    done[0] = 1;
    return;
  }
  H[2 * (it * m + it - 1)] = nrm;
  H[2 * (it * m + it - 1) + 1] = 0.0;
  // err = dt^(it-2) H[1][0] |psi| prod H[i+1][i] / i, complex
  double er = pw * H[2 * m] * ks[2 * m * m];
  double ei = pw * H[2 * m + 1] * ks[2 * m * m];
  for (int i = 1; i < it - 2; ++i) {
    const double hr = qr[i], hi = qi[i];
    const double nr = er * hr - ei * hi, ni = er * hi + ei * hr;
    er = nr;
    ei = ni;
  }
  if (hypot(er, ei) < a.conv) done[1] = 1;  // after this iteration's vector is stored
}

// ---- fused Krylov launches: a pass over the vectors, its dot product's
// block partials, and the finishing scalar work in the block that arrives
// last (an atomic ticket: no block waits for another).  The updates are
// FMAs (y - s x per component); multiplications by 1 and 0 that a complex
// product would spend are left out (each binary64 instruction holds a
// sub-partition's FP64 unit for ~70-80 cycles).

// True in the one block whose ticket is the last of the grid; its threads
// then see every block's partials (each block fenced before its ticket).
__device__ __forceinline__ bool arrive_last(unsigned int *ticket) {
  __shared__ unsigned int last;
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    last = atomicAdd(ticket, 1u) == gridDim.x - 1 ? 1u : 0u;
  }
  __syncthreads();
  return last != 0;
}

// Partials of a per-state dot product whose terms t(s, i) = conj(a) b are
// produced by a functor (which may also update the vectors).
template <typename Term>
__device__ __forceinline__ void dots_terms(int S, long long npts, double *partials, Term term) {
  __shared__ double red[66];
  for (int s = 0; s < S; ++s) {
    double re = 0, im = 0;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < npts;
         i += (long long)gridDim.x * blockDim.x) {
      cplx<double> x, y;
      term((long long)s * npts + i, x, y);
      re += x.re * y.re + x.im * y.im;
      im += x.re * y.im - x.im * y.re;
    }
    block_sum2(re, im, red);
    if (threadIdx.x == 0) {
      partials[((long long)blockIdx.x * S + s) * 2 + 0] = re;
      partials[((long long)blockIdx.x * S + s) * 2 + 1] = im;
    }
    __syncthreads();
  }
}

// <a|b> finished into the Lanczos scalars (alpha, beta or |psi|)
template <typename T, typename U>
__global__ void dots_ks_kernel(const cplx<T> *a, const cplx<U> *b, int S, long long npts, double *partials,
                               KsFinish f, double *ks, int *done, unsigned int *ticket) {
  if (*done) return;
  dots_body<T, U>(a, b, S, npts, partials);
  if (!arrive_last(ticket)) return;
  ks_finish_body(partials, f, ks, done);
  if (threadIdx.x == 0) *ticket = 0;
}
// y -= alpha x1 (rounded to T), y -= beta x2, then |y|^2 finished as beta
// with the error estimate
template <typename T>
__global__ void ks_lincomb2_dot_kernel(cplx<T> *y, const cplx<T> *x1, int i1, const cplx<T> *x2, int i2, int S,
                                       long long npts, double *partials, KsFinish f, double *ks, int *done,
                                       unsigned int *ticket) {
  if (*done) return;
  const double b1 = -ks[i1], b2 = -ks[i2];
  dots_terms(S, npts, partials, [&](long long g, cplx<double> &xa, cplx<double> &xb) {
    const cplx<double> u = ccast<double>(ld(y + g)), v1 = ccast<double>(ld(x1 + g));
    const cplx<T> r1 = ccast<T>(cplx<double>{fma(b1, v1.re, u.re), fma(b1, v1.im, u.im)});
    const cplx<double> w = ccast<double>(r1), v2 = ccast<double>(ld(x2 + g));
    const cplx<T> r2 = ccast<T>(cplx<double>{fma(b2, v2.re, w.re), fma(b2, v2.im, w.im)});
    st(y + g, r2);
    xa = xb = ccast<double>(r2);
  });
  if (!arrive_last(ticket)) return;
  ks_finish_body(partials, f, ks, done);
  if (threadIdx.x == 0) *ticket = 0;
}
// y /= ks[idx], then done[0] |= done[1] in the last block, once every block
// has read done[0]
template <typename T>
__global__ void ks_scale_commit_kernel(cplx<T> *y, const double *ks, int idx, long long n, int *done,
                                       unsigned int *ticket) {
  if (*done) return;
  const double a = 1.0 / ks[idx];
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const cplx<double> u = ccast<double>(ld(y + i));
    st(y + i, ccast<T>(cplx<double>{u.re * a, u.im * a}));
  }
  if (!arrive_last(ticket)) return;
  if (threadIdx.x == 0) {
    if (done[1]) done[0] = 1;
    *ticket = 0;
  }
}
// <a|b> finished into the Arnoldi scalars (KA_LAST: skipped for j >= order)
template <typename T, typename U>
__global__ void dots_ka_kernel(const cplx<T> *a, const cplx<U> *b, int S, long long npts, double *partials,
                               KaArgs ka, int op, int j, int col, double *ks, int *ia, int *done,
                               unsigned int *ticket) {
  if (op != KA_LAST && *done) return;
  if (op == KA_LAST && j >= ia[0]) return;
  dots_body<T, U>(a, b, S, npts, partials);
  if (!arrive_last(ticket)) return;
  ka_finish_body(partials, ka, op, j, col, ks, ia, done);
  if (threadIdx.x == 0) *ticket = 0;
}
// one modified Gram-Schmidt step y -= H[jc][col] x, then the next dot
// product <a|y> (a = nullptr: <y|y>) finished as op
template <typename T>
__global__ void ka_lincomb_dot_kernel(cplx<T> *y, const cplx<T> *x, const cplx<T> *a, int jc, int S,
                                      long long npts, double *partials, KaArgs ka, int op, int j, int col, double *ks,
                                      int *ia, int *done, unsigned int *ticket) {
  if (*done) return;
  const int m = ka.m;
  const double br = -ks[2 * (jc * m + col)], bi = -ks[2 * (jc * m + col) + 1];
  dots_terms(S, npts, partials, [&](long long g, cplx<double> &xa, cplx<double> &xb) {
    const cplx<double> u = ccast<double>(ld(y + g)), v = ccast<double>(ld(x + g));
    const cplx<T> r = ccast<T>(cplx<double>{fma(v.re, br, fma(-v.im, bi, u.re)), fma(v.re, bi, fma(v.im, br, u.im))});
    st(y + g, r);
    xb = ccast<double>(r);
    xa = a ? ccast<double>(ld(a + g)) : xb;
  });
  if (!arrive_last(ticket)) return;
  ka_finish_body(partials, ka, op, j, col, ks, ia, done);
  if (threadIdx.x == 0) *ticket = 0;
}
// q = buf / H[it][it-1], and in the last block ia[0] = it + 1,
// done[0] |= done[1]
template <typename T>
__global__ void ka_scale_commit_kernel(cplx<T> *q, const cplx<T> *buf, const double *ks, int idx, long long n, int it,
                                       int *ia, int *done, unsigned int *ticket) {
  if (*done) return;
  const double a = 1.0 / ks[idx];
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const cplx<double> u = ccast<double>(ld(buf + i));
    st(q + i, ccast<T>(cplx<double>{u.re * a, u.im * a}));
  }
  if (!arrive_last(ticket)) return;
  if (threadIdx.x == 0) {
    ia[0] = it + 1;
    if (done[1]) done[0] = 1;
    *ticket = 0;
  }
}

template <typename T, typename U>
cudaError_t launch_dots_ks(const cplx<T> *a, const cplx<U> *b, int S, long long npts, double *partials,
                           const KsFinish &f, double *ks, int *done, unsigned int *ticket, cudaStream_t st) {
  dots_ks_kernel<T, U><<<f.grid, 256, 0, st>>>(a, b, S, npts, partials, f, ks, done, ticket);
  COUNT_LAUNCH();
  return cudaGetLastError();
}
template <typename T>
cudaError_t launch_ks_lincomb2_dot(cplx<T> *y, const cplx<T> *x1, int i1, const cplx<T> *x2, int i2, int S,
                                   long long npts, double *partials, const KsFinish &f, double *ks, int *done,
                                   unsigned int *ticket, cudaStream_t st) {
  ks_lincomb2_dot_kernel<T><<<f.grid, 256, 0, st>>>(y, x1, i1, x2, i2, S, npts, partials, f, ks, done, ticket);
  COUNT_LAUNCH();
  return cudaGetLastError();
}
template <typename T>
cudaError_t launch_ks_scale_commit(cplx<T> *y, const double *ks, int idx, long long n, int *done, unsigned int *ticket,
                                   cudaStream_t st) {
  ks_scale_commit_kernel<T><<<ew_grid(n), 256, 0, st>>>(y, ks, idx, n, done, ticket);
  COUNT_LAUNCH();
  return cudaGetLastError();
}
template <typename T, typename U>
cudaError_t launch_dots_ka(const cplx<T> *a, const cplx<U> *b, int S, long long npts, double *partials,
                           const KaArgs &ka, int op, int j, int col, double *ks, int *ia, int *done,
                           unsigned int *ticket, cudaStream_t st) {
  dots_ka_kernel<T, U><<<ka.grid, 256, 0, st>>>(a, b, S, npts, partials, ka, op, j, col, ks, ia, done, ticket);
  COUNT_LAUNCH();
  return cudaGetLastError();
}
template <typename T>
cudaError_t launch_ka_lincomb_dot(cplx<T> *y, const cplx<T> *x, const cplx<T> *a, int jc, int S, long long npts,
                                  double *partials, const KaArgs &ka, int op, int j, int col, double *ks, int *ia,
                                  int *done, unsigned int *ticket, cudaStream_t st) {
  ka_lincomb_dot_kernel<T><<<ka.grid, 256, 0, st>>>(y, x, a, jc, S, npts, partials, ka, op, j, col, ks, ia, done,
                                                    ticket);
  COUNT_LAUNCH();
  return cudaGetLastError();
}
template <typename T>
cudaError_t launch_ka_scale_commit(cplx<T> *q, const cplx<T> *buf, const double *ks, int idx, long long n, int it,
                                   int *ia, int *done, unsigned int *ticket, cudaStream_t st) {
  ka_scale_commit_kernel<T><<<ew_grid(n), 256, 0, st>>>(q, buf, ks, idx, n, it, ia, done, ticket);
  COUNT_LAUNCH();
  return cudaGetLastError();
}
#define QDG_KRYLOV_FUSED(T)                                                                                         \
  template cudaError_t launch_ks_lincomb2_dot<T>(cplx<T> *, const cplx<T> *, int, const cplx<T> *, int, int,          \
                                                 long long, double *, const KsFinish &, double *, int *,             \
                                                 unsigned int *, cudaStream_t);                                      \
  template cudaError_t launch_ks_scale_commit<T>(cplx<T> *, const double *, int, long long, int *, unsigned int *,   \
                                                 cudaStream_t);                                                      \
  template cudaError_t launch_ka_lincomb_dot<T>(cplx<T> *, const cplx<T> *, const cplx<T> *, int, int, long long,     \
                                                double *, const KaArgs &, int, int, int, double *, int *, int *,      \
                                                unsigned int *, cudaStream_t);                                       \
  template cudaError_t launch_ka_scale_commit<T>(cplx<T> *, const cplx<T> *, const double *, int, long long, int,    \
                                                 int *, int *, unsigned int *, cudaStream_t);                        \
  template cudaError_t launch_dots_ks<T, T>(const cplx<T> *, const cplx<T> *, int, long long, double *,              \
                                            const KsFinish &, double *, int *, unsigned int *, cudaStream_t);        \
  template cudaError_t launch_dots_ka<T, T>(const cplx<T> *, const cplx<T> *, int, long long, double *,              \
                                            const KaArgs &, int, int, int, double *, int *, int *, unsigned int *,   \
                                            cudaStream_t);
QDG_KRYLOV_FUSED(double)
QDG_KRYLOV_FUSED(float)
#undef QDG_KRYLOV_FUSED



template <typename T>
__global__ void ka_select_kernel(cplx<T> *dst, KaBasis<T> b, const int *ia, long long n) {
  const cplx<T> *src = b.q[ia[0] - 1];
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    dst[i] = src[i];
}
template <typename T>
cudaError_t launch_ka_select(cplx<T> *dst, const KaBasis<T> &b, const int *ia, long long n, cudaStream_t st) {
  ka_select_kernel<T><<<ew_grid(n), 256, 0, st>>>(dst, b, ia, n);
  COUNT_LAUNCH();
  return cudaGetLastError();
}
template cudaError_t launch_ka_select<double>(cplx<double> *, const KaBasis<double> &, const int *, long long,
                                              cudaStream_t);
template cudaError_t launch_ka_select<float>(cplx<float> *, const KaBasis<float> &, const int *, long long,
                                             cudaStream_t);


template <typename T>
__global__ void kcombine_kernel(cplx<double> *psi, KCombine<T> k, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    cplx<double> r = dmul(ld(psi + i), k.c[0]);
    for (int j = 1; j < k.m; ++j) r = r + dmul(ccast<double>(ld(k.q[j] + i)), k.c[j]);
    st(psi + i, r);
  }
}
template <typename T>
cudaError_t launch_kcombine(cplx<double> *psi, const KCombine<T> &k, long long n, cudaStream_t st) {
  kcombine_kernel<T><<<ew_grid(n), 256, 0, st>>>(psi, k, n);
  COUNT_LAUNCH();
  return cudaGetLastError();
}
template cudaError_t launch_kcombine<double>(cplx<double> *, const KCombine<double> &, long long, cudaStream_t);
template cudaError_t launch_kcombine<float>(cplx<double> *, const KCombine<float> &, long long, cudaStream_t);


template <typename T>
__global__ void ks_lincomb_kernel(cplx<T> *y, const cplx<T> *x, const double *ks, int idx, long long n,
                                  const int *done) {
  if (*done) return;
  // the arithmetic of lincomb_kernel with a = 1, b = -s (or a = 1/s, no x)
  const double sc = ks[idx];
  const cplx<double> a = x ? cplx<double>{1.0, 0.0} : cplx<double>{1.0 / sc, 0.0};
  const cplx<double> b = cplx<double>{-sc, 0.0};
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    cplx<double> r = dmul(ccast<double>(ld(y + i)), a);
    if (x) r = r + dmul(ccast<double>(ld(x + i)), b);
    st(y + i, ccast<T>(r));
  }
}
template <typename T>
cudaError_t launch_ks_lincomb(cplx<T> *y, const cplx<T> *x, const double *ks, int idx, long long n, const int *done,
                              cudaStream_t st) {
  ks_lincomb_kernel<T><<<ew_grid(n), 256, 0, st>>>(y, x, ks, idx, n, done);
  COUNT_LAUNCH();
  return cudaGetLastError();
}
template cudaError_t launch_ks_lincomb<double>(cplx<double> *, const cplx<double> *, const double *, int, long long,
                                               const int *, cudaStream_t);
template cudaError_t launch_ks_lincomb<float>(cplx<float> *, const cplx<float> *, const double *, int, long long,
                                              const int *, cudaStream_t);
template cudaError_t launch_dots<double, double>(const cplx<double> *, const cplx<double> *, int, long long, double *,
                                                 int, cudaStream_t);
template cudaError_t launch_dots<float, float>(const cplx<float> *, const cplx<float> *, int, long long, double *,
                                               int, cudaStream_t);
template cudaError_t launch_dots<double, float>(const cplx<double> *, const cplx<float> *, int, long long, double *,
                                                int, cudaStream_t);
template cudaError_t launch_dots<float, double>(const cplx<float> *, const cplx<double> *, int, long long, double *,
                                                int, cudaStream_t);

// ------------------------------------------------------------------ GSPO
__device__ __forceinline__ cplx<double> cexpd(cplx<double> z) {
  double s, c;
  sincos(z.im, &s, &c);
  const double e = exp(z.re);
  return mk(e * c, e * s);
}

// exp(c M) psi at one point for a real symmetric 1x1 / 2x2 matrix M.
// 2x2: exp(cM) = e^{c m} [cosh(c r) I + sinh(c r)/r (M - m I)], m = (a+d)/2,
// r = sqrt(((a-d)/2)^2 + b^2) -- the spectral form of the per-point
// eigenbasis transform of TransformMSD (TransformMSD.cpp:47-62,84-98).
// exp(c M) of a real symmetric S x S matrix m (row-major, destroyed): cyclic
// Jacobi rotations give M = Z diag(w) Z^T, then E = Z diag(exp(c w)) Z^T --
// the per-point diagonalisation and transformation of ODMultistate and
// TransformMSD (ODMultistate.cpp:133-152, TransformMSD.cpp:31-100).  At most
// 50 sweeps; the rotations stop when the off-diagonal part is below 1e-32 of
// the matrix's square norm.
__device__ __forceinline__ bool offdiag_nonzero(const double *m, int S) {
  for (int a = 0; a < S; ++a)
    for (int b = 0; b < S; ++b)
      if (a != b && m[a * S + b] != 0.0) return true;
  return false;
}
__device__ void expm_sym(double *m, int S, cplx<double> c, cplx<double> *E) {
  double z[kMaxStates * kMaxStates];
  for (int i = 0; i < S * S; ++i) z[i] = 0.0;
  for (int i = 0; i < S; ++i) z[i * S + i] = 1.0;
  double tot = 0.0;
  for (int i = 0; i < S * S; ++i) tot += m[i] * m[i];
  for (int sweep = 0; sweep < 50; ++sweep) {
    double off = 0.0;
    for (int p = 0; p < S; ++p)
      for (int q = p + 1; q < S; ++q) off += m[p * S + q] * m[p * S + q];
    if (!(off > 1e-32 * tot)) break;
    for (int p = 0; p < S; ++p)
      for (int q = p + 1; q < S; ++q) {
        const double apq = m[p * S + q];
        if (fabs(apq) < 1e-300) continue;
        const double theta = (m[q * S + q] - m[p * S + p]) / (2.0 * apq);
        const double t = (theta >= 0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1.0));
        const double cs = 1.0 / sqrt(t * t + 1.0), sn = t * cs;
        for (int k = 0; k < S; ++k) {
          const double akp = m[k * S + p], akq = m[k * S + q];
          m[k * S + p] = cs * akp - sn * akq;
          m[k * S + q] = sn * akp + cs * akq;
        }
        for (int k = 0; k < S; ++k) {
          const double apk = m[p * S + k], aqk = m[q * S + k];
          m[p * S + k] = cs * apk - sn * aqk;
          m[q * S + k] = sn * apk + cs * aqk;
        }
        for (int k = 0; k < S; ++k) {
          const double zkp = z[k * S + p], zkq = z[k * S + q];
          z[k * S + p] = cs * zkp - sn * zkq;
          z[k * S + q] = sn * zkp + cs * zkq;
        }
      }
  }
  cplx<double> ew[kMaxStates];
  for (int k = 0; k < S; ++k) ew[k] = cexpd(mk(c.re * m[k * S + k], c.im * m[k * S + k]));
  for (int a = 0; a < S; ++a)
    for (int b = 0; b < S; ++b) {
      cplx<double> acc = mk(0.0, 0.0);
      for (int k = 0; k < S; ++k) {
        const double zz = z[a * S + k] * z[b * S + k];
        acc = acc + mk(zz * ew[k].re, zz * ew[k].im);
      }
      E[a * S + b] = acc;
    }
}

template <typename T>
__global__ void gspo_potential_kernel(cplx<T> *psi, int S, long long npts, const Couplings *cp, const double *coef,
                                      const T *grids, cplx<double> c) {
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < npts; p += (long long)gridDim.x * blockDim.x) {
    double m[kMaxStates * kMaxStates];
    for (int i = 0; i < S * S; ++i) m[i] = 0;
    for (int e = 0; e < cp->ne; ++e) m[cp->row[e] * S + cp->col[e]] += coef[e] * (double)grids[(long long)cp->gid[e] * npts + p];
    if (S == 2 && (m[1] != 0.0 || m[2] != 0.0)) {
      const double a = m[0], d = m[3], b = m[1];
      const double mm = 0.5 * (a + d), h = 0.5 * (a - d);
      const double r = sqrt(h * h + b * b);
      const cplx<double> em = cexpd(mk(c.re * mm, c.im * mm));
      const cplx<double> z = mk(c.re * r, c.im * r);
      const cplx<double> ep = cexpd(z), en = cexpd(mk(-z.re, -z.im));
      const cplx<double> ch = mk(0.5 * (ep.re + en.re), 0.5 * (ep.im + en.im));
      cplx<double> shr;  // sinh(z)/r
      if (r * sqrt(c.re * c.re + c.im * c.im) < 1e-4) {
        const cplx<double> z2 = dmul(z, z);
        shr = dmul(c, mk(1.0 + z2.re / 6.0, z2.im / 6.0));
      } else {
        shr = mk(0.5 * (ep.re - en.re) / r, 0.5 * (ep.im - en.im) / r);
      }
      const cplx<double> x0 = ccast<double>(ld(psi + p));
      const cplx<double> x1 = ccast<double>(ld(psi + npts + p));
      // (M - m I) = [[h, b], [b, -h]]
      const cplx<double> y0 = dmul(ch, x0) + dmul(shr, mk(h * x0.re + b * x1.re, h * x0.im + b * x1.im));
      const cplx<double> y1 = dmul(ch, x1) + dmul(shr, mk(b * x0.re - h * x1.re, b * x0.im - h * x1.im));
      st(psi + p, ccast<T>(dmul(em, y0)));
      st(psi + npts + p, ccast<T>(dmul(em, y1)));
    } else if (S > 2 && offdiag_nonzero(m, S)) {
      cplx<double> E[kMaxStates * kMaxStates], x[kMaxStates];
      expm_sym(m, S, c, E);
      for (int s = 0; s < S; ++s) x[s] = ccast<double>(ld(psi + s * npts + p));
      for (int a = 0; a < S; ++a) {
        cplx<double> y = mk(0.0, 0.0);
        for (int b = 0; b < S; ++b) y = y + dmul(E[a * S + b], x[b]);
        st(psi + a * npts + p, ccast<T>(y));
      }
    } else {
      for (int s = 0; s < S; ++s) {
        const double v = m[s * S + s];
        const cplx<double> f = cexpd(mk(c.re * v, c.im * v));
        st(psi + s * npts + p, ccast<T>(dmul(f, ccast<double>(ld(psi + s * npts + p)))));
      }
    }
  }
}

// The same exponent as gspo_potential_kernel, stored instead of applied.
__global__ void gspo_umat_kernel(cplx<double> *U, int S, long long npts, const Couplings *cp, const double *coef,
                                 const double *grids, cplx<double> c) {
  const int kU = S == 2 ? 3 : S * S;
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < npts; p += (long long)gridDim.x * blockDim.x) {
    double m[kMaxStates * kMaxStates];
    for (int i = 0; i < S * S; ++i) m[i] = 0;
    for (int e = 0; e < cp->ne; ++e) m[cp->row[e] * S + cp->col[e]] += coef[e] * grids[(long long)cp->gid[e] * npts + p];
    cplx<double> *u = U + (long long)kU * p;
    if (S == 2 && (m[1] != 0.0 || m[2] != 0.0)) {
      const double a = m[0], d = m[3], b = m[1];
      const double mm = 0.5 * (a + d), h = 0.5 * (a - d);
      const double r = sqrt(h * h + b * b);
      const cplx<double> em = cexpd(mk(c.re * mm, c.im * mm));
      const cplx<double> z = mk(c.re * r, c.im * r);
      const cplx<double> ep = cexpd(z), en = cexpd(mk(-z.re, -z.im));
      const cplx<double> ch = mk(0.5 * (ep.re + en.re), 0.5 * (ep.im + en.im));
      cplx<double> shr;  // sinh(z)/r
      if (r * sqrt(c.re * c.re + c.im * c.im) < 1e-4) {
        const cplx<double> z2 = dmul(z, z);
        shr = dmul(c, mk(1.0 + z2.re / 6.0, z2.im / 6.0));
      } else {
        shr = mk(0.5 * (ep.re - en.re) / r, 0.5 * (ep.im - en.im) / r);
      }
      // em [ch I + shr (M - m I)], (M - m I) = [[h, b], [b, -h]]
      u[0] = dmul(em, ch + mk(shr.re * h, shr.im * h));
      u[1] = dmul(em, mk(shr.re * b, shr.im * b));
      u[2] = dmul(em, ch - mk(shr.re * h, shr.im * h));
    } else if (S == 2) {
      u[0] = cexpd(mk(c.re * m[0], c.im * m[0]));
      u[1] = mk(0.0, 0.0);
      u[2] = cexpd(mk(c.re * m[3], c.im * m[3]));
    } else if (S == 1) {
      u[0] = cexpd(mk(c.re * m[0], c.im * m[0]));
    } else {
      expm_sym(m, S, c, u);  // S > 2: the full per-point matrix
    }
  }
}
cudaError_t launch_gspo_umat(cplx<double> *U, int S, long long npts, const Couplings *cp, const double *coef,
                             const double *grids, cplx<double> c, cudaStream_t st) {
  gspo_umat_kernel<<<ew_grid(npts), 256, 0, st>>>(U, S, npts, cp, coef, grids, c);
  COUNT_LAUNCH();
  return cudaGetLastError();
}

template <typename T>
__global__ void gspo_apply_kernel(cplx<T> *psi, int S, long long npts, const cplx<double> *U) {
  const int kU = S == 2 ? 3 : S * S;
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < npts; p += (long long)gridDim.x * blockDim.x) {
    const cplx<double> *u = U + (long long)kU * p;
    if (S > 2) {
      cplx<double> x[kMaxStates];
      for (int s = 0; s < S; ++s) x[s] = ccast<double>(ld(psi + s * npts + p));
      for (int a = 0; a < S; ++a) {
        cplx<double> y = mk(0.0, 0.0);
        for (int b = 0; b < S; ++b) y = y + dmul(u[a * S + b], x[b]);
        st(psi + a * npts + p, ccast<T>(y));
      }
    } else if (S == 2) {
      const cplx<double> x0 = ccast<double>(ld(psi + p)), x1 = ccast<double>(ld(psi + npts + p));
      st(psi + p, ccast<T>(dmul(u[0], x0) + dmul(u[1], x1)));
      st(psi + npts + p, ccast<T>(dmul(u[1], x0) + dmul(u[2], x1)));
    } else {
      for (int s = 0; s < S; ++s)
        st(psi + s * npts + p, ccast<T>(dmul(u[s], ccast<double>(ld(psi + s * npts + p)))));
    }
  }
}
template <typename T>
cudaError_t launch_gspo_apply(cplx<T> *psi, int S, long long npts, const cplx<double> *U, cudaStream_t st) {
  gspo_apply_kernel<T><<<ew_grid(npts), 256, 0, st>>>(psi, S, npts, U);
  COUNT_LAUNCH();
  return cudaGetLastError();
}
template cudaError_t launch_gspo_apply<double>(cplx<double> *, int, long long, const cplx<double> *, cudaStream_t);
template cudaError_t launch_gspo_apply<float>(cplx<float> *, int, long long, const cplx<double> *, cudaStream_t);

template <typename T>
cudaError_t launch_gspo_potential(cplx<T> *psi, int S, long long npts, const Couplings *cp, const double *coef,
                                  const T *grids, cplx<double> c, cudaStream_t st) {
  gspo_potential_kernel<T><<<ew_grid(npts), 256, 0, st>>>(psi, S, npts, cp, coef, grids, c);
  COUNT_LAUNCH();
  return cudaGetLastError();
}
template cudaError_t launch_gspo_potential<double>(cplx<double> *, int, long long, const Couplings *, const double *,
                                                   const double *, cplx<double>, cudaStream_t);
template cudaError_t launch_gspo_potential<float>(cplx<float> *, int, long long, const Couplings *, const double *,
                                                  const float *, cplx<double>, cudaStream_t);

}  // namespace qdg
