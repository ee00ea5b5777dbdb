// qdg_device.cuh -- device-side building blocks of the propagation engine.
//
// Complex arithmetic, the shared-memory Stockham FFT used for the grid
// kinetic operator, and deterministic block reductions.  Everything is
// templated on the arithmetic type T (double for the FP64 drop-in path,
// float for the FP32 bulk of the mixed path).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace qdg {

template <typename T> struct cplx { T re, im; };

template <typename T> struct vec2;
template <> struct vec2<double> { typedef double2 type; };
template <> struct vec2<float> { typedef float2 type; };

template <typename T> __device__ __forceinline__ cplx<T> mk(T r, T i) { cplx<T> c; c.re = r; c.im = i; return c; }
template <typename T> __device__ __forceinline__ cplx<T> operator+(cplx<T> a, cplx<T> b) { return mk(a.re + b.re, a.im + b.im); }
template <typename T> __device__ __forceinline__ cplx<T> operator-(cplx<T> a, cplx<T> b) { return mk(a.re - b.re, a.im - b.im); }
template <typename T> __device__ __forceinline__ cplx<T> cmul(cplx<T> a, cplx<T> b) {
  return mk(a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re);
}
template <typename T> __device__ __forceinline__ cplx<T> cmulr(cplx<T> a, T r) { return mk(a.re * r, a.im * r); }
template <typename T> __device__ __forceinline__ T cabs2(cplx<T> a) { return a.re * a.re + a.im * a.im; }
template <typename T, typename U> __device__ __forceinline__ cplx<T> ccast(cplx<U> a) { return mk((T)a.re, (T)a.im); }

template <typename T> __device__ __forceinline__ cplx<T> ldg(const cplx<T> *p) {
  typedef typename vec2<T>::type V;
  V v = __ldg(reinterpret_cast<const V *>(p));
  return mk<T>(v.x, v.y);
}
template <typename T> __device__ __forceinline__ cplx<T> ld(const cplx<T> *p) {
  typedef typename vec2<T>::type V;
  V v = *reinterpret_cast<const V *>(p);
  return mk<T>(v.x, v.y);
}
template <typename T> __device__ __forceinline__ void st(cplx<T> *p, cplx<T> c) {
  typedef typename vec2<T>::type V;
  V v; v.x = c.re; v.y = c.im;
  *reinterpret_cast<V *>(p) = v;
}

// Radix plan of one line length: N = prod radix[i], radices in {4, 2, 3, 5}.
struct RadixPlan {
  int n;
  int nstages;
  int radix[16];
};

// One Stockham stage over `nlines` lines of length N stored line after line
// in `in` (line stride N); result in `out`.  Items are spread over all
// threads of the block.  tw[m] = exp(-2 pi i m / N); sign = -1 forward
// (FFTW_FORWARD), +1 backward.  The Stockham autosort indexing follows the
// classic formulation (Stockham 1966; Govindaraju et al., SC'08): item j
// reads in[j + r*N/R], applies the stage twiddles w^(r*k), does the R-point
// DFT and writes out[(j/Ns)*Ns*R + k + r*Ns], k = j mod Ns.
template <typename T, int R>
__device__ __forceinline__ void stockham_stage(const cplx<T> *__restrict__ in, cplx<T> *__restrict__ out,
                                               int N, int nlines, int Ns, const cplx<T> *__restrict__ tw,
                                               int sign) {
  const int M = N / R;
  const int step = N / (Ns * R);
  const int items = nlines * M;
  for (int it = threadIdx.x; it < items; it += blockDim.x) {
    const int line = it / M;
    const int j = it - line * M;
    const int k = j % Ns;
    const cplx<T> *src = in + line * N;
    cplx<T> v[R];
#pragma unroll
    for (int r = 0; r < R; ++r) v[r] = src[j + r * M];
    if (k) {
#pragma unroll
      for (int r = 1; r < R; ++r) {
        cplx<T> w = tw[r * k * step];  // r*k*step < R*Ns*step = N
        if (sign > 0) w.im = -w.im;
        v[r] = cmul(v[r], w);
      }
    }
    cplx<T> y[R];
    if (R == 2) {
      y[0] = v[0] + v[1];
      y[1] = v[0] - v[1];
    } else if (R == 4) {
      cplx<T> a0 = v[0] + v[2], a1 = v[0] - v[2], a2 = v[1] + v[3], d = v[1] - v[3];
      cplx<T> a3 = sign < 0 ? mk(d.im, -d.re) : mk(-d.im, d.re);
      y[0] = a0 + a2; y[2] = a0 - a2; y[1] = a1 + a3; y[3] = a1 - a3;
    } else {
      // direct R-point DFT with the table entries of the R-th roots of unity
#pragma unroll
      for (int q = 0; q < R; ++q) {
        cplx<T> s = v[0];
#pragma unroll
        for (int r = 1; r < R; ++r) {
          cplx<T> w = tw[((r * q) % R) * M];
          if (sign > 0) w.im = -w.im;
          s = s + cmul(v[r], w);
        }
        y[q] = s;
      }
    }
    cplx<T> *dst = out + line * N + (j / Ns) * Ns * R + k;
#pragma unroll
    for (int r = 0; r < R; ++r) dst[r * Ns] = y[r];
  }
}

// Full unnormalised FFT of `nlines` lines in shared memory.  Data starts in
// buf[0]; returns the buffer index (0/1) that holds the result.  Every
// thread of the block must call it (it synchronises between stages).
template <typename T>
__device__ int fft_lines(cplx<T> *buf0, cplx<T> *buf1, const RadixPlan &rp, int nlines,
                         const cplx<T> *tw, int sign) {
  cplx<T> *b[2] = {buf0, buf1};
  int cur = 0;
  int Ns = 1;
  for (int s = 0; s < rp.nstages; ++s) {
    const int R = rp.radix[s];
    if (R == 4) stockham_stage<T, 4>(b[cur], b[cur ^ 1], rp.n, nlines, Ns, tw, sign);
    else if (R == 2) stockham_stage<T, 2>(b[cur], b[cur ^ 1], rp.n, nlines, Ns, tw, sign);
    else if (R == 3) stockham_stage<T, 3>(b[cur], b[cur ^ 1], rp.n, nlines, Ns, tw, sign);
    else stockham_stage<T, 5>(b[cur], b[cur ^ 1], rp.n, nlines, Ns, tw, sign);
    __syncthreads();
    cur ^= 1;
    Ns *= R;
  }
  return cur;
}

// Point (w, i) of a tile of TW lines from a flat index: consecutive indices
// walk the contiguous direction in memory (along the line when es == 1,
// across the TW lines otherwise) so that global accesses coalesce.
__device__ __forceinline__ void tile_coord(int idx, int TW, int N, int es, int &w, int &i) {
  if (es == 1) { w = idx / N; i = idx - w * N; }
  else { i = idx / TW; w = idx - i * TW; }
}

// Deterministic block sum of one double per thread (fixed shuffle tree).
__device__ __forceinline__ double block_sum(double v, double *red) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) red[warp] = v;
  __syncthreads();
  double t = 0;
  if (threadIdx.x == 0) {
    const int nw = (blockDim.x + 31) >> 5;
    for (int w = 0; w < nw; ++w) t += red[w];
  }
  return t;  // valid on thread 0
}

}  // namespace qdg
