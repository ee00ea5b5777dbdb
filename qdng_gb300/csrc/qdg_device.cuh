// qdg_device.cuh -- device-side building blocks of the propagation engine.
//
// Complex arithmetic, the shared-memory Stockham FFT used for the grid
// kinetic operator, and deterministic block reductions.  Everything is
// templated on the arithmetic type T (double for the FP64 drop-in path,
// float for the FP32 bulk of the mixed path).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <type_traits>

#include "qdg_schedule.h"

namespace qdg {

template <typename T> struct cplx { T re, im; };

// ---- double-float: an unevaluated sum hi + lo of two FP32 numbers ---------
// GB300 executes FP64 at 1/64 of the FP32 rate.  The DF64 precision form
// (QDG_PREC_DF64) runs the bulk and the FFTs of its multi-dimensional step
// kernel in this type; the FP64 form is binary64 throughout.  About 48 significant bits (error-free transformations:
// Knuth's TwoSum, Dekker/FMA products; the addition is the "sloppy" form,
// whose error is bounded by ~2^-47 of the operands' magnitude, which is what
// a normwise FFT error bound needs).  The round-to-nearest intrinsics keep
// the compiler from contracting the transformations.
struct dfl {
  float hi, lo;
  __host__ __device__ constexpr dfl() : hi(0.0f), lo(0.0f) {}
  __host__ __device__ constexpr dfl(float h, float l) : hi(h), lo(l) {}
  __host__ __device__ constexpr dfl(double x) : hi((float)x), lo((float)(x - (double)(float)x)) {}
  __host__ __device__ constexpr dfl(int x) : hi((float)x), lo(0.0f) {}
};
// A complex double-float is 16 bytes, like a complex double; aligned so that
// shared-memory and global accesses move it with one 128-bit instruction.
template <> struct __align__(16) cplx<dfl> { dfl re, im; };

__device__ __forceinline__ dfl df_fast(float s, float e) {  // |s| >= |e|
  const float h = __fadd_rn(s, e);
  return dfl(h, __fsub_rn(e, __fsub_rn(h, s)));
}
__device__ __forceinline__ dfl operator+(dfl a, dfl b) {
  const float s = __fadd_rn(a.hi, b.hi);
  const float bb = __fsub_rn(s, a.hi);
  float e = __fadd_rn(__fsub_rn(a.hi, __fsub_rn(s, bb)), __fsub_rn(b.hi, bb));
  e = __fadd_rn(e, __fadd_rn(a.lo, b.lo));
  return df_fast(s, e);
}
__device__ __forceinline__ dfl operator-(dfl a) { return dfl(-a.hi, -a.lo); }
__device__ __forceinline__ dfl operator-(dfl a, dfl b) { return a + (-b); }
__device__ __forceinline__ dfl operator*(dfl a, dfl b) {
  const float p = __fmul_rn(a.hi, b.hi);
  float e = __fmaf_rn(a.hi, b.hi, -p);
  e = __fmaf_rn(a.hi, b.lo, e);
  e = __fmaf_rn(a.lo, b.hi, e);
  return df_fast(p, e);
}
__device__ __forceinline__ double df_to_double(dfl a) { return (double)a.hi + (double)a.lo; }
__device__ __forceinline__ dfl df_from_double(double x) {
  const float h = __double2float_rn(x);
  return dfl(h, __double2float_rn(x - (double)h));
}

// Bulk-type helpers for float, double and double-float (the step kernel's
// phi, T_d phi and potential values).
__device__ __forceinline__ double b2d(float x) { return (double)x; }
__device__ __forceinline__ double b2d(double x) { return x; }
__device__ __forceinline__ double fma_b(double a, double b, double c) { return fma(a, b, c); }
__device__ __forceinline__ double b2d(dfl x) { return df_to_double(x); }
__device__ __forceinline__ float fma_b(float a, float b, float c) { return fmaf(a, b, c); }
__device__ __forceinline__ dfl fma_b(dfl a, dfl b, dfl c) { return a * b + c; }
template <typename B> __device__ __forceinline__ B d2b(double x);
template <> __device__ __forceinline__ float d2b<float>(double x) { return (float)x; }
template <> __device__ __forceinline__ dfl d2b<dfl>(double x) { return df_from_double(x); }
template <> __device__ __forceinline__ double d2b<double>(double x) { return x; }
__device__ __forceinline__ double ldg_b(const double *p) { return __ldg(p); }
__device__ __forceinline__ float ldg_b(const float *p) { return __ldg(p); }
__device__ __forceinline__ dfl ldg_b(const dfl *p) {
  const float2 v = __ldg(reinterpret_cast<const float2 *>(p));
  return dfl(v.x, v.y);
}
__device__ __forceinline__ cplx<dfl> ldcg(const cplx<dfl> *p) {
  const float4 v = __ldcg(reinterpret_cast<const float4 *>(p));
  return cplx<dfl>{dfl(v.x, v.y), dfl(v.z, v.w)};
}
__device__ __forceinline__ void st(cplx<dfl> *p, cplx<dfl> c) {
  *reinterpret_cast<float4 *>(p) = make_float4(c.re.hi, c.re.lo, c.im.hi, c.im.lo);
}

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
// The operand of a potential-matrix entry: x, or -i x for an entry that acts
// as a negative imaginary potential (selects and a sign flip, no arithmetic).
template <typename T> __device__ __forceinline__ cplx<T> nim_operand(cplx<T> x, int nim) {
  return nim ? mk(x.im, -x.re) : x;
}
template <typename T, typename U> __device__ __forceinline__ cplx<T> ccast(cplx<U> a) { return mk((T)a.re, (T)a.im); }

template <typename T> __device__ __forceinline__ cplx<T> ldg(const cplx<T> *p) {
  typedef typename vec2<T>::type V;
  V v = __ldg(reinterpret_cast<const V *>(p));
  return mk<T>(v.x, v.y);
}
// Asynchronous global -> shared copies (cp.async): 16-byte copies through L2
// only (data written by other blocks of the same kernel), 8-byte copies of
// read-only data through L1; committed as groups and awaited by count.
__device__ __forceinline__ void cp_async16(void *dst, const void *src) {
  const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async8(void *dst, const void *src) {
  const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N> __device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

// Load through L2 only: data written by other blocks earlier in the same
// kernel (after a grid barrier) must not come from a stale L1 line.
template <typename T> __device__ __forceinline__ cplx<T> ldcg(const cplx<T> *p) {
  typedef typename vec2<T>::type V;
  V v = __ldcg(reinterpret_cast<const V *>(p));
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


// ---- small DFTs in registers ---------------------------------------------
// Constants of the 8th and 16th roots of unity (mathematical values).
#define QDG_SQRT1_2 0.70710678118654752440
#define QDG_COS_PI8 0.92387953251128675613
#define QDG_SIN_PI8 0.38268343236508977173

// multiply by -i (sign < 0) or +i (sign > 0)
template <typename T> __device__ __forceinline__ cplx<T> rot90(cplx<T> a, int sign) {
  return sign < 0 ? mk(a.im, -a.re) : mk(-a.im, a.re);
}

// 4-point DFT, in place: y_k = sum_n x_n exp(sign 2 pi i nk/4)
template <typename T> __device__ __forceinline__ void dft4(cplx<T> &x0, cplx<T> &x1, cplx<T> &x2, cplx<T> &x3,
                                                          int sign) {
  const cplx<T> a0 = x0 + x2, a1 = x0 - x2, a2 = x1 + x3, a3 = rot90(x1 - x3, sign);
  x0 = a0 + a2; x2 = a0 - a2; x1 = a1 + a3; x3 = a1 - a3;
}

// a * exp(sign 2 pi i m/16) for m = 1..9 with the special values of the
// 8th roots of unity; m is a compile-time constant after unrolling.
template <typename T> __device__ __forceinline__ cplx<T> tw16(cplx<T> a, int m, int sign) {
  const T c = (T)QDG_COS_PI8, sn = (T)QDG_SIN_PI8, h = (T)QDG_SQRT1_2;
  const T sg = sign < 0 ? (T)-1 : (T)1;
  switch (m) {
    case 0: return a;
    case 1: return cmul(a, mk(c, sg * sn));
    case 2: return mk(h * (a.re - sg * a.im), h * (a.im + sg * a.re));
    case 3: return cmul(a, mk(sn, sg * c));
    case 4: return rot90(a, sign);
    case 6: return mk(h * (-a.re - sg * a.im), h * (-a.im + sg * a.re));
    case 9: return cmul(a, mk(-c, -sg * sn));
  }
  return a;
}

// 8-point DFT (4 x 2): y[k1 + 4 k2] = sum_n2 W2^(n2 k2) W8^(n2 k1) sum_n1 x[2 n1 + n2] W4^(n1 k1)
template <typename T> __device__ __forceinline__ void dft8(cplx<T> *x, int sign) {
  dft4(x[0], x[2], x[4], x[6], sign);
  dft4(x[1], x[3], x[5], x[7], sign);
  // now x[2 k1 + n2] holds a[n2][k1]
  cplx<T> y[8];
#pragma unroll
  for (int k1 = 0; k1 < 4; ++k1) {
    const cplx<T> a0 = x[2 * k1];
    const cplx<T> a1 = tw16(x[2 * k1 + 1], 2 * k1, sign);  // W8^k1 = W16^(2 k1)
    y[k1] = a0 + a1;
    y[k1 + 4] = a0 - a1;
  }
#pragma unroll
  for (int k = 0; k < 8; ++k) x[k] = y[k];
}

// 16-point DFT (4 x 4): y[k1 + 4 k2] = sum_n2 W4^(n2 k2) W16^(n2 k1) sum_n1 x[4 n1 + n2] W4^(n1 k1)
template <typename T> __device__ __forceinline__ void dft16(cplx<T> *x, int sign) {
#pragma unroll
  for (int n2 = 0; n2 < 4; ++n2) dft4(x[n2], x[4 + n2], x[8 + n2], x[12 + n2], sign);
  // x[4 k1 + n2] holds a[n2][k1]
  cplx<T> y[16];
#pragma unroll
  for (int k1 = 0; k1 < 4; ++k1) {
    cplx<T> b0 = x[4 * k1 + 0];
    cplx<T> b1 = tw16(x[4 * k1 + 1], k1, sign);
    cplx<T> b2 = tw16(x[4 * k1 + 2], 2 * k1, sign);
    cplx<T> b3 = tw16(x[4 * k1 + 3], 3 * k1, sign);
    dft4(b0, b1, b2, b3, sign);
    y[k1] = b0; y[k1 + 4] = b1; y[k1 + 8] = b2; y[k1 + 12] = b3;
  }
#pragma unroll
  for (int k = 0; k < 16; ++k) x[k] = y[k];
}

// Twiddles w^(r*k) and the R-point DFT of one Stockham item, in registers;
// twf(m) returns w^m = exp(-2 pi i m / N).
template <typename T, int R, typename TwF>
__device__ __forceinline__ void stage_butterfly_t(cplx<T> (&v)[R], int k, int step, int M, TwF twf, int sign) {
  if (k) {
#pragma unroll
    for (int r = 1; r < R; ++r) {
      cplx<T> w = twf(r * k * step);  // r*k*step < R*Ns*step = N
      if (sign > 0) w.im = -w.im;
      v[r] = cmul(v[r], w);
    }
  }
  if (R == 2) {
    const cplx<T> a = v[0];
    v[0] = a + v[1];
    v[1] = a - v[1];
  } else if (R == 4) {
    dft4(v[0], v[1], v[2], v[3], sign);
  } else if (R == 8) {
    dft8(v, sign);
  } else if (R == 16) {
    dft16(v, sign);
  } else {
    // direct R-point DFT with the table entries of the R-th roots of unity
    cplx<T> y[R];
#pragma unroll
    for (int qq = 0; qq < R; ++qq) {
      cplx<T> s = v[0];
#pragma unroll
      for (int r = 1; r < R; ++r) {
        cplx<T> w = twf(((r * qq) % R) * M);
        if (sign > 0) w.im = -w.im;
        s = s + cmul(v[r], w);
      }
      y[qq] = s;
    }
#pragma unroll
    for (int qq = 0; qq < R; ++qq) v[qq] = y[qq];
  }
}

template <typename T, int R>
__device__ __forceinline__ void stage_butterfly(cplx<T> (&v)[R], int k, int step, int M,
                                                const cplx<T> *__restrict__ tw, int sign) {
  stage_butterfly_t<T, R>(v, k, step, M, [tw](int m) { return tw[m]; }, sign);
}

// Shared-memory layout of a batch of lines: line l starts at l * lstride(N)
// and element i of a line sits at lpos(i) = i + i/16.  The gap after every 16
// elements spreads the stride-R stores of a Stockham stage with Ns = 1 (and
// of radix-16 chains in general) over distinct banks; the odd line stride
// does the same for accesses that walk across lines (the gather and scatter
// of lines along dimensions other than 0, where consecutive threads take
// consecutive lines so that the global accesses coalesce).
__host__ __device__ __forceinline__ int lstride(int N) { return (N + (N >> 4)) | 1; }
__device__ __forceinline__ int lpos(int i) { return i + (i >> 4); }
__host__ __device__ __forceinline__ int lidx(int l, int i, int LS) { return l * LS + i + (i >> 4); }
// Complex elements of a line-batch buffer of nlines lines of length N.
__host__ __device__ __forceinline__ size_t line_buf_elems(int N, int nlines) { return (size_t)nlines * lstride(N); }

// One Stockham stage over `nlines` lines of length N stored in the layout
// above in `in`; result in `out`.  Items are spread over all
// threads of the block.  tw[m] = exp(-2 pi i m / N); sign = -1 forward
// (FFTW_FORWARD), +1 backward.  The Stockham autosort indexing follows the
// classic formulation (Stockham 1966; Govindaraju et al., SC'08): item j
// reads in[j + r*N/R], applies the stage twiddles w^(r*k), does the R-point
// DFT in registers and writes out[(j/Ns)*Ns*R + k + r*Ns], k = j mod Ns.
template <typename T, int R>
__device__ __forceinline__ void stockham_stage(const cplx<T> *__restrict__ in, cplx<T> *__restrict__ out,
                                               int N, int nlines, int Ns, const cplx<T> *__restrict__ tw,
                                               int sign) {
  const int M = N / R;
  const int step = N / (Ns * R);
  const int items = nlines * M;
  // powers of two (the usual case): shifts and masks instead of divisions
  const bool pow2 = ((M & (M - 1)) == 0) && ((Ns & (Ns - 1)) == 0);
  const int lgM = __ffs(M) - 1, lgNs = __ffs(Ns) - 1;
  const int LS = lstride(N);
  for (int it = threadIdx.x; it < items; it += blockDim.x) {
    int line, j, k, q;
    if (pow2) {
      line = it >> lgM;
      j = it & (M - 1);
      k = j & (Ns - 1);
      q = j >> lgNs;
    } else {
      line = it / M;
      j = it - line * M;
      q = j / Ns;
      k = j - q * Ns;
    }
    const cplx<T> *src = in + line * LS;
    cplx<T> v[R];
#pragma unroll
    for (int r = 0; r < R; ++r) v[r] = src[lpos(j + r * M)];
    stage_butterfly<T, R>(v, k, step, M, tw, sign);
    cplx<T> *dst = out + line * LS;
    const int o = q * Ns * R + k;
#pragma unroll
    for (int r = 0; r < R; ++r) dst[lpos(o + r * Ns)] = v[r];
  }
}

// A stage of a prime radix R outside {2, 3, 5} (a line length with other
// prime factors, which FFTW takes too): the same Stockham indexing with R a
// runtime value; each output is a direct R-point sum over the twiddled
// inputs, read from shared memory again for every output (O(R^2) work per
// item, no register array of R values).
template <typename T>
__device__ __noinline__ void stockham_stage_gen(const cplx<T> *__restrict__ in, cplx<T> *__restrict__ out, int N,
                                                int R, int nlines, int Ns, const cplx<T> *__restrict__ tw,
                                                int sign) {
  const int M = N / R;
  const int step = N / (Ns * R);
  const int items = nlines * M;
  const int LS = lstride(N);
  for (int it = threadIdx.x; it < items; it += blockDim.x) {
    const int line = it / M, j = it - line * M;
    const int q = j / Ns, k = j - q * Ns;
    const cplx<T> *src = in + line * LS;
    cplx<T> *dst = out + line * LS;
    const int o = q * Ns * R + k;
    for (int qq = 0; qq < R; ++qq) {
      cplx<T> acc = src[lpos(j)];
      int e = 0;  // (r qq) mod R
      for (int r = 1; r < R; ++r) {
        e += qq;
        if (e >= R) e -= R;
        cplx<T> v = src[lpos(j + r * M)];
        if (k) {
          cplx<T> w = tw[r * k * step];  // r k step < R Ns step = N
          if (sign > 0) w.im = -w.im;
          v = cmul(v, w);
        }
        cplx<T> w = tw[e * M];
        if (sign > 0) w.im = -w.im;
        acc = acc + cmul(v, w);
      }
      dst[lpos(o + qq * Ns)] = acc;
    }
  }
}

// The same stage with the element reads and writes as functors, load(idx)
// and store(idx, value) with idx = line * N + position, so that a caller can
// fuse a multiply into the loads of a stage or its point update into the
// stores of the last one.
template <typename T, int R, typename Load, typename Store, typename TwF>
__device__ __forceinline__ void stockham_stage_io(Load load, Store store, int N, int nlines, int Ns, TwF twf,
                                                  int sign) {
  const int M = N / R;
  const int step = N / (Ns * R);
  const int items = nlines * M;
  const bool pow2 = ((M & (M - 1)) == 0) && ((Ns & (Ns - 1)) == 0);
  const int lgM = __ffs(M) - 1, lgNs = __ffs(Ns) - 1;
  for (int it = threadIdx.x; it < items; it += blockDim.x) {
    int line, j, k, q;
    if (pow2) {
      line = it >> lgM;
      j = it & (M - 1);
      k = j & (Ns - 1);
      q = j >> lgNs;
    } else {
      line = it / M;
      j = it - line * M;
      q = j / Ns;
      k = j - q * Ns;
    }
    cplx<T> v[R];
#pragma unroll
    for (int r = 0; r < R; ++r) v[r] = load(line * N + j + r * M);
    stage_butterfly_t<T, R>(v, k, step, M, twf, sign);
    const int dst = line * N + q * Ns * R + k;
#pragma unroll
    for (int r = 0; r < R; ++r) store(dst + r * Ns, v[r]);
  }
}

// One functor stage of any radix of a plan; twf(m) returns w^m.
template <typename T, typename Load, typename Store, typename TwF>
__device__ __forceinline__ void stage_any(int R, Load load, Store store, int N, int nlines, int Ns, TwF twf,
                                          int sign) {
  if (R == 16) stockham_stage_io<T, 16>(load, store, N, nlines, Ns, twf, sign);
  else if (R == 8) stockham_stage_io<T, 8>(load, store, N, nlines, Ns, twf, sign);
  else if (R == 4) stockham_stage_io<T, 4>(load, store, N, nlines, Ns, twf, sign);
  else if (R == 2) stockham_stage_io<T, 2>(load, store, N, nlines, Ns, twf, sign);
  else if (R == 3) stockham_stage_io<T, 3>(load, store, N, nlines, Ns, twf, sign);
  else stockham_stage_io<T, 5>(load, store, N, nlines, Ns, twf, sign);
}

// Full unnormalised FFT of `nlines` lines in shared memory (layout above,
// line_buf_elems(N, nlines) elements per buffer).  Data starts in buf0;
// returns the buffer index (0/1) that holds the result.  Every
// thread of the block must call it (it synchronises between stages).
template <typename T>
__device__ int fft_lines(cplx<T> *buf0, cplx<T> *buf1, const RadixPlan &rp, int nlines,
                         const cplx<T> *tw, int sign) {
  cplx<T> *b[2] = {buf0, buf1};
  int cur = 0;
  int Ns = 1;
  for (int s = 0; s < rp.nstages; ++s) {
    const int R = rp.radix[s];
    if (R == 16) stockham_stage<T, 16>(b[cur], b[cur ^ 1], rp.n, nlines, Ns, tw, sign);
    else if (R == 8) stockham_stage<T, 8>(b[cur], b[cur ^ 1], rp.n, nlines, Ns, tw, sign);
    else if (R == 4) stockham_stage<T, 4>(b[cur], b[cur ^ 1], rp.n, nlines, Ns, tw, sign);
    else if (R == 2) stockham_stage<T, 2>(b[cur], b[cur ^ 1], rp.n, nlines, Ns, tw, sign);
    else if (R == 3) stockham_stage<T, 3>(b[cur], b[cur ^ 1], rp.n, nlines, Ns, tw, sign);
    else if (R == 5) stockham_stage<T, 5>(b[cur], b[cur ^ 1], rp.n, nlines, Ns, tw, sign);
    else stockham_stage_gen<T>(b[cur], b[cur ^ 1], rp.n, R, nlines, Ns, tw, sign);
    __syncthreads();
    cur ^= 1;
    Ns *= R;
  }
  return cur;
}

// ---- transforms with the direction known at compile time ----------------
// SIGN = -1: forward (FFTW_FORWARD, exp(-2 pi i nk/N)); +1: backward.  With
// the direction a template constant the +-1 factors of the butterflies fold
// into additions and subtractions: on GB300 every binary64 operation costs
// 1/64 of an FP32 one, so none is spent on a sign.
template <int SIGN, typename T> __device__ __forceinline__ cplx<T> rot90s(cplx<T> a) {
  if constexpr (SIGN < 0) return mk(a.im, -a.re);
  else return mk(-a.im, a.re);
}
template <int SIGN, typename T>
__device__ __forceinline__ void dft4s(cplx<T> &x0, cplx<T> &x1, cplx<T> &x2, cplx<T> &x3) {
  const cplx<T> a0 = x0 + x2, a1 = x0 - x2, a2 = x1 + x3, a3 = rot90s<SIGN>(x1 - x3);
  x0 = a0 + a2; x2 = a0 - a2; x1 = a1 + a3; x3 = a1 - a3;
}
// a * exp(SIGN 2 pi i m/16); m is a constant after unrolling.
template <int SIGN, typename T> __device__ __forceinline__ cplx<T> tw16s(cplx<T> a, int m) {
  const T c = (T)QDG_COS_PI8, sn = (T)QDG_SIN_PI8, h = (T)QDG_SQRT1_2;
  if constexpr (SIGN < 0) {
    switch (m) {
      case 0: return a;
      case 1: return mk(c * a.re + sn * a.im, c * a.im - sn * a.re);
      case 2: return mk(h * (a.re + a.im), h * (a.im - a.re));
      case 3: return mk(sn * a.re + c * a.im, sn * a.im - c * a.re);
      case 4: return mk(a.im, -a.re);
      case 6: return mk(h * (a.im - a.re), -(h * (a.re + a.im)));
      case 9: return mk(-(c * a.re + sn * a.im), sn * a.re - c * a.im);
    }
  } else {
    switch (m) {
      case 0: return a;
      case 1: return mk(c * a.re - sn * a.im, c * a.im + sn * a.re);
      case 2: return mk(h * (a.re - a.im), h * (a.im + a.re));
      case 3: return mk(sn * a.re - c * a.im, sn * a.im + c * a.re);
      case 4: return mk(-a.im, a.re);
      case 6: return mk(-(h * (a.re + a.im)), h * (a.re - a.im));
      case 9: return mk(sn * a.im - c * a.re, -(c * a.im + sn * a.re));
    }
  }
  return a;
}
template <int SIGN, typename T> __device__ __forceinline__ void dft8s(cplx<T> *x) {
  dft4s<SIGN>(x[0], x[2], x[4], x[6]);
  dft4s<SIGN>(x[1], x[3], x[5], x[7]);
  cplx<T> y[8];
#pragma unroll
  for (int k1 = 0; k1 < 4; ++k1) {
    const cplx<T> a0 = x[2 * k1];
    const cplx<T> a1 = tw16s<SIGN>(x[2 * k1 + 1], 2 * k1);
    y[k1] = a0 + a1;
    y[k1 + 4] = a0 - a1;
  }
#pragma unroll
  for (int k = 0; k < 8; ++k) x[k] = y[k];
}
template <int SIGN, typename T> __device__ __forceinline__ void dft16s(cplx<T> *x) {
#pragma unroll
  for (int n2 = 0; n2 < 4; ++n2) dft4s<SIGN>(x[n2], x[4 + n2], x[8 + n2], x[12 + n2]);
  cplx<T> y[16];
#pragma unroll
  for (int k1 = 0; k1 < 4; ++k1) {
    cplx<T> b0 = x[4 * k1 + 0];
    cplx<T> b1 = tw16s<SIGN>(x[4 * k1 + 1], k1);
    cplx<T> b2 = tw16s<SIGN>(x[4 * k1 + 2], 2 * k1);
    cplx<T> b3 = tw16s<SIGN>(x[4 * k1 + 3], 3 * k1);
    dft4s<SIGN>(b0, b1, b2, b3);
    y[k1] = b0; y[k1 + 4] = b1; y[k1 + 8] = b2; y[k1 + 12] = b3;
  }
#pragma unroll
  for (int k = 0; k < 16; ++k) x[k] = y[k];
}
// a * w (SIGN < 0) or a * conj(w) (SIGN > 0), w from the forward table
template <int SIGN, typename T> __device__ __forceinline__ cplx<T> twmul(cplx<T> a, cplx<T> w) {
  if constexpr (SIGN < 0) return mk(a.re * w.re - a.im * w.im, a.re * w.im + a.im * w.re);
  else return mk(a.re * w.re + a.im * w.im, a.im * w.re - a.re * w.im);
}
// Stage twiddles w^(r k step) and the R-point DFT of one Stockham item;
// twf(m) returns exp(-2 pi i m/N).
template <typename T, int R, int SIGN, typename TwF>
__device__ __forceinline__ void butterfly_s(cplx<T> (&v)[R], int k, int step, int M, TwF twf) {
  if (k) {
#pragma unroll
    for (int r = 1; r < R; ++r) v[r] = twmul<SIGN>(v[r], twf(r * k * step));
  }
  if constexpr (R == 2) {
    const cplx<T> a = v[0];
    v[0] = a + v[1];
    v[1] = a - v[1];
  } else if constexpr (R == 4) {
    dft4s<SIGN>(v[0], v[1], v[2], v[3]);
  } else if constexpr (R == 8) {
    dft8s<SIGN>(v);
  } else if constexpr (R == 16) {
    dft16s<SIGN>(v);
  } else {
    cplx<T> y[R];
#pragma unroll
    for (int qq = 0; qq < R; ++qq) {
      cplx<T> s = v[0];
#pragma unroll
      for (int r = 1; r < R; ++r) s = s + twmul<SIGN>(v[r], twf(((r * qq) % R) * M));
      y[qq] = s;
    }
#pragma unroll
    for (int qq = 0; qq < R; ++qq) v[qq] = y[qq];
  }
}

// One Stockham stage of `nlines` lines read from the padded shared-memory
// layout `in`; outputs go to store(line, position, value).  lfast: items
// are spread with the line index fastest (consecutive threads take the same
// position of consecutive lines, so a global store along a strided
// dimension coalesces); otherwise the position within a line is fastest.
template <typename T, int R, int SIGN, typename Store, typename TwF>
__device__ __forceinline__ void stage_s(const cplx<T> *__restrict__ in, Store store, int N, int nlines, int Ns,
                                        bool lfast, TwF twf) {
  const int M = N / R;
  const int step = N / (Ns * R);
  const int items = nlines * M;
  const bool pow2 = ((M & (M - 1)) == 0) && ((Ns & (Ns - 1)) == 0);
  const int lgM = __ffs(M) - 1, lgNs = __ffs(Ns) - 1;
  const int LS = lstride(N);
  for (int it = threadIdx.x; it < items; it += blockDim.x) {
    int line, j;
    if (lfast) { j = it / nlines; line = it - j * nlines; }
    else if (pow2) { line = it >> lgM; j = it & (M - 1); }
    else { line = it / M; j = it - line * M; }
    int q, k;
    if (pow2) { q = j >> lgNs; k = j & (Ns - 1); }
    else { q = j / Ns; k = j - q * Ns; }
    const cplx<T> *src = in + line * LS;
    cplx<T> v[R];
#pragma unroll
    for (int r = 0; r < R; ++r) v[r] = src[lpos(j + r * M)];
    butterfly_s<T, R, SIGN>(v, k, step, M, twf);
    const int o = q * Ns * R + k;
#pragma unroll
    for (int r = 0; r < R; ++r) store(line, o + r * Ns, v[r]);
  }
}

// stage_s with a runtime prime radix R (the direct sum of stockham_stage_gen).
template <typename T, int SIGN, typename Store, typename TwF>
__device__ void stage_s_gen(int R, const cplx<T> *__restrict__ in, Store store, int N, int nlines, int Ns,
                            bool lfast, TwF twf) {
  const int M = N / R;
  const int step = N / (Ns * R);
  const int items = nlines * M;
  const int LS = lstride(N);
  for (int it = threadIdx.x; it < items; it += blockDim.x) {
    int line, j;
    if (lfast) { j = it / nlines; line = it - j * nlines; }
    else { line = it / M; j = it - line * M; }
    const int q = j / Ns, k = j - q * Ns;
    const cplx<T> *src = in + line * LS;
    const int o = q * Ns * R + k;
    for (int qq = 0; qq < R; ++qq) {
      cplx<T> acc = src[lpos(j)];
      int e = 0;
      for (int r = 1; r < R; ++r) {
        e += qq;
        if (e >= R) e -= R;
        cplx<T> v = src[lpos(j + r * M)];
        if (k) v = twmul<SIGN>(v, twf(r * k * step));
        acc = acc + twmul<SIGN>(v, twf(e * M));
      }
      store(line, o + qq * Ns, acc);
    }
  }
}

// GEN: also take prime radices outside {2, 3, 5} (callers whose plans may
// hold them; the step kernels' plans never do).
template <typename T, int SIGN, bool GEN = false, typename Store, typename TwF>
__device__ __forceinline__ void stage_s_any(int R, const cplx<T> *__restrict__ in, Store store, int N, int nlines,
                                            int Ns, bool lfast, TwF twf) {
  if (R == 16) stage_s<T, 16, SIGN>(in, store, N, nlines, Ns, lfast, twf);
  else if (R == 8) stage_s<T, 8, SIGN>(in, store, N, nlines, Ns, lfast, twf);
  else if (R == 4) stage_s<T, 4, SIGN>(in, store, N, nlines, Ns, lfast, twf);
  else if (R == 2) stage_s<T, 2, SIGN>(in, store, N, nlines, Ns, lfast, twf);
  else if (R == 3) stage_s<T, 3, SIGN>(in, store, N, nlines, Ns, lfast, twf);
  else if (!GEN || R == 5) stage_s<T, 5, SIGN>(in, store, N, nlines, Ns, lfast, twf);
  else stage_s_gen<T, SIGN>(R, in, store, N, nlines, Ns, lfast, twf);
}

// T_d of a batch of lines held in shared memory: forward FFT, the kinetic
// multiplier applied by the last forward stage (kmul(line, k-index, value)),
// inverse FFT whose last stage hands its outputs to out(line, position,
// value).  Data start in b0; b1 is the second ping-pong buffer.  Every
// thread of the block calls it; it synchronises between stages but not
// after the last one.
template <typename T, typename KMul, typename Out>
__device__ __forceinline__ void kinetic_lines(cplx<T> *b0, cplx<T> *b1, const RadixPlan &rp, int nlines,
                                              const cplx<T> *tw, KMul kmul, Out out, bool lfast_out) {
  cplx<T> *bb[2] = {b0, b1};
  const int N = rp.n, LS = lstride(N);
  auto twf = [tw](int m) { return tw[m]; };
  int cur = 0, Ns = 1;
  for (int s = 0; s < rp.nstages; ++s) {
    cplx<T> *dst = bb[cur ^ 1];
    if (s + 1 < rp.nstages) {
      stage_s_any<T, -1>(rp.radix[s], bb[cur], [dst, LS](int l, int i, cplx<T> v) { dst[lidx(l, i, LS)] = v; },
                         N, nlines, Ns, false, twf);
    } else {
      stage_s_any<T, -1>(rp.radix[s], bb[cur],
                         [dst, LS, kmul](int l, int i, cplx<T> v) { dst[lidx(l, i, LS)] = kmul(l, i, v); }, N,
                         nlines, Ns, false, twf);
    }
    __syncthreads();
    cur ^= 1;
    Ns *= rp.radix[s];
  }
  Ns = 1;
  for (int s = 0; s < rp.nstages; ++s) {
    cplx<T> *dst = bb[cur ^ 1];
    if (s + 1 < rp.nstages) {
      stage_s_any<T, 1>(rp.radix[s], bb[cur], [dst, LS](int l, int i, cplx<T> v) { dst[lidx(l, i, LS)] = v; }, N,
                        nlines, Ns, false, twf);
      __syncthreads();
    } else {
      stage_s_any<T, 1>(rp.radix[s], bb[cur], out, N, nlines, Ns, lfast_out, twf);
    }
    cur ^= 1;
    Ns *= rp.radix[s];
  }
}

// Point (w, i) of a tile of TW lines from a flat index: consecutive indices
// walk the contiguous direction in memory (along the line when es == 1,
// across the TW lines otherwise) so that global accesses coalesce.
__device__ __forceinline__ void tile_coord(int idx, int TW, int N, int es, int &w, int &i) {
  if (es == 1) { w = idx / N; i = idx - w * N; }
  else { i = idx / TW; w = idx - i * TW; }
}

// Deterministic block sum of one double per thread (fixed shuffle tree).
// Fixed-order block sum: a shuffle tree within each warp, then the warp sums
// by a second shuffle tree in warp 0 (a serial sum in one thread would be a
// chain of binary64 adds, ~80 cycles of the FP64 pipe each).
__device__ __forceinline__ double block_sum(double v, double *red) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) red[warp] = v;
  __syncthreads();
  double t = 0;
  if (warp == 0) {
    const int nw = (blockDim.x + 31) >> 5;
    t = lane < nw ? red[lane] : 0.0;
    for (int o = 16; o > 0; o >>= 1) t += __shfl_down_sync(0xffffffffu, t, o);
  }
  return t;  // valid on thread 0
}

}  // namespace qdg
