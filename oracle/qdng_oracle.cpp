/*
 * qdng_oracle.cpp -- CPU oracle for QDng's propagation hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker: a plain C++
 * restatement of the reference algorithms, used by tests/, by
 * __graft_entry__.smoke() and by bench.py's CPU-baseline leg.  The engine
 * (qdng_gb300/) never links or calls it.
 *
 * QDng itself cannot be compiled here: its hot path needs FFTW3, LAPACK,
 * the vendored Fortran SLATEC Bessel routines (no gfortran) and protobuf
 * generated headers.  So every function below restates the reference's
 * algorithm from its source, citing the file:line it follows (paths are
 * relative to the QDng source tree).  Third-party arithmetic is restated
 * from the published algorithms:
 *   - FFTW3 (unpinned; nixpkgs b7c2ada9 in flake.lock): unnormalised c2c
 *     DFT, forward sign -1, backward +1 (src/fft/fft.cpp:82-122,250-290).
 *     Here: mixed-radix Stockham autosort FFT.
 *   - SLATEC ZBESJ/ZBESI (src/slatec, kode 1 / kode 2): J_n(x), e^-x I_n(x)
 *     for n = 0..N-1.  Here: Miller's backward recurrence with the
 *     normalisation sums J0 + 2 sum J2k = 1 and e^-x (I0 + 2 sum Ik) = 1
 *     (Abramowitz & Stegun 9.1.46, 9.6.36), long double.
 *   - LAPACK dsyev/dstev (symmetric eigenproblems): cyclic Jacobi rotations.
 *   - LAPACK zhseqr/zhsein/zgetri (Arnoldi exp via eigenvectors):
 *     exp(c H) e0 by scaling and squaring of a Taylor series (long double).
 * Parity of the oracle itself is pinned against the golden values in QDng's
 * tests/checktests.sh (tests/test_oracle_golden.py).
 */
#include "../include/qdg.h"

#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <string>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

typedef std::complex<double> cd;
typedef std::complex<long double> cld;

namespace orc {

static thread_local std::string g_err;
static int fail(int code, const std::string &m) { g_err = m; return code; }

/* ------------------------------------------------------------------ FFT */
/* Unnormalised c2c DFT (FFTW contract, src/fft/fft.cpp:98-122): X_k = sum_j x_j e^{sign 2 pi i jk/n}. */
struct FFT1 {
  int n = 0;
  std::vector<int> radix;
  std::vector<cd> tw;  /* tw[m] = exp(-2 pi i m / n) */

  void init(int n_) {
    n = n_;
    radix.clear();
    int m = n;
    while (m % 4 == 0) { radix.push_back(4); m /= 4; }
    while (m % 2 == 0) { radix.push_back(2); m /= 2; }
    for (int p = 3; m > 1; p += 2) while (m % p == 0) { radix.push_back(p); m /= p; }
    tw.resize(n);
    const long double pi = 3.141592653589793238462643383279502884L;
    for (int k = 0; k < n; ++k) {
      long double a = -2.0L * pi * (long double)k / (long double)n;
      tw[k] = cd((double)cosl(a), (double)sinl(a));
    }
  }
  inline cd w(long m, int sign) const {
    cd t = tw[(size_t)(m % n)];
    return sign < 0 ? t : std::conj(t);
  }
  /* In place on x (contiguous), work has n entries. Stockham autosort. */
  void exec(cd *x, cd *work, int sign) const {
    if (n == 1) return;
    cd *in = x, *out = work;
    long Ns = 1;
    int rmax = 1;
    for (int R : radix) rmax = std::max(rmax, R);
    /* any prime factor is a direct R-point DFT; radices above 64 take heap buffers */
    cd vs[64], ys[64];
    std::vector<cd> vh, yh;
    if (rmax > 64) { vh.resize(rmax); yh.resize(rmax); }
    cd *v = rmax > 64 ? vh.data() : vs, *y = rmax > 64 ? yh.data() : ys;
    for (int R : radix) {
      long M = n / R;
      long step = n / (Ns * R);
      for (long j = 0; j < M; ++j) {
        long k = j % Ns;
        for (int r = 0; r < R; ++r) v[r] = in[j + r * M];
        if (k) for (int r = 1; r < R; ++r) v[r] *= w(r * k * step, sign);
        if (R == 2) {
          y[0] = v[0] + v[1]; y[1] = v[0] - v[1];
        } else if (R == 4) {
          cd a0 = v[0] + v[2], a1 = v[0] - v[2], a2 = v[1] + v[3], d = v[1] - v[3];
          cd a3 = sign < 0 ? cd(d.imag(), -d.real()) : cd(-d.imag(), d.real());
          y[0] = a0 + a2; y[2] = a0 - a2; y[1] = a1 + a3; y[3] = a1 - a3;
        } else {
          for (int q = 0; q < R; ++q) {
            cd s = 0;
            for (int r = 0; r < R; ++r) s += v[r] * w((long)((r * q) % R) * (n / R), sign);
            y[q] = s;
          }
        }
        long base = (j / Ns) * Ns * R + k;
        for (int r = 0; r < R; ++r) out[base + r * Ns] = y[r];
      }
      std::swap(in, out);
      Ns *= R;
    }
    if (in != x) std::memcpy(x, in, sizeof(cd) * n);
  }
};

/* N-D transform over a grid (dims reversed to C order in fft.cpp:93 is the
 * same set of 1-D transforms along every dimension). */
struct FFTN {
  int nd = 0; int n[QDG_MAX_DIMS]; long npts = 1;
  FFT1 f[QDG_MAX_DIMS];
  void init(const qdg_grid &g) {
    nd = g.ndims; npts = 1;
    for (int d = 0; d < nd; ++d) { n[d] = g.n[d]; npts *= n[d]; f[d].init(n[d]); }
  }
  void exec(cd *x, int sign) const {
    long stride = 1;
    for (int d = 0; d < nd; ++d) {
      long nl = n[d];
      long nlines = npts / nl;
      #pragma omp parallel if (nlines >= 16)
      {
        std::vector<cd> line(nl), work(nl);
        #pragma omp for schedule(static)
        for (long l = 0; l < nlines; ++l) {
          long lo = l % stride, hi = l / stride;
          cd *base = x + hi * stride * nl + lo;
          for (long i = 0; i < nl; ++i) line[i] = base[i * stride];
          f[d].exec(line.data(), work.data(), sign);
          for (long i = 0; i < nl; ++i) base[i * stride] = line[i];
        }
      }
      stride *= nl;
    }
  }
};

/* --------------------------------------------------------------- Bessel */
/* Start index of the backward recurrence: far enough above both the
 * highest wanted order and x that the neglected tail is below rounding. */
static int miller_start(int N, double x) {
  long double m = std::max<long double>(N, x);
  int s = (int)(m + 40 + 6 * sqrtl(m));
  return s + (s & 1);
}

/* ZBESJ underflow limit: components below it are set to zero (NZ). */
static int count_underflow(std::vector<double> &out) {
  const double ascle = 1.0e3 * 2.2250738585072014e-308 / 2.220446049250313e-16;
  int zeroes = 0;
  for (int i = (int)out.size() - 1; i >= 0; --i) {
    if (std::fabs(out[i]) < ascle) { out[i] = 0; ++zeroes; } else break;
  }
  return zeroes;
}

/* J_n(x), n = 0..N-1 (ZBESJ kode=1 as called in src/linalg/Bessel.cpp:22-58).
 * Miller: J_{k-1} = (2k/x) J_k - J_{k+1}, normalised by J_0 + 2 sum J_2k = 1.
 * Returns the number of trailing values that underflow to zero. */
static int bessel_j(int N, double x, std::vector<double> &out) {
  out.assign(N, 0.0);
  if (x == 0) { out[0] = 1; return count_underflow(out); }
  int M = miller_start(N, x);
  std::vector<long double> J(M + 2, 0.0L);
  J[M + 1] = 0; J[M] = 1e-30L;
  const long double big = 1e1000L;
  for (int k = M; k >= 1; --k) {
    J[k - 1] = (2.0L * k / (long double)x) * J[k] - J[k + 1];
    if (fabsl(J[k - 1]) > big)
      for (int i = k - 1; i <= M + 1; ++i) J[i] /= big;
  }
  long double sum = J[0];
  for (int k = 2; k <= M; k += 2) sum += 2 * J[k];
  for (int i = 0; i < N; ++i) out[i] = (double)(J[i] / sum);
  return count_underflow(out);
}

/* e^{-x} I_n(x), n = 0..N-1 (ZBESI kode=2, src/linalg/Bessel.cpp:61-97).
 * Miller: I_{k-1} = (2k/x) I_k + I_{k+1}, normalised by I_0 + 2 sum I_k = e^x. */
static int bessel_i_scaled(int N, double x, std::vector<double> &out) {
  out.assign(N, 0.0);
  if (x == 0) { out[0] = 1; return count_underflow(out); }
  int M = miller_start(N, x);
  std::vector<long double> I(M + 2, 0.0L);
  I[M + 1] = 0; I[M] = 1e-30L;
  const long double big = 1e1000L;
  for (int k = M; k >= 1; --k) {
    I[k - 1] = (2.0L * k / (long double)x) * I[k] + I[k + 1];
    if (I[k - 1] > big)
      for (int i = k - 1; i <= M + 1; ++i) I[i] /= big;
  }
  long double sum = I[0];
  for (int k = 1; k <= M; ++k) sum += 2 * I[k];
  for (int i = 0; i < N; ++i) out[i] = (double)(I[i] / sum);
  return count_underflow(out);
}

/* ------------------------------------------------------- small eigen */
/* Symmetric eigenproblem by cyclic Jacobi (stands in for LAPACK dsyev/dstev,
 * src/linalg/LapackDiag.cpp:22-100). a is n x n row-major, overwritten.
 * Eigenvalues ascending in w; eigenvectors as columns of z (row-major). */
static void jacobi_eig(int n, std::vector<long double> a, std::vector<long double> &w,
                       std::vector<long double> &z) {
  z.assign(n * n, 0); for (int i = 0; i < n; ++i) z[i * n + i] = 1;
  for (int sweep = 0; sweep < 100; ++sweep) {
    long double off = 0;
    for (int p = 0; p < n; ++p) for (int q = p + 1; q < n; ++q) off += a[p * n + q] * a[p * n + q];
    if (off < 1e-60L) break;
    for (int p = 0; p < n; ++p) for (int q = p + 1; q < n; ++q) {
      long double apq = a[p * n + q];
      if (fabsl(apq) < 1e-300L) continue;
      long double theta = (a[q * n + q] - a[p * n + p]) / (2 * apq);
      long double t = (theta >= 0 ? 1 : -1) / (fabsl(theta) + sqrtl(theta * theta + 1));
      long double c = 1 / sqrtl(t * t + 1), s = t * c;
      for (int k = 0; k < n; ++k) {
        long double akp = a[k * n + p], akq = a[k * n + q];
        a[k * n + p] = c * akp - s * akq; a[k * n + q] = s * akp + c * akq;
      }
      for (int k = 0; k < n; ++k) {
        long double apk = a[p * n + k], aqk = a[q * n + k];
        a[p * n + k] = c * apk - s * aqk; a[q * n + k] = s * apk + c * aqk;
      }
      for (int k = 0; k < n; ++k) {
        long double zkp = z[k * n + p], zkq = z[k * n + q];
        z[k * n + p] = c * zkp - s * zkq; z[k * n + q] = s * zkp + c * zkq;
      }
    }
  }
  std::vector<int> idx(n); for (int i = 0; i < n; ++i) idx[i] = i;
  std::sort(idx.begin(), idx.end(), [&](int x, int y) { return a[x * n + x] < a[y * n + y]; });
  w.resize(n);
  std::vector<long double> z2(n * n);
  for (int j = 0; j < n; ++j) {
    w[j] = a[idx[j] * n + idx[j]];
    for (int k = 0; k < n; ++k) z2[k * n + j] = z[k * n + idx[j]];
  }
  z = z2;
}

/* exp(c A) e0 for a small complex matrix by scaling and squaring. */
static std::vector<cd> expm_e0(int n, const std::vector<cd> &A, cd c) {
  std::vector<cld> M(n * n);
  long double nrm = 0;
  for (int i = 0; i < n * n; ++i) { M[i] = cld(A[i].real(), A[i].imag()) * cld(c.real(), c.imag()); nrm = std::max(nrm, (long double)std::abs(M[i])); }
  nrm *= n;
  int s = 0;
  while (nrm > 0.25L) { nrm *= 0.5L; ++s; }
  long double scale = ldexpl(1.0L, -s);
  for (auto &x : M) x *= scale;
  /* E = sum_k M^k / k! */
  std::vector<cld> E(n * n, 0), T(n * n, 0), Tn(n * n);
  for (int i = 0; i < n; ++i) { E[i * n + i] = 1; T[i * n + i] = 1; }
  for (int k = 1; k < 40; ++k) {
    for (int i = 0; i < n; ++i) for (int j = 0; j < n; ++j) {
      cld acc = 0; for (int l = 0; l < n; ++l) acc += T[i * n + l] * M[l * n + j];
      Tn[i * n + j] = acc / (long double)k;
    }
    T = Tn;
    for (int i = 0; i < n * n; ++i) E[i] += T[i];
  }
  for (int q = 0; q < s; ++q) {
    for (int i = 0; i < n; ++i) for (int j = 0; j < n; ++j) {
      cld acc = 0; for (int l = 0; l < n; ++l) acc += E[i * n + l] * E[l * n + j];
      Tn[i * n + j] = acc;
    }
    E = Tn;
  }
  std::vector<cd> v(n);
  for (int i = 0; i < n; ++i) v[i] = cd((double)E[i * n].real(), (double)E[i * n].imag());
  return v;
}

/* ------------------------------------------------------------- system */
struct System {
  qdg_grid g;
  int S = 1; long npts = 1;
  double dx[QDG_MAX_DIMS];
  std::vector<qdg_hterm> terms;
  std::vector<std::vector<double>> grids, lasers;
  int laser_nt = 0;
  bool hermitian = true;                  /* OMultistate _hermitian (OMultistate.cpp:14,52-53,83-85) */
  std::vector<std::vector<double>> ktab;  /* per kinetic term: collective k-space table */
  FFTN fft;
};

/* Kspace::Init1Dddx (src/qdlib/Kspace.cpp:60-96) for dimension d, spread over
 * the grid (OGridNabla::_InitDim, OGridNabla.cpp:172-180): k_d(p) * factor. */
static void kspace_ddx(const System &s, int d, double factor, std::vector<double> &tab) {
  long stride = 1;
  for (int i = 0; i < d; ++i) stride *= s.g.n[i];
  int Nx = s.g.n[d];
  double dp = (2 * M_PI) / (s.g.xmax[d] - s.g.xmin[d] + s.dx[d]);
  dp *= factor;
  std::vector<double> k1(Nx);
  if (Nx % 2 == 0) {
    for (int i = 0; i < Nx / 2; ++i) {
      k1[i] = double(i) * dp;
      k1[Nx - i - 1] = -1 * double(i + 1) * dp;
    }
  } else {
    k1[0] = 0;
    for (int i = 1; i < (Nx + 1) / 2; ++i) {
      k1[i] = double(i) * dp;
      k1[Nx - i] = -1 * double(i) * dp;
    }
  }
  tab.assign(s.npts, 0.0);
  for (long p = 0; p < s.npts; ++p) tab[p] = k1[(p / stride) % Nx];
}

/* Kspace::Init1Dd2dx2 (src/qdlib/Kspace.cpp:22-50) summed over dims
 * (Diff::_InitKspace collective part, src/qdlib/Diff.cpp:119-139). */
static void kspace_table(const System &s, const double *mass, std::vector<double> &tab) {
  tab.assign(s.npts, 0.0);
  long stride = 1;
  for (int d = 0; d < s.g.ndims; ++d) {
    int Nx = s.g.n[d];
    double L = s.g.xmax[d] - s.g.xmin[d];
    double dp = (2 * M_PI) / (L + s.dx[d]);
    dp *= dp;
    double factor = -1. / 2. / mass[d];   /* OGridNablaSq::Init, OGridNablaSq.cpp:51 */
    dp *= -factor;
    std::vector<double> k1(Nx);
    if (Nx % 2 == 0) {
      for (int i = 0; i < Nx / 2; ++i) {
        k1[i] = (double(i) * double(i)) * dp;
        k1[Nx - i - 1] = (double(i + 1) * double(i + 1)) * dp;
      }
    } else {
      k1[0] = 0;
      for (int i = 1; i < (Nx + 1) / 2; ++i) {
        k1[i] = (double(i) * double(i)) * dp;
        k1[Nx - i] = (double(i) * double(i)) * dp;
      }
    }
    for (long p = 0; p < s.npts; ++p) tab[p] += k1[(p / stride) % Nx];
    stride *= Nx;
  }
}

static double vec_max(const std::vector<double> &v) { double m = v[0]; for (double x : v) m = std::max(m, x); return m; }
static double vec_min(const std::vector<double> &v) { double m = v[0]; for (double x : v) m = std::min(m, x); return m; }

/* Element (i, j) of the matrix: the hermitian copy (OMultistate.cpp:122-132)
 * puts an off-diagonal element at (j, i) too. */
static bool term_at(const System &s, const qdg_hterm &t, int i, int j) {
  return (t.row == i && t.col == j) || (s.hermitian && t.row != t.col && t.row == j && t.col == i);
}

static double gmat_emax(const System &s, const qdg_hterm &t);
static double gmat_emin(const System &s, const qdg_hterm &t);

/* Emax/Emin of one operator: OGridNablaSq.cpp:89-106, OGridPotential.cpp:124-132, OGridDipole.cpp:36-44. */
static cd term_emax(const System &s, const qdg_hterm &t) {
  if (t.kind == QDG_TERM_KINETIC) {
    double T = 0;
    for (int d = 0; d < s.g.ndims; ++d) if (t.mass[d] > 0) T += 1 / (t.mass[d] * s.dx[d] * s.dx[d]);
    T *= (M_PI * M_PI / 2);
    return T;
  }
  if (t.kind == QDG_TERM_POTENTIAL) return vec_max(s.grids[t.grid]);
  if (t.kind == QDG_TERM_GMAT) return gmat_emax(s, t);
  if (t.kind == QDG_TERM_HOFD) {  /* OGridHOFD::Emax (OGridHOFD.cpp:97-111) */
    if (t.flags & 2) return cd(0, M_PI / s.dx[0]);
    double T = 0;
    for (int d = 0; d < s.g.ndims; ++d) {
      const double m = (t.flags & 4) ? t.mass[d] : 1.0;
      if (m > 0) T += 1 / (m * s.dx[d] * s.dx[d]);
    }
    return T * (M_PI * M_PI / 2);
  }
  if (t.kind == QDG_TERM_GOBBLER) return t.mass[0];  /* OGobbler::Emax = gain (OGobbler.cpp:161-164) */
  if (t.kind == QDG_TERM_NAC) {  /* OGridNAC::Emax (OGridNAC.cpp:105-115): dx of dim 0 */
    double m = 0;
    for (int d = 0; d < s.g.ndims; ++d) m += vec_max(s.grids[t.grid + d]);
    return m * M_PI / t.mass[0] / s.dx[0];
  }
  return vec_max(s.grids[t.grid]) * vec_max(s.lasers[t.laser]);
}
/* OGridNAC::Emin (OGridNAC.cpp:118-128) never adds the minima it computes and
 * returns 0; that is kept. */
static cd term_emin(const System &s, const qdg_hterm &t) {
  if (t.kind == QDG_TERM_POTENTIAL) return vec_min(s.grids[t.grid]);
  if (t.kind == QDG_TERM_GMAT) return gmat_emin(s, t);
  if (t.kind == QDG_TERM_HOFD) return (t.flags & 2) ? cd(0, -M_PI / s.dx[0]) : cd(0);  /* OGridHOFD.cpp:113-118 */
  /* OGobbler::Emin (OGobbler.cpp:166-170): -i gain as negative imaginary potential */
  if (t.kind == QDG_TERM_GOBBLER) return t.laser == 1 ? cd(0, -t.mass[0]) : cd(0);
  return 0.0;
}

/* OSum::Emax/Emin (OSum.cpp:28-51) and OMultistate::Emax/Emin (OMultistate.cpp:163-203). */
static void erange(const System &s, cd &emax, cd &emin) {
  if (s.S == 1) {
    emax = 0; emin = 0;
    for (auto &t : s.terms) { emax += term_emax(s, t); emin += term_emin(s, t); }
    return;
  }
  /* dsyev with uplo 'U' on the column-major matrix (LapackDiag.cpp:22-47)
   * reads the elements (i, j), i <= j, only. */
  int S = s.S;
  std::vector<long double> mx(S * S, 0), mn(S * S, 0);
  for (int i = 0; i < S; ++i) for (int j = i; j < S; ++j) {
    cd a = 0, b = 0; bool any = false;
    for (auto &t : s.terms) if (term_at(s, t, i, j)) { a += term_emax(s, t); b += term_emin(s, t); any = true; }
    if (any) {
      mx[i * S + j] = mx[j * S + i] = std::abs(a);
      mn[i * S + j] = mn[j * S + i] = std::abs(b);
    }
  }
  std::vector<long double> w, z;
  jacobi_eig(S, mx, w, z); emax = (double)w[S - 1];
  jacobi_eig(S, mn, w, z); emin = (double)w[0];
}

static double laser_at(const System &s, int l, long step) {
  if (step < 0 || step >= s.laser_nt) return 0.0;
  return s.lasers[l][step];
}

/* OGridNAC::Apply (OGridNAC.cpp:131-148) added to o: for every dimension d,
 * f_d (c d/dx_d x) and c d/dx_d (f_d x), c = sign/(2 mass); each derivative is
 * OGridNabla::Apply (OGridNabla.cpp:76-115): full FFT, times i k_d c / N
 * (MultElementsComplexEq, codelets/MultElementsComplexEqCCDd.h), inverse FFT.
 * The element's result is summed first and then added (Operator::ApplyAdd,
 * Operator.h:307-316). */
static void nac_apply(const System &s, const qdg_hterm &t, const cd *x, cd *o) {
  const long N = s.npts;
  const double sign = t.sign == 0 ? 1.0 : t.sign;
  const double c = 0.5 * sign / t.mass[0];
  std::vector<cd> b(N), acc(N, 0.0);
  std::vector<double> k;
  for (int d = 0; d < s.g.ndims; ++d) {
    const double *f = s.grids[t.grid + d].data();
    kspace_ddx(s, d, 1.0, k);
    const double fac = c / double(N);
    /* 1/2 f del psi */
    for (long p = 0; p < N; ++p) b[p] = x[p];
    s.fft.exec(b.data(), -1);
    for (long p = 0; p < N; ++p) b[p] = b[p] * (k[p] * cd(0, 1)) * fac;
    s.fft.exec(b.data(), +1);
    for (long p = 0; p < N; ++p) acc[p] += b[p] * f[p];
    /* 1/2 del f psi */
    for (long p = 0; p < N; ++p) b[p] = x[p] * f[p];
    s.fft.exec(b.data(), -1);
    for (long p = 0; p < N; ++p) b[p] = b[p] * (k[p] * cd(0, 1)) * fac;
    s.fft.exec(b.data(), +1);
    for (long p = 0; p < N; ++p) acc[p] += b[p];
  }
  for (long p = 0; p < N; ++p) o[p] += acc[p];
}

/* Central finite-difference weights in the layout of QDng's HOFD table
 * (HOFD.h:31-36, filled from cfd_table_1.h / cfd_table_2.h at HOFD.h:99-103):
 * cf[o2] weighs the point itself and cf[o2 - k] the neighbours at distance k
 * (for the first derivative cf is the lower neighbour's weight and the upper
 * one gets -cf).  The oracle does not read that table: it evaluates the
 * closed form of the central-difference weights on 2 o2 + 1 points
 * (B. Fornberg, Math. Comp. 51 (1988) 699-706), with r_k = (o2!)^2 /
 * ((o2 - k)! (o2 + k)!):
 *   second derivative  w_k = 2 (-1)^(k+1) r_k / k^2,  w_0 = -2 sum_k 1/k^2
 *   first derivative   w_+k = (-1)^(k+1) r_k / k,     w_0 = 0. */
static void fd_weights(int deriv, int order, std::vector<double> &cf) {
  const int o2 = order / 2;
  cf.assign(o2 + 1, 0.0);
  long double r = 1, c0 = 0;
  for (int k = 1; k <= o2; ++k) {
    r *= (long double)(o2 - k + 1) / (long double)(o2 + k);
    const long double sg = (k % 2) ? 1.0L : -1.0L;
    if (deriv == 2) {
      cf[o2 - k] = (double)(2.0L * sg * r / ((long double)k * k));
      c0 += 1.0L / ((long double)k * k);
    } else {
      cf[o2 - k] = (double)(-sg * r / (long double)k);
    }
  }
  cf[o2] = deriv == 2 ? (double)(-2.0L * c0) : 0.0;
}

/* OGridNablaSq with method="HOFD": Diff::DnDxn (Diff.cpp:203-218) sets the
 * scalar factor to 1 and calls HOFD::Diff over all dimensions
 * (HOFD.h:124-176) with the per-dimension factors -1/(2 m_d)
 * (OGridNablaSq.cpp:47-52), h_d = 1/dx_d^2 * 1 * (-1/(2 m_d)).  The neighbour
 * rules are the reference's, for every point i (flat index, dim 0 fastest),
 * dimension d with stride lo and size N, and lrep = i / N:
 *   above: i + k lo while (i + k lo) / N == lrep;
 *   below: (N + i - k lo) mod N while (N + k lo) / N == lrep + 1;
 *   pbc:   (i + k lo) mod N and (N + i - k lo) mod N for every k.
 * On a one-dimensional grid that is: neighbours above the grid are dropped,
 * those below it wrap around to its top end (or periodic with pbc).  With
 * more dimensions the rule is not a per-dimension Laplacian, and it is
 * reproduced as it stands: every index it forms is inside the grid (pbc is
 * one-dimensional only: the reference's pbc index can leave the grid there). */
static void fd_apply(const System &s, const qdg_hterm &t, const cd *x, cd *o) {
  std::vector<double> cf;
  fd_weights(2, t.fd_order, cf);
  const int o2 = t.fd_order / 2;
  const bool pbc = (t.flags & 1) != 0;
  const double df = 1;  /* even derivative (HOFD.h:130-131) */
  const int nd = s.g.ndims;
  double h[QDG_MAX_DIMS];
  int lo[QDG_MAX_DIMS];
  int stride = 1;
  for (int d = 0; d < nd; ++d) {
    h[d] = 1. / (s.dx[d] * s.dx[d]) * 1.0 * (-1. / 2. / t.mass[d]);
    lo[d] = stride;
    stride *= s.g.n[d];
  }
  const int np = (int)s.npts;
  #pragma omp parallel for schedule(static) if (np >= 8192)
  for (int i = 0; i < np; ++i) {
    cd D = 0;
    for (int d = 0; d < nd; ++d) {
      const int N = s.g.n[d], l = lo[d];
      const int lrep = i / N;
      cd v = cf[o2] * x[i];
      if (pbc) {
        int step = l;
        for (int j = o2 - 1; j >= 0; --j) {
          v += df * cf[j] * x[(i + step) % N];
          v += cf[j] * x[(N + i - step) % N];
          step += l;
        }
      } else {
        int step = i + l;
        for (int j = o2 - 1; j >= 0 && step / N == lrep; --j) {
          v += df * cf[j] * x[step];
          step += l;
        }
        step = i - l;
        for (int j = o2 - 1; j >= 0 && (N + i - step) / N == lrep + 1; --j) {
          v += cf[j] * x[(N + step) % N];
          step -= l;
        }
      }
      D += h[d] * v;
    }
    o[i] += D;
  }
}

/* OGridHOFD::Apply (OGridHOFD.cpp:120-128) with HOFD::Diff along one
 * dimension (HOFD.h:188-211) and _DiffSingleDim (HOFD.h:372-433): along the
 * dimension d (all, or the one of `laser`), point c of a line gets
 * h (cf[o2] x_c + sum_k cf[o2-k] (x_{c-k} + df x_{c+k})), df = -1 for the
 * first derivative and 1 for the second, h = factor / dx_d^deriv; points
 * beyond the line's ends are zero, or wrap around with pbc.  factor =
 * -1/(2 m) of the last dimension's mass when "mass" is given (the loop of
 * OGridHOFD.cpp:80-86 assigns the whole vector each time), else 1. */
static void hofd_apply(const System &s, const qdg_hterm &t, const cd *x, cd *o) {
  const int deriv = (t.flags & 2) ? 1 : 2;
  std::vector<double> cf;
  fd_weights(deriv, t.fd_order, cf);
  const int o2 = t.fd_order / 2;
  const bool pbc = (t.flags & 1) != 0;
  const double df = deriv % 2 ? -1.0 : 1.0;
  const int nd = s.g.ndims;
  const double factor = (t.flags & 4) ? -1. / (2 * t.mass[nd - 1]) : 1.0;
  long lo = 1;
  for (int d = 0; d < nd; ++d) {
    const long N = s.g.n[d];
    if (t.laser < 0 || t.laser == d) {
      const double h = 1. / std::pow(s.dx[d], deriv) * 1.0 * factor;
      for (long i = 0; i < s.npts; ++i) {
        const long c = (i / lo) % N;
        cd v = cf[o2] * x[i];
        for (int k = 1; k <= o2; ++k) {
          cd lw = 0, up = 0;
          if (c - k >= 0) lw = x[i - k * lo];
          else if (pbc) lw = x[i + (N - k) * lo];
          if (c + k < N) up = x[i + k * lo];
          else if (pbc) up = x[i + (k - N) * lo];
          v += cf[o2 - k] * (lw + df * up);
        }
        o[i] += h * v;
      }
    }
    lo *= N;
  }
}

/* Source of G-matrix element (i, j), i >= j: 0 none, 1 grid, 2 constant. */
static int gmat_src(const qdg_hterm &t, int i, int j) {
  if (i < j) std::swap(i, j);
  return (t.flags >> (2 * (i * (i + 1) / 2 + j))) & 3;
}
static const std::vector<double> &gmat_grid(const System &s, const qdg_hterm &t, int i, int j) {
  if (i < j) std::swap(i, j);
  return s.grids[t.grid + i * (i + 1) / 2 + j];
}

/* OGridGMat::Emax (OGridGMat.cpp:250-284): pi^2/2 sum over the lower
 * triangle; a constant off-diagonal element enters without 1/(dx_i dx_j). */
static double gmat_emax(const System &s, const qdg_hterm &t) {
  double T = 0;
  for (int i = 0; i < s.g.ndims; ++i)
    for (int j = 0; j <= i; ++j) {
      const int src = gmat_src(t, i, j);
      if (i != j) {
        double mx = 0, mn = 0;
        if (src == 1) {
          mx = vec_max(gmat_grid(s, t, i, j)) / (s.dx[i] * s.dx[j]);
          mn = vec_min(gmat_grid(s, t, i, j)) / (s.dx[i] * s.dx[j]);
        } else if (src == 2) {
          mx = mn = gmat_grid(s, t, i, j)[0];
        }
        if (mn < 0 && std::fabs(mn) > std::fabs(mx)) T += 2 * std::fabs(mn);
        else T += 2 * mx;
      } else if (src == 1) {
        T += vec_max(gmat_grid(s, t, i, j)) / (s.dx[i] * s.dx[j]);
      } else if (src == 2) {
        T += gmat_grid(s, t, i, j)[0] / (s.dx[i] * s.dx[j]);
      }
    }
  return T * (M_PI * M_PI / 2);
}
/* OGridGMat::Emin (OGridGMat.cpp:286-305): negative off-diagonal minima only. */
static double gmat_emin(const System &s, const qdg_hterm &t) {
  double T = 0;
  for (int i = 0; i < s.g.ndims; ++i)
    for (int j = 0; j < i; ++j) {
      const int src = gmat_src(t, i, j);
      double mn = 0;
      if (src == 1) mn = vec_min(gmat_grid(s, t, i, j)) / (s.dx[i] * s.dx[j]);
      else if (src == 2) mn = gmat_grid(s, t, i, j)[0];
      if (mn < 0) T += mn;
    }
  return T;
}

/* one FFT derivative along d times fac: Diff::DnDxn / DnDxnAdd with method
 * FFT (Diff.cpp:223-272), as the full transform with k_d (the oracle's
 * transform is N-dimensional; k_d depends on the index along d only) */
static void fft_ddx(const System &s, int d, double fac, std::vector<cd> &b) {
  std::vector<double> k;
  kspace_ddx(s, d, 1.0, k);
  const double f = fac / double(s.npts);
  s.fft.exec(b.data(), -1);
  for (long p = 0; p < s.npts; ++p) b[p] = b[p] * (k[p] * cd(0, 1)) * f;
  s.fft.exec(b.data(), +1);
}

/* OGridGMat::ApplyAdd (OGridGMat.cpp:313-386) without chain rule and PML:
 * for every i, w_i = d/dx_i psi; for every j with an element, a grid element
 * adds d/dx_j (G_ij w_i) times -1/2, a constant one d/dx_j w_i times
 * -G_ij / 2. */
static void gmat_apply(const System &s, const qdg_hterm &t, const cd *x, cd *o) {
  const long N = s.npts;
  std::vector<cd> w(N), b(N), acc(N, 0.0);
  for (int i = 0; i < s.g.ndims; ++i) {
    for (long p = 0; p < N; ++p) w[p] = x[p];
    fft_ddx(s, i, 1.0, w);
    for (int j = 0; j < s.g.ndims; ++j) {
      const int src = gmat_src(t, i, j);
      if (src == 0) continue;
      const std::vector<double> &g = gmat_grid(s, t, i, j);
      if (src == 1) {
        for (long p = 0; p < N; ++p) b[p] = w[p] * g[p];
        fft_ddx(s, j, -0.5, b);
      } else {
        for (long p = 0; p < N; ++p) b[p] = w[p];
        fft_ddx(s, j, -0.5 * g[0], b);
      }
      for (long p = 0; p < N; ++p) acc[p] += b[p];
    }
  }
  for (long p = 0; p < N; ++p) o[p] += acc[p];
}

/* H psi: OMultistate::Apply (OMultistate.cpp:206-231) over OSum::Apply/ApplyAdd
 * (OSum.cpp:53-60); kinetic via Diff::DnDxn (Diff.cpp:203-218); potential
 * MultElementsAdd (OGridPotential.cpp:139-142); dipole with -E(step)
 * (OGridDipole.cpp:51-54). */
static void h_apply(const System &s, const cd *in, cd *out, long step) {
  long N = s.npts;
  std::vector<cd> buf(N);
  for (int i = 0; i < s.S; ++i) {
    cd *o = out + i * N;
    #pragma omp parallel for schedule(static) if (N >= 8192)
    for (long p = 0; p < N; ++p) o[p] = 0;
    for (int j = 0; j < s.S; ++j) {
      const cd *x = in + j * N;
      int kt = 0;
      for (size_t ti = 0; ti < s.terms.size(); ++ti) {
        const qdg_hterm &t = s.terms[ti];
        bool kin = t.kind == QDG_TERM_KINETIC;
        if (term_at(s, t, i, j)) {
          /* elementwise codelets are OpenMP loops in the reference (src/math/codelets) */
          if (t.kind == QDG_TERM_NAC) {
            nac_apply(s, t, x, o);
          } else if (t.kind == QDG_TERM_GMAT) {
            gmat_apply(s, t, x, o);
          } else if (t.kind == QDG_TERM_HOFD) {
            hofd_apply(s, t, x, o);
          } else if (kin && t.fd_order > 0) {
            fd_apply(s, t, x, o);
          } else if (kin) {
            cd *b = buf.data();
            #pragma omp parallel for schedule(static) if (N >= 8192)
            for (long p = 0; p < N; ++p) b[p] = x[p];
            s.fft.exec(b, -1);
            const double *tab = s.ktab[kt].data();
            double d = 1.0 / double(N);
            #pragma omp parallel for schedule(static) if (N >= 8192)
            for (long p = 0; p < N; ++p) b[p] = b[p] * tab[p] * d;
            s.fft.exec(b, +1);
            #pragma omp parallel for schedule(static) if (N >= 8192)
            for (long p = 0; p < N; ++p) o[p] += b[p];
          } else if (t.kind == QDG_TERM_POTENTIAL) {
            const double *v = s.grids[t.grid].data();
            #pragma omp parallel for schedule(static) if (N >= 8192)
            for (long p = 0; p < N; ++p) o[p] += x[p] * v[p];
          } else if (t.kind == QDG_TERM_GOBBLER) {
            /* OGobbler::Apply (OGobbler.cpp:187-206): psi * W, or psi * (-i W) as NIP */
            const double *v = s.grids[t.grid].data();
            const cd f = t.laser == 1 ? cd(0, -1) : cd(1, 0);
            #pragma omp parallel for schedule(static) if (N >= 8192)
            for (long p = 0; p < N; ++p) o[p] += x[p] * (f * v[p]);
          } else {
            const double *v = s.grids[t.grid].data();
            double e = (-1) * laser_at(s, t.laser, step);
            #pragma omp parallel for schedule(static) if (N >= 8192)
            for (long p = 0; p < N; ++p) o[p] += x[p] * v[p] * e;
          }
        }
        if (kin) ++kt;
      }
    }
  }
}

/* Compensated (Neumaier) summation for the oracle's reductions.  QDng sums
 * with OpenMP reductions whose order depends on the thread count, so the
 * reference has no fixed summation order; the oracle sums to within one
 * rounding of the exact value instead (a plain serial sum over the 2M points
 * of a 128^3 grid is off by ~1e-12 relative), which makes its norms a
 * reference for any summation order. */
struct CSum {
  double s = 0, c = 0;
  void add(double x) {
    const double t = s + x;
    if (std::fabs(s) >= std::fabs(x)) c += (s - t) + x;
    else c += (x - t) + s;
    s = t;
  }
  double get() const { return s + c; }
};

/* WFGridCartesian::operator* summed over states (WFGridCartesian.cpp:62-117,
 * WFMultistate.cpp:200-222): <a|b> * prod dx. */
static cd dot(const System &s, const cd *a, const cd *b) {
  cd tot = 0;
  for (int st = 0; st < s.S; ++st) {
    CSum re, im;
    for (long p = 0; p < s.npts; ++p) {
      const cd v = std::conj(a[st * s.npts + p]) * b[st * s.npts + p];
      re.add(v.real());
      im.add(v.imag());
    }
    cd c(re.get(), im.get());
    for (int d = 0; d < s.g.ndims; ++d) c *= s.dx[d];
    tot += c;
  }
  return tot;
}
static double norm(const System &s, const cd *a) { return std::sqrt(dot(s, a, a).real()); }

/* ---------------------------------------------------------- propagators */
struct Prop {
  System *sys;
  std::string name;
  std::map<std::string, std::string> params;
  double dt; bool imag, backward;
  cd c0;
  /* Cheby */
  int order = 0; double scaling = 1, prec = 1e-10; cd offset = 0; cd cexp_ = 0;
  std::vector<double> coeff;
  std::vector<cd> k0, k1, k2, buf;
  /* GSPO */
  int ngroups = 0; long laststep = -1; cd lastexp = 0;
  std::vector<std::vector<cd>> expt;
  /* SIL / Arnoldi */
  int kord = 20; double err = 1e-12, conv = 1e-12; int aorder = 0;
  std::vector<std::vector<cd>> lzb;
  int last_terms = 0;
};

static bool has(const Prop &p, const char *k) { return p.params.count(k) > 0; }
static double getd(const Prop &p, const char *k) { return atof(p.params.at(k).c_str()); }

/* OPropagator exponent c0 (OPropagator.h:44-131). */
static cd exponent(double dt, bool imag, bool backward) {
  const cd I(0, 1);
  if (imag) return backward ? cd(-dt) : cd(dt);
  return backward ? I * dt : -I * dt;
}

/* OCheby::Init (OCheby.cpp:358-493). */
static int cheby_init(Prop &p) {
  System &s = *p.sys;
  p.order = has(p, "order") ? atoi(p.params["order"].c_str()) : 0;
  if (has(p, "order") && p.order < 1) return fail(QDG_EINVAL, "Chebychev recursion order invalid");
  cd Emax, Emin; erange(s, Emax, Emin);
  if (has(p, "Emax")) Emax.real(getd(p, "Emax"));
  if (has(p, "Emax_im")) Emax.imag(getd(p, "Emax_im"));
  if (has(p, "Emin")) Emin.real(getd(p, "Emin"));
  if (has(p, "Emin_im")) Emin.imag(getd(p, "Emin_im"));
  if (!p.imag) p.offset = cd((Emax + Emin).real() / 2, (Emax + Emin).imag());
  else p.offset = Emin - std::abs(Emin) * 0.05;
  if (p.offset.imag() != 0 || std::fabs(p.c0.imag()) == 0) p.scaling = std::abs(Emax - Emin) * 1.05;
  else p.scaling = std::abs(Emax - Emin) / 2;
  if (p.order <= 0) p.order = std::abs(int(20 * p.scaling * p.dt));
  if (p.order < 10) p.order = 10;
  if (has(p, "scaling")) p.scaling = getd(p, "scaling");
  if (has(p, "order")) p.order = atoi(p.params["order"].c_str());
  if (p.order < 3) return fail(QDG_EINVAL, "Chebychev recursion must be at least 3");
  std::vector<double> bessel; int zeroes;
  if (std::fabs(p.c0.imag()) != 0 && std::fabs(p.c0.real()) == 0) zeroes = bessel_j(p.order, p.scaling * p.dt, bessel);
  else if (std::fabs(p.c0.imag()) == 0 && std::fabs(p.c0.real()) != 0) zeroes = bessel_i_scaled(p.order, p.scaling * p.dt, bessel);
  else return fail(QDG_EINVAL, "Chebychev propagator doesn't support mixed real/complex exponents");
  p.order -= zeroes;
  if (!has(p, "order")) {
    double precission = 1e-32;   /* BESSEL_DELTA, OCheby.h:10 */
    int i = 2;
    while (i < p.order && std::fabs(bessel[i - 1] - bessel[i - 2]) > precission) i++;
    p.order = i;
  }
  if (p.order > 0 && !p.imag && p.order <= int(p.scaling * p.dt))
    return fail(QDG_EINVAL, "Chebychev recursion order is to small");
  p.coeff.assign(p.order, 0);
  p.coeff[0] = bessel[0];
  for (int i = 1; i < p.order; ++i) p.coeff[i] = 2.0 * bessel[i];
  if (has(p, "prec")) p.prec = getd(p, "prec");
  p.cexp_ = p.c0 / p.dt;
  long n = s.npts * s.S;
  p.k0.assign(n, 0); p.k1.assign(n, 0); p.k2.assign(n, 0); p.buf.assign(n, 0);
  return QDG_OK;
}

static double raw_norm(long n, const cd *x) {  /* OCheby::raw_norm, OCheby.cpp:64-90 */
  CSum nrm;
  for (long j = 0; j < n; ++j) nrm.add((std::conj(x[j]) * x[j]).real());
  return nrm.get();
}

/* OCheby::real_time_step / imag_time_step (OCheby.cpp:92-297). */
static int cheby_step(Prop &p, cd *psi, long step) {
  System &s = *p.sys;
  long n = s.npts * s.S;
  double norm0 = raw_norm(n, psi);
  double norm_last = 0;
  cd ex = p.c0 / p.dt;
  cd *k0 = p.k0.data(), *k1 = p.k1.data(), *k2 = p.k2.data(), *bf = p.buf.data();
  std::copy(psi, psi + n, k0);
  h_apply(s, psi, k1, step);
  for (long j = 0; j < n; ++j) k1[j] += psi[j] * (-1.0 * p.offset);   /* AddElements */
  cd f = ex / p.scaling;
  for (long j = 0; j < n; ++j) k1[j] *= f;
  cd ph = std::exp(p.c0 * p.offset);
  cd c0 = p.coeff[0] * ph, c1 = p.coeff[1] * ph;
  for (long j = 0; j < n; ++j) psi[j] *= c0;
  for (long j = 0; j < n; ++j) bf[j] = k1[j] * c1;
  for (long j = 0; j < n; ++j) psi[j] += bf[j];
  cd exp2 = 2.0 * ex;
  int used = 2;
  for (int i = 2; i < p.order; ++i) {
    CSum acc;
    cd coeff = p.coeff[i] * ph;
    h_apply(s, k1, bf, step);
    for (long j = 0; j < n; ++j) {
      bf[j] = (bf[j] - p.offset * k1[j]) / p.scaling;
      bf[j] *= exp2;
      k2[j] = p.imag ? bf[j] - k0[j] : bf[j] + k0[j];
      k0[j] = k2[j];
      psi[j] += k2[j] * coeff;
      acc.add((std::conj(psi[j]) * psi[j]).real());
    }
    const double accnorm = acc.get();
    used = i + 1;
    if (!p.imag) {
      double nconv = std::fabs(norm0 - accnorm) / norm0;
      if (nconv < p.prec && p.offset.imag() == 0) break;
    } else {
      if (std::fabs(accnorm - norm_last) / norm_last < p.prec) break;
      norm_last = accnorm;
    }
    std::swap(k1, k0);
  }
  /* keep buffer identity stable between steps */
  p.last_terms = used;
  return QDG_OK;
}

/* GSPO groups: OGSPO::Init/InitExp/Apply (OGSPO.cpp:30-52,61-143) with
 * ODMultistate/TransformMSD per-point diagonalisation (ODMultistate.cpp:115-182,
 * TransformMSD.cpp:31-100) and FFT-transform normalisation (OGSPO.cpp:38-41). */
struct GroupInfo { bool kinetic = false, timedep = false, offdiag = false; };

static GroupInfo group_info(const System &s, int g) {
  GroupInfo gi;
  for (auto &t : s.terms) if (t.group == g) {
    if (t.kind == QDG_TERM_KINETIC) gi.kinetic = true;
    if (t.kind == QDG_TERM_DIPOLE) gi.timedep = true;
    if (t.row != t.col) gi.offdiag = true;
  }
  return gi;
}

static int gspo_init(Prop &p) {
  System &s = *p.sys;
  int ng = 0;
  for (auto &t : s.terms) ng = std::max(ng, t.group + 1);
  p.ngroups = ng;
  if (ng < 1) return fail(QDG_EINVAL, "GSPO is empty!");
  for (int g = 0; g < ng; ++g) {
    bool any = false, kin = false, pot = false;
    for (auto &t : s.terms) if (t.group == g) { any = true; if (t.kind == QDG_TERM_KINETIC) kin = true; else pot = true; }
    if (!any) return fail(QDG_EINVAL, "GSPO misses an operator. Sequence must be A, B, C, ...");
    /* OGridGMat is no ODSpace; OGridNablaSq with method HOFD has no k-space table (Diff.cpp:52-54) */
    for (auto &t : s.terms)
      if (t.group == g && (t.kind == QDG_TERM_GMAT || t.kind == QDG_TERM_HOFD ||
                           (t.kind == QDG_TERM_KINETIC && t.fd_order > 0)))
        return fail(QDG_EUNSUPPORTED, "GSPO members need a diagonal representation (no HOFD, no GridGMat)");
    if (kin && pot) return fail(QDG_EUNSUPPORTED, "GSPO: Operator has no diagonal representation");
    if (kin) for (int st = 0; st < s.S; ++st) {
      int c = 0; for (auto &t : s.terms) if (t.group == g && t.kind == QDG_TERM_KINETIC && t.row == st) ++c;
      if (c != 1) return fail(QDG_EUNSUPPORTED, "GSPO kinetic member needs one GridNablaSq per state");
    }
  }
  p.expt.assign(ng, std::vector<cd>(s.npts * s.S * (s.S > 1 ? s.S : 1)));
  p.laststep = -1;
  return QDG_OK;
}

/* per-point potential matrix of group g at point q */
static void point_matrix(const System &s, int g, long q, long step, std::vector<long double> &m) {
  int S = s.S;
  m.assign(S * S, 0);
  for (auto &t : s.terms) if (t.group == g && t.kind != QDG_TERM_KINETIC) {
    double v = s.grids[t.grid][q];
    if (t.kind == QDG_TERM_DIPOLE) v = v * ((-1) * laser_at(s, t.laser, step));
    m[t.row * S + t.col] += v;
    if (t.row != t.col) m[t.col * S + t.row] += v;
  }
}

static void gspo_initexp(Prop &p, long step) {
  System &s = *p.sys;
  long N = s.npts; int S = s.S;
  double sf = 1;
  for (int g = 0; g < p.ngroups; ++g) {
    GroupInfo gi = group_info(s, g);
    if ((gi.timedep && p.laststep != step) || p.laststep == -1 || p.lastexp != p.c0) {
      cd c = p.c0 * sf;
      std::vector<cd> &E = p.expt[g];
      if (gi.kinetic) {
        int kt = 0;
        for (auto &t : s.terms) {
          if (t.kind != QDG_TERM_KINETIC) continue;
          if (t.group == g) {
            const std::vector<double> &tab = s.ktab[kt];
            for (long q = 0; q < N; ++q) E[t.row * N + q] = std::exp(c * tab[q]) * (1.0 / double(N));
          }
          ++kt;
        }
      } else if (!gi.offdiag) {
        std::vector<long double> m;
        for (long q = 0; q < N; ++q) {
          point_matrix(s, g, q, step, m);
          for (int st = 0; st < S; ++st) E[st * N + q] = std::exp(c * (double)m[st * S + st]);
        }
      } else {
        /* store the full per-point propagator matrix X diag(e^{c lambda}) X^T */
        std::vector<long double> m, w, z;
        for (long q = 0; q < N; ++q) {
          point_matrix(s, g, q, step, m);
          jacobi_eig(S, m, w, z);
          for (int a = 0; a < S; ++a) for (int b = 0; b < S; ++b) {
            cd acc = 0;
            for (int k = 0; k < S; ++k) acc += (double)(z[a * S + k] * z[b * S + k]) * std::exp(c * (double)w[k]);
            E[(a * S + b) * N + q] = acc;
          }
        }
      }
    }
    sf = 0.5;
  }
  p.lastexp = p.c0;
  p.laststep = step;
}

static void gspo_apply_group(Prop &p, int g, cd *psi) {
  System &s = *p.sys;
  long N = s.npts; int S = s.S;
  GroupInfo gi = group_info(s, g);
  std::vector<cd> &E = p.expt[g];
  if (gi.kinetic) {
    for (int st = 0; st < S; ++st) {
      s.fft.exec(psi + st * N, -1);
      for (long q = 0; q < N; ++q) psi[st * N + q] *= E[st * N + q];
      s.fft.exec(psi + st * N, +1);
    }
  } else if (!gi.offdiag) {
    for (long q = 0; q < N * S; ++q) psi[q] *= E[q];
  } else {
    std::vector<cd> v(S);
    for (long q = 0; q < N; ++q) {
      for (int a = 0; a < S; ++a) { cd acc = 0; for (int b = 0; b < S; ++b) acc += E[(a * S + b) * N + q] * psi[b * N + q]; v[a] = acc; }
      for (int a = 0; a < S; ++a) psi[a * N + q] = v[a];
    }
  }
}

static int gspo_step(Prop &p, cd *psi, long step) {
  gspo_initexp(p, step);
  for (int i = p.ngroups - 1; i > 0; --i) gspo_apply_group(p, i, psi);
  for (int i = 0; i < p.ngroups; ++i) gspo_apply_group(p, i, psi);
  p.last_terms = 2 * p.ngroups - 1;
  return QDG_OK;
}

/* OSIL::BuildLZB / DiagLZB (OSIL.cpp:83-185). */
static int sil_step(Prop &p, cd *psi, long step) {
  System &s = *p.sys;
  long n = s.npts * s.S;
  int order = p.kord;
  std::vector<double> alpha(order, 0), beta(order, 0);
  p.lzb.assign(order, std::vector<cd>(n));
  std::vector<cd> buf0(n);
  double psinorm = norm(s, psi);
  std::copy(psi, psi + n, p.lzb[0].begin());
  h_apply(s, p.lzb[0].data(), buf0.data(), step);
  alpha[0] = dot(s, p.lzb[0].data(), buf0.data()).real();
  for (long j = 0; j < n; ++j) p.lzb[1][j] = buf0[j] - p.lzb[0][j] * alpha[0];
  beta[0] = norm(s, p.lzb[1].data());
  for (long j = 0; j < n; ++j) p.lzb[1][j] *= 1 / beta[0];
  int convorder = 2, it;
  for (it = 2; it < order; ++it) {
    double err = std::pow(p.dt, it - 2) * beta[0];
    for (int i = 1; i < it - 2; ++i) err *= beta[i] / double(i);
    err = std::fabs(err);
    convorder++;
    h_apply(s, p.lzb[it - 1].data(), p.lzb[it].data(), step);
    alpha[it - 1] = dot(s, p.lzb[it - 1].data(), p.lzb[it].data()).real();
    for (long j = 0; j < n; ++j) p.lzb[it][j] -= p.lzb[it - 1][j] * alpha[it - 1];
    for (long j = 0; j < n; ++j) p.lzb[it][j] -= p.lzb[it - 2][j] * beta[it - 2];
    beta[it - 1] = norm(s, p.lzb[it].data());
    for (long j = 0; j < n; ++j) p.lzb[it][j] *= 1 / beta[it - 1];
    if (err < p.err * psinorm) break;
  }
  {
    h_apply(s, p.lzb[it - 1].data(), buf0.data(), step);
    alpha[it - 1] = dot(s, p.lzb[it - 1].data(), buf0.data()).real();
  }
  /* dstev on the full order x order tridiagonal matrix */
  std::vector<long double> T(order * order, 0), w, z;
  for (int i = 0; i < order; ++i) T[i * order + i] = alpha[i];
  for (int i = 0; i + 1 < order; ++i) { T[i * order + i + 1] = beta[i]; T[(i + 1) * order + i] = beta[i]; }
  jacobi_eig(order, T, w, z);
  std::vector<cd> vect(order);
  for (int i = 0; i < order; ++i) {
    cd acc = 0;
    for (int k = 0; k < order; ++k) acc += (double)(z[i * order + k] * z[0 * order + k]) * std::exp(p.c0 * (double)w[k]);
    vect[i] = acc;
  }
  for (long j = 0; j < n; ++j) psi[j] *= vect[0];
  for (int i = 1; i < convorder; ++i) for (long j = 0; j < n; ++j) psi[j] += p.lzb[i][j] * vect[i];
  p.last_terms = convorder;
  return QDG_OK;
}

/* OArnoldi::BuildLZB / DiagLZB / Propagate (OArnoldi.cpp:86-199). */
/* OArnoldi::BuildLZB (OArnoldi.cpp:86-152): the basis in p.lzb, the
 * Hessenberg matrix HA (order x order) */
static int arnoldi_build(Prop &p, const cd *psi, long step, std::vector<cd> &HA) {
  System &s = *p.sys;
  long n = s.npts * s.S;
  int maxorder = p.kord;
  if (p.aorder == 0) p.aorder = maxorder;
  p.lzb.resize(maxorder);
  for (auto &v : p.lzb) v.resize(n);
  std::vector<cd> tHA(maxorder * maxorder, 0), buf0(n);
  double PsiNorm = norm(s, psi);
  std::copy(psi, psi + n, p.lzb[0].begin());
  for (int it = 1; it < maxorder; ++it) {
    h_apply(s, p.lzb[it - 1].data(), buf0.data(), step);
    for (int j = 0; j <= it - 1; ++j) {
      cd h = dot(s, p.lzb[j].data(), buf0.data());
      tHA[j * maxorder + it - 1] = h;
      for (long q = 0; q < n; ++q) buf0[q] += p.lzb[j][q] * (-1.0 * h);
    }
    double nrm = norm(s, buf0.data());
    if (nrm < 1e-11) break;  /* ARNOLDI_UNDERRUN */
    tHA[it * maxorder + it - 1] = nrm;
    for (long q = 0; q < n; ++q) buf0[q] *= 1. / nrm;
    std::copy(buf0.begin(), buf0.end(), p.lzb[it].begin());
    p.aorder = it + 1;
    cd err = std::pow(p.dt, it - 2) * tHA[1 * maxorder + 0] * PsiNorm;
    for (int i = 1; i < it - 2; ++i) err *= tHA[(i + 1) * maxorder + i] / double(i);
    if (std::abs(err) < p.conv) break;
  }
  int order = p.aorder;
  h_apply(s, p.lzb[order - 1].data(), buf0.data(), step);
  for (int j = 0; j < order; ++j) tHA[j * maxorder + order - 1] = dot(s, p.lzb[j].data(), buf0.data());
  HA.assign(order * order, 0);
  for (int i = 0; i < order; ++i) for (int j = 0; j < order; ++j) HA[i * order + j] = tHA[i * maxorder + j];
  return order;
}

static int arnoldi_step(Prop &p, cd *psi, long step) {
  System &s = *p.sys;
  long n = s.npts * s.S;
  std::vector<cd> HA;
  const int order = arnoldi_build(p, psi, step, HA);
  std::vector<cd> vect = expm_e0(order, HA, p.c0);
  for (long q = 0; q < n; ++q) psi[q] *= vect[0];
  for (int i = 1; i < order; ++i) for (long q = 0; q < n; ++q) psi[q] += p.lzb[i][q] * vect[i];
  p.last_terms = order;
  return QDG_OK;
}

static void parse_params(const char *s, std::map<std::string, std::string> &out) {
  if (!s) return;
  std::string str(s);
  for (char &c : str) if (c == ';' || c == ',' || c == '\t' || c == '\n') c = ' ';
  size_t i = 0;
  while (i < str.size()) {
    while (i < str.size() && str[i] == ' ') ++i;
    size_t j = i; while (j < str.size() && str[j] != ' ') ++j;
    std::string kv = str.substr(i, j - i);
    size_t eq = kv.find('=');
    if (eq != std::string::npos) out[kv.substr(0, eq)] = kv.substr(eq + 1);
    i = j;
  }
}

}  // namespace orc

using namespace orc;

extern "C" {

const char *orc_last_error(void) { return g_err.c_str(); }

int orc_num_threads(int n) {
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
  return omp_get_max_threads();
#else
  (void)n; return 1;
#endif
}

/* Unnormalised 1-D FFT in place on interleaved complex data. */
int orc_fft1(int n, double *data, int sign) {
  FFT1 f; f.init(n);
  std::vector<cd> work(n);
  f.exec(reinterpret_cast<cd *>(data), work.data(), sign);
  return 0;
}

int orc_fftn(const qdg_grid *g, double *data, int sign) {
  FFTN f; f.init(*g);
  f.exec(reinterpret_cast<cd *>(data), sign);
  return 0;
}

void *orc_system_create(const qdg_hplan_desc *d) {
  System *s = new System;
  s->g = d->grid; s->S = d->nstates; s->npts = 1;
  for (int i = 0; i < d->grid.ndims; ++i) {
    s->npts *= d->grid.n[i];
    s->dx[i] = (d->grid.xmax[i] - d->grid.xmin[i]) / double(d->grid.n[i] - 1);
  }
  s->terms.assign(d->terms, d->terms + d->nterms);
  s->hermitian = !d->nonhermitian;
  for (auto &a : s->terms)
    for (auto &b : s->terms)
      if (a.row != a.col && a.row == b.col && a.col == b.row) s->hermitian = false;  /* OMultistate.cpp:52-53 */
  for (int i = 0; i < d->ngrids; ++i) s->grids.emplace_back(d->grid_data + i * s->npts, d->grid_data + (i + 1) * s->npts);
  s->laser_nt = d->laser_nt;
  for (int i = 0; i < d->nlasers; ++i) s->lasers.emplace_back(d->laser_data + (long)i * d->laser_nt, d->laser_data + (long)(i + 1) * d->laser_nt);
  for (auto &t : s->terms) if (t.kind == QDG_TERM_KINETIC) { s->ktab.emplace_back(); kspace_table(*s, t.mass, s->ktab.back()); }
  s->fft.init(s->g);
  return s;
}

void orc_system_destroy(void *s) { delete static_cast<System *>(s); }

int orc_erange(void *sp, double *emax, double *emin) {
  cd a, b; erange(*static_cast<System *>(sp), a, b);
  emax[0] = a.real(); emax[1] = a.imag(); emin[0] = b.real(); emin[1] = b.imag();
  return 0;
}

int orc_h_apply(void *sp, const double *in, double *out, long step) {
  h_apply(*static_cast<System *>(sp), reinterpret_cast<const cd *>(in), reinterpret_cast<cd *>(out), step);
  return 0;
}

/* ---- expectation filters (FiltersList.cpp:289-308), renormalised by
 * <psi|psi> as ProgPropa sets them (ProgPropa.cpp:260,276), computed as the
 * reference applies the operators: N-dimensional FFT, multiplier / N,
 * inverse FFT, scalar product. */
static double raw_dot_re(long n, const cd *a, const cd *b) {
  CSum r;
  for (long j = 0; j < n; ++j) r.add((std::conj(a[j]) * b[j]).real());
  return r.get();
}

/* <psi| O |psi> / <psi|psi> for O = IFFT tab_s FFT / N on state s (tabs: one
 * table for all states, or one per state) */
static double expec_kspace(const System &s, const cd *psi, const std::vector<std::vector<double>> &tabs) {
  long N = s.npts;
  std::vector<cd> b(N);
  double num = 0, den = 0;
  for (int st = 0; st < s.S; ++st) {
    const cd *x = psi + st * N;
    const std::vector<double> &tab = tabs.size() == 1 ? tabs[0] : tabs[st];
    for (long p = 0; p < N; ++p) b[p] = x[p];
    s.fft.exec(b.data(), -1);
    for (long p = 0; p < N; ++p) b[p] *= tab[p] / double(N);
    s.fft.exec(b.data(), +1);
    num += raw_dot_re(N, x, b.data());
    den += raw_dot_re(N, x, x);
  }
  return num / den;
}

/* OGridPosition::_InitDim (OGridPosition.cpp:41-53): (xmin + dx n) scale, summed over dims for dim < 0 */
double orc_expec_position(void *sp, const double *psi_, int dim, double scale) {
  const System &s = *static_cast<System *>(sp);
  const cd *psi = reinterpret_cast<const cd *>(psi_);
  CSum num, den;
  for (int st = 0; st < s.S; ++st)
    for (long p = 0; p < s.npts; ++p) {
      double x = 0;
      long stride = 1;
      for (int d = 0; d < s.g.ndims; ++d) {
        if (dim < 0 || d == dim) x += (s.g.xmin[d] + s.dx[d] * double((p / stride) % s.g.n[d])) * scale;
        stride *= s.g.n[d];
      }
      const double m = std::norm(psi[st * s.npts + p]);
      num.add(x * m);
      den.add(m);
    }
  return num.get() / den.get();
}

/* GridMomentum: OGridNabla(momentum) with Kspace::Init1Dddx (Kspace.cpp:60-96) summed over dims for dim < 0 */
double orc_expec_momentum(void *sp, const double *psi_, int dim, double factor) {
  const System &s = *static_cast<System *>(sp);
  std::vector<double> tab(s.npts, 0.0);
  long stride = 1;
  for (int d = 0; d < s.g.ndims; ++d) {
    const int Nx = s.g.n[d];
    const double dp = 2 * M_PI / (s.g.xmax[d] - s.g.xmin[d] + s.dx[d]);
    std::vector<double> k1(Nx);
    if (Nx % 2 == 0) {
      for (int i = 0; i < Nx / 2; ++i) { k1[i] = double(i) * dp; k1[Nx - i - 1] = -1 * double(i + 1) * dp; }
    } else {
      k1[0] = 0;
      for (int i = 1; i < (Nx + 1) / 2; ++i) { k1[i] = double(i) * dp; k1[Nx - i] = -1 * double(i) * dp; }
    }
    if (dim < 0 || d == dim)
      for (long p = 0; p < s.npts; ++p) tab[p] += factor * k1[(p / stride) % Nx];
    stride *= Nx;
  }
  return expec_kspace(s, reinterpret_cast<const cd *>(psi_), {tab});
}

/* the kinetic terms (OGridNablaSq) of the system, each on its own state */
double orc_expec_kinetic(void *sp, const double *psi_) {
  const System &s = *static_cast<System *>(sp);
  bool direct = false;
  for (auto &t : s.terms)
    if (t.kind == QDG_TERM_GMAT || t.kind == QDG_TERM_HOFD || (t.kind == QDG_TERM_KINETIC && t.fd_order > 0))
      direct = true;
  if (direct) {
    /* finite differences and the G-matrix have no k-space table:
     * <psi|T psi> / <psi|psi> from the operator applied on each state */
    const cd *psi = reinterpret_cast<const cd *>(psi_);
    std::vector<cd> tp(s.npts);
    CSum num, den;
    for (int st = 0; st < s.S; ++st) {
      const cd *x = psi + st * s.npts;
      std::fill(tp.begin(), tp.end(), cd(0));
      for (auto &t : s.terms) {
        if (t.row != st || t.col != st) continue;
        if (t.kind == QDG_TERM_GMAT) gmat_apply(s, t, x, tp.data());
        else if (t.kind == QDG_TERM_HOFD) hofd_apply(s, t, x, tp.data());
        else if (t.kind == QDG_TERM_KINETIC) fd_apply(s, t, x, tp.data());
      }
      for (long p = 0; p < s.npts; ++p) {
        num.add((std::conj(x[p]) * tp[p]).real());
        den.add(std::norm(x[p]));
      }
    }
    return num.get() / den.get();
  }
  std::vector<std::vector<double>> tabs(s.S, std::vector<double>(s.npts, 0.0));
  size_t kt = 0;
  for (auto &t : s.terms)
    if (t.kind == QDG_TERM_KINETIC) {
      for (long p = 0; p < s.npts; ++p) tabs[t.row][p] += s.ktab[kt][p];
      ++kt;
    }
  return expec_kspace(s, reinterpret_cast<const cd *>(psi_), tabs);
}

/* a real diagonal grid on every state (OGridPotential, OGobbler without nip) */
double orc_expec_grid(void *sp, const double *psi_, int grid) {
  const System &s = *static_cast<System *>(sp);
  const cd *psi = reinterpret_cast<const cd *>(psi_);
  const double *v = s.grids[grid].data();
  CSum num, den;
  for (int st = 0; st < s.S; ++st)
    for (long p = 0; p < s.npts; ++p) {
      const double m = std::norm(psi[st * s.npts + p]);
      num.add(v[p] * m);
      den.add(m);
    }
  return num.get() / den.get();
}

/* OProjection::MatrixElement (OProjection.cpp:133-149): sum_k |<phi_k|psi>|^2, scalar products with the volume element */
double orc_expec_projection(void *sp, const double *psi_, const double *funcs, int nfun) {
  const System &s = *static_cast<System *>(sp);
  const cd *psi = reinterpret_cast<const cd *>(psi_);
  const long n = s.npts * s.S;
  double dv = 1;
  for (int d = 0; d < s.g.ndims; ++d) dv *= s.dx[d];
  double acc = 0;
  for (int k = 0; k < nfun; ++k) {
    const cd *f = reinterpret_cast<const cd *>(funcs) + k * n;
    CSum re, im;
    for (long j = 0; j < n; ++j) { const cd c = std::conj(f[j]) * psi[j]; re.add(c.real()); im.add(c.imag()); }
    acc += std::norm(cd(re.get(), im.get()) * dv);
  }
  return acc / (raw_dot_re(n, psi, psi) * dv);
}

/* Reporter::Analyze (Reporter.cpp:99-141): norm^2, pops, <H>, <psi|psi0>. */
int orc_observables(void *sp, const double *psi_, const double *psi0_, long step, double *out) {
  System &s = *static_cast<System *>(sp);
  const cd *psi = reinterpret_cast<const cd *>(psi_);
  long N = s.npts;
  double nrm = norm(s, psi);
  out[0] = nrm * nrm;
  System one = s;  /* per-state norms with the single-state product */
  for (int st = 0; st < s.S; ++st) {
    CSum re;
    for (long p = 0; p < N; ++p) re.add(std::norm(psi[st * N + p]));
    cd c(re.get(), 0.0);
    for (int d = 0; d < s.g.ndims; ++d) c *= s.dx[d];
    double n1 = std::sqrt(c.real());
    out[1 + st] = n1 * n1;
  }
  std::vector<cd> hp(N * s.S);
  h_apply(s, psi, hp.data(), step);
  out[1 + s.S] = dot(s, psi, hp.data()).real();
  cd ac = psi0_ ? dot(s, psi, reinterpret_cast<const cd *>(psi0_)) : cd(0);
  out[2 + s.S] = ac.real(); out[3 + s.S] = ac.imag();
  return 0;
}

void *orc_prop_create(void *sp, const char *name, const char *params, double dt, int imag, int backward) {
  Prop *p = new Prop;
  p->sys = static_cast<System *>(sp);
  p->name = name;
  parse_params(params, p->params);
  p->dt = dt; p->imag = imag != 0; p->backward = backward != 0;
  p->c0 = exponent(dt, p->imag, p->backward);
  int rc;
  if (p->name == "Cheby") rc = cheby_init(*p);
  else if (p->name == "GSPO") rc = gspo_init(*p);
  else if (p->name == "SIL" || p->name == "Arnoldi") {
    p->kord = 20;  /* SIL_DEF_ORDER (OSIL.h:11), ARNOLDI_DEF_ORDER (OArnoldi.h:11) */
    if (has(*p, "order")) p->kord = atoi(p->params["order"].c_str());
    if (p->kord < 3) rc = fail(QDG_EINVAL, "order doesn't make sense");
    else rc = QDG_OK;
    if (has(*p, "err")) p->err = getd(*p, "err");
    if (has(*p, "conv")) p->conv = getd(*p, "conv");
  } else rc = fail(QDG_EINVAL, "unknown propagator " + p->name);
  if (rc != QDG_OK) { delete p; return nullptr; }
  return p;
}

void orc_prop_destroy(void *p) { delete static_cast<Prop *>(p); }

/* order, scaling, offset re/im, exponent re/im */
int orc_prop_info(void *pp, double *out) {
  Prop &p = *static_cast<Prop *>(pp);
  out[0] = p.order; out[1] = p.scaling; out[2] = p.offset.real(); out[3] = p.offset.imag();
  out[4] = p.c0.real(); out[5] = p.c0.imag();
  return 0;
}

int orc_prop_coeffs(void *pp, double *out, int cap) {
  Prop &p = *static_cast<Prop *>(pp);
  int n = std::min<int>(cap, (int)p.coeff.size());
  for (int i = 0; i < n; ++i) out[i] = p.coeff[i];
  return (int)p.coeff.size();
}

int orc_prop_apply(void *pp, double *psi, long step) {
  Prop &p = *static_cast<Prop *>(pp);
  cd *x = reinterpret_cast<cd *>(psi);
  int rc;
  if (p.name == "Cheby") rc = cheby_step(p, x, step);
  else if (p.name == "GSPO") rc = gspo_step(p, x, step);
  else if (p.name == "SIL") rc = sil_step(p, x, step);
  else rc = arnoldi_step(p, x, step);
  return rc == QDG_OK ? p.last_terms : -rc;
}

/* ProgPropa::Run step loop (ProgPropa.cpp:317-327): for i = 1..nsteps,
 * Reporter::Analyze(psi) at clock step start+i-1, then U->Apply(psi).
 * obs receives (3 + S + 1) doubles per step; terms receives terms used. */
int orc_propagate(void *pp, double *psi, const double *psi0, long start, int nsteps,
                  double *obs, int *terms) {
  Prop &p = *static_cast<Prop *>(pp);
  int S = p.sys->S;
  for (int i = 0; i < nsteps; ++i) {
    long step = start + i;
    if (obs) orc_observables(p.sys, psi, psi0, step, obs + (long)i * (4 + S));
    int t = orc_prop_apply(pp, psi, step);
    if (t < 0) return t;
    if (terms) terms[i] = t;
  }
  return 0;
}

/* ProgEigen::ImagTimeEF + DiagBasis (ProgEigen.cpp:318-409, 94-138) with
 * OProjection (OProjection.cpp:133-149). The propagator must be created
 * with imag=1, backward=1 (ProgEigen.cpp:692-693). efs receives nef
 * eigenfunctions, e_raw/e_diag the raw and diagonalised energies,
 * steps the relaxation steps per function. */
/* ProgEigen::AutoCorrEF (ProgEigen.cpp:414-600) with its PeakFinder
 * (src/tools/PeakFinder.cpp) and FunctionGenerator::Hann: propagation kept
 * in memory, autocorrelation <psi_s|psi_0> (a_0 = 1), Hann window, forward
 * FFT, peaks of |spectrum|, time integration at the peak energies,
 * normalisation, <psi|H|psi>. */
static void pf_mean_sigma(const std::vector<double> &d, size_t b, size_t e, double &mean, double &sigma) {
  mean = 0;
  for (size_t i = b; i < e; ++i) mean += d[i];
  mean /= double(e - b);
  sigma = 0;
  for (size_t i = b; i < e; ++i) sigma += (d[i] - mean) * (d[i] - mean);
  sigma = std::sqrt(1. / double(e - b) * sigma);
}
static std::vector<int> pf_find(const std::vector<double> &d, double tol, int width) {
  std::vector<int> pk;
  const size_t n = d.size();
  if (width <= 0) {  /* PeakFinder::Find / _FindData */
    double mean, sigma;
    pf_mean_sigma(d, 0, n, mean, sigma);
    bool start = false;
    double dmax = 0;
    int indmax = -1;
    for (size_t i = 0; i < n; ++i) {
      if (!start && d[i] > mean + tol * sigma) { start = true; dmax = 0; indmax = -1; }
      if (start && d[i] < mean + tol * sigma) { start = false; pk.push_back(indmax); }
      if (start && d[i] > dmax) { dmax = d[i]; indmax = int(i); }
    }
    if (start && indmax != -1 && d[n - 1] < dmax) pk.push_back(indmax);
    return pk;
  }
  /* PeakFinder::Find(data, winsize) over PeakFinder::Maximas */
  double delta = 0;
  std::vector<size_t> maxima;
  for (size_t i = 1; i < n; ++i) {
    if (d[i] < d[i - 1] && delta > 0) maxima.push_back(i - 1);
    delta = d[i] - d[i - 1];
  }
  for (size_t m : maxima) {
    size_t lo = m < size_t(width) ? 0 : m - width;
    size_t hi = m + width > n - 1 ? n - 1 : m + width;
    double mean, sigma;
    pf_mean_sigma(d, lo, hi, mean, sigma);
    if (d[m] > mean + tol * sigma) pk.push_back(int(m));
  }
  return pk;
}

int orc_eigen_ac(void *pp, const double *psi_init, int nsteps, double tol, int width, int win, int max_nef,
                 double *energies, int *nef_out, double *efs, double *spectrum) {
  Prop &p = *static_cast<Prop *>(pp);
  System &s = *p.sys;
  const long n = s.npts * s.S;
  const int M = nsteps;
  std::vector<std::vector<cd>> buf(M, std::vector<cd>(n));
  const cd *init = reinterpret_cast<const cd *>(psi_init);
  std::copy(init, init + n, buf[0].begin());
  std::vector<cd> psi(buf[0]);
  std::vector<cd> ac(M);
  ac[0] = 1;
  for (int i = 1; i < M; ++i) {
    if (orc_prop_apply(pp, reinterpret_cast<double *>(psi.data()), i - 1) < 0) return -1;
    buf[i] = psi;
    ac[i] = dot(s, psi.data(), buf[0].data());
    if (std::isnan(ac[i].real())) { g_err = "Correlation is not a number"; return -QDG_ENONFINITE; }
  }
  if (win)
    for (int i = 0; i < M; ++i) ac[i] *= 0.5 * (1. - std::cos(2 * M_PI * double(i) / double(M - 1)));
  FFT1 f; f.init(M);
  std::vector<cd> work(M), spec(ac);
  f.exec(spec.data(), work.data(), -1);
  std::vector<double> power(M);
  for (int i = 0; i < M; ++i) power[i] = std::abs(spec[i]);
  const std::vector<int> pk = pf_find(power, tol, width);
  *nef_out = int(pk.size());
  if (spectrum) std::copy(spec.begin(), spec.end(), reinterpret_cast<cd *>(spectrum));
  const double dw = 2 * M_PI / (p.dt * double(M));
  std::vector<cd> ef(n), hef(n);
  for (int k = 0; k < std::min(int(pk.size()), max_nef); ++k) {
    const int index = pk[k];
    const double energy = index < M / 2 ? double(index) * dw : double(index - M) * dw;
    ef = buf[0];
    for (int st = 1; st < M; ++st) {
      const cd c(std::cos(energy * double(st) * p.dt), std::sin(energy * double(st) * p.dt));
      for (long j = 0; j < n; ++j) ef[j] += buf[st][j] * c;
    }
    const double nn = norm(s, ef.data());
    for (auto &v : ef) v *= 1 / nn;
    h_apply(s, ef.data(), hef.data(), 0);
    energies[k] = dot(s, ef.data(), hef.data()).real();
    if (efs) std::copy(ef.begin(), ef.end(), reinterpret_cast<cd *>(efs) + (long)k * n);
  }
  return 0;
}

/* ProgEigen::LanczosEF (ProgEigen.cpp:604-648) + DiagBasis (ProgEigen.cpp:94-138):
 * OArnoldi::BuildLZB, the Ritz pairs of the Hessenberg matrix (its symmetric
 * part by Jacobi rotations, standing in for zhseqr/zhsein; eigenvectors
 * scaled to a largest component of modulus 1 as zhsein scales them), the
 * Ritz functions, H in that basis (diagonal: the Ritz values) diagonalised. */
int orc_eigen_lanczos(void *pp, const double *psi_init, int max_nef, double *e_raw, double *e_diag, int *nef_out,
                      double *efs) {
  Prop &p = *static_cast<Prop *>(pp);
  System &s = *p.sys;
  const long n = s.npts * s.S;
  std::vector<cd> HA;
  const int order = arnoldi_build(p, reinterpret_cast<const cd *>(psi_init), 0, HA);
  *nef_out = order;
  std::vector<long double> A(order * order), w, z;
  for (int i = 0; i < order; ++i)
    for (int j = 0; j < order; ++j) A[i * order + j] = 0.5L * ((long double)HA[i * order + j].real() + HA[j * order + i].real());
  jacobi_eig(order, A, w, z);
  std::vector<std::vector<cd>> rf(order, std::vector<cd>(n, 0.0));
  for (int i = 0; i < order; ++i) {
    long double zmax = 0;
    for (int j = 0; j < order; ++j) zmax = std::max(zmax, fabsl(z[j * order + i]));
    for (int j = 0; j < order; ++j) {
      const double c = (double)(z[j * order + i] / zmax);
      for (long q = 0; q < n; ++q) rf[i][q] += p.lzb[j][q] * c;
    }
  }
  std::vector<long double> Sm(order * order, 0), wd, zd;
  std::vector<cd> hb(n);
  for (int i = 0; i < order; ++i) {
    for (int j = 0; j < i; ++j) {
      h_apply(s, rf[j].data(), hb.data(), 0);
      Sm[j * order + i] = Sm[i * order + j] = dot(s, rf[i].data(), hb.data()).real();
    }
    Sm[i * order + i] = w[i];
  }
  jacobi_eig(order, Sm, wd, zd);
  for (int k = 0; k < std::min(order, max_nef); ++k) {
    e_raw[k] = (double)w[k];
    e_diag[k] = (double)wd[k];
    if (efs) {
      cd *out = reinterpret_cast<cd *>(efs) + (long)k * n;
      for (long q = 0; q < n; ++q) out[q] = 0;
      for (int j = 0; j < order; ++j)
        for (long q = 0; q < n; ++q) out[q] += rf[j][q] * (double)zd[j * order + k];
    }
  }
  return 0;
}

int orc_eigen_imag(void *pp, const double *psi_init, int nef, int maxsteps, double convergence,
                   int diag, double *efs, double *e_raw, double *e_diag, int *steps) {
  Prop &p = *static_cast<Prop *>(pp);
  System &s = *p.sys;
  long n = s.npts * s.S;
  std::vector<cd> init(reinterpret_cast<const cd *>(psi_init), reinterpret_cast<const cd *>(psi_init) + n);
  double nn = norm(s, init.data());
  for (auto &x : init) x *= 1 / nn;
  std::vector<std::vector<cd>> P;
  std::vector<cd> psi(n), old(n), hp(n);
  for (int i = 0; i < nef; ++i) {
    psi = init;
    int st = 0; double diff = 1;
    while (st < maxsteps && diff > convergence) {
      old = psi;
      int t = orc_prop_apply(pp, reinterpret_cast<double *>(psi.data()), st);
      if (t < 0) return t;
      if (i > 0) {
        std::vector<cd> buf(n, 0);
        for (auto &w : P) {
          cd c = dot(s, w.data(), psi.data()) * 1.0;
          for (long q = 0; q < n; ++q) buf[q] += w[q] * c;
        }
        for (long q = 0; q < n; ++q) psi[q] -= buf[q];
      }
      double nr = norm(s, psi.data());
      for (auto &x : psi) x *= 1 / nr;
      diff = std::abs(1.0 - dot(s, old.data(), psi.data()));
      ++st;
    }
    P.push_back(psi);
    h_apply(s, psi.data(), hp.data(), 0);
    e_raw[i] = dot(s, psi.data(), hp.data()).real();
    if (steps) steps[i] = st;
  }
  if (diag) {
    std::vector<long double> Sm(nef * nef, 0), w, z;
    for (int i = 0; i < nef; ++i) {
      for (int j = 0; j < i; ++j) {
        h_apply(s, P[j].data(), hp.data(), 0);
        double v = dot(s, P[i].data(), hp.data()).real();
        Sm[j * nef + i] = v; Sm[i * nef + j] = v;
      }
      Sm[i * nef + i] = e_raw[i];
    }
    jacobi_eig(nef, Sm, w, z);
    for (int i = 0; i < nef; ++i) {
      e_diag[i] = (double)w[i];
      if (efs) {
        cd *o = reinterpret_cast<cd *>(efs) + (long)i * n;
        for (long q = 0; q < n; ++q) {
          cd acc = 0;
          for (int j = 0; j < nef; ++j) acc += P[j][q] * (double)z[j * nef + i];
          o[q] = acc;
        }
      }
    }
  } else {
    for (int i = 0; i < nef; ++i) {
      e_diag[i] = e_raw[i];
      if (efs) std::copy(P[i].begin(), P[i].end(), reinterpret_cast<cd *>(efs) + (long)i * n);
    }
  }
  return 0;
}

int orc_bessel(int kind, int n, double x, double *out) {
  std::vector<double> v;
  int z = kind == 0 ? bessel_j(n, x, v) : bessel_i_scaled(n, x, v);
  std::copy(v.begin(), v.end(), out);
  return z;
}

}  // extern "C"
