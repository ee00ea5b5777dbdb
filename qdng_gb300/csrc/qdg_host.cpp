// qdg_host.cpp -- host-side numerics of the engine (see qdg_host.h).
#include "qdg_host.h"

#include <algorithm>
#include <cmath>
#include <cstdlib>

namespace qdg {
namespace host {

// AMOS/SLATEC underflow limit: 1000 * tiny / eps.
static int trailing_underflow(std::vector<double> &out) {
  const double ascle = 1.0e3 * 2.2250738585072014e-308 / 2.220446049250313e-16;
  int nz = 0;
  for (int i = (int)out.size() - 1; i >= 0; --i) {
    if (std::fabs(out[i]) < ascle) { out[i] = 0.0; ++nz; } else break;
  }
  return nz;
}

static int miller_top(int N, double x) {
  const double m = std::max<double>(N, x);
  int s = (int)(m + 40 + 6 * std::sqrt(m));
  return s + (s & 1);
}

// Miller's backward recurrence (Abramowitz & Stegun 9.12 / 9.6.26): start
// far above the wanted orders, recur J_{k-1} = (2k/x) J_k - J_{k+1}, and
// normalise with J_0 + 2 (J_2 + J_4 + ...) = 1 (A&S 9.1.46).  Values are
// rescaled in place when they grow large; the extended exponent range of
// long double keeps the tail of very high orders representable.
int bessel_j(int N, double x, std::vector<double> &out) {
  out.assign(N, 0.0);
  if (N <= 0) return 0;
  if (x == 0.0) { out[0] = 1.0; return trailing_underflow(out); }
  const int top = miller_top(N, x);
  std::vector<long double> v(top + 2, 0.0L);
  v[top] = 1e-20L;
  const long double lim = 1e300L;
  const long double ix = 1.0L / (long double)x;
  for (int k = top; k >= 1; --k) {
    v[k - 1] = (2.0L * k) * ix * v[k] - v[k + 1];
    if (fabsl(v[k - 1]) > lim) {
      for (int j = k - 1; j <= top; ++j) v[j] /= lim;
    }
  }
  long double norm = v[0];
  for (int k = 2; k <= top; k += 2) norm += 2.0L * v[k];
  for (int n = 0; n < N; ++n) out[n] = (double)(v[n] / norm);
  return trailing_underflow(out);
}

// Same recurrence for I_n with a plus sign; e^x = I_0 + 2 sum_{k>=1} I_k (A&S 9.6.37).
int bessel_i_scaled(int N, double x, std::vector<double> &out) {
  out.assign(N, 0.0);
  if (N <= 0) return 0;
  if (x == 0.0) { out[0] = 1.0; return trailing_underflow(out); }
  const int top = miller_top(N, x);
  std::vector<long double> v(top + 2, 0.0L);
  v[top] = 1e-20L;
  const long double lim = 1e300L;
  const long double ix = 1.0L / (long double)x;
  for (int k = top; k >= 1; --k) {
    v[k - 1] = (2.0L * k) * ix * v[k] + v[k + 1];
    if (v[k - 1] > lim) {
      for (int j = k - 1; j <= top; ++j) v[j] /= lim;
    }
  }
  long double norm = v[0];
  for (int k = 1; k <= top; ++k) norm += 2.0L * v[k];
  for (int n = 0; n < N; ++n) out[n] = (double)(v[n] / norm);
  return trailing_underflow(out);
}

// Cyclic Jacobi rotations (Golub & Van Loan, 8.5) in double precision.
void sym_eig(int n, const std::vector<double> &a_in, std::vector<double> &w, std::vector<double> &z) {
  std::vector<double> a = a_in;
  z.assign((size_t)n * n, 0.0);
  for (int i = 0; i < n; ++i) z[(size_t)i * n + i] = 1.0;
  for (int sweep = 0; sweep < 64; ++sweep) {
    double off = 0.0, diag = 0.0;
    for (int p = 0; p < n; ++p) {
      diag += a[(size_t)p * n + p] * a[(size_t)p * n + p];
      for (int q = p + 1; q < n; ++q) off += a[(size_t)p * n + q] * a[(size_t)p * n + q];
    }
    if (off <= 1e-34 * (diag + 1e-300)) break;
    for (int p = 0; p < n; ++p) {
      for (int q = p + 1; q < n; ++q) {
        const double apq = a[(size_t)p * n + q];
        if (apq == 0.0) continue;
        const double theta = (a[(size_t)q * n + q] - a[(size_t)p * n + p]) / (2.0 * apq);
        const double t = (theta >= 0 ? 1.0 : -1.0) / (std::fabs(theta) + std::sqrt(theta * theta + 1.0));
        const double c = 1.0 / std::sqrt(t * t + 1.0), s = t * c;
        for (int k = 0; k < n; ++k) {
          const double akp = a[(size_t)k * n + p], akq = a[(size_t)k * n + q];
          a[(size_t)k * n + p] = c * akp - s * akq;
          a[(size_t)k * n + q] = s * akp + c * akq;
        }
        for (int k = 0; k < n; ++k) {
          const double apk = a[(size_t)p * n + k], aqk = a[(size_t)q * n + k];
          a[(size_t)p * n + k] = c * apk - s * aqk;
          a[(size_t)q * n + k] = s * apk + c * aqk;
        }
        for (int k = 0; k < n; ++k) {
          const double zkp = z[(size_t)k * n + p], zkq = z[(size_t)k * n + q];
          z[(size_t)k * n + p] = c * zkp - s * zkq;
          z[(size_t)k * n + q] = s * zkp + c * zkq;
        }
      }
    }
  }
  std::vector<int> idx(n);
  for (int i = 0; i < n; ++i) idx[i] = i;
  std::sort(idx.begin(), idx.end(), [&](int x, int y) { return a[(size_t)x * n + x] < a[(size_t)y * n + y]; });
  w.resize(n);
  std::vector<double> zs((size_t)n * n);
  for (int j = 0; j < n; ++j) {
    w[j] = a[(size_t)idx[j] * n + idx[j]];
    for (int k = 0; k < n; ++k) zs[(size_t)k * n + j] = z[(size_t)k * n + idx[j]];
  }
  z.swap(zs);
}

// Scaling and squaring with a Taylor polynomial (Moler & Van Loan 2003,
// method 3) applied to the first column only after the squarings.
std::vector<cd> expm_e0(int n, const std::vector<cd> &A, cd c) {
  std::vector<cd> M((size_t)n * n);
  double nrm = 0.0;
  for (int i = 0; i < n; ++i) {
    double row = 0.0;
    for (int j = 0; j < n; ++j) { M[(size_t)i * n + j] = A[(size_t)i * n + j] * c; row += std::abs(M[(size_t)i * n + j]); }
    nrm = std::max(nrm, row);
  }
  int s = 0;
  while (nrm > 0.5) { nrm *= 0.5; ++s; }
  const double sc = std::ldexp(1.0, -s);
  for (auto &x : M) x *= sc;
  std::vector<cd> E((size_t)n * n, 0.0), P((size_t)n * n, 0.0), Q((size_t)n * n);
  for (int i = 0; i < n; ++i) { E[(size_t)i * n + i] = 1.0; P[(size_t)i * n + i] = 1.0; }
  for (int k = 1; k <= 30; ++k) {
    for (int i = 0; i < n; ++i)
      for (int j = 0; j < n; ++j) {
        cd acc = 0.0;
        for (int l = 0; l < n; ++l) acc += P[(size_t)i * n + l] * M[(size_t)l * n + j];
        Q[(size_t)i * n + j] = acc / (double)k;
      }
    P.swap(Q);
    for (size_t i = 0; i < E.size(); ++i) E[i] += P[i];
  }
  for (int r = 0; r < s; ++r) {
    for (int i = 0; i < n; ++i)
      for (int j = 0; j < n; ++j) {
        cd acc = 0.0;
        for (int l = 0; l < n; ++l) acc += E[(size_t)i * n + l] * E[(size_t)l * n + j];
        Q[(size_t)i * n + j] = acc;
      }
    E.swap(Q);
  }
  std::vector<cd> v(n);
  for (int i = 0; i < n; ++i) v[i] = E[(size_t)i * n];
  return v;
}

std::string cheby_series(cd Emax, cd Emin, double dt, cd c0, bool imag,
                         const std::map<std::string, std::string> &params, ChebySeries &out) {
  auto has = [&](const char *k) { return params.count(k) > 0; };
  auto getd = [&](const char *k) { return atof(params.at(k).c_str()); };
  out = ChebySeries();
  int order = 0;
  if (has("order")) {
    order = atoi(params.at("order").c_str());
    if (order < 1) return "Chebychev recursion order invalid";
  }
  if (has("Emax")) Emax.real(getd("Emax"));
  if (has("Emax_im")) Emax.imag(getd("Emax_im"));
  if (has("Emin")) Emin.real(getd("Emin"));
  if (has("Emin_im")) Emin.imag(getd("Emin_im"));
  cd offset;
  double scaling;
  if (!imag) offset = cd((Emax + Emin).real() / 2, (Emax + Emin).imag());
  else offset = Emin - std::abs(Emin) * 0.05;
  if (offset.imag() != 0 || std::fabs(c0.imag()) == 0) scaling = std::abs(Emax - Emin) * 1.05;
  else scaling = std::abs(Emax - Emin) / 2;
  if (order <= 0) order = std::abs(int(20 * scaling * dt));
  if (order < 10) order = 10;
  if (has("scaling")) scaling = getd("scaling");
  if (has("order")) order = atoi(params.at("order").c_str());
  if (order < 3) return "Chebychev recursion must be at least 3";
  std::vector<double> b;
  int zeroes;
  const double R = scaling * dt;
  if (std::fabs(c0.imag()) != 0 && std::fabs(c0.real()) == 0) zeroes = bessel_j(order, R, b);
  else if (std::fabs(c0.imag()) == 0 && std::fabs(c0.real()) != 0) zeroes = bessel_i_scaled(order, R, b);
  else return "Chebychev propagator doesn't support mixed real/complex exponents";
  order -= zeroes;
  if (!has("order")) {
    const double precission = 1e-32;  // BESSEL_DELTA (OCheby.h:10)
    int i = 2;
    while (i < order && std::fabs(b[i - 1] - b[i - 2]) > precission) i++;
    order = i;
  }
  if (order > 0 && !imag && order <= int(scaling * dt)) return "Chebychev recursion order is to small";
  out.order = order;
  out.scaling = scaling;
  out.offset = offset;
  out.coeff.assign(order, 0.0);
  out.coeff[0] = b[0];
  for (int i = 1; i < order; ++i) out.coeff[i] = 2.0 * b[i];
  if (has("prec")) out.prec = getd("prec");
  return std::string();
}

// Recursive decimation in time: n = p m with p the smallest prime factor;
// the p sub-sequences x[j p + r] are transformed (length m) and combined
// with twiddles from long double sin/cos.
static void dft_rec(const cd *x, long stride, long n, int sign, cd *out) {
  if (n == 1) { out[0] = x[0]; return; }
  long p = 2;
  while (n % p) ++p;
  const long m = n / p;
  std::vector<cd> sub((size_t)n);
  for (long r = 0; r < p; ++r) dft_rec(x + r * stride, stride * p, m, sign, sub.data() + r * m);
  const long double pi = 3.141592653589793238462643383279502884L;
  for (long k = 0; k < n; ++k) {
    std::complex<long double> acc = 0;
    for (long r = 0; r < p; ++r) {
      const long double ang = sign * 2.0L * pi * (long double)((r * k) % n) / (long double)n;
      const cd v = sub[(size_t)(r * m + k % m)];
      acc += std::complex<long double>(v.real(), v.imag()) * std::complex<long double>(cosl(ang), sinl(ang));
    }
    out[k] = cd((double)acc.real(), (double)acc.imag());
  }
}

std::vector<cd> dft(const std::vector<cd> &x, int sign) {
  std::vector<cd> out(x.size());
  if (!x.empty()) dft_rec(x.data(), 1, (long)x.size(), sign < 0 ? -1 : 1, out.data());
  return out;
}

static void mean_sigma(const std::vector<double> &d, size_t b, size_t e, double &mean, double &sigma) {
  mean = 0;
  for (size_t i = b; i < e; ++i) mean += d[i];
  mean /= double(e - b);
  sigma = 0;
  for (size_t i = b; i < e; ++i) sigma += (d[i] - mean) * (d[i] - mean);
  sigma = std::sqrt(sigma / double(e - b));
}

void fd_weights2(int order, double *cf) {
  const int o2 = order / 2;
  long double ratio = 1, center = 0;  // ratio = (o2!)^2 / ((o2 - k)! (o2 + k)!)
  for (int k = 1; k <= o2; ++k) {
    ratio = ratio * (long double)(o2 + 1 - k) / (long double)(o2 + k);
    const long double kk = (long double)k * (long double)k;
    cf[o2 - k] = (double)((k & 1 ? 2.0L : -2.0L) * ratio / kk);
    center += 1.0L / kk;
  }
  cf[o2] = (double)(-2.0L * center);
}

void fd_weights1(int order, double *cf) {
  const int o2 = order / 2;
  long double ratio = 1;
  for (int k = 1; k <= o2; ++k) {
    ratio = ratio * (long double)(o2 + 1 - k) / (long double)(o2 + k);
    cf[o2 - k] = (double)((k & 1 ? -1.0L : 1.0L) * ratio / (long double)k);
  }
  cf[o2] = 0.0;
}

std::vector<int> find_peaks(const std::vector<double> &data, double tol, int width) {
  std::vector<int> peaks;
  const size_t n = data.size();
  if (n < 2) return peaks;
  if (width <= 0) {
    double mean, sigma;
    mean_sigma(data, 0, n, mean, sigma);
    const double thr = mean + tol * sigma;
    bool open = false;
    double dmax = 0;
    int imax = -1;
    for (size_t i = 0; i < n; ++i) {
      if (!open && data[i] > thr) { open = true; dmax = 0; imax = -1; }
      if (open && data[i] < thr) { open = false; peaks.push_back(imax); }
      if (open && data[i] > dmax) { dmax = data[i]; imax = (int)i; }
    }
    // a region still open at the end counts if the last value is below its maximum
    if (open && imax != -1 && data[n - 1] < dmax) peaks.push_back(imax);
    return peaks;
  }
  double delta = 0;
  for (size_t i = 1; i < n; ++i) {  // local maxima: a rise followed by a fall
    if (data[i] < data[i - 1] && delta > 0) {
      const size_t c = i - 1;
      const size_t lo = c < (size_t)width ? 0 : c - width;
      const size_t hi = c + width > n - 1 ? n - 1 : c + width;
      double mean, sigma;
      mean_sigma(data, lo, hi, mean, sigma);
      if (data[c] > mean + tol * sigma) peaks.push_back((int)c);
    }
    delta = data[i] - data[i - 1];
  }
  return peaks;
}

}  // namespace host
}  // namespace qdg
