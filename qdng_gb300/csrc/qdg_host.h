// qdg_host.h -- host-side numerics of the engine (no CUDA).
//
// Small problems that QDng hands to SLATEC and LAPACK and that stay on the
// host here: Bessel coefficients of the Chebyshev expansion, symmetric
// eigenproblems of the Multistate energy range and of the Lanczos matrix,
// and the exponential of the small Arnoldi Hessenberg matrix.
#pragma once

#include <complex>
#include <map>
#include <string>
#include <vector>

namespace qdg {
namespace host {

typedef std::complex<double> cd;

// J_n(x), n = 0..N-1, as SLATEC ZBESJ (kode 1) returns them to
// QDLIB::BesselJ0 (src/linalg/Bessel.cpp:22-58); returns the number of
// trailing components that underflow (ZBESJ's NZ).
int bessel_j(int N, double x, std::vector<double> &out);
// e^{-x} I_n(x), n = 0..N-1 (ZBESI kode 2, src/linalg/Bessel.cpp:61-97).
int bessel_i_scaled(int N, double x, std::vector<double> &out);

// Real symmetric eigenproblem (stands in for LAPACK dsyev/dstev as wrapped
// in src/linalg/LapackDiag.cpp:22-100): a is n x n row-major; eigenvalues
// ascending in w, eigenvectors as columns of z (row-major).
void sym_eig(int n, const std::vector<double> &a, std::vector<double> &w, std::vector<double> &z);

// v = exp(c A) e_0 for a small complex matrix A (row-major), the vector
// OArnoldi::Propagate forms with zhseqr/zhsein/zgetri (OArnoldi.cpp:169-186).
std::vector<cd> expm_e0(int n, const std::vector<cd> &A, cd c);

// Series of OCheby::Init (src/qdlib/OCheby.cpp:358-493) for a Hamiltonian
// with energy range [emin, emax] and exponent c0 (OPropagator::Exponent).
struct ChebySeries {
  int order = 0;
  double scaling = 1.0;
  cd offset = 0.0;
  double prec = 1e-10;          // DEFAULT_PREC (OCheby.h:11)
  std::vector<double> coeff;    // a_0 = J_0 (I_0), a_i = 2 J_i (2 I_i)
};
// Returns an empty string on success, else the reference's error message.
std::string cheby_series(cd emax, cd emin, double dt, cd c0, bool imag,
                         const std::map<std::string, std::string> &params, ChebySeries &out);

// Unnormalised DFT of any length (sign -1 forward, as FFTW_FORWARD): mixed
// radix by decimation in time over the prime factors of n.
std::vector<cd> dft(const std::vector<cd> &x, int sign);

// QDng's PeakFinder (src/tools/PeakFinder.cpp) on a power spectrum: with
// width <= 0 the regions above mean + tol sigma of the whole spectrum and
// the maximum of each; otherwise every local maximum that stands above
// mean + tol sigma of the window [i - width, i + width).  Ascending indices.
std::vector<int> find_peaks(const std::vector<double> &data, double tol, int width);

// Central finite-difference weights of the second derivative on 2 o2 + 1
// points in the layout of QDng's HOFD table (src/qdlib/HOFD.h:31-36):
// cf[o2] weighs the point, cf[o2 - k] both neighbours at distance k.  From
// the closed form w_k = 2 (-1)^(k+1) (o2!)^2 / (k^2 (o2 - k)! (o2 + k)!),
// w_0 = -2 sum_k 1/k^2 (Fornberg, Math. Comp. 51 (1988) 699-706), evaluated
// in long double and rounded once.
void fd_weights2(int order, double *cf);
// The same layout for the first derivative: cf[o2 - k] is the weight of the
// lower neighbour at distance k (the upper one takes -cf), -w_k with
// w_k = (-1)^(k+1) (o2!)^2 / (k (o2 - k)! (o2 + k)!), and cf[o2] = 0.
void fd_weights1(int order, double *cf);

}  // namespace host
}  // namespace qdg
