// qdg_api.cu -- the C ABI of include/qdg.h.
//
// Host-side orchestration of the engine: plans (device copy of the QDng
// Hamiltonian tree), wave functions, and the four propagators that replace
// OCheby, OGSPO, OSIL and OArnoldi.  All numerics run on the device except
// the small problems of qdg_host.cpp.  No exception leaves this file; every
// entry point returns a qdg_status and leaves a message for qdg_last_error().
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <string>
#include <type_traits>
#include <vector>

#include "../../include/qdg.h"
#include "qdg_host.h"
#include "qdg_kernels.cuh"

using qdg::cplx;
typedef std::complex<double> cd;

namespace {

thread_local std::string g_last_error;

qdg_status fail(qdg_status s, const std::string &msg) {
  g_last_error = msg;
  return s;
}

}  // namespace

void qdg::set_last_error(const std::string &msg) { g_last_error = msg; }

namespace {

#define CK(...)                                                                           \
  do {                                                                                    \
    cudaError_t e_ = (__VA_ARGS__);                                                       \
    if (e_ != cudaSuccess) return fail(QDG_ECUDA, std::string(#__VA_ARGS__) + ": " + cudaGetErrorString(e_)); \
  } while (0)

cplx<double> C(cd z) { cplx<double> c; c.re = z.real(); c.im = z.imag(); return c; }

enum { KIN_FFT = 0, KIN_FD = 1, KIN_GMAT = 2 };

// Per-dimension line geometry and FFT tables.
struct DimInfo {
  int n;
  long long stride;   // prod of n[k], k < d
  qdg::RadixPlan rp;
  void *tw;           // n twiddles (cplx<T>)
  double *kfac;       // [S] dk^2/(2m)/n for H passes
  void *ktab;         // [S][n] kfac[s] * min(i, n-i)^2 in the bulk type
  void *twdf = nullptr;  // DF64 plans: twiddles and k^2 multipliers in double-float
  void *ktdf = nullptr;
  int TW_k, TW_e;     // lines per tile: kinetic-only passes, coupled epilogue pass
};

}  // namespace

struct qdg_plan {
  qdg_grid grid;
  int S = 1;
  int nd = 1;
  long long npts = 1;
  int precision = QDG_PREC_FP64;
  size_t csize = 16;  // bytes per complex of the bulk type
  double dx[QDG_MAX_DIMS], dk[QDG_MAX_DIMS];
  std::vector<qdg_hterm> terms;
  std::vector<double> grids_h, lasers_h;
  int ngrids = 0, nlasers = 0, laser_nt = 0;
  cd emax = 0, emin = 0;
  // OMultistate's hermitian copy of off-diagonal elements (OMultistate.cpp:122-132)
  bool hermitian = true;
  // OGridNAC elements as applied: (row, col) plus the hermitian copy
  struct NacEntry { int row, col, grid; double c; };
  std::vector<NacEntry> nac;
  size_t nac_smem = 0;
  int nac_per_sm = 1;
  int nac_tw[QDG_MAX_DIMS] = {1, 1, 1, 1};
  // Kinetic operators without a k-space table: OGridNablaSq with method
  // HOFD (finite differences) or OGridGMat.  Either replaces the FFT kinetic
  // pass of the graph path; the fused step kernels do not take them.
  int kin_form = 0;                               // KIN_FFT, KIN_FD or KIN_GMAT
  // a line length with a prime factor above 5: direct-DFT stages, graph path only
  bool generic_fft = false;
  int fd_order = 0, fd_pbc = 0;
  int fd_mode = 0, fd_deriv = 2;                  // mode 1: OGridHOFD (per-dimension lines), deriv 1 or 2
  double fd_h[qdg::kMaxStates][4] = {};           // -1/(2 m_d) / dx_d^2 per state, summed over terms
  long long gm_base[qdg::kMaxStates];             // first G grid of each state, -1 = none
  unsigned gm_mask[qdg::kMaxStates] = {};
  int gm_grid = 1;
  // device
  void *d_grids = nullptr;      // bulk type
  void *d_grids_df = nullptr;   // DF64 plans: the grids in double-float
  double *d_lasers = nullptr;
  DimInfo dim[QDG_MAX_DIMS];
  qdg::Couplings cp_h;           // all potential/dipole entries of H
  qdg::Couplings *d_cp = nullptr;
  double *d_coef = nullptr;
  void *d_P = nullptr;           // kinetic partial sums (bulk type)
  void *d_Pd[QDG_MAX_DIMS] = {nullptr, nullptr, nullptr, nullptr};  // T_d phi per dimension
  void *d_Pd2[QDG_MAX_DIMS] = {nullptr, nullptr, nullptr, nullptr}; // second set (step kernel double buffer)
  size_t kin_smem = 0;
  int kin_grid = 1, comb_grid = 1;
  std::map<long long, int> occ_cache;  // (mode, smem) -> resident blocks per SM
  void *d_scratch = nullptr;     // bulk-type wave function (mixed H apply input / output)
  void *d_scratch2 = nullptr;
  double *d_partials = nullptr;
  int max_parts = 0;
  qdg::GridBarrier *d_bar = nullptr;
  qdg::GridBarrier *h_bar = nullptr;  // pinned copy for the timeout check
  double *h_partials = nullptr;  // pinned
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  int sm_count = 1;
  // Wave functions and propagators of this plan still alive.  A plan whose
  // destroy call comes first is freed with its last child (callers such as
  // QDng's Collector release objects in no fixed order).
  int children = 0;
  bool destroy_pending = false;
  // optional per-launch timing of the line passes
  bool profiling = false;
  std::vector<cudaEvent_t> ev_pool;
  std::vector<int> ev_mode;   // mode of launch i (events 2i, 2i+1)
};

struct qdg_wf {
  qdg_plan *plan;
  cplx<double> *d = nullptr;  // S * npts complex128
};

struct qdg_prop {
  qdg_plan *plan;          // the plan the series runs on
  qdg_plan *user = nullptr;  // the caller's plan (wave functions belong to it)
  qdg_plan *twin = nullptr;  // owned FP64 copy of a mixed plan (imaginary-time Chebyshev)
  std::string name;
  int kind = 0;
  std::map<std::string, std::string> params;
  double dt = 0;
  bool imag = false, backward = false;
  cd c0 = 0;
  bool inited = false;
  // Cheby
  int order = 0;
  double scaling = 1, prec = 1e-10;
  cd offset = 0;
  std::vector<double> coeff;
  void *k0 = nullptr, *k1 = nullptr, *k2 = nullptr;  // bulk type
  qdg::ChebyState *d_cs = nullptr;
  qdg::ChebyState *h_cs = nullptr;    // pinned
  // one captured graph of the whole Chebyshev step per (psi buffer, stream)
  cudaGraphExec_t graph = nullptr;
  void *graph_psi = nullptr;
  cudaStream_t graph_stream = nullptr;
  long long graph_launches = 0;     // kernels of the prologue and epilogue
  long long body_launches = 0;      // kernels of one term of the while body
  bool graphs_ok = true;
  bool while_ok = true;             // device-driven term loop (conditional while node)
  bool graph_is_while = false;
  cplx<double> *d_coeffs = nullptr; // coeff[i] exp(c0 offset), i < order
  double *d_a = nullptr;            // real coefficients coeff[i]
  int step_grid = 0;                // persistent step kernel: blocks (0: unavailable)
  size_t step_smem = 0;
  int step_tw1 = 1;
  long long line_start[QDG_MAX_DIMS + 1] = {0, 0, 0, 0, 0};
  int lmax[QDG_MAX_DIMS] = {1, 1, 1, 1};
  long long *d_bstart = nullptr;    // [step_grid + 1] first kinetic line of each block
  long long *d_bstartA = nullptr;   // the same for the lines of dimension 0 (two-phase terms)
  long long *d_bstartB = nullptr;   // ... and for the lines of the other dimensions
  bool two_phase = false;           // grids of 3+ dimensions: phi_i stored once per term
  // persistent step kernel: the kinetic tables and the potential grids
  // multiplied by the series factor f once, -f offset per point as a value
  // and its rounding residual (scaled_setup)
  int scaled = 0, scaled_rt = 0;
  int scaled_ne = 0;                   // entries of the scaled potential matrix
  int cluster = 0;                     // 1-D single line on a cluster: 1 qdg_step_cluster.cu, 2 qdg_step_line64.cu
  int cluster_size = 8;                // blocks of the cluster
  qdg::RadixPlan crp;                  // its M = N/8-point transforms
  double soff_hi = 0, soff_lo = 0;
  void *sk[QDG_MAX_DIMS] = {nullptr, nullptr, nullptr, nullptr};  // [S][N_d] f kfac k^2 (step bulk type)
  void *sgrids = nullptr;              // [S + extra][npts] (step bulk type)
  qdg::Couplings *d_scp = nullptr;     // entries over sgrids; lid = index of the plan entry (coefficient) or -1
  // GSPO
  int ngroups = 0;
  std::vector<int> group_kinetic;     // 1: FFT member, 0: potential member
  std::vector<qdg::Couplings> gcp_h;
  std::vector<qdg::Couplings *> gcp_d;
  std::vector<double *> gcoef_d;
  std::vector<std::vector<void *>> gtab;  // [group][dim] S*n exp tables
  std::vector<int> gdyn;                  // [group] member has a time-dependent (dipole) term
  std::vector<void *> gU;                 // [group] precomputed per-point exp(c M(x)) of static members
  // Krylov
  int kord = 20, aorder = 0;
  double err = 1e-12, conv = 1e-12;
  std::vector<void *> lzb;
  double *d_ks = nullptr;   // Lanczos scalars on the device: alpha, beta, |psi|, order reached
  double *h_ks = nullptr;   // pinned copy read by the host after the step
  int *h_kdone = nullptr;
  int *d_kdone = nullptr;   // [0]: stop the step's remaining kernels, [1]: error estimate reached
  void *kbuf = nullptr;
  void *kwide = nullptr;  // FP64 copy of one basis vector (mixed precision)
};

namespace {

template <typename T> struct Bulk;

long long wf_elems(const qdg_plan *p) { return p->npts * p->S; }

// Plans whose storage type is binary64 (FP64 and DF64 forms); mixed plans
// store FP32.
bool is64(const qdg_plan *p) { return p->precision != QDG_PREC_MIXED; }

double parse_d(const qdg_prop *p, const char *k) { return atof(p->params.at(k).c_str()); }
bool has(const qdg_prop *p, const char *k) { return p->params.count(k) > 0; }

void parse_params(const char *s, std::map<std::string, std::string> &out) {
  if (!s) return;
  std::string str(s);
  for (char &c : str)
    if (c == ';' || c == ',' || c == '\t' || c == '\n') c = ' ';
  size_t i = 0;
  while (i < str.size()) {
    while (i < str.size() && str[i] == ' ') ++i;
    size_t j = i;
    while (j < str.size() && str[j] != ' ') ++j;
    std::string kv = str.substr(i, j - i);
    size_t eq = kv.find('=');
    if (eq != std::string::npos) out[kv.substr(0, eq)] = kv.substr(eq + 1);
    i = j;
  }
}

// ------------------------------------------------------ energy range
// G-matrix element (i, j) of a GMAT term: its source code (0 none, 1 grid,
// 2 constant) and its grid values (lower triangle, row by row).
int gmat_code(const qdg_hterm &t, int i, int j) {
  if (i < j) std::swap(i, j);
  return (t.flags >> (2 * (i * (i + 1) / 2 + j))) & 3;
}
const double *gmat_values(const qdg_plan *p, const qdg_hterm &t, int i, int j) {
  if (i < j) std::swap(i, j);
  return p->grids_h.data() + (long long)(t.grid + i * (i + 1) / 2 + j) * p->npts;
}

// OGridGMat::Emax (OGridGMat.cpp:250-284): pi^2/2 times the diagonal maxima
// over dx_i^2 plus twice the larger of the off-diagonal maximum and |minimum|
// over dx_i dx_j; a constant off-diagonal element enters as it is.
double gmat_emax(const qdg_plan *p, const qdg_hterm &t) {
  const long long n = p->npts;
  double T = 0;
  for (int i = 0; i < p->nd; ++i)
    for (int j = 0; j <= i; ++j) {
      const int c = gmat_code(t, i, j);
      if (c == 0) continue;
      const double *g = gmat_values(p, t, i, j);
      const double hx = p->dx[i] * p->dx[j];
      if (i != j) {
        const double mx = c == 1 ? *std::max_element(g, g + n) / hx : g[0];
        const double mn = c == 1 ? *std::min_element(g, g + n) / hx : g[0];
        T += (mn < 0 && std::fabs(mn) > std::fabs(mx)) ? 2 * std::fabs(mn) : 2 * mx;
      } else {
        T += (c == 1 ? *std::max_element(g, g + n) : g[0]) / hx;
      }
    }
  return T * (M_PI * M_PI / 2);
}
// OGridGMat::Emin (OGridGMat.cpp:286-305): the negative off-diagonal minima.
double gmat_emin(const qdg_plan *p, const qdg_hterm &t) {
  double T = 0;
  for (int i = 0; i < p->nd; ++i)
    for (int j = 0; j < i; ++j) {
      const int c = gmat_code(t, i, j);
      if (c == 0) continue;
      const double *g = gmat_values(p, t, i, j);
      const double mn = c == 1 ? *std::min_element(g, g + p->npts) / (p->dx[i] * p->dx[j]) : g[0];
      if (mn < 0) T += mn;
    }
  return T;
}

// Emax/Emin of one operator (OGridNablaSq.cpp:89-106 for either method,
// OGridPotential.cpp:124-132, OGridDipole.cpp:36-44).
cd term_emax(const qdg_plan *p, const qdg_hterm &t) {
  const long long n = p->npts;
  if (t.kind == QDG_TERM_GMAT) return gmat_emax(p, t);
  if (t.kind == QDG_TERM_HOFD) {  // OGridHOFD::Emax (OGridHOFD.cpp:97-111)
    if (t.flags & 2) return cd(0.0, M_PI / p->dx[0]);
    double T = 0;
    for (int d = 0; d < p->nd; ++d) {
      const double m = (t.flags & 4) ? t.mass[d] : 1.0;
      if (m > 0) T += 1 / (m * p->dx[d] * p->dx[d]);
    }
    return T * (M_PI * M_PI / 2);
  }
  if (t.kind == QDG_TERM_KINETIC) {
    double T = 0;
    for (int d = 0; d < p->nd; ++d)
      if (t.mass[d] > 0) T += 1 / (t.mass[d] * p->dx[d] * p->dx[d]);
    return T * (M_PI * M_PI / 2);
  }
  const double *g = p->grids_h.data() + (long long)t.grid * n;
  if (t.kind == QDG_TERM_NAC) {  // OGridNAC::Emax (OGridNAC.cpp:105-115): dx of dimension 0
    double m = 0;
    for (int d = 0; d < p->nd; ++d) m += *std::max_element(g + d * n, g + (d + 1) * n);
    return m * M_PI / t.mass[0] / p->dx[0];
  }
  if (t.kind == QDG_TERM_GOBBLER) return t.mass[0];  // OGobbler::Emax = gain (OGobbler.cpp:161-164)
  double gm = *std::max_element(g, g + n);
  if (t.kind == QDG_TERM_POTENTIAL) return gm;
  const double *l = p->lasers_h.data() + (long long)t.laser * p->laser_nt;
  return gm * *std::max_element(l, l + p->laser_nt);
}
// OGridNAC::Emin (OGridNAC.cpp:118-128) computes minima but never adds them:
// it returns 0, and so does this.
cd term_emin(const qdg_plan *p, const qdg_hterm &t) {
  // OGobbler::Emin (OGobbler.cpp:166-170): -i gain as a negative imaginary potential, else 0
  if (t.kind == QDG_TERM_GOBBLER) return t.laser == 1 ? cd(0.0, -t.mass[0]) : cd(0.0);
  if (t.kind == QDG_TERM_GMAT) return gmat_emin(p, t);
  if (t.kind == QDG_TERM_HOFD) return (t.flags & 2) ? cd(0.0, -M_PI / p->dx[0]) : cd(0.0);  // OGridHOFD.cpp:113-118
  if (t.kind != QDG_TERM_POTENTIAL) return 0.0;
  const double *g = p->grids_h.data() + (long long)t.grid * p->npts;
  return *std::min_element(g, g + p->npts);
}
bool term_at(const qdg_plan *p, const qdg_hterm &t, int i, int j) {
  return (t.row == i && t.col == j) || (p->hermitian && t.row != t.col && t.row == j && t.col == i);
}

// OSum::Emax/Emin (OSum.cpp:28-51) for one state; OMultistate::Emax/Emin
// (OMultistate.cpp:163-203): extreme eigenvalue of the |E_ij| matrix.
void compute_erange(qdg_plan *p) {
  if (p->S == 1) {
    cd a = 0, b = 0;
    for (auto &t : p->terms) { a += term_emax(p, t); b += term_emin(p, t); }
    p->emax = a; p->emin = b;
    return;
  }
  // dsyev with uplo 'U' on the column-major matrix (LapackDiag.cpp:22-47)
  // reads the elements (i, j), i <= j: the lower ones matter only through
  // the hermitian copy.
  const int S = p->S;
  std::vector<double> mx(S * S, 0.0), mn(S * S, 0.0), w, z;
  for (int i = 0; i < S; ++i)
    for (int j = i; j < S; ++j) {
      cd a = 0, b = 0;
      bool any = false;
      for (auto &t : p->terms)
        if (term_at(p, t, i, j)) { a += term_emax(p, t); b += term_emin(p, t); any = true; }
      if (any) {
        mx[i * S + j] = mx[j * S + i] = std::abs(a);
        mn[i * S + j] = mn[j * S + i] = std::abs(b);
      }
    }
  qdg::host::sym_eig(S, mx, w, z);
  p->emax = w[S - 1];
  qdg::host::sym_eig(S, mn, w, z);
  p->emin = w[0];
}

// ---------------------------------------------------------- geometry
int choose_tw(const qdg_plan *p, int d, int nsub) {
  const DimInfo &di = p->dim[d];
  const long long lines = p->npts / di.n;
  const long long limit = (d == 0) ? lines : di.stride;  // TW must divide this
  const int target_elems = is64(p) ? 2048 : 4096;
  int best = 1;
  for (int tw = 2; tw <= 32; tw *= 2) {
    if (limit % tw) break;
    if ((long long)tw * nsub * di.n > target_elems) break;
    const long long items = (lines / tw) * (p->S / nsub);
    if (items < p->sm_count) break;  // keep every SM busy
    best = tw;
  }
  return best;
}

// Twiddles plus two line-batch buffers of TW * nsub lines (padded layout).
size_t pass_smem(const qdg_plan *p, int d, int TW, int nsub) {
  const int n = p->dim[d].n;
  return ((size_t)n + 2 * qdg::line_buf_elems(n, TW * nsub)) * p->csize;
}

template <typename T>
void fill_geometry(const qdg_plan *p, int d, int nsub, qdg::PassArgs<T> &a) {
  const DimInfo &di = p->dim[d];
  const int TW = nsub == 1 ? di.TW_k : di.TW_e;
  a.N = di.n;
  a.TW = TW;
  a.S = p->S;
  a.nsub = nsub;
  a.npts = p->npts;
  a.rp = di.rp;
  a.tw = reinterpret_cast<const cplx<T> *>(di.tw);
  a.kfac = di.kfac;
  if (d == 0) {
    a.es = 1; a.ls = di.n; a.tiles_per_hi = 1; a.hi_stride = (long long)TW * di.n;
  } else {
    a.es = (int)di.stride; a.ls = 1; a.tiles_per_hi = (int)(di.stride / TW); a.hi_stride = di.stride * di.n;
  }
  a.ntiles = p->npts / ((long long)di.n * TW);
}

template <typename T>
qdg_status prof_begin(qdg_plan *p, int mode, size_t *slot);
qdg_status prof_end(qdg_plan *p, size_t slot);

template <typename T>
qdg_status launch_one(qdg_plan *p, int mode, int d, qdg::PassArgs<T> &a, int *nblocks_out) {
  const int nsub = a.nsub;
  const size_t smem = pass_smem(p, d, a.TW, nsub);
  if (smem > 227 * 1024) return fail(QDG_EUNSUPPORTED, "grid line too long for the shared-memory FFT at this precision/state count");
  const int block = 256;
  const long long key = ((long long)mode << 40) | ((long long)(sizeof(T)) << 32) | (long long)smem;
  auto it = p->occ_cache.find(key);
  int per_sm;
  if (it != p->occ_cache.end()) per_sm = it->second;
  else p->occ_cache[key] = per_sm = qdg::pass_max_blocks<T>(mode, p->S, block, smem);
  const long long items = a.ntiles * (p->S / nsub);
  long long grid = std::min<long long>(items, (long long)per_sm * p->sm_count);
  if (grid > p->max_parts) grid = p->max_parts;
  if (grid < 1) grid = 1;
  if (nblocks_out) *nblocks_out = (int)grid;
  size_t slot = 0;
  qdg_status s = prof_begin<T>(p, mode, &slot);
  if (s != QDG_OK) return s;
  CK(qdg::launch_pass<T>(mode, a, (int)grid, block, smem, p->stream));
  return prof_end(p, slot);
}

// Epilogue arguments of one H application.
struct Epi {
  void *out = nullptr;
  cplx<double> *psi = nullptr;
  void *k0 = nullptr;
  cd offset = 0, fac = 0, fac_lo = 0, c0p = 0, c1p = 0, coeff = 0;
  int imag = 0;
  const int *done = nullptr;
  qdg::ChebyCut cut{};
  const void *bufs[2] = {nullptr, nullptr};  // device-driven term loop (cut.dyn)
};

template <typename T>
qdg_status prof_begin(qdg_plan *p, int mode, size_t *slot) {
  if (!p->profiling) return QDG_OK;
  const size_t i = p->ev_mode.size();
  while (p->ev_pool.size() < 2 * (i + 1)) {
    cudaEvent_t e;
    CK(cudaEventCreate(&e));
    p->ev_pool.push_back(e);
  }
  p->ev_mode.push_back(mode);
  *slot = i;
  CK(cudaEventRecord(p->ev_pool[2 * i], p->stream));
  return QDG_OK;
}
qdg_status prof_end(qdg_plan *p, size_t slot) {
  if (!p->profiling) return QDG_OK;
  CK(cudaEventRecord(p->ev_pool[2 * slot + 1], p->stream));
  return QDG_OK;
}

// One application of H.  One-dimensional grids: a single fused line pass
// (FFT, k^2, inverse FFT, potential matrix and epilogue).  Higher
// dimensions: one launch computing T_d phi for all d, then one point-wise
// launch that sums them, adds the potential matrix and runs the epilogue.
// OGridNAC elements, after the kinetic pass: one launch per element and
// dimension, each adding into T_0 phi of its row state.
template <typename T>
qdg_status run_nac(qdg_plan *p, const cplx<T> *phi, const Epi &e) {
  for (const auto &ne : p->nac) {
    for (int d = 0; d < p->nd; ++d) {
      const DimInfo &di = p->dim[d];
      qdg::NacArgs<T> a;
      memset(&a, 0, sizeof(a));
      const int TW = p->nac_tw[d];
      a.N = di.n;
      a.TW = TW;
      if (d == 0) {
        a.es = 1; a.ls = di.n; a.tiles_per_hi = 1; a.hi_stride = (long long)TW * di.n;
      } else {
        a.es = (int)di.stride; a.ls = 1; a.tiles_per_hi = (int)(di.stride / TW); a.hi_stride = di.stride * di.n;
      }
      a.ntiles = p->npts / ((long long)di.n * TW);
      a.npts = p->npts;
      a.rp = di.rp;
      a.tw = reinterpret_cast<const cplx<T> *>(di.tw);
      a.kfac = p->dk[d] * ne.c / (double)di.n;
      a.phi = phi;
      a.col = ne.col;
      a.f = reinterpret_cast<const T *>(p->d_grids) + (long long)(ne.grid + d) * p->npts;
      a.out = reinterpret_cast<cplx<T> *>(p->d_Pd[0]) + (long long)ne.row * p->npts;
      a.done = e.done;
      a.cs = e.cut.cs;
      a.dyn = e.cut.dyn;
      a.bufs[0] = reinterpret_cast<const cplx<T> *>(e.bufs[0]);
      a.bufs[1] = reinterpret_cast<const cplx<T> *>(e.bufs[1]);
      const int grid = (int)std::max<long long>(1, std::min<long long>(a.ntiles, (long long)p->nac_per_sm * p->sm_count));
      CK(qdg::launch_nac<T>(a, grid, 256, p->nac_smem, p->stream));
    }
  }
  return QDG_OK;
}

// The point-wise pass of an H application on grids with more than one
// dimension (or extra line passes): H phi = sum of the nP kinetic partial
// results + the potential matrix, then the series epilogue.
template <typename T>
qdg_status run_combine(qdg_plan *p, int final_mode, const cplx<T> *phi, const Epi &e, int nP) {
  qdg::CombArgs<T> c;
  memset(&c, 0, sizeof(c));
  c.S = p->S;
  c.nd = nP;
  c.npts = p->npts;
  c.phi = phi;
  for (int d = 0; d < nP; ++d) c.P[d] = reinterpret_cast<const cplx<T> *>(p->d_Pd[d]);
  c.out = reinterpret_cast<cplx<T> *>(e.out);
  c.psi = e.psi;
  c.k0 = reinterpret_cast<cplx<T> *>(e.k0);
  c.cp = p->d_cp;
  c.coef = p->d_coef;
  c.grids = reinterpret_cast<const T *>(p->d_grids);
  c.offset = C(e.offset); c.fac = C(e.fac); c.fac_lo = C(e.fac_lo); c.c0p = C(e.c0p); c.c1p = C(e.c1p); c.coeff = C(e.coeff);
  c.imag = e.imag;
  c.partials = p->d_partials;
  c.cut = e.cut;
  c.bufs[0] = reinterpret_cast<const cplx<T> *>(e.bufs[0]);
  c.bufs[1] = reinterpret_cast<const cplx<T> *>(e.bufs[1]);
  size_t slot = 0;
  qdg_status s = prof_begin<T>(p, final_mode, &slot);
  if (s != QDG_OK) return s;
  CK(qdg::launch_combine<T>(final_mode, c, p->comb_grid, 256, p->stream));
  return prof_end(p, slot);
}

// The kinetic pass of a plan whose kinetic operator has no k-space table:
// finite differences into P[0] (one launch), or the G-matrix line passes
// (D_i = d/dx_i phi, then P_j).  tw: each dimension's twiddles in type T;
// with tw_lines > 0 the line tiles hold at most that many lines (the
// binary64 expectation value on a mixed plan, whose tiles were sized for FP32).
template <typename T>
qdg_status run_kin_tablefree(qdg_plan *p, const cplx<T> *phi, const int *done, const qdg::ChebyState *cs, int dyn,
                             const void *const *bufs, const cplx<T> *const *tw, const T *grids, cplx<T> *const *D,
                             cplx<T> *const *P, int tw_lines) {
  if (p->kin_form == KIN_FD) {
    qdg::FdArgs<T> a;
    memset(&a, 0, sizeof(a));
    a.nd = p->nd; a.S = p->S; a.o2 = p->fd_order / 2; a.pbc = p->fd_pbc; a.npts = p->npts;
    a.mode = p->fd_mode;
    a.df = p->fd_deriv == 1 ? -1.0 : 1.0;
    for (int d = 0; d < p->nd; ++d) { a.n[d] = p->dim[d].n; a.lo[d] = p->dim[d].stride; }
    if (p->fd_deriv == 1) qdg::host::fd_weights1(p->fd_order, a.cf);
    else qdg::host::fd_weights2(p->fd_order, a.cf);
    memcpy(a.h, p->fd_h, sizeof(a.h));
    a.phi = phi; a.out = P[0]; a.done = done; a.cs = cs; a.dyn = dyn;
    a.bufs[0] = static_cast<const cplx<T> *>(bufs[0]);
    a.bufs[1] = static_cast<const cplx<T> *>(bufs[1]);
    const long long blocks = (p->npts * p->S + 255) / 256;
    CK(qdg::launch_fd_kinetic<T>(a, (int)std::max<long long>(1, std::min<long long>(blocks, 8LL * p->sm_count)), p->stream));
    return QDG_OK;
  }
  qdg::GmatArgs<T> a;
  memset(&a, 0, sizeof(a));
  a.nd = p->nd; a.S = p->S; a.npts = p->npts;
  long long items = 0;
  size_t smem = 0;
  for (int d = 0; d < p->nd; ++d) {
    const DimInfo &di = p->dim[d];
    int TW = di.TW_k;
    if (tw_lines > 0) TW = std::min(TW, tw_lines);
    qdg::DimPass<T> &g = a.dp[d];
    g.N = di.n; g.TW = TW; g.rp = di.rp; g.tw = tw[d];
    if (d == 0) { g.es = 1; g.ls = di.n; g.tiles_per_hi = 1; g.hi_stride = (long long)TW * di.n; }
    else { g.es = (int)di.stride; g.ls = 1; g.tiles_per_hi = (int)(di.stride / TW); g.hi_stride = di.stride * di.n; }
    g.ntiles = p->npts / ((long long)di.n * TW);
    a.item_start[d] = items;
    items += g.ntiles * p->S;
    a.kmul[d] = p->dk[d] / (double)di.n;  // Diff::DnDxn factor 1 (Diff.cpp:229-232)
    smem = std::max(smem, ((size_t)di.n + 2 * qdg::line_buf_elems(di.n, TW)) * sizeof(cplx<T>));
    a.D[d] = D[d];
    a.P[d] = P[d];
  }
  a.item_start[p->nd] = items;
  if (smem > 227 * 1024) return fail(QDG_EUNSUPPORTED, "grid line too long for the shared-memory FFT");
  for (int st = 0; st < qdg::kMaxStates; ++st) { a.gbase[st] = p->gm_base[st]; a.gmask[st] = p->gm_mask[st]; }
  a.grids = grids;
  a.phi = phi; a.done = done; a.cs = cs; a.dyn = dyn;
  a.bufs[0] = static_cast<const cplx<T> *>(bufs[0]);
  a.bufs[1] = static_cast<const cplx<T> *>(bufs[1]);
  const int grid = (int)std::max<long long>(1, std::min<long long>(items, (long long)qdg::gmat_max_blocks<T>(256, smem) * p->sm_count));
  a.pass = 0;
  CK(qdg::launch_gmat_pass<T>(a, grid, 256, smem, p->stream));
  a.pass = 1;
  for (int d = 0; d < p->nd; ++d) a.kmul[d] = -0.5 * p->dk[d] / (double)p->dim[d].n;  // DnDxnAdd factor -1/2
  CK(qdg::launch_gmat_pass<T>(a, grid, 256, smem, p->stream));
  return QDG_OK;
}

// Binary64 plans of at most 2^17 points (all states) whose lines are powers
// of two up to 1024 take the latency-oriented radix-2 kinetic pass (the
// Krylov, observable and eigen H applications on such grids are a chain of
// small launches, each bound by the length of its FP64 instruction chains).
template <typename T>
bool kin_r2_ok(const qdg_plan *p) {
  if (sizeof(T) != sizeof(double) || p->npts * p->S > (1LL << 17)) return false;
  for (int d = 0; d < p->nd; ++d) {
    const int N = p->dim[d].n;
    if (N < 2 || N > 1024 || (N & (N - 1))) return false;
  }
  return true;
}
cudaError_t launch_kin_r2_plan(qdg_plan *p, const cplx<double> *phi, const Epi &e) {
  qdg::KinR2Args r;
  memset(&r, 0, sizeof(r));
  r.nd = p->nd;
  r.S = p->S;
  r.npts = p->npts;
  // N/2 threads per line; short lines share a block up to 64 threads
  int maxN = 2;
  for (int d = 0; d < p->nd; ++d) maxN = std::max(maxN, p->dim[d].n);
  r.threads = std::max(64, maxN / 2);
  long long items = 0;
  for (int d = 0; d < p->nd; ++d) {
    const int N = p->dim[d].n;
    int lg = 0;
    while ((1 << lg) < N) ++lg;
    const long long lines = p->npts / N;
    const int L = (int)std::min<long long>(std::max(1, r.threads / (N / 2)), lines);
    r.N[d] = N;
    r.lgN[d] = lg;
    r.L[d] = L;
    r.stride[d] = p->dim[d].stride;
    r.groups[d] = lines / L;
    r.item_start[d] = items;
    items += r.groups[d] * p->S;
    r.kfac[d] = p->dim[d].kfac;
    r.tw[d] = reinterpret_cast<const cplx<double> *>(p->dim[d].tw);
    r.P[d] = reinterpret_cast<cplx<double> *>(p->d_Pd[d]);
  }
  r.item_start[p->nd] = items;
  r.phi = phi;
  r.done = e.done;
  r.cs = e.cut.cs;
  r.dyn = e.cut.dyn;
  r.bufs[0] = reinterpret_cast<const cplx<double> *>(e.bufs[0]);
  r.bufs[1] = reinterpret_cast<const cplx<double> *>(e.bufs[1]);
  return qdg::launch_kin_r2(r, p->stream);
}

template <typename T>
qdg_status run_h(qdg_plan *p, int final_mode, const cplx<T> *phi, const Epi &e) {
  if (p->kin_form != KIN_FFT) {
    size_t slot = 0;
    qdg_status s = prof_begin<T>(p, qdg::PM_KIN_FIRST, &slot);
    if (s != QDG_OK) return s;
    const cplx<T> *tw[QDG_MAX_DIMS] = {};
    cplx<T> *D[QDG_MAX_DIMS] = {}, *P[QDG_MAX_DIMS] = {};
    for (int d = 0; d < p->nd; ++d) {
      tw[d] = reinterpret_cast<const cplx<T> *>(p->dim[d].tw);
      D[d] = reinterpret_cast<cplx<T> *>(p->d_Pd2[d]);
      P[d] = reinterpret_cast<cplx<T> *>(p->d_Pd[d]);
    }
    if ((s = run_kin_tablefree<T>(p, phi, e.done, e.cut.cs, e.cut.dyn, e.bufs, tw,
                                  reinterpret_cast<const T *>(p->d_grids), D, P, 0)) != QDG_OK)
      return s;
    if ((s = prof_end(p, slot)) != QDG_OK) return s;
    if (!p->nac.empty() && (s = run_nac<T>(p, phi, e)) != QDG_OK) return s;
    return run_combine<T>(p, final_mode, phi, e, p->kin_form == KIN_FD ? 1 : p->nd);
  }
  if (p->nd == 1 && p->nac.empty()) {
    qdg::PassArgs<T> a;
    memset(&a, 0, sizeof(a));
    fill_geometry<T>(p, 0, p->S, a);
    a.phi = phi;
    a.out = reinterpret_cast<cplx<T> *>(e.out);
    a.psi = e.psi;
    a.k0 = reinterpret_cast<cplx<T> *>(e.k0);
    a.cp = p->d_cp;
    a.coef = p->d_coef;
    a.grids = reinterpret_cast<const T *>(p->d_grids);
    a.multi_pass = 0;
    a.offset = C(e.offset); a.fac = C(e.fac); a.fac_lo = C(e.fac_lo); a.c0p = C(e.c0p); a.c1p = C(e.c1p); a.coeff = C(e.coeff);
    a.imag = e.imag;
    a.partials = p->d_partials;
    a.done = e.done;
    a.cut = e.cut;
    a.bufs[0] = reinterpret_cast<const cplx<T> *>(e.bufs[0]);
    a.bufs[1] = reinterpret_cast<const cplx<T> *>(e.bufs[1]);
    return launch_one<T>(p, final_mode, 0, a, nullptr);
  }
  qdg::KinArgs<T> k;
  memset(&k, 0, sizeof(k));
  k.nd = p->nd;
  k.S = p->S;
  k.npts = p->npts;
  k.phi = phi;
  k.done = e.done;
  k.cs = e.cut.cs;
  k.dyn = e.cut.dyn;
  k.bufs[0] = reinterpret_cast<const cplx<T> *>(e.bufs[0]);
  k.bufs[1] = reinterpret_cast<const cplx<T> *>(e.bufs[1]);
  long long items = 0;
  for (int d = 0; d < p->nd; ++d) {
    qdg::PassArgs<T> g;
    memset(&g, 0, sizeof(g));
    fill_geometry<T>(p, d, 1, g);
    qdg::DimPass<T> &dp = k.dp[d];
    dp.N = g.N; dp.es = g.es; dp.ls = g.ls; dp.TW = g.TW; dp.tiles_per_hi = g.tiles_per_hi;
    dp.hi_stride = g.hi_stride; dp.ntiles = g.ntiles; dp.rp = g.rp; dp.tw = g.tw; dp.kfac = g.kfac;
    dp.P = reinterpret_cast<cplx<T> *>(p->d_Pd[d]);
    k.item_start[d] = items;
    items += g.ntiles * p->S;
  }
  k.item_start[p->nd] = items;
  size_t slot = 0;
  qdg_status s = prof_begin<T>(p, qdg::PM_KIN_FIRST, &slot);
  if (s != QDG_OK) return s;
  if (kin_r2_ok<T>(p)) {
    CK(launch_kin_r2_plan(p, reinterpret_cast<const cplx<double> *>(phi), e));
  } else {
    CK(qdg::launch_kin_all<T>(k, (int)std::min<long long>(items, p->kin_grid), 256, p->kin_smem, p->stream));
  }
  if ((s = prof_end(p, slot)) != QDG_OK) return s;
  if (!p->nac.empty() && (s = run_nac<T>(p, phi, e)) != QDG_OK) return s;

  return run_combine<T>(p, final_mode, phi, e, p->nd);
}

template <typename T>
qdg_status upload_tables(qdg_plan *p) {
  const int S = p->S;
  for (int d = 0; d < p->nd; ++d) {
    DimInfo &di = p->dim[d];
    const int n = di.n;
    std::vector<cplx<T>> tw(n);
    const long double pi = 3.141592653589793238462643383279502884L;
    for (int m = 0; m < n; ++m) {
      const long double ang = -2.0L * pi * (long double)m / (long double)n;
      tw[m].re = (T)cosl(ang);
      tw[m].im = (T)sinl(ang);
    }
    CK(cudaMalloc(&di.tw, sizeof(cplx<T>) * n));
    CK(cudaMemcpy(di.tw, tw.data(), sizeof(cplx<T>) * n, cudaMemcpyHostToDevice));
    // kinetic multipliers per state: sum over the state's GridNablaSq terms
    std::vector<double> kf(S, 0.0);
    for (auto &t : p->terms)
      if (t.kind == QDG_TERM_KINETIC && t.fd_order == 0) kf[t.row] += (p->dk[d] * p->dk[d]) / (2.0 * t.mass[d]) / (double)n;
    CK(cudaMalloc(&di.kfac, sizeof(double) * S));
    CK(cudaMemcpy(di.kfac, kf.data(), sizeof(double) * S, cudaMemcpyHostToDevice));
    std::vector<T> kt((size_t)S * n);
    for (int st = 0; st < S; ++st)
      for (int i = 0; i < n; ++i) {
        const double kq = std::min(i, n - i);
        kt[(size_t)st * n + i] = (T)(kf[st] * kq * kq);
      }
    CK(cudaMalloc(&di.ktab, sizeof(T) * kt.size()));
    CK(cudaMemcpy(di.ktab, kt.data(), sizeof(T) * kt.size(), cudaMemcpyHostToDevice));
    if (p->precision == QDG_PREC_DF64) {
      // double-float copies for the FFTs of the DF64 step kernel
      std::vector<qdg::cplx<qdg::dfl>> twd(n);
      for (int m = 0; m < n; ++m) {
        const long double ang = -2.0L * pi * (long double)m / (long double)n;
        const long double c = cosl(ang), sn = sinl(ang);
        twd[m].re = qdg::dfl((float)c, (float)(c - (long double)(float)c));
        twd[m].im = qdg::dfl((float)sn, (float)(sn - (long double)(float)sn));
      }
      std::vector<qdg::dfl> ktd(kt.size());
      for (size_t i = 0; i < kt.size(); ++i) ktd[i] = qdg::dfl((double)kt[i]);
      CK(cudaMalloc(&di.twdf, sizeof(qdg::cplx<qdg::dfl>) * n));
      CK(cudaMemcpy(di.twdf, twd.data(), sizeof(qdg::cplx<qdg::dfl>) * n, cudaMemcpyHostToDevice));
      CK(cudaMalloc(&di.ktdf, sizeof(qdg::dfl) * ktd.size()));
      CK(cudaMemcpy(di.ktdf, ktd.data(), sizeof(qdg::dfl) * ktd.size(), cudaMemcpyHostToDevice));
    }
  }
  // grids in the bulk type
  std::vector<T> g(p->grids_h.size());
  for (size_t i = 0; i < g.size(); ++i) g[i] = (T)p->grids_h[i];
  CK(cudaMalloc(&p->d_grids, sizeof(T) * std::max<size_t>(1, g.size())));
  if (!g.empty()) CK(cudaMemcpy(p->d_grids, g.data(), sizeof(T) * g.size(), cudaMemcpyHostToDevice));
  if (p->precision == QDG_PREC_DF64) {
    std::vector<qdg::dfl> gd(p->grids_h.size());
    for (size_t i = 0; i < gd.size(); ++i) gd[i] = qdg::dfl(p->grids_h[i]);
    CK(cudaMalloc(&p->d_grids_df, sizeof(qdg::dfl) * std::max<size_t>(1, gd.size())));
    if (!gd.empty()) CK(cudaMemcpy(p->d_grids_df, gd.data(), sizeof(qdg::dfl) * gd.size(), cudaMemcpyHostToDevice));
  }
  CK(cudaMalloc(&p->d_P, sizeof(cplx<T>) * wf_elems(p)));
  if (p->nd > 1 || !p->nac.empty() || p->kin_form != KIN_FFT) {
    size_t smem = 0;
    long long items = 0;
    for (int d = 0; d < p->nd; ++d) {
      CK(cudaMalloc(&p->d_Pd[d], sizeof(cplx<T>) * wf_elems(p)));
      CK(cudaMalloc(&p->d_Pd2[d], sizeof(cplx<T>) * wf_elems(p)));
      smem = std::max(smem, pass_smem(p, d, p->dim[d].TW_k, 1));
      items += (p->npts / ((long long)p->dim[d].n * p->dim[d].TW_k)) * p->S;
    }
    if (smem > 227 * 1024) return fail(QDG_EUNSUPPORTED, "grid line too long for the shared-memory FFT");
    p->kin_smem = smem;
    const int per_sm = qdg::kin_all_max_blocks<T>(256, smem);
    p->kin_grid = (int)std::min<long long>(items, (long long)per_sm * p->sm_count);
  }
  if (!p->nac.empty()) {
    // NAC tiles hold 2 TW lines twice (phi and f phi, ping-pong buffers)
    size_t smem = 0;
    for (int d = 0; d < p->nd; ++d) {
      int tw = p->dim[d].TW_k;
      const int n = p->dim[d].n;
      auto bytes = [&](int t) { return ((size_t)n + 2 * qdg::line_buf_elems(n, 2 * t)) * sizeof(cplx<T>); };
      while (tw > 1 && bytes(tw) > 200 * 1024) tw /= 2;
      p->nac_tw[d] = tw;
      smem = std::max(smem, bytes(tw));
    }
    if (smem > 227 * 1024) return fail(QDG_EUNSUPPORTED, "grid line too long for the shared-memory FFT");
    p->nac_smem = smem;
    p->nac_per_sm = qdg::nac_max_blocks<T>(256, smem);
  }
  {
    long long g = (p->npts + 255) / 256;
    g = std::min<long long>(g, 8LL * p->sm_count);
    p->comb_grid = (int)std::min<long long>(std::max<long long>(g, 1), p->max_parts);
  }
  CK(cudaMalloc(&p->d_scratch, sizeof(cplx<T>) * wf_elems(p)));
  CK(cudaMalloc(&p->d_scratch2, sizeof(cplx<T>) * wf_elems(p)));
  return QDG_OK;
}

void free_plan(qdg_plan *p) {
  for (int d = 0; d < QDG_MAX_DIMS; ++d) {
    if (p->dim[d].tw) cudaFree(p->dim[d].tw);
    if (p->dim[d].kfac) cudaFree(p->dim[d].kfac);
    if (p->dim[d].ktab) cudaFree(p->dim[d].ktab);
    if (p->dim[d].twdf) cudaFree(p->dim[d].twdf);
    if (p->dim[d].ktdf) cudaFree(p->dim[d].ktdf);
  }
  if (p->d_grids) cudaFree(p->d_grids);
  if (p->d_grids_df) cudaFree(p->d_grids_df);
  if (p->d_lasers) cudaFree(p->d_lasers);
  if (p->d_cp) cudaFree(p->d_cp);
  if (p->d_coef) cudaFree(p->d_coef);
  if (p->d_P) cudaFree(p->d_P);
  for (int d = 0; d < QDG_MAX_DIMS; ++d) {
    if (p->d_Pd[d]) cudaFree(p->d_Pd[d]);
    if (p->d_Pd2[d]) cudaFree(p->d_Pd2[d]);
  }
  if (p->d_scratch) cudaFree(p->d_scratch);
  if (p->d_scratch2) cudaFree(p->d_scratch2);
  if (p->d_partials) cudaFree(p->d_partials);
  if (p->d_bar) cudaFree(p->d_bar);
  if (p->h_bar) cudaFreeHost(p->h_bar);
  if (p->h_partials) cudaFreeHost(p->h_partials);
  if (p->own_stream && p->stream) cudaStreamDestroy(p->stream);
  for (auto e : p->ev_pool) cudaEventDestroy(e);
  delete p;
}

void release_child(qdg_plan *p) {
  if (--p->children == 0 && p->destroy_pending) {
    cudaStreamSynchronize(p->stream);
    free_plan(p);
  }
}

// Couplings of the terms selected by `pick` (kinetic terms excluded).
template <typename F>
qdg_status build_couplings(const qdg_plan *p, F pick, qdg::Couplings &cp) {
  struct E { int row, col, gid, lid, nim; };
  std::vector<E> es;
  for (auto &t : p->terms) {
    if (t.kind == QDG_TERM_KINETIC || t.kind == QDG_TERM_NAC || t.kind == QDG_TERM_GMAT || t.kind == QDG_TERM_HOFD ||
        !pick(t))
      continue;
    const int nrep = (p->hermitian && t.row != t.col) ? 2 : 1;
    const int nim = t.kind == QDG_TERM_GOBBLER && t.laser == 1 ? 1 : 0;  // -i W (negative imaginary potential)
    for (int r = 0; r < nrep; ++r)
      es.push_back({r ? t.col : t.row, r ? t.row : t.col, t.grid, t.kind == QDG_TERM_DIPOLE ? t.laser : -1, nim});
  }
  if ((int)es.size() > qdg::kMaxCouplings) return fail(QDG_EUNSUPPORTED, "too many potential/dipole matrix entries");
  std::stable_sort(es.begin(), es.end(), [](const E &a, const E &b) { return a.row < b.row; });
  memset(&cp, 0, sizeof(cp));
  cp.ne = (int)es.size();
  for (int e = 0; e < cp.ne; ++e) {
    cp.row[e] = es[e].row; cp.col[e] = es[e].col; cp.gid[e] = es[e].gid; cp.lid[e] = es[e].lid;
    cp.nim[e] = es[e].nim;
    if (es[e].nim) cp.any_nim = 1;
  }
  for (int s = 0, e = 0; s <= qdg::kMaxStates; ++s) {
    while (e < cp.ne && cp.row[e] < s) ++e;
    cp.rs[s] = e;
  }
  return QDG_OK;
}

// Largest number of potential-matrix entries in one row.
int max_row_entries(const qdg::Couplings &cp) {
  int m = 0;
  for (int s = 0; s < qdg::kMaxStates; ++s) m = std::max(m, cp.rs[s + 1] - cp.rs[s]);
  return m;
}

// Sum of per-block per-state partial dot products (fixed order on the host).
qdg_status finish_dots(qdg_plan *p, int grid, std::vector<cd> &per_state) {
  const int S = p->S;
  CK(cudaMemcpyAsync(p->h_partials, p->d_partials, sizeof(double) * 2 * S * grid, cudaMemcpyDeviceToHost, p->stream));
  CK(cudaStreamSynchronize(p->stream));
  per_state.assign(S, 0.0);
  for (int b = 0; b < grid; ++b)
    for (int s = 0; s < S; ++s)
      per_state[s] += cd(p->h_partials[(b * S + s) * 2], p->h_partials[(b * S + s) * 2 + 1]);
  return QDG_OK;
}

int dots_grid(const qdg_plan *p) {
  long long g = (p->npts + 255) / 256;
  g = std::min<long long>(g, std::min<long long>(p->max_parts / std::max(1, p->S), 2LL * p->sm_count));
  return (int)std::max<long long>(1, g);
}

// <a|b> per state with the grid weight prod dx (WFGridCartesian.cpp:62-117).
template <typename TA, typename TB>
qdg_status dots(qdg_plan *p, const cplx<TA> *a, const cplx<TB> *b, std::vector<cd> &per_state) {
  const int grid = dots_grid(p);
  CK(qdg::launch_dots<TA, TB>(a, b, p->S, p->npts, p->d_partials, grid, p->stream));
  qdg_status s = finish_dots(p, grid, per_state);
  if (s != QDG_OK) return s;
  double w = 1.0;
  for (int d = 0; d < p->nd; ++d) w *= p->dx[d];
  for (auto &v : per_state) v *= w;
  return QDG_OK;
}

cd total(const std::vector<cd> &v) {
  cd t = 0;
  for (auto &x : v) t += x;
  return t;
}

// H psi into the bulk-type scratch buffer `out` (psi is FP64).
template <typename T>
qdg_status h_apply_bulk(qdg_plan *p, const cplx<double> *psi, cplx<T> *out, long long step) {
  CK(qdg::launch_set_coefs(p->d_coef, p->d_cp, p->d_lasers, p->laser_nt, step, p->stream));
  const cplx<T> *in;
  if (sizeof(T) == sizeof(double)) {
    in = reinterpret_cast<const cplx<T> *>(psi);
  } else {
    CK(qdg::launch_convert<T>(reinterpret_cast<cplx<T> *>(p->d_scratch2), psi, wf_elems(p), p->stream));
    in = reinterpret_cast<const cplx<T> *>(p->d_scratch2);
  }
  Epi e;
  e.out = out;
  return run_h<T>(p, qdg::PM_HAPPLY, in, e);
}

// ------------------------------------------------------------ Chebyshev
// Persistent step kernel configuration (cooperative launch: every block
// resident).  step_grid stays 0 when the kernel cannot be made resident.
int step_bulk(const qdg_plan *p) {
  return p->precision == QDG_PREC_MIXED ? qdg::BULK_F32 : p->precision == QDG_PREC_DF64 ? qdg::BULK_DF64 : qdg::BULK_F64;
}

// Kinetic lines of the multi-dimensional step kernel per block.  The lines
// of one dimension and one state form a segment; a block whose lines span
// two segments transforms two partial batches, and the blocks of a term wait
// for the slowest one.  So every segment gets a whole number of blocks, in
// proportion to its work (lines x N (log2 N + 4): the transforms and the
// point work), and its lines are split evenly among them.  With fewer
// blocks than segments the even split over the lines stays (no table).
// Tables for the dimensions [d0, d1): first line of every block, G + 1
// entries, in the kernel's global line numbering.
static bool line_table(const qdg_prop *P, int d0, int d1, std::vector<long long> &bs) {
  const qdg_plan *p = P->plan;
  const int G = P->step_grid;
  const int nseg = (d1 - d0) * p->S;
  bs.clear();
  if (G < nseg || (has(P, "partition") && P->params.at("partition") == "even")) return false;
  std::vector<double> cost(nseg);
  std::vector<long long> nl(nseg);
  double total = 0;
  for (int d = d0; d < d1; ++d)
    for (int s = 0; s < p->S; ++s) {
      const int n = p->dim[d].n, k = (d - d0) * p->S + s;
      nl[k] = p->npts / n;
      cost[k] = (double)(p->npts / n) * n * (std::log2((double)n) + 4.0);
      total += cost[k];
    }
  std::vector<int> nb(nseg);
  int used = 0;
  for (int k = 0; k < nseg; ++k) {
    nb[k] = (int)std::max<long long>(1, std::min<long long>(nl[k], std::llround(G * cost[k] / total)));
    used += nb[k];
  }
  // settle the count: take from or give to the segment with the most / least lines per block
  while (used != G) {
    int best = -1;
    for (int k = 0; k < nseg; ++k) {
      if (used > G && nb[k] <= 1) continue;
      if (used < G && nb[k] >= nl[k]) continue;
      const double lpb = (double)nl[k] / nb[k];
      if (best < 0 || (used > G ? lpb < (double)nl[best] / nb[best] : lpb > (double)nl[best] / nb[best])) best = k;
    }
    if (best < 0) return false;  // cannot settle: keep the even split
    nb[best] += used > G ? -1 : 1;
    used += used > G ? -1 : 1;
  }
  bs.reserve(G + 1);
  long long base = P->line_start[d0];
  for (int k = 0; k < nseg; ++k) {
    for (int j = 0; j < nb[k]; ++j) bs.push_back(base + nl[k] * j / nb[k]);
    base += nl[k];
  }
  bs.push_back(base);
  return true;
}

// Grids of three or more dimensions take two phases per term: the lines of
// dimension 0 finish phi_i (and psi, its norm) and store it, then, after a
// grid barrier, the lines of the other dimensions load phi_i instead of
// recomputing it from the kinetic parts of every dimension, both phi
// buffers and the potentials (cfg3 128^3: that recomputation was a sixth of
// the FP64 work and most of the DRAM traffic).  Two-dimensional grids keep
// one phase per term (their 1024 lines over 152 blocks: a second barrier
// per term costs more than the recomputation).
qdg_status partition_lines(qdg_prop *P) {
  qdg_plan *p = P->plan;
  std::vector<long long> bs;
  if (line_table(P, 0, p->nd, bs)) {
    CK(cudaMalloc(&P->d_bstart, sizeof(long long) * bs.size()));
    CK(cudaMemcpy(P->d_bstart, bs.data(), sizeof(long long) * bs.size(), cudaMemcpyHostToDevice));
  }
  P->two_phase = p->nd >= 3 && !(has(P, "phases") && atoi(P->params.at("phases").c_str()) == 1);
  if (!P->two_phase) return QDG_OK;
  for (int ph = 0; ph < 2; ++ph) {
    if (!line_table(P, ph == 0 ? 0 : 1, ph == 0 ? 1 : p->nd, bs)) continue;
    long long *&dst = ph == 0 ? P->d_bstartA : P->d_bstartB;
    CK(cudaMalloc(&dst, sizeof(long long) * bs.size()));
    CK(cudaMemcpy(dst, bs.data(), sizeof(long long) * bs.size(), cudaMemcpyHostToDevice));
  }
  return QDG_OK;
}

template <typename T>
qdg_status step_setup(qdg_prop *P) {
  qdg_plan *p = P->plan;
  // "path=graph" among the propagator parameters selects the multi-launch
  // graph form of the step (a cross-check of the persistent kernel)
  if (has(P, "path") && P->params.at("path") == "graph") return QDG_OK;
  if (!p->nac.empty()) return QDG_OK;  // NAC elements run as extra line passes (graph path)
  if (p->kin_form != KIN_FFT) return QDG_OK;  // HOFD / GridGMat kinetic passes (graph path)
  if (p->generic_fft) return QDG_OK;          // prime radices above 5 (graph path)
  // The DF64 form's multi-dimensional step kernel computes its bulk in
  // double-float (~48 bits, FP32 exponent range).  Imaginary-time series
  // reach the low states through cancellations of terms ~1/sqrt(2 pi R) down
  // to e^{-R(1-X)}, which need the last bits of binary64: they take the graph
  // path (binary64).
  if (P->imag && p->precision == QDG_PREC_DF64 && p->nd > 1) return QDG_OK;
  const int bulk = step_bulk(p);
  const size_t cs = p->csize;
  if (p->nd == 1) {
    P->step_tw1 = p->dim[0].TW_e;
    const size_t smem = pass_smem(p, 0, P->step_tw1, p->S);
    if (smem > 227 * 1024) return QDG_OK;
    const int per_sm = qdg::cheby_step_max_blocks(bulk, p->S, p->nd, 256, smem);
    if (per_sm <= 0) return QDG_OK;
    long long want = p->npts / ((long long)p->dim[0].n * P->step_tw1);
    want = std::min<long long>(want, (long long)per_sm * p->sm_count);
    P->step_grid = (int)std::max<long long>(1, std::min<long long>(want, p->max_parts));
    P->step_smem = smem;
    return QDG_OK;
  }
  if (max_row_entries(p->cp_h) > qdg::kMaxRowEntries) return QDG_OK;
  // kinetic lines of all dimensions, split into one contiguous run per block
  long long total = 0;
  for (int d = 0; d < p->nd; ++d) {
    P->line_start[d] = total;
    total += (p->npts / p->dim[d].n) * p->S;
  }
  P->line_start[p->nd] = total;
  // shared memory per block for the line buffers: a kernel that fits one
  // block per SM anyway (its registers) takes most of the SM's 228 KB, so
  // large grids transform more lines per batch; otherwise two blocks fit
  const size_t budget =
      qdg::cheby_step_max_blocks(bulk, p->S, p->nd, 256, 16 * 1024) == 1 ? 200 * 1024 : 112 * 1024;
  // the staging slots of the gather (binary64 and double-float bulk, one or
  // two states) sit in front of the twiddles and line buffers
  const size_t stage = (bulk != qdg::BULK_F32 && qdg::step_staged((int)cs, p->S))
                           ? (size_t)qdg::step_stage_bytes_c(p->nd, p->S) : 0;
  if (stage + 16 * 1024 > budget) return QDG_OK;
  int grid = 0;
  size_t smem = 0;
  for (int iter = 0, per_sm = 0; iter < 3; ++iter) {
    const size_t probe = iter == 0 ? stage + 16 * 1024 : smem;
    per_sm = qdg::cheby_step_max_blocks(bulk, p->S, p->nd, 256, probe);
    if (per_sm <= 0) return QDG_OK;
    grid = (int)std::min<long long>((long long)per_sm * p->sm_count, std::min<long long>(total, p->max_parts));
    const long long chunk = (total + grid - 1) / grid;
    smem = 0;
    for (int d = 0; d < p->nd; ++d) {
      const long long n = p->dim[d].n;
      long long cap = (long long)(((budget - stage) / cs - n) / (2 * (size_t)qdg::lstride((int)n)));
      int lm = (int)std::max<long long>(1, std::min<long long>(std::min<long long>(chunk, cap), qdg::kMaxBatchLines));
      const int tuned = qdg::schedule_lines(qdg::SCHED_PLAN, (int)n, p->precision);
      if (tuned > 0) lm = std::min(lm, tuned);
      P->lmax[d] = lm;
      smem = std::max(smem, stage + ((size_t)n + 2 * qdg::line_buf_elems((int)n, lm)) * cs);
    }
    if (smem > 227 * 1024) return QDG_OK;
    if (qdg::cheby_step_max_blocks(bulk, p->S, p->nd, 256, smem) >= per_sm) break;
  }
  const int per_sm = qdg::cheby_step_max_blocks(bulk, p->S, p->nd, 256, smem);
  if (per_sm <= 0) return QDG_OK;
  P->step_grid = std::min(grid, per_sm * p->sm_count);
  if (has(P, "step_blocks")) P->step_grid = std::max(1, std::min(P->step_grid, atoi(P->params.at("step_blocks").c_str())));
  P->step_smem = smem;
  return partition_lines(P);
}

// Device copy of host values in the step kernel's bulk type (binary64,
// double-float for the DF64 form, FP32 for the mixed form).
// The scaled tables in the step kernel's bulk type: FP32 (mixed), double-
// float (the DF64 form's multi-dimensional kernel) or binary64 (FP64, and
// one-dimensional grids in both FP64 forms).
qdg_status upload_bulk(const qdg_plan *p, const std::vector<long double> &v, void **out) {
  if (p->precision == QDG_PREC_MIXED) {
    std::vector<float> h(v.begin(), v.end());
    CK(cudaMalloc(out, sizeof(float) * std::max<size_t>(1, h.size())));
    CK(cudaMemcpy(*out, h.data(), sizeof(float) * h.size(), cudaMemcpyHostToDevice));
  } else if (p->precision == QDG_PREC_DF64 && p->nd > 1) {
    std::vector<qdg::dfl> h(v.size());
    for (size_t i = 0; i < v.size(); ++i) {
      const float hi = (float)v[i];
      h[i] = qdg::dfl(hi, (float)(v[i] - (long double)hi));
    }
    CK(cudaMalloc(out, sizeof(qdg::dfl) * std::max<size_t>(1, h.size())));
    CK(cudaMemcpy(*out, h.data(), sizeof(qdg::dfl) * h.size(), cudaMemcpyHostToDevice));
  } else {
    std::vector<double> h(v.begin(), v.end());
    CK(cudaMalloc(out, sizeof(double) * std::max<size_t>(1, h.size())));
    CK(cudaMemcpy(*out, h.data(), sizeof(double) * h.size(), cudaMemcpyHostToDevice));
  }
  return QDG_OK;
}

// Pre-scaled point work of the step kernel (real offset and a purely
// imaginary or real series factor, i.e. every hermitian Hamiltonian).
// phi_n = fac (H - offset) phi_{n-1} +- phi_{n-2} with fac = i f (real time)
// or f (imaginary time): T'_d = f T_d, W_ss = f (sum of the static diagonal
// potentials of row s), W_e = f V_e for every other entry (its field
// coefficient stays separate), and -f offset applied per point as a value
// plus its rounding residual; the first term's factor is fac/2.  Same series,
// rounding of the products only, and every rounding depends on the data: a
// rounded constant multiplying every point (f, or f offset) would scale or
// shift the series argument coherently, a phase error that grows with every
// time step (3e-12 in the autocorrelation after 500 steps of the 1-D Morse
// line with offset 18.6 hartree).
qdg_status scaled_setup(qdg_prop *P) {
  qdg_plan *p = P->plan;
  if (P->step_grid <= 0) return QDG_OK;
  if (p->cp_h.any_nim) return QDG_OK;  // negative imaginary potentials: the unscaled point work
  const cd fac = 2.0 * (P->c0 / P->dt) / P->scaling;
  if (P->offset.imag() != 0 || (fac.real() != 0 && fac.imag() != 0)) return QDG_OK;
  const bool rt = fac.real() == 0;
  const long double f = 2.0L * (rt ? (long double)P->c0.imag() : (long double)P->c0.real()) / (long double)P->dt /
                        (long double)P->scaling;
  const long double off = P->offset.real();
  const int S = p->S;
  const long long n = p->npts;
  const qdg::Couplings &cp = p->cp_h;
  // rows: the diagonal grid first, then every entry not folded into it
  struct E { int row, col, gid, lid; };
  std::vector<E> es;
  std::vector<int> extra;  // plan entry index of each extra scaled grid
  for (int st = 0; st < S; ++st) {
    es.push_back({st, st, st, -1});
    for (int e = cp.rs[st]; e < cp.rs[st + 1]; ++e) {
      if (cp.col[e] == st && cp.lid[e] < 0) continue;  // folded into the diagonal grid
      es.push_back({st, cp.col[e], S + (int)extra.size(), cp.lid[e] >= 0 ? e : -1});
      extra.push_back(e);
    }
  }
  qdg::Couplings sc;
  memset(&sc, 0, sizeof(sc));
  sc.ne = (int)es.size();
  if (sc.ne > qdg::kMaxCouplings) return QDG_OK;
  for (int e = 0; e < sc.ne; ++e) { sc.row[e] = es[e].row; sc.col[e] = es[e].col; sc.gid[e] = es[e].gid; sc.lid[e] = es[e].lid; }
  for (int st = 0, e = 0; st <= qdg::kMaxStates; ++st) {
    while (e < sc.ne && sc.row[e] < st) ++e;
    sc.rs[st] = e;
  }
  if (p->nd > 1 && max_row_entries(sc) > qdg::kMaxRowEntries) return QDG_OK;
  std::vector<long double> g((size_t)(S + extra.size()) * n);
  for (int st = 0; st < S; ++st) {
    long double *d = g.data() + (size_t)st * n;
    for (long long i = 0; i < n; ++i) d[i] = 0;
    for (int e = cp.rs[st]; e < cp.rs[st + 1]; ++e) {
      if (cp.col[e] != st || cp.lid[e] >= 0) continue;
      const double *v = p->grids_h.data() + (size_t)cp.gid[e] * n;
      for (long long i = 0; i < n; ++i) d[i] += v[i];
    }
    for (long long i = 0; i < n; ++i) d[i] = f * d[i];
  }
  for (size_t j = 0; j < extra.size(); ++j) {
    const double *v = p->grids_h.data() + (size_t)cp.gid[extra[j]] * n;
    long double *d = g.data() + (size_t)(S + j) * n;
    for (long long i = 0; i < n; ++i) d[i] = f * (long double)v[i];
  }
  qdg_status s = upload_bulk(p, g, &P->sgrids);
  if (s != QDG_OK) return s;
  for (int d = 0; d < p->nd; ++d) {
    const int nd = p->dim[d].n;
    std::vector<long double> kf(S, 0.0L);
    for (auto &t : p->terms)
      if (t.kind == QDG_TERM_KINETIC) kf[t.row] += ((long double)p->dk[d] * p->dk[d]) / (2.0L * t.mass[d]) / nd;
    std::vector<long double> k((size_t)S * nd);
    for (int st = 0; st < S; ++st)
      for (int i = 0; i < nd; ++i) {
        const long double kq = std::min(i, nd - i);
        k[(size_t)st * nd + i] = f * kf[st] * kq * kq;
      }
    if ((s = upload_bulk(p, k, &P->sk[d])) != QDG_OK) return s;
  }
  CK(cudaMalloc(&P->d_scp, sizeof(qdg::Couplings)));
  CK(cudaMemcpy(P->d_scp, &sc, sizeof(sc), cudaMemcpyHostToDevice));
  const long double so = -f * off;
  P->soff_hi = (double)so;
  P->soff_lo = (double)(so - (long double)P->soff_hi);
  P->scaled = 1;
  P->scaled_rt = rt ? 1 : 0;
  P->scaled_ne = sc.ne;
  return QDG_OK;
}

// One line of a 1-D single-state grid with only a static potential goes to
// a cluster kernel: in binary64 with N a power of two from 512 to 2048, the
// one-component-per-thread kernel on 16 (or 8) blocks; otherwise, when
// N = 8 M with M a multiple of 8 (the exchange splits the M columns evenly
// over the 8 blocks), the radix-plan kernel on 8 blocks.  The propagator
// parameter cluster=0 keeps the line on the single-block step kernel,
// cluster=1 selects the radix-plan kernel.
void cluster_setup(qdg_prop *P) {
  qdg_plan *p = P->plan;
  if (!P->scaled || p->nd != 1 || p->S != 1 || P->scaled_ne != 1) return;
  const int want = has(P, "cluster") ? atoi(P->params.at("cluster").c_str()) : 2;
  if (want == 0) return;
  const int N = p->dim[0].n;
  if (want == 2 && is64(p) && (N & (N - 1)) == 0) {
    const int C = qdg::line64_cluster_size(N);
    if (C > 0) {
      P->cluster = 2;
      P->cluster_size = C;
      return;
    }
  }
  if (N % 64 != 0 || N < 512 || N > 8192) return;
  if (!qdg::schedule_radix(qdg::SCHED_PLAN, N / 8, p->precision, P->crp)) return;
  P->cluster = 1;
  P->cluster_size = 8;
}

template <typename T>
qdg_status cheby_step_cluster(qdg_prop *P, cplx<double> *psi) {
  qdg_plan *p = P->plan;
  qdg::ClusterStepArgs<T> a;
  memset(&a, 0, sizeof(a));
  a.N = p->dim[0].n;
  a.M = a.N / 8;
  a.rp = P->crp;
  a.twN = reinterpret_cast<const cplx<T> *>(p->dim[0].tw);
  a.ktab = reinterpret_cast<const T *>(P->sk[0]);
  a.V = reinterpret_cast<const T *>(P->sgrids);
  a.psi = psi;
  a.psi_out = psi;
  a.soff_hi = P->soff_hi;
  a.soff_lo = P->soff_lo;
  a.rt = P->scaled_rt;
  a.a = P->d_a;
  a.order = P->order;
  a.prec = P->prec;
  a.imag = P->imag ? 1 : 0;
  a.offim0 = P->offset.imag() == 0 ? 1 : 0;
  a.diff = p->precision == QDG_PREC_MIXED ? 1 : 0;
  a.ph = C(std::exp(P->c0 * P->offset));
  a.cs = P->d_cs;
  size_t slot = 0;
  qdg_status s = prof_begin<T>(p, 6, &slot);
  if (s != QDG_OK) return s;
  if constexpr (std::is_same<T, double>::value) {
    if (P->cluster == 2) {
      CK(qdg::launch_cheby_line64(a, P->cluster_size, p->stream));
      return prof_end(p, slot);
    }
  }
  CK(qdg::launch_cheby_step_cluster<T>(a, p->stream));
  return prof_end(p, slot);
}

template <typename T>
qdg_status cheby_step_persistent(qdg_prop *P, cplx<double> *psi, long long step) {
  qdg_plan *p = P->plan;
  if (P->cluster) return cheby_step_cluster<T>(P, psi);
  CK(qdg::launch_set_coefs(p->d_coef, p->d_cp, p->d_lasers, p->laser_nt, step, p->stream));
  qdg::StepArgs<T> a;
  memset(&a, 0, sizeof(a));
  a.bulk = step_bulk(p);
  a.nd = p->nd;
  a.S = p->S;
  a.npts = p->npts;
  long long items = 0;
  for (int d = 0; d < p->nd; ++d) {
    qdg::PassArgs<T> g;
    memset(&g, 0, sizeof(g));
    fill_geometry<T>(p, d, 1, g);
    qdg::DimPass<T> &dp = a.dp[d];
    dp.N = g.N; dp.es = g.es; dp.ls = g.ls; dp.TW = g.TW; dp.tiles_per_hi = g.tiles_per_hi;
    dp.hi_stride = g.hi_stride; dp.ntiles = g.ntiles; dp.rp = g.rp; dp.tw = g.tw; dp.kfac = g.kfac;
    dp.P = reinterpret_cast<cplx<T> *>(p->d_Pd[d]);
    dp.ktab = reinterpret_cast<const T *>(P->scaled ? P->sk[d] : p->dim[d].ktab);
    dp.twdf = reinterpret_cast<const cplx<qdg::dfl> *>(p->dim[d].twdf);
    dp.ktdf = reinterpret_cast<const qdg::dfl *>(P->scaled ? P->sk[d] : p->dim[d].ktdf);
    a.item_start[d] = items;
    items += g.ntiles * p->S;
  }
  a.item_start[p->nd] = items;
  for (int d = 0; d <= p->nd; ++d) a.line_start[d] = P->line_start[d];
  for (int d = 0; d < p->nd; ++d) a.lmax[d] = P->lmax[d];
  a.bstart = P->d_bstart;
  a.bstartA = P->d_bstartA;
  a.bstartB = P->d_bstartB;
  a.two_phase = P->two_phase ? 1 : 0;
  a.TW1 = P->step_tw1;
  a.psi = psi;
  a.buf[0] = reinterpret_cast<cplx<T> *>(P->k0);
  a.buf[1] = reinterpret_cast<cplx<T> *>(P->k1);
  a.buf[2] = reinterpret_cast<cplx<T> *>(P->k2);
  for (int d = 0; d < p->nd; ++d) {
    a.Pn[0][d] = reinterpret_cast<cplx<T> *>(p->d_Pd[d]);
    a.Pn[1][d] = reinterpret_cast<cplx<T> *>(p->d_Pd2[d]);
  }
  a.cp = p->d_cp;
  a.coef = p->d_coef;
  a.grids = reinterpret_cast<const T *>(p->d_grids);
  a.gdf = reinterpret_cast<const qdg::dfl *>(p->d_grids_df);
  a.scaled = P->scaled;
  a.scaled_rt = P->scaled_rt;
  a.soff_hi = P->soff_hi;
  a.soff_lo = P->soff_lo;
  a.scp = P->d_scp;
  a.sgrids = P->sgrids;
  const cd ex = P->c0 / P->dt;
  a.offset = C(P->offset);
  a.fac1 = C(ex / P->scaling);
  a.fac = C(2.0 * ex / P->scaling);
  a.ph = C(std::exp(P->c0 * P->offset));
  a.a = P->d_a;
  a.order = P->order;
  a.prec = P->prec;
  a.imag = P->imag ? 1 : 0;
  a.offim0 = P->offset.imag() == 0 ? 1 : 0;
  a.diff = p->precision == QDG_PREC_MIXED ? 1 : 0;
  a.partials = p->d_partials;
  a.cs = P->d_cs;
  a.bar = p->d_bar;
  // phase timing of one block (block 0 unless QDG_TRACE_BLOCK names another)
  const char *tb = getenv("QDG_TRACE_BLOCK");
  a.trace = p->profiling ? 1 + (tb ? std::max(0, std::min(atoi(tb), P->step_grid - 1)) : 0) : 0;
  size_t slot = 0;
  qdg_status s = prof_begin<T>(p, 6, &slot);
  if (s != QDG_OK) return s;
  CK(qdg::launch_cheby_step<T>(a, P->step_grid, 256, P->step_smem, p->stream));
  return prof_end(p, slot);
}

// OCheby::Init (src/qdlib/OCheby.cpp:358-493).
qdg_status cheby_init(qdg_prop *P) {
  qdg_plan *p = P->plan;
  qdg::host::ChebySeries cs;
  const std::string err = qdg::host::cheby_series(p->emax, p->emin, P->dt, P->c0, P->imag, P->params, cs);
  if (!err.empty()) return fail(QDG_EINVAL, err);
  P->order = cs.order;
  P->scaling = cs.scaling;
  P->offset = cs.offset;
  P->coeff = cs.coeff;
  P->prec = cs.prec;
  const size_t bytes = p->csize * wf_elems(p);
  CK(cudaMalloc(&P->k0, bytes));
  CK(cudaMalloc(&P->k1, bytes));
  CK(cudaMalloc(&P->k2, bytes));
  CK(cudaMalloc(&P->d_cs, sizeof(qdg::ChebyState)));
  CK(cudaMemset(P->d_cs, 0, sizeof(qdg::ChebyState)));
  {
    const cd ph = std::exp(P->c0 * P->offset);
    std::vector<cplx<double>> hc(P->order);
    for (int i = 0; i < P->order; ++i) hc[i] = C(P->coeff[i] * ph);
    CK(cudaMalloc(&P->d_coeffs, sizeof(cplx<double>) * P->order));
    CK(cudaMemcpy(P->d_coeffs, hc.data(), sizeof(cplx<double>) * P->order, cudaMemcpyHostToDevice));
    CK(cudaMalloc(&P->d_a, sizeof(double) * P->order));
    CK(cudaMemcpy(P->d_a, P->coeff.data(), sizeof(double) * P->order, cudaMemcpyHostToDevice));
  }
  qdg_status ps = is64(p) ? step_setup<double>(P) : step_setup<float>(P);
  if (ps != QDG_OK) return ps;
  if (!has(P, "scaled") || atoi(P->params.at("scaled").c_str()) != 0)
    if ((ps = scaled_setup(P)) != QDG_OK) return ps;
  cluster_setup(P);
  CK(cudaMallocHost(&P->h_cs, sizeof(qdg::ChebyState)));
  return QDG_OK;
}

// The series factor m exp/scaling (m = 1 for the first term, 2 after) as a
// rounded value and its residual, from a long double evaluation.
void series_factor(const qdg_prop *P, double m, Epi &e) {
  const std::complex<long double> ex((long double)P->c0.real() / P->dt, (long double)P->c0.imag() / P->dt);
  const std::complex<long double> f = ex * (long double)m / (long double)P->scaling;
  e.fac = cd((double)f.real(), (double)f.imag());
  e.fac_lo = cd((double)(f.real() - (long double)e.fac.real()), (double)(f.imag() - (long double)e.fac.imag()));
}

// Epilogue arguments shared by all terms of a Chebyshev step.
template <typename T>
Epi cheby_epi(qdg_prop *P, cplx<double> *psi) {
  Epi e;
  e.psi = psi;
  e.offset = P->offset;
  e.imag = P->imag ? 1 : 0;
  e.done = &P->d_cs->done;
  e.cut.cs = P->d_cs;
  e.cut.prec = P->prec;
  e.cut.imag = e.imag;
  e.cut.offim0 = P->offset.imag() == 0 ? 1 : 0;
  e.cut.diff = P->plan->precision == QDG_PREC_MIXED ? 1 : 0;
  e.cut.order = P->order;
  e.cut.coeffs = P->d_coeffs;
  e.bufs[0] = P->k0;
  e.bufs[1] = P->k1;
  return e;
}

// Begin, psi copy and the first two terms of the series (OCheby.cpp:99-111):
// phi_1 = (H - offset) psi exp/scaling; psi = psi c0 + phi_1 c1.
template <typename T>
qdg_status cheby_prologue(qdg_prop *P, cplx<double> *psi, unsigned long long cond, int use_cond) {
  qdg_plan *p = P->plan;
  CK(qdg::launch_cheby_begin(P->d_cs, P->order, cond, use_cond, p->stream));
  cplx<T> *k0 = reinterpret_cast<cplx<T> *>(P->k0);
  CK(qdg::launch_convert<T>(k0, psi, wf_elems(p), p->stream));  // ket0 = Psi
  const cd ex = P->c0 / P->dt;
  const cd ph = std::exp(P->c0 * P->offset);
  Epi e = cheby_epi<T>(P, psi);
  e.k0 = P->k1;
  series_factor(P, 1.0, e);
  e.c0p = P->coeff[0] * ph;
  e.c1p = P->coeff[1] * ph;
  e.cut.first = 1;
  e.cut.term = 1;
  e.cut.cond = cond;
  e.cut.use_cond = use_cond;
  return run_h<T>(p, qdg::PM_CHEBY_FIRST, k0, e);
}

// The device work of one Chebyshev step (OCheby::real_time_step /
// imag_time_step), every term launched from the host: no host
// synchronisation; the series cut is decided on the device by the last
// block of each term and later terms skip their work.
template <typename T>
qdg_status cheby_body(qdg_prop *P, cplx<double> *psi) {
  qdg_plan *p = P->plan;
  qdg_status s = cheby_prologue<T>(P, psi, 0, 0);
  if (s != QDG_OK) return s;
  cplx<T> *k0 = reinterpret_cast<cplx<T> *>(P->k0);
  cplx<T> *k1 = reinterpret_cast<cplx<T> *>(P->k1);
  const cd ex = P->c0 / P->dt;
  const cd ph = std::exp(P->c0 * P->offset);
  Epi e = cheby_epi<T>(P, psi);
  series_factor(P, 2.0, e);
  for (int i = 2; i < P->order; ++i) {
    e.k0 = k0;  // phi_{n-2} in, phi_n out
    e.coeff = P->coeff[i] * ph;
    e.cut.term = i;
    if ((s = run_h<T>(p, qdg::PM_CHEBY_TERM, k1, e)) != QDG_OK) return s;
    std::swap(k0, k1);
  }
  CK(qdg::launch_cheby_end(P->d_cs, p->stream));
  return QDG_OK;
}

// One term of the device-driven loop: the term index, the buffers and the
// coefficient come from the device state; the last block of the term ends
// the loop (conditional while node) once the series is cut.
template <typename T>
qdg_status cheby_dyn_term(qdg_prop *P, cplx<double> *psi, unsigned long long cond) {
  Epi e = cheby_epi<T>(P, psi);
  series_factor(P, 2.0, e);
  e.cut.dyn = 1;
  e.cut.cond = cond;
  e.cut.use_cond = 1;
  return run_h<T>(P->plan, qdg::PM_CHEBY_TERM, nullptr, e);
}

// Graph of a whole step with a conditional while node around one term:
// terms after the series cut cost nothing.
template <typename T>
qdg_status build_while_graph(qdg_prop *P, cplx<double> *psi, cudaGraphExec_t *exec) {
  qdg_plan *p = P->plan;
  cudaStream_t st = p->stream;
  cudaGraph_t g = nullptr;
  CK(cudaGraphCreate(&g, 0));
  cudaGraphConditionalHandle cond;
  if (cudaGraphConditionalHandleCreate(&cond, g, 1, cudaGraphCondAssignDefault) != cudaSuccess) {
    cudaGraphDestroy(g);
    return fail(QDG_ECUDA, "conditional handle");
  }
  const long long l0 = qdg::launch_counter();
  if (cudaStreamBeginCaptureToGraph(st, g, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed) != cudaSuccess) {
    cudaGraphDestroy(g);
    return fail(QDG_ECUDA, "capture to graph");
  }
  qdg_status s = cheby_prologue<T>(P, psi, cond, 1);
  cudaStreamCaptureStatus cst;
  const cudaGraphNode_t *deps = nullptr;
  size_t ndeps = 0;
  cudaGraphNode_t wnode = nullptr;
  cudaGraph_t body = nullptr;
  bool ok = s == QDG_OK && cudaStreamGetCaptureInfo(st, &cst, nullptr, nullptr, &deps, nullptr, &ndeps) == cudaSuccess;
  if (ok) {
    cudaGraphNodeParams np = {cudaGraphNodeTypeConditional};
    np.conditional.handle = cond;
    np.conditional.type = cudaGraphCondTypeWhile;
    np.conditional.size = 1;
    ok = cudaGraphAddNode(&wnode, g, deps, nullptr, ndeps, &np) == cudaSuccess;
    if (ok) {
      body = np.conditional.phGraph_out[0];
      ok = cudaStreamUpdateCaptureDependencies(st, &wnode, nullptr, 1, cudaStreamSetCaptureDependencies) == cudaSuccess;
    }
  }
  if (ok) ok = qdg::launch_cheby_end(P->d_cs, st) == cudaSuccess;
  cudaGraph_t gout = nullptr;
  const bool ended = cudaStreamEndCapture(st, &gout) == cudaSuccess;
  const long long l1 = qdg::launch_counter();
  if (ok && ended) {
    ok = cudaStreamBeginCaptureToGraph(st, body, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed) == cudaSuccess;
    if (ok) {
      qdg_status s2 = cheby_dyn_term<T>(P, psi, cond);
      cudaGraph_t bout = nullptr;
      ok = cudaStreamEndCapture(st, &bout) == cudaSuccess && s2 == QDG_OK;
    }
  }
  if (ok && ended) ok = cudaGraphInstantiate(exec, g, 0) == cudaSuccess;
  cudaGraphDestroy(g);
  const long long l2 = qdg::launch_counter();
  qdg::add_launches(-(l2 - l0));
  if (!ok || !ended) {
    cudaGetLastError();
    if (s != QDG_OK) return s;
    return fail(QDG_ECUDA, "conditional graph unavailable");
  }
  P->graph_launches = l1 - l0;
  P->body_launches = l2 - l1;
  return QDG_OK;
}

template <typename T>
qdg_status build_static_graph(qdg_prop *P, cplx<double> *psi, cudaGraphExec_t *exec) {
  qdg_plan *p = P->plan;
  cudaGraph_t g = nullptr;
  const long long l0 = qdg::launch_counter();
  CK(cudaStreamBeginCapture(p->stream, cudaStreamCaptureModeRelaxed));
  qdg_status s = cheby_body<T>(P, psi);
  cudaError_t ce = cudaStreamEndCapture(p->stream, &g);
  const long long l1 = qdg::launch_counter();
  qdg::add_launches(-(l1 - l0));
  if (s != QDG_OK) { if (g) cudaGraphDestroy(g); return s; }
  if (ce != cudaSuccess || cudaGraphInstantiate(exec, g, 0) != cudaSuccess) {
    if (g) cudaGraphDestroy(g);
    cudaGetLastError();
    return fail(QDG_ECUDA, "stream capture unavailable");
  }
  cudaGraphDestroy(g);
  P->graph_launches = l1 - l0;
  P->body_launches = 0;
  return QDG_OK;
}

template <typename T>
qdg_status cheby_enqueue(qdg_prop *P, cplx<double> *psi, long long step) {
  qdg_plan *p = P->plan;
  CK(qdg::launch_set_coefs(p->d_coef, p->d_cp, p->d_lasers, p->laser_nt, step, p->stream));
  if (p->profiling || !P->graphs_ok) return cheby_body<T>(P, psi);
  if (!P->graph || P->graph_psi != psi || P->graph_stream != p->stream) {
    if (P->graph) { cudaGraphExecDestroy(P->graph); P->graph = nullptr; }
    qdg_status s = QDG_ECUDA;
    if (P->while_ok) {
      s = build_while_graph<T>(P, psi, &P->graph);
      P->graph_is_while = s == QDG_OK;
      if (s != QDG_OK) { P->while_ok = false; P->graph = nullptr; }
    }
    if (s != QDG_OK) {
      s = build_static_graph<T>(P, psi, &P->graph);
      P->graph_is_while = false;
      if (s != QDG_OK) { P->graphs_ok = false; P->graph = nullptr; return cheby_body<T>(P, psi); }
    }
    P->graph_psi = psi;
    P->graph_stream = p->stream;
  }
  CK(cudaGraphLaunch(P->graph, p->stream));
  qdg::add_launches(P->graph_launches);
  return QDG_OK;
}

// After a synchronisation: did a grid barrier of the step kernel time out?
qdg_status check_barrier(qdg_plan *p) {
  CK(cudaMemcpy(p->h_bar, p->d_bar, sizeof(qdg::GridBarrier), cudaMemcpyDeviceToHost));
  if (p->h_bar->err) {
    qdg::GridBarrier z{};
    CK(cudaMemcpy(p->d_bar, &z, sizeof(z), cudaMemcpyHostToDevice));
    return fail(QDG_ETIMEOUT, "grid barrier of the Chebyshev step kernel timed out");
  }
  return QDG_OK;
}

// Kernels the while body ran: (terms - 2) term bodies per step.
void count_body_launches(qdg_prop *P, long long terms, long long steps) {
  if (P->graph && P->graph_is_while) qdg::add_launches(P->body_launches * std::max(0LL, terms - 2 * steps));
}

// ------------------------------------------------------------------ GSPO
// OGSPO::Init (OGSPO.cpp:61-105): members A, B, C, ... must each have a
// diagonal representation: an FFT member (GridNablaSq on every state) or a
// potential member (per grid point S x S matrix).
qdg_status gspo_init(qdg_prop *P) {
  qdg_plan *p = P->plan;
  int ng = 0;
  for (auto &t : p->terms) ng = std::max(ng, t.group + 1);
  if (ng < 1) return fail(QDG_EINVAL, "GSPO is empty!");
  if (ng > QDG_MAX_GROUPS) return fail(QDG_EINVAL, "too many GSPO members");
  for (auto &t : p->terms)  // OGSPO::Init takes ODSpace members only (OGSPO.cpp:71-85); OGridNAC is none
    if (t.kind == QDG_TERM_NAC || t.kind == QDG_TERM_GOBBLER)
      return fail(QDG_EUNSUPPORTED, "GSPO members must be ODSpace operators (no GridNAC, no Gobbler)");
  // OGridGMat is no ODSpace; OGridNablaSq with method HOFD has no k-space
  // table to exponentiate (Diff::_InitKspace returns early, Diff.cpp:52-54)
  if (p->kin_form != KIN_FFT)
    return fail(QDG_EUNSUPPORTED, "GSPO members need a diagonal representation (no HOFD, no GridGMat)");
  if (!p->hermitian) return fail(QDG_EUNSUPPORTED, "GSPO members must be hermitian matrices");
  P->ngroups = ng;
  P->group_kinetic.assign(ng, 0);
  P->gcp_h.resize(ng);
  P->gcp_d.assign(ng, nullptr);
  P->gcoef_d.assign(ng, nullptr);
  P->gtab.assign(ng, std::vector<void *>(p->nd, nullptr));
  P->gdyn.assign(ng, 0);
  P->gU.assign(ng, nullptr);
  for (auto &t : p->terms)
    if (t.kind == QDG_TERM_DIPOLE) P->gdyn[t.group] = 1;
  for (int g = 0; g < ng; ++g) {
    bool any = false, kin = false, pot = false;
    for (auto &t : p->terms)
      if (t.group == g) { any = true; (t.kind == QDG_TERM_KINETIC ? kin : pot) = true; }
    if (!any) return fail(QDG_EINVAL, "GSPO misses an operator. Sequence must be A, B, C, ...");
    if (kin && pot) return fail(QDG_EUNSUPPORTED, "GSPO: Operator has no diagonal representation");
    P->group_kinetic[g] = kin ? 1 : 0;
    const double sf = g == 0 ? 1.0 : 0.5;  // OGSPO::InitExp: first member full step, others half
    if (kin) {
      for (int s = 0; s < p->S; ++s) {
        int c = 0;
        for (auto &t : p->terms)
          if (t.group == g && t.kind == QDG_TERM_KINETIC && t.row == s) ++c;
        if (c != 1) return fail(QDG_EUNSUPPORTED, "GSPO kinetic member needs one GridNablaSq per state");
      }
      // exp(c sf dk^2 k^2/(2m)) / N_d per dimension and state (time independent)
      for (int d = 0; d < p->nd; ++d) {
        const int n = p->dim[d].n;
        std::vector<std::complex<long double>> tab((size_t)p->S * n);
        for (auto &t : p->terms) {
          if (t.group != g || t.kind != QDG_TERM_KINETIC) continue;
          const long double f = (long double)p->dk[d] * p->dk[d] / (2.0L * t.mass[d]);
          for (int i = 0; i < n; ++i) {
            const long double kq = std::min(i, n - i);
            const std::complex<long double> z = std::complex<long double>(P->c0.real(), P->c0.imag()) * (long double)sf * (f * kq * kq);
            tab[(size_t)t.row * n + i] = std::exp(z) / (long double)n;
          }
        }
        if (is64(p)) {
          std::vector<cplx<double>> h(tab.size());
          for (size_t i = 0; i < tab.size(); ++i) { h[i].re = (double)tab[i].real(); h[i].im = (double)tab[i].imag(); }
          CK(cudaMalloc(&P->gtab[g][d], sizeof(cplx<double>) * h.size()));
          CK(cudaMemcpy(P->gtab[g][d], h.data(), sizeof(cplx<double>) * h.size(), cudaMemcpyHostToDevice));
        } else {
          std::vector<cplx<float>> h(tab.size());
          for (size_t i = 0; i < tab.size(); ++i) { h[i].re = (float)tab[i].real(); h[i].im = (float)tab[i].imag(); }
          CK(cudaMalloc(&P->gtab[g][d], sizeof(cplx<float>) * h.size()));
          CK(cudaMemcpy(P->gtab[g][d], h.data(), sizeof(cplx<float>) * h.size(), cudaMemcpyHostToDevice));
        }
      }
    } else {
      qdg_status s = build_couplings(p, [g](const qdg_hterm &t) { return t.group == g; }, P->gcp_h[g]);
      if (s != QDG_OK) return s;
      // coupled members of any number of states: per-point S x S exponentials
      // (closed form for S = 2, Jacobi rotations above)
      CK(cudaMalloc(&P->gcp_d[g], sizeof(qdg::Couplings)));
      CK(cudaMemcpy(P->gcp_d[g], &P->gcp_h[g], sizeof(qdg::Couplings), cudaMemcpyHostToDevice));
      CK(cudaMalloc(&P->gcoef_d[g], sizeof(double) * qdg::kMaxCouplings));
    }
  }
  if (!is64(p)) CK(cudaMalloc(&P->k0, p->csize * wf_elems(p)));
  return QDG_OK;
}

template <typename T>
qdg_status gspo_member(qdg_prop *P, int g, cplx<T> *x, long long step) {
  qdg_plan *p = P->plan;
  const double sf = g == 0 ? 1.0 : 0.5;
  if (P->group_kinetic[g]) {
    qdg::PassArgs<T> a;
    memset(&a, 0, sizeof(a));
    for (int d = 0; d < p->nd; ++d) {
      fill_geometry<T>(p, d, 1, a);
      a.phi = x;
      a.out = x;
      a.gtab = reinterpret_cast<const cplx<T> *>(P->gtab[g][d]);
      qdg_status s = launch_one<T>(p, qdg::PM_GSPO_KIN, d, a, nullptr);
      if (s != QDG_OK) return s;
    }
  } else if (!P->gdyn[g]) {
    // static member (OGSPO::InitExp computes its exponential once, OGSPO.cpp:30-52)
    if (!P->gU[g]) {
      const int kU = p->S == 2 ? 3 : p->S * p->S;  // S > 2: the full per-point matrix
      CK(cudaMalloc(&P->gU[g], sizeof(cplx<double>) * kU * (size_t)p->npts));
      CK(qdg::launch_set_coefs(P->gcoef_d[g], P->gcp_d[g], p->d_lasers, p->laser_nt, step, p->stream));
      double *g64 = nullptr;  // the grids in binary64 (a mixed plan keeps FP32 copies)
      const size_t gb = sizeof(double) * std::max<size_t>(1, p->grids_h.size());
      CK(cudaMalloc(&g64, gb));
      if (!p->grids_h.empty())
        CK(cudaMemcpyAsync(g64, p->grids_h.data(), sizeof(double) * p->grids_h.size(), cudaMemcpyHostToDevice, p->stream));
      CK(qdg::launch_gspo_umat(reinterpret_cast<cplx<double> *>(P->gU[g]), p->S, p->npts, P->gcp_d[g], P->gcoef_d[g],
                               g64, C(P->c0 * sf), p->stream));
      CK(cudaStreamSynchronize(p->stream));
      cudaFree(g64);
    }
    CK(qdg::launch_gspo_apply<T>(x, p->S, p->npts, reinterpret_cast<const cplx<double> *>(P->gU[g]), p->stream));
  } else {
    CK(qdg::launch_set_coefs(P->gcoef_d[g], P->gcp_d[g], p->d_lasers, p->laser_nt, step, p->stream));
    CK(qdg::launch_gspo_potential<T>(x, p->S, p->npts, P->gcp_d[g], P->gcoef_d[g],
                                     reinterpret_cast<const T *>(p->d_grids), C(P->c0 * sf), p->stream));
  }
  return QDG_OK;
}

// OGSPO::Apply (OGSPO.cpp:114-139): e^{C/2} e^{B/2} e^{A} e^{B/2} e^{C/2}.
template <typename T>
qdg_status gspo_enqueue(qdg_prop *P, cplx<double> *psi, long long step) {
  qdg_plan *p = P->plan;
  cplx<T> *x;
  if (sizeof(T) == sizeof(double)) x = reinterpret_cast<cplx<T> *>(psi);
  else {
    x = reinterpret_cast<cplx<T> *>(P->k0);
    CK(qdg::launch_convert<T>(x, psi, wf_elems(p), p->stream));
  }
  for (int i = P->ngroups - 1; i > 0; --i) {
    qdg_status s = gspo_member<T>(P, i, x, step);
    if (s != QDG_OK) return s;
  }
  for (int i = 0; i < P->ngroups; ++i) {
    qdg_status s = gspo_member<T>(P, i, x, step);
    if (s != QDG_OK) return s;
  }
  if (sizeof(T) != sizeof(double)) CK(qdg::launch_widen<T>(psi, x, wf_elems(p), p->stream));
  return QDG_OK;
}

// ---------------------------------------------------------------- Krylov
template <typename T>
qdg_status krylov_alloc(qdg_prop *P) {
  qdg_plan *p = P->plan;
  P->lzb.assign(P->kord + 1, nullptr);
  for (auto &v : P->lzb) CK(cudaMalloc(&v, sizeof(cplx<T>) * wf_elems(p)));
  CK(cudaMalloc(&P->kbuf, sizeof(cplx<T>) * wf_elems(p)));
  // Krylov scalars: Lanczos alpha, beta, |psi|, order (2 m + 2); Arnoldi H (2 m^2) and |psi|
  const size_t nks = std::max<size_t>(2 * (size_t)P->kord + 2, 2 * (size_t)P->kord * P->kord + 1);
  CK(cudaMalloc(&P->d_ks, sizeof(double) * nks));
  // stop flags [0], [1]; Arnoldi order [2]; [3] the ticket of the fused launches
  CK(cudaMalloc(&P->d_kdone, 4 * sizeof(int)));
  const int o0[4] = {0, 0, P->kord, 0};          // the reference starts at the full order
  CK(cudaMemcpy(P->d_kdone, o0, sizeof(o0), cudaMemcpyHostToDevice));
  CK(cudaMallocHost(&P->h_ks, sizeof(double) * nks));
  CK(cudaMallocHost(&P->h_kdone, sizeof(int)));
  if (sizeof(T) != sizeof(double)) CK(cudaMalloc(&P->kwide, sizeof(cplx<double>) * wf_elems(p)));
  return QDG_OK;
}

template <typename T>
qdg_status hq(qdg_prop *P, const cplx<T> *q, cplx<T> *out, long long step) {
  Epi e;
  e.out = out;
  return run_h<T>(P->plan, qdg::PM_HAPPLY, q, e);
}

// OSIL::BuildLZB / DiagLZB (src/qdlib/OSIL.cpp:83-185), FP64 scalars.
// The Lanczos recursion runs with its scalars on the device: every dot
// product is finished into P->d_ks by the last block of the launch that
// computes it (fixed summation order), the basis updates read their
// coefficient from there,
// and the reference's error estimate sets a flag that turns the remaining
// kernels of the step into no-ops.  The host reads alpha, beta and the order
// once per step for the tridiagonal eigenproblem.
// The recursion of one step as a fixed sequence of launches (captured once
// in a CUDA graph per psi buffer); results land in the pinned P->h_ks.
template <typename T>
qdg_status sil_body(qdg_prop *P, cplx<double> *psi) {
  qdg_plan *p = P->plan;
  const long long n = wf_elems(p);
  const int order = P->kord;
  std::vector<cplx<T> *> L(order);
  for (int i = 0; i < order; ++i) L[i] = reinterpret_cast<cplx<T> *>(P->lzb[i]);
  cplx<T> *buf0 = reinterpret_cast<cplx<T> *>(P->kbuf);
  double *ks = P->d_ks;
  int *done = P->d_kdone;
  const int grid = dots_grid(p);
  double w = 1.0;
  for (int d = 0; d < p->nd; ++d) w *= p->dx[d];
  Epi e;
  e.done = done;
  auto hq_if = [&](const cplx<T> *q, cplx<T> *out) {
    e.out = out;
    return run_h<T>(p, qdg::PM_HAPPLY, q, e);
  };
  qdg_status s;
  // each dot product's block partials are finished by the last block of its
  // own launch (the fused kernels), so an iteration is H q, <q|H q> -> alpha,
  // the two updates with |w|^2 -> beta, and the normalisation with the commit
  unsigned int *ticket = reinterpret_cast<unsigned int *>(done + 3);
  auto fin = [&](int mode, int slot, int it) {
    qdg::KsFinish f;
    f.grid = grid; f.S = p->S; f.mode = mode; f.slot = slot; f.order = order; f.w = w;
    f.it = it; f.dt = P->dt; f.tol = P->err;
    return f;
  };
  CK(cudaMemsetAsync(ks, 0, sizeof(double) * (2 * order + 2), p->stream));
  CK(cudaMemsetAsync(done, 0, 2 * sizeof(int), p->stream));
  CK(qdg::launch_dots_ks<double, double>(psi, psi, p->S, p->npts, p->d_partials, fin(qdg::KS_PSN, 2 * order, 0), ks,
                                         done, ticket, p->stream));
  CK(qdg::launch_convert<T>(L[0], psi, n, p->stream));
  if ((s = hq_if(L[0], L[1])) != QDG_OK) return s;
  CK(qdg::launch_dots_ks<T, T>(L[0], L[1], p->S, p->npts, p->d_partials, fin(qdg::KS_ALPHA, 0, 0), ks, done, ticket,
                               p->stream));
  CK(qdg::launch_ks_lincomb<T>(L[1], L[0], ks, 0, n, done, p->stream));
  CK(qdg::launch_dots_ks<T, T>(L[1], L[1], p->S, p->npts, p->d_partials, fin(qdg::KS_BETA, order + 0, 0), ks, done,
                               ticket, p->stream));
  CK(qdg::launch_ks_scale_commit<T>(L[1], ks, order + 0, n, done, ticket, p->stream));
  for (int it = 2; it < order; ++it) {
    if ((s = hq_if(L[it - 1], L[it])) != QDG_OK) return s;
    CK(qdg::launch_dots_ks<T, T>(L[it - 1], L[it], p->S, p->npts, p->d_partials, fin(qdg::KS_ALPHA, it - 1, it), ks,
                                 done, ticket, p->stream));
    CK(qdg::launch_ks_lincomb2_dot<T>(L[it], L[it - 1], it - 1, L[it - 2], order + it - 2, p->S, p->npts,
                                      p->d_partials, fin(qdg::KS_BETA, order + it - 1, it), ks, done, ticket,
                                      p->stream));
    CK(qdg::launch_ks_scale_commit<T>(L[it], ks, order + it - 1, n, done, ticket, p->stream));
  }
  // alpha of the last vector when the recursion ran to the full order
  if ((s = hq_if(L[order - 1], buf0)) != QDG_OK) return s;
  CK(qdg::launch_dots_ks<T, T>(L[order - 1], buf0, p->S, p->npts, p->d_partials,
                               fin(qdg::KS_ALPHA, order - 1, order), ks, done, ticket, p->stream));
  CK(cudaMemcpyAsync(P->h_ks, ks, sizeof(double) * (2 * order + 2), cudaMemcpyDeviceToHost, p->stream));
  CK(cudaMemcpyAsync(P->h_kdone, done, sizeof(int), cudaMemcpyDeviceToHost, p->stream));
  return QDG_OK;
}

template <typename T>
qdg_status sil_enqueue(qdg_prop *P, cplx<double> *psi) {
  qdg_plan *p = P->plan;
  if (p->profiling || !P->graphs_ok) return sil_body<T>(P, psi);
  if (!P->graph || P->graph_psi != psi || P->graph_stream != p->stream) {
    if (P->graph) { cudaGraphExecDestroy(P->graph); P->graph = nullptr; }
    cudaGraph_t g = nullptr;
    const long long l0 = qdg::launch_counter();
    CK(cudaStreamBeginCapture(p->stream, cudaStreamCaptureModeRelaxed));
    qdg_status s = sil_body<T>(P, psi);
    cudaError_t ce = cudaStreamEndCapture(p->stream, &g);
    const long long l1 = qdg::launch_counter();
    qdg::add_launches(-(l1 - l0));
    if (s != QDG_OK) { if (g) cudaGraphDestroy(g); return s; }
    if (ce != cudaSuccess || cudaGraphInstantiate(&P->graph, g, 0) != cudaSuccess) {
      if (g) cudaGraphDestroy(g);
      cudaGetLastError();
      P->graphs_ok = false;
      P->graph = nullptr;
      return sil_body<T>(P, psi);
    }
    cudaGraphDestroy(g);
    P->graph_launches = l1 - l0;
    P->graph_psi = psi;
    P->graph_stream = p->stream;
  }
  CK(cudaGraphLaunch(P->graph, p->stream));
  qdg::add_launches(P->graph_launches);
  return QDG_OK;
}

// OSIL::BuildLZB / DiagLZB (src/qdlib/OSIL.cpp:83-185), FP64 scalars.
// The Lanczos recursion runs with its scalars on the device: every dot
// product is finished into P->d_ks by the last block of the launch that
// computes it (fixed summation order), the basis updates read their
// coefficient from there,
// and the reference's error estimate sets a flag that turns the remaining
// kernels of the step into no-ops.  The host reads alpha, beta and the order
// once per step for the tridiagonal eigenproblem.
template <typename T>
qdg_status sil_step(qdg_prop *P, cplx<double> *psi, long long step, int *used) {
  qdg_plan *p = P->plan;
  const long long n = wf_elems(p);
  const int order = P->kord;
  if (order > qdg::kMaxKrylov) return fail(QDG_EUNSUPPORTED, "Krylov order above 64");
  CK(qdg::launch_set_coefs(p->d_coef, p->d_cp, p->d_lasers, p->laser_nt, step, p->stream));
  qdg_status s = sil_enqueue<T>(P, psi);
  if (s != QDG_OK) return s;
  CK(cudaStreamSynchronize(p->stream));
  const double *hks = P->h_ks;
  const int convorder = *P->h_kdone ? (int)hks[2 * order + 1] : order;
  if (!std::isfinite(hks[2 * order])) return fail(QDG_ENONFINITE, "Norm is not a number");
  // Z exp(c0 Lambda) Z^T e0 of the full order x order tridiagonal matrix (LapackDiag dstev)
  std::vector<double> Tm((size_t)order * order, 0.0), wv, z;
  for (int i = 0; i < order; ++i) Tm[(size_t)i * order + i] = hks[i];
  for (int i = 0; i + 1 < order; ++i) {
    Tm[(size_t)i * order + i + 1] = hks[order + i];
    Tm[(size_t)(i + 1) * order + i] = hks[order + i];
  }
  qdg::host::sym_eig(order, Tm, wv, z);
  // psi = vect[0] psi + sum_i vect[i] q_i, accumulated in FP64
  qdg::KCombine<T> kc;
  memset(&kc, 0, sizeof(kc));
  kc.m = convorder;
  for (int i = 0; i < order; ++i) {
    cd acc = 0;
    for (int k = 0; k < order; ++k) acc += z[(size_t)i * order + k] * z[k] * std::exp(P->c0 * wv[k]);
    if (i < convorder) kc.c[i] = C(acc);
    kc.q[i] = reinterpret_cast<const cplx<T> *>(P->lzb[i]);
  }
  CK(qdg::launch_kcombine<T>(psi, kc, n, p->stream));
  if (used) *used = convorder;
  return QDG_OK;
}

// OArnoldi::BuildLZB / DiagLZB / Propagate (src/qdlib/OArnoldi.cpp:86-199):
// modified Gram-Schmidt in the reference order, FP64 scalars.
// The Arnoldi recursion of one step as a fixed launch sequence with its
// scalars on the device (captured once in a CUDA graph per psi buffer);
// H, |psi| and the order land in the pinned P->h_ks / P->h_kdone.
template <typename T>
qdg_status arnoldi_body(qdg_prop *P, cplx<double> *psi) {
  qdg_plan *p = P->plan;
  const long long n = wf_elems(p);
  const int m = P->kord;
  std::vector<cplx<T> *> L(m);
  for (int i = 0; i < m; ++i) L[i] = reinterpret_cast<cplx<T> *>(P->lzb[i]);
  cplx<T> *buf0 = reinterpret_cast<cplx<T> *>(P->kbuf);
  cplx<T> *last = reinterpret_cast<cplx<T> *>(P->lzb[m]);  // spare basis slot
  double *ks = P->d_ks;
  int *done = P->d_kdone;
  int *ia = P->d_kdone + 2;
  const int grid = dots_grid(p);
  qdg::KaArgs ka;
  ka.grid = grid; ka.S = p->S; ka.m = m; ka.w = 1.0; ka.dt = P->dt; ka.conv = P->conv;
  for (int d = 0; d < p->nd; ++d) ka.w *= p->dx[d];
  Epi e;
  e.done = done;
  auto hq_if = [&](const cplx<T> *q, cplx<T> *out) {
    e.out = out;
    return run_h<T>(p, qdg::PM_HAPPLY, q, e);
  };
  qdg_status s;
  // fused launches (each dot product finished by the last block of its own
  // launch): H q, <q_0|H q>, then per Gram-Schmidt step the update together
  // with the next dot product (the last one with |w|^2), and the
  // normalisation together with the commit
  unsigned int *ticket = reinterpret_cast<unsigned int *>(done + 3);
  CK(cudaMemsetAsync(ks, 0, sizeof(double) * (2 * (size_t)m * m + 1), p->stream));
  CK(cudaMemsetAsync(done, 0, 2 * sizeof(int), p->stream));
  CK(qdg::launch_dots_ka<double, double>(psi, psi, p->S, p->npts, p->d_partials, ka, qdg::KA_PSN, 0, 0, ks, ia, done,
                                         ticket, p->stream));
  CK(qdg::launch_convert<T>(L[0], psi, n, p->stream));
  for (int it = 1; it < m; ++it) {
    if ((s = hq_if(L[it - 1], buf0)) != QDG_OK) return s;
    CK(qdg::launch_dots_ka<T, T>(L[0], buf0, p->S, p->npts, p->d_partials, ka, qdg::KA_H, 0, it - 1, ks, ia, done,
                                 ticket, p->stream));
    for (int j = 0; j <= it - 1; ++j) {  // modified Gram-Schmidt
      const bool next = j + 1 <= it - 1;
      CK(qdg::launch_ka_lincomb_dot<T>(buf0, L[j], next ? L[j + 1] : nullptr, j, p->S, p->npts, p->d_partials, ka,
                                       next ? qdg::KA_H : qdg::KA_NORM, next ? j + 1 : it, it - 1, ks, ia, done,
                                       ticket, p->stream));
    }
    CK(qdg::launch_ka_scale_commit<T>(L[it], buf0, ks, 2 * (it * m + it - 1), n, it, ia, done, ticket, p->stream));
  }
  // last column H[j][order-1] from H q_{order-1}
  qdg::KaBasis<T> kb;
  memset(&kb, 0, sizeof(kb));
  for (int i = 0; i < m; ++i) kb.q[i] = L[i];
  CK(qdg::launch_ka_select<T>(last, kb, ia, n, p->stream));
  e.done = nullptr;
  if ((s = hq_if(last, buf0)) != QDG_OK) return s;
  for (int j = 0; j < m; ++j)
    CK(qdg::launch_dots_ka<T, T>(L[j], buf0, p->S, p->npts, p->d_partials, ka, qdg::KA_LAST, j, 0, ks, ia, done,
                                 ticket, p->stream));
  CK(cudaMemcpyAsync(P->h_ks, ks, sizeof(double) * (2 * (size_t)m * m + 1), cudaMemcpyDeviceToHost, p->stream));
  CK(cudaMemcpyAsync(P->h_kdone, ia, sizeof(int), cudaMemcpyDeviceToHost, p->stream));
  return QDG_OK;
}

template <typename T>
qdg_status arnoldi_enqueue(qdg_prop *P, cplx<double> *psi) {
  qdg_plan *p = P->plan;
  if (p->profiling || !P->graphs_ok) return arnoldi_body<T>(P, psi);
  if (!P->graph || P->graph_psi != psi || P->graph_stream != p->stream) {
    if (P->graph) { cudaGraphExecDestroy(P->graph); P->graph = nullptr; }
    cudaGraph_t g = nullptr;
    const long long l0 = qdg::launch_counter();
    CK(cudaStreamBeginCapture(p->stream, cudaStreamCaptureModeRelaxed));
    qdg_status s = arnoldi_body<T>(P, psi);
    cudaError_t ce = cudaStreamEndCapture(p->stream, &g);
    const long long l1 = qdg::launch_counter();
    qdg::add_launches(-(l1 - l0));
    if (s != QDG_OK) { if (g) cudaGraphDestroy(g); return s; }
    if (ce != cudaSuccess || cudaGraphInstantiate(&P->graph, g, 0) != cudaSuccess) {
      if (g) cudaGraphDestroy(g);
      cudaGetLastError();
      P->graphs_ok = false;
      P->graph = nullptr;
      return arnoldi_body<T>(P, psi);
    }
    cudaGraphDestroy(g);
    P->graph_launches = l1 - l0;
    P->graph_psi = psi;
    P->graph_stream = p->stream;
  }
  CK(cudaGraphLaunch(P->graph, p->stream));
  qdg::add_launches(P->graph_launches);
  return QDG_OK;
}

// OArnoldi::BuildLZB / DiagLZB / Propagate (src/qdlib/OArnoldi.cpp:86-199):
// modified Gram-Schmidt in the reference order, FP64 scalars, the
// reference's order kept across steps.  Each dot product is finished on the
// device into H, the Gram-Schmidt updates read their coefficients there,
// and the underrun / error tests set flags that turn the remaining kernels
// of the step into no-ops; the host reads H once per step.
template <typename T>
qdg_status arnoldi_step(qdg_prop *P, cplx<double> *psi, long long step, int *used) {
  qdg_plan *p = P->plan;
  const long long n = wf_elems(p);
  const int m = P->kord;
  if (m > qdg::kMaxKrylov) return fail(QDG_EUNSUPPORTED, "Krylov order above 64");
  CK(qdg::launch_set_coefs(p->d_coef, p->d_cp, p->d_lasers, p->laser_nt, step, p->stream));
  qdg_status s = arnoldi_enqueue<T>(P, psi);
  if (s != QDG_OK) return s;
  CK(cudaStreamSynchronize(p->stream));
  const double *H = P->h_ks;
  const int order = *P->h_kdone;
  P->aorder = order;
  if (!std::isfinite(H[2 * m * m])) return fail(QDG_ENONFINITE, "Norm is not a number");
  std::vector<cd> HA((size_t)order * order);
  for (int i = 0; i < order; ++i)
    for (int j = 0; j < order; ++j) HA[(size_t)i * order + j] = cd(H[2 * (i * m + j)], H[2 * (i * m + j) + 1]);
  std::vector<cd> vect = qdg::host::expm_e0(order, HA, P->c0);
  qdg::KCombine<T> kc;
  memset(&kc, 0, sizeof(kc));
  kc.m = order;
  for (int i = 0; i < order; ++i) {
    kc.c[i] = C(vect[i]);
    kc.q[i] = reinterpret_cast<const cplx<T> *>(P->lzb[i]);
  }
  CK(qdg::launch_kcombine<T>(psi, kc, n, p->stream));
  if (used) *used = order;
  return QDG_OK;
}

template <typename T>
qdg_status prop_step_t(qdg_prop *P, cplx<double> *psi, long long step, int *used, bool sync) {
  qdg_plan *p = P->plan;
  if (P->kind == 1) {
    qdg_status s = P->step_grid > 0 ? cheby_step_persistent<T>(P, psi, step) : cheby_enqueue<T>(P, psi, step);
    if (s != QDG_OK) return s;
    if (sync) {
      CK(cudaMemcpyAsync(P->h_cs, P->d_cs, sizeof(qdg::ChebyState), cudaMemcpyDeviceToHost, p->stream));
      CK(cudaStreamSynchronize(p->stream));
      if (used) *used = P->h_cs->terms;
      count_body_launches(P, P->h_cs->terms, 1);
      if (P->step_grid > 0) { qdg_status sb = check_barrier(p); if (sb != QDG_OK) return sb; }
      if (P->h_cs->status == QDG_ENONFINITE) return fail(QDG_ENONFINITE, "Norm is not a number");
    }
    return QDG_OK;
  }
  if (P->kind == 2) {
    qdg_status s = gspo_enqueue<T>(P, psi, step);
    if (used) *used = 2 * P->ngroups - 1;
    if (s == QDG_OK && sync) CK(cudaStreamSynchronize(p->stream));
    return s;
  }
  if (P->kind == 3) return sil_step<T>(P, psi, step, used);
  return arnoldi_step<T>(P, psi, step, used);
}

qdg_status prop_step(qdg_prop *P, cplx<double> *psi, long long step, int *used, bool sync) {
  if (is64(P->plan)) return prop_step_t<double>(P, psi, step, used, sync);
  return prop_step_t<float>(P, psi, step, used, sync);
}

// <a|H|b> (all states, grid weights) with H applied at step 0 into the plan's scratch.
qdg_status h_expec(qdg_plan *p, const cplx<double> *a, const cplx<double> *b, cd *out) {
  std::vector<cd> d;
  qdg_status s;
  if (is64(p)) {
    cplx<double> *o = reinterpret_cast<cplx<double> *>(p->d_scratch);
    if ((s = h_apply_bulk<double>(p, b, o, 0)) != QDG_OK) return s;
    if ((s = dots<double, double>(p, a, o, d)) != QDG_OK) return s;
  } else {
    cplx<float> *o = reinterpret_cast<cplx<float> *>(p->d_scratch);
    if ((s = h_apply_bulk<float>(p, b, o, 0)) != QDG_OK) return s;
    if ((s = dots<double, float>(p, a, o, d)) != QDG_OK) return s;
  }
  *out = total(d);
  return QDG_OK;
}

// ProgEigen::ImagTimeEF (src/ProgEigen.cpp:318-409): relax each function in
// imaginary time from the same start, projecting out the functions already
// found after every step (OProjection::Apply, OProjection.cpp:133-149),
// normalising, until |1 - <psi_old|psi>| <= convergence; then DiagBasis
// (ProgEigen.cpp:94-138) diagonalises H in the basis found.
qdg_status eigen_imag(qdg_prop *P, const double *psi_init, int nef, int maxsteps, double conv, int diag,
                      double *efs, double *e_raw, double *e_diag, int32_t *steps) {
  qdg_plan *p = P->plan;
  const long long n = wf_elems(p);
  const size_t bytes = sizeof(cplx<double>) * (size_t)n;
  std::vector<cplx<double> *> bufs;
  auto cleanup = [&](qdg_status st) {
    cudaStreamSynchronize(p->stream);
    for (auto *b : bufs) cudaFree(b);
    return st;
  };
  for (int i = 0; i < nef + 3; ++i) {  // nef functions, psi, old, init
    cplx<double> *b = nullptr;
    if (cudaMalloc(&b, bytes) != cudaSuccess) return cleanup(fail(QDG_ENOMEM, "device allocation failed"));
    bufs.push_back(b);
  }
  cplx<double> *psi = bufs[nef], *old = bufs[nef + 1], *init = bufs[nef + 2];
  qdg_status s;
  std::vector<cd> d;
#define ECHK(expr) do { if ((s = (expr)) != QDG_OK) return cleanup(s); } while (0)
#define ECUDA(expr) do { if ((expr) != cudaSuccess) return cleanup(fail(QDG_ECUDA, #expr)); } while (0)
  ECUDA(cudaMemcpyAsync(init, psi_init, bytes, cudaMemcpyHostToDevice, p->stream));
  ECHK((dots<double, double>(p, init, init, d)));
  const double n0 = std::sqrt(total(d).real());
  if (!(n0 > 0) || !std::isfinite(n0)) return cleanup(fail(QDG_ENONFINITE, "Norm is not a number"));
  ECUDA(qdg::launch_lincomb<double>(init, (const cplx<double> *)nullptr, cplx<double>{1.0 / n0, 0}, cplx<double>{0, 0}, n, p->stream));
  for (int i = 0; i < nef; ++i) {
    ECUDA(cudaMemcpyAsync(psi, init, bytes, cudaMemcpyDeviceToDevice, p->stream));
    int st = 0;
    double diff = 1;
    while (st < maxsteps && diff > conv) {
      ECUDA(cudaMemcpyAsync(old, psi, bytes, cudaMemcpyDeviceToDevice, p->stream));
      int used = 0;
      ECHK(prop_step(P, psi, st, &used, true));
      if (i > 0) {
        std::vector<cd> c(i);
        for (int j = 0; j < i; ++j) {  // all overlaps against the propagated psi first
          ECHK((dots<double, double>(p, bufs[j], psi, d)));
          c[j] = total(d);
        }
        for (int j = 0; j < i; ++j)
          ECUDA(qdg::launch_lincomb<double>(psi, bufs[j], cplx<double>{1, 0}, C(-c[j]), n, p->stream));
      }
      ECHK((dots<double, double>(p, psi, psi, d)));
      const double nr = std::sqrt(total(d).real());
      if (!std::isfinite(nr) || !(nr > 0)) return cleanup(fail(QDG_ENONFINITE, "Norm is not a number"));
      ECUDA(qdg::launch_lincomb<double>(psi, (const cplx<double> *)nullptr, cplx<double>{1.0 / nr, 0}, cplx<double>{0, 0}, n, p->stream));
      ECHK((dots<double, double>(p, old, psi, d)));
      diff = std::abs(1.0 - total(d));
      ++st;
    }
    ECUDA(cudaMemcpyAsync(bufs[i], psi, bytes, cudaMemcpyDeviceToDevice, p->stream));
    cd e;
    ECHK(h_expec(p, psi, psi, &e));
    e_raw[i] = e.real();
    if (steps) steps[i] = st;
  }
  if (diag) {
    std::vector<double> Sm((size_t)nef * nef, 0.0), w, z;
    for (int i = 0; i < nef; ++i) {
      for (int j = 0; j < i; ++j) {
        cd v;
        ECHK(h_expec(p, bufs[i], bufs[j], &v));
        Sm[(size_t)j * nef + i] = Sm[(size_t)i * nef + j] = v.real();
      }
      Sm[(size_t)i * nef + i] = e_raw[i];
    }
    qdg::host::sym_eig(nef, Sm, w, z);
    for (int i = 0; i < nef; ++i) {
      e_diag[i] = w[i];
      if (!efs) continue;
      ECUDA(qdg::launch_lincomb<double>(psi, bufs[0], cplx<double>{0, 0}, cplx<double>{z[(size_t)0 * nef + i], 0}, n, p->stream));
      for (int j = 1; j < nef; ++j)
        ECUDA(qdg::launch_lincomb<double>(psi, bufs[j], cplx<double>{1, 0}, cplx<double>{z[(size_t)j * nef + i], 0}, n, p->stream));
      ECUDA(cudaMemcpyAsync(efs + 2 * (size_t)i * n, psi, bytes, cudaMemcpyDeviceToHost, p->stream));
    }
  } else {
    for (int i = 0; i < nef; ++i) {
      e_diag[i] = e_raw[i];
      if (efs) ECUDA(cudaMemcpyAsync(efs + 2 * (size_t)i * n, bufs[i], bytes, cudaMemcpyDeviceToHost, p->stream));
    }
  }
#undef ECHK
#undef ECUDA
  return cleanup(QDG_OK);
}

// A propagator on an FP64 twin of the caller's plan queues its work on the
// caller's stream, so it stays ordered with the caller's other calls.
void sync_twin(qdg_prop *P) {
  if (!P->twin || P->twin->stream == P->user->stream) return;
  if (P->twin->own_stream) {
    cudaStreamSynchronize(P->twin->stream);
    cudaStreamDestroy(P->twin->stream);
    P->twin->own_stream = false;
  }
  P->twin->stream = P->user->stream;
}

}  // namespace

// ====================================================================== ABI
extern "C" {

const char *qdg_last_error(void) { return g_last_error.c_str(); }
int32_t qdg_abi_version(void) { return QDG_ABI_VERSION; }

qdg_status qdg_plan_create(const qdg_hplan_desc *desc, int32_t precision, qdg_plan **out) {
  if (!desc || !out) return fail(QDG_EINVAL, "null argument");
  *out = nullptr;
  if (precision != QDG_PREC_FP64 && precision != QDG_PREC_MIXED && precision != QDG_PREC_DF64)
    return fail(QDG_EINVAL, "unknown precision");
  const qdg_grid &g = desc->grid;
  if (g.ndims < 1 || g.ndims > QDG_MAX_DIMS) return fail(QDG_EINVAL, "invalid number of grid dimensions");
  if (desc->nstates < 1 || desc->nstates > qdg::kMaxStates) return fail(QDG_EUNSUPPORTED, "number of states outside 1..8");
  if (desc->nterms < 1 || !desc->terms) return fail(QDG_EINVAL, "Hamiltonian is empty");
  int dev = 0;
  CK(cudaGetDevice(&dev));
  qdg_plan *p = new qdg_plan();
  p->grid = g;
  p->S = desc->nstates;
  p->nd = g.ndims;
  p->precision = precision;
  p->csize = is64(p) ? sizeof(cplx<double>) : sizeof(cplx<float>);
  long long stride = 1;
  for (int d = 0; d < g.ndims; ++d) {
    if (g.n[d] < 2) { free_plan(p); return fail(QDG_EINVAL, "Zero points grid defined"); }
    if (g.xmax[d] - g.xmin[d] <= 0) { free_plan(p); return fail(QDG_EINVAL, "Zero length grid defined"); }
    p->dx[d] = (g.xmax[d] - g.xmin[d]) / double(g.n[d] - 1);          // GridSystem::Dx
    p->dk[d] = (2 * M_PI) / (g.xmax[d] - g.xmin[d] + p->dx[d]);        // Kspace::Dk
    p->dim[d].n = g.n[d];
    p->dim[d].stride = stride;
    // the autotuner's schedule for this line length, else the greedy order
    // (largest radices first: 256 = 16 x 16, 1024 = 16 x 16 x 4, 384 = 16 x 8 x 3);
    // other prime factors become direct-DFT stages of the graph path's
    // transforms (FFTW takes any N, src/fft/fft.cpp:98-122)
    if (!qdg::schedule_radix(qdg::SCHED_PLAN, g.n[d], precision, p->dim[d].rp)) {
      if (!qdg::any_radix(g.n[d], p->dim[d].rp)) {
        free_plan(p);
        return fail(QDG_EUNSUPPORTED, "grid size has more than 16 prime factors");
      }
      p->generic_fft = true;
    }
    stride *= g.n[d];
  }
  p->npts = stride;
  p->terms.assign(desc->terms, desc->terms + desc->nterms);
  p->ngrids = desc->ngrids;
  p->nlasers = desc->nlasers;
  p->laser_nt = desc->laser_nt;
  for (auto &t : p->terms) {
    if (t.row < 0 || t.col < 0 || t.row >= p->S || t.col >= p->S) { free_plan(p); return fail(QDG_EINVAL, "matrix element outside the states"); }
    if (t.kind == QDG_TERM_KINETIC) {
      if (t.row != t.col) { free_plan(p); return fail(QDG_EUNSUPPORTED, "kinetic operator off the diagonal"); }
      for (int d = 0; d < p->nd; ++d)
        if (!(t.mass[d] > 0)) { free_plan(p); return fail(QDG_EINVAL, "Zero mass defined"); }
      // HOFD::_CheckSetup (HOFD.h:82-89)
      if (t.fd_order != 0 && (t.fd_order < 2 || t.fd_order > 2 * qdg::kMaxFdHalf || t.fd_order % 2 != 0)) {
        free_plan(p); return fail(QDG_EINVAL, "Invalid order of FD derivative");
      }
      if (t.fd_order != 0 && (t.flags & 1) && (p->nd != 1 || p->dim[0].n <= t.fd_order / 2)) {
        free_plan(p); return fail(QDG_EUNSUPPORTED, "HOFD with pbc needs a one-dimensional grid longer than order/2");
      }
    } else if (t.kind == QDG_TERM_HOFD) {
      if (t.row != t.col) { free_plan(p); return fail(QDG_EUNSUPPORTED, "GridHOFD off the diagonal"); }
      if (t.fd_order < 2 || t.fd_order > 2 * qdg::kMaxFdHalf || t.fd_order % 2 != 0) {
        free_plan(p); return fail(QDG_EINVAL, "Invalid order of FD derivative");
      }
      if (t.laser < -1 || t.laser >= p->nd) { free_plan(p); return fail(QDG_EINVAL, "Invalid number of active dimension"); }
      for (int d = 0; d < p->nd; ++d) {
        if ((t.laser < 0 || t.laser == d) && p->dim[d].n < t.fd_order) {
          free_plan(p); return fail(QDG_EUNSUPPORTED, "GridHOFD needs lines of at least order points");
        }
        if ((t.flags & 4) && t.mass[d] == 0) { free_plan(p); return fail(QDG_EINVAL, "Zero mass defined"); }
      }
    } else if (t.kind == QDG_TERM_GMAT) {
      if (t.row != t.col) { free_plan(p); return fail(QDG_EUNSUPPORTED, "GridGMat off the diagonal"); }
      const int ne = p->nd * (p->nd + 1) / 2;
      if (t.grid < 0 || t.grid + ne > p->ngrids || !desc->grid_data) { free_plan(p); return fail(QDG_EINVAL, "G-matrix grid index out of range"); }
      for (int k = 0; k < ne; ++k)
        if (((t.flags >> (2 * k)) & 3) == 3) { free_plan(p); return fail(QDG_EINVAL, "bad G-matrix element source"); }
    } else if (t.kind == QDG_TERM_NAC) {
      if (t.grid < 0 || t.grid + p->nd > p->ngrids || !desc->grid_data) { free_plan(p); return fail(QDG_EINVAL, "NACME grid index out of range"); }
      if (!(t.mass[0] > 0)) { free_plan(p); return fail(QDG_EINVAL, "Zero mass defined"); }
    } else if (t.kind == QDG_TERM_POTENTIAL || t.kind == QDG_TERM_DIPOLE || t.kind == QDG_TERM_GOBBLER) {
      if (t.grid < 0 || t.grid >= p->ngrids || !desc->grid_data) { free_plan(p); return fail(QDG_EINVAL, "potential grid index out of range"); }
      if (t.kind == QDG_TERM_GOBBLER && t.row != t.col) { free_plan(p); return fail(QDG_EUNSUPPORTED, "Gobbler off the diagonal"); }
      if (t.kind == QDG_TERM_DIPOLE && (t.laser < 0 || t.laser >= p->nlasers || p->laser_nt < 1 || !desc->laser_data)) {
        free_plan(p); return fail(QDG_EINVAL, "dipole operator without a laser field");
      }
    } else { free_plan(p); return fail(QDG_EUNSUPPORTED, "unknown term kind"); }
  }
  if (p->ngrids > 0) p->grids_h.assign(desc->grid_data, desc->grid_data + (long long)p->ngrids * p->npts);
  if (p->nlasers > 0) p->lasers_h.assign(desc->laser_data, desc->laser_data + (long long)p->nlasers * p->laser_nt);
  for (double v : p->grids_h) if (!std::isfinite(v)) { free_plan(p); return fail(QDG_EINVAL, "non-finite value in a potential grid"); }
  // OMultistate: the "nonhermitian" parameter, or elements at both (i, j) and
  // (j, i), switch the hermitian copy off (OMultistate.cpp:52-53,83-85)
  p->hermitian = !desc->nonhermitian;
  for (auto &a : p->terms)
    for (auto &b : p->terms)
      if (a.row != a.col && a.row == b.col && a.col == b.row) p->hermitian = false;
  // one kinetic form per plan: FFT, finite differences (one order and
  // boundary rule) or the G-matrix (one per state)
  {
    bool fft = false, fd = false, gm = false;
    for (int st = 0; st < qdg::kMaxStates; ++st) p->gm_base[st] = -1;
    for (auto &t : p->terms) {
      if (t.kind == QDG_TERM_KINETIC && t.fd_order == 0) fft = true;
      if ((t.kind == QDG_TERM_KINETIC && t.fd_order != 0) || t.kind == QDG_TERM_HOFD) {
        const int mode = t.kind == QDG_TERM_HOFD ? 1 : 0;
        const int deriv = (t.kind == QDG_TERM_HOFD && (t.flags & 2)) ? 1 : 2;
        if (fd && (t.fd_order != p->fd_order || (t.flags & 1) != p->fd_pbc || mode != p->fd_mode ||
                   deriv != p->fd_deriv)) {
          free_plan(p);
          return fail(QDG_EUNSUPPORTED, "finite-difference terms of different form, order, derivative or boundaries");
        }
        fd = true;
        p->fd_order = t.fd_order;
        p->fd_pbc = t.flags & 1;
        p->fd_mode = mode;
        p->fd_deriv = deriv;
        if (mode == 0) {
          for (int d = 0; d < p->nd; ++d)  // HOFD.h:136-138: 1/dx^2 * 1 * (-1/(2 m_d))
            p->fd_h[t.row][d] += 1. / (p->dx[d] * p->dx[d]) * 1.0 * (-1. / 2. / t.mass[d]);
        } else {
          // OGridHOFD.cpp:74-91 and HOFD.h:190: 1/dx^deriv * 1 * factor, factor
          // -1/(2 m) of the last dimension's mass for every dimension, else 1
          const double factor = (t.flags & 4) ? -1. / (2 * t.mass[p->nd - 1]) : 1.0;
          for (int d = 0; d < p->nd; ++d)
            if (t.laser < 0 || t.laser == d) p->fd_h[t.row][d] += 1. / std::pow(p->dx[d], deriv) * 1.0 * factor;
        }
      }
      if (t.kind == QDG_TERM_GMAT) {
        if (p->gm_base[t.row] >= 0) { free_plan(p); return fail(QDG_EUNSUPPORTED, "two GridGMat operators on one state"); }
        gm = true;
        p->gm_base[t.row] = t.grid;
        const int ne = p->nd * (p->nd + 1) / 2;
        for (int k = 0; k < ne; ++k)
          if ((t.flags >> (2 * k)) & 3) p->gm_mask[t.row] |= 1u << k;
      }
    }
    if ((int)fft + (int)fd + (int)gm > 1) {
      free_plan(p); return fail(QDG_EUNSUPPORTED, "one kinetic form per plan: FFT, HOFD or GridGMat");
    }
    p->kin_form = fd ? KIN_FD : gm ? KIN_GMAT : KIN_FFT;
  }
  for (auto &t : p->terms) {
    if (t.kind != QDG_TERM_NAC) continue;
    const double c = 0.5 * (t.sign == 0 ? 1.0 : t.sign) / t.mass[0];  // PreFactor(0.5 sign / mass)
    p->nac.push_back({t.row, t.col, t.grid, c});
    if (p->hermitian && t.row != t.col) p->nac.push_back({t.col, t.row, t.grid, c});
  }
  compute_erange(p);
  cudaDeviceProp prop;
  if (cudaGetDeviceProperties(&prop, dev) != cudaSuccess) { free_plan(p); return fail(QDG_ECUDA, "cudaGetDeviceProperties failed"); }
  p->sm_count = prop.multiProcessorCount;
  for (int d = 0; d < p->nd; ++d) {
    p->dim[d].TW_k = choose_tw(p, d, 1);
    p->dim[d].TW_e = choose_tw(p, d, p->S);
  }
  qdg_status s = build_couplings(p, [](const qdg_hterm &) { return true; }, p->cp_h);
  if (s != QDG_OK) { free_plan(p); return s; }
  auto cleanup = [&](qdg_status st) { free_plan(p); return st; };
  if (cudaStreamCreateWithFlags(&p->stream, cudaStreamNonBlocking) != cudaSuccess) return cleanup(fail(QDG_ECUDA, "stream"));
  p->own_stream = true;
  if (cudaMalloc(&p->d_cp, sizeof(qdg::Couplings)) != cudaSuccess ||
      cudaMemcpy(p->d_cp, &p->cp_h, sizeof(qdg::Couplings), cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMalloc(&p->d_coef, sizeof(double) * qdg::kMaxCouplings) != cudaSuccess)
    return cleanup(fail(QDG_ENOMEM, "device allocation failed"));
  const size_t lbytes = sizeof(double) * std::max<size_t>(1, p->lasers_h.size());
  if (cudaMalloc(&p->d_lasers, lbytes) != cudaSuccess) return cleanup(fail(QDG_ENOMEM, "device allocation failed"));
  if (!p->lasers_h.empty() && cudaMemcpy(p->d_lasers, p->lasers_h.data(), lbytes, cudaMemcpyHostToDevice) != cudaSuccess)
    return cleanup(fail(QDG_ECUDA, "laser upload"));
  p->max_parts = std::max(4096, 2 * qdg::kMaxStates * 2 * p->sm_count);
  if (cudaMalloc(&p->d_partials, sizeof(double) * 2 * qdg::kMaxStates * p->max_parts) != cudaSuccess ||
      cudaMallocHost(&p->h_partials, sizeof(double) * 2 * qdg::kMaxStates * p->max_parts) != cudaSuccess)
    return cleanup(fail(QDG_ENOMEM, "device allocation failed"));
  if (cudaMalloc(&p->d_bar, sizeof(qdg::GridBarrier)) != cudaSuccess ||
      cudaMemset(p->d_bar, 0, sizeof(qdg::GridBarrier)) != cudaSuccess ||
      cudaMallocHost(&p->h_bar, sizeof(qdg::GridBarrier)) != cudaSuccess)
    return cleanup(fail(QDG_ENOMEM, "device allocation failed"));
  s = is64(p) ? upload_tables<double>(p) : upload_tables<float>(p);
  if (s != QDG_OK) return cleanup(s);
  *out = p;
  return QDG_OK;
}

qdg_status qdg_plan_destroy(qdg_plan *plan) {
  if (!plan) return QDG_OK;
  cudaStreamSynchronize(plan->stream);
  if (plan->children > 0) {
    plan->destroy_pending = true;
    return QDG_OK;
  }
  free_plan(plan);
  return QDG_OK;
}

qdg_status qdg_plan_erange(const qdg_plan *plan, double emax[2], double emin[2]) {
  if (!plan || !emax || !emin) return fail(QDG_EINVAL, "null argument");
  emax[0] = plan->emax.real(); emax[1] = plan->emax.imag();
  emin[0] = plan->emin.real(); emin[1] = plan->emin.imag();
  return QDG_OK;
}

qdg_status qdg_plan_set_stream(qdg_plan *plan, void *cuda_stream) {
  if (!plan) return fail(QDG_EINVAL, "null plan");
  CK(cudaStreamSynchronize(plan->stream));
  if (cuda_stream) {
    if (plan->own_stream) cudaStreamDestroy(plan->stream);
    plan->stream = (cudaStream_t)cuda_stream;
    plan->own_stream = false;
  }
  return QDG_OK;
}

qdg_status qdg_plan_synchronize(qdg_plan *plan) {
  if (!plan) return fail(QDG_EINVAL, "null plan");
  CK(cudaStreamSynchronize(plan->stream));
  return QDG_OK;
}

qdg_status qdg_wf_create(qdg_plan *plan, qdg_wf **out) {
  if (!plan || !out) return fail(QDG_EINVAL, "null argument");
  qdg_wf *w = new qdg_wf();
  w->plan = plan;
  if (cudaMalloc(&w->d, sizeof(cplx<double>) * wf_elems(plan)) != cudaSuccess) {
    delete w;
    return fail(QDG_ENOMEM, "device allocation failed");
  }
  cudaMemsetAsync(w->d, 0, sizeof(cplx<double>) * wf_elems(plan), plan->stream);
  plan->children++;
  *out = w;
  return QDG_OK;
}

qdg_status qdg_wf_destroy(qdg_wf *wf) {
  if (!wf) return QDG_OK;
  qdg_plan *p = wf->plan;
  cudaStreamSynchronize(p->stream);
  cudaFree(wf->d);
  delete wf;
  release_child(p);
  return QDG_OK;
}

qdg_status qdg_wf_upload(qdg_wf *wf, const double *host) {
  if (!wf || !host) return fail(QDG_EINVAL, "null argument");
  CK(cudaMemcpyAsync(wf->d, host, sizeof(cplx<double>) * wf_elems(wf->plan), cudaMemcpyHostToDevice, wf->plan->stream));
  CK(cudaStreamSynchronize(wf->plan->stream));
  return QDG_OK;
}

qdg_status qdg_wf_download(const qdg_wf *wf, double *host) {
  if (!wf || !host) return fail(QDG_EINVAL, "null argument");
  CK(cudaMemcpyAsync(host, wf->d, sizeof(cplx<double>) * wf_elems(wf->plan), cudaMemcpyDeviceToHost, wf->plan->stream));
  CK(cudaStreamSynchronize(wf->plan->stream));
  return QDG_OK;
}

qdg_status qdg_wf_copy(qdg_wf *dst, const qdg_wf *src) {
  if (!dst || !src || dst->plan != src->plan) return fail(QDG_EINVAL, "wave functions of different plans");
  CK(cudaMemcpyAsync(dst->d, src->d, sizeof(cplx<double>) * wf_elems(dst->plan), cudaMemcpyDeviceToDevice, dst->plan->stream));
  return QDG_OK;
}

qdg_status qdg_h_apply(qdg_plan *plan, const qdg_wf *in, qdg_wf *out, int64_t step) {
  if (!plan || !in || !out || in->plan != plan || out->plan != plan) return fail(QDG_EINVAL, "bad arguments");
  if (in == out) return fail(QDG_EINVAL, "H apply needs distinct input and output");
  qdg_status s;
  if (is64(plan)) {
    s = h_apply_bulk<double>(plan, in->d, out->d, step);
  } else {
    cplx<float> *o = reinterpret_cast<cplx<float> *>(plan->d_scratch);
    s = h_apply_bulk<float>(plan, in->d, o, step);
    if (s == QDG_OK) CK(qdg::launch_widen<float>(out->d, o, wf_elems(plan), plan->stream));
  }
  if (s != QDG_OK) return s;
  CK(cudaStreamSynchronize(plan->stream));
  return QDG_OK;
}

// ---- expectation filters (FiltersList expec / expeconly) -----------------
namespace {
struct DevBuf {
  void *p = nullptr;
  ~DevBuf() { if (p) cudaFree(p); }
};

int expec_grid(const qdg_plan *p) {
  const long long items = (p->npts * p->S + 255) / 256;
  return (int)std::max<long long>(1, std::min<long long>(items, 4LL * p->sm_count));
}

// sum w |psi|^2 and sum |psi|^2 (weights: a binary64 device grid, or the coordinate)
qdg_status expec_point(qdg_plan *p, const qdg_wf *psi, const double *grid, int dim, double scale, double &ws,
                       double &ns) {
  const int G = expec_grid(p);
  DevBuf part;
  CK(cudaMalloc(&part.p, sizeof(double) * 2 * G));
  qdg::PointExpecArgs a;
  memset(&a, 0, sizeof(a));
  a.psi = psi->d;
  a.npts = p->npts;
  a.S = p->S;
  a.grid = grid;
  a.nd = p->nd;
  a.dim = dim;
  a.scale = scale;
  for (int d = 0; d < p->nd; ++d) {
    a.stride[d] = p->dim[d].stride;
    a.n[d] = p->dim[d].n;
    a.xmin[d] = p->grid.xmin[d];
    a.dx[d] = p->dx[d];
  }
  a.partials = static_cast<double *>(part.p);
  CK(qdg::launch_point_expec(a, G, p->stream));
  std::vector<double> h(2 * G);
  CK(cudaMemcpyAsync(h.data(), part.p, sizeof(double) * 2 * G, cudaMemcpyDeviceToHost, p->stream));
  CK(cudaStreamSynchronize(p->stream));
  ws = 0;
  ns = 0;
  for (int b = 0; b < G; ++b) { ws += h[2 * b]; ns += h[2 * b + 1]; }
  return QDG_OK;
}

// sum over the lines of dimension d of sum_k w[s][k] |FFT_d psi (k)|^2
qdg_status expec_spectral(qdg_plan *p, const qdg_wf *psi, int d, const std::vector<double> &w, double &out) {
  const int N = p->dim[d].n;
  if (qdg::spectral_expec_smem(N) > 227 * 1024) return fail(QDG_EUNSUPPORTED, "line too long for the filter transform");
  std::vector<cplx<double>> tw(N);
  const long double pi = 3.141592653589793238462643383279502884L;
  for (int m = 0; m < N; ++m) {
    const long double ang = -2.0L * pi * (long double)m / (long double)N;
    tw[m] = cplx<double>{(double)cosl(ang), (double)sinl(ang)};
  }
  const long long lines = (p->npts / N) * p->S;
  const int G = (int)std::max<long long>(1, std::min<long long>(lines, 4LL * p->sm_count));
  DevBuf dtw, dw, part;
  CK(cudaMalloc(&dtw.p, sizeof(cplx<double>) * N));
  CK(cudaMalloc(&dw.p, sizeof(double) * w.size()));
  CK(cudaMalloc(&part.p, sizeof(double) * G));
  CK(cudaMemcpyAsync(dtw.p, tw.data(), sizeof(cplx<double>) * N, cudaMemcpyHostToDevice, p->stream));
  CK(cudaMemcpyAsync(dw.p, w.data(), sizeof(double) * w.size(), cudaMemcpyHostToDevice, p->stream));
  qdg::SpecExpecArgs a;
  memset(&a, 0, sizeof(a));
  a.psi = psi->d;
  a.npts = p->npts;
  a.S = p->S;
  a.N = N;
  a.es = p->dim[d].stride;
  a.rp = p->dim[d].rp;
  a.tw = static_cast<const cplx<double> *>(dtw.p);
  a.w = static_cast<const double *>(dw.p);
  a.partials = static_cast<double *>(part.p);
  CK(qdg::launch_spectral_expec(a, G, p->stream));
  std::vector<double> h(G);
  CK(cudaMemcpyAsync(h.data(), part.p, sizeof(double) * G, cudaMemcpyDeviceToHost, p->stream));
  CK(cudaStreamSynchronize(p->stream));
  out = 0;
  for (int b = 0; b < G; ++b) out += h[b];
  return QDG_OK;
}

qdg_status expec_check(const qdg_plan *plan, const qdg_wf *psi, const double *out) {
  if (!plan || !psi || !out || psi->plan != plan) return fail(QDG_EINVAL, "bad arguments");
  return QDG_OK;
}

// Kinetic operators without a k-space table (HOFD, GridGMat): Re <psi|T psi>
// / <psi|psi> with T psi from the binary64 kinetic kernels on the binary64
// psi (twiddles and G grids uploaded in binary64 for the call on a mixed plan).
qdg_status expec_kinetic_direct(qdg_plan *p, const qdg_wf *psi, double *out) {
  const int nd = p->nd;
  const size_t n = (size_t)p->npts * p->S;
  DevBuf Pb[QDG_MAX_DIMS], Db[QDG_MAX_DIMS], twb[QDG_MAX_DIMS], gb;
  const cplx<double> *tw[QDG_MAX_DIMS] = {};
  cplx<double> *D[QDG_MAX_DIMS] = {}, *P[QDG_MAX_DIMS] = {};
  const int nP = p->kin_form == KIN_FD ? 1 : nd;
  for (int d = 0; d < nP; ++d) {
    CK(cudaMalloc(&Pb[d].p, sizeof(cplx<double>) * n));
    P[d] = static_cast<cplx<double> *>(Pb[d].p);
  }
  const double *grids = is64(p) ? static_cast<const double *>(p->d_grids) : nullptr;
  if (p->kin_form == KIN_GMAT) {
    const long double pi = 3.141592653589793238462643383279502884L;
    for (int d = 0; d < nd; ++d) {
      CK(cudaMalloc(&Db[d].p, sizeof(cplx<double>) * n));
      D[d] = static_cast<cplx<double> *>(Db[d].p);
      if (is64(p)) {
        tw[d] = static_cast<const cplx<double> *>(p->dim[d].tw);
      } else {
        const int N = p->dim[d].n;
        std::vector<cplx<double>> h(N);
        for (int m = 0; m < N; ++m) {
          const long double ang = -2.0L * pi * (long double)m / (long double)N;
          h[m] = cplx<double>{(double)cosl(ang), (double)sinl(ang)};
        }
        CK(cudaMalloc(&twb[d].p, sizeof(cplx<double>) * N));
        CK(cudaMemcpyAsync(twb[d].p, h.data(), sizeof(cplx<double>) * N, cudaMemcpyHostToDevice, p->stream));
        tw[d] = static_cast<const cplx<double> *>(twb[d].p);
      }
    }
    if (!is64(p)) {
      CK(cudaMalloc(&gb.p, sizeof(double) * p->grids_h.size()));
      CK(cudaMemcpyAsync(gb.p, p->grids_h.data(), sizeof(double) * p->grids_h.size(), cudaMemcpyHostToDevice, p->stream));
      grids = static_cast<const double *>(gb.p);
    }
  }
  const void *bufs[2] = {nullptr, nullptr};
  qdg_status s = run_kin_tablefree<double>(p, psi->d, nullptr, nullptr, 0, bufs, tw, grids, D, P, is64(p) ? 0 : 1);
  if (s != QDG_OK) return s;
  std::vector<cd> dd;
  double num = 0;
  for (int d = 0; d < nP; ++d) {
    if ((s = dots<double, double>(p, psi->d, P[d], dd)) != QDG_OK) return s;
    num += total(dd).real();
  }
  if ((s = dots<double, double>(p, psi->d, psi->d, dd)) != QDG_OK) return s;
  *out = num / total(dd).real();
  return QDG_OK;
}
}  // namespace

qdg_status qdg_expec_position(qdg_plan *plan, const qdg_wf *psi, int32_t dim, double scale, double *out) {
  qdg_status s = expec_check(plan, psi, out);
  if (s != QDG_OK) return s;
  if (dim >= plan->nd) return fail(QDG_EINVAL, "Dimension for position operator exceeds dimensions of Wavefunction");
  double ws, ns;
  if ((s = expec_point(plan, psi, nullptr, dim, scale, ws, ns)) != QDG_OK) return s;
  *out = ws / ns;
  return QDG_OK;
}

qdg_status qdg_expec_momentum(qdg_plan *plan, const qdg_wf *psi, int32_t dim, double factor, double *out) {
  qdg_status s = expec_check(plan, psi, out);
  if (s != QDG_OK) return s;
  if (dim >= plan->nd) return fail(QDG_EINVAL, "Dimension for momentum operator exceeds dimensions of Wavefunction");
  double ws, ns, num = 0;
  if ((s = expec_point(plan, psi, nullptr, 0, 1.0, ws, ns)) != QDG_OK) return s;
  for (int d = 0; d < plan->nd; ++d) {
    if (dim >= 0 && d != dim) continue;
    // Kspace::Init1Dddx (Kspace.cpp:60-96): k_j = j dk below the middle,
    // (j - N) dk above it, both parities; OGridNabla divides by N
    const int N = plan->dim[d].n;
    std::vector<double> w((size_t)plan->S * N);
    for (int st = 0; st < plan->S; ++st)
      for (int j = 0; j < N; ++j) {
        const double k = (j < (N + 1) / 2 ? (double)j : (double)(j - N)) * plan->dk[d];
        w[(size_t)st * N + j] = factor * k / (double)N;
      }
    double v;
    if ((s = expec_spectral(plan, psi, d, w, v)) != QDG_OK) return s;
    num += v;
  }
  *out = num / ns;
  return QDG_OK;
}

qdg_status qdg_expec_kinetic(qdg_plan *plan, const qdg_wf *psi, double *out) {
  qdg_status s = expec_check(plan, psi, out);
  if (s != QDG_OK) return s;
  if (plan->kin_form != KIN_FFT) return expec_kinetic_direct(plan, psi, out);
  double ws, ns, num = 0;
  if ((s = expec_point(plan, psi, nullptr, 0, 1.0, ws, ns)) != QDG_OK) return s;
  for (int d = 0; d < plan->nd; ++d) {
    // OGridNablaSq: k^2 / (2 m_d) of every kinetic term on the state, 1/N of the transform pair
    const int N = plan->dim[d].n;
    std::vector<double> kf(plan->S, 0.0);
    bool any = false;
    for (auto &t : plan->terms)
      if (t.kind == QDG_TERM_KINETIC) { kf[t.row] += plan->dk[d] * plan->dk[d] / (2.0 * t.mass[d]) / N; any = true; }
    if (!any) continue;
    std::vector<double> w((size_t)plan->S * N);
    for (int st = 0; st < plan->S; ++st)
      for (int j = 0; j < N; ++j) {
        const double kq = std::min(j, N - j);
        w[(size_t)st * N + j] = kf[st] * kq * kq;
      }
    double v;
    if ((s = expec_spectral(plan, psi, d, w, v)) != QDG_OK) return s;
    num += v;
  }
  *out = num / ns;
  return QDG_OK;
}

qdg_status qdg_expec_grid(qdg_plan *plan, const qdg_wf *psi, int32_t grid, double *out) {
  qdg_status s = expec_check(plan, psi, out);
  if (s != QDG_OK) return s;
  if (grid < 0 || grid >= plan->ngrids) return fail(QDG_EINVAL, "grid index out of range");
  DevBuf g;
  CK(cudaMalloc(&g.p, sizeof(double) * plan->npts));
  CK(cudaMemcpyAsync(g.p, plan->grids_h.data() + (size_t)grid * plan->npts, sizeof(double) * plan->npts,
                     cudaMemcpyHostToDevice, plan->stream));
  double ws, ns;
  if ((s = expec_point(plan, psi, static_cast<const double *>(g.p), 0, 1.0, ws, ns)) != QDG_OK) return s;
  *out = ws / ns;
  return QDG_OK;
}

qdg_status qdg_expec_projection(qdg_plan *plan, const qdg_wf *psi, const double *const *funcs, int32_t nfun,
                                double *out) {
  qdg_status s = expec_check(plan, psi, out);
  if (s != QDG_OK) return s;
  if (nfun < 0 || (nfun > 0 && !funcs)) return fail(QDG_EINVAL, "bad projection functions");
  const size_t n = (size_t)plan->npts * plan->S;
  DevBuf f;
  CK(cudaMalloc(&f.p, sizeof(cplx<double>) * n));
  std::vector<cd> d;
  double acc = 0;
  for (int k = 0; k < nfun; ++k) {
    if (!funcs[k]) return fail(QDG_EINVAL, "null projection function");
    CK(cudaMemcpyAsync(f.p, funcs[k], sizeof(cplx<double>) * n, cudaMemcpyHostToDevice, plan->stream));
    if ((s = dots<double, double>(plan, static_cast<const cplx<double> *>(f.p), psi->d, d)) != QDG_OK) return s;
    acc += std::norm(total(d));
  }
  if ((s = dots<double, double>(plan, psi->d, psi->d, d)) != QDG_OK) return s;
  *out = acc / total(d).real();
  return QDG_OK;
}

qdg_status qdg_observables_compute(qdg_plan *plan, const qdg_wf *psi, const qdg_wf *psi0, int64_t step,
                                   qdg_observables *out) {
  if (!plan || !psi || !out || psi->plan != plan) return fail(QDG_EINVAL, "bad arguments");
  memset(out, 0, sizeof(*out));
  std::vector<cd> d;
  qdg_status s;
  if ((s = dots<double, double>(plan, psi->d, psi->d, d)) != QDG_OK) return s;
  double n2 = 0;
  for (int i = 0; i < plan->S; ++i) { out->pops[i] = d[i].real(); n2 += d[i].real(); }
  out->norm2 = n2;
  if (!std::isfinite(n2)) return fail(QDG_ENONFINITE, "Norm is not a number");
  if (is64(plan)) {
    cplx<double> *o = reinterpret_cast<cplx<double> *>(plan->d_scratch);
    if ((s = h_apply_bulk<double>(plan, psi->d, o, step)) != QDG_OK) return s;
    if ((s = dots<double, double>(plan, psi->d, o, d)) != QDG_OK) return s;
  } else {
    cplx<float> *o = reinterpret_cast<cplx<float> *>(plan->d_scratch);
    if ((s = h_apply_bulk<float>(plan, psi->d, o, step)) != QDG_OK) return s;
    if ((s = dots<double, float>(plan, psi->d, o, d)) != QDG_OK) return s;
  }
  out->energy = total(d).real();
  if (psi0) {
    if (psi0->plan != plan) return fail(QDG_EINVAL, "psi0 of another plan");
    if ((s = dots<double, double>(plan, psi->d, psi0->d, d)) != QDG_OK) return s;
    const cd ac = total(d);
    out->autocorr_re = ac.real();
    out->autocorr_im = ac.imag();
  }
  return QDG_OK;
}

qdg_status qdg_prop_create(qdg_plan *plan, const char *name, const char *params, double dt, int32_t imaginary_time,
                           int32_t backward, qdg_prop **out) {
  if (!plan || !name || !out) return fail(QDG_EINVAL, "null argument");
  *out = nullptr;
  if (!(dt != 0) || !std::isfinite(dt)) return fail(QDG_EINVAL, "No time step defined");
  qdg_prop *P = new qdg_prop();
  P->plan = plan;
  P->user = plan;
  P->name = name;
  parse_params(params, P->params);
  P->dt = dt;
  P->imag = imaginary_time != 0;
  P->backward = backward != 0;
  // OPropagator exponent c0 (OPropagator.h:44-131)
  const cd I(0, 1);
  if (P->imag) P->c0 = P->backward ? cd(-dt) : cd(dt);
  else P->c0 = P->backward ? I * dt : -I * dt;
  if (P->name == "Cheby") P->kind = 1;
  else if (P->name == "GSPO") P->kind = 2;
  else if (P->name == "SIL") P->kind = 3;
  else if (P->name == "Arnoldi") P->kind = 4;
  else { delete P; return fail(QDG_EINVAL, "unknown propagator: " + std::string(name)); }
  if (P->kind >= 3) {
    if (has(P, "order")) P->kord = atoi(P->params["order"].c_str());
    if (P->kord < 3) { delete P; return fail(QDG_EINVAL, "order doesn't make sense"); }
    if (has(P, "err")) P->err = parse_d(P, "err");
    if (has(P, "conv")) P->conv = parse_d(P, "conv");
  }
  // Propagators that FP32 H phi cannot carry run on an FP64 copy of a mixed
  // plan (same host data, the caller's stream):
  // * imaginary-time Chebyshev: its scaled-I_n series (OCheby.cpp:427-433)
  //   reaches the low states through cancellations of terms ~1/sqrt(2 pi R)
  //   down to e^{-R (1 - X)}, far below FP32 resolution;
  // * Lanczos / Arnoldi: each new basis vector is (H q - alpha q - beta q')/beta,
  //   so the FP32 error of H q (~1e-7 of the spectral range) is amplified by
  //   range/beta, and the energies it perturbs turn into a phase error that
  //   grows with the propagation time (6e-4 in the autocorrelation after
  //   2000 a.u. on the 128^2 double well).  The parameter krylov_fp32=1 keeps
  //   the FP32 basis (about 1.2x faster there);
  // * Chebyshev on one line of 512 to 2048 points (a power of two): the
  //   binary64 cluster kernel (one component per thread, qdg_step_line64.cu)
  //   is latency bound and faster than the FP32 line kernels (1-D Morse,
  //   1024 points: 1.20 against 1.85 ms per step), so the mixed form takes
  //   the binary64 step there; cluster=0 or cluster=1 keeps the FP32 kernels.
  const bool krylov_twin = P->kind >= 3 && !(has(P, "krylov_fp32") && atoi(P->params["krylov_fp32"].c_str()) != 0);
  bool line_twin = false;
  if (P->kind == 1 && plan->precision == QDG_PREC_MIXED && plan->nd == 1 && plan->S == 1 && !has(P, "cluster")) {
    const int N = plan->dim[0].n;
    line_twin = (N & (N - 1)) == 0 && N >= 512 && N <= 2048 && qdg::line64_cluster_size(N) > 0;
  }
  if (plan->precision == QDG_PREC_MIXED && ((P->kind == 1 && P->imag) || krylov_twin || line_twin)) {
    qdg_hplan_desc d;
    memset(&d, 0, sizeof(d));
    d.grid = plan->grid;
    d.nstates = plan->S;
    d.nterms = (int32_t)plan->terms.size();
    d.terms = plan->terms.data();
    d.ngrids = plan->ngrids;
    d.grid_data = plan->grids_h.empty() ? nullptr : plan->grids_h.data();
    d.nlasers = plan->nlasers;
    d.laser_nt = plan->laser_nt;
    d.laser_data = plan->lasers_h.empty() ? nullptr : plan->lasers_h.data();
    d.nonhermitian = plan->hermitian ? 0 : 1;
    qdg_plan *tw = nullptr;
    const qdg_status s = qdg_plan_create(&d, QDG_PREC_FP64, &tw);
    if (s != QDG_OK) { delete P; return s; }
    P->twin = tw;
    P->plan = tw;
    sync_twin(P);
  }
  plan->children++;
  *out = P;
  return QDG_OK;
}

qdg_status qdg_prop_destroy(qdg_prop *P) {
  if (!P) return QDG_OK;
  qdg_plan *plan = P->user;
  cudaStreamSynchronize(plan->stream);
  if (P->k0) cudaFree(P->k0);
  if (P->k1) cudaFree(P->k1);
  if (P->k2) cudaFree(P->k2);
  if (P->graph) cudaGraphExecDestroy(P->graph);
  if (P->d_coeffs) cudaFree(P->d_coeffs);
  if (P->d_a) cudaFree(P->d_a);
  if (P->d_cs) cudaFree(P->d_cs);
  if (P->d_bstart) cudaFree(P->d_bstart);
  if (P->d_bstartA) cudaFree(P->d_bstartA);
  if (P->d_bstartB) cudaFree(P->d_bstartB);
  if (P->h_cs) cudaFreeHost(P->h_cs);
  for (auto &g : P->gtab) for (auto v : g) if (v) cudaFree(v);
  for (auto v : P->gcp_d) if (v) cudaFree(v);
  for (auto v : P->gcoef_d) if (v) cudaFree(v);
  for (auto v : P->gU) if (v) cudaFree(v);
  for (auto v : P->lzb) if (v) cudaFree(v);
  if (P->kbuf) cudaFree(P->kbuf);
  if (P->d_ks) cudaFree(P->d_ks);
  if (P->d_kdone) cudaFree(P->d_kdone);
  if (P->h_ks) cudaFreeHost(P->h_ks);
  if (P->h_kdone) cudaFreeHost(P->h_kdone);
  if (P->kwide) cudaFree(P->kwide);
  for (auto v : P->sk) if (v) cudaFree(v);
  if (P->sgrids) cudaFree(P->sgrids);
  if (P->d_scp) cudaFree(P->d_scp);
  if (P->twin) {
    if (P->twin->own_stream) cudaStreamDestroy(P->twin->stream);
    P->twin->own_stream = false;
    P->twin->stream = nullptr;
    free_plan(P->twin);
  }
  delete P;
  release_child(plan);
  return QDG_OK;
}

qdg_status qdg_prop_init(qdg_prop *P) {
  if (!P) return fail(QDG_EINVAL, "null propagator");
  if (P->inited) return QDG_OK;  // avoid init twice (OCheby.cpp:371)
  qdg_status s;
  if (P->kind == 1) s = cheby_init(P);
  else if (P->kind == 2) s = gspo_init(P);
  else s = is64(P->plan) ? krylov_alloc<double>(P) : krylov_alloc<float>(P);
  if (s == QDG_OK) P->inited = true;
  return s;
}

qdg_status qdg_prop_get_info(const qdg_prop *P, qdg_prop_info *info) {
  if (!P || !info) return fail(QDG_EINVAL, "null argument");
  info->kind = P->kind;
  info->order = P->kind == 1 ? P->order : P->kord;
  info->scaling = P->scaling;
  info->offset_re = P->offset.real();
  info->offset_im = P->offset.imag();
  info->exponent_re = P->c0.real();
  info->exponent_im = P->c0.imag();
  return QDG_OK;
}

qdg_status qdg_prop_get_coeffs(const qdg_prop *P, double *coeffs, int32_t capacity) {
  if (!P) return fail(QDG_EINVAL, "null propagator");
  const int n = std::min<int>(capacity, (int)P->coeff.size());
  for (int i = 0; i < n; ++i) coeffs[i] = P->coeff[i];
  return QDG_OK;
}

qdg_status qdg_prop_apply(qdg_prop *P, qdg_wf *psi, int64_t step, int32_t *terms_used) {
  if (!P || !psi || psi->plan != P->user) return fail(QDG_EINVAL, "bad arguments");
  sync_twin(P);
  if (!P->inited) return fail(QDG_EINVAL, "propagator not initialised");
  int used = 0;
  qdg_status s = prop_step(P, psi->d, step, &used, true);
  if (terms_used) *terms_used = used;
  return s;
}

// The host-psi step: every state block copied in, one step, copied back.
// states[s] points to state s's npoints complex128 values.
qdg_status apply_host_states(qdg_prop *P, qdg_wf *scratch, double *const *states, long long step, int32_t *terms_used) {
  sync_twin(P);
  qdg_plan *p = P->plan;
  const size_t sb = sizeof(cplx<double>) * (size_t)p->npts;
  for (int st = 0; st < p->S; ++st)
    CK(cudaMemcpyAsync(scratch->d + (size_t)st * p->npts, states[st], sb, cudaMemcpyHostToDevice, p->stream));
  int used = 0;
  qdg_status s = prop_step(P, scratch->d, step, &used, false);
  if (s != QDG_OK) return s;
  for (int st = 0; st < p->S; ++st)
    CK(cudaMemcpyAsync(states[st], scratch->d + (size_t)st * p->npts, sb, cudaMemcpyDeviceToHost, p->stream));
  if (P->kind == 1) CK(cudaMemcpyAsync(P->h_cs, P->d_cs, sizeof(qdg::ChebyState), cudaMemcpyDeviceToHost, p->stream));
  CK(cudaStreamSynchronize(p->stream));
  if (P->kind == 1) {
    used = P->h_cs->terms;
    count_body_launches(P, used, 1);
    if (P->step_grid > 0) { qdg_status sb2 = check_barrier(p); if (sb2 != QDG_OK) return sb2; }
    if (P->h_cs->status == QDG_ENONFINITE) return fail(QDG_ENONFINITE, "Norm is not a number");
  }
  if (terms_used) *terms_used = used;
  return QDG_OK;
}

qdg_status qdg_prop_apply_host(qdg_prop *P, qdg_wf *scratch, double *host_psi, int64_t step, int32_t *terms_used) {
  if (!P || !scratch || !host_psi || scratch->plan != P->user) return fail(QDG_EINVAL, "bad arguments");
  std::vector<double *> states(P->user->S);
  for (int st = 0; st < P->user->S; ++st) states[st] = host_psi + 2 * (size_t)st * P->user->npts;
  return apply_host_states(P, scratch, states.data(), step, terms_used);
}

qdg_status qdg_prop_apply_host_states(qdg_prop *P, qdg_wf *scratch, double *const *state_psi, int64_t step,
                                      int32_t *terms_used) {
  if (!P || !scratch || !state_psi || scratch->plan != P->user) return fail(QDG_EINVAL, "bad arguments");
  for (int st = 0; st < P->user->S; ++st)
    if (!state_psi[st]) return fail(QDG_EINVAL, "null state block");
  return apply_host_states(P, scratch, state_psi, step, terms_used);
}

qdg_status qdg_plan_inject_barrier_stall(qdg_plan *plan) {
  if (!plan || !plan->d_bar) return fail(QDG_EINVAL, "bad arguments");
  CK(cudaStreamSynchronize(plan->stream));
  // an arrival count no block index can complete (arrived == gridDim.x - 1
  // never holds), so every block runs into its spin limit
  qdg::GridBarrier b{};
  b.count = 0x80000000u;
  CK(cudaMemcpy(plan->d_bar, &b, sizeof(b), cudaMemcpyHostToDevice));
  return QDG_OK;
}

qdg_status qdg_eigen_imag(qdg_prop *P, const double *psi_init, int32_t nef, int32_t maxsteps, double convergence,
                          int32_t diag, double *efs, double *e_raw, double *e_diag, int32_t *steps) {
  if (!P || !psi_init || nef < 1 || maxsteps < 1 || !e_raw || !e_diag) return fail(QDG_EINVAL, "bad arguments");
  if (!P->inited) return fail(QDG_EINVAL, "propagator not initialised");
  if (!P->imag) return fail(QDG_EINVAL, "ImagTimeEF needs an imaginary-time propagator");
  return eigen_imag(P, psi_init, nef, maxsteps, convergence, diag, efs, e_raw, e_diag, steps);
}

qdg_status qdg_eigen_autocorr(qdg_prop *P, const double *psi_init, int32_t nsteps, double tol, int32_t width,
                              int32_t win, int32_t max_nef, double *energies, int32_t *nef_out, double *efs,
                              double *spectrum) {
  if (!P || !psi_init || nsteps < 2 || max_nef < 0 || !nef_out || (max_nef > 0 && !energies))
    return fail(QDG_EINVAL, "bad arguments");
  if (!(tol >= 0)) return fail(QDG_EINVAL, "Tolerance factor for peak finder is non-sense. Must >= 0");
  if (!P->inited) return fail(QDG_EINVAL, "propagator not initialised");
  if (P->imag) return fail(QDG_EINVAL, "AutoCorrEF needs a real-time propagator");
  sync_twin(P);
  qdg_plan *p = P->plan;
  const long long n = wf_elems(p);
  const int M = nsteps;
  const size_t wbytes = sizeof(cplx<double>) * (size_t)n;
  std::vector<void *> bufs;
  auto cleanup = [&](qdg_status st) {
    cudaStreamSynchronize(p->stream);
    for (void *b : bufs) cudaFree(b);
    return st;
  };
  auto alloc = [&](size_t bytes) -> void * {
    void *b = nullptr;
    if (cudaMalloc(&b, std::max<size_t>(bytes, 16)) != cudaSuccess) return nullptr;
    bufs.push_back(b);
    return b;
  };
  // the propagation psi_0 .. psi_{M-1} (the reference's WFBuffer)
  cplx<double> *T = static_cast<cplx<double> *>(alloc(wbytes * (size_t)M));
  cplx<double> *psi = static_cast<cplx<double> *>(alloc(wbytes));
  cplx<double> *d_a = static_cast<cplx<double> *>(alloc(sizeof(cplx<double>) * (size_t)M));
  if (!T || !psi || !d_a) return cleanup(fail(QDG_ENOMEM, "device allocation for the stored propagation failed"));
  qdg_status s;
  std::vector<cd> d;
#define ECHK(expr) do { if ((s = (expr)) != QDG_OK) return cleanup(s); } while (0)
#define ECUDA(expr) do { if ((expr) != cudaSuccess) return cleanup(fail(QDG_ECUDA, #expr)); } while (0)
  ECUDA(cudaMemcpyAsync(T, psi_init, wbytes, cudaMemcpyHostToDevice, p->stream));
  ECUDA(cudaMemcpyAsync(psi, T, wbytes, cudaMemcpyDeviceToDevice, p->stream));
  for (int st = 1; st < M; ++st) {
    int used = 0;
    ECHK(prop_step(P, psi, st - 1, &used, P->kind >= 3));
    ECUDA(cudaMemcpyAsync(T + (size_t)st * n, psi, wbytes, cudaMemcpyDeviceToDevice, p->stream));
  }
  // autocorrelation <psi_s|psi_0> with the volume element (a_0 = 1, ProgEigen.cpp:445)
  ECUDA(qdg::launch_step_overlaps(T, n, M, d_a, p->sm_count, p->stream));
  std::vector<cplx<double>> ha(M);
  ECUDA(cudaMemcpyAsync(ha.data(), d_a, sizeof(cplx<double>) * M, cudaMemcpyDeviceToHost, p->stream));
  ECUDA(cudaStreamSynchronize(p->stream));
  double dv = 1.0;
  for (int k = 0; k < p->nd; ++k) dv *= p->dx[k];
  std::vector<cd> a(M);
  a[0] = 1.0;
  for (int st = 1; st < M; ++st) {
    a[st] = cd(ha[st].re, ha[st].im) * dv;
    if (!std::isfinite(a[st].real())) return cleanup(fail(QDG_ENONFINITE, "Correlation is not a number"));
  }
  // Hann window (FunctionGenerator::Hann), FFT, power spectrum, peaks
  if (win)
    for (int st = 0; st < M; ++st) a[st] *= 0.5 * (1. - cos(2 * M_PI * double(st) / double(M - 1)));
  const std::vector<cd> spec = qdg::host::dft(a, -1);
  std::vector<double> power(M);
  for (int st = 0; st < M; ++st) power[st] = std::abs(spec[st]);
  const std::vector<int> peaks = qdg::host::find_peaks(power, tol, width);
  *nef_out = (int32_t)peaks.size();
  if (spectrum) memcpy(spectrum, spec.data(), sizeof(cd) * M);
  const int K = std::min<int>((int)peaks.size(), max_nef);
  if (K > 0) {
    // eigenfunctions by time integration at the peak energies (ProgEigen.cpp:560-580)
    const double dw = 2 * M_PI / (P->dt * double(M));
    std::vector<cplx<double>> C((size_t)K * M);
    std::vector<double> E(K);
    for (int k = 0; k < K; ++k) {
      const int idx = peaks[k];
      E[k] = idx < M / 2 ? double(idx) * dw : double(idx - M) * dw;
      for (int st = 0; st < M; ++st) {
        const double ang = E[k] * double(st) * P->dt;
        C[(size_t)k * M + st] = cplx<double>{cos(ang), sin(ang)};
      }
    }
    cplx<double> *dC = static_cast<cplx<double> *>(alloc(sizeof(cplx<double>) * C.size()));
    cplx<double> *ef = static_cast<cplx<double> *>(alloc(wbytes * (size_t)K));
    if (!dC || !ef) return cleanup(fail(QDG_ENOMEM, "device allocation failed"));
    ECUDA(cudaMemcpyAsync(dC, C.data(), sizeof(cplx<double>) * C.size(), cudaMemcpyHostToDevice, p->stream));
    ECUDA(qdg::launch_integrate_steps(T, n, M, dC, K, ef, p->sm_count, p->stream));
    for (int k = 0; k < K; ++k) {
      cplx<double> *f = ef + (size_t)k * n;
      ECHK((dots<double, double>(p, f, f, d)));
      const double nr = std::sqrt(total(d).real());
      if (!std::isfinite(nr) || !(nr > 0)) return cleanup(fail(QDG_ENONFINITE, "Norm is not a number"));
      ECUDA(qdg::launch_lincomb<double>(f, (const cplx<double> *)nullptr, cplx<double>{1.0 / nr, 0}, cplx<double>{0, 0},
                                        n, p->stream));
      cd e;
      ECHK(h_expec(p, f, f, &e));
      energies[k] = e.real();
      if (efs) ECUDA(cudaMemcpyAsync(efs + 2 * (size_t)k * n, f, wbytes, cudaMemcpyDeviceToHost, p->stream));
    }
  }
#undef ECHK
#undef ECUDA
  return cleanup(QDG_OK);
}

// ProgEigen::LanczosEF (src/ProgEigen.cpp:604-648) with DiagBasis
// (ProgEigen.cpp:94-138): the Arnoldi basis of psi_init (OArnoldi::BuildLZB,
// the propagator's own basis build), the Ritz pairs of its Hessenberg
// matrix, the Ritz functions sum_j z_ji v_j, then the Hamiltonian in that
// basis diagonalised.  For a hermitian H the Hessenberg matrix is real
// symmetric tridiagonal up to rounding, so its symmetric part is
// diagonalised by Jacobi rotations in place of LAPACK's zhseqr/zhsein; each
// eigenvector is scaled as zhsein scales it (largest component of modulus
// 1), which DiagBasis sees through its off-diagonal matrix elements.
extern "C++" {
template <typename T>
qdg_status eigen_lanczos(qdg_prop *P, const double *psi_init, int max_nef, double *e_raw, double *e_diag,
                         int32_t *nef_out, double *efs) {
  qdg_plan *p = P->plan;
  const long long n = wf_elems(p);
  const size_t wbytes = sizeof(cplx<double>) * (size_t)n;
  const int m = P->kord;
  if (m > qdg::kMaxKrylov) return fail(QDG_EUNSUPPORTED, "Krylov order above 64");
  std::vector<cplx<double> *> bufs;
  auto cleanup = [&](qdg_status st) {
    cudaStreamSynchronize(p->stream);
    for (auto *b : bufs) cudaFree(b);
    return st;
  };
  auto alloc = [&]() -> cplx<double> * {
    cplx<double> *b = nullptr;
    if (cudaMalloc(&b, wbytes) != cudaSuccess) return nullptr;
    bufs.push_back(b);
    return b;
  };
  cplx<double> *psi = alloc();
  if (!psi) return cleanup(fail(QDG_ENOMEM, "device allocation failed"));
  qdg_status s;
  std::vector<cd> d;
#define ECHK(expr) do { if ((s = (expr)) != QDG_OK) return cleanup(s); } while (0)
#define ECUDA(expr) do { if ((expr) != cudaSuccess) return cleanup(fail(QDG_ECUDA, #expr)); } while (0)
  ECUDA(cudaMemcpyAsync(psi, psi_init, wbytes, cudaMemcpyHostToDevice, p->stream));
  ECUDA(qdg::launch_set_coefs(p->d_coef, p->d_cp, p->d_lasers, p->laser_nt, 0, p->stream));
  // the basis of the propagator's step (OArnoldi::BuildLZB: lzb[0] = psi);
  // psi itself is left as it is
  ECHK(arnoldi_body<T>(P, psi));
  ECUDA(cudaStreamSynchronize(p->stream));
  const int order = *P->h_kdone;
  const double *H = P->h_ks;
  if (!std::isfinite(H[2 * m * m])) return cleanup(fail(QDG_ENONFINITE, "Norm is not a number"));
  std::vector<double> A((size_t)order * order), w, z;
  for (int i = 0; i < order; ++i)
    for (int j = 0; j < order; ++j)
      A[(size_t)i * order + j] = 0.5 * (H[2 * (i * m + j)] + H[2 * (j * m + i)]);
  qdg::host::sym_eig(order, A, w, z);
  const int K = std::min(order, max_nef);
  *nef_out = order;
  // Ritz functions
  std::vector<cplx<double> *> rf(order, nullptr);
  for (int i = 0; i < order; ++i) {
    if (!(rf[i] = alloc())) return cleanup(fail(QDG_ENOMEM, "device allocation failed"));
    double zmax = 0;
    for (int j = 0; j < order; ++j) zmax = std::max(zmax, std::fabs(z[(size_t)j * order + i]));
    qdg::KCombine<T> kc;
    memset(&kc, 0, sizeof(kc));
    kc.m = order;
    for (int j = 0; j < order; ++j) {
      kc.c[j] = cplx<double>{z[(size_t)j * order + i] / zmax, 0.0};
      kc.q[j] = reinterpret_cast<const cplx<T> *>(P->lzb[j]);
    }
    // kcombine forms rf c_0 + sum_{j >= 1} c_j q_j: rf starts as v_0 = psi
    ECUDA(cudaMemcpyAsync(rf[i], psi, wbytes, cudaMemcpyDeviceToDevice, p->stream));
    ECUDA(qdg::launch_kcombine<T>(rf[i], kc, n, p->stream));
  }
  // DiagBasis: S(j, i) = Re <f_i|H|f_j> for j < i, S(i, i) = the Ritz value
  std::vector<double> Sm((size_t)order * order, 0.0), wd, zd;
  for (int i = 0; i < order; ++i) {
    for (int j = 0; j < i; ++j) {
      cd e;
      ECHK(h_expec(p, rf[i], rf[j], &e));
      Sm[(size_t)j * order + i] = Sm[(size_t)i * order + j] = e.real();
    }
    Sm[(size_t)i * order + i] = w[i];
  }
  qdg::host::sym_eig(order, Sm, wd, zd);
  for (int k = 0; k < K; ++k) {
    e_raw[k] = w[k];
    e_diag[k] = wd[k];
  }
  if (efs) {
    cplx<double> *out = alloc();
    if (!out) return cleanup(fail(QDG_ENOMEM, "device allocation failed"));
    for (int k = 0; k < K; ++k) {
      ECUDA(cudaMemsetAsync(out, 0, wbytes, p->stream));
      for (int j = 0; j < order; ++j)
        ECUDA(qdg::launch_lincomb<double>(out, rf[j], cplx<double>{1, 0}, cplx<double>{zd[(size_t)j * order + k], 0},
                                          n, p->stream));
      ECUDA(cudaMemcpyAsync(efs + 2 * (size_t)k * n, out, wbytes, cudaMemcpyDeviceToHost, p->stream));
    }
  }
#undef ECHK
#undef ECUDA
  return cleanup(QDG_OK);
}
}  // extern "C++"

qdg_status qdg_eigen_lanczos(qdg_prop *P, const double *psi_init, int32_t max_nef, double *e_raw, double *e_diag,
                             int32_t *nef_out, double *efs) {
  if (!P || !psi_init || max_nef < 0 || !nef_out || (max_nef > 0 && (!e_raw || !e_diag)))
    return fail(QDG_EINVAL, "bad arguments");
  if (!P->inited) return fail(QDG_EINVAL, "propagator not initialised");
  if (P->kind != 4) return fail(QDG_EINVAL, "Arnoldi Propagator is needed to find Lanczos Eigenvalues");
  sync_twin(P);
  if (is64(P->plan)) return eigen_lanczos<double>(P, psi_init, max_nef, e_raw, e_diag, nef_out, efs);
  return eigen_lanczos<float>(P, psi_init, max_nef, e_raw, e_diag, nef_out, efs);
}

qdg_status qdg_prop_run(qdg_prop *P, qdg_wf *psi, int64_t step0, int32_t nsteps, int64_t *terms_total) {
  if (!P || !psi || psi->plan != P->user || nsteps < 0) return fail(QDG_EINVAL, "bad arguments");
  sync_twin(P);
  if (!P->inited) return fail(QDG_EINVAL, "propagator not initialised");
  long long tot = 0, before = 0;
  if (P->kind == 1) {
    CK(cudaMemcpyAsync(P->h_cs, P->d_cs, sizeof(qdg::ChebyState), cudaMemcpyDeviceToHost, P->plan->stream));
    CK(cudaStreamSynchronize(P->plan->stream));
    before = P->h_cs->total;
  }
  for (int i = 0; i < nsteps; ++i) {
    int used = 0;
    // Chebyshev and GSPO steps are queued without host synchronisation;
    // the Chebyshev term count is read back once at the end.
    const bool sync = P->kind >= 3;
    qdg_status s = prop_step(P, psi->d, step0 + i, &used, sync);
    if (s != QDG_OK) return s;
    tot += used;
  }
  CK(cudaStreamSynchronize(P->plan->stream));
  if (P->kind == 1) {
    CK(cudaMemcpy(P->h_cs, P->d_cs, sizeof(qdg::ChebyState), cudaMemcpyDeviceToHost));
    if (P->h_cs->status == QDG_ENONFINITE) return fail(QDG_ENONFINITE, "Norm is not a number");
    tot = P->h_cs->total - before;
    count_body_launches(P, tot, nsteps);
    if (P->step_grid > 0) { qdg_status sb = check_barrier(P->plan); if (sb != QDG_OK) return sb; }
  }
  if (terms_total) *terms_total = tot;
  return QDG_OK;
}

int64_t qdg_kernel_launches(void) { return qdg::launch_counter(); }

qdg_status qdg_prop_phase_times(qdg_prop *P, double ns[4]) {
  if (!P || !ns) return fail(QDG_EINVAL, "null argument");
  for (int k = 0; k < 4; ++k) ns[k] = 0;
  if (P->kind != 1 || !P->d_cs) return QDG_OK;
  CK(cudaStreamSynchronize(P->plan->stream));
  qdg::ChebyState cs;
  CK(cudaMemcpy(&cs, P->d_cs, sizeof(cs), cudaMemcpyDeviceToHost));
  for (int k = 0; k < 4; ++k) ns[k] = (double)cs.t_phase[k];
  unsigned long long z[4] = {0, 0, 0, 0};
  CK(cudaMemcpy(reinterpret_cast<char *>(P->d_cs) + offsetof(qdg::ChebyState, t_phase), z, sizeof(z),
                cudaMemcpyHostToDevice));
  return QDG_OK;
}

qdg_status qdg_profile_enable(qdg_plan *plan, int32_t on) {
  if (!plan) return fail(QDG_EINVAL, "null plan");
  CK(cudaStreamSynchronize(plan->stream));
  plan->profiling = on != 0;
  plan->ev_mode.clear();
  return QDG_OK;
}

qdg_status qdg_profile_read(qdg_plan *plan, double ms[8], int64_t launches[8]) {
  if (!plan || !ms || !launches) return fail(QDG_EINVAL, "null argument");
  for (int i = 0; i < 8; ++i) { ms[i] = 0; launches[i] = 0; }
  CK(cudaStreamSynchronize(plan->stream));
  for (size_t i = 0; i < plan->ev_mode.size(); ++i) {
    float t = 0;
    CK(cudaEventElapsedTime(&t, plan->ev_pool[2 * i], plan->ev_pool[2 * i + 1]));
    const int m = plan->ev_mode[i];
    if (m >= 0 && m < 8) { ms[m] += t; launches[m]++; }
  }
  plan->ev_mode.clear();
  return QDG_OK;
}

}  // extern "C"
