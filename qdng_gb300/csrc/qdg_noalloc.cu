// qdg_noalloc.cu -- H psi without any device allocation.
//
// Some callers cannot allocate device memory: host frameworks that own all
// device memory through their own caching pool, plug-ins that must not
// change the process's allocation state, or time-step loops where the
// implicit device synchronisation of cudaMalloc would stall the pipeline.  qdg_h_apply_noalloc() gives them H psi on arrays they
// already own.  The scratch the kinetic passes need (the per-dimension parts
// T_d psi, FFT twiddle tables, the potential-matrix list) lives in one
// statically sized device array of this file, QDG_NOALLOC_SCRATCH_BYTES
// bytes, which every GPU that loads the library holds until the process
// exits.  Problems that do not fit are rejected with QDG_EINVAL.
//
// All calls share that array and each call overwrites what it needs, so two
// calls whose kernels overlap on the GPU (different streams, or other
// threads) race on it; serialise them on one stream.  The first call on a
// device looks up the array's device address (cudaGetSymbolAddress) with
// that device current.
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <mutex>
#include <string>

#include "../../include/qdg.h"
#include "qdg_kernels.cuh"
#include "qdg_schedule.h"

namespace qdg {
// The shared scratch of qdg_h_apply_noalloc (see the file comment).
static __device__ __align__(256) unsigned char g_noalloc_scratch[QDG_NOALLOC_SCRATCH_BYTES];
}

namespace {

using qdg::cplx;

qdg_status na_fail(qdg_status s, const std::string &m) {
  qdg::set_last_error(m);
  return s;
}

const int kMaxDevices = 64;
std::mutex g_addr_mutex;
void *g_addr[kMaxDevices] = {nullptr};

// Device address of the scratch array on the current device (looked up once
// per device, with that device current).
qdg_status scratch_address(void **out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices)
    return na_fail(QDG_ECUDA, "no current CUDA device");
  std::lock_guard<std::mutex> lock(g_addr_mutex);
  if (!g_addr[dev]) {
    void *p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, qdg::g_noalloc_scratch);
    if (e != cudaSuccess || !p) return na_fail(QDG_ECUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
    g_addr[dev] = p;
  }
  *out = g_addr[dev];
  return QDG_OK;
}

size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

struct Tables {
  qdg::Couplings cp;
  int nd, S;
  int n[QDG_MAX_DIMS];
  double kfac[QDG_MAX_DIMS][qdg::kMaxStates];
  long long tw_off[QDG_MAX_DIMS];  // offset (complex elements) of the twiddles of dim d
  long long laser_nt;
  long long step;
};

// Writes the potential-matrix list, the kinetic multipliers, the field
// coefficients of `step` and the twiddles exp(-2 pi i m/N_d) into the scratch.
__global__ void noalloc_setup_kernel(Tables t, const double *lasers, qdg::Couplings *cp_out, double *coef_out,
                                     double *kfac_out, cplx<double> *tw_out) {
  const int tid = blockIdx.x * blockDim.x + threadIdx.x;
  const int nthr = gridDim.x * blockDim.x;
  if (tid == 0) *cp_out = t.cp;
  for (int e = tid; e < t.cp.ne; e += nthr) {
    const int l = t.cp.lid[e];
    coef_out[e] = l < 0 ? 1.0 : ((t.step >= 0 && t.step < t.laser_nt) ? -lasers[(long long)l * t.laser_nt + t.step] : 0.0);
  }
  for (int i = tid; i < t.nd * t.S; i += nthr) kfac_out[i] = t.kfac[i / t.S][i % t.S];
  for (int d = 0; d < t.nd; ++d) {
    const int N = t.n[d];
    for (int m = tid; m < N; m += nthr) {
      double s, c;
      sincospi(-2.0 * (double)m / (double)N, &s, &c);
      tw_out[t.tw_off[d] + m].re = c;
      tw_out[t.tw_off[d] + m].im = s;
    }
  }
}

bool radix_plan_na(int n, qdg::RadixPlan &rp) {
  rp.n = n;
  rp.nstages = 0;
  int m = n;
  while (m % 16 == 0) { rp.radix[rp.nstages++] = 16; m /= 16; }
  if (m % 8 == 0) { rp.radix[rp.nstages++] = 8; m /= 8; }
  if (m % 4 == 0) { rp.radix[rp.nstages++] = 4; m /= 4; }
  if (m % 2 == 0) { rp.radix[rp.nstages++] = 2; m /= 2; }
  while (m % 3 == 0) { rp.radix[rp.nstages++] = 3; m /= 3; }
  while (m % 5 == 0) { rp.radix[rp.nstages++] = 5; m /= 5; }
  if (m == 1) return rp.nstages <= 16;
  // other prime factors: direct-DFT stages of the line passes' transforms
  return qdg::any_radix(n, rp);
}

}  // namespace

extern "C" {

qdg_status qdg_h_apply_noalloc(const qdg_hplan_desc *desc, const double *psi_in, double *psi_out, int64_t step,
                               void *cuda_stream) {
  if (!desc || !psi_in || !psi_out) return na_fail(QDG_EINVAL, "null argument");
  if (psi_in == psi_out) return na_fail(QDG_EINVAL, "H apply needs distinct input and output");
  const qdg_grid &g = desc->grid;
  const int S = desc->nstates;
  if (g.ndims < 1 || g.ndims > QDG_MAX_DIMS) return na_fail(QDG_EINVAL, "invalid number of grid dimensions");
  if (S < 1 || S > qdg::kMaxStates) return na_fail(QDG_EUNSUPPORTED, "number of states outside 1..8");
  if (desc->nterms < 1 || !desc->terms) return na_fail(QDG_EINVAL, "Hamiltonian is empty");
  cudaStream_t st = (cudaStream_t)cuda_stream;

  Tables t;
  memset(&t, 0, sizeof(t));
  t.nd = g.ndims;
  t.S = S;
  t.laser_nt = desc->laser_nt;
  t.step = step;
  long long npts = 1, stride[QDG_MAX_DIMS];
  double dx[QDG_MAX_DIMS], dk[QDG_MAX_DIMS];
  qdg::RadixPlan rp[QDG_MAX_DIMS];
  for (int d = 0; d < g.ndims; ++d) {
    if (g.n[d] < 2 || !(g.xmax[d] > g.xmin[d])) return na_fail(QDG_EINVAL, "invalid grid");
    if (!radix_plan_na(g.n[d], rp[d])) return na_fail(QDG_EUNSUPPORTED, "grid size has more than 16 prime factors");
    stride[d] = npts;
    npts *= g.n[d];
    t.n[d] = g.n[d];
    dx[d] = (g.xmax[d] - g.xmin[d]) / double(g.n[d] - 1);   // GridSystem::Dx
    dk[d] = (2 * M_PI) / (g.xmax[d] - g.xmin[d] + dx[d]);   // Kspace::Dk
  }
  // potential-matrix list sorted by row (hermitian mirrors explicit)
  int er[qdg::kMaxCouplings], ec[qdg::kMaxCouplings], eg[qdg::kMaxCouplings], el[qdg::kMaxCouplings];
  int nent = 0;
  // OMultistate's hermitian copy, off for "nonhermitian" or when elements sit
  // at both (i, j) and (j, i) (OMultistate.cpp:52-53,83-85)
  bool hermitian = !desc->nonhermitian;
  for (int i = 0; i < desc->nterms; ++i)
    for (int j = 0; j < desc->nterms; ++j) {
      const qdg_hterm &a = desc->terms[i], &b = desc->terms[j];
      if (a.row != a.col && a.row == b.col && a.col == b.row) hermitian = false;
    }
  for (int i = 0; i < desc->nterms; ++i) {
    const qdg_hterm &h = desc->terms[i];
    if (h.row < 0 || h.col < 0 || h.row >= S || h.col >= S) return na_fail(QDG_EINVAL, "matrix element outside the states");
    if (h.kind == QDG_TERM_KINETIC) {
      if (h.row != h.col) return na_fail(QDG_EUNSUPPORTED, "kinetic operator off the diagonal");
      if (h.fd_order != 0) return na_fail(QDG_EUNSUPPORTED, "finite-difference kinetic (method HOFD) needs a plan");
      for (int d = 0; d < g.ndims; ++d) {
        if (!(h.mass[d] > 0)) return na_fail(QDG_EINVAL, "Zero mass defined");
        t.kfac[d][h.row] += (dk[d] * dk[d]) / (2.0 * h.mass[d]) / (double)g.n[d];
      }
      continue;
    }
    if (h.kind != QDG_TERM_POTENTIAL && h.kind != QDG_TERM_DIPOLE) return na_fail(QDG_EUNSUPPORTED, "unknown term kind");
    if (h.grid < 0 || h.grid >= desc->ngrids || !desc->grid_data) return na_fail(QDG_EINVAL, "potential grid index out of range");
    if (h.kind == QDG_TERM_DIPOLE && (h.laser < 0 || h.laser >= desc->nlasers || !desc->laser_data))
      return na_fail(QDG_EINVAL, "dipole operator without a laser field");
    for (int r = 0; r < (hermitian && h.row != h.col ? 2 : 1); ++r) {
      if (nent >= qdg::kMaxCouplings) return na_fail(QDG_EUNSUPPORTED, "too many potential/dipole matrix entries");
      er[nent] = r ? h.col : h.row;
      ec[nent] = r ? h.row : h.col;
      eg[nent] = h.grid;
      el[nent] = h.kind == QDG_TERM_DIPOLE ? h.laser : -1;
      ++nent;
    }
  }
  t.cp.ne = 0;
  for (int s = 0; s < S; ++s)
    for (int e = 0; e < nent; ++e)
      if (er[e] == s) {
        const int k = t.cp.ne++;
        t.cp.row[k] = er[e]; t.cp.col[k] = ec[e]; t.cp.gid[k] = eg[e]; t.cp.lid[k] = el[e];
      }
  for (int s = 0, e = 0; s <= qdg::kMaxStates; ++s) {
    while (e < t.cp.ne && t.cp.row[e] < s) ++e;
    t.cp.rs[s] = e;
  }

  // scratch layout: couplings | coef | kfac | twiddles | T_d psi (dims > 1)
  size_t off = 0;
  const size_t o_cp = off; off = align256(off + sizeof(qdg::Couplings));
  const size_t o_coef = off; off = align256(off + sizeof(double) * qdg::kMaxCouplings);
  const size_t o_kfac = off; off = align256(off + sizeof(double) * QDG_MAX_DIMS * qdg::kMaxStates);
  const size_t o_tw = off;
  long long twn = 0;
  for (int d = 0; d < g.ndims; ++d) { t.tw_off[d] = twn; twn += g.n[d]; }
  off = align256(off + sizeof(cplx<double>) * twn);
  const size_t o_P = off;
  const size_t pbytes = g.ndims > 1 ? sizeof(cplx<double>) * (size_t)npts * S : 0;
  off += g.ndims * pbytes;
  if (off > (size_t)QDG_NOALLOC_SCRATCH_BYTES)
    return na_fail(QDG_EINVAL, "problem needs " + std::to_string(off) + " bytes of scratch, more than the " +
                                   std::to_string((long long)QDG_NOALLOC_SCRATCH_BYTES) + " bytes of qdg_h_apply_noalloc");

  void *base = nullptr;
  qdg_status s = scratch_address(&base);
  if (s != QDG_OK) return s;
  unsigned char *b = static_cast<unsigned char *>(base);
  qdg::Couplings *d_cp = reinterpret_cast<qdg::Couplings *>(b + o_cp);
  double *d_coef = reinterpret_cast<double *>(b + o_coef);
  double *d_kfac = reinterpret_cast<double *>(b + o_kfac);
  cplx<double> *d_tw = reinterpret_cast<cplx<double> *>(b + o_tw);

  noalloc_setup_kernel<<<8, 256, 0, st>>>(t, desc->laser_data, d_cp, d_coef, d_kfac, d_tw);
  if (cudaGetLastError() != cudaSuccess) return na_fail(QDG_ECUDA, "setup kernel launch failed");
  qdg::add_launches(1);

  int dev = 0, sms = 1;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const cplx<double> *in = reinterpret_cast<const cplx<double> *>(psi_in);
  cplx<double> *out = reinterpret_cast<cplx<double> *>(psi_out);

  if (g.ndims == 1) {
    // one fused line pass: FFT, k^2, inverse FFT, potential matrix
    qdg::PassArgs<double> a;
    memset(&a, 0, sizeof(a));
    a.N = g.n[0]; a.TW = 1; a.S = S; a.nsub = S; a.npts = npts; a.rp = rp[0];
    a.es = 1; a.ls = g.n[0]; a.tiles_per_hi = 1; a.hi_stride = g.n[0]; a.ntiles = npts / g.n[0];
    a.tw = d_tw + t.tw_off[0];
    a.kfac = d_kfac;
    a.phi = in; a.out = out; a.cp = d_cp; a.coef = d_coef; a.grids = desc->grid_data;
    const size_t smem = ((size_t)g.n[0] + 2 * qdg::line_buf_elems(g.n[0], S)) * sizeof(cplx<double>);
    if (smem > 227 * 1024) return na_fail(QDG_EUNSUPPORTED, "grid line too long for the shared-memory FFT");
    const int grid = (int)std::min<long long>(a.ntiles, 4LL * sms);
    if (qdg::launch_pass<double>(qdg::PM_HAPPLY, a, grid, 256, smem, st) != cudaSuccess)
      return na_fail(QDG_ECUDA, "line pass launch failed");
    return QDG_OK;
  }
  qdg::KinArgs<double> k;
  memset(&k, 0, sizeof(k));
  k.nd = g.ndims; k.S = S; k.npts = npts; k.phi = in;
  long long items = 0;
  size_t smem = 0;
  for (int d = 0; d < g.ndims; ++d) {
    qdg::DimPass<double> &dp = k.dp[d];
    const int N = g.n[d];
    int TW = 1;  // lines per tile: keep the tile near 2048 points
    const long long limit = d == 0 ? npts / N : stride[d];
    while (TW < 16 && limit % (2 * TW) == 0 && 2 * TW * N <= 2048) TW *= 2;
    dp.N = N; dp.TW = TW; dp.rp = rp[d];
    if (d == 0) { dp.es = 1; dp.ls = N; dp.tiles_per_hi = 1; dp.hi_stride = (long long)TW * N; }
    else { dp.es = (int)stride[d]; dp.ls = 1; dp.tiles_per_hi = (int)(stride[d] / TW); dp.hi_stride = stride[d] * N; }
    dp.ntiles = npts / ((long long)N * TW);
    dp.tw = d_tw + t.tw_off[d];
    dp.kfac = d_kfac + d * S;
    dp.P = reinterpret_cast<cplx<double> *>(b + o_P + d * pbytes);
    k.item_start[d] = items;
    items += dp.ntiles * S;
    smem = std::max(smem, ((size_t)N + 2 * qdg::line_buf_elems(N, TW)) * sizeof(cplx<double>));
  }
  k.item_start[g.ndims] = items;
  if (smem > 227 * 1024) return na_fail(QDG_EUNSUPPORTED, "grid line too long for the shared-memory FFT");
  const int kgrid = (int)std::min<long long>(items, 4LL * sms);
  if (qdg::launch_kin_all<double>(k, kgrid, 256, smem, st) != cudaSuccess)
    return na_fail(QDG_ECUDA, "kinetic launch failed");
  qdg::CombArgs<double> c;
  memset(&c, 0, sizeof(c));
  c.S = S; c.nd = g.ndims; c.npts = npts; c.phi = in;
  for (int d = 0; d < g.ndims; ++d) c.P[d] = k.dp[d].P;
  c.out = out; c.cp = d_cp; c.coef = d_coef; c.grids = desc->grid_data;
  const int cgrid = (int)std::min<long long>((npts + 255) / 256, 8LL * sms);
  if (qdg::launch_combine<double>(qdg::PM_HAPPLY, c, cgrid, 256, st) != cudaSuccess)
    return na_fail(QDG_ECUDA, "combine launch failed");
  return QDG_OK;
}

}  // extern "C"
