// qdg_kernels.cuh -- kernel argument blocks and launch entry points shared by
// the kernel translation units and the host API.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>

#include "qdg_device.cuh"

namespace qdg {

// Epilogue of a line pass.
enum PassMode {
  PM_KIN_FIRST = 0,   // P  = T_d phi                   (first of several kinetic passes)
  PM_KIN_ACC = 1,     // P += T_d phi                   (middle passes)
  PM_HAPPLY = 2,      // out = P + T_d phi + W phi       (last pass: H phi)
  PM_CHEBY_FIRST = 3, // last pass of H psi + first Chebyshev terms (OCheby.cpp:99-111)
  PM_CHEBY_TERM = 4,  // last pass of H phi_{n-1} + recurrence + accumulation (OCheby.cpp:120-175)
  PM_GSPO_KIN = 5     // phi <- IFFT_d exp(c T_d) FFT_d phi / N_d in place (OGSPO kinetic member)
};

static const int kMaxStates = 8;      // states handled by the fused kernels
static const int kMaxCouplings = 64;  // potential / dipole matrix entries

// Potential-matrix entries of H: H_{row,col} += coef_e * grid[gid][x] with
// coef_e = 1 (OGridPotential) or -E_lid(step) (OGridDipole, field lid).
// Hermitian mirrors are listed explicitly.
struct Couplings {
  int ne;
  int row[kMaxCouplings];
  int col[kMaxCouplings];
  int gid[kMaxCouplings];
  int lid[kMaxCouplings];  // -1: static potential
  int nim[kMaxCouplings];  // 1: the entry acts as -i coef grid (OGobbler as a negative imaginary potential)
  int any_nim;
  // entries sorted by row: entries of row s are [rs[s], rs[s+1]) (the list above is in this order)
  int rs[kMaxStates + 1];
};
static const int kMaxRowEntries = 4;  // entries per row the fused step kernel unrolls
static const int kMaxBatchLines = 64; // lines one block of the step kernel transforms at once
// The multi-dimensional step kernel stages the gather's operands in shared
// memory with asynchronous copies when its bulk elements are 16-byte
// complex numbers (binary64, double-float) and it handles one or two
// states: kStageDepth slots of one point per thread (256 threads).
static const int kStageDepth = 3;
__host__ __device__ constexpr bool step_staged(int cplx_bytes, int states) { return cplx_bytes == 16 && states <= 2; }
__host__ __device__ constexpr int step_stage_bytes_c(int nd, int states) {
  return kStageDepth * (((nd + states + 1) * 256 * 16) + kMaxRowEntries * 256 * 8 + 256 * 16);
}

// Per-step Chebyshev control block in device memory.
struct ChebyState {
  long long total;   // terms summed over all steps since the propagator was set up
  double norm0;      // raw norm of psi before the step
  double norm_last;  // imaginary time: previous accumulated norm
  int done;          // series converged (or error): later terms are skipped
  int terms;         // terms used in the step
  int status;        // QDG_OK or QDG_ENONFINITE
  unsigned int arrive;  // blocks of the current reduction that have stored their partial sum
  int i;             // index of the next term (device-driven term loop)
  double acc_last;   // accumulated norm after the previous term (differential cut)
  // phase timing of the persistent step kernel as seen by one block (ns,
  // accumulated over the terms after the first while tracing): gathering
  // and finishing phi, the FFTs, the whole term, the norm reduction and the
  // grid barrier
  unsigned long long t_phase[4];
};

// Series-cut parameters handed to the kernel that finishes a Chebyshev term:
// its last block sums the per-block norms in a fixed order and applies the
// reference's criterion (OCheby.cpp:178-182 real time, 285-289 imaginary).
struct ChebyCut {
  ChebyState *cs;   // nullptr: no reduction (H apply)
  int first;        // 1: raw norm of psi before the step (OCheby::raw_norm)
  int term;         // index i of the term just added (static launches)
  double prec;
  int imag;
  int offim0;       // offset has no imaginary part (break allowed)
  int diff;         // mixed precision: compare with the previous term's norm, not the initial one
  // device-driven term loop (one graph body per term inside a while node)
  int dyn;                      // take the term index from cs->i and the buffers by its parity
  int order;
  const cplx<double> *coeffs;   // [order] coeff[i] exp(c0 offset)
  unsigned long long cond;      // cudaGraphConditionalHandle of the while node
  int use_cond;
};

template <typename T>
struct PassArgs {
  // geometry of the lines of this pass
  int N;            // line length
  int es;           // element stride along a line
  int ls;           // stride between the TW lines of a tile
  int TW;           // lines per tile (per state)
  int tiles_per_hi; // tiles inside one block of stride_d * N_d points
  long long hi_stride;  // stride_d * N_d
  long long ntiles;
  int S;            // states of the wave function
  int nsub;         // states per work item (1, or S when the epilogue couples states)
  long long npts;   // points per state
  RadixPlan rp;
  const cplx<T> *tw;   // N twiddles exp(-2 pi i m/N)
  const double *kfac;  // [S] kinetic multiplier for this dim: dk^2/(2m) (times 1/N for H passes)
  // buffers (state stride npts)
  const cplx<T> *phi;  // input
  cplx<T> *P;          // kinetic partial sums of earlier passes
  cplx<T> *out;        // PM_HAPPLY output, PM_GSPO_KIN in-place target
  cplx<double> *psi;   // Chebyshev accumulator (always FP64)
  cplx<T> *k0;         // phi_{n-2} in, phi_n out (PM_CHEBY_TERM); phi_1 out (PM_CHEBY_FIRST)
  // potential matrix
  const Couplings *cp;     // device copy
  const double *coef;      // [ne] coefficient of each entry at this step
  const T *grids;          // [ngrids][npts]
  int multi_pass;          // P holds kinetic parts of earlier passes
  // Chebyshev scalars (FP64)
  cplx<double> offset;     // energy offset (OCheby::_offset)
  cplx<double> fac;        // _exp/_scaling (first) or 2*_exp/_scaling (terms)
  cplx<double> fac_lo;     // fac's rounding residual: the exact factor is fac + fac_lo
  cplx<double> c0p, c1p;   // coeff[0], coeff[1] times exp(c0*offset)
  cplx<double> coeff;      // coeff[i] times exp(c0*offset)
  int imag;                // imaginary-time recursion (minus sign, OCheby.cpp:276)
  double *partials;        // per-block partial sums (norms)
  const int *done;         // Chebyshev series converged: skip the work
  ChebyCut cut;            // fused series cut (Chebyshev modes)
  const cplx<T> *bufs[2];  // device-driven term loop: phi = bufs[(i+1)&1], k0 = bufs[i&1]
  // GSPO kinetic member: per-state exp(c T_d(k)) / N_d tables, S x N entries
  const cplx<T> *gtab;
};

// One dimension of an all-dimension kinetic launch.
template <typename T>
struct DimPass {
  int N, es, ls, TW, tiles_per_hi;
  long long hi_stride, ntiles;
  RadixPlan rp;
  const cplx<T> *tw;
  const double *kfac;   // [S] dk^2/(2m)/N
  cplx<T> *P;           // T_d phi output (state stride npts)
  const T *ktab;        // [S][N] kinetic multipliers kfac[s] * min(i, N-i)^2 (precomputed)
  const cplx<dfl> *twdf;  // DF64 form: twiddles and multipliers in double-float (the FFT type)
  const dfl *ktdf;
};

// T_d phi for every dimension d in one launch (the kinetic operator is a sum
// of independent one-dimensional parts).
template <typename T>
struct KinArgs {
  int nd, S;
  long long npts;
  const cplx<T> *phi;
  DimPass<T> dp[4];
  long long item_start[5];  // first work item of each dimension
  const int *done;
  // device-driven term loop: phi = bufs[(cs->i + 1) & 1]
  const ChebyState *cs;
  const cplx<T> *bufs[2];
  int dyn;
};

// T_d phi of every dimension for binary64 lines of N = 2^p <= 1024 points,
// latency-oriented (kin_r2_kernel): a block holds L lines, N/2 threads per
// line, one radix-2 Stockham butterfly per thread and stage.
struct KinR2Args {
  int nd, S, threads;
  long long npts;
  int N[4], L[4], lgN[4];
  long long stride[4];
  long long groups[4];          // line groups of L lines per state
  long long item_start[5];      // first block of each dimension
  const double *kfac[4];        // [S] dk^2 / (2 m) / N of each dimension
  const cplx<double> *tw[4];    // exp(-2 pi i m / N)
  const cplx<double> *phi;
  cplx<double> *P[4];
  const int *done;
  const ChebyState *cs;
  const cplx<double> *bufs[2];
  int dyn;
};
cudaError_t launch_kin_r2(const KinR2Args &a, cudaStream_t st);

// One OGridNAC element along one dimension d (src/qdlib/OGridNAC.cpp:131-148):
// out += c [f_d d/dx_d phi + d/dx_d (f_d phi)], c = sign/(2 mass), added to
// the kinetic result T_0 phi of the row state, which the combine pass reads.
template <typename T>
struct NacArgs {
  int N, TW, es, ls, tiles_per_hi;
  long long hi_stride, ntiles, npts;
  RadixPlan rp;
  const cplx<T> *tw;
  double kfac;            // dk * c / N: the multiplier of line index q is i q kfac
  const cplx<T> *phi;     // all states; the column state is read
  int col;
  const T *f;             // f_d, grid-shaped
  cplx<T> *out;           // T_0 phi of the row state (read-modify-write)
  const int *done;
  const ChebyState *cs;
  const cplx<T> *bufs[2];
  int dyn;
};

// Point-wise finish of H phi: sum_d T_d phi + potential matrix, then the
// epilogue (H apply output or the Chebyshev recurrence).
template <typename T>
struct CombArgs {
  int S, nd;
  long long npts;
  const cplx<T> *phi;
  const cplx<T> *P[4];
  cplx<T> *out;
  cplx<double> *psi;
  cplx<T> *k0;
  const Couplings *cp;
  const double *coef;
  const T *grids;
  cplx<double> offset, fac, fac_lo, c0p, c1p, coeff;  // fac_lo: rounding residual of fac
  int imag;
  double *partials;
  ChebyCut cut;
  const cplx<T> *bufs[2];  // device-driven term loop: phi = bufs[(i+1)&1], k0 = bufs[i&1]
};

// OGridNablaSq with method="HOFD" (src/qdlib/HOFD.h:124-176): the kinetic
// energy of every state by central finite differences over all dimensions,
// with QDng's neighbour rule (qdg_fdkin.cu), written to out (state stride npts).
static const int kMaxFdHalf = 25;  // order 50 (HOFD_MAXORDER, HOFD.h:17)
// mode 1: OGridHOFD (HOFD.h:372-433), each dimension's lines with zero or
// periodic ends, df = -1 for the first derivative.
template <typename T>
struct FdArgs {
  int nd, S, o2, pbc, mode;
  double df;
  long long npts;
  int n[4];
  long long lo[4];                 // stride of each dimension
  double cf[kMaxFdHalf + 1];       // cf[o2] the point, cf[o2 - k] the neighbours at distance k
  double h[kMaxStates][4];         // per state and dimension: -1/(2 m_d) / dx_d^2, 0 = no term
  const cplx<T> *phi;
  cplx<T> *out;
  const int *done;
  const ChebyState *cs;            // device-driven term loop: phi = bufs[(cs->i + 1) & 1]
  const cplx<T> *bufs[2];
  int dyn;
};

// OGridGMat (src/qdlib/OGridGMat.cpp:313-386) in two launches of line
// passes over all dimensions (qdg_fdkin.cu): pass 0 stores D_i = d/dx_i phi,
// pass 1 stores P_j = -1/2 d/dx_j sum_i G_ij D_i, which the combine pass sums.
template <typename T>
struct GmatArgs {
  int nd, S, pass;
  long long npts;
  DimPass<T> dp[4];                // geometry and twiddles of each dimension (kfac, P unused)
  long long item_start[5];
  double kmul[4];                  // dk_d / N_d (pass 0) or -dk_d / (2 N_d) (pass 1)
  long long gbase[kMaxStates];     // per state: first of its nd (nd + 1) / 2 G grids, -1 = none
  unsigned gmask[kMaxStates];      // per state: bit k set = lower-triangle element k present
  const T *grids;
  const cplx<T> *phi;
  cplx<T> *D[4];
  cplx<T> *P[4];
  const int *done;
  const ChebyState *cs;
  const cplx<T> *bufs[2];
  int dyn;
};

// Grid-wide barrier state of the persistent step kernel (device memory,
// zeroed once; the last block of each barrier resets `count`).
struct GridBarrier {
  unsigned int count;
  unsigned int gen;
  int err;   // a block gave up waiting (bounded spin)
  int pad;
};
// Polls of a barrier flag before a block gives up (~0.3 s with back-off).
static const unsigned int kBarrierSpinLimit = 1u << 22;

// Arithmetic of the persistent step kernel's bulk (phi, T_d phi, potential
// values, FFTs) on grids of two or more dimensions: FP32 (mixed form),
// binary64 (the drop-in form) or double-float (DF64 form).
enum StepBulk { BULK_F32 = 0, BULK_F64 = 1, BULK_DF64 = 2 };

// One Chebyshev step in one cooperative launch (qdg_step.cuh, launched by
// qdg_persistent.cu).
template <typename T>
struct StepArgs {
  int bulk;                  // StepBulk
  int nd, S;
  long long npts;
  DimPass<T> dp[4];          // kinetic passes (P_d outputs); dp[0] also the 1-D line geometry
  long long item_start[5];
  long long line_start[5];   // kinetic lines of dims < d (all states)
  int lmax[4];               // lines of dim d one block transforms at once (shared memory)
  const long long *bstart;   // first line of each block (segment-aligned), or null: even split
  const long long *bstartA;  // two-phase terms: the same for the lines of dimension 0 ...
  const long long *bstartB;  // ... and for the lines of the other dimensions
  int two_phase;             // grids of 3+ dimensions: phi_i stored by dimension 0, loaded by the others
  int TW1;                   // 1-D grids: lines per tile (all states in one block)
  cplx<double> *psi;
  cplx<T> *buf[3];           // rotating phi buffers (phi_{i-2}, phi_{i-1}, phi_i)
  cplx<T> *Pn[2][4];         // kinetic parts T_d phi of the previous / next term (double buffered)
  const Couplings *cp;
  const double *coef;
  const T *grids;
  const dfl *gdf;            // DF64 form: the grids in double-float (the phases' bulk type)
  cplx<double> offset, fac1, fac, ph;  // offset, exp/scaling, 2 exp/scaling, exp(c0 offset)
  const double *a;           // real series coefficients a_i (J_0, 2 J_i / I_0, 2 I_i)
  int order;
  double prec;
  int imag, offim0, diff;
  double *partials;
  ChebyState *cs;
  GridBarrier *bar;
  int trace;                 // record phase times in cs->t_phase
  // pre-scaled point work: dp[].ktab / ktdf hold f T_d, sgrids the scaled
  // potential grids over the entries of scp (lid: the plan entry whose field
  // coefficient applies, or -1), -f offset applied per point as soff_hi + soff_lo
  int scaled, scaled_rt;
  double soff_hi, soff_lo;
  const Couplings *scp;
  const void *sgrids;
};

int cheby_step_max_blocks(int bulk, int S, int nd, int block, size_t smem);

// The Chebyshev step of one 1-D line of N = 8 M points on a cluster of 8
// blocks (qdg_step_cluster.cu), pre-scaled point work.
template <typename T>
struct ClusterStepArgs {
  int N, M;
  RadixPlan rp;              // plan of the M-point transforms
  const cplx<T> *twN;        // N twiddles exp(-2 pi i m/N)
  const T *ktab;             // [N] f kfac min(k, N - k)^2
  const T *V;                // [N] f V
  const cplx<double> *psi;
  cplx<double> *psi_out;
  double soff_hi, soff_lo;   // -f offset as value and residual
  int rt;                    // real time: phi_n = i H' phi ...
  const double *a;
  int order;
  double prec;
  int imag, offim0, diff;
  cplx<double> ph;
  ChebyState *cs;
};
template <typename T>
cudaError_t launch_cheby_step_cluster(const ClusterStepArgs<T> &a, cudaStream_t st);
template <typename T>
size_t cluster_step_smem(int M);
// ProgEigen::AutoCorrEF on the device (qdg_eigen_ac.cu): overlaps of M stored
// steps with step 0, and the integration of the steps at K energies.
cudaError_t launch_step_overlaps(const cplx<double> *T, long long n, int M, cplx<double> *out, int sm_count,
                                 cudaStream_t st);
cudaError_t launch_integrate_steps(const cplx<double> *T, long long n, int M, const cplx<double> *C, int K,
                                   cplx<double> *out, int sm_count, cudaStream_t st);

// Expectation values of filter operators (qdg_filters.cu).
struct PointExpecArgs {
  const cplx<double> *psi;
  long long npts;
  int S;
  const double *grid;  // [npts] weights, or null: the coordinate
  int nd, dim;         // coordinate of dimension dim (dim < 0: the sum over all)
  long long stride[4];
  int n[4];
  double xmin[4], dx[4], scale;
  double *partials;  // [2 gridDim]: weighted sum, plain sum
};
struct SpecExpecArgs {
  const cplx<double> *psi;
  long long npts;
  int S;
  int N;
  long long es;  // element stride of the dimension's lines
  RadixPlan rp;
  const cplx<double> *tw;  // [N] exp(-2 pi i m / N)
  const double *w;         // [S][N] multiplier per k index (with the 1/N)
  double *partials;        // [gridDim]
};
cudaError_t launch_point_expec(const PointExpecArgs &a, int grid, cudaStream_t st);
cudaError_t launch_spectral_expec(const SpecExpecArgs &a, int grid, cudaStream_t st);
size_t spectral_expec_smem(int N);

// One binary64 line of N points on a cluster of 16 or 8 blocks, one real
// component per thread (qdg_step_line64.cu).  line64_cluster_size returns
// the cluster size the device schedules for N, or 0.
int line64_cluster_size(int N);
cudaError_t launch_cheby_line64(const ClusterStepArgs<double> &a, int C, cudaStream_t st);
template <typename T>
cudaError_t launch_cheby_step(const StepArgs<T> &a, int grid, int block, size_t smem, cudaStream_t st);

template <typename T>
cudaError_t launch_kin_all(const KinArgs<T> &a, int grid, int block, size_t smem, cudaStream_t st);
template <typename T>
int kin_all_max_blocks(int block, size_t smem);
template <typename T>
cudaError_t launch_nac(const NacArgs<T> &a, int grid, int block, size_t smem, cudaStream_t st);
template <typename T>
int nac_max_blocks(int block, size_t smem);
template <typename T>
cudaError_t launch_combine(int mode, const CombArgs<T> &a, int grid, int block, cudaStream_t st);
template <typename T>
cudaError_t launch_fd_kinetic(const FdArgs<T> &a, int grid, cudaStream_t st);
template <typename T>
cudaError_t launch_gmat_pass(const GmatArgs<T> &a, int grid, int block, size_t smem, cudaStream_t st);
template <typename T>
int gmat_max_blocks(int block, size_t smem);

// coef[e] for clock step `step` (Laser::Get, src/qdlib/Laser.cpp:125-128).
cudaError_t launch_set_coefs(double *coef, const Couplings *cp, const double *lasers, int laser_nt, long long step,
                             cudaStream_t st);

// Message for qdg_last_error() on the calling thread (qdg_api.cu).
void set_last_error(const std::string &msg);

// Kernels launched by this library in the process (all launchers count;
// replays of captured graphs are added by the caller).
long long launch_counter();
void add_launches(long long n);

// launchers (qdg_kernels.cu)
template <typename T>
cudaError_t launch_pass(int mode, const PassArgs<T> &a, int grid, int block, size_t smem, cudaStream_t st);
template <typename T>
int pass_max_blocks(int mode, int S, int block, size_t smem);

cudaError_t launch_cheby_finalize(ChebyState *cs, const double *partials, int nparts, int first, int term,
                                  int order, double prec, int imag, int offset_imag_zero, cudaStream_t st);
cudaError_t launch_cheby_begin(ChebyState *cs, int order, unsigned long long cond, int use_cond, cudaStream_t st);
cudaError_t launch_cheby_end(ChebyState *cs, cudaStream_t st);

// psi (FP64) -> phi (T) copy (OCheby: ket0->FastCopy(*Psi))
template <typename T>
cudaError_t launch_convert(cplx<T> *dst, const cplx<double> *src, long long n, cudaStream_t st);
template <typename T>
cudaError_t launch_widen(cplx<double> *dst, const cplx<T> *src, long long n, cudaStream_t st);

// Per-state complex dot products sum conj(a)*b: partials[block][state] (re, im).
template <typename T, typename U>
cudaError_t launch_dots(const cplx<T> *a, const cplx<U> *b, int S, long long npts, double *partials, int grid,
                        cudaStream_t st);

// GSPO potential member: psi <- exp(c * M(x)) psi per grid point, where
// M(x) = sum coef_e grid_e(x) over the member's entries (ODMultistate with
// TransformMSD per-point diagonalisation, ODMultistate.cpp:115-182).
// Time-independent potential members: the per-point propagator
// exp(c M(x)) once (S = 2: u00, u01 = u10, u11; otherwise the S diagonal
// factors), then a per-point matrix-vector product each half step.
cudaError_t launch_gspo_umat(cplx<double> *U, int S, long long npts, const Couplings *cp, const double *coef,
                             const double *grids, cplx<double> c, cudaStream_t st);
template <typename T>
cudaError_t launch_gspo_apply(cplx<T> *psi, int S, long long npts, const cplx<double> *U, cudaStream_t st);
template <typename T>
cudaError_t launch_gspo_potential(cplx<T> *psi, int S, long long npts, const Couplings *cp, const double *coef,
                                  const T *grids, cplx<double> c, cudaStream_t st);

// y = a*y + b*x over n complex values (Krylov updates, normalisation).
template <typename T>
cudaError_t launch_lincomb(cplx<T> *y, const cplx<T> *x, cplx<double> a, cplx<double> b, long long n,
                           cudaStream_t st);

// ---- Lanczos with its scalars on the device (no host round trip per
// iteration).  ks holds alpha[order], beta[order], then KS_PSN (the norm of
// psi) and KS_CONV (the order reached); *done stops every later kernel.
enum KsMode { KS_ALPHA = 0, KS_BETA = 1, KS_PSN = 2 };
struct KsFinish {
  int grid, S, mode, slot, order;
  double w;        // grid weight prod dx
  int it;          // KS_BETA: Lanczos iteration (convergence test for it >= 2)
  double dt, tol;  // error estimate dt^(it-2) beta_0 prod beta_i / i < tol * |psi|
};
// ---- Arnoldi with its scalars on the device.  ks holds the Hessenberg
// matrix H (m x m complex, row-major, re/im interleaved), then |psi|;
// ia[0] is the order reached (kept across steps, like the reference's
// _order), done[0]/done[1] as for the Lanczos flags.
struct KaArgs {
  int grid, S, m;
  double w, dt, conv;
};
enum KaOp { KA_H = 0, KA_NORM = 1, KA_PSN = 2, KA_LAST = 3 };
// A finished dot product goes into H[j][col] (KA_H), the subdiagonal with
// the underrun and error tests (KA_NORM, it = col + 1), |psi| (KA_PSN), or
// the last column H[j][order-1] (KA_LAST, skipped for j >= order).
// Krylov launches: a pass over the vectors together with a dot product,
// whose block partials the block taking the last ticket finishes into the
// scalars (then resetting the ticket): <a|b> into the Lanczos / Arnoldi
// scalars; Lanczos y -= alpha x1, y -= beta x2 with |y|^2 -> beta (it >= 2:
// the error estimate, done[1]); y /= beta with done[0] |= done[1]; a
// Gram-Schmidt step y -= H[jc][col] x with the next dot product; the Arnoldi
// normalisation q_it = y / H[it][it-1] with order = it + 1 and
// done[0] |= done[1].  Each is skipped once done[0] is set.
template <typename T, typename U>
cudaError_t launch_dots_ks(const cplx<T> *a, const cplx<U> *b, int S, long long npts, double *partials,
                           const KsFinish &f, double *ks, int *done, unsigned int *ticket, cudaStream_t st);
template <typename T>
cudaError_t launch_ks_lincomb2_dot(cplx<T> *y, const cplx<T> *x1, int i1, const cplx<T> *x2, int i2, int S,
                                   long long npts, double *partials, const KsFinish &f, double *ks, int *done,
                                   unsigned int *ticket, cudaStream_t st);
template <typename T>
cudaError_t launch_ks_scale_commit(cplx<T> *y, const double *ks, int idx, long long n, int *done, unsigned int *ticket,
                                   cudaStream_t st);
template <typename T, typename U>
cudaError_t launch_dots_ka(const cplx<T> *a, const cplx<U> *b, int S, long long npts, double *partials,
                           const KaArgs &ka, int op, int j, int col, double *ks, int *ia, int *done,
                           unsigned int *ticket, cudaStream_t st);
template <typename T>
cudaError_t launch_ka_lincomb_dot(cplx<T> *y, const cplx<T> *x, const cplx<T> *a, int jc, int S, long long npts,
                                  double *partials, const KaArgs &ka, int op, int j, int col, double *ks, int *ia,
                                  int *done, unsigned int *ticket, cudaStream_t st);
template <typename T>
cudaError_t launch_ka_scale_commit(cplx<T> *q, const cplx<T> *buf, const double *ks, int idx, long long n, int it,
                                   int *ia, int *done, unsigned int *ticket, cudaStream_t st);
// dst = q_{order-1} (the basis vector the last column is built from)
template <typename T>
struct KaBasis { const cplx<T> *q[64]; };
template <typename T>
cudaError_t launch_ka_select(cplx<T> *dst, const KaBasis<T> &b, const int *ia, long long n, cudaStream_t st);

// psi = c[0] psi + sum_{i=1}^{m-1} c[i] q_i in FP64, term by term in that order
constexpr int kMaxKrylov = 64;
template <typename T>
struct KCombine {
  const cplx<T> *q[kMaxKrylov];
  cplx<double> c[kMaxKrylov];
  int m;
};
template <typename T>
cudaError_t launch_kcombine(cplx<double> *psi, const KCombine<T> &k, long long n, cudaStream_t st);
// y -= ks[idx] x (x != null) or y *= 1 / ks[idx] (x == null), skipped once *done
template <typename T>
cudaError_t launch_ks_lincomb(cplx<T> *y, const cplx<T> *x, const double *ks, int idx, long long n, const int *done,
                              cudaStream_t st);

}  // namespace qdg
