/*
 * qdg.h -- C ABI of the GB300 propagation engine (libqdg.so).
 *
 * This is the drop-in boundary for QDng's time-stepping hot path. A QDng
 * operator module (a C++ OPropagator subclass built against the QDng
 * headers; qdng_module/OGPUProp.h in this repository) walks its Hamiltonian
 * tree once in Init(WaveFunction*), fills a qdg_hplan_desc and then calls
 * the entry points below once per time step from Apply(WaveFunction*).
 *
 * Plain C: fixed-width integers, doubles and opaque handles, no exceptions,
 * integer status codes.  Complex arrays are interleaved (re, im) doubles,
 * the layout of QDng's dcomplex/cVec (src/math/dcomplex.h); a multistate
 * wave function is stored state after state, each state contiguous with
 * grid dimension 0 fastest (src/qdlib/WFMultistate.cpp:89-140,
 * src/qdlib/GridSystem.h:23-27).
 *
 * Reference files are cited relative to the QDng source tree.
 */
#ifndef QDG_H
#define QDG_H

#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define QDG_ABI_VERSION 3

/* Limits of the reference: MAX_DIMS (src/math/typedefs.h:28),
 * QD_MAX_STATES (src/qdlib/WFMultistate.h:10). */
#define QDG_MAX_DIMS 4
#define QDG_MAX_STATES 64
#define QDG_MAX_GROUPS 8   /* GSPO split members A, B, C ... (MAX_OPS) */

/* Status codes. The QDng module maps them onto the reference exceptions
 * (src/tools/Exception.h): EINVAL -> EParamProblem, EUNSUPPORTED ->
 * EIncompatible, ENONFINITE -> EOverflow, ECUDA/ENOMEM/ETIMEOUT -> EIOError. */
typedef enum qdg_status {
  QDG_OK = 0,
  QDG_EINVAL = 1,        /* bad argument or parameter */
  QDG_ENONFINITE = 2,    /* NaN/Inf norm (Reporter.cpp:112-113) */
  QDG_ETIMEOUT = 3,      /* bounded device wait ran out */
  QDG_ECUDA = 4,         /* CUDA runtime error */
  QDG_ENOMEM = 5,        /* device allocation failed */
  QDG_EUNSUPPORTED = 6,  /* operator tree or grid the engine does not cover */
  QDG_ENOTCONVERGED = 7  /* informational: series not converged (warning in the reference) */
} qdg_status;

/* Hamiltonian term kinds (one per QDng operator class on the path). */
typedef enum qdg_term_kind {
  QDG_TERM_KINETIC = 1,    /* OGridNablaSq: -1/(2m) Laplacian via FFT, or by finite differences with
                              fd_order (src/qdlib/OGridNablaSq.cpp:28-111) */
  QDG_TERM_POTENTIAL = 2,  /* OGridPotential: V(x) psi (src/qdlib/OGridPotential.cpp:134-142) */
  QDG_TERM_DIPOLE = 3,     /* OGridDipole: -mu(x) E(t) psi (src/qdlib/OGridDipole.cpp:46-60) */
  QDG_TERM_NAC = 4,        /* OGridNAC: sign/(2 mass) sum_d [f_d d/dx_d psi + d/dx_d (f_d psi)]
                              (src/qdlib/OGridNAC.cpp:131-148), derivatives by FFT (OGridNabla.cpp:76-95) */
  QDG_TERM_GOBBLER = 5,    /* OGobbler (src/qdlib/OGobbler.cpp:30-84,176-204): a diagonal grid term W(x)
                              = gain x (product of Butterworth filters); laser = 1 makes it a negative
                              imaginary potential, H psi += -i W psi (nip="true"), else H psi += W psi;
                              mass[0] = gain (Emax = gain, Emin = -i gain with nip, else 0).
                              Not a member type of GSPO (OGSPO.cpp:71-85 needs ODSpace operators). */
  QDG_TERM_GMAT = 6,       /* OGridGMat (src/qdlib/OGridGMat.cpp:307-386): -1/2 sum_ij d/dx_j G_ij(x) d/dx_i,
                              first derivatives by FFT (Diff.cpp:223-272); diagonal only.  grid = index of
                              the first of ndims (ndims + 1) / 2 grid arrays G_ij, lower triangle row by
                              row ((0,0), (1,0), (1,1), (2,0), ...); flags holds two bits per element k =
                              i (i + 1) / 2 + j: 0 = no element ("x" in Gdef, or coup="false" off the
                              diagonal), 1 = a grid, 2 = a constant (its grid array holds the constant;
                              Emax and Emin then follow OGridGMat.cpp:250-305 for constants).
                              Not a member type of GSPO (not an ODSpace operator). */
  QDG_TERM_HOFD = 7        /* OGridHOFD (src/qdlib/OGridHOFD.cpp:32-128, HOFD.h:188-211,372-433): central
                              finite differences of order fd_order along each dimension with zero (or,
                              flags bit 0, periodic) boundaries; flags bit 1: first derivative (deriv=1),
                              else second; laser = the dimension it acts on (dim), -1 = all; with flags
                              bit 2 the "mass" parameter is given in mass[] and the factor is
                              -1/(2 mass[ndims-1]) for every dimension (OGridHOFD.cpp:74-91), else 1.
                              Diagonal only; not a member type of GSPO. */
} qdg_term_kind;

/* Arithmetic of a plan.  FP64 is the drop-in form: every value (psi, phi_n,
 * H phi, the FFTs, potentials, coefficients and reductions) is IEEE binary64,
 * as in the reference.  MIXED keeps H phi, phi_n and the FFTs in FP32 and
 * the series coefficients, the psi accumulator, norms, energies, overlaps
 * and Krylov scalars in binary64.  DF64 is binary64 except for the
 * Chebyshev step of grids with two or more dimensions, whose phi_n, H phi,
 * potential values and FFTs are double-float (an unevaluated sum of two
 * FP32 numbers: about 48 significant bits and the FP32 exponent range;
 * wave-function values below ~1e-38 of the scale are lost), with psi and
 * the reductions binary64. */
typedef enum qdg_precision {
  QDG_PREC_FP64 = 0,
  QDG_PREC_MIXED = 1,
  QDG_PREC_DF64 = 2
} qdg_precision;

/* Grid description: QDng GridSystem (src/qdlib/GridSystem.cpp:195-215).
 * dx = (xmax - xmin)/(n - 1); dk = 2 pi/(xmax - xmin + dx) (src/qdlib/Kspace.h:20-23). */
typedef struct qdg_grid {
  int32_t ndims;
  int32_t n[QDG_MAX_DIMS];
  double xmin[QDG_MAX_DIMS];
  double xmax[QDG_MAX_DIMS];
} qdg_grid;

/* One operator of the Hamiltonian matrix H_{row,col}.
 * The matrix is a QDng "Multistate" of "Sum"s (src/qdlib/OMultistate.cpp:206-231,
 * src/qdlib/OSum.cpp:53-60); an off-diagonal term given at (row, col) is also
 * applied at (col, row) (hermitian pointer copy, OMultistate.cpp:122-132)
 * unless the matrix is non-hermitian (qdg_hplan_desc.nonhermitian, or terms
 * given at both (i, j) and (j, i), OMultistate.cpp:52-53).
 * A single-state Hamiltonian is a plain Sum (nstates = 1). */
typedef struct qdg_hterm {
  int32_t kind;                  /* qdg_term_kind */
  int32_t row, col;              /* matrix element; KINETIC must be diagonal */
  int32_t grid;                  /* POTENTIAL/DIPOLE: index of the grid array in grid_data;
                                    NAC: index of f_0, with f_1 .. f_{ndims-1} following it */
  int32_t laser;                 /* DIPOLE: index of the field in laser_data */
  int32_t group;                 /* GSPO split member: 0 = "A" (full step), 1 = "B", ... (OGSPO.cpp:71-85) */
  double mass[QDG_MAX_DIMS];     /* KINETIC: masses per dimension, all > 0;
                                    NAC: mass[0] = the reduced mass (1 for N-D, OGridNAC.cpp:83-85) */
  double sign;                   /* NAC: sign of the element (+1 or -1; 0 means the default +1) */
  int32_t fd_order;              /* KINETIC: 0 = FFT (OGridNablaSq method="FFT"); an even order 2..50 =
                                    central finite differences (method="HOFD", Diff.cpp:203-218 ->
                                    HOFD::Diff over all dimensions, src/qdlib/HOFD.h:124-176) */
  int32_t flags;                 /* KINETIC with fd_order: 1 = periodic boundaries (pbc="true"; grids
                                    of one dimension only); GMAT: the element sources (see above) */
} qdg_hterm;

typedef struct qdg_hplan_desc {
  qdg_grid grid;
  int32_t nstates;
  int32_t nterms;
  const qdg_hterm *terms;
  int32_t ngrids;
  const double *grid_data;       /* ngrids * npoints doubles, dim 0 fastest */
  int32_t nlasers;
  int32_t laser_nt;              /* samples per field; E(step) = laser[step] (Laser.cpp:125-128) */
  const double *laser_data;      /* nlasers * laser_nt doubles */
  int32_t nonhermitian;          /* Multistate "nonhermitian" (OMultistate.cpp:83-85): no (col, row) copies */
} qdg_hplan_desc;

/* Per-step observables of QDng's Reporter (src/Reporter.cpp:65-154). */
typedef struct qdg_observables {
  double norm2;                  /* <psi|psi> with dx weights (Norm()^2) */
  double pops[QDG_MAX_STATES];   /* per-state <psi_i|psi_i> */
  double energy;                 /* Re <psi|H|psi> (Operator::Expec) */
  double autocorr_re;            /* <psi(t)|psi0> (Reporter.cpp:137) */
  double autocorr_im;
} qdg_observables;

/* Propagator information after Init (the values the reference stores in its
 * ParamContainer, OCheby.cpp:470-491). */
typedef struct qdg_prop_info {
  int32_t kind;                  /* 1 Cheby, 2 GSPO, 3 SIL, 4 Arnoldi */
  int32_t order;                 /* Cheby recursion order / Krylov max order */
  double scaling;                /* Cheby Delta E (scaling) */
  double offset_re, offset_im;   /* Cheby energy offset */
  double exponent_re, exponent_im; /* OPropagator::Exponent() = c0 */
} qdg_prop_info;

typedef struct qdg_plan qdg_plan;  /* device H-plan: grids, fields, kinetic tables */
typedef struct qdg_wf qdg_wf;      /* device wave function (all states) */
typedef struct qdg_prop qdg_prop;  /* a propagator bound to a plan */

/* ---- errors ---------------------------------------------------------- */

/* Text of the last error on the calling thread ("" if none). */
const char *qdg_last_error(void);
int32_t qdg_abi_version(void);

/* ---- plan: replaces the operator tree's Init(WaveFunction*) ------------ */

/* Builds the device H-plan: copies grid arrays and fields to HBM, checks the
 * tree (OGridNablaSq::Init masses > 0, OGridPotential::Init grid match,
 * Laser::Clock dt), computes Emax/Emin host-side (OSum.cpp:28-51,
 * OMultistate.cpp:163-203, OGridNablaSq.cpp:89-106, OGridPotential.cpp:124-132,
 * OGridDipole.cpp:36-44). precision is a qdg_precision. */
qdg_status qdg_plan_create(const qdg_hplan_desc *desc, int32_t precision, qdg_plan **out);
qdg_status qdg_plan_destroy(qdg_plan *plan);
/* Operator::Emax()/Emin() of the whole Hamiltonian (complex). */
qdg_status qdg_plan_erange(const qdg_plan *plan, double emax[2], double emin[2]);
/* Run the plan's work on a caller CUDA stream (cudaStream_t passed as void*;
 * NULL = the plan's own stream). */
qdg_status qdg_plan_set_stream(qdg_plan *plan, void *cuda_stream);
qdg_status qdg_plan_synchronize(qdg_plan *plan);

/* ---- wave functions ---------------------------------------------------- */

qdg_status qdg_wf_create(qdg_plan *plan, qdg_wf **out);
qdg_status qdg_wf_destroy(qdg_wf *wf);
/* Host <-> device copies of nstates*npoints complex128 values. */
qdg_status qdg_wf_upload(qdg_wf *wf, const double *host_psi);
qdg_status qdg_wf_download(const qdg_wf *wf, double *host_psi);
qdg_status qdg_wf_copy(qdg_wf *dst, const qdg_wf *src);

/* ---- Hamiltonian application ------------------------------------------ */

/* out = H(step) in (Operator::Apply(dest, src), src/qdlib/Operator.h:276). */
qdg_status qdg_h_apply(qdg_plan *plan, const qdg_wf *in, qdg_wf *out, int64_t step);

/* Reporter::Analyze values of psi at clock step `step` (psi0 may be NULL). */
qdg_status qdg_observables_compute(qdg_plan *plan, const qdg_wf *psi, const qdg_wf *psi0,
                                   int64_t step, qdg_observables *out);

/* ---- expectation filters: FiltersList expec / expeconly
 * (src/FiltersList.cpp:289-308), renormalised by <psi|psi> as ProgPropa
 * sets them (ProgPropa.cpp:260,276). Values are Re <psi|O|psi> / <psi|psi>. */

/* OGridPosition (OGridPosition.cpp:41-80): x of dimension dim (dim < 0: the
 * sum over all dimensions), times scale. */
qdg_status qdg_expec_position(qdg_plan *plan, const qdg_wf *psi, int32_t dim, double scale, double *out);
/* GridMomentum = OGridNabla(momentum) (OGridNabla.cpp:76-95, Kspace.cpp:60-96):
 * k of dimension dim (dim < 0: the sum over all dimensions), times factor. */
qdg_status qdg_expec_momentum(qdg_plan *plan, const qdg_wf *psi, int32_t dim, double factor, double *out);
/* The kinetic terms of the plan (OGridNablaSq): sum of their expectation values. */
qdg_status qdg_expec_kinetic(qdg_plan *plan, const qdg_wf *psi, double *out);
/* A real diagonal grid of the plan (grid index into grid_data) on every
 * state: OGridPotential / OGobbler (no nip) as a filter operator. */
qdg_status qdg_expec_grid(qdg_plan *plan, const qdg_wf *psi, int32_t grid, double *out);
/* OProjection (OProjection.cpp:133-149): sum_k |<phi_k|psi>|^2 over nfun
 * functions given as host arrays of the wave function's size (complex128). */
qdg_status qdg_expec_projection(qdg_plan *plan, const qdg_wf *psi, const double *const *funcs, int32_t nfun,
                                double *out);

/* ---- propagators: replace OCheby / OGSPO / OSIL / OArnoldi ------------- */

/* name: "Cheby", "GSPO", "SIL" or "Arnoldi"; params: the XML attributes of
 * the <propagator> node as "key=value" pairs separated by ';' or spaces
 * (Cheby: order, prec, scaling, Emax, Emax_im, Emin, Emin_im -- OCheby.cpp:53-61,386-401;
 * SIL: order, err -- OSIL.cpp:38-52; Arnoldi: order, conv -- OArnoldi.cpp:39-59).
 * dt is the clock's time step; direction flags mirror OPropagator::Forward/
 * Backward/ImaginaryTime (src/qdlib/OPropagator.h:62-131). */
qdg_status qdg_prop_create(qdg_plan *plan, const char *name, const char *params,
                           double dt, int32_t imaginary_time, int32_t backward,
                           qdg_prop **out);
qdg_status qdg_prop_destroy(qdg_prop *prop);
/* OPropagator::Init(WaveFunction*): coefficients, order, scratch buffers. */
qdg_status qdg_prop_init(qdg_prop *prop);
qdg_status qdg_prop_get_info(const qdg_prop *prop, qdg_prop_info *info);
/* Cheby coefficients after Init (complex, `order` entries) including the
 * exp(c0*offset) phase used in the sum (OCheby.cpp:107,122). */
qdg_status qdg_prop_get_coeffs(const qdg_prop *prop, double *coeffs, int32_t capacity);

/* One time step psi <- U(step) psi on device (OPropagator::Apply(Psi)).
 * `step` is QDClock::TimeStep() at the call, used by time-dependent terms.
 * terms_used (may be NULL) receives the Chebyshev terms / Krylov basis size
 * actually used. */
qdg_status qdg_prop_apply(qdg_prop *prop, qdg_wf *psi, int64_t step, int32_t *terms_used);

/* The same step with the wave function in host memory (the drop-in call:
 * host psi stays authoritative, upload before and download after). */
qdg_status qdg_prop_apply_host(qdg_prop *prop, qdg_wf *scratch, double *host_psi,
                               int64_t step, int32_t *terms_used);

/* The same drop-in step with the wave function as one host block per state
 * (state_psi[s]: npoints complex128 values of state s), the layout of QDng's
 * WFMultistate (src/qdlib/WFMultistate.cpp:89-140): no gather into one
 * buffer on the host. */
qdg_status qdg_prop_apply_host_states(qdg_prop *prop, qdg_wf *scratch, double *const *state_psi,
                                      int64_t step, int32_t *terms_used);

/* `nsteps` consecutive steps on device starting at clock step `step0`
 * (ProgPropa.cpp:317-327 without the per-step report). */
qdg_status qdg_prop_run(qdg_prop *prop, qdg_wf *psi, int64_t step0, int32_t nsteps,
                        int64_t *terms_total);

/* Eigenstates by imaginary-time relaxation: ProgEigen::ImagTimeEF
 * (src/ProgEigen.cpp:318-409) with OProjection (OProjection.cpp:133-149)
 * and, with diag != 0, DiagBasis (ProgEigen.cpp:94-138).  prop must be an
 * imaginary-time propagator (QDng builds it backward, ProgEigen.cpp:692-693).
 * Every function starts from the normalised psi_init (host, nstates*npoints
 * complex128) and is stepped, projected against the ones already found and
 * normalised until |1 - <psi_old|psi>| <= convergence or maxsteps.  Outputs
 * (host): e_raw[nef] = <psi_i|H|psi_i>, e_diag[nef] (eigenvalues of H in the
 * basis, or e_raw without diag), steps[nef] (may be NULL), efs
 * (nef * nstates*npoints complex128, may be NULL): the diagonalised basis. */
qdg_status qdg_eigen_imag(qdg_prop *prop, const double *psi_init, int32_t nef, int32_t maxsteps,
                          double convergence, int32_t diag, double *efs, double *e_raw, double *e_diag,
                          int32_t *steps);

/* ProgEigen::AutoCorrEF (src/ProgEigen.cpp:414-600) with a real-time
 * propagator: psi_init (host, as given; the reference normalises it on
 * input) is propagated for nsteps - 1 steps and every step is kept in device
 * memory; a_s = <psi_s|psi_init> (a_0 = 1), Hann window when win != 0,
 * forward FFT, peaks of |spectrum| by QDng's PeakFinder (mean + tol sigma
 * over the spectrum, or over windows of +-width around local maxima when
 * width > 0); for each peak at E = index dw (index - nsteps above the middle,
 * dw = 2 pi / (dt nsteps)) the eigenfunction psi_0 + sum_s exp(i E s dt)
 * psi_s, normalised, and its energy Re <psi|H|psi>.  nef_out = the number of
 * peaks; the first max_nef are returned in energies, efs (max_nef x
 * nstates*npoints complex128, may be NULL) and the spectrum (nsteps
 * complex128, may be NULL). */
qdg_status qdg_eigen_autocorr(qdg_prop *prop, const double *psi_init, int32_t nsteps, double tol, int32_t width,
                              int32_t win, int32_t max_nef, double *energies, int32_t *nef_out, double *efs,
                              double *spectrum);

/* ProgEigen::LanczosEF (src/ProgEigen.cpp:604-648) + DiagBasis with an
 * Arnoldi propagator: the Krylov basis of psi_init (OArnoldi::BuildLZB, the
 * propagator's order and convergence), the Ritz values and functions of its
 * Hessenberg matrix, then H diagonalised in that basis.  nef_out = the basis
 * size; the first max_nef values ascending in e_raw (Ritz values) and e_diag,
 * and the diagonalised functions in efs (max_nef x nstates*npoints
 * complex128, may be NULL). */
qdg_status qdg_eigen_lanczos(qdg_prop *prop, const double *psi_init, int32_t max_nef, double *e_raw,
                             double *e_diag, int32_t *nef_out, double *efs);

/* ---- batched ensemble of independent wavepackets ------------------------ */

/* One member: a single-state Hamiltonian Sum(GridNablaSq, GridPotential,
 * GridDipole x laser) on its own 1-D or 2-D grid -- the operator tree of
 * QDng's laser-driven grid propagations (tests/TGPL-IR-Pulse-Cheby.qdi.in) --
 * propagated with OCheby's series (src/qdlib/OCheby.cpp:92-198, 358-493).
 * Arrays are host memory, npoints doubles (laser: laser_nt samples, E(step)
 * = laser[step], Laser.cpp:125-128); dipole/laser may be NULL. */
typedef struct qdg_ensemble_member {
  qdg_grid grid;
  double mass[QDG_MAX_DIMS];
  const double *potential;
  const double *dipole;
  const double *laser;
  int32_t laser_nt;
} qdg_ensemble_member;

typedef struct qdg_ensemble qdg_ensemble;

/* Builds the device image of n members, each with its own Chebyshev series
 * (params: the OCheby attributes, shared by all members; forward real time
 * with time step dt).  Members run in one persistent launch, taken from a
 * device queue in descending cost order. */
qdg_status qdg_ensemble_create(const qdg_ensemble_member *members, int32_t n, double dt, const char *params,
                               int32_t precision, qdg_ensemble **out);
qdg_status qdg_ensemble_destroy(qdg_ensemble *e);
/* psi of all members, concatenated in member order (complex128). */
qdg_status qdg_ensemble_upload(qdg_ensemble *e, const double *psi_all);
qdg_status qdg_ensemble_download(const qdg_ensemble *e, double *psi_all);
/* nsteps time steps of every member from clock step step0 (ProgPropa.cpp:317-327);
 * terms_total receives the Chebyshev terms summed over members and steps. */
qdg_status qdg_ensemble_run(qdg_ensemble *e, int64_t step0, int32_t nsteps, int64_t *terms_total);
/* Series parameters of member i after create (order, scaling, offset). */
qdg_status qdg_ensemble_member_info(const qdg_ensemble *e, int32_t i, qdg_prop_info *info);
/* Schedule of the last qdg_ensemble_run: for every member its start and end
 * on the GPU clock in ns relative to the launch's first start
 * (start_end[2 i], start_end[2 i + 1]) and the block that ran it (block[i],
 * may be NULL).  A tuning aid for the work-queue order; no counterpart in
 * the reference. */
qdg_status qdg_ensemble_timeline(const qdg_ensemble *e, int64_t *start_end, int32_t *block);

/* ---- engine instrumentation (no counterpart in the reference) ---------- */

/* Kernels this library has launched in the process so far. */
int64_t qdg_kernel_launches(void);
/* Time every line-pass launch of the plan with CUDA events on its stream. */
qdg_status qdg_profile_enable(qdg_plan *plan, int32_t on);
/* Per pass mode (0 kinetic first, 1 kinetic middle, 2 H apply, 3 Chebyshev
 * first term, 4 Chebyshev term, 5 split-operator kinetic): summed device ms
 * and launch counts since the last read; resets the counters. */
qdg_status qdg_profile_read(qdg_plan *plan, double ms[8], int64_t launches[8]);
/* Chebyshev persistent step kernel, profiled steps since the last call:
 * ns spent by block 0 in its own kinetic work, waiting at the barrier after
 * it, in its own point work, and waiting at the norm barrier; resets them. */
qdg_status qdg_prop_phase_times(qdg_prop *prop, double ns[4]);
/* Failure-path test aid: the next persistent step kernel launched for this
 * plan finds its grid barrier's arrival count preset so that no arrival
 * completes it.  Every block then waits out its bounded spin, raises the
 * barrier's error flag and leaves; the step returns QDG_ETIMEOUT, the
 * barrier is reset, and psi must be restored by the caller (the step was
 * cut short).  No device wait is unbounded and nothing faults. */
qdg_status qdg_plan_inject_barrier_stall(qdg_plan *plan);

/* ---- FFT schedules (the FFTW planning/wisdom counterpart) --------------- */

/* The line transforms of a plan (context 0) or of an ensemble member
 * (context 1) of line length n and precision (a qdg_precision) use a radix
 * order and, in the persistent step kernel, a number of lines per batch.
 * They come from the autotuner's table, fft_schedules.txt next to the
 * library (or the file QDG_FFT_SCHEDULES names), written by
 * qdng_gb300/autotune.py after timing the candidates on the GPU; sizes
 * without an entry use the greedy order (largest radices first).  This is
 * the role of FFTW's planning and wisdom in the reference
 * (src/fft/FFTGlobal.cpp:26-84, src/fft/fft.cpp:98-122).
 * _set installs an override for plans and ensembles created afterwards in
 * this process (radices from {2, 3, 4, 5, 8, 16} whose product is n; lines
 * 0 = automatic, up to 64); _get returns the schedule a new plan would use;
 * _reset drops the overrides and, with use_table = 0, ignores the table
 * too (greedy orders). */
qdg_status qdg_fft_schedule_set(int32_t context, int32_t n, int32_t precision, const int32_t *radices,
                                int32_t nstages, int32_t lines);
qdg_status qdg_fft_schedule_get(int32_t context, int32_t n, int32_t precision, int32_t *radices,
                                int32_t *nstages, int32_t *lines);
qdg_status qdg_fft_schedule_reset(int32_t use_table);

/* ---- H psi without device allocation ------------------------------------ */

/* Bytes of the library's static device scratch used by qdg_h_apply_noalloc
 * (held on every GPU that loads the library until the process exits). */
#define QDG_NOALLOC_SCRATCH_BYTES (8 << 20)

/* out = H(step) in, like qdg_h_apply, for callers that cannot allocate
 * device memory (frameworks whose caching pool owns all device memory,
 * plug-ins that must leave the process's allocation state alone, loops
 * where the implicit device synchronisation of cudaMalloc is too costly).  It calls no cudaMalloc/cudaFree: desc is a
 * host struct whose grid_data and laser_data point to DEVICE arrays, psi_in
 * and psi_out are device arrays of nstates*npoints complex128, and all
 * scratch lives in one static device array of QDG_NOALLOC_SCRATCH_BYTES.
 * Problems needing more scratch (ndims > 1: ndims * nstates * npoints * 16
 * bytes plus small tables) fail with QDG_EINVAL.  FP64 only.  Work is
 * queued on cuda_stream (NULL: the legacy default stream) without
 * synchronising.  Every call shares the scratch array: calls whose kernels
 * overlap on the GPU race, so serialise them on one stream.  The first call
 * on a device looks up the array's address with that device current and
 * keeps it; a cudaDeviceReset ends the context that holds the array, so a
 * process that resets a device must not call this entry point on it again.  This
 * entry point has no counterpart in the reference. */
qdg_status qdg_h_apply_noalloc(const qdg_hplan_desc *desc, const double *psi_in, double *psi_out,
                               int64_t step, void *cuda_stream);

#ifdef __cplusplus
}
#endif

#endif /* QDG_H */
