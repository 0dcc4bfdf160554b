/*
 * heom_gb300.h -- C ABI of the GB300 (sm_103a) HEOM Liouvillian library.
 *
 * Drop-in for the sparse-mode hot path of HEOM-QUICK2.  The reference routines
 * keep their arguments in Fortran modules; here they are passed once through
 * heom_tables (a plain view of the module arrays) and live in an opaque context
 * that owns the device copies.  All entry points return 0 on success or a
 * negative HEOM_E* code and never abort; heom_last_error() describes the failure.
 * A context is single-stream and not thread-safe, like the reference routines
 * (whose SAVE counters make them non-reentrant).  Every entry point makes the
 * context's device current for the duration of the call and gives the caller's
 * current device back on return.
 *
 * Complex data are double _Complex / float _Complex, i.e. interleaved (re, im),
 * which is complex(c_double_complex) in ISO_C_BINDING.  Table values keep the
 * reference conventions: 1-based ADO, drawer and matrix indices, column-major
 * matrices.
 */
#ifndef HEOM_GB300_H
#define HEOM_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* 4: heom_grad_opts.precision, heom_solve_opts.interleave (in place of a reserved field),
 *    heom_batch_set_tiers, HEOM_PROP_CHEBYSHEV_MIXED, heom_td_gradient_ex
 * 5: heom_solve_opts.lane_instances, heom_bench_inner_layout, heom_tuned_layout */
#define HEOM_ABI_VERSION 5

enum {
    HEOM_OK = 0,
    HEOM_E_ARG = -1,        /* invalid argument / inconsistent table */
    HEOM_E_CUDA = -2,       /* CUDA runtime failure (no device, launch error, ...) */
    HEOM_E_NOMEM = -3,      /* host or device allocation failed */
    HEOM_E_UNSUPPORTED = -4,/* option the library does not implement (e.g. lad, lsimple) */
    HEOM_E_BREAKDOWN = -5,  /* TFQMR breakdown (reference ierr = 8) */
    HEOM_E_NOCONV = -6,     /* iteration limit reached before convergence */
    HEOM_E_TIMEOUT = -7     /* a bounded device-side wait gave up */
};

/* Precision of the steady-state solver. */
/* Solver precision.  MIXED: inner TFQMR in FP32x2 (double-float, about 48 significant
 * bits, on the FP32 pipe) on a regularised operator, refined with FP64 residuals.
 * MIXED_FP32: the same with plain FP32 inner arithmetic; it converges only where the
 * operator's conditioning times 6e-8 stays well below one (the single-orbital model at
 * T = 0.1 does, the double dot does not). */
enum { HEOM_PREC_FP64 = 0, HEOM_PREC_MIXED = 1, HEOM_PREC_MIXED_FP32 = 2, HEOM_PREC_FP64_REFINED = 3 };
/* FP64_REFINED: the refinement of MIXED with FP64 inner solves; slower, for reference
 * solutions below the FP64 TFQMR floor (||b - A x|| down to about 1e-13). */

/* View of the module data the reference keeps for the sparse path
 * (module/matmod.f90:4-52, module/sparsemod.f90:34-42, include/common).  The
 * arrays are read during heom_ctx_create only; the caller keeps ownership. */
typedef struct {
    int32_t norbs, nspin, nalf, ncor;       /* nvar = 2*norbs*nspin*nalf*ncor drawers */
    int32_t ntier;                          /* reference ntier = truncation tier + 1 */
    int32_t nrho;                           /* (2*nspin)^norbs */
    int32_t nams;                           /* nonzeros per a_{ms} */
    int32_t lscreen;                        /* drawers of screened operators are absent */
    int64_t nunk, lall, lunk_spa;
    /* per drawer (nvar entries, reference order sgn > spin > orbs > alf > cor) */
    const double _Complex *cgamma;          /* damping rate of each drawer */
    const double *dipm;                     /* +1 / -1 */
    const int32_t *mpm, *morbs, *mspin, *ilead, *mcor;
    const int32_t *indexdraw;               /* first-tier ADO of a + drawer (0 if screened) */
    /* cb, cd laid out as cb(norbs, nspin, ncor, nalf, 2), column-major */
    const double _Complex *cb, *cd;
    const double *eleadinfty;               /* (nalf, nspin): lead shift as t -> infinity */
    /* hierarchy tables (main/buildcoefindex.f90) */
    const int64_t *nfirst, *nlast;          /* ntier entries */
    const int64_t *ifirst;                  /* ntier entries */
    const int32_t *indextable;              /* drawer tuples of every ADO */
    const int64_t *index_coef_ref;          /* nunk entries: first coupling of each ADO */
    const int64_t *indexcoef;               /* lall: target ADO (1-based) */
    const int8_t *itypecoef, *ifactfcoef, *ifactrcoef;
    /* a_{ms} in signed COO (main/arrangeoperator.f90): (nams, norbs, nspin) */
    const int32_t *rowams, *colams, *sgnams;
    /* system Hamiltonian in internal units (energy / hbar), nrho x nrho */
    const double _Complex *hs;
    /* per-ADO sparsity (fermion/prelude_spa.f90) */
    const int32_t *nnz_spa;
    const int64_t *ind_spa;
    const int32_t *irow_spa, *icol_spa;
} heom_tables;

/* ------------------------------------------------------------------------- */
/* Model builder.  Stands in for the Fortran driver's set-up when the caller has
 * no Fortran (main/evaluatepara.f90, buildoperator, calchs, ball2drawer,
 * buildcoefindex, prelude_spa): it produces tables identical to the reference's
 * for the Lorentzian-PSD input subset below. */
typedef struct {
    int32_t norbs, nspin, nalf, nmats, ntier;
    double bandwidth[2], linewidth[2][3], temperature[2], engyshift[2][2];
    int32_t lscreen, doubledot;
    int32_t model;            /* 1 $para1, 4 $para4, 5 Kanamori (lreadhs data), 9 hs given */
    double eup, edown, uu;
    double e1up, e1down, e2up, e2down, uu1, uu2, u12, t12;
    double kan_u, kan_j, kan_eps;
    const double _Complex *hs_in;     /* model 9: nrho*nrho, internal units */
    double tchar[2][2];               /* fieldtype = 0 switch-on time of the lead shift */
    /* Prony scheme (psfjob, main/zpout_psf.f90; cb, cd, cgama at main/evaluatepara.f90:1993-2000):
     * npsf > 0 replaces the Drude pole and the Pade terms by npsf fitted exponentials (nmats is
     * then taken as npsf).  The caller supplies the fitted table: psf_coef and psf_pole (zcoef and
     * zpole of zpout_psf; one set of poles serves both signs), the fit's reference temperature
     * tpsf and its band ratio rpsf (band half-width rpsf * T, centred at 0).  The reference's
     * built-in itype_psf tables are not part of this library. */
    int32_t npsf;
    double tpsf, rpsf;
    const double _Complex *psf_coef, *psf_pole;
} heom_params;

typedef struct heom_model heom_model;

int  heom_model_build(const heom_params *p, heom_model **out);
void heom_model_destroy(heom_model *m);
/* Borrowed view of the built tables (valid while the model lives). */
const heom_tables *heom_model_tables(const heom_model *m);
/* Boltzmann reduced density matrix at the lead-1 temperature on the RDO pattern,
 * zero ADOs (main/analyze_hs.f90:144-176 + fermion/initialize1_spa.f90). rho: lunk_spa. */
int  heom_model_initial_guess(const heom_model *m, double _Complex *rho);
/* Lead shifts / amplitudes of the model (nalf x nspin, column-major, internal units). */
int  heom_model_field(const heom_model *m, double *amps, double *tchar);
/* Copy a named derived quantity: "hs", "dhs_deps", "dhs_du" (nrho^2 complex),
 * "cpcoef", "cppole", "amsori" (dense a_{ms}, real). Returns HEOM_E_ARG for an unknown name. */
int  heom_model_get(const heom_model *m, const char *name, void *dst);

/* ------------------------------------------------------------------------- */
/* Context: device-resident plan of one model.  */
typedef struct heom_ctx heom_ctx;

typedef struct {
    int32_t device;           /* CUDA device ordinal */
    int32_t build_adjoint;    /* also build the transpose (adjoint) plan */
    const double *amps;       /* (nalf, nspin) lead-shift amplitude for heom_calcderiv; NULL = eleadinfty */
    const double *tchar;      /* (nalf, nspin) switch-on time, NULL = 0 (step) */
    const double _Complex *dhs[4];  /* optional parameter derivatives of hs for gradients */
} heom_ctx_opts;

int  heom_ctx_create(const heom_tables *t, const heom_ctx_opts *opts, heom_ctx **out);
void heom_ctx_destroy(heom_ctx *ctx);
int64_t heom_ctx_lunk(const heom_ctx *ctx);
const char *heom_last_error(void);

/* y = A x  (calc_ax_tfqmr_spa_omp, tfqmr_double/calc_ax_tfqmr_spa_omp.f90:1).
 * x, y: ldim+1 complex (host memory); ldim must equal lunk_spa; y[ldim] = Tr rho0. */
int heom_calc_ax(heom_ctx *ctx, int64_t ldim, const double _Complex *x, double _Complex *y);
/* dRho/dt at time t (calcderiv_spa_omp, td/calcderiv_spa_omp.f90:1): x, y lunk entries. */
int heom_calcderiv(heom_ctx *ctx, double t, const double _Complex *x, double _Complex *y);
/* y = A^H x, the adjoint of heom_calc_ax in the real inner product <u,v> = Re(u^H v)
 * (the role calc_atrx_bicg_omp, bicg/calc_atrx_bicg_omp.f90:1, plays for the dense
 * BiCG path, here on the sparse layout). x, y: ldim+1 complex. */
int heom_calc_atrx(heom_ctx *ctx, int64_t ldim, const double _Complex *x, double _Complex *y);
/* Device-pointer variants (pointers in the context's device memory space, stream 0 order). */
int heom_calc_ax_dev(heom_ctx *ctx, const void *dx, void *dy);
int heom_calc_atrx_dev(heom_ctx *ctx, const void *dx, void *dy);
int heom_calc_ax_fp32_dev(heom_ctx *ctx, const void *dx, void *dy);
/* The FP32x2 apply of the mixed-precision inner solves (the unregularised operator): dx, dy
 * hold lunk_spa + 1 values as float4 (re_hi, im_hi, re_lo, im_lo), each value hi + lo.  No
 * reference counterpart (the reference has no mixed precision); it exposes the packed
 * double-float kernel for checks against the FP64 apply. */
int heom_calc_ax_fp32x2_dev(heom_ctx *ctx, const void *dx, void *dy);
/* The operator of the mixed-precision inner solves: the regularised operator (A on the
 * Hermitian part of the RDO block, the regularising blocks on the rest, the trace unknown on
 * the RDO diagonal) with, when precond != 0, every row of ADO n scaled by the inner
 * preconditioner 1 / (|sum of its damping rates| + ||H||_inf).  precision selects the number
 * type of dx, dy (lunk_spa + 1 values each): HEOM_PREC_MIXED float4 (FP32x2, as in
 * heom_calc_ax_fp32x2_dev), HEOM_PREC_MIXED_FP32 float2, HEOM_PREC_FP64(_REFINED) double2.
 * No reference counterpart; it lets the inner arithmetic be checked against FP64. */
int heom_calc_ax_inner_dev(heom_ctx *ctx, int32_t precision, int32_t precond, const void *dx, void *dy);

/* Steady state by TFQMR (solve_tfqmr, tfqmr_double/solve_tfqmr.f90:1). */
typedef struct {
    double crit;              /* ||b - A x|| target (reference $converge crit) */
    int32_t maxit0;           /* reference maxit0 (TFQMR limit = maxit0/2) */
    int32_t precision;        /* HEOM_PREC_FP64, HEOM_PREC_MIXED or HEOM_PREC_MIXED_FP32 */
    double inner_tol;         /* MIXED*: an inner solve stops at ||r|| <= max(crit, inner_tol ||r0||),
                                 r0 its FP64 right-hand side; <= 0 selects the default
                                 (1e-10 for MIXED and FP64_REFINED: one round to the target
                                 unless the inner arithmetic's floor stops it; 1e-2 for
                                 MIXED_FP32) */
    int32_t max_refine;       /* MIXED: outer refinement rounds; a round that fails to halve an
                                 instance's FP64 residual hands the solve to up to max_refine
                                 rounds of FP64 inner solves on the same regularised operator
                                 (a round of those that fails to halve one changes the inner
                                 solves' shadow vector) */
    int32_t stag_window;      /* MIXED: an inner solve also stops after this many every-50-applies
                                 tests without halving its residual; <= 0 selects 40 */
    int32_t inner_precond;    /* MIXED, MIXED_FP32: left diagonal preconditioning of the FP32x2 /
                                 FP32 inner solves (the rows of ADO n scaled by
                                 1 / (|sum of its damping rates| + ||H||_inf)); 0 (default) or
                                 1 = on, -1 = off.  FP64 inner solves are not scaled. */
    int32_t interleave;       /* MIXED: instances interleaved per entry group in the FP32x2 inner
                                 kernels (lanes of one entry share the plan's control flow and
                                 reads); 1 = none, 2..32 a power of two, 0 (default) = automatic
                                 choice of interleave and lane_instances: the context times its
                                 first mixed batch solves of each batch size (and kind: whole or
                                 truncated hierarchies) with each candidate layout -- none;
                                 interleave 2 with two instances per lane; when g = the
                                 smallest power of two >= nbatch (at most 32) exceeds 2, g with
                                 one and with two instances per lane (truncated batches: none
                                 and g with one) --
                                 and keeps the fastest for that size and kind
                                 (heom_tuned_layout); single solves use none.  An interleaved group runs until all its instances have
                                 finished. */
    int32_t lane_instances;   /* MIXED with interleave >= 2: instances of a group served by one
                                 thread of the inner kernels, 1 (0 selects 1) or 2: two adjacent
                                 instances share the decode of the plan (entry, couplings, map
                                 words, coefficients) while more than half of a group's
                                 instances run; with interleave 2 their iterates are those of
                                 interleave 1.  2 is refused for truncated batches. */
} heom_solve_opts;

typedef struct {
    int32_t iters;            /* operator applies of the Krylov iterations */
    int32_t ierr;             /* reference dutfx ierr of the last (inner) solve */
    int32_t refinements;      /* MIXED: outer rounds used */
    int32_t converged;
    double resid;             /* final ||b - A x|| in FP64 (worst instance of a batch) */
    double seconds;           /* device time of the solve */
    int64_t launches;         /* kernels launched by the solve (graph nodes included) */
} heom_solve_info;

/* rho: lunk_spa complex (host), initial guess in, steady state out. */
int heom_solve_tfqmr(heom_ctx *ctx, const heom_solve_opts *o, double _Complex *rho, heom_solve_info *info);

/* Steady state by Jacobi sweeps (solve_jacobi, jacobi/solve_jacobi.f90:1, methodss = 4):
 * x_n <- P_n (ejac - g_n + i [H, .])^-1 (ejac x_n + couplings of n), from the Hermitised rho,
 * with the true residual ||A x - e_trace|| tested after sweep 0 and every 50 sweeps until it
 * is <= o->crit or o->maxit0 sweeps are done (info->converged tells which).  ejac in
 * energy / hbar; <= 0 selects the rule of prelude_jacobi (heom_jacobi_shift).  nrho <= 32. */
int heom_solve_jacobi(heom_ctx *ctx, const heom_solve_opts *o, double ejac, double _Complex *rho,
                      heom_solve_info *info);
/* The shift of jacobi/prelude_jacobi.f90:84-111: max(span of the nonzero eigenvalues of
 * [H, .], sqrt((ntier - 1) max |cb|)). */
int heom_jacobi_shift(heom_ctx *ctx, double *ejac);

/* Observables of a host rho (td/calcj.f90, main/calcocc.f90).
 * jt: nalf*nspin (ialf fastest) in reference current units; occ: norbs*nspin. */
int heom_current(heom_ctx *ctx, const double _Complex *rho, double *jt);
int heom_occupation(heom_ctx *ctx, const double _Complex *rho, double *occ);

/* Time propagation (td/intstp.f90 RK4; td/chebyshev.f90 Chebyshev, on the sparse
 * layout).  rho (host, lunk) advanced from t0 by nstep steps of dt.  If jt_out is
 * non-NULL it receives the current jt (nalf*nspin) at the start of every step
 * (nstep rows), like curr.data.  HEOM_PROP_CHEBYSHEV_MIXED: the Chebyshev steps with the
 * state, the recurrence and the applies in FP32x2 (about 48 bits; the coefficients, the
 * lead shifts and the currents in FP64); no counterpart in the reference. */
enum { HEOM_PROP_RK4 = 0, HEOM_PROP_CHEBYSHEV = 1, HEOM_PROP_CHEBYSHEV_MIXED = 2 };
int heom_propagate(heom_ctx *ctx, int32_t method, double t0, double dt, int32_t nstep,
                   double _Complex *rho, double *jt_out);

/* Steady-state sensitivities by the adjoint method: for the lead-1 current
 * I = sum_s jt(1,s), dI/dtheta for theta in {V (bias, engyshift = +-V/2),
 * Gamma (all linewidths scaled together), U, eps} given as 4 partial derivatives
 * of (eleadinfty, cb/cd, hs).  rho: converged steady state (host).  dI: 4 doubles.
 * which: bitmask of the parameters wanted (bit k <-> theta k). */
typedef struct {
    const double *deshift;            /* (nalf,nspin) d eleadinfty / dV */
    double gamma;                     /* current linewidth scale for dA/dGamma = A_lower / Gamma */
    const double _Complex *dhs_du;    /* d hs / dU (nrho^2) */
    const double _Complex *dhs_deps;  /* d hs / d eps (nrho^2) */
    double crit;                      /* adjoint solve tolerance */
    int32_t maxit0;
    int32_t precision;                /* adjoint solve: HEOM_PREC_FP64 (0, restarted FP64 TFQMR) or
                                         HEOM_PREC_MIXED (FP32x2 TFQMR rounds on the regularised
                                         adjoint, FP64 residual refinement to the same tolerance) */
} heom_grad_opts;
int heom_steady_gradient(heom_ctx *ctx, const heom_grad_opts *o, const double _Complex *rho,
                         int32_t which, double *dI, heom_solve_info *info);

/* Time-dependent sensitivity: d/dA of int_0^{nstep dt} I_L(t) dt for a Chebyshev
 * propagation under the step bias amplitude scale A (eshift = A * amps), by a
 * reverse pass with checkpoints every k steps. rho0: initial state (host, lunk). */
int heom_td_gradient(heom_ctx *ctx, double dt, int32_t nstep, int32_t checkpoint_every,
                     const double _Complex *rho0, double *integral, double *dintegral);
/* The same through the steps of `method`: HEOM_PROP_CHEBYSHEV (as heom_td_gradient) or
 * HEOM_PROP_CHEBYSHEV_MIXED (forward and reverse passes with FP32x2 vectors and applies). */
int heom_td_gradient_ex(heom_ctx *ctx, int32_t method, double dt, int32_t nstep, int32_t checkpoint_every,
                        const double _Complex *rho0, double *integral, double *dintegral);

/* Batched steady states: many instances that share one table set and differ in
 * hs and eleadinfty are solved together (one vector per instance, one launch per
 * step for all of them).  hs_batch: nbatch * nrho^2, eshift_batch: nbatch*nalf*nspin.
 * rho_batch: nbatch * lunk (host, in/out). */
int heom_solve_batch(heom_ctx *ctx, int32_t nbatch, const double _Complex *hs_batch,
                     const double *eshift_batch, const heom_solve_opts *o,
                     double _Complex *rho_batch, heom_solve_info *info);

/* The same batch with its parameters kept on the device between solves.
 * heom_batch_solve_dev: x_dev holds nbatch FP64 complex vectors of stride
 * heom_batch_stride() elements (entry lunk of each is the unused trace slot), with the
 * initial guesses on entry and the steady states on return. */
typedef struct heom_batch heom_batch;
int heom_batch_create(heom_ctx *ctx, int32_t nbatch, const double _Complex *hs_batch, const double *eshift_batch,
                      heom_batch **out);
int64_t heom_batch_stride(const heom_batch *b);
int heom_batch_solve_dev(heom_batch *b, const heom_solve_opts *o, void *x_dev, heom_solve_info *info);
void heom_batch_destroy(heom_batch *b);
/* Truncated batches: instance b is solved on the hierarchy truncated at ntier[b] tiers
 * (1 <= ntier[b] <= the context's ntier; the reference counts the RDO as tier 1, as
 * in ntier of the input file).  The reference's tables are tier-major (main/ball2drawer.f90,
 * main/buildcoefindex.f90), so the tables of a shallower hierarchy of the same model family
 * are a prefix of the context's; one batch then holds instances of several depths and is
 * solved in one launch sequence.  In place of one heom_ctx per depth (the reference runs
 * one depth per job).  The states keep the context's layout: the entries beyond an
 * instance's tier are set to zero by heom_batch_solve_dev and stay zero; the trace slot
 * stays at the context's lunk.  ntier == NULL returns every instance to the whole
 * hierarchy. */
int heom_batch_set_tiers(heom_batch *b, const int32_t *ntier);

/* Lead currents jt[b][ialf + nalf*ispin] (b < nbatch) of nbatch device-resident states
 * x_dev (FP64 complex, instance stride vstride >= lunk + 1 elements, e.g. the vectors of
 * heom_batch_solve_dev), without any device allocation: the sums go through a file-scope
 * device array of 4096 x 4 doubles (128 KiB), so nbatch > 4096 is rejected.  It has no
 * counterpart in the reference (calcj, td/calcj.f90:40-85, works on one host state).  It
 * serves callers that must not allocate between solver rounds or time steps (cudaFree
 * synchronises the whole device).  The first call on a device does a one-time address
 * lookup and should come before any stream capture; calls that overlap in time share the
 * scratch and race.  The kernel runs on the context's own (non-blocking) stream, which is
 * not ordered after the caller's streams: x_dev must be complete when the call is made
 * (e.g. the caller synchronises the stream that wrote it). */
int heom_batch_current_static(heom_ctx *ctx, const void *x_dev, int32_t nbatch, int64_t vstride, double *jt);

/* Measurement hook: time `reps` back-to-back applies on `nbatch` instances on device, in
 * the form each solver precision uses (HEOM_PREC_FP64: the FP64 apply; HEOM_PREC_MIXED and
 * HEOM_PREC_MIXED_FP32: the regularised FP32x2 / FP32 apply of the inner solves), and
 * return the average kernel time in seconds and the algorithmic bytes of one launch. */
int heom_bench_apply(heom_ctx *ctx, int32_t precision, int32_t nbatch, int32_t reps, double *seconds, double *bytes);

/* Measurement hook: time `reps` launches of each of the two fused kernels of one inner
 * TFQMR iteration (the apply of w with the first half of the vector updates, and the apply
 * of v with the second half) on `nbatch` instances, in the number type of `precision`
 * (HEOM_PREC_MIXED: FP32x2, HEOM_PREC_MIXED_FP32: FP32, HEOM_PREC_FP64_REFINED: FP64).
 * seconds[0..1] and bytes[0..1] receive the average kernel time and the algorithmic bytes
 * of one launch of each kernel.  No reference counterpart (the reference has no mixed
 * precision). */
int heom_bench_inner(heom_ctx *ctx, int32_t precision, int32_t nbatch, int32_t reps, double *seconds, double *bytes);

/* heom_bench_inner in FP32x2 with a given layout of the instances (heom_solve_opts.interleave
 * >= 1 and lane_instances 1 or 2) instead of the one the batch solves use. */
int heom_bench_inner_layout(heom_ctx *ctx, int32_t nbatch, int32_t reps, int32_t interleave, int32_t lane_instances,
                            double *seconds, double *bytes);

/* The layout the automatic choice keeps for mixed batch solves of nbatch instances (truncated
 * != 0: batches with heom_batch_set_tiers): *interleave, *lane_instances as in heom_solve_opts,
 * or 0, 0 while the context has not yet timed every candidate. */
int heom_tuned_layout(heom_ctx *ctx, int32_t nbatch, int32_t truncated, int32_t *interleave, int32_t *lane_instances);

/* ------------------------------------------------------------------------- */
/* Correlation functions and spectral functions in the frequency domain (corrfunc/).
 * For B = a_{iorbs,ispin} the unknown holds two components h and a (the reference's
 * rcga, rcgb), each on the correlation-function pattern below; vectors of the device
 * solves are laid out [h (lunkcf); a (lunkcf)], the order of the reference's qmrvecs_cf. */
typedef struct {
    int32_t iorbs, ispin;                 /* B = a_{iorbs,ispin} (iorbs_dos, ispin_dos) */
    int64_t lunkcf_spa;
    const int32_t *nnzcf_spa;             /* nunk */
    const int64_t *indcf_spa;             /* nunk, 1-based */
    const int32_t *irowcf_spa, *icolcf_spa;   /* lunkcf_spa, 1-based */
} heom_cf_tables;

/* The pattern of prelude_cf_spa (corrfunc/prelude_cf_spa.f90:146-760): the tier rule of
 * prelude_spa seeded with the RDO structure of exp(0.314 H) (a + a^dag) exp(0.314 H).
 * The arrays belong to the model (valid while it lives; a later call for another
 * spin-orbital replaces them). */
int heom_model_cf_pattern(heom_model *m, int32_t iorbs, int32_t ispin, heom_cf_tables *out);

typedef struct heom_cf heom_cf;
/* Device plan of the correlation-function operator on the pattern `cf` (the caller's
 * nnzcf_spa etc., e.g. from the Fortran prelude_cf_spa, or heom_model_cf_pattern).
 * t: the same tables the context was created from.  The arrays are read here only. */
int  heom_cf_create(heom_ctx *ctx, const heom_tables *t, const heom_cf_tables *cf, heom_cf **out);
/* A heom_cf uses its context's stream and parameters: destroy it before the context. */
void heom_cf_destroy(heom_cf *cf);
int64_t heom_cf_lunk(const heom_cf *cf);

/* (rhsa, rhsb) = L_cf (rcga, rcgb)  (calc_ax_cf_spa_omp, corrfunc/calc_ax_cf_spa_omp.f90:1)
 * at frequency dfreq (internal units, energy / hbar) with the sign of the reference's
 * lplus_cf: isgnw = 1 (+i omega), 2 (-i omega).  All vectors ldim = lunkcf complex (host). */
int heom_cf_calc_ax(heom_cf *cf, double dfreq, int32_t isgnw, int64_t ldim, const double _Complex *rcga,
                    const double _Complex *rcgb, double _Complex *rhsa, double _Complex *rhsb);

/* solve_cf_tfqmr_spa (corrfunc/solve_cf_tfqmr_spa.f90:1) for nfreq frequencies at once:
 * L_cf(dfreq_k, isgnw) x_k = -(B rho) with brhoh = op(a) rho + rho op'(a),
 * brhoa = -i op(a) rho + i rho op'(a) (isgnb = 1: op = a^dag, op' = a; isgnb = 2: the
 * reverse).  rho: steady state (lunk_spa complex, host).  Each solve starts from x = 0,
 * runs TFQMR with tolerance 1e-3 crit and stops at ||b - L x|| <= crit (o->crit,
 * o->maxit0).  o->precision HEOM_PREC_FP64 is the reference algorithm; HEOM_PREC_MIXED
 * refines FP64 residuals with fused FP32x2 inner solves to the same criterion.  zouth, zouta: nfreq dense nrho x nrho RDO blocks (column-major)
 * of the two components, as the reference returns them; either may be NULL. */
int heom_cf_solve(heom_cf *cf, const double _Complex *rho, int32_t isgnb, int32_t isgnw, int32_t nfreq,
                  const double *dfreq, const heom_solve_opts *o, double _Complex *zouth, double _Complex *zouta,
                  heom_solve_info *info);

/* The time-domain branch of corrfunc (corrfunc/corrfunc.f90:364-630, lfreq_dos = F): X(0) = B rho
 * (a rho + rho a^dag on the cf pattern) propagated by RK4 steps of dt under the cf operator
 * without frequency terms; with ljw also Y(0) = B^dag rho.  corr[2k], corr[2k+1] receive
 * Tr[a^dag (X_h + i X_a)/2] and conj(Tr[a (Y_h + i Y_a)/2]) (0 without ljw) at t = k dt
 * (at t = 0: <a^dag a> and <a a^dag>),
 * k = 0..nstep.  rdo_h, rdo_a (optional): the dense RDO blocks of X_h, X_a at every step
 * ((nstep + 1) nrho^2 complex each). */
int heom_cf_propagate(heom_cf *cf, const double _Complex *rho, double dt, int32_t nstep, int32_t ljw,
                      double _Complex *corr, double _Complex *rdo_h, double _Complex *rdo_a);

/* The frequency-domain spectral function of corrfunc (corrfunc/corrfunc.f90:146-217,
 * lfreq_dos with ljw_dos): for every frequency freq_ev[k] (eV) the two solves
 * (isgnb, isgnw) = (2, 2) and (1, 1), batched together, and
 *   out[5k+0] = A(w) = out[5k+1] + out[5k+2]                     (1/eV)
 *   out[5k+1] = Re Tr[a^dag X_22] / pi / hbar  (occupied part, C_{B^dag B})
 *   out[5k+2] = Re Tr[a X_11] / pi / hbar      (empty part, C_{B B^dag})
 *   out[5k+3], out[5k+4] = Re, Im G^r(w) = -i (conj Tr[a^dag X_22] + Tr[a X_11]) / hbar
 * with X = (zouth + i zouta) / 2. */
int heom_cf_dos(heom_cf *cf, const double _Complex *rho, int32_t nfreq, const double *freq_ev,
                const heom_solve_opts *o, double *out, heom_solve_info *info);

/* Measurement hook: average time of `reps` back-to-back FP64 correlation-function applies on
 * `nbatch` instances (frequencies) and the algorithmic bytes of one launch (each instance's
 * vector read once and written once, plus the plan).  No reference counterpart. */
int heom_cf_bench_apply(heom_cf *cf, int32_t nbatch, int32_t reps, double *seconds, double *bytes);
/* Measurement hook of the mixed-precision cf solve: out[0], out[1] = seconds per launch of
 * the two fused FP32x2 inner-iteration kernels over `nbatch` instances; out[2], out[3] =
 * their algorithmic bytes per launch. */
int heom_cf_bench_inner(heom_cf *cf, int32_t nbatch, int32_t reps, double *out /* 4 */);

/* Measurement hook of the Jacobi sweep: out[0], out[1] = seconds per launch of the sector
 * transform kernel and of the apply (reps launches each), out[2] = the transform's
 * algorithmic bytes, out[3] = its complex multiply-adds per launch.  ejac <= 0: the rule. */
int heom_bench_jacobi(heom_ctx *ctx, double ejac, int32_t reps, double *out /* 4 */);

/* Plan statistics of the forward apply (per instance): [0] stored entries + 1, [1] ADOs
 * with entries, [2] pattern classes, [3] coupling records, [4] gather maps, [5] useful
 * gathers (nonzero map halves), [6] same-tier terms, [7] lower-tier (complex-coefficient)
 * gathers, [8] plan bytes read per apply (records, maps, per-entry and per-ADO arrays). */
int heom_ctx_stats(const heom_ctx *ctx, double *out /* 9 */);

#ifdef __cplusplus
}
#endif
#endif
