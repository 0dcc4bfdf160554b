/*
 * heom_oracle.h -- CPU FP64 restatement of HEOM-QUICK2's sparse-mode HEOM path.
 *
 * TEST INFRASTRUCTURE ONLY.  The GB300 library's results are tested against it:
 * only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may load it.
 * The product path never calls it.
 *
 * Parity status: UNPINNED against the reference.  HEOM-QUICK2 ships no tests,
 * fixtures or example outputs, and its Fortran/MKL build cannot be compiled in
 * this environment, so this restatement cannot be checked against outputs of the
 * reference itself.  It is instead pinned by self-derived known answers
 * (U=0 Landauer current, particle-hole symmetry, V=0 zero current, closed-form
 * table counts, trace preservation) in tests/.
 *
 * Conventions: every table keeps the reference's VALUES (1-based ADO, drawer,
 * operator and matrix indices) stored in 0-based C arrays, so
 * indexcoef[k-1] == reference indexcoef(k).  Matrices are column-major.
 */
#ifndef HEOM_ORACLE_H
#define HEOM_ORACLE_H

#include <stdint.h>
#include <complex.h>

typedef double _Complex ozc;

#define ORC_MAXALF 2
#define ORC_MAXORB 3
#define ORC_MAXMATS 64
#define ORC_MAXTIER 8

/* Physical constants, include/sizes:23,26,27 of the reference. */
#define ORC_HBAR 0.658211928
#define ORC_PI 3.141592653589793238
#define ORC_JCONST 1.602177e5
#define ORC_DSMALL 1e-32
#define ORC_DPICO 1e-12

enum { ORC_MODEL_PARA1 = 1, ORC_MODEL_PARA4 = 4, ORC_MODEL_KANAMORI = 5, ORC_MODEL_READHS = 9 };

/* Input of one job: the positional lines of the reference input file
 * (main/evaluatepara.f90:71-84) plus the namelist values the configs use. */
typedef struct {
    int norbs, nspin, nalf, nmats;
    int ntier;                                   /* reference ntier = truncation tier L + 1 */
    double bandwidth[ORC_MAXALF];                /* W */
    double linewidth[ORC_MAXALF][ORC_MAXORB];    /* linewidth(ialf, iorbs) */
    double temperature[ORC_MAXALF];              /* dinvbeta */
    double engyshift[ORC_MAXALF][2];             /* engyshift(ialf, ispin), energy units */
    int lscreen, doubledot;
    int model;
    double eup, edown, uu;                                   /* $para1 */
    double e1up, e1down, e2up, e2down, uu1, uu2, u12, t12;   /* $para4 */
    double kan_u, kan_j, kan_eps;                            /* Kanamori (lreadhs data) */
    const ozc *hs_in;                            /* model READHS: nrho*nrho, internal units */
    double tchar[ORC_MAXALF][2];                 /* fieldtype=0 switch-on time */
    unsigned long long pattern_seed;             /* seed of the random mixing in the pattern build */
    /* Prony scheme (psfjob, main/zpout_psf.f90): npsf > 0 replaces the Drude pole and the Pade
     * terms by npsf fitted exponentials, zcoef = psf_coef, zpole = psf_pole (the same for both
     * signs), fitted at temperature tpsf for a band of half-width rpsf * T centred at 0 */
    int npsf;
    double tpsf, rpsf;
    const ozc *psf_coef, *psf_pole;
} orc_params;

typedef struct {
    /* sizes (main/evaluatepara.f90:1204-1232) */
    int norbs, nspin, nalf, nmats, ntier, nsgn, ndrude, ncor, nopr, nvar, nrho, nams;
    int lscreen;
    /* Pade decomposition (main/zpout_psd.f90) */
    double cpcoef[ORC_MAXMATS];
    ozc cppole[ORC_MAXMATS][2];
    /* Prony scheme (main/zpout_psf.f90): fitted coefficients and poles, npsf of them */
    int npsf;
    double tpsf;
    ozc psfcoef[ORC_MAXMATS], psfpole[ORC_MAXMATS];
    /* bath coefficients, laid out as cb(norbs,nspin,ncor,nalf,nsgn) */
    ozc *cb, *cd, *cgama;
    ozc *cgamma; double *dipm;                       /* per drawer */
    int *mpm, *morbs, *mspin, *ilead, *mcor, *mopr;  /* per drawer, 1-based values */
    int *iredex, *indexdraw;                         /* per drawer */
    int *jpm, *jspin, *jorbs, *jalf, *jredex, *jomit;/* per operator */
    double zxip[ORC_MAXALF][ORC_MAXORB];             /* zxip(iorbs, *, ialf) (spin independent) */
    double hybrid[ORC_MAXALF][ORC_MAXORB];           /* prelude_spa hybrid(i,i,ialf) */
    double eleadinfty[ORC_MAXALF][2];
    double temperature[ORC_MAXALF];
    double amps[ORC_MAXALF][2], tchar[ORC_MAXALF][2];
    /* operators */
    double *amsori;                                  /* (nrho,nrho,norbs,nspin) */
    int *rowams, *colams, *sgnams;                   /* (nams,norbs,nspin) */
    /* partial-permutation maps of each a_{ms}: row of column c / column of row r
     * (0 = none) with the sign of that element; (nrho+1) entries per operator */
    int *op_rofc, *op_cofr, *op_srofc, *op_scofr;
    ozc *hs;                                         /* (nrho,nrho), internal units */
    /* hierarchy tables */
    int64_t ifirst[ORC_MAXTIER], ilast[ORC_MAXTIER], nfirst[ORC_MAXTIER], nlast[ORC_MAXTIER];
    int64_t nunk, ntable;
    int *indextable;
    int64_t *index_coef_ref;
    int64_t lall;
    int64_t *indexcoef;
    int8_t *itypecoef, *ifactfcoef, *ifactrcoef;
    /* sparsity (module/sparsemod.f90:34-42) */
    int64_t lunk;
    int *nnz_spa;
    int64_t *ind_spa;
    int *irow_spa, *icol_spa;
    int64_t pattern_values_mismatch;  /* entries where order 10 and 11 exp patterns differed */
} orc_model;

/* model construction / destruction */
int  orc_build(const orc_params *p, orc_model **out);
void orc_free(orc_model *m);
const char *orc_last_error(void);

/* applies.  x, y have lunk+1 complex entries (the last is the trace slot). */
void orc_calc_ax(const orc_model *m, const ozc *x, ozc *y, int nthreads);
/* dRho/dt at time t with eshift(t); x, y have lunk entries */
void orc_calcderiv(const orc_model *m, double t, const ozc *x, ozc *y, int nthreads);
/* generic apply with explicit lead shifts: steady (with_trace=1) or derivative */
void orc_apply_shift(const orc_model *m, const double eshift[ORC_MAXALF][2],
                     const ozc *x, ozc *y, int with_trace, int nthreads);
void orc_eshift(const orc_model *m, double t, double eshift[ORC_MAXALF][2]);

/* observables: jt(ialf,ispin) in reference current units (td/calcj.f90) */
void orc_current(const orc_model *m, const ozc *rho, double *jt /* [nalf*nspin], ialf fastest */);
void orc_occupation(const orc_model *m, const ozc *rho, double *occ /* [norbs*nspin] */);

/* initial guess: Boltzmann RDO at lead-1 temperature, all ADOs zero */
void orc_initial_guess(const orc_model *m, ozc *rho);

/* TFQMR steady-state solve (tfqmr_double/solve_tfqmr.f90 + dutfx.f90). rho in/out (lunk entries). */
typedef struct { int iters, axb, ierr, exit_reason; double resid; } orc_solve_info;
int orc_solve_tfqmr(const orc_model *m, double crit, int maxit0, ozc *rho, orc_solve_info *info, int nthreads);

/* RK4 step (td/intstp.f90) from t to t+dt */
void orc_rk4_step(const orc_model *m, double t, double dt, ozc *rho, int nthreads);
/* Chebyshev propagation of a step bias (restated from td/chebyshev.f90 on the sparse operator) */
double orc_cheby_delta(const orc_model *m);
int  orc_cheby_nterms(double delta, double dt, double dpre);
void orc_cheby_step(const orc_model *m, double t, double delta, int nterms, double dt, ozc *rho, int nthreads);
/* flat accessors for the ctypes binding: sizes by key, arrays copied by name */
int64_t orc_info(const orc_model *m, const char *key);
int orc_copy(const orc_model *m, const char *name, void *dst);
double orc_besselj_ext(int n, double x);

/* drandn stream (tfqmr_double/drandn.f90) */
void orc_drandn(int64_t n, double *dx, int seed);
double orc_dnrm2(int64_t n, const double *x);

/* Correlation-function system of B rho, B = a_{iorbs,ispin} (corrfunc/prelude_cf_spa.f90,
 * calc_ax_cf_spa_omp.f90, solve_cf_tfqmr_spa.f90).  The unknown has two components h and a
 * (rcga, rcgb), each lunkcf entries on the pattern nnzcf/indcf/irowcf/icolcf. */
typedef struct {
    int iorbs, ispin;
    int64_t lunkcf;
    int *nnzcf; int64_t *indcf;
    int *irowcf, *icolcf;
} orc_cf;
int  orc_cf_build(const orc_model *m, int iorbs, int ispin, unsigned long long seed, orc_cf **out);
void orc_cf_free(orc_cf *cf);
/* (yh, ya) = L_cf(omega, isgnw) (xh, xa) */
void orc_cf_apply(const orc_model *m, const orc_cf *cf, double omega, int isgnw, const ozc *xh, const ozc *xa,
                  ozc *yh, ozc *ya, int nthreads);
/* the reference's TFQMR solve of L_cf x = -(B rho) from x = 0 (solve_cf_tfqmr_spa.f90) */
int orc_cf_solve(const orc_model *m, const orc_cf *cf, const ozc *rho, int isgnb, int isgnw, double omega, double crit,
                 int maxit0, ozc *xh, ozc *xa, orc_solve_info *info, int nthreads);
/* brhoh, brhoa from the steady rho (lunk entries); isgnb 1: a^dag rho + rho a, 2: a rho + rho a^dag */
void orc_cf_rhs(const orc_model *m, const orc_cf *cf, const ozc *rho, int isgnb, ozc *bh, ozc *ba);
int64_t orc_cf_info(const orc_cf *cf, const char *key);

/* Jacobi steady-state iteration (jacobi/prelude_jacobi.f90, calc_ax_jacobi_spa_omp.f90,
 * solve_jacobi.f90) */
typedef struct orc_jacobi orc_jacobi;
void orc_herm_eig(int n, ozc *a, double *w, ozc *v);
int  orc_jacobi_build(const orc_model *m, double ejac_in, orc_jacobi **out);
void orc_jacobi_free(orc_jacobi *J);
double orc_jacobi_ejac(const orc_jacobi *J);
void orc_jacobi_sweep(const orc_model *m, const orc_jacobi *J, const ozc *x, ozc *xn);
int  orc_solve_jacobi(const orc_model *m, const orc_jacobi *J, double crit, int maxit0, ozc *rho, orc_solve_info *info);
int orc_cf_copy(const orc_cf *cf, int64_t nunk, const char *name, void *dst);

#endif
