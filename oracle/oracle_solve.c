/*
 * oracle_solve.c -- TFQMR steady-state solve, RK4 and Chebyshev propagation of
 * HEOM-QUICK2, restated in plain C.  TEST INFRASTRUCTURE ONLY (see heom_oracle.h).
 *
 * TFQMR follows the published algorithm of R. W. Freund (SIAM J. Sci. Comput. 14
 * (1993) 470-482) with the vector roles, tolerances and stopping tests of the
 * reverse-communication driver in tfqmr_double/dutfx.f90 and solve_tfqmr.f90.
 */
#include "oracle_internal.h"

/* tfqmr_double/drandn.f90: multiplicative congruential generator on 32-bit integers
 * (products wrap modulo 2^32 like Fortran default integers). */
void orc_drandn(int64_t n, double *dx, int seed)
{
    int32_t im = 1, j = 0;
    for (int i = 1; i <= 31; i++) {
        j++;
        int32_t twice = (int32_t)((uint32_t)im * 2u);
        if (twice <= im) break;
        im = twice;
    }
    int32_t imax = (int32_t)(((uint32_t)(im - 1) * 2u) + 1u);
    double dmax = (double)imax;
    for (int i = 1; i <= j % 3; i++) im /= 2;
    im += 5;
    int32_t is = (int32_t)((uint32_t)im * 30107u) % imax; if (is < 0) is = -is;
    if (seed > 0) is = (seed / 2) * 2 + 1;
    for (int64_t i = 0; i < n; i++) {
        dx[i] = (double)is / dmax;
        int32_t prod = (int32_t)((uint32_t)im * (uint32_t)is);
        int32_t r = prod % imax;
        is = r < 0 ? -r : r;
    }
}

/* tfqmr_double/ddot_long.f90 (unit stride, 5-way unrolled accumulation order) */
static double orc_ddot(int64_t n, const double *x, const double *y)
{
    double t = 0.0;
    if (n <= 0) return 0.0;
    int64_t mrem = n % 5;
    for (int64_t i = 0; i < mrem; i++) t += x[i] * y[i];
    for (int64_t i = mrem; i < n; i += 5)
        t = t + x[i] * y[i] + x[i + 1] * y[i + 1] + x[i + 2] * y[i + 2] + x[i + 3] * y[i + 3] + x[i + 4] * y[i + 4];
    return t;
}

/* 2-norm (tfqmr_double/dnrm2_long.f90 reduces to this sum of squares for mid-range data) */
double orc_dnrm2(int64_t n, const double *x)
{
    double s = 0.0;
    for (int64_t i = 0; i < n; i++) s += x[i] * x[i];
    return sqrt(s);
}

static void axpby(int64_t n, double *z, double a, const double *x, double b, const double *y)
{ for (int64_t i = 0; i < n; i++) z[i] = a * x[i] + b * y[i]; }

typedef struct tfq_ctx {
    const orc_model *m; int nthreads; int64_t lnum; double *V[10];
    int iter; double crit; int exited;
    void (*ax)(struct tfq_ctx *c, const double *x, double *y);   /* the operator */
    const orc_cf *cf; double omega; int isgnw;
} tfq_ctx;

static void ax_steady(tfq_ctx *c, const double *x, double *y) { orc_calc_ax(c->m, (const ozc *)x, (ozc *)y, c->nthreads); }

/* solve_tfqmr.f90:194-280: before every AXB requested by dutfx (and at its final
 * return), every iter_show=50 calls, test the true residual ||A x - b|| <= crit. */
static int tfq_check(tfq_ctx *c)
{
    if (c->iter % 50 == 0) {
        c->ax(c, c->V[1], c->V[9]);
        axpby(c->lnum, c->V[9], 1.0, c->V[9], -1.0, c->V[2]);
        double e = orc_dnrm2(c->lnum, c->V[9]);
        if (e <= c->crit) { c->exited = 1; return 1; }
    }
    return 0;
}
static int tfq_axb(tfq_ctx *c, int colx, int colb)
{
    if (tfq_check(c)) return 1;
    c->iter++;
    c->ax(c, c->V[colx], c->V[colb]);
    return 0;
}

/* tfqmr_double/dutfx.f90:152-357 run to completion with direct applies */
static int orc_dutfx(tfq_ctx *c, int nlim, double tol, int *ierr_out)
{
    int64_t N = c->lnum;
    double **V = c->V;
    int ierr;
    axpby(N, V[5], 1.0, V[2], 0.0, V[5]);
    axpby(N, V[1], 0.0, V[1], 0.0, V[1]);
    double r0 = orc_dnrm2(N, V[5]);
    if (tol >= 1.0 || r0 == 0.0) { *ierr_out = 0; return 0; }
    orc_drandn(N, V[3], 1);
    int n = 1;
    double resn = 1.0, rho = 1.0, var = 0.0, eta = 0.0, tau = r0 * r0, alpha = 0, beta, cosv, unrm, uchk, dtmp;
    ierr = 8;
    axpby(N, V[8], 0.0, V[8], 0.0, V[8]);
    axpby(N, V[4], 0.0, V[4], 0.0, V[4]);
    axpby(N, V[6], 0.0, V[6], 0.0, V[6]);
    for (;;) {
        dtmp = orc_ddot(N, V[3], V[5]);
        beta = dtmp / rho; rho = dtmp;
        axpby(N, V[4], beta, V[4], 1.0, V[8]);
        axpby(N, V[6], 1.0, V[5], beta, V[6]);
        if (tfq_axb(c, 6, 9)) goto stop;
        axpby(N, V[4], beta, V[4], 1.0, V[9]);
        dtmp = orc_ddot(N, V[3], V[4]);
        if (dtmp == 0.0 || rho == 0.0) { ierr = 8; goto done; }
        alpha = rho / dtmp;
        dtmp = var * eta / alpha;
        axpby(N, V[7], 1.0, V[6], dtmp, V[7]);
        axpby(N, V[5], 1.0, V[5], -alpha, V[9]);
        dtmp = orc_dnrm2(N, V[5]); dtmp *= dtmp;
        var = dtmp / tau; cosv = 1.0 / (1.0 + var); tau = dtmp * cosv; eta = alpha * cosv;
        axpby(N, V[1], 1.0, V[1], eta, V[7]);
        unrm = sqrt((double)(2 * n) * tau) / r0; uchk = unrm;
        if (!(unrm / tol > 10.0)) {
            if (tfq_axb(c, 1, 9)) goto stop;
            axpby(N, V[9], 1.0, V[2], -1.0, V[9]);
            resn = orc_dnrm2(N, V[9]) / r0; uchk = resn;
        }
        if (resn <= tol) { ierr = 0; goto done; }
        else if (unrm < uchk / 100.0) { ierr = 4; goto done; }
        axpby(N, V[6], 1.0, V[6], -alpha, V[4]);
        dtmp = var * cosv;
        axpby(N, V[7], 1.0, V[6], dtmp, V[7]);
        if (tfq_axb(c, 6, 8)) goto stop;
        axpby(N, V[5], 1.0, V[5], -alpha, V[8]);
        dtmp = orc_dnrm2(N, V[5]); dtmp *= dtmp;
        var = dtmp / tau; cosv = 1.0 / (1.0 + var); tau = dtmp * cosv; eta = alpha * cosv;
        axpby(N, V[1], 1.0, V[1], eta, V[7]);
        unrm = sqrt((double)(2 * n + 1) * tau) / r0; uchk = unrm;
        if (!((unrm / tol > 10.0) && (n < nlim))) {
            if (tfq_axb(c, 1, 9)) goto stop;
            axpby(N, V[9], 1.0, V[2], -1.0, V[9]);
            resn = orc_dnrm2(N, V[9]) / r0; uchk = unrm;
        }
        if (resn <= tol) { ierr = 0; goto done; }
        else if (unrm < uchk / 100.0) { ierr = 4; goto done; }
        else if (n >= nlim) { ierr = 4; goto done; }
        n++;
    }
done:
    *ierr_out = ierr;
    tfq_check(c);          /* the driver tests once more when dutfx returns */
    return 0;
stop:
    *ierr_out = ierr;
    return 1;
}

int orc_solve_tfqmr(const orc_model *m, double crit, int maxit0, ozc *rho, orc_solve_info *info, int nthreads)
{
    tfq_ctx c; memset(&c, 0, sizeof c);
    c.m = m; c.nthreads = nthreads; c.lnum = 2 * (m->lunk + 1); c.crit = crit; c.ax = ax_steady;
    for (int k = 1; k <= 9; k++) c.V[k] = calloc(c.lnum, sizeof(double));
    /* zmat_herm_coo('u') on the RDO: upper triangle defines the lower one, real diagonal */
    {
        int n = m->nrho, nz = m->nnz_spa[0];
        ozc *t = calloc((size_t)n * n, sizeof(ozc));
        for (int q = 0; q < nz; q++) {
            int r = m->irow_spa[q], cc = m->icol_spa[q];
            if (cc > r) { t[(r - 1) + (size_t)(cc - 1) * n] = rho[q]; t[(cc - 1) + (size_t)(r - 1) * n] = conj(rho[q]); }
            if (cc == r) t[(r - 1) + (size_t)(cc - 1) * n] = creal(rho[q]);
        }
        for (int q = 0; q < nz; q++) rho[q] = t[(m->irow_spa[q] - 1) + (size_t)(m->icol_spa[q] - 1) * n];
        free(t);
    }
    ozc *xpad = calloc(m->lunk + 1, sizeof(ozc));
    memcpy(xpad, rho, sizeof(ozc) * m->lunk);
    orc_calc_ax(m, xpad, (ozc *)c.V[2], nthreads);
    for (int64_t k = 0; k < c.lnum; k++) c.V[2][k] = -c.V[2][k];
    c.V[2][c.lnum - 2] += 1.0;
    double r = orc_dnrm2(c.lnum, c.V[2]);
    int ierr = 0;
    if (r > crit) orc_dutfx(&c, maxit0 / 2, crit * 1e-3, &ierr);
    for (int64_t k = 0; k < m->lunk; k++) rho[k] += ((ozc *)c.V[1])[k];
    memcpy(xpad, rho, sizeof(ozc) * m->lunk); xpad[m->lunk] = 0;
    orc_calc_ax(m, xpad, (ozc *)c.V[9], nthreads);
    c.V[9][c.lnum - 2] -= 1.0;
    if (info) { info->iters = c.iter; info->axb = c.iter; info->ierr = ierr; info->exit_reason = c.exited; info->resid = orc_dnrm2(c.lnum, c.V[9]); }
    for (int k = 1; k <= 9; k++) free(c.V[k]);
    free(xpad);
    return 0;
}

/* corrfunc/solve_cf_tfqmr_spa.f90: the vector is [h; a] (qmrvecs_cf), the right-hand side
 * -(brhoh; brhoa) (lines 185-197), x0 = 0, dutfx with tolerance 1e-3 crit and the driver's
 * every-50-applies test ||b - L x|| <= crit (lines 56-60, 262-290). */
static void ax_cf(tfq_ctx *c, const double *x, double *y)
{
    int64_t L = c->cf->lunkcf;
    orc_cf_apply(c->m, c->cf, c->omega, c->isgnw, (const ozc *)x, (const ozc *)x + L, (ozc *)y, (ozc *)y + L, c->nthreads);
}

int orc_cf_solve(const orc_model *m, const orc_cf *cf, const ozc *rho, int isgnb, int isgnw, double omega, double crit,
                 int maxit0, ozc *xh, ozc *xa, orc_solve_info *info, int nthreads)
{
    int64_t L = cf->lunkcf;
    tfq_ctx c; memset(&c, 0, sizeof c);
    c.m = m; c.nthreads = nthreads; c.lnum = 4 * L; c.crit = crit; c.ax = ax_cf;
    c.cf = cf; c.omega = omega; c.isgnw = isgnw;
    for (int k = 1; k <= 9; k++) c.V[k] = calloc(c.lnum, sizeof(double));
    ozc *b = (ozc *)c.V[2];
    orc_cf_rhs(m, cf, rho, isgnb, b, b + L);
    for (int64_t k = 0; k < c.lnum; k++) c.V[2][k] = -c.V[2][k];
    int ierr = 0;
    if (orc_dnrm2(c.lnum, c.V[2]) > crit) orc_dutfx(&c, maxit0 / 2, crit * 1e-3, &ierr);
    memcpy(xh, c.V[1], sizeof(ozc) * L);
    memcpy(xa, (ozc *)c.V[1] + L, sizeof(ozc) * L);
    ax_cf(&c, c.V[1], c.V[9]);
    axpby(c.lnum, c.V[9], 1.0, c.V[9], -1.0, c.V[2]);
    if (info) { info->iters = c.iter; info->axb = c.iter; info->ierr = ierr; info->exit_reason = c.exited; info->resid = orc_dnrm2(c.lnum, c.V[9]); }
    for (int k = 1; k <= 9; k++) free(c.V[k]);
    return 0;
}

/* td/intstp.f90:31-99 */
void orc_rk4_step(const orc_model *m, double t, double dt, ozc *rho, int nthreads)
{
    int64_t L = m->lunk;
    ozc *r0 = malloc(sizeof(ozc) * L), *rt = malloc(sizeof(ozc) * L), *k = malloc(sizeof(ozc) * L);
    memcpy(r0, rho, sizeof(ozc) * L); memcpy(rt, rho, sizeof(ozc) * L);
    double dt2 = dt / 2, dt3 = dt / 3, dt6 = dt / 6;
    orc_calcderiv(m, t, rt, k, nthreads);
    for (int64_t i = 0; i < L; i++) { rt[i] = r0[i] + dt2 * k[i]; rho[i] += dt6 * k[i]; }
    orc_calcderiv(m, t + dt2, rt, k, nthreads);
    for (int64_t i = 0; i < L; i++) { rt[i] = r0[i] + dt2 * k[i]; rho[i] += dt3 * k[i]; }
    orc_calcderiv(m, t + dt2, rt, k, nthreads);
    for (int64_t i = 0; i < L; i++) { rt[i] = r0[i] + dt * k[i]; rho[i] += dt3 * k[i]; }
    orc_calcderiv(m, t + dt, rt, k, nthreads);
    for (int64_t i = 0; i < L; i++) rho[i] += dt6 * k[i];
    free(r0); free(rt); free(k);
}

/* Bessel function of the first kind J_n(x), n >= 0, by Miller's downward recurrence
 * normalised with J_0 + 2 sum J_2k = 1 (Abramowitz & Stegun 9.1.46). */
static double orc_besselj(int nn, double x)
{
    if (x == 0.0) return nn == 0 ? 1.0 : 0.0;
    double ax = fabs(x);
    int start = 2 * ((nn > (int)ax ? nn : (int)ax) + 15 + (int)sqrt(40.0 * (nn + ax + 10.0)));
    double jp1 = 0.0, j = 1e-300, res = 0.0, norm = 0.0;
    for (int k = start; k >= 0; k--) {
        double jm1 = 2.0 * (k + 1) / ax * j - jp1;
        if (k == 0) norm += jm1; else if (k % 2 == 0) norm += 2.0 * jm1;
        if (k == nn) res = jm1;
        jp1 = j; j = jm1;
        if (fabs(j) > 1e250) { j *= 1e-250; jp1 *= 1e-250; res *= 1e-250; norm *= 1e-250; }
    }
    double v = res / norm;
    if (x < 0 && (nn % 2)) v = -v;
    return v;
}

/* td/prechebyshev.f90:56-110: spectral width = spread of the real parts of the
 * Liouville diagonal over all ADOs (the H part is purely imaginary on it). */
double orc_cheby_delta(const orc_model *m)
{
    double rmax = -1e20, rmin = 1e20;
    for (int itier = 1; itier <= m->ntier; itier++) {
        int nb = itier - 1;
        for (int64_t lni = m->nfirst[itier - 1]; lni <= m->nlast[itier - 1]; lni++) {
            double g = 0;
            for (int b = 0; b < nb; b++) g += creal(m->cgamma[m->indextable[m->ifirst[itier - 1] - 1 + (lni - m->nfirst[itier - 1]) * nb + b] - 1]);
            if (g > rmax) rmax = g;
            if (g < rmin) rmin = g;
        }
    }
    return rmax - rmin;
}

/* td/prechebyshev.f90:117-130 */
int orc_cheby_nterms(double delta, double dt, double dpre)
{
    double s = 0, r = 1; int n = 0;
    while (r >= dpre) { double b = orc_besselj(n, delta * dt); s += fabs(b); r = fabs(b) / s; n++; }
    return n;
}

/* td/chebyshev.f90:150-200: rho(t+dt) = J0 P0 + 2 sum_n J_n(delta dt) P_n with
 * P1 = L P0 / delta, P_n = P_{n-2} + (2/delta) L P_{n-1}; L is dRho/dt at time t. */
void orc_cheby_step(const orc_model *m, double t, double delta, int nterms, double dt, ozc *rho, int nthreads)
{
    int64_t L = m->lunk;
    ozc *pm2 = malloc(sizeof(ozc) * L), *pm1 = malloc(sizeof(ozc) * L), *lp = malloc(sizeof(ozc) * L);
    double x = delta * dt;
    memcpy(pm2, rho, sizeof(ozc) * L);
    double j0 = orc_besselj(0, x);
    for (int64_t i = 0; i < L; i++) rho[i] = j0 * pm2[i];
    orc_calcderiv(m, t, pm2, lp, nthreads);
    for (int64_t i = 0; i < L; i++) pm1[i] = lp[i] / delta;
    double c = 2.0 * orc_besselj(1, x);
    for (int64_t i = 0; i < L; i++) rho[i] += c * pm1[i];
    for (int k = 2; k < nterms; k++) {
        orc_calcderiv(m, t, pm1, lp, nthreads);
        for (int64_t i = 0; i < L; i++) { ozc pn = pm2[i] + (2.0 / delta) * lp[i]; pm2[i] = pm1[i]; pm1[i] = pn; }
        c = 2.0 * orc_besselj(k, x);
        for (int64_t i = 0; i < L; i++) rho[i] += c * pm1[i];
    }
    free(pm2); free(pm1); free(lp);
}

double orc_besselj_ext(int n, double x) { return orc_besselj(n, x); }
