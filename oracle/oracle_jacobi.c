/*
 * oracle_jacobi.c -- the Jacobi steady-state iteration of HEOM-QUICK2's sparse mode,
 * restated in plain C.  TEST INFRASTRUCTURE ONLY.
 *
 * jacobi/prelude_jacobi.f90:20-126        eigen-decomposition of the system Liouvillian
 *                                         L = H (x) 1 - 1 (x) H^T (nrho^2 x nrho^2, Hermitian)
 *                                         and the shift ejac
 * jacobi/calc_ax_jacobi_spa_omp.f90:72-353 one sweep: per ADO n, Y = ejac x_n + (couplings of
 *                                         n), x_n' = (ejac - g_n + i L)^-1 Y, restricted to
 *                                         the pattern of n
 * jacobi/solve_jacobi.f90:100-280         the driver: sweeps until the every-50-sweeps true
 *                                         residual ||A x - e_trace|| <= crit
 *
 * The couplings of n are A x - g x + i P[H, x] on the pattern of n (the steady operator of
 * oracle_apply.c less its same-tier part), which is what the reference accumulates.
 */
#include "oracle_internal.h"

#define ORC_DPICO 1e-12

/* Hermitian eigen-decomposition by cyclic complex Jacobi rotations: A (n x n, column-major)
 * is destroyed; w ascending is not guaranteed; V columns are the eigenvectors. */
void orc_herm_eig(int n, ozc *a, double *w, ozc *v)
{
    for (size_t k = 0; k < (size_t)n * n; k++) v[k] = 0;
    for (int i = 0; i < n; i++) v[i + (size_t)i * n] = 1;
    for (int sweep = 0; sweep < 100; sweep++) {
        double off = 0, tot = 0;
        for (int j = 0; j < n; j++) for (int i = 0; i < n; i++) {
            double t = creal(a[i + (size_t)j * n] * conj(a[i + (size_t)j * n]));
            tot += t;
            if (i != j) off += t;
        }
        if (off <= 1e-30 * (tot > 0 ? tot : 1)) break;
        for (int p = 0; p < n; p++) for (int q = p + 1; q < n; q++) {
            ozc apq = a[p + (size_t)q * n];
            double r = cabs(apq);
            if (r < 1e-300) continue;
            ozc ph = apq / r;                       /* e^{i phi} */
            /* D = diag(1, conj(ph)) on q makes a_pq real: column q *= conj(ph), row q *= ph */
            for (int k = 0; k < n; k++) a[k + (size_t)q * n] *= conj(ph);
            for (int k = 0; k < n; k++) a[q + (size_t)k * n] *= ph;
            for (int k = 0; k < n; k++) v[k + (size_t)q * n] *= conj(ph);
            double app = creal(a[p + (size_t)p * n]), aqq = creal(a[q + (size_t)q * n]);
            double th = (aqq - app) / (2 * r);
            double t = (th >= 0 ? 1.0 : -1.0) / (fabs(th) + sqrt(th * th + 1));
            double c = 1 / sqrt(t * t + 1), s = t * c;
            for (int k = 0; k < n; k++) {
                ozc x = a[k + (size_t)p * n], y = a[k + (size_t)q * n];
                a[k + (size_t)p * n] = c * x - s * y; a[k + (size_t)q * n] = s * x + c * y;
            }
            for (int k = 0; k < n; k++) {
                ozc x = a[p + (size_t)k * n], y = a[q + (size_t)k * n];
                a[p + (size_t)k * n] = c * x - s * y; a[q + (size_t)k * n] = s * x + c * y;
            }
            for (int k = 0; k < n; k++) {
                ozc x = v[k + (size_t)p * n], y = v[k + (size_t)q * n];
                v[k + (size_t)p * n] = c * x - s * y; v[k + (size_t)q * n] = s * x + c * y;
            }
        }
    }
    for (int i = 0; i < n; i++) w[i] = creal(a[i + (size_t)i * n]);
}

struct orc_jacobi {
    int n2, nnzjac;
    double ejac;
    double *val;   /* nonzero eigenvalues of L */
    ozc *vec;      /* their eigenvectors, n2 x nnzjac */
};

/* prelude_jacobi.f90:40-126: L from hs (igroundsteady: hs + dhs, dhs = 0 for a static
 * Hamiltonian), its nonzero eigenpairs, ejac = max(gap of L, sqrt((ntier-1) max|cb|)) unless
 * given (e_jacobi of the $jacobi group, in energy / hbar). */
int orc_jacobi_build(const orc_model *m, double ejac_in, orc_jacobi **out)
{
    int n = m->nrho, n2 = n * n;
    ozc *L = calloc((size_t)n2 * n2, sizeof(ozc)), *V = calloc((size_t)n2 * n2, sizeof(ozc));
    double *w = calloc(n2, sizeof(double));
    /* column-major vec: X(i,j) -> i + j n; (H X)(i,j) = H(i,k) X(k,j); (X H)(i,j) = X(i,k) H(k,j) */
    for (int j = 0; j < n; j++) for (int i = 0; i < n; i++)
        for (int k = 0; k < n; k++) {
            L[(i + j * n) + (size_t)(k + j * n) * n2] += m->hs[i + (size_t)k * n];
            L[(i + j * n) + (size_t)(i + k * n) * n2] -= m->hs[k + (size_t)j * n];
        }
    orc_herm_eig(n2, L, w, V);
    orc_jacobi *J = calloc(1, sizeof(orc_jacobi));
    J->n2 = n2;
    J->val = calloc(n2, sizeof(double));
    J->vec = calloc((size_t)n2 * n2, sizeof(ozc));
    double lo = 0, hi = 0;
    for (int k = 0; k < n2; k++) {
        if (fabs(w[k]) <= ORC_DPICO) continue;
        if (J->nnzjac == 0 || w[k] < lo) lo = w[k];
        if (J->nnzjac == 0 || w[k] > hi) hi = w[k];
        J->val[J->nnzjac] = w[k];
        memcpy(J->vec + (size_t)J->nnzjac * n2, V + (size_t)k * n2, sizeof(ozc) * n2);
        J->nnzjac++;
    }
    double gap = J->nnzjac > 0 ? hi - lo : 0.0, cbmax = 0;
    size_t ncb = (size_t)m->norbs * m->nspin * m->ncor * m->nalf * 2;
    for (size_t k = 0; k < ncb; k++) if (cabs(m->cb[k]) > cbmax) cbmax = cabs(m->cb[k]);
    double e2 = sqrt((double)(m->ntier - 1) * cbmax);
    J->ejac = ejac_in > 0 ? ejac_in : (gap > e2 ? gap : e2);
    free(L); free(V); free(w);
    *out = J;
    return 0;
}

void orc_jacobi_free(orc_jacobi *J)
{
    if (!J) return;
    free(J->val); free(J->vec); free(J);
}

double orc_jacobi_ejac(const orc_jacobi *J) { return J->ejac; }

/* (ejac - g + i L)^-1 restricted to nonzero eigenpairs plus the null-space part
 * (calc_ax_jacobi_spa_omp.f90:159-176, 324-346): Z = V diag(f) V^H Y + Y / (ejac - g) */
static void jac_transform(const orc_jacobi *J, ozc g, const ozc *y, ozc *z, ozc *tmp)
{
    int n2 = J->n2;
    ozc d = J->ejac - g;
    int small = cabs(d) <= ORC_DPICO;
    for (int k = 0; k < J->nnzjac; k++) {
        const ozc *vk = J->vec + (size_t)k * n2;
        ozc s = 0;
        for (int i = 0; i < n2; i++) s += conj(vk[i]) * y[i];
        ozc f = small ? 1.0 / (I * J->val[k]) : 1.0 / (I * J->val[k] + d) - 1.0 / d;
        tmp[k] = s * f;
    }
    for (int i = 0; i < n2; i++) {
        ozc s = 0;
        for (int k = 0; k < J->nnzjac; k++) s += J->vec[i + (size_t)k * n2] * tmp[k];
        z[i] = s + (small ? 0.0 : y[i] / d);
    }
}

/* one sweep x -> xn (lunk entries each); y = A x from the steady apply (lunk + 1 entries) */
void orc_jacobi_sweep(const orc_model *m, const orc_jacobi *J, const ozc *x, ozc *xn)
{
    int n = m->nrho, n2 = n * n;
    ozc *xp = calloc(m->lunk + 1, sizeof(ozc)), *y = calloc(m->lunk + 1, sizeof(ozc));
    memcpy(xp, x, sizeof(ozc) * m->lunk);
    orc_calc_ax(m, xp, y, 0);
#pragma omp parallel
    {
    ozc *X = calloc(n2, sizeof(ozc)), *Y = calloc(n2, sizeof(ozc)), *Z = calloc(n2, sizeof(ozc)), *T = calloc(n2, sizeof(ozc));
#pragma omp for schedule(dynamic, 16)
    for (int64_t u = 1; u <= m->nunk; u++) {
        int nz = m->nnz_spa[u - 1];
        if (nz == 0) continue;
        int64_t st = m->ind_spa[u - 1] - 1;
        int itier = 1;
        while (itier < m->ntier && u > m->nlast[itier - 1]) itier++;
        ozc g = 0;
        for (int b = 0; b < itier - 1; b++) {
            int d = m->indextable[m->ifirst[itier - 1] - 1 + (u - m->nfirst[itier - 1]) * (itier - 1) + b];
            g += m->cgamma[d - 1] + I * m->dipm[d - 1] * m->eleadinfty[m->ilead[d - 1] - 1][m->mspin[d - 1] - 1];
        }
        for (int k = 0; k < n2; k++) X[k] = Y[k] = 0;
        for (int q = 0; q < nz; q++) X[(m->irow_spa[st + q] - 1) + (size_t)(m->icol_spa[st + q] - 1) * n] = x[st + q];
        /* Y = ejac x + C x on the pattern, C x = A x - g x + i P[H, x] */
        for (int q = 0; q < nz; q++) {
            int r = m->irow_spa[st + q] - 1, c = m->icol_spa[st + q] - 1;
            ozc comm = 0;
            for (int k = 0; k < n; k++)
                comm += m->hs[r + (size_t)k * n] * X[k + (size_t)c * n] - X[r + (size_t)k * n] * m->hs[k + (size_t)c * n];
            Y[r + (size_t)c * n] = J->ejac * x[st + q] + y[st + q] - g * x[st + q] + I * comm;
        }
        jac_transform(J, g, Y, Z, T);
        for (int q = 0; q < nz; q++) xn[st + q] = Z[(m->irow_spa[st + q] - 1) + (size_t)(m->icol_spa[st + q] - 1) * n];
    }
    free(X); free(Y); free(Z); free(T);
    }
    free(xp); free(y);
}

/* solve_jacobi.f90:100-280: rho (lunk) in/out */
int orc_solve_jacobi(const orc_model *m, const orc_jacobi *J, double crit, int maxit0, ozc *rho, orc_solve_info *info)
{
    int64_t L = m->lunk;
    ozc *x = calloc(L + 1, sizeof(ozc)), *xn = calloc(L + 1, sizeof(ozc)), *r = calloc(L + 1, sizeof(ozc));
    memcpy(x, rho, sizeof(ozc) * L);
    int iter = 0, conv = 0;
    double res = 0;
    for (;;) {
        orc_jacobi_sweep(m, J, x, xn);
        memcpy(x, xn, sizeof(ozc) * L);
        if (iter % 50 == 0) {
            orc_calc_ax(m, x, r, 0);
            r[L] -= 1.0;
            res = orc_dnrm2(2 * (L + 1), (const double *)r);
            if (res <= crit) { conv = 1; break; }
        }
        if (iter >= maxit0) break;
        iter++;
    }
    memcpy(rho, x, sizeof(ozc) * L);
    x[L] = 0;
    orc_calc_ax(m, x, r, 0);
    r[L] -= 1.0;
    if (info) { info->iters = iter; info->axb = iter; info->ierr = conv ? 0 : 1; info->exit_reason = conv; info->resid = orc_dnrm2(2 * (L + 1), (const double *)r); }
    free(x); free(xn); free(r);
    return 0;
}
