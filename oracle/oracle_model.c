/*
 * oracle_model.c -- bath coefficients, fermionic operators and system
 * Hamiltonians of HEOM-QUICK2, restated in plain C (FP64).
 * TEST INFRASTRUCTURE ONLY (see heom_oracle.h).
 */
#include "oracle_internal.h"

static char g_err[256];
const char *orc_last_error(void) { return g_err; }
void orc_set_error(const char *msg) { snprintf(g_err, sizeof g_err, "%s", msg); }

/* ---- small dense symmetric eigensolver (cyclic Jacobi), ascending eigenvalues ---- */
void orc_symeig(int n, double *a /* n*n col-major, destroyed */, double *w, double *v /* may be NULL */)
{
    if (v) { for (int i = 0; i < n * n; i++) v[i] = 0.0; for (int i = 0; i < n; i++) v[i + i * n] = 1.0; }
    for (int sweep = 0; sweep < 100; sweep++) {
        double off = 0.0;
        for (int j = 0; j < n; j++) for (int i = 0; i < j; i++) off += a[i + j * n] * a[i + j * n];
        if (off < 1e-30) break;
        for (int p = 0; p < n; p++) for (int q = p + 1; q < n; q++) {
            double apq = a[p + q * n];
            if (fabs(apq) < 1e-300) continue;
            double app = a[p + p * n], aqq = a[q + q * n];
            double theta = (aqq - app) / (2.0 * apq);
            double t = (theta >= 0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1.0));
            double c = 1.0 / sqrt(t * t + 1.0), s = t * c;
            for (int k = 0; k < n; k++) {
                double akp = a[k + p * n], akq = a[k + q * n];
                a[k + p * n] = c * akp - s * akq;
                a[k + q * n] = s * akp + c * akq;
            }
            for (int k = 0; k < n; k++) {
                double apk = a[p + k * n], aqk = a[q + k * n];
                a[p + k * n] = c * apk - s * aqk;
                a[q + k * n] = s * apk + c * aqk;
            }
            if (v) for (int k = 0; k < n; k++) {
                double vkp = v[k + p * n], vkq = v[k + q * n];
                v[k + p * n] = c * vkp - s * vkq;
                v[k + q * n] = s * vkp + c * vkq;
            }
        }
    }
    /* sort ascending (selection sort carrying vectors) */
    for (int i = 0; i < n; i++) w[i] = a[i + i * n];
    for (int i = 0; i < n; i++) {
        int k = i;
        for (int j = i + 1; j < n; j++) if (w[j] < w[k]) k = j;
        if (k != i) {
            double t = w[i]; w[i] = w[k]; w[k] = t;
            if (v) for (int r = 0; r < n; r++) { double tv = v[r + i * n]; v[r + i * n] = v[r + k * n]; v[r + k * n] = tv; }
        }
    }
}

/* main/zpout_psd.f90:23-114: Pade poles/residues of the Fermi function,
 * f(z) = 1/2 + sum_i zcoef_i (1/(z+zpole_i) + 1/(z-zpole_i)). */
static void orc_pade(int mpole, double *coef, ozc pole[][2])
{
    int n0 = mpole, dim0 = 2 * mpole, dim1 = dim0 - 1;
    double *m0 = calloc((size_t)dim0 * dim0, sizeof(double));
    double *m1 = calloc((size_t)(dim1 > 0 ? dim1 : 1) * (dim1 > 0 ? dim1 : 1), sizeof(double));
    double *w0 = calloc(dim0, sizeof(double)), *w1 = calloc(dim0, sizeof(double));
    for (int j = 1; j <= dim0; j++) for (int i = 1; i <= dim0; i++)
        if (i == j + 1 || i == j - 1) m0[(i - 1) + (j - 1) * dim0] = 1.0 / sqrt((2.0 * i - 1.0) * (2.0 * j - 1.0));
    for (int j = 1; j <= dim1; j++) for (int i = 1; i <= dim1; i++)
        if (i == j + 1 || i == j - 1) m1[(i - 1) + (j - 1) * dim1] = 1.0 / sqrt((2.0 * i + 1.0) * (2.0 * j + 1.0));
    orc_symeig(dim0, m0, w0, NULL);
    if (dim1 > 0) orc_symeig(dim1, m1, w1, NULL);
    double eval0[ORC_MAXMATS], eval1[ORC_MAXMATS];
    for (int i = 0; i < n0; i++) eval0[i] = 4.0 / (w0[i] * w0[i]);
    for (int i = 0; i < n0 - 1; i++) eval1[i] = 4.0 / (w1[i] * w1[i]);
    for (int j = 0; j < n0; j++) {
        double t = 1.0;
        for (int k = 0; k < j; k++) t *= (eval1[k] - eval0[j]) / (eval0[k] - eval0[j]);
        for (int k = j + 1; k < n0; k++) t *= (eval1[k - 1] - eval0[j]) / (eval0[k] - eval0[j]);
        double eta = 0.5 * (double)(n0 * (2 * n0 + 1)) * t;
        coef[j] = -eta;
        double s = sqrt(eval0[j]);
        pole[j][0] = I * fabs(s);
        pole[j][1] = conj(pole[j][0]);
    }
    free(m0); free(m1); free(w0); free(w1);
}

/* main/fermifunc.f90:17-23 (Pade branch) */
static ozc orc_fermifunc(const orc_model *m, int isgn, ozc cin)
{
    ozc c = 0.5;
    for (int i = 0; i < m->nmats; i++)
        c += m->cpcoef[i] / (cin + m->cppole[i][isgn - 1]) + m->cpcoef[i] / (cin - m->cppole[i][isgn - 1]);
    return c;
}

/* ---- occupation-number basis: orbital 1 changes fastest, per-orbital digit
 * 0, u, d, 2 (main/calcams.f90:21-52) ---- */
static void orc_decode(int nspin, int norbs, int idx1, int occ[][2])
{
    int r = idx1 - 1;
    for (int o = 0; o < norbs; o++) {
        if (nspin == 2) { int d = r % 4; r /= 4; occ[o][0] = d & 1; occ[o][1] = (d >> 1) & 1; }
        else { int d = r % 2; r /= 2; occ[o][0] = d; occ[o][1] = 0; }
    }
}
static int orc_encode(int nspin, int norbs, int occ[][2])
{
    int r = 0, base = 1;
    for (int o = 0; o < norbs; o++) {
        int d = (nspin == 2) ? occ[o][0] + 2 * occ[o][1] : occ[o][0];
        r += d * base; base *= (nspin == 2) ? 4 : 2;
    }
    return r + 1;
}
/* main/swapms.f90: exchange spin-s occupations of orbitals iorbs-1 and iorbs */
static void orc_swapms(int nspin, int norbs, int irow, int icol, int iorbs, int ispin, int *orow, int *ocol, int *osgn)
{
    int occ[ORC_MAXORB][2] = {{0}}, sgr, sgc, t;
    orc_decode(nspin, norbs, irow, occ);
    sgr = (occ[iorbs - 2][ispin - 1] == 1 && occ[iorbs - 1][ispin - 1] == 1) ? -1 : 1;
    t = occ[iorbs - 2][ispin - 1]; occ[iorbs - 2][ispin - 1] = occ[iorbs - 1][ispin - 1]; occ[iorbs - 1][ispin - 1] = t;
    *orow = orc_encode(nspin, norbs, occ);
    orc_decode(nspin, norbs, icol, occ);
    sgc = (occ[iorbs - 2][ispin - 1] == 1 && occ[iorbs - 1][ispin - 1] == 1) ? -1 : 1;
    t = occ[iorbs - 2][ispin - 1]; occ[iorbs - 2][ispin - 1] = occ[iorbs - 1][ispin - 1]; occ[iorbs - 1][ispin - 1] = t;
    *ocol = orc_encode(nspin, norbs, occ);
    *osgn = sgr * sgc;
}
/* main/swapspin.f90: exchange up/down occupations of orbital iorbs */
static void orc_swapspin(int norbs, int irow, int icol, int iorbs, int *orow, int *ocol, int *osgn)
{
    int occ[ORC_MAXORB][2] = {{0}}, sgr, sgc, t;
    orc_decode(2, norbs, irow, occ);
    sgr = (occ[iorbs - 1][0] == 1 && occ[iorbs - 1][1] == 1) ? -1 : 1;
    t = occ[iorbs - 1][0]; occ[iorbs - 1][0] = occ[iorbs - 1][1]; occ[iorbs - 1][1] = t;
    *orow = orc_encode(2, norbs, occ);
    orc_decode(2, norbs, icol, occ);
    sgc = (occ[iorbs - 1][0] == 1 && occ[iorbs - 1][1] == 1) ? -1 : 1;
    t = occ[iorbs - 1][0]; occ[iorbs - 1][0] = occ[iorbs - 1][1]; occ[iorbs - 1][1] = t;
    *ocol = orc_encode(2, norbs, occ);
    *osgn = sgr * sgc;
}

#define AMS(m, i, j, o, s) (m)->amsori[((size_t)(i) - 1) + ((size_t)(j) - 1) * (m)->nrho + ((size_t)(o) - 1) * (m)->nrho * (m)->nrho + ((size_t)(s) - 1) * (m)->nrho * (m)->nrho * (m)->norbs]

/* main/calcams.f90 + main/buildoperator.f90:18-120 + main/arrangeoperator.f90:25-55 */
static int orc_build_operators(orc_model *m)
{
    int n = m->nrho, norbs = m->norbs, nspin = m->nspin;
    m->amsori = calloc((size_t)n * n * norbs * nspin, sizeof(double));
    double *a0 = calloc((size_t)n * n, sizeof(double));
    /* calcams(iorbs=1, ispin=1) */
    if (nspin == 1) {
        int len0 = n / (1 << norbs);
        for (int ni = 1; ni <= (1 << (norbs - 1)); ni++) {
            int r0 = (ni - 1) * len0 * 2 + 1, c0 = r0 + len0;
            for (int nj = 1; nj <= len0; nj++) a0[(r0 + nj - 2) + (size_t)(c0 + nj - 2) * n] = 1.0;
        }
    } else {
        int len0 = 1, nb = 1;
        for (int k = 0; k < norbs - 1; k++) nb *= 4;
        for (int ni = 1; ni <= nb; ni++) {
            int r0 = (ni - 1) * len0 * 4 + 1, r1 = r0 + 2 * len0, c0 = r0 + len0, c1 = r0 + 3 * len0;
            for (int nj = 1; nj <= len0; nj++) {
                a0[(r0 + nj - 2) + (size_t)(c0 + nj - 2) * n] = 1.0;
                a0[(r1 + nj - 2) + (size_t)(c1 + nj - 2) * n] = 1.0;
            }
        }
    }
    for (int i = 0; i < n * n; i++) m->amsori[i] = a0[i];
    int nunity = (nspin == 1) ? (1 << (norbs - 1)) : 2 * (int)pow(4.0, norbs - 1);
    int *irow = calloc((size_t)nunity * 2, sizeof(int)), *icol = calloc((size_t)nunity * 2, sizeof(int)),
        *isg = calloc((size_t)nunity * 2, sizeof(int));
#define IR(k, s) irow[(k) + (s - 1) * nunity]
#define IC(k, s) icol[(k) + (s - 1) * nunity]
#define IS(k, s) isg[(k) + (s - 1) * nunity]
    int nk = 0;
    for (int ni = 1; ni <= n; ni++) for (int nj = 1; nj <= n; nj++)
        if (fabs(a0[(ni - 1) + (size_t)(nj - 1) * n] - 1.0) <= 1e-9) { IR(nk, 1) = ni; IC(nk, 1) = nj; IS(nk, 1) = 1; nk++; }
    if (nk != nunity) { orc_set_error("operator build: unexpected nonzero count"); return -1; }
    if (!(nspin * norbs == 1)) {
        if (nspin == 1) {
            for (int ni = 2; ni <= norbs; ni++) {
                double *d = &AMS(m, 1, 1, ni, 1);
                for (int k = 0; k < nunity; k++) {
                    int r, c, s; orc_swapms(1, norbs, IR(k, 1), IC(k, 1), ni, 1, &r, &c, &s);
                    d[(r - 1) + (size_t)(c - 1) * n] = (double)s * IS(k, 1);
                    IR(k, 1) = r; IC(k, 1) = c; IS(k, 1) = s * IS(k, 1);
                }
            }
        } else {
            double *d = &AMS(m, 1, 1, 1, 2);
            for (int k = 0; k < nunity; k++) {
                int r, c, s; orc_swapspin(norbs, IR(k, 1), IC(k, 1), 1, &r, &c, &s);
                IR(k, 2) = r; IC(k, 2) = c; IS(k, 2) = s * IS(k, 1);
                d[(r - 1) + (size_t)(c - 1) * n] = IS(k, 2);
            }
            int ispin = 2;
            for (int ni = 2; ni <= norbs; ni++) {
                d = &AMS(m, 1, 1, ni, ispin);
                for (int k = 0; k < nunity; k++) {
                    int r, c, s; orc_swapms(2, norbs, IR(k, ispin), IC(k, ispin), ni, ispin, &r, &c, &s);
                    int v = IS(k, ispin) * s;
                    d[(r - 1) + (size_t)(c - 1) * n] = v;
                    IR(k, ispin) = r; IC(k, ispin) = c; IS(k, ispin) = v;
                }
                ispin = 3 - ispin;
                d = &AMS(m, 1, 1, ni, ispin);
                for (int k = 0; k < nunity; k++) {
                    int r, c, s; orc_swapspin(norbs, IR(k, 3 - ispin), IC(k, 3 - ispin), ni, &r, &c, &s);
                    int v = IS(k, 3 - ispin) * s;
                    d[(r - 1) + (size_t)(c - 1) * n] = v;
                    IR(k, ispin) = r; IC(k, ispin) = c; IS(k, ispin) = v;
                }
            }
        }
    }
#undef IR
#undef IC
#undef IS
    free(irow); free(icol); free(isg); free(a0);
    /* arrangeoperator: column-major scan of each dense operator */
    m->nams = nunity;
    size_t tot = (size_t)m->nams * norbs * nspin;
    m->rowams = calloc(tot, sizeof(int)); m->colams = calloc(tot, sizeof(int)); m->sgnams = calloc(tot, sizeof(int));
    for (int s = 1; s <= nspin; s++) for (int o = 1; o <= norbs; o++) {
        int cnt = 0; size_t base = (size_t)m->nams * ((o - 1) + (size_t)(s - 1) * norbs);
        for (int j = 1; j <= n; j++) for (int i = 1; i <= n; i++) {
            double v = AMS(m, i, j, o, s);
            if (fabs(v) >= ORC_DPICO) {
                if (cnt >= m->nams) { orc_set_error("operator build: too many nonzeros"); return -1; }
                m->rowams[base + cnt] = i; m->colams[base + cnt] = j; m->sgnams[base + cnt] = v > 0 ? 0 : 1; cnt++;
            }
        }
        if (cnt != m->nams) { orc_set_error("operator build: nams mismatch"); return -1; }
    }
    /* partial-permutation maps of each operator */
    size_t nm = (size_t)(n + 1) * norbs * nspin;
    m->op_rofc = calloc(nm, sizeof(int)); m->op_cofr = calloc(nm, sizeof(int));
    m->op_srofc = calloc(nm, sizeof(int)); m->op_scofr = calloc(nm, sizeof(int));
    for (int s = 1; s <= nspin; s++) for (int o = 1; o <= norbs; o++) {
        size_t base = orc_opbase(m, o, s), mb = (size_t)(n + 1) * ((o - 1) + (size_t)(s - 1) * norbs);
        for (int e = 0; e < m->nams; e++) {
            int r = m->rowams[base + e], c = m->colams[base + e], sg = m->sgnams[base + e] ? -1 : 1;
            if (m->op_rofc[mb + c] || m->op_cofr[mb + r]) { orc_set_error("operator is not a partial permutation"); return -1; }
            m->op_rofc[mb + c] = r; m->op_srofc[mb + c] = sg;
            m->op_cofr[mb + r] = c; m->op_scofr[mb + r] = sg;
        }
    }
    return 0;
}

/* dense products for the Hamiltonian builders */
static void mat_dag_mul(int n, const double *a, const double *b, ozc *c, ozc alpha, int accumulate)
{   /* c (+)= alpha * a^T b, a and b real (operators are real) */
    for (int j = 0; j < n; j++) for (int i = 0; i < n; i++) {
        double s = 0; for (int k = 0; k < n; k++) s += a[k + (size_t)i * n] * b[k + (size_t)j * n];
        if (accumulate) c[i + (size_t)j * n] += alpha * s; else c[i + (size_t)j * n] = alpha * s;
    }
}
static void cmat_mul(int n, const ozc *a, const ozc *b, ozc *c)
{
    for (int j = 0; j < n; j++) for (int i = 0; i < n; i++) {
        ozc s = 0; for (int k = 0; k < n; k++) s += a[i + (size_t)k * n] * b[k + (size_t)j * n];
        c[i + (size_t)j * n] = s;
    }
}

/* main/calchs.f90: para1 (:257-330, 363-380), para4 (:464-577); Kanamori H for the
 * lreadhs path (:78-85) built from the same operators. */
static int orc_build_hs(orc_model *m, const orc_params *p)
{
    int n = m->nrho;
    size_t nn = (size_t)n * n;
    m->hs = calloc(nn, sizeof(ozc));
    ozc *t1 = calloc(nn, sizeof(ozc)), *t2 = calloc(nn, sizeof(ozc)), *t3 = calloc(nn, sizeof(ozc));
    const double hb = ORC_HBAR;
    if (p->model == ORC_MODEL_PARA1) {
        if (!(m->norbs == 1 && m->nspin == 2)) { orc_set_error("para1 needs norbs=1,nspin=2"); return -1; }
        const double *cu = &AMS(m, 1, 1, 1, 1), *cd = &AMS(m, 1, 1, 1, 2);
        mat_dag_mul(n, cu, cu, t1, 1.0, 0);   /* n_up */
        mat_dag_mul(n, cd, cd, t2, 1.0, 0);   /* n_down */
        cmat_mul(n, t1, t2, t3);
        for (size_t k = 0; k < nn; k++) m->hs[k] = (p->eup / hb) * t1[k] + (p->edown / hb) * t2[k] + (p->uu / hb) * t3[k];
    } else if (p->model == ORC_MODEL_PARA4) {
        if (!(m->norbs == 2 && m->nspin == 2)) { orc_set_error("para4 needs norbs=2,nspin=2"); return -1; }
        const double *c1u = &AMS(m, 1, 1, 1, 1), *c1d = &AMS(m, 1, 1, 1, 2), *c2u = &AMS(m, 1, 1, 2, 1), *c2d = &AMS(m, 1, 1, 2, 2);
        ozc *n1u = calloc(nn, sizeof(ozc)), *n1d = calloc(nn, sizeof(ozc)), *n2u = calloc(nn, sizeof(ozc)), *n2d = calloc(nn, sizeof(ozc));
        ozc *n1 = calloc(nn, sizeof(ozc)), *n2 = calloc(nn, sizeof(ozc)), *hop = calloc(nn, sizeof(ozc));
        mat_dag_mul(n, c1u, c1u, n1u, 1.0, 0); mat_dag_mul(n, c1d, c1d, n1d, 1.0, 0);
        mat_dag_mul(n, c2u, c2u, n2u, 1.0, 0); mat_dag_mul(n, c2d, c2d, n2d, 1.0, 0);
        for (size_t k = 0; k < nn; k++) {
            m->hs[k] = (p->e1up / hb) * n1u[k] + (p->e1down / hb) * n1d[k] + (p->e2up / hb) * n2u[k] + (p->e2down / hb) * n2d[k];
            n1[k] = n1u[k] + n1d[k]; n2[k] = n2u[k] + n2d[k];
        }
        cmat_mul(n, n1u, n1d, t1); cmat_mul(n, n2u, n2d, t2); cmat_mul(n, n1, n2, t3);
        for (size_t k = 0; k < nn; k++) m->hs[k] += (p->uu1 / hb) * t1[k] + (p->uu2 / hb) * t2[k] + (p->u12 / hb) * t3[k];
        mat_dag_mul(n, c1u, c2u, hop, 1.0, 0); mat_dag_mul(n, c2u, c1u, hop, 1.0, 1);
        mat_dag_mul(n, c1d, c2d, hop, 1.0, 1); mat_dag_mul(n, c2d, c1d, hop, 1.0, 1);
        for (size_t k = 0; k < nn; k++) m->hs[k] += (p->t12 / hb) * hop[k];
        free(n1u); free(n1d); free(n2u); free(n2d); free(n1); free(n2); free(hop);
    } else if (p->model == ORC_MODEL_KANAMORI) {
        /* Kanamori: eps*sum n + U sum n_up n_dn + U' sum_{m!=m'} n_mu n_m'd + (U'-J) sum_{m<m',s} n_ms n_m's
         *           - J sum_{m!=m'} c+_mu c_md c+_m'd c_m'u + J sum_{m!=m'} c+_mu c+_md c_m'd c_m'u,  U' = U - 2J */
        int no = m->norbs;
        double U = p->kan_u / hb, J = p->kan_j / hb, Up = U - 2.0 * J, eps = p->kan_eps / hb;
        ozc *c[ORC_MAXORB][2], *cd[ORC_MAXORB][2], *nm[ORC_MAXORB][2];
        for (int o = 0; o < no; o++) for (int s = 0; s < 2; s++) {
            c[o][s] = calloc(nn, sizeof(ozc)); cd[o][s] = calloc(nn, sizeof(ozc)); nm[o][s] = calloc(nn, sizeof(ozc));
            const double *a = &AMS(m, 1, 1, o + 1, s + 1);
            for (int j = 0; j < n; j++) for (int i = 0; i < n; i++) {
                c[o][s][i + (size_t)j * n] = a[i + (size_t)j * n];
                cd[o][s][i + (size_t)j * n] = a[j + (size_t)i * n];
            }
            cmat_mul(n, cd[o][s], c[o][s], nm[o][s]);
        }
        ozc *w1 = calloc(nn, sizeof(ozc)), *w2 = calloc(nn, sizeof(ozc));
        for (int o = 0; o < no; o++) {
            for (size_t k = 0; k < nn; k++) m->hs[k] += eps * (nm[o][0][k] + nm[o][1][k]);
            cmat_mul(n, nm[o][0], nm[o][1], t1);
            for (size_t k = 0; k < nn; k++) m->hs[k] += U * t1[k];
        }
        for (int o = 0; o < no; o++) for (int q = 0; q < no; q++) {
            if (o == q) continue;
            cmat_mul(n, nm[o][0], nm[q][1], t1);
            for (size_t k = 0; k < nn; k++) m->hs[k] += Up * t1[k];
            if (o < q) for (int s = 0; s < 2; s++) {
                cmat_mul(n, nm[o][s], nm[q][s], t1);
                for (size_t k = 0; k < nn; k++) m->hs[k] += (Up - J) * t1[k];
            }
            /* spin flip: -J c+_ou c_od c+_qd c_qu */
            cmat_mul(n, cd[o][0], c[o][1], w1); cmat_mul(n, w1, cd[q][1], w2); cmat_mul(n, w2, c[q][0], t1);
            for (size_t k = 0; k < nn; k++) m->hs[k] += -J * t1[k];
            /* pair hopping: +J c+_ou c+_od c_qd c_qu */
            cmat_mul(n, cd[o][0], cd[o][1], w1); cmat_mul(n, w1, c[q][1], w2); cmat_mul(n, w2, c[q][0], t1);
            for (size_t k = 0; k < nn; k++) m->hs[k] += J * t1[k];
        }
        for (int o = 0; o < no; o++) for (int s = 0; s < 2; s++) { free(c[o][s]); free(cd[o][s]); free(nm[o][s]); }
        free(w1); free(w2);
    } else if (p->model == ORC_MODEL_READHS) {
        if (!p->hs_in) { orc_set_error("READHS model without hs_in"); return -1; }
        for (size_t k = 0; k < nn; k++) m->hs[k] = p->hs_in[k];
    } else { orc_set_error("unknown model"); return -1; }
    free(t1); free(t2); free(t3);
    return 0;
}

#define CBIDX(m, iorbs, ispin, icor, ialf, isgn) \
    (((((size_t)(isgn) - 1) * (m)->nalf + ((ialf) - 1)) * (m)->ncor + ((icor) - 1)) * (m)->nspin * (m)->norbs + ((size_t)(ispin) - 1) * (m)->norbs + ((iorbs) - 1))

size_t orc_cbidx(const orc_model *m, int iorbs, int ispin, int icor, int ialf, int isgn)
{ return CBIDX(m, iorbs, ispin, icor, ialf, isgn); }

/* main/evaluatepara.f90:1155-1232 (sizes), 1442-1497 (zxip), 1555-1562 (doubledot),
 * 1666-1773 (operator/drawer order and complement maps), 1897-2020 (cb, cd, cgama for
 * the Lorentzian PSD case), 2210-2227 (cgamma per drawer), 2297 + 2427-2435 (eleadinfty),
 * 3054-3100 (jomit / indexdraw). */
static int orc_build_coefficients(orc_model *m, const orc_params *p)
{
    const double hb = ORC_HBAR;
    m->nsgn = 2;
    m->ndrude = 1;             /* yshift = 1e10 > bandwidth (evaluatepara.f90:978,1166-1185) */
    double width[ORC_MAXALF];
    for (int a = 0; a < m->nalf; a++) width[a] = p->bandwidth[a];
    m->npsf = p->npsf > 0 ? p->npsf : 0;
    if (m->npsf) {
        /* psfjob (evaluatepara.f90:256-722, 1187-1189): nmats = npsf fitted terms, no Drude
         * pole, bandwidth = dinvbeta * rpsf, band centre 0 */
        if (m->npsf > ORC_MAXMATS || !p->psf_coef || !p->psf_pole || !(p->tpsf > 0) || !(p->rpsf > 0)) {
            orc_set_error("psfjob needs 1..64 coefficients and poles, tpsf > 0, rpsf > 0");
            return -1;
        }
        m->ndrude = 0;
        m->nmats = m->npsf;
        m->tpsf = p->tpsf;
        for (int k = 0; k < m->npsf; k++) { m->psfcoef[k] = p->psf_coef[k]; m->psfpole[k] = p->psf_pole[k]; }
        for (int a = 0; a < m->nalf; a++) width[a] = p->temperature[a] * p->rpsf;
    }
    m->ncor = m->ndrude + m->nmats;
    m->nopr = m->nsgn * m->norbs * m->nspin * m->nalf;
    m->nvar = m->nopr * m->ncor;
    m->nrho = 1; for (int k = 0; k < m->norbs; k++) m->nrho *= m->nspin * 2;
    if (!m->npsf) orc_pade(m->nmats, m->cpcoef, m->cppole);
    /* zxip (offcor = F) */
    for (int a = 0; a < m->nalf; a++) for (int o = 0; o < m->norbs; o++)
        m->zxip[a][o] = p->linewidth[a][o] * width[a] * width[a] * 0.5;
    double lw[ORC_MAXALF][ORC_MAXORB];
    for (int a = 0; a < m->nalf; a++) for (int o = 0; o < m->norbs; o++) lw[a][o] = p->linewidth[a][o];
    if (p->doubledot) {
        if (m->norbs != 2 || m->nalf != 2) { orc_set_error("doubledot needs norbs=2,nalf=2"); return -1; }
        lw[0][1] = 0.0; lw[1][0] = 0.0;
        for (int a = 0; a < 2; a++) for (int o = 0; o < 2; o++) m->zxip[a][o] = 0.0;
        m->zxip[0][0] = lw[0][0] * width[0] * width[0] * 0.5;
        m->zxip[1][1] = lw[1][1] * width[1] * width[1] * 0.5;
    }
    for (int a = 0; a < m->nalf; a++) for (int o = 0; o < m->norbs; o++) m->hybrid[a][o] = lw[a][o] / hb;
    size_t ncb = (size_t)m->norbs * m->nspin * m->ncor * m->nalf * m->nsgn;
    m->cb = calloc(ncb, sizeof(ozc)); m->cd = calloc(ncb, sizeof(ozc)); m->cgama = calloc(ncb, sizeof(ozc));
    const double dpm[2] = {1.0, -1.0};
    for (int ni = 1; ni <= 2; ni++) for (int nm = 1; nm <= m->nspin; nm++) for (int nk = 1; nk <= m->norbs; nk++)
    for (int nj = 1; nj <= m->nalf; nj++) for (int np = 1; np <= m->ncor; np++) {
        double T = p->temperature[nj - 1], beta = 1.0 / T, W = width[nj - 1];
        double zx = m->zxip[nj - 1][nk - 1], gp = W, dwp = 0.0;
        size_t id = CBIDX(m, nk, nm, np, nj, ni);
        if (m->npsf) {
            /* PSF scheme (evaluatepara.f90:1993-2000): cgama = T / tpsf zpole, cb = T / tpsf zcoef
             * 2 zxip / W^2, cd = conj(cb); the same fit serves both signs (zpout_psf.f90) */
            const double s = T / m->tpsf;
            m->cgama[id] = s * m->psfpole[np - 1];
            m->cb[id] = s * m->psfcoef[np - 1] * (zx / (W * W) * 2.0);
            m->cd[id] = conj(m->cb[id]);
        } else if (np <= m->ndrude) {
            m->cgama[id] = (-gp + I * dpm[ni - 1] * dwp) / hb;
            ozc c1 = beta * (dpm[ni - 1] * dwp + I * gp);
            ozc f1 = orc_fermifunc(m, ni, c1);
            m->cb[id] = zx / gp * f1 / (hb * hb);
            ozc c2 = beta * (dpm[2 - ni] * dwp + I * gp);
            ozc f2 = orc_fermifunc(m, 3 - ni, c2);
            m->cd[id] = conj(zx / gp * f2) / (hb * hb);
        } else {
            int im = np - m->ndrude - 1;
            ozc pole = m->cppole[im][ni - 1], polet = m->cppole[im][2 - ni];
            m->cgama[id] = dpm[ni - 1] * I * T * pole / hb;
            ozc num = I * 2.0 * m->cpcoef[im] * zx * T;
            m->cb[id] = num / ((pole * T - dwp) * (pole * T - dwp) + gp * gp) / (hb * hb);
            m->cd[id] = conj(num) / conj((polet * T - dwp) * (polet * T - dwp) + gp * gp) / (hb * hb);
        }
    }
    /* operators and drawers */
    m->jpm = calloc(m->nopr, sizeof(int)); m->jspin = calloc(m->nopr, sizeof(int));
    m->jorbs = calloc(m->nopr, sizeof(int)); m->jalf = calloc(m->nopr, sizeof(int));
    m->jredex = calloc(m->nopr, sizeof(int)); m->jomit = calloc(m->nopr, sizeof(int));
    int half = m->nopr / 2;
    for (int l = 1; l <= m->nopr; l++) m->jredex[l - 1] = l <= half ? l + half : l - half;
    int nq = 0;
    for (int s = 1; s <= 2; s++) for (int sp = 1; sp <= m->nspin; sp++) for (int o = 1; o <= m->norbs; o++)
    for (int a = 1; a <= m->nalf; a++) {
        m->jpm[nq] = s; m->jspin[nq] = sp; m->jorbs[nq] = o; m->jalf[nq] = a;
        m->jomit[nq] = fabs(m->zxip[a - 1][o - 1]) < ORC_DSMALL ? 1 : 0;
        nq++;
    }
    m->cgamma = calloc(m->nvar, sizeof(ozc)); m->dipm = calloc(m->nvar, sizeof(double));
    m->mpm = calloc(m->nvar, sizeof(int)); m->morbs = calloc(m->nvar, sizeof(int)); m->mspin = calloc(m->nvar, sizeof(int));
    m->ilead = calloc(m->nvar, sizeof(int)); m->mcor = calloc(m->nvar, sizeof(int)); m->mopr = calloc(m->nvar, sizeof(int));
    m->iredex = calloc(m->nvar, sizeof(int)); m->indexdraw = calloc(m->nvar, sizeof(int));
    nq = 0;
    for (int s = 1; s <= 2; s++) for (int sp = 1; sp <= m->nspin; sp++) for (int o = 1; o <= m->norbs; o++)
    for (int a = 1; a <= m->nalf; a++) {
        int isopr = (s - 1) * m->nspin * m->norbs + (sp - 1) * m->norbs + o;
        int iopr = (isopr - 1) * m->nalf + a;
        for (int k = 1; k <= m->ncor; k++) {
            m->mopr[nq] = iopr; m->dipm[nq] = s == 1 ? 1.0 : -1.0; m->mpm[nq] = s;
            m->ilead[nq] = a; m->morbs[nq] = o; m->mspin[nq] = sp; m->mcor[nq] = k;
            m->cgamma[nq] = m->cgama[CBIDX(m, o, sp, k, a, s)];
            nq++;
        }
    }
    int nhalf = m->nvar / 2;
    for (int l = 1; l <= m->nvar; l++) m->iredex[l - 1] = l <= nhalf ? l + nhalf : l - nhalf;
    int np = 0;
    for (int d = 1; d <= m->nvar; d++) {
        if (m->lscreen && m->jomit[m->mopr[d - 1] - 1] == 1) m->indexdraw[d - 1] = 0;
        else m->indexdraw[d - 1] = ++np;
    }
    for (int a = 0; a < m->nalf; a++) m->temperature[a] = p->temperature[a];
    for (int a = 0; a < m->nalf; a++) for (int s = 0; s < m->nspin; s++) {
        m->amps[a][s] = p->engyshift[a][s] / hb;
        m->tchar[a][s] = p->tchar[a][s];
        m->eleadinfty[a][s] = m->amps[a][s];   /* getengyshift(1e10), fieldtype 0 */
    }
    return 0;
}

/* td/getengyshift.f90 (fieldtype 0): eshift = amps (1 - exp(-t/tchar)) */
void orc_eshift(const orc_model *m, double t, double es[ORC_MAXALF][2])
{
    for (int a = 0; a < ORC_MAXALF; a++) for (int s = 0; s < 2; s++) es[a][s] = 0.0;
    for (int a = 0; a < m->nalf; a++) for (int s = 0; s < m->nspin; s++) {
        double tc = m->tchar[a][s];
        if (tc > 0) es[a][s] = m->amps[a][s] * (1.0 - exp(-t / tc));
        else es[a][s] = t > 0 ? m->amps[a][s] : 0.0;
    }
}

int orc_build(const orc_params *p, orc_model **out)
{
    *out = NULL;
    if (p->norbs < 1 || p->norbs > ORC_MAXORB || (p->nspin != 1 && p->nspin != 2) || p->nalf < 1 || p->nalf > ORC_MAXALF
        || p->nmats < 1 || p->nmats > ORC_MAXMATS || p->ntier < 2 || p->ntier > ORC_MAXTIER) {
        orc_set_error("parameters out of range"); return -1;
    }
    orc_model *m = calloc(1, sizeof(orc_model));
    m->norbs = p->norbs; m->nspin = p->nspin; m->nalf = p->nalf; m->nmats = p->nmats; m->ntier = p->ntier;
    m->lscreen = p->lscreen;
    if (orc_build_coefficients(m, p) || orc_build_operators(m) || orc_build_hs(m, p)
        || orc_build_tables(m) || orc_build_pattern(m, p->pattern_seed ? p->pattern_seed : 20261203ULL)) {
        orc_free(m); return -1;
    }
    *out = m;
    return 0;
}

void orc_free(orc_model *m)
{
    if (!m) return;
    void *ptrs[] = {m->cb, m->cd, m->cgama, m->cgamma, m->dipm, m->mpm, m->morbs, m->mspin, m->ilead, m->mcor, m->mopr,
                    m->iredex, m->indexdraw, m->jpm, m->jspin, m->jorbs, m->jalf, m->jredex, m->jomit, m->amsori,
                    m->rowams, m->colams, m->sgnams, m->op_rofc, m->op_cofr, m->op_srofc, m->op_scofr, m->hs, m->indextable, m->index_coef_ref, m->indexcoef,
                    m->itypecoef, m->ifactfcoef, m->ifactrcoef, m->nnz_spa, m->ind_spa, m->irow_spa, m->icol_spa};
    for (size_t i = 0; i < sizeof ptrs / sizeof ptrs[0]; i++) free(ptrs[i]);
    free(m);
}
