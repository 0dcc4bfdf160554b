/*
 * oracle_cf.c -- the frequency-domain correlation-function system of HEOM-QUICK2's sparse
 * mode, restated in plain C.  TEST INFRASTRUCTURE ONLY.
 *
 * corrfunc/prelude_cf_spa.f90:146-760   the hierarchy pattern of B rho (B = a or a^dagger
 *                                       of one spin-orbital): RDO seed E a E + E a^dag E,
 *                                       E = exp(0.314 H), then the tier recursion of
 *                                       prelude_spa with its random mixing
 * corrfunc/calc_ax_cf_spa_omp.f90       the operator on the two components (h, a) of the
 *                                       unknown: same-tier terms per component, couplings
 *                                       and the +-omega shift across components
 * corrfunc/solve_cf_tfqmr_spa.f90:130-160  the right-hand sides brhoh, brhoa
 *
 * The products follow the same per-entry accumulation as oracle_apply.c, on the patterns
 * of this file.
 */
#include "oracle_internal.h"
#ifdef _OPENMP
#include <omp.h>
#endif

/* dense a_{iorbs,ispin}: a(ra, ca) = sign */
static void cf_dense_op(const orc_model *m, int iorbs, int ispin, ozc *a)
{
    int n = m->nrho;
    for (size_t k = 0; k < (size_t)n * n; k++) a[k] = 0;
    size_t ob = orc_opbase(m, iorbs, ispin);
    for (int e = 0; e < m->nams; e++)
        a[(m->rowams[ob + e] - 1) + (size_t)(m->colams[ob + e] - 1) * n] = m->sgnams[ob + e] ? -1.0 : 1.0;
}

static void cf_matmul(int n, const ozc *a, const ozc *b, ozc *c)
{
    for (int j = 0; j < n; j++) for (int i = 0; i < n; i++) {
        ozc s = 0; for (int k = 0; k < n; k++) s += a[i + (size_t)k * n] * b[k + (size_t)j * n];
        c[i + (size_t)j * n] = s;
    }
}

int orc_cf_build(const orc_model *m, int iorbs, int ispin, unsigned long long seed, orc_cf **out)
{
    if (iorbs < 1 || iorbs > m->norbs || ispin < 1 || ispin > m->nspin) { orc_set_error("orc_cf_build: invalid spin-orbital"); return -1; }
    int n = m->nrho; size_t nn = (size_t)n * n;
    orc_rng_seed(seed);
    orc_cf *cf = calloc(1, sizeof(orc_cf));
    cf->iorbs = iorbs; cf->ispin = ispin;
    ozc *e10 = calloc(nn, sizeof(ozc)), *a = calloc(nn, sizeof(ozc)), *t1 = calloc(nn, sizeof(ozc));
    ozc *t7 = calloc(nn, sizeof(ozc)), *t8 = calloc(nn, sizeof(ozc)), *seedm = calloc(nn, sizeof(ozc));
    orc_exp_taylor(n, m->hs, 0.31415926, 10, e10);
    cf_dense_op(m, iorbs, ispin, a);
    /* cmtmp7 = E (a E), cmtmp8 = (E a^dagger) E (prelude_cf_spa.f90:585-600) */
    cf_matmul(n, a, e10, t1); cf_matmul(n, e10, t1, t7);
    ozc *ad = calloc(nn, sizeof(ozc));
    for (int j = 0; j < n; j++) for (int i = 0; i < n; i++) ad[i + (size_t)j * n] = conj(a[j + (size_t)i * n]);
    cf_matmul(n, e10, ad, t1); cf_matmul(n, t1, e10, t8);
    ozc c1, c2;
    do { c1 = orc_normal() + I * orc_normal(); c2 = orc_normal() + I * orc_normal(); }
    while (!(cabs(c1) > 1e-6 && cabs(c2) > 1e-6));
    for (size_t k = 0; k < nn; k++) seedm[k] = c1 * t7[k] + c2 * t8[k];
    int64_t cap = (int64_t)nn * 64;
    cf->nnzcf = calloc(m->nunk, sizeof(int)); cf->indcf = calloc(m->nunk, sizeof(int64_t));
    int *ir = malloc(sizeof(int) * cap), *ic = malloc(sizeof(int) * cap);
    ozc *val = malloc(sizeof(ozc) * cap);
    int64_t lunk = 0;
    for (int j = 1; j <= n; j++) for (int i = 1; i <= n; i++) {
        ozc v = seedm[(i - 1) + (size_t)(j - 1) * n];
        if (cabs(v) > ORC_DSMALL) { ir[lunk] = i; ic[lunk] = j; val[lunk] = v; lunk++; }
    }
    cf->nnzcf[0] = (int)lunk; cf->indcf[0] = 1;
    /* E by columns: its nonzeros as COO, column-major */
    int e0n = 0;
    int *e0r = malloc(sizeof(int) * nn), *e0c = malloc(sizeof(int) * nn); ozc *e0v = malloc(sizeof(ozc) * nn);
    for (int j = 1; j <= n; j++) for (int i = 1; i <= n; i++) {
        ozc v = e10[(i - 1) + (size_t)(j - 1) * n];
        if (cabs(v) > ORC_DSMALL) { e0r[e0n] = i; e0c[e0n] = j; e0v[e0n] = v; e0n++; }
    }
    int *e0cp = calloc(n + 2, sizeof(int));
    for (int q = 0; q < e0n; q++) e0cp[e0c[q]]++;
    for (int j = 1; j <= n + 1; j++) e0cp[j] += e0cp[j - 1];
    ozc *acc = calloc(nn, sizeof(ozc));
    int *tr = malloc(sizeof(int) * nn), *tc = malloc(sizeof(int) * nn); ozc *tv = malloc(sizeof(ozc) * nn);
    for (int itier = 2; itier <= m->ntier; itier++) {
        int nb = itier - 1;
        for (int64_t lni = m->nfirst[itier - 1]; lni <= m->nlast[itier - 1]; lni++) {
            int64_t lnl = m->index_coef_ref[lni - 1];
            for (size_t k = 0; k < nn; k++) acc[k] = 0;
            double dmin = 1e300;
            for (int b = 1; b <= nb; b++) {
                int d = m->indextable[m->ifirst[itier - 1] - 1 + (lni - m->nfirst[itier - 1]) * nb + b - 1];
                int64_t lnj = m->indexcoef[lnl - 1]; int itype = m->itypecoef[lnl - 1];
                lnl++;
                int isgn = m->mpm[d - 1], io = m->morbs[d - 1], is = m->mspin[d - 1], ia = m->ilead[d - 1];
                double hyb = fabs(m->hybrid[ia - 1][io - 1]);
                if (hyb < dmin) dmin = hyb;
                if (hyb < ORC_DSMALL) continue;
                int64_t st = cf->indcf[lnj - 1] - 1; int nz = cf->nnzcf[lnj - 1];
                ozc m1, m2;
                do { m1 = orc_normal() + I * orc_normal(); m2 = orc_normal() + I * orc_normal(); }
                while (!(cabs(m1) > 1e-6 && cabs(m2) > 1e-6));
                for (int side = 0; side < 2; side++) {
                    int cnt = orc_ams_coo(m, side == 0, isgn == 1, itype != 0, io, is, nz, ir + st, ic + st, val + st, tr, tc, tv);
                    ozc cm = side == 0 ? m1 : m2;
                    for (int q = 0; q < cnt; q++) {
                        int k = tr[q], j = tc[q];
                        for (int e = e0cp[k - 1]; e < e0cp[k]; e++)
                            acc[(e0r[e] - 1) + (size_t)(j - 1) * n] += cm * (e0v[e] * tv[q]);
                    }
                }
            }
            int na = 0;
            if (dmin > ORC_DSMALL) {
                for (int j = 1; j <= n; j++) for (int i = 1; i <= n; i++) {
                    ozc v = acc[(i - 1) + (size_t)(j - 1) * n];
                    if (cabs(v) >= ORC_DSMALL) {
                        if (lunk + 1 > cap) {
                            cap *= 2; ir = realloc(ir, sizeof(int) * cap); ic = realloc(ic, sizeof(int) * cap);
                            val = realloc(val, sizeof(ozc) * cap);
                        }
                        ir[lunk] = i; ic[lunk] = j; val[lunk] = v; lunk++; na++;
                    }
                }
            }
            cf->nnzcf[lni - 1] = na;
            cf->indcf[lni - 1] = cf->indcf[lni - 2] + cf->nnzcf[lni - 2];
        }
    }
    cf->lunkcf = lunk;
    cf->irowcf = realloc(ir, sizeof(int) * (lunk > 0 ? lunk : 1));
    cf->icolcf = realloc(ic, sizeof(int) * (lunk > 0 ? lunk : 1));
    free(val); free(e10); free(a); free(ad); free(t1); free(t7); free(t8); free(seedm);
    free(e0r); free(e0c); free(e0v); free(e0cp); free(acc); free(tr); free(tc); free(tv);
    *out = cf;
    return 0;
}

void orc_cf_free(orc_cf *cf)
{
    if (!cf) return;
    free(cf->nnzcf); free(cf->indcf); free(cf->irowcf); free(cf->icolcf); free(cf);
}

static inline ozc cfb(const orc_model *m, int d)
{ return m->cb[orc_cbidx(m, m->morbs[d - 1], m->mspin[d - 1], m->mcor[d - 1], m->ilead[d - 1], m->mpm[d - 1])]; }
static inline ozc cfd(const orc_model *m, int d)
{ return m->cd[orc_cbidx(m, m->morbs[d - 1], m->mspin[d - 1], m->mcor[d - 1], m->ilead[d - 1], m->mpm[d - 1])]; }

/* y_n += cl op(a) op(X_j) + cr op(X_j) op(a) on the cf pattern of n (pos map); X_j from x */
static void cf_add_coupling(const orc_model *m, const orc_cf *cf, const int *pos, ozc *yn, const ozc *x, int64_t j,
                            int itype, int iorbs, int ispin, int dag_a, ozc cl, ozc cr)
{
    int n = m->nrho, nz = cf->nnzcf[j - 1];
    int64_t st = cf->indcf[j - 1] - 1;
    for (int q = 0; q < nz; q++) {
        int br = cf->irowcf[st + q], bc = cf->icolcf[st + q];
        ozc v = x[st + q];
        if (itype) { int t = br; br = bc; bc = t; v = conj(v); }
        int sg, i = orc_left_row(m, iorbs, ispin, dag_a, br, &sg);
        if (i) { int p = pos[(i - 1) + (bc - 1) * n]; if (p >= 0) yn[p] += cl * (sg * v); }
        int jj = orc_right_col(m, iorbs, ispin, dag_a, bc, &sg);
        if (jj) { int p = pos[(br - 1) + (jj - 1) * n]; if (p >= 0) yn[p] += cr * (sg * v); }
    }
}

void orc_cf_apply(const orc_model *m, const orc_cf *cf, double omega, int isgnw, const ozc *xh, const ozc *xa,
                  ozc *yh, ozc *ya, int nthreads)
{
    int n = m->nrho;
    size_t nn = (size_t)n * n;
    const double sw = isgnw == 1 ? 1.0 : -1.0, fa = -sw, fb = sw;   /* dfacta, dfactb (lplus_cf) */
    const ozc zfront = -I, zrear = I;
    for (int64_t k = 0; k < cf->lunkcf; k++) yh[k] = ya[k] = 0;
    /* nonzeros of H by column and by row */
    int *hc_ptr = calloc(n + 1, sizeof(int)), *hr_ptr = calloc(n + 1, sizeof(int));
    int *hc_row = malloc(sizeof(int) * nn), *hr_col = malloc(sizeof(int) * nn);
    ozc *hc_val = malloc(sizeof(ozc) * nn), *hr_val = malloc(sizeof(ozc) * nn);
    for (int c = 0; c < n; c++) {
        hc_ptr[c + 1] = hc_ptr[c];
        for (int r = 0; r < n; r++) if (cabs(m->hs[r + (size_t)c * n]) >= ORC_DSMALL) {
            hc_row[hc_ptr[c + 1]] = r; hc_val[hc_ptr[c + 1]] = m->hs[r + (size_t)c * n]; hc_ptr[c + 1]++;
        }
    }
    for (int r = 0; r < n; r++) {
        hr_ptr[r + 1] = hr_ptr[r];
        for (int c = 0; c < n; c++) if (cabs(m->hs[r + (size_t)c * n]) >= ORC_DSMALL) {
            hr_col[hr_ptr[r + 1]] = c; hr_val[hr_ptr[r + 1]] = m->hs[r + (size_t)c * n]; hr_ptr[r + 1]++;
        }
    }
    /* ---- RDO (calc_ax_cf_spa_omp.f90 first tier) ---- */
    {
        int nz = cf->nnzcf[0];
        ozc *x0h = calloc(nn, sizeof(ozc)), *x0a = calloc(nn, sizeof(ozc));
        ozc *c1 = calloc(nn, sizeof(ozc)), *c2 = calloc(nn, sizeof(ozc)), *s4 = calloc(nn, sizeof(ozc)), *s5 = calloc(nn, sizeof(ozc));
        for (int q = 0; q < nz; q++) {
            size_t k = (cf->irowcf[q] - 1) + (size_t)(cf->icolcf[q] - 1) * n;
            x0h[k] = xh[q]; x0a[k] = xa[q];
        }
        for (int q = 0; q < nz; q++) {
            int r = cf->irowcf[q] - 1, c = cf->icolcf[q] - 1;
            ozc hxh = 0, xhh = 0, hxa = 0, xah = 0;
            for (int k = 0; k < n; k++) {
                hxh += m->hs[r + (size_t)k * n] * x0h[k + (size_t)c * n]; xhh += x0h[r + (size_t)k * n] * m->hs[k + (size_t)c * n];
                hxa += m->hs[r + (size_t)k * n] * x0a[k + (size_t)c * n]; xah += x0a[r + (size_t)k * n] * m->hs[k + (size_t)c * n];
            }
            yh[q] = -I * hxh + I * xhh + fa * omega * xa[q];
            ya[q] = -I * hxa + I * xah + fb * omega * xh[q];
        }
        for (int ispin = 1; ispin <= m->nspin; ispin++) for (int io = 1; io <= m->norbs; io++) {
            for (size_t k = 0; k < nn; k++) s4[k] = s5[k] = 0;
            for (int ia = 1; ia <= m->nalf; ia++) {
                int isopr = (ispin - 1) * m->norbs + io, iopr = (isopr - 1) * m->nalf + ia;
                if (m->lscreen && m->jomit[iopr - 1] == 1) continue;
                for (int k = 1; k <= m->ncor; k++) {
                    int d = (iopr - 1) * m->ncor + k;
                    int64_t lni = m->nfirst[1] - 1 + m->indexdraw[d - 1];
                    int64_t st = cf->indcf[lni - 1] - 1;
                    for (int q = 0; q < cf->nnzcf[lni - 1]; q++) {
                        size_t kk = (cf->irowcf[st + q] - 1) + (size_t)(cf->icolcf[st + q] - 1) * n;
                        s4[kk] += xa[st + q];   /* cmtmp4 from rcgb */
                        s5[kk] += xh[st + q];   /* cmtmp5 from rcga */
                    }
                }
            }
            size_t ob = orc_opbase(m, io, ispin);
            for (int e = 0; e < m->nams; e++) {
                int ra = m->rowams[ob + e] - 1, ca = m->colams[ob + e] - 1;
                double sg = m->sgnams[ob + e] ? -1.0 : 1.0;
                for (int j = 0; j < n; j++) {
                    c2[ra + (size_t)j * n] += -sg * s4[ca + (size_t)j * n];   /* - a S4 */
                    c1[ra + (size_t)j * n] += sg * s5[ca + (size_t)j * n];    /*   a S5 */
                }
                for (int i = 0; i < n; i++) {
                    c2[i + (size_t)ca * n] += -sg * s4[i + (size_t)ra * n];   /* - S4 a */
                    c1[i + (size_t)ca * n] += sg * s5[i + (size_t)ra * n];    /*   S5 a */
                }
            }
        }
        for (int q = 0; q < nz; q++) {
            int r = cf->irowcf[q] - 1, c = cf->icolcf[q] - 1;
            yh[q] += c2[r + (size_t)c * n] + conj(c2[c + (size_t)r * n]);
            ya[q] += c1[r + (size_t)c * n] + conj(c1[c + (size_t)r * n]);
        }
        free(x0h); free(x0a); free(c1); free(c2); free(s4); free(s5);
    }
    /* ---- tiers 2..ntier ---- */
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#endif
    for (int itier = 2; itier <= m->ntier; itier++) {
        int nb = itier - 1;
#pragma omp parallel
        {
        int *pos = malloc(sizeof(int) * nn);
        for (size_t k = 0; k < nn; k++) pos[k] = -1;
#pragma omp for schedule(dynamic, 16)
        for (int64_t lni = m->nfirst[itier - 1]; lni <= m->nlast[itier - 1]; lni++) {
            int nz = cf->nnzcf[lni - 1];
            if (nz == 0) continue;
            int64_t st = cf->indcf[lni - 1] - 1;
            const int *ir = cf->irowcf + st, *ic = cf->icolcf + st;
            ozc *yhn = yh + st, *yan = ya + st;
            for (int q = 0; q < nz; q++) pos[(ir[q] - 1) + (ic[q] - 1) * n] = q;
            const int *drw = m->indextable + m->ifirst[itier - 1] - 1 + (lni - m->nfirst[itier - 1]) * nb;
            ozc g = 0;
            for (int b = 0; b < nb; b++) {
                int d = drw[b];
                g += m->cgamma[d - 1] + I * m->dipm[d - 1] * m->eleadinfty[m->ilead[d - 1] - 1][m->mspin[d - 1] - 1];
            }
            for (int q = 0; q < nz; q++) {
                int r = ir[q] - 1, c = ic[q] - 1;
                ozc vh = xh[st + q], va = xa[st + q];
                yhn[q] += g * vh + fa * omega * va;
                yan[q] += g * va + fb * omega * vh;
                for (int k = hc_ptr[r]; k < hc_ptr[r + 1]; k++) {   /* H(i, r) x -> (i, c) */
                    int p = pos[hc_row[k] + (size_t)c * n];
                    if (p >= 0) { yhn[p] += -I * (hc_val[k] * vh); yan[p] += -I * (hc_val[k] * va); }
                }
                for (int k = hr_ptr[c]; k < hr_ptr[c + 1]; k++) {   /* x H(c, j) -> (r, j) */
                    int p = pos[r + (size_t)hr_col[k] * n];
                    if (p >= 0) { yhn[p] += I * (vh * hr_val[k]); yan[p] += I * (va * hr_val[k]); }
                }
            }
            int64_t lnl = m->index_coef_ref[lni - 1];
            for (int b = 0; b < nb; b++) {   /* lower tier: h from a-component, a from h-component */
                int d = drw[b];
                int64_t j = m->indexcoef[lnl - 1]; int itype = m->itypecoef[lnl - 1];
                double ff = m->ifactfcoef[lnl - 1], fr = m->ifactrcoef[lnl - 1];
                lnl++;
                ozc cl = cfb(m, d) * (-I * ff) * zfront, cr = cfd(m, d) * (I * fr) * zrear;
                cf_add_coupling(m, cf, pos, yhn, xa, j, itype != 0, m->morbs[d - 1], m->mspin[d - 1], m->mpm[d - 1] == 1, cl, cr);
                cf_add_coupling(m, cf, pos, yan, xh, j, itype != 0, m->morbs[d - 1], m->mspin[d - 1], m->mpm[d - 1] == 1, -cl, -cr);
            }
            if (itier < m->ntier) {          /* higher tier */
                for (int isgn = 1; isgn <= 2; isgn++) for (int ispin = 1; ispin <= m->nspin; ispin++)
                for (int io = 1; io <= m->norbs; io++) for (int ia = 1; ia <= m->nalf; ia++) {
                    int isopr = (isgn - 1) * m->nspin * m->norbs + (ispin - 1) * m->norbs + io;
                    int iopr = (isopr - 1) * m->nalf + ia;
                    if (m->lscreen && m->jomit[iopr - 1] == 1) continue;
                    for (int k = 1; k <= m->ncor; k++) {
                        int64_t j = m->indexcoef[lnl - 1]; int itype = m->itypecoef[lnl - 1];
                        double ff = m->ifactfcoef[lnl - 1], fr = m->ifactrcoef[lnl - 1];
                        lnl++;
                        if (cf->nnzcf[j - 1] == 0) continue;
                        ozc cl = (-I * ff) * zfront, cr = (I * fr) * zrear;
                        cf_add_coupling(m, cf, pos, yhn, xa, j, itype != 0, io, ispin, isgn != 1, cl, cr);
                        cf_add_coupling(m, cf, pos, yan, xh, j, itype != 0, io, ispin, isgn != 1, -cl, -cr);
                    }
                }
            }
            for (int q = 0; q < nz; q++) pos[(ir[q] - 1) + (ic[q] - 1) * n] = -1;
        }
        free(pos);
        }
    }
    free(hc_ptr); free(hr_ptr); free(hc_row); free(hr_col); free(hc_val); free(hr_val);
}

void orc_cf_rhs(const orc_model *m, const orc_cf *cf, const ozc *rho, int isgnb, ozc *bh, ozc *ba)
{
    int n = m->nrho;
    size_t nn = (size_t)n * n;
    const int dag_l = isgnb == 1, dag_r = isgnb != 1;   /* isgnb 1: a^dag rho + rho a; 2: a rho + rho a^dag */
    ozc *r = calloc(nn, sizeof(ozc)), *l = calloc(nn, sizeof(ozc)), *rr = calloc(nn, sizeof(ozc));
    for (int64_t k = 0; k < cf->lunkcf; k++) bh[k] = ba[k] = 0;
    for (int64_t lni = 1; lni <= m->nunk; lni++) {
        if (m->nnz_spa[lni - 1] == 0 || cf->nnzcf[lni - 1] == 0) continue;
        for (size_t k = 0; k < nn; k++) r[k] = l[k] = rr[k] = 0;
        int64_t st = m->ind_spa[lni - 1] - 1;
        for (int q = 0; q < m->nnz_spa[lni - 1]; q++)
            r[(m->irow_spa[st + q] - 1) + (size_t)(m->icol_spa[st + q] - 1) * n] = rho[st + q];
        for (int c = 1; c <= n; c++) for (int i0 = 1; i0 <= n; i0++) {
            ozc v = r[(i0 - 1) + (size_t)(c - 1) * n];
            if (v == 0) continue;
            int sg, i = orc_left_row(m, cf->iorbs, cf->ispin, dag_l, i0, &sg);
            if (i) l[(i - 1) + (size_t)(c - 1) * n] += sg * v;            /* op_l(a) rho */
            int jj = orc_right_col(m, cf->iorbs, cf->ispin, dag_r, c, &sg);
            if (jj) rr[(i0 - 1) + (size_t)(jj - 1) * n] += sg * v;        /* rho op_r(a) */
        }
        int64_t sc = cf->indcf[lni - 1] - 1;
        for (int q = 0; q < cf->nnzcf[lni - 1]; q++) {
            size_t k = (cf->irowcf[sc + q] - 1) + (size_t)(cf->icolcf[sc + q] - 1) * n;
            bh[sc + q] = l[k] + rr[k];
            ba[sc + q] = -I * l[k] + I * rr[k];
        }
    }
    free(r); free(l); free(rr);
}

int64_t orc_cf_info(const orc_cf *cf, const char *key)
{
    if (!strcmp(key, "lunkcf")) return cf->lunkcf;
    if (!strcmp(key, "iorbs")) return cf->iorbs;
    if (!strcmp(key, "ispin")) return cf->ispin;
    return -1;
}

int orc_cf_copy(const orc_cf *cf, int64_t nunk, const char *name, void *dst)
{
    if (!strcmp(name, "nnzcf_spa")) { memcpy(dst, cf->nnzcf, sizeof(int) * nunk); return 0; }
    if (!strcmp(name, "indcf_spa")) { memcpy(dst, cf->indcf, sizeof(int64_t) * nunk); return 0; }
    if (!strcmp(name, "irowcf_spa")) { memcpy(dst, cf->irowcf, sizeof(int) * cf->lunkcf); return 0; }
    if (!strcmp(name, "icolcf_spa")) { memcpy(dst, cf->icolcf, sizeof(int) * cf->lunkcf); return 0; }
    return -1;
}
