/*
 * oracle_apply.c -- the sparse-mode HEOM Liouvillian of HEOM-QUICK2, restated in
 * plain C with OpenMP over the ADOs of one tier.  TEST INFRASTRUCTURE ONLY.
 *
 * Every product of the reference is restricted to the stored COO pattern of the
 * output ADO, and the stored COO values of the input ADO are the only nonzeros
 * of its matrix (utility/zamsmm1_coo.f90, zamsmm2_coo.f90, zmat_zcoomm2.f90,
 * zmat_accu_coo2dns_pair.f90).  The restatement below accumulates the same
 * products entry by entry through a per-thread position map of the output
 * pattern, which is the same arithmetic in a different summation order.
 */
#include "oracle_internal.h"
#ifdef _OPENMP
#include <omp.h>
#endif

static inline ozc cb_of(const orc_model *m, int d)
{ return m->cb[orc_cbidx(m, m->morbs[d - 1], m->mspin[d - 1], m->mcor[d - 1], m->ilead[d - 1], m->mpm[d - 1])]; }
static inline ozc cd_of(const orc_model *m, int d)
{ return m->cd[orc_cbidx(m, m->morbs[d - 1], m->mspin[d - 1], m->mcor[d - 1], m->ilead[d - 1], m->mpm[d - 1])]; }

/* y_n += cl op(a) op(X_j) + cr op(X_j) op(a), restricted to the pattern of n (pos map) */
static void add_coupling(const orc_model *m, const int *pos, ozc *yn, const ozc *x, int64_t j, int itype,
                         int iorbs, int ispin, int dag_a, ozc cl, ozc cr)
{
    int n = m->nrho, nz = m->nnz_spa[j - 1];
    int64_t st = m->ind_spa[j - 1] - 1;
    for (int q = 0; q < nz; q++) {
        int br = m->irow_spa[st + q], bc = m->icol_spa[st + q];
        ozc v = x[st + q];
        if (itype) { int t = br; br = bc; bc = t; v = conj(v); }
        int sg, i = orc_left_row(m, iorbs, ispin, dag_a, br, &sg);
        if (i) { int p = pos[(i - 1) + (bc - 1) * n]; if (p >= 0) yn[p] += cl * (sg * v); }
        int jj = orc_right_col(m, iorbs, ispin, dag_a, bc, &sg);
        if (jj) { int p = pos[(br - 1) + (jj - 1) * n]; if (p >= 0) yn[p] += cr * (sg * v); }
    }
}

void orc_apply_shift(const orc_model *m, const double es[ORC_MAXALF][2], const ozc *x, ozc *y, int with_trace, int nthreads)
{
    int n = m->nrho;
    size_t nn = (size_t)n * n;
    for (int64_t k = 0; k < m->lunk; k++) y[k] = 0;
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

    /* ---- RDO row, tfqmr_double/calc_ax_tfqmr_spa_omp.f90:136-205 ---- */
    {
        ozc *x0 = calloc(nn, sizeof(ozc)), *c2 = calloc(nn, sizeof(ozc)), *s4 = calloc(nn, sizeof(ozc));
        int nz = m->nnz_spa[0];
        for (int q = 0; q < nz; q++) x0[(m->irow_spa[q] - 1) + (size_t)(m->icol_spa[q] - 1) * n] = x[q];
        /* -i (H x0 - x0 H), zmat_zcoomm('r') then ('l') */
        for (int q = 0; q < nz; q++) {
            int r = m->irow_spa[q] - 1, c = m->icol_spa[q] - 1;
            ozc hx = 0, xh = 0;
            for (int k = 0; k < n; k++) { hx += m->hs[r + (size_t)k * n] * x0[k + (size_t)c * n]; xh += x0[r + (size_t)k * n] * m->hs[k + (size_t)c * n]; }
            y[q] = -I * hx + I * xh;
        }
        /* C = sum_{s,m} (-i a S + i S a), S = sum_{alf,k} first-tier ADO (+,alf,m,s,k) */
        for (int ispin = 1; ispin <= m->nspin; ispin++) for (int io = 1; io <= m->norbs; io++) {
            for (size_t k = 0; k < nn; k++) s4[k] = 0;
            for (int ia = 1; ia <= m->nalf; ia++) {
                int isopr = (ispin - 1) * m->norbs + io, iopr = (isopr - 1) * m->nalf + ia;
                if (m->lscreen && m->jomit[iopr - 1] == 1) continue;
                for (int k = 1; k <= m->ncor; k++) {
                    int d = (iopr - 1) * m->ncor + k;
                    int64_t lni = m->nfirst[1] - 1 + m->indexdraw[d - 1];
                    int64_t st = m->ind_spa[lni - 1] - 1;
                    for (int q = 0; q < m->nnz_spa[lni - 1]; q++)
                        s4[(m->irow_spa[st + q] - 1) + (size_t)(m->icol_spa[st + q] - 1) * n] += x[st + q];
                }
            }
            size_t ob = orc_opbase(m, io, ispin);
            for (int e = 0; e < m->nams; e++) {
                int ra = m->rowams[ob + e] - 1, ca = m->colams[ob + e] - 1;
                double sg = m->sgnams[ob + e] ? -1.0 : 1.0;
                for (int j = 0; j < n; j++) c2[ra + (size_t)j * n] += -I * sg * s4[ca + (size_t)j * n];   /* a S */
                for (int i = 0; i < n; i++) c2[i + (size_t)ca * n] += I * sg * s4[i + (size_t)ra * n];    /* S a */
            }
        }
        for (int q = 0; q < nz; q++) {
            int r = m->irow_spa[q] - 1, c = m->icol_spa[q] - 1;
            y[q] += c2[r + (size_t)c * n] + conj(c2[c + (size_t)r * n]);
        }
        free(x0); free(c2); free(s4);
    }

    /* ---- tiers 2..ntier, calc_ax_tfqmr_spa_omp.f90:209-441 ---- */
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
                int nz = m->nnz_spa[lni - 1];
                if (nz == 0) continue;
                int64_t st = m->ind_spa[lni - 1] - 1;
                const int *ir = m->irow_spa + st, *ic = m->icol_spa + st;
                const ozc *xn = x + st; ozc *yn = y + st;
                for (int q = 0; q < nz; q++) pos[(ir[q] - 1) + (ic[q] - 1) * n] = q;
                const int *drw = m->indextable + m->ifirst[itier - 1] - 1 + (lni - m->nfirst[itier - 1]) * nb;
                ozc g = 0;
                for (int b = 0; b < nb; b++) {
                    int d = drw[b];
                    g += m->cgamma[d - 1] + I * m->dipm[d - 1] * es[m->ilead[d - 1] - 1][m->mspin[d - 1] - 1];
                }
                /* same tier: g x - i H x + i x H */
                for (int q = 0; q < nz; q++) {
                    int r = ir[q] - 1, c = ic[q] - 1; ozc v = xn[q];
                    yn[q] += g * v;
                    for (int k = hc_ptr[r]; k < hc_ptr[r + 1]; k++) {   /* H(i, r) v -> (i, c) */
                        int p = pos[hc_row[k] + (size_t)c * n]; if (p >= 0) yn[p] += -I * (hc_val[k] * v);
                    }
                    for (int k = hr_ptr[c]; k < hr_ptr[c + 1]; k++) {   /* v H(c, j) -> (r, j) */
                        int p = pos[r + (size_t)hr_col[k] * n]; if (p >= 0) yn[p] += I * (v * hr_val[k]);
                    }
                }
                int64_t lnl = m->index_coef_ref[lni - 1];
                /* lower tier */
                for (int b = 0; b < nb; b++) {
                    int d = drw[b];
                    int64_t j = m->indexcoef[lnl - 1]; int itype = m->itypecoef[lnl - 1];
                    double ff = m->ifactfcoef[lnl - 1], fr = m->ifactrcoef[lnl - 1];
                    lnl++;
                    ozc cl = cb_of(m, d) * (-I * ff), cr = cd_of(m, d) * (I * fr);
                    add_coupling(m, pos, yn, x, j, itype != 0, m->morbs[d - 1], m->mspin[d - 1], m->mpm[d - 1] == 1, cl, cr);
                }
                /* higher tier */
                if (itier < m->ntier) {
                    for (int isgn = 1; isgn <= 2; isgn++) for (int ispin = 1; ispin <= m->nspin; ispin++)
                    for (int io = 1; io <= m->norbs; io++) for (int ia = 1; ia <= m->nalf; ia++) {
                        int isopr = (isgn - 1) * m->nspin * m->norbs + (ispin - 1) * m->norbs + io;
                        int iopr = (isopr - 1) * m->nalf + ia;
                        if (m->lscreen && m->jomit[iopr - 1] == 1) continue;
                        for (int k = 1; k <= m->ncor; k++) {
                            int64_t j = m->indexcoef[lnl - 1]; int itype = m->itypecoef[lnl - 1];
                            double ff = m->ifactfcoef[lnl - 1], fr = m->ifactrcoef[lnl - 1];
                            lnl++;
                            if (m->nnz_spa[j - 1] == 0) continue;
                            add_coupling(m, pos, yn, x, j, itype != 0, io, ispin, isgn != 1, -I * ff, I * fr);
                        }
                    }
                }
                for (int q = 0; q < nz; q++) pos[(ir[q] - 1) + (ic[q] - 1) * n] = -1;
            }
            free(pos);
        }
    }
    if (with_trace) {
        ozc t = 0;
        for (int q = 0; q < m->nnz_spa[0]; q++) if (m->irow_spa[q] == m->icol_spa[q]) t += x[q];
        y[m->lunk] = t;
    }
    free(hc_ptr); free(hr_ptr); free(hc_row); free(hr_col); free(hc_val); free(hr_val);
}

void orc_calc_ax(const orc_model *m, const ozc *x, ozc *y, int nthreads)
{
    orc_apply_shift(m, m->eleadinfty, x, y, 1, nthreads);
}

void orc_calcderiv(const orc_model *m, double t, const ozc *x, ozc *y, int nthreads)
{
    double es[ORC_MAXALF][2];
    orc_eshift(m, t, es);
    orc_apply_shift(m, es, x, y, 0, nthreads);
}

/* td/calcj.f90:40-85 with utility/zams_trace_ab_spa.f90 ('n'): jt(ialf,ispin) */
void orc_current(const orc_model *m, const ozc *rho, double *jt)
{
    for (int a = 0; a < m->nalf * m->nspin; a++) jt[a] = 0;
    for (int ispin = 1; ispin <= m->nspin; ispin++) for (int io = 1; io <= m->norbs; io++)
    for (int ia = 1; ia <= m->nalf; ia++) {
        ozc c2 = 0;
        size_t ob = orc_opbase(m, io, ispin);
        for (int k = 1; k <= m->ncor; k++) {
            int isopr = (ispin - 1) * m->norbs + io, iopr = (isopr - 1) * m->nalf + ia;
            int d = (iopr - 1) * m->ncor + k;
            int64_t lni = m->nfirst[1] - 1 + m->indexdraw[d - 1];
            int64_t st = m->ind_spa[lni - 1] - 1; int nz = m->nnz_spa[lni - 1];
            ozc tr = 0;
            for (int e = 0; e < m->nams; e++) {
                int mi = m->rowams[ob + e], mk = m->colams[ob + e];
                for (int q = 0; q < nz; q++) {
                    if (m->irow_spa[st + q] != mk || m->icol_spa[st + q] != mi) continue;
                    tr += m->sgnams[ob + e] ? -rho[st + q] : rho[st + q];
                }
            }
            c2 += tr;
        }
        jt[(ia - 1) + (ispin - 1) * m->nalf] += -2.0 * cimag(c2);
    }
    for (int a = 0; a < m->nalf * m->nspin; a++) jt[a] *= ORC_JCONST;
}

/* main/calcocc.f90:32-60: occ(m,s) = Re tr(n_ms rho0) */
void orc_occupation(const orc_model *m, const ozc *rho, double *occ)
{
    int n = m->nrho;
    for (int ispin = 1; ispin <= m->nspin; ispin++) for (int io = 1; io <= m->norbs; io++) {
        size_t ob = orc_opbase(m, io, ispin);
        double s = 0;
        /* n = a^T a is diagonal: n(c,c) = 1 for every column c of a that holds an entry */
        for (int e = 0; e < m->nams; e++) {
            int c = m->colams[ob + e];
            for (int q = 0; q < m->nnz_spa[0]; q++)
                if (m->irow_spa[q] == c && m->icol_spa[q] == c) s += creal(rho[q]);
        }
        (void)n;
        occ[(io - 1) + (ispin - 1) * m->norbs] = s;
    }
}

/* main/analyze_hs.f90:144-176 (lbzman) + fermion/initialize1_spa.f90: Boltzmann RDO at the
 * temperature of lead 1, projected on the RDO pattern; all ADOs zero. */
void orc_initial_guess(const orc_model *m, ozc *rho)
{
    int n = m->nrho, n2 = 2 * n;
    double *a = calloc((size_t)n2 * n2, sizeof(double)), *v = calloc((size_t)n2 * n2, sizeof(double)), *w = calloc(n2, sizeof(double));
    for (int j = 0; j < n; j++) for (int i = 0; i < n; i++) {
        ozc h = m->hs[i + (size_t)j * n];
        a[i + (size_t)j * n2] = creal(h); a[(i + n) + (size_t)(j + n) * n2] = creal(h);
        a[(i + n) + (size_t)j * n2] = cimag(h); a[i + (size_t)(j + n) * n2] = -cimag(h);
    }
    orc_symeig(n2, a, w, v);
    double emin = w[0], tlead = m->temperature[0];
    ozc *r = calloc((size_t)n * n, sizeof(ozc));
    double tr = 0;
    for (int k = 0; k < n2; k++) {
        double f = exp(-(w[k] - emin) * ORC_HBAR / tlead);
        for (int j = 0; j < n; j++) for (int i = 0; i < n; i++) {
            double re = f * v[i + (size_t)k * n2] * v[j + (size_t)k * n2];
            double im = f * v[(i + n) + (size_t)k * n2] * v[j + (size_t)k * n2];
            r[i + (size_t)j * n] += re + I * im;
        }
    }
    for (int i = 0; i < n; i++) tr += creal(r[i + (size_t)i * n]);
    for (int64_t k = 0; k < m->lunk; k++) rho[k] = 0;
    for (int q = 0; q < m->nnz_spa[0]; q++) rho[q] = r[(m->irow_spa[q] - 1) + (size_t)(m->icol_spa[q] - 1) * n] / tr;
    free(a); free(v); free(w); free(r);
}
