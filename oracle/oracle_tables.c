/*
 * oracle_tables.c -- ADO enumeration, coupling tables and per-ADO sparsity of
 * HEOM-QUICK2, restated in plain C.  TEST INFRASTRUCTURE ONLY (see heom_oracle.h).
 */
#include "oracle_internal.h"

/* main/findoprindex.f90 + compareoprindex: binary search of a record (or of its
 * complement) among nrec records of length lrec starting at table[start]. */
static int64_t orc_find_record(const int *table, int64_t start, int64_t nrec, int lrec, const int *rec,
                               const int *redex, int complement, int *fact)
{
    int work[ORC_MAXTIER];
    *fact = 1;
    if (!complement) for (int i = 0; i < lrec; i++) work[i] = rec[i];
    else {
        for (int i = 0; i < lrec; i++) work[i] = redex[rec[lrec - 1 - i] - 1];
        for (int i = 0; i < lrec - 1; i++) for (int j = i + 1; j < lrec; j++)
            if (work[i] > work[j]) { int t = work[i]; work[i] = work[j]; work[j] = t; *fact = -*fact; }
    }
    int64_t low = 1, high = nrec, mid = (high + low) / 2;
    if (high < low) return -1;
    while (low <= high) {
        const int *r = table + start + (mid - 1) * lrec;
        int igel = 0;
        for (int i = 0; i < lrec; i++) { if (r[i] > work[i]) { igel = 1; break; } if (r[i] < work[i]) { igel = -1; break; } }
        if (low == high && igel != 0) return -1;
        if (igel > 0) high = mid - 1 > 1 ? mid - 1 : 1;
        else if (igel < 0) low = mid + 1 < nrec ? mid + 1 : nrec;
        else return mid;             /* 1-based record number */
        mid = (high + low) / 2;
    }
    return -1;
}

static const orc_model *g_sort_model;
static int g_sort_len;
static int cmp_rows(const void *a, const void *b)
{
    const int *x = a, *y = b;
    for (int i = 0; i < g_sort_len; i++) { if (x[i] < y[i]) return -1; if (x[i] > y[i]) return 1; }
    return 0;
}

/* main/ball2drawer.f90:26-257 (lsdraw = T, no lomit/lfilter/lad), fermion/sortindextable3.f90
 * (rows are unique, so any correct lexicographic sort gives the reference order),
 * main/examindextable.f90 and main/clearindextable.f90 (no rows removed without lsimple). */
static int orc_ball2drawer(orc_model *m)
{
    int nopr = m->nopr, ncor = m->ncor;
    /* upper bound on the table size: sum over tiers of C(nopr+n-1, n) * ncor^n * n */
    int64_t cap = 1, cap_ops = 1;
    for (int it = 2; it <= m->ntier; it++) {
        int nb = it - 1; double c = 1; for (int k = 1; k <= nb; k++) c = c * (nopr + k - 1) / k;
        double pw = 1; for (int k = 0; k < nb; k++) pw *= ncor;
        cap += (int64_t)(c * pw * nb + 0.5); cap_ops += (int64_t)(c * nb + 0.5);
    }
    m->indextable = calloc(cap + 1, sizeof(int));
    int *oprtable = calloc(cap_ops + 1, sizeof(int));
    m->ifirst[0] = m->ilast[0] = m->nfirst[0] = m->nlast[0] = 1;
    m->indextable[0] = 0;
    int64_t ioprlast_prev = 1;
    for (int itier = 2; itier <= m->ntier; itier++) {
        int nb = itier - 1;
        m->ifirst[itier - 1] = m->ilast[itier - 2] + 1;
        m->nfirst[itier - 1] = m->nlast[itier - 2] + 1;
        int64_t iopr_first = ioprlast_prev + 1;   /* 1-based position in oprtable */
        int64_t ni = iopr_first, nrec = 0;
        int ipoint[ORC_MAXTIER];
        for (int k = 0; k < nb - 1; k++) ipoint[k] = 1;
        ipoint[nb - 1] = 0;
        for (;;) {
            int nj = nb - 1;
            for (;;) {
                ipoint[nj]++;
                if (ipoint[nj] <= nopr) break;
                nj--;
                if (nj < 0) goto ops_done;
            }
            for (int k = nj + 1; k < nb; k++) ipoint[k] = ipoint[nj];
            if (m->lscreen) {
                int skip = 0;
                for (int k = 0; k < nb; k++) if (m->jomit[ipoint[k] - 1] == 1) skip = 1;
                if (skip) continue;
            }
            int found = -1, fact;
            if (nrec > 0) found = (int)orc_find_record(oprtable, iopr_first - 1, nrec, nb, ipoint, m->jredex, 1, &fact);
            if (found < 0) {
                for (int k = 0; k < nb; k++) oprtable[ni - 1 + k] = ipoint[k];
                ni += nb; nrec++;
            }
        }
    ops_done:
        ioprlast_prev = iopr_first - 1 + nrec * nb;
        /* memory-component lists (lexicographic over ncor^nb) */
        int64_t nlist = 1; for (int k = 0; k < nb; k++) nlist *= ncor;
        int64_t pos = m->ifirst[itier - 1], cnt = 0;
        for (int64_t r = 0; r < nrec; r++) {
            const int *ops = oprtable + iopr_first - 1 + r * nb;
            int cor[ORC_MAXTIER];
            for (int k = 0; k < nb; k++) cor[k] = 1;
            for (int64_t il = 0; il < nlist; il++) {
                if (il > 0) {   /* odometer, last position fastest */
                    int k = nb - 1;
                    while (1) { cor[k]++; if (cor[k] <= ncor) break; cor[k] = 1; k--; }
                }
                int rec = 1;
                for (int a = 0; a < nb - 1 && rec; a++) for (int b = a + 1; b < nb; b++)
                    if (ops[a] == ops[b] && cor[a] > cor[b]) { rec = 0; break; }
                if (!rec) continue;
                for (int k = 0; k < nb; k++) m->indextable[pos - 1 + k] = (ops[k] - 1) * ncor + cor[k];
                pos += nb; cnt++;
            }
        }
        m->nlast[itier - 1] = m->nlast[itier - 2] + cnt;
        m->ilast[itier - 1] = m->ilast[itier - 2] + cnt * nb;
        /* sort rows of this tier */
        g_sort_model = m; g_sort_len = nb;
        qsort(m->indextable + m->ifirst[itier - 1] - 1, (size_t)cnt, sizeof(int) * nb, cmp_rows);
        /* examindextable: rows must be non-decreasing */
        for (int64_t r = 0; r < cnt; r++) {
            const int *row = m->indextable + m->ifirst[itier - 1] - 1 + r * nb;
            for (int k = 0; k < nb - 1; k++) if (row[k + 1] < row[k]) { orc_set_error("indextable row not sorted"); free(oprtable); return -1; }
        }
    }
    m->nunk = m->nlast[m->ntier - 1];
    m->ntable = m->ilast[m->ntier - 1];
    free(oprtable);
    return 0;
}

/* main/findindex.f90 on the drawer table of one tier; returns the 1-based ADO index or -1 */
static int64_t orc_findindex(const orc_model *m, int tier, int lrec, const int *rec, int complement, int *fact)
{
    int64_t nrec = m->nlast[tier - 1] - m->nfirst[tier - 1] + 1;
    int64_t r = orc_find_record(m->indextable, m->ifirst[tier - 1] - 1, nrec, lrec, rec, m->iredex, complement, fact);
    if (r < 0) return -1;
    return m->nfirst[tier - 1] + r - 1;
}

/* main/buildcoefindex.f90:192-362 with main/findlowertier.f90 and main/findhighertier.f90 */
static int orc_buildcoefindex(orc_model *m)
{
    int64_t cap = 0;
    for (int it = 2; it <= m->ntier; it++)
        cap += (m->nlast[it - 1] - m->nfirst[it - 1] + 1) * ((it - 1) + (it < m->ntier ? m->nvar : 0));
    m->index_coef_ref = calloc(m->nunk + 1, sizeof(int64_t));
    m->indexcoef = calloc(cap + 1, sizeof(int64_t));
    m->itypecoef = calloc(cap + 1, 1); m->ifactfcoef = calloc(cap + 1, 1); m->ifactrcoef = calloc(cap + 1, 1);
    int64_t lnl = 1, lall = 0;
#define PUSH(lnk, iout, ff, fr) do { m->indexcoef[lall] = (lnk); m->itypecoef[lall] = (int8_t)(iout); \
        m->ifactfcoef[lall] = (int8_t)(ff); m->ifactrcoef[lall] = (int8_t)(fr); lall++; lnl++; } while (0)
    for (int itier = 2; itier <= m->ntier; itier++) {
        int nb = itier - 1;
        for (int64_t lni = m->nfirst[itier - 1]; lni <= m->nlast[itier - 1]; lni++) {
            m->index_coef_ref[lni - 1] = lnl;
            const int *nk = m->indextable + m->ifirst[itier - 1] - 1 + (lni - m->nfirst[itier - 1]) * nb;
            /* nearest lower tier */
            for (int ni = 1; ni <= nb; ni++) {
                int64_t lnk; int iout, fact = 1;
                if (itier == 2) { lnk = 1; iout = 0; }
                else {
                    int rec[ORC_MAXTIER], c = 0;
                    for (int k = 1; k <= nb; k++) if (k != ni) rec[c++] = nk[k - 1];
                    lnk = orc_findindex(m, itier - 1, nb - 1, rec, 0, &fact);
                    iout = 0;
                    if (lnk < 0) { lnk = orc_findindex(m, itier - 1, nb - 1, rec, 1, &fact); iout = 1; }
                    if (lnk < 0) { orc_set_error("findlowertier: not found"); return -1; }
                }
                int ff = (ni % 2 == 0) ? -1 : 1;
                int fr = ((itier - 1 - ni) % 2 == 0) ? 1 : -1;
                if (iout == 1) { ff *= fact; fr *= fact; }
                PUSH(lnk, iout, ff, fr);
            }
            /* nearest higher tier */
            if (itier < m->ntier) {
                for (int isgn = 1; isgn <= 2; isgn++) for (int ispin = 1; ispin <= m->nspin; ispin++)
                for (int io = 1; io <= m->norbs; io++) for (int ia = 1; ia <= m->nalf; ia++) {
                    int isopr = (isgn - 1) * m->nspin * m->norbs + (ispin - 1) * m->norbs + io;
                    int iopr = (isopr - 1) * m->nalf + ia;
                    if (m->lscreen && m->jomit[iopr - 1] == 1) continue;
                    for (int imats = 1; imats <= m->ncor; imats++) {
                        int nplus = (iopr - 1) * m->ncor + imats;
                        int mi[ORC_MAXTIER], ffact = 1, rfact = 1;
                        /* front: [nplus, nk...] exchange-sorted */
                        mi[0] = nplus; for (int k = 0; k < nb; k++) mi[k + 1] = nk[k];
                        for (int a = 0; a < itier - 1; a++) for (int b = a + 1; b < itier; b++)
                            if (mi[a] > mi[b]) { int t = mi[a]; mi[a] = mi[b]; mi[b] = t; ffact = -ffact; }
                        /* rear: [nk..., nplus] exchange-sorted */
                        for (int k = 0; k < nb; k++) mi[k] = nk[k];
                        mi[nb] = nplus;
                        for (int a = 0; a < itier - 1; a++) for (int b = a + 1; b < itier; b++)
                            if (mi[a] > mi[b]) { int t = mi[a]; mi[a] = mi[b]; mi[b] = t; rfact = -rfact; }
                        int fact = 1, iout = 0;
                        int64_t lnk = orc_findindex(m, itier + 1, itier, mi, 0, &fact);
                        if (lnk < 0) { lnk = orc_findindex(m, itier + 1, itier, mi, 1, &fact); iout = 1; }
                        if (lnk < 0) { orc_set_error("findhighertier: not found"); return -1; }
                        PUSH(lnk, iout, ffact * fact, rfact * fact);
                    }
                }
            }
        }
    }
#undef PUSH
    m->lall = lall;
    return 0;
}

int orc_build_tables(orc_model *m)
{
    if (orc_ball2drawer(m)) return -1;
    return orc_buildcoefindex(m);
}

/* ---------------- sparsity (fermion/prelude_spa.f90:146-747) ---------------- */

static unsigned long long g_rng;
void orc_rng_seed(unsigned long long seed) { g_rng = seed * 2654435761ULL + 88172645463325252ULL; }
static double orc_uniform(void)
{
    g_rng ^= g_rng << 13; g_rng ^= g_rng >> 7; g_rng ^= g_rng << 17;
    return ((g_rng >> 11) + 0.5) * (1.0 / 9007199254740992.0);
}
double orc_normal(void)
{
    double u1 = orc_uniform(), u2 = orc_uniform();
    return sqrt(-2.0 * log(u1)) * cos(2.0 * ORC_PI * u2);
}

/* utility/calc_exp_hmat.f90: 1 + sum_{k<=kmax} (alpha H)^k / k! */
void orc_exp_taylor(int n, const ozc *h, double alpha, int kmax, ozc *out)
{
    size_t nn = (size_t)n * n;
    ozc *c1 = calloc(nn, sizeof(ozc)), *c2 = calloc(nn, sizeof(ozc));
    for (size_t k = 0; k < nn; k++) out[k] = 0;
    for (int i = 0; i < n; i++) out[i + (size_t)i * n] = 1.0, c1[i + (size_t)i * n] = 1.0;
    double f = 1.0;
    for (int k = 1; k <= kmax; k++) {
        f /= k;
        for (int j = 0; j < n; j++) for (int i = 0; i < n; i++) {
            ozc s = 0; for (int q = 0; q < n; q++) s += c1[i + (size_t)q * n] * h[q + (size_t)j * n];
            c2[i + (size_t)j * n] = alpha * s;
        }
        for (size_t q = 0; q < nn; q++) { out[q] += f * c2[q]; c1[q] = c2[q]; }
    }
    free(c1); free(c2);
}

/* zamsmm_coo semantics (utility/zamsmm_coo.f90): op(a) op(B) (left) or op(B) op(a) (right)
 * for B in COO; the result of a partial permutation times a COO matrix is returned
 * as a COO list (no duplicates can arise). */
int orc_ams_coo(const orc_model *m, int left, int dag_a, int dag_b, int iorbs, int ispin,
                int nnz, const int *ir, const int *ic, const ozc *v, int *orow, int *ocol, ozc *oval)
{
    int cnt = 0;
    for (int q = 0; q < nnz; q++) {
        int br = dag_b ? ic[q] : ir[q], bc = dag_b ? ir[q] : ic[q];
        ozc bv = dag_b ? conj(v[q]) : v[q];
        int sg;
        if (left) { int i = orc_left_row(m, iorbs, ispin, dag_a, br, &sg); if (i) { orow[cnt] = i; ocol[cnt] = bc; oval[cnt] = sg * bv; cnt++; } }
        else { int j = orc_right_col(m, iorbs, ispin, dag_a, bc, &sg); if (j) { orow[cnt] = br; ocol[cnt] = j; oval[cnt] = sg * bv; cnt++; } }
    }
    return cnt;
}

int orc_build_pattern(orc_model *m, unsigned long long seed)
{
    int n = m->nrho; size_t nn = (size_t)n * n;
    orc_rng_seed(seed);
    ozc *e10 = calloc(nn, sizeof(ozc)), *e11 = calloc(nn, sizeof(ozc));
    orc_exp_taylor(n, m->hs, 0.31415926, 10, e10);
    orc_exp_taylor(n, m->hs, 0.31415926, 11, e11);
    for (size_t k = 0; k < nn; k++) {
        int a = cabs(e10[k]) >= ORC_DSMALL, b = cabs(e11[k]) >= ORC_DSMALL;   /* checksparsity */
        if (a != b) { orc_set_error("prelude_spa: exp(H) sparsity differs between orders 10 and 11"); free(e10); free(e11); return -1; }
    }
    /* worst case storage nunk * nrho^2 is too large for the bigger models: grow dynamically */
    int64_t cap = (int64_t)nn * 64;
    m->nnz_spa = calloc(m->nunk, sizeof(int)); m->ind_spa = calloc(m->nunk, sizeof(int64_t));
    int *ir = malloc(sizeof(int) * cap), *ic = malloc(sizeof(int) * cap);
    ozc *val = malloc(sizeof(ozc) * cap);
    int64_t lunk = 0;
    /* RDO */
    for (int j = 1; j <= n; j++) for (int i = 1; i <= n; i++) {
        ozc v = e10[(i - 1) + (size_t)(j - 1) * n];
        if (cabs(v) > ORC_DSMALL) { ir[lunk] = i; ic[lunk] = j; val[lunk] = v; lunk++; }
    }
    m->nnz_spa[0] = (int)lunk; m->ind_spa[0] = 1;
    int e0n = (int)lunk;
    int *e0r = malloc(sizeof(int) * e0n), *e0c = malloc(sizeof(int) * e0n); ozc *e0v = malloc(sizeof(ozc) * e0n);
    memcpy(e0r, ir, sizeof(int) * e0n); memcpy(e0c, ic, sizeof(int) * e0n); memcpy(e0v, val, sizeof(ozc) * e0n);
    /* E0 by columns (its COO is column-major) */
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
                int64_t st = m->ind_spa[lnj - 1] - 1; int nz = m->nnz_spa[lnj - 1];
                ozc c1, c2;
                do { c1 = orc_normal() + I * orc_normal(); c2 = orc_normal() + I * orc_normal(); }
                while (!(cabs(c1) > 1e-6 && cabs(c2) > 1e-6));
                for (int side = 0; side < 2; side++) {
                    /* side 0: E0 (op(a) op(B)); side 1: E0 (op(B) op(a)); mkl_zcoomm with E0 in COO */
                    int cnt = orc_ams_coo(m, side == 0, isgn == 1, itype != 0, io, is, nz, ir + st, ic + st, val + st, tr, tc, tv);
                    ozc cm = side == 0 ? c1 : c2;
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
            m->nnz_spa[lni - 1] = na;
            m->ind_spa[lni - 1] = m->ind_spa[lni - 2] + m->nnz_spa[lni - 2];
        }
    }
    m->lunk = lunk;
    m->irow_spa = realloc(ir, sizeof(int) * (lunk > 0 ? lunk : 1));
    m->icol_spa = realloc(ic, sizeof(int) * (lunk > 0 ? lunk : 1));
    free(val); free(e0r); free(e0c); free(e0v); free(e0cp); free(acc); free(tr); free(tc); free(tv); free(e10); free(e11);
    return 0;
}
