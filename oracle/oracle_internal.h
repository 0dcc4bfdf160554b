/* Internal helpers shared by the oracle's translation units. TEST INFRASTRUCTURE ONLY. */
#ifndef HEOM_ORACLE_INTERNAL_H
#define HEOM_ORACLE_INTERNAL_H
#include "heom_oracle.h"
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

void orc_set_error(const char *msg);
int orc_build_tables(orc_model *m);
int orc_build_pattern(orc_model *m, unsigned long long seed);
void orc_symeig(int n, double *a, double *w, double *v);
size_t orc_cbidx(const orc_model *m, int iorbs, int ispin, int icor, int ialf, int isgn);
/* shared by the steady and correlation-function pattern builders */
void orc_rng_seed(unsigned long long seed);
double orc_normal(void);
void orc_exp_taylor(int n, const ozc *h, double alpha, int kmax, ozc *out);
int orc_ams_coo(const orc_model *m, int left, int dag_a, int dag_b, int iorbs, int ispin,
                int nnz, const int *ir, const int *ic, const ozc *v, int *orow, int *ocol, ozc *oval);

/* operator entry k (0-based) of a_{iorbs,ispin} */
static inline size_t orc_opbase(const orc_model *m, int iorbs, int ispin)
{ return (size_t)m->nams * (((size_t)iorbs - 1) + ((size_t)ispin - 1) * m->norbs); }

/* op(a) element lookups.  For op = a (dag=0) or a^dagger (dag=1):
 *   left product  (op(a) B)(i, c): source row r maps to output row i = orc_left_row(r)
 *   right product (B op(a))(r, j): source col c maps to output col j = orc_right_col(c)
 * Return 0 when the source row/col is annihilated. */
static inline int orc_left_row(const orc_model *m, int iorbs, int ispin, int dag, int r, int *sg)
{
    size_t mb = (size_t)(m->nrho + 1) * (((size_t)iorbs - 1) + ((size_t)ispin - 1) * m->norbs);
    if (!dag) { *sg = m->op_srofc[mb + r]; return m->op_rofc[mb + r]; }
    *sg = m->op_scofr[mb + r]; return m->op_cofr[mb + r];
}
static inline int orc_right_col(const orc_model *m, int iorbs, int ispin, int dag, int c, int *sg)
{
    size_t mb = (size_t)(m->nrho + 1) * (((size_t)iorbs - 1) + ((size_t)ispin - 1) * m->norbs);
    if (!dag) { *sg = m->op_scofr[mb + c]; return m->op_cofr[mb + c]; }
    *sg = m->op_srofc[mb + c]; return m->op_rofc[mb + c];
}

#endif
