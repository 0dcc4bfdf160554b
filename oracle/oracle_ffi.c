/* Flat accessors used by the ctypes binding of the oracle.  TEST INFRASTRUCTURE ONLY. */
#include "oracle_internal.h"

int64_t orc_info(const orc_model *m, const char *k)
{
#define K(name, val) if (!strcmp(k, name)) return (int64_t)(val)
    K("norbs", m->norbs); K("nspin", m->nspin); K("nalf", m->nalf); K("nmats", m->nmats); K("ntier", m->ntier);
    K("ncor", m->ncor); K("nopr", m->nopr); K("nvar", m->nvar); K("nrho", m->nrho); K("nams", m->nams);
    K("nunk", m->nunk); K("ntable", m->ntable); K("lall", m->lall); K("lunk", m->lunk); K("lscreen", m->lscreen);
#undef K
    return -1;
}

int orc_copy(const orc_model *m, const char *k, void *dst)
{
    size_t nvar = m->nvar, nopr = m->nopr, nn = (size_t)m->nrho * m->nrho;
    size_t ncb = (size_t)m->norbs * m->nspin * m->ncor * m->nalf * 2;
    size_t nam = (size_t)m->nams * m->norbs * m->nspin;
#define C(name, ptr, bytes) if (!strcmp(k, name)) { memcpy(dst, ptr, bytes); return 0; }
    C("cb", m->cb, ncb * sizeof(ozc)); C("cd", m->cd, ncb * sizeof(ozc)); C("cgama", m->cgama, ncb * sizeof(ozc));
    C("cgamma", m->cgamma, nvar * sizeof(ozc)); C("dipm", m->dipm, nvar * sizeof(double));
    C("mpm", m->mpm, nvar * sizeof(int)); C("morbs", m->morbs, nvar * sizeof(int)); C("mspin", m->mspin, nvar * sizeof(int));
    C("ilead", m->ilead, nvar * sizeof(int)); C("mcor", m->mcor, nvar * sizeof(int)); C("mopr", m->mopr, nvar * sizeof(int));
    C("iredex", m->iredex, nvar * sizeof(int)); C("indexdraw", m->indexdraw, nvar * sizeof(int));
    C("jredex", m->jredex, nopr * sizeof(int)); C("jomit", m->jomit, nopr * sizeof(int));
    C("amsori", m->amsori, nn * m->norbs * m->nspin * sizeof(double));
    C("rowams", m->rowams, nam * sizeof(int)); C("colams", m->colams, nam * sizeof(int)); C("sgnams", m->sgnams, nam * sizeof(int));
    C("hs", m->hs, nn * sizeof(ozc));
    C("cpcoef", m->cpcoef, m->nmats * sizeof(double)); C("cppole", m->cppole, m->nmats * 2 * sizeof(ozc));
    C("ifirst", m->ifirst, m->ntier * sizeof(int64_t)); C("ilast", m->ilast, m->ntier * sizeof(int64_t));
    C("nfirst", m->nfirst, m->ntier * sizeof(int64_t)); C("nlast", m->nlast, m->ntier * sizeof(int64_t));
    C("indextable", m->indextable, m->ntable * sizeof(int));
    C("index_coef_ref", m->index_coef_ref, m->nunk * sizeof(int64_t));
    C("indexcoef", m->indexcoef, m->lall * sizeof(int64_t)); C("itypecoef", m->itypecoef, m->lall);
    C("ifactfcoef", m->ifactfcoef, m->lall); C("ifactrcoef", m->ifactrcoef, m->lall);
    C("nnz_spa", m->nnz_spa, m->nunk * sizeof(int)); C("ind_spa", m->ind_spa, m->nunk * sizeof(int64_t));
    C("irow_spa", m->irow_spa, m->lunk * sizeof(int)); C("icol_spa", m->icol_spa, m->lunk * sizeof(int));
    C("eleadinfty", m->eleadinfty, sizeof m->eleadinfty); C("zxip", m->zxip, sizeof m->zxip);
#undef C
    return -1;
}
