// Host construction of the device plan from the reference's tables.
//
// Semantics (tfqmr_double/calc_ax_tfqmr_spa_omp.f90:136-441, td/calcderiv_spa_omp.f90):
// for an ADO n with stored pattern P_n and a source ADO j coupled to it,
//     y_n += P_n( cL op(a) op_b(X_j) + cR op_b(X_j) op(a) )
// where op(a) is a_{ms} or its adjoint (a signed partial permutation), op_b is the
// identity or the conjugate transpose (itypecoef = 1), and X_j holds only the stored
// entries of j.  Each (class of n, class of j, operator, op_b) therefore defines a
// fixed gather map: for every output entry, at most one source entry through the
// left product and one through the right product, each with a sign.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <unordered_map>

#include "plan.h"

namespace heom {

namespace {

struct ClassInfo {
    int nnz = 0;
    std::vector<int32_t> rows, cols;   // 0-based
    std::vector<int32_t> pos;          // dense n*n -> local index or -1
};

// unit pair (i sL, i sR) with sL, sR = +-1 -> its code, else -1
int32_t unit_code(cd l, cd r)
{
    if (l.real() == 0.0 && r.real() == 0.0 && std::fabs(l.imag()) == 1.0 && std::fabs(r.imag()) == 1.0)
        return kCoefUnit | (l.imag() < 0 ? 1 : 0) | (r.imag() < 0 ? 2 : 0);
    return -1;
}
void decode_coef(const HostPlan &P, int32_t cid, cd &l, cd &r)
{
    if (cid & kCoefUnit) { l = cd(0, (cid & 1) ? -1.0 : 1.0); r = cd(0, (cid & 2) ? -1.0 : 1.0); }
    else { l = P.cl[cid & 0x3FFFFFFF]; r = P.cr[cid & 0x3FFFFFFF]; }
}

struct MapKey {
    int cout, cin, o, s, dag, tr;
    bool operator<(const MapKey &k) const {
        return std::tie(cout, cin, o, s, dag, tr) < std::tie(k.cout, k.cin, k.o, k.s, k.dag, k.tr);
    }
};

// Plan-building state shared by the forward construction.
struct Builder {
    const heom_tables &t;
    int n = 0;
    std::vector<int32_t> cls_of;             // per ADO (0-based), -1 for empty ADOs
    std::vector<ClassInfo> classes;
    std::vector<int32_t> rofc, cofr, srofc, scofr;   // per operator, (n+1) entries, 1-based rows/cols
    std::map<MapKey, int32_t> map_ids;       // -> map base or -2 if the map is empty
    std::map<std::pair<std::pair<double, double>, std::pair<double, double>>, int32_t> coef_ids;

    explicit Builder(const heom_tables &tt) : t(tt), n(tt.nrho) {}

    int opidx(int o, int s) const { return (o - 1) + (s - 1) * t.norbs; }

    void make_operator_maps() {
        int nop = t.norbs * t.nspin;
        rofc.assign((size_t)nop * (n + 1), 0); cofr = rofc; srofc = rofc; scofr = rofc;
        for (int s = 1; s <= t.nspin; s++)
            for (int o = 1; o <= t.norbs; o++) {
                size_t base = (size_t)t.nams * opidx(o, s), mb = (size_t)(n + 1) * opidx(o, s);
                for (int k = 0; k < t.nams; k++) {
                    int r = t.rowams[base + k], c = t.colams[base + k], sg = t.sgnams[base + k] ? -1 : 1;
                    if (r < 1 || r > n || c < 1 || c > n) fail(HEOM_E_ARG, "operator index out of range");
                    if (rofc[mb + c] || cofr[mb + r]) fail(HEOM_E_ARG, "a_{ms} is not a signed partial permutation");
                    rofc[mb + c] = r; srofc[mb + c] = sg; cofr[mb + r] = c; scofr[mb + r] = sg;
                }
            }
    }

    void make_classes() {
        std::map<std::vector<int32_t>, int32_t> intern;
        cls_of.assign(t.nunk, -1);
        for (int64_t u = 0; u < t.nunk; u++) {
            int nz = t.nnz_spa[u];
            if (nz < 0 || nz > n * n) fail(HEOM_E_ARG, "nnz_spa out of range");
            if (nz == 0) continue;
            int64_t st = t.ind_spa[u] - 1;
            if (st < 0 || st + nz > t.lunk_spa) fail(HEOM_E_ARG, "ind_spa out of range");
            std::vector<int32_t> key(2 * (size_t)nz);
            for (int q = 0; q < nz; q++) {
                key[2 * q] = t.irow_spa[st + q]; key[2 * q + 1] = t.icol_spa[st + q];
                if (key[2 * q] < 1 || key[2 * q] > n || key[2 * q + 1] < 1 || key[2 * q + 1] > n)
                    fail(HEOM_E_ARG, "irow_spa/icol_spa out of range");
            }
            auto it = intern.find(key);
            if (it == intern.end()) {
                ClassInfo ci;
                ci.nnz = nz;
                ci.pos.assign((size_t)n * n, -1);
                for (int q = 0; q < nz; q++) {
                    ci.rows.push_back(key[2 * q] - 1); ci.cols.push_back(key[2 * q + 1] - 1);
                    ci.pos[(size_t)(key[2 * q] - 1) + (size_t)(key[2 * q + 1] - 1) * n] = q;
                }
                int32_t id = (int32_t)classes.size();
                classes.push_back(std::move(ci));
                it = intern.emplace(std::move(key), id).first;
            }
            cls_of[u] = it->second;
        }
    }

    // source row index for the left product op(a)(i, k): returns k (1-based) or 0
    int left_src(int o, int s, bool dag, int i1, int &sg) const {
        size_t mb = (size_t)(n + 1) * opidx(o, s);
        if (!dag) { sg = scofr[mb + i1]; return cofr[mb + i1]; }   // a(i,k) != 0 -> k = col of row i
        sg = srofc[mb + i1]; return rofc[mb + i1];                  // a+(i,k) = a(k,i) -> k = row of col i
    }
    // source col index for the right product op(a)(k, c): returns k (1-based) or 0
    int right_src(int o, int s, bool dag, int c1, int &sg) const {
        size_t mb = (size_t)(n + 1) * opidx(o, s);
        if (!dag) { sg = srofc[mb + c1]; return rofc[mb + c1]; }   // a(k,c) -> k = row of col c
        sg = scofr[mb + c1]; return cofr[mb + c1];                  // a+(k,c) = a(c,k) -> k = col of row c
    }

    int32_t get_map(HostPlan &P, int cout, int cin, int o, int s, bool dag, bool tr) {
        MapKey key{cout, cin, o, s, dag ? 1 : 0, tr ? 1 : 0};
        auto it = map_ids.find(key);
        if (it != map_ids.end()) return it->second;
        const ClassInfo &co = classes[cout], &ci = classes[cin];
        std::vector<uint32_t> words(co.nnz, 0);
        bool any = false;
        double hits = 0;
        for (int p = 0; p < co.nnz; p++) {
            int i = co.rows[p], c = co.cols[p];
            uint32_t w = 0;
            int sg;
            int k = left_src(o, s, dag, i + 1, sg);          // op(a)(i,k) op_b(X)(k,c)
            if (k) {
                int q = tr ? ci.pos[(size_t)c + (size_t)(k - 1) * n] : ci.pos[(size_t)(k - 1) + (size_t)c * n];
                if (q >= 0) { w |= (uint32_t)(q + 1) | (sg < 0 ? 0x8000u : 0u); hits++; }
            }
            k = right_src(o, s, dag, c + 1, sg);             // op_b(X)(i,k) op(a)(k,c)
            if (k) {
                int q = tr ? ci.pos[(size_t)(k - 1) + (size_t)i * n] : ci.pos[(size_t)i + (size_t)(k - 1) * n];
                if (q >= 0) { w |= ((uint32_t)(q + 1) | (sg < 0 ? 0x8000u : 0u)) << 16; hits++; }
            }
            words[p] = w;
            any = any || w;
        }
        int32_t id = -2;
        if (any) {
            id = (int32_t)P.maps.size();
            P.maps.insert(P.maps.end(), words.begin(), words.end());
            P.n_maps++;
        }
        map_ids.emplace(key, id);
        return id;
    }

    int32_t get_coef(HostPlan &P, cd l, cd r, int8_t kind) {
        int32_t u = unit_code(l, r);
        if (u >= 0) return u;
        auto key = std::make_pair(std::make_pair(l.real(), l.imag()), std::make_pair(r.real(), r.imag()));
        auto it = coef_ids.find(key);
        if (it != coef_ids.end()) return it->second;
        int32_t id = (int32_t)P.cl.size();
        P.cl.push_back(l); P.cr.push_back(r); P.coef_kind.push_back(kind);
        coef_ids.emplace(key, id);
        return id;
    }
};

}  // namespace

HStructure make_hstructure(const heom_tables &t, const std::vector<const double _Complex *> &extra) {
    HStructure h;
    h.n = t.nrho;
    int n = h.n;
    h.idx.assign((size_t)n * n, -1);
    const cd *hs = reinterpret_cast<const cd *>(t.hs);
    for (int j = 0; j < n; j++)
        for (int i = 0; i < n; i++) {
            bool nz = i == j || std::abs(hs[(size_t)i + (size_t)j * n]) >= kDsmall;
            for (auto *e : extra)
                if (e && std::abs(reinterpret_cast<const cd *>(e)[(size_t)i + (size_t)j * n]) >= kDsmall) nz = true;
            if (nz) {
                h.idx[(size_t)i + (size_t)j * n] = (int32_t)h.rows.size();
                h.rows.push_back(i); h.cols.push_back(j);
            }
        }
    if (h.rows.size() >= (1u << 15)) fail(HEOM_E_UNSUPPORTED, "Hamiltonian structure too large");
    return h;
}

void build_forward_plan(const heom_tables &t, const HStructure &hst, HostPlan &P) {
    if (t.norbs < 1 || t.nspin < 1 || t.nalf < 1 || t.nalf * t.nspin > 4 || t.ncor < 1 || t.ntier < 2)
        fail(HEOM_E_ARG, "table sizes out of range");
    if (t.nrho > 64) fail(HEOM_E_UNSUPPORTED, "nrho > 64 is not supported");
    if (t.lunk_spa >= (int64_t)1 << 31) fail(HEOM_E_UNSUPPORTED, "more than 2^31 stored entries");
    Builder B(t);
    const int n = t.nrho;
    B.make_operator_maps();
    B.make_classes();
    P = HostPlan();
    P.lunk = t.lunk_spa;
    P.nslots = t.nalf * t.nspin;
    P.nh = (int32_t)hst.rows.size();
    P.n_classes = (int64_t)B.classes.size();
    const int nvar = 2 * t.norbs * t.nspin * t.nalf * t.ncor;
    const cd *cb = reinterpret_cast<const cd *>(t.cb), *cdv = reinterpret_cast<const cd *>(t.cd);
    const cd *cgamma = reinterpret_cast<const cd *>(t.cgamma);
    auto cbidx = [&](int d) {
        int o = t.morbs[d - 1], s = t.mspin[d - 1], k = t.mcor[d - 1], a = t.ilead[d - 1], sg = t.mpm[d - 1];
        return ((((size_t)(sg - 1) * t.nalf + (a - 1)) * t.ncor + (k - 1)) * t.nspin + (s - 1)) * t.norbs + (o - 1);
    };
    // same-tier terms of every class
    for (auto &ci : B.classes) {
        P.cls_tptr.push_back((int32_t)P.term_ptr.size());
        for (int p = 0; p < ci.nnz; p++) {
            P.term_ptr.push_back((int32_t)P.terms.size());
            int i = ci.rows[p], c = ci.cols[p];
            for (int k = 0; k < n; k++) {          // -i H(i,k) X(k,c)
                int h = hst.idx[(size_t)i + (size_t)k * n], q = ci.pos[(size_t)k + (size_t)c * n];
                if (h >= 0 && q >= 0) P.terms.push_back((uint32_t)q | ((uint32_t)h << 16));
            }
            for (int k = 0; k < n; k++) {          // +i X(i,k) H(k,c)
                int h = hst.idx[(size_t)k + (size_t)c * n], q = ci.pos[(size_t)i + (size_t)k * n];
                if (h >= 0 && q >= 0) P.terms.push_back((uint32_t)q | ((uint32_t)h << 16) | 0x80000000u);
            }
        }
        P.term_ptr.push_back((int32_t)P.terms.size());
    }
    P.n_terms_same = 0;
    // ADOs with entries, in table order
    std::vector<int64_t> ados;
    for (int64_t u = 0; u < t.nunk; u++)
        if (t.nnz_spa[u] > 0) ados.push_back(u + 1);
    P.nado = (int32_t)ados.size();
    P.ent_ado.assign(P.lunk, -1);
    P.ado_off.resize(P.nado + 1);
    P.coup_ptr.push_back(0);
    auto tier_of = [&](int64_t u) {
        int it = 1;
        while (it < t.ntier && u > t.nlast[it - 1]) it++;
        return it;
    };
    for (int32_t a = 0; a < P.nado; a++) {
        int64_t u = ados[a];
        int64_t st = t.ind_spa[u - 1] - 1;
        int nz = t.nnz_spa[u - 1];
        int cls = B.cls_of[u - 1];
        P.ado_off[a] = (int32_t)st;
        P.ado_cls.push_back(cls);
        for (int q = 0; q < nz; q++) P.ent_ado[st + q] = a;
        P.n_terms_same += P.term_ptr[P.cls_tptr[cls] + nz] - P.term_ptr[P.cls_tptr[cls]];
        int it = tier_of(u), nb = it - 1;
        cd g0 = 0;
        int8_t cnt[4] = {0, 0, 0, 0};
        auto push = [&](int64_t src, int o, int s, bool dag, bool tr, cd l, cd r, int8_t kind) {
            if (src < 1 || src > t.nunk) fail(HEOM_E_ARG, "coupling target out of range");
            int cin = B.cls_of[src - 1];
            if (cin < 0) return;                          // source ADO stores nothing
            int32_t mb = B.get_map(P, cls, cin, o, s, dag, tr);
            if (mb < 0) return;                           // no entry of n is reached
            CoupRec rec{(int32_t)(t.ind_spa[src - 1] - 1), mb, B.get_coef(P, l, r, kind) | (tr ? kCoefConj : 0), 0};
            P.coup.push_back(rec);
            for (int p = 0; p < nz; p++) P.gather_hits += ((P.maps[mb + p] & 0xFFFFu) != 0) + ((P.maps[mb + p] >> 16) != 0);
        };
        const cd mi(0, -1), pi(0, 1);
        if (it == 1) {
            // RDO: -i a S + i S a and its Hermitian conjugate, S = sum of first-tier + ADOs
            for (int s = 1; s <= t.nspin; s++)
                for (int o = 1; o <= t.norbs; o++)
                    for (int al = 1; al <= t.nalf; al++)
                        for (int k = 1; k <= t.ncor; k++) {
                            int iopr = ((s - 1) * t.norbs + o - 1) * t.nalf + al;
                            int d = (iopr - 1) * t.ncor + k;
                            if (t.indexdraw[d - 1] == 0) continue;      // screened operator
                            int64_t src = t.nfirst[1] - 1 + t.indexdraw[d - 1];
                            push(src, o, s, false, false, mi, pi, 0);
                            push(src, o, s, true, true, mi, pi, 0);
                        }
        } else {
            const int32_t *drw = &t.indextable[t.ifirst[it - 1] - 1 + (u - t.nfirst[it - 1]) * nb];
            for (int b = 0; b < nb; b++) {
                int d = drw[b];
                if (d < 1 || d > nvar) fail(HEOM_E_ARG, "indextable entry out of range");
                g0 += cgamma[d - 1];
                int slot = (t.ilead[d - 1] - 1) + (t.mspin[d - 1] - 1) * t.nalf;
                cnt[slot] += (int8_t)(t.dipm[d - 1] > 0 ? 1 : -1);
            }
            int64_t lnl = t.index_coef_ref[u - 1];
            if (lnl < 1 || lnl > t.lall) fail(HEOM_E_ARG, "index_coef_ref out of range");
            for (int b = 0; b < nb; b++, lnl++) {
                int d = drw[b];
                double ff = t.ifactfcoef[lnl - 1], fr = t.ifactrcoef[lnl - 1];
                push(t.indexcoef[lnl - 1], t.morbs[d - 1], t.mspin[d - 1], t.mpm[d - 1] == 1, t.itypecoef[lnl - 1] != 0,
                     cb[cbidx(d)] * cd(0, -ff), cdv[cbidx(d)] * cd(0, fr), 1);
            }
            if (it < t.ntier) {
                for (int sg = 1; sg <= 2; sg++)
                    for (int s = 1; s <= t.nspin; s++)
                        for (int o = 1; o <= t.norbs; o++)
                            for (int al = 1; al <= t.nalf; al++) {
                                int iopr = ((sg - 1) * t.nspin * t.norbs + (s - 1) * t.norbs + o - 1) * t.nalf + al;
                                if (t.indexdraw[(iopr - 1) * t.ncor] == 0) continue;    // screened operator
                                for (int k = 1; k <= t.ncor; k++, lnl++) {
                                    double ff = t.ifactfcoef[lnl - 1], fr = t.ifactrcoef[lnl - 1];
                                    push(t.indexcoef[lnl - 1], o, s, sg != 1, t.itypecoef[lnl - 1] != 0,
                                         cd(0, -ff), cd(0, fr), 0);
                                }
                            }
            }
        }
        P.g0.push_back(g0);
        uint32_t packed = 0;
        for (int k = 0; k < 4; k++) packed |= (uint32_t)(uint8_t)cnt[k] << (8 * k);
        P.ado_cnt.push_back((int32_t)packed);
        P.coup_ptr.push_back((int32_t)P.coup.size());
    }
    P.ado_off[P.nado] = (int32_t)P.lunk;
    for (int64_t e = 0; e < P.lunk; e++)
        if (P.ent_ado[e] < 0) fail(HEOM_E_ARG, "stored entries do not tile the vector");
    // trace slot: diagonal entries of the RDO pattern
    if (t.nnz_spa[0] > 0)
        for (int q = 0; q < t.nnz_spa[0]; q++)
            if (t.irow_spa[q] == t.icol_spa[q]) P.trace_idx.push_back(q);
    P.n_couplings = (int64_t)P.coup.size();
    split_couplings(P);
    if (P.maps.size() >= (size_t)1 << 31 || P.cl.size() >= (size_t)1 << 30) fail(HEOM_E_UNSUPPORTED, "plan too large");
}

void build_adjoint_plan(const heom_tables &t, const HostPlan &F, HostPlan &A) {
    // Transpose of the forward plan in the real inner product Re(u^H v): a linear
    // term y_p += c x_q becomes x_q += conj(c) y_p; a conjugate term y_p += c conj(x_q)
    // becomes x_q += c conj(y_p).  Each coupling map is a partial permutation per side,
    // so its transpose is again a map (one source per side per output entry).
    A = HostPlan();
    A.adjoint = 1;
    A.lunk = F.lunk; A.nado = F.nado; A.nslots = F.nslots; A.nh = F.nh;
    A.ent_ado = F.ent_ado; A.ado_off = F.ado_off; A.ado_cls = F.ado_cls; A.ado_cnt = F.ado_cnt; A.g0 = F.g0;
    A.n_classes = F.n_classes;
    // same-tier class terms transposed within the class: out q <- in p, coefficient conj'ed in-kernel
    int ncls = (int)F.cls_tptr.size();
    std::vector<int> nnzc(ncls);
    for (int32_t a = 0; a < F.nado; a++) nnzc[F.ado_cls[a]] = F.ado_off[a + 1] - F.ado_off[a];
    for (int c = 0; c < ncls; c++) {
        int nz = nnzc[c];
        std::vector<std::vector<uint32_t>> rows(nz);
        for (int p = 0; p < nz; p++)
            for (int k = F.term_ptr[F.cls_tptr[c] + p]; k < F.term_ptr[F.cls_tptr[c] + p + 1]; k++) {
                uint32_t w = F.terms[k];
                int q = (int)(w & 0xFFFF);
                rows[q].push_back((w & 0xFFFF0000u) | (uint32_t)p);
            }
        A.cls_tptr.push_back((int32_t)A.term_ptr.size());
        for (int q = 0; q < nz; q++) {
            A.term_ptr.push_back((int32_t)A.terms.size());
            A.terms.insert(A.terms.end(), rows[q].begin(), rows[q].end());
        }
        A.term_ptr.push_back((int32_t)A.terms.size());
    }
    A.n_terms_same = F.n_terms_same;
    // couplings: gather per output (= forward source) ADO
    std::vector<std::vector<std::pair<int32_t, int64_t>>> by_src(F.nado);   // (forward out ADO, record index)
    for (int32_t a = 0; a < F.nado; a++)
        for (int e = F.coup_ptr[a]; e < F.coup_ptr[a + 1]; e++) {
            int32_t src_ado = F.ent_ado[F.coup[e].src_off];
            by_src[src_ado].push_back({a, e});
        }
    std::map<std::pair<int32_t, int32_t>, int32_t> tmaps;   // (forward map base, out ADO class nnz) -> adjoint base
    std::map<std::pair<std::pair<double, double>, std::pair<double, double>>, int32_t> coef_ids;
    auto coef = [&](cd l, cd r, int8_t kind) {
        int32_t u = unit_code(l, r);
        if (u >= 0) return u;
        auto key = std::make_pair(std::make_pair(l.real(), l.imag()), std::make_pair(r.real(), r.imag()));
        auto it = coef_ids.find(key);
        if (it != coef_ids.end()) return it->second;
        int32_t id = (int32_t)A.cl.size();
        A.cl.push_back(l); A.cr.push_back(r); A.coef_kind.push_back(kind);
        coef_ids.emplace(key, id);
        return id;
    };
    A.coup_ptr.push_back(0);
    for (int32_t j = 0; j < F.nado; j++) {
        int nzj = F.ado_off[j + 1] - F.ado_off[j];
        for (auto &pr : by_src[j]) {
            int32_t a = pr.first;
            const CoupRec &r = F.coup[pr.second];
            int nza = F.ado_off[a + 1] - F.ado_off[a];
            auto key = std::make_pair(r.map_base, j);
            auto it = tmaps.find(key);
            int32_t base;
            if (it == tmaps.end()) {
                std::vector<uint32_t> words(nzj, 0);
                for (int p = 0; p < nza; p++) {
                    uint32_t w = F.maps[r.map_base + p];
                    uint32_t lo = w & 0xFFFF, hi = w >> 16;
                    if (lo) { int q = (int)(lo & 0x7FFF) - 1; words[q] |= (uint32_t)(p + 1) | (lo & 0x8000u); }
                    if (hi) { int q = (int)(hi & 0x7FFF) - 1; words[q] |= ((uint32_t)(p + 1) | (hi & 0x8000u)) << 16; }
                }
                base = (int32_t)A.maps.size();
                A.maps.insert(A.maps.end(), words.begin(), words.end());
                A.n_maps++;
                tmaps.emplace(key, base);
            } else {
                base = it->second;
            }
            bool tr = (r.cid & kCoefConj) != 0;
            cd l, rr;
            decode_coef(F, r.cid & ~kCoefConj, l, rr);
            int8_t kind = (r.cid & kCoefUnit) ? 0 : F.coef_kind[r.cid & 0x3FFFFFFF];
            if (!tr) { l = std::conj(l); rr = std::conj(rr); }
            CoupRec rec{F.ado_off[a], base, coef(l, rr, kind) | (tr ? kCoefConj : 0), 0};
            A.coup.push_back(rec);
        }
        // trace slot: y[lunk] = sum of RDO diagonal entries  ->  adjoint adds x[lunk] to them
        if (j == 0 && !F.trace_idx.empty() && F.ado_off[0] == 0) {
            std::vector<uint32_t> words(nzj, 0);
            for (int q : F.trace_idx) words[q] = 1u;   // left source index 0 (the trace slot), plus sign
            int32_t base = (int32_t)A.maps.size();
            A.maps.insert(A.maps.end(), words.begin(), words.end());
            CoupRec rec{(int32_t)F.lunk, base, coef(cd(1, 0), cd(0, 0), 0), 0};
            A.coup.push_back(rec);
        }
        A.coup_ptr.push_back((int32_t)A.coup.size());
    }
    A.n_couplings = (int64_t)A.coup.size();
    split_couplings(A);
    (void)t;
}

void split_couplings(HostPlan &P)
{
    P.coup_mid.assign(P.nado, 0);
    for (int32_t a = 0; a < P.nado; a++) {
        auto b = P.coup.begin() + P.coup_ptr[a], e = P.coup.begin() + P.coup_ptr[a + 1];
        auto mid = std::stable_partition(b, e, [](const CoupRec &r) { return (r.cid & kCoefUnit) == 0; });
        P.coup_mid[a] = (int32_t)(mid - P.coup.begin());
    }
}

double plan_read_bytes(const HostPlan &P) {
    double mapwords = 0;
    for (int32_t a = 0; a < P.nado; a++)
        mapwords += (double)(P.coup_ptr[a + 1] - P.coup_ptr[a]) * (P.ado_off[a + 1] - P.ado_off[a]);
    return (double)P.coup.size() * 16.0 + mapwords * 4.0 + (double)P.lunk * 4.0 + (double)P.nado * 32.0;
}

void gamma_derivative_coefs(const heom_tables &, const HostPlan &F, double gamma, std::vector<cd> &cl, std::vector<cd> &cr) {
    cl.assign(F.cl.size(), 0.0);
    cr.assign(F.cr.size(), 0.0);
    for (size_t k = 0; k < F.cl.size(); k++)
        if (F.coef_kind[k] == 1) { cl[k] = F.cl[k] / gamma; cr[k] = F.cr[k] / gamma; }
}

// Plan of the correlation-function operator (corrfunc/calc_ax_cf_spa_omp.f90) on the
// entries [h (lunkcf); a (lunkcf)].  Each component has the steady operator's same-tier
// terms on the cf pattern; every coupling crosses the components: the h rows gather from
// a with the coefficients (cL zfront, cR zrear), zfront = -i, zrear = +i, and the a rows
// gather from h with the negated pair (calc_ax_cf_spa_omp.f90:344-416, 467-510).  The RDO
// rows' Hermitian-conjugate pushes (c2 + c2^dag for h, c1 + c1^dag for a, lines 161-235)
// transform the same way, because the conjugate of zrear is zfront.  A unit pair
// (i sL, i sR) becomes the real pair (sL, -sR) in h rows and (-sL, sR) in a rows: the
// kernel adds the unit gathers without the factor i when it runs the cf operator.  The
// +-omega terms between h and a are added by the kernel from the per-instance frequency.
void build_cf_plan(const heom_tables &t, const heom_cf_tables &cf, const HStructure &hst, HostPlan &out) {
    if (cf.lunkcf_spa < 1 || !cf.nnzcf_spa || !cf.indcf_spa || !cf.irowcf_spa || !cf.icolcf_spa)
        fail(HEOM_E_ARG, "empty correlation-function pattern");
    if (cf.nnzcf_spa[0] < 1) fail(HEOM_E_ARG, "correlation-function pattern without RDO entries");
    if (2 * cf.lunkcf_spa >= (int64_t)1 << 31) fail(HEOM_E_UNSUPPORTED, "more than 2^30 correlation-function entries");
    heom_tables tc = t;
    tc.lunk_spa = cf.lunkcf_spa;
    tc.nnz_spa = cf.nnzcf_spa; tc.ind_spa = cf.indcf_spa;
    tc.irow_spa = cf.irowcf_spa; tc.icol_spa = cf.icolcf_spa;
    HostPlan P;
    build_forward_plan(tc, hst, P);
    const int64_t L = P.lunk;
    const int32_t na = P.nado, ncoef = (int32_t)P.cl.size(), ncp = (int32_t)P.coup.size();
    out = HostPlan();
    out.lunk = 2 * L; out.nado = 2 * na; out.nslots = P.nslots; out.nh = P.nh;
    out.ent_ado.resize(2 * L);
    for (int64_t e = 0; e < L; e++) { out.ent_ado[e] = P.ent_ado[e]; out.ent_ado[L + e] = P.ent_ado[e] + na; }
    out.ado_off.resize(2 * (size_t)na + 1);
    for (int32_t a = 0; a < na; a++) { out.ado_off[a] = P.ado_off[a]; out.ado_off[na + a] = (int32_t)(L + P.ado_off[a]); }
    out.ado_off[2 * na] = (int32_t)(2 * L);
    for (int h = 0; h < 2; h++) {
        out.ado_cls.insert(out.ado_cls.end(), P.ado_cls.begin(), P.ado_cls.end());
        out.ado_cnt.insert(out.ado_cnt.end(), P.ado_cnt.begin(), P.ado_cnt.end());
        out.g0.insert(out.g0.end(), P.g0.begin(), P.g0.end());
    }
    out.cls_tptr = P.cls_tptr; out.term_ptr = P.term_ptr; out.terms = P.terms; out.maps = P.maps;
    const cd zf(0, -1), zr(0, 1);
    out.cl.resize(2 * (size_t)ncoef); out.cr.resize(2 * (size_t)ncoef); out.coef_kind.resize(2 * (size_t)ncoef);
    for (int32_t k = 0; k < ncoef; k++) {
        out.cl[k] = P.cl[k] * zf; out.cr[k] = P.cr[k] * zr;
        out.cl[ncoef + k] = -out.cl[k]; out.cr[ncoef + k] = -out.cr[k];
        out.coef_kind[k] = out.coef_kind[ncoef + k] = P.coef_kind[k];
    }
    out.coup.resize(2 * (size_t)ncp);
    out.coup_ptr.resize(2 * (size_t)na + 1);
    out.coup_mid.resize(2 * (size_t)na);
    for (int h = 0; h < 2; h++) {
        for (int32_t k = 0; k < ncp; k++) {
            CoupRec r = P.coup[k];
            const int32_t conj = r.cid & kCoefConj, id = r.cid & ~kCoefConj;
            if (h == 0) r.src_off = (int32_t)(r.src_off + L);     // h rows read a
            int32_t nid;
            if (id & kCoefUnit) nid = id ^ (h == 0 ? 2 : 1);       // (sL, -sR) / (-sL, sR)
            else nid = id + (h == 0 ? 0 : ncoef);
            r.cid = nid | conj;
            out.coup[(size_t)h * ncp + k] = r;
        }
        for (int32_t a = 0; a < na; a++) {
            out.coup_ptr[(size_t)h * na + a] = P.coup_ptr[a] + h * ncp;
            out.coup_mid[(size_t)h * na + a] = P.coup_mid[a] + h * ncp;
        }
    }
    out.coup_ptr[2 * (size_t)na] = 2 * ncp;
    out.n_terms_same = 2 * P.n_terms_same; out.n_couplings = 2 * P.n_couplings; out.n_maps = P.n_maps;
    out.n_classes = P.n_classes; out.gather_hits = 2 * P.gather_hits;
}

}  // namespace heom
