// Host-side model builder: the set-up work the Fortran driver of HEOM-QUICK2 does
// before its sparse hot path (main/evaluatepara.f90, main/buildoperator.f90,
// main/calchs.f90, main/ball2drawer.f90, main/buildcoefindex.f90,
// fermion/prelude_spa.f90), producing tables identical to the reference's for the
// Lorentzian/Pade input subset.  The algorithms here are independent of the
// reference's: bisection for the Pade eigenvalues, a closed-form Jordan-Wigner
// construction of the operators, hashed multiset lookups for the coupling tables
// and a boolean structural propagation for the per-ADO sparsity.
#include <algorithm>
#include <exception>
#include <mutex>
#include <thread>
#include <array>
#include <cmath>
#include <cstring>
#include <map>
#include <unordered_map>
#include <unordered_set>

#include "common.h"

using heom::cd;

struct heom_model {
    heom_params p{};
    int norbs = 0, nspin = 0, nalf = 0, nmats = 0, ntier = 0, ncor = 0, nopr = 0, nvar = 0, nrho = 0, nams = 0;
    std::vector<double> cpcoef;
    std::vector<cd> cppole;                       // (nmats, 2)
    std::vector<cd> psfcoef, psfpole;             // Prony scheme: the caller's fitted table (npsf)
    std::vector<cd> cb, cdd, cgama, cgamma;
    std::vector<double> dipm, eleadinfty, amps, tcharv, hybrid;
    std::vector<int32_t> mpm, morbs, mspin, ilead, mcor, mopr, iredex, indexdraw, jredex, jomit;
    std::vector<double> amsori;                   // (nrho, nrho, norbs, nspin)
    std::vector<int32_t> rowams, colams, sgnams;
    std::vector<cd> hs, dhs_deps, dhs_du;
    std::vector<int64_t> nfirst, nlast, ifirst, ilast;
    std::vector<int32_t> indextable;
    std::vector<int64_t> index_coef_ref, indexcoef;
    std::vector<int8_t> itypecoef, ifactfcoef, ifactrcoef;
    std::vector<int32_t> nnz_spa, irow_spa, icol_spa;
    std::vector<int64_t> ind_spa;
    int64_t nunk = 0, lall = 0, lunk = 0;
    heom_tables view{};
    // correlation-function pattern of the last heom_model_cf_pattern call
    std::vector<int32_t> cf_nnz, cf_irow, cf_icol;
    std::vector<int64_t> cf_ind;
    int64_t cf_lunk = 0;
    int cf_iorbs = 0, cf_ispin = 0;
};

namespace {

// ---- Pade decomposition of the Fermi function (role of main/zpout_psd.f90) ----
// Eigenvalues of a symmetric tridiagonal matrix with zero diagonal by Sturm-sequence bisection.
std::vector<double> tridiag_eigs(const std::vector<double> &off) {
    int n = (int)off.size() + 1;
    double bound = 0;
    for (double b : off) bound = std::max(bound, 2 * std::fabs(b));
    bound += 1.0;
    auto count_below = [&](double x) {
        int cnt = 0;
        double q = -x;
        if (q < 0) cnt++;
        for (int i = 1; i < n; i++) {
            double qq = (q == 0.0) ? 1e-300 : q;
            q = -x - off[i - 1] * off[i - 1] / qq;
            if (q < 0) cnt++;
        }
        return cnt;
    };
    std::vector<double> ev(n);
    for (int k = 0; k < n; k++) {
        double lo = -bound, hi = bound;
        for (int it = 0; it < 200; it++) {
            double mid = 0.5 * (lo + hi);
            if (count_below(mid) > k) hi = mid; else lo = mid;
            if (hi - lo <= 1e-17 * std::max(1.0, std::fabs(mid))) break;
        }
        ev[k] = 0.5 * (lo + hi);
    }
    return ev;
}

void pade(int M, std::vector<double> &coef, std::vector<cd> &pole) {
    std::vector<double> o0(2 * M - 1), o1(std::max(0, 2 * M - 2));
    for (int i = 1; i < 2 * M; i++) o0[i - 1] = 1.0 / std::sqrt((2.0 * i - 1) * (2.0 * i + 1));
    for (int i = 1; i < 2 * M - 1; i++) o1[i - 1] = 1.0 / std::sqrt((2.0 * i + 1) * (2.0 * i + 3));
    std::vector<double> e0 = tridiag_eigs(o0), e1 = o1.empty() ? std::vector<double>() : tridiag_eigs(o1);
    std::vector<double> xi(M), zeta(std::max(0, M - 1));
    for (int i = 0; i < M; i++) xi[i] = 4.0 / (e0[i] * e0[i]);
    for (int i = 0; i < M - 1; i++) zeta[i] = 4.0 / (e1[i] * e1[i]);
    coef.assign(M, 0.0);
    pole.assign(2 * M, cd(0, 0));
    for (int j = 0; j < M; j++) {
        double t = 1.0;
        for (int k = 0; k < M; k++) {
            if (k == j) continue;
            double zk = k < j ? zeta[k] : zeta[k - 1];
            t *= (zk - xi[j]) / (xi[k] - xi[j]);
        }
        coef[j] = -0.5 * M * (2 * M + 1) * t;
        pole[j] = cd(0, std::sqrt(xi[j]));
        pole[M + j] = std::conj(pole[j]);
    }
}

cd fermi_pade(const heom_model &m, int isgn, cd z) {
    cd c(0.5, 0);
    for (int i = 0; i < m.nmats; i++) {
        cd pl = m.cppole[(isgn - 1) * m.nmats + i];
        c += m.cpcoef[i] / (z + pl) + m.cpcoef[i] / (z - pl);
    }
    return c;
}

size_t cbidx(const heom_model &m, int o, int s, int k, int a, int sg) {
    return ((((size_t)(sg - 1) * m.nalf + (a - 1)) * m.ncor + (k - 1)) * m.nspin + (s - 1)) * m.norbs + (o - 1);
}

// ---- operators: Jordan-Wigner strings over the mode order in which orbital o
// lists spin up before spin down when o is odd and spin down first when o is
// even (this is the convention the reference's swap chain of
// main/buildoperator.f90 produces). Basis index = sum_o digit_o 4^(o-1),
// digit = up + 2*down, 1-based. ----
void build_operators(heom_model &m) {
    const int n = m.nrho, no = m.norbs, ns = m.nspin;
    m.amsori.assign((size_t)n * n * no * ns, 0.0);
    std::vector<std::pair<int, int>> order;   // (orbital, spin) 0-based, JW order
    for (int o = 0; o < no; o++) {
        if (ns == 1) order.push_back({o, 0});
        else if (o % 2 == 0) { order.push_back({o, 0}); order.push_back({o, 1}); }
        else { order.push_back({o, 1}); order.push_back({o, 0}); }
    }
    auto bit = [&](int o, int s) { return ns == 2 ? 2 * o + s : o; };
    for (int o = 0; o < no; o++)
        for (int s = 0; s < ns; s++) {
            int pos = (int)(std::find(order.begin(), order.end(), std::make_pair(o, s)) - order.begin());
            for (int c = 0; c < n; c++) {
                if (!((c >> bit(o, s)) & 1)) continue;
                int par = 0;
                for (int k = 0; k < pos; k++) par += (c >> bit(order[k].first, order[k].second)) & 1;
                int r = c - (1 << bit(o, s));
                m.amsori[(size_t)r + (size_t)c * n + ((size_t)o + (size_t)s * no) * n * n] = (par & 1) ? -1.0 : 1.0;
            }
        }
    m.nams = ns == 2 ? 2 * (int)std::pow(4.0, no - 1) : (1 << (no - 1));
    size_t tot = (size_t)m.nams * no * ns;
    m.rowams.assign(tot, 0); m.colams.assign(tot, 0); m.sgnams.assign(tot, 0);
    for (int s = 0; s < ns; s++)
        for (int o = 0; o < no; o++) {
            size_t base = (size_t)m.nams * (o + (size_t)s * no);
            int cnt = 0;
            for (int j = 0; j < n; j++)
                for (int i = 0; i < n; i++) {
                    double v = m.amsori[(size_t)i + (size_t)j * n + ((size_t)o + (size_t)s * no) * n * n];
                    if (v != 0.0) {
                        m.rowams[base + cnt] = i + 1; m.colams[base + cnt] = j + 1; m.sgnams[base + cnt] = v > 0 ? 0 : 1;
                        cnt++;
                    }
                }
            if (cnt != m.nams) heom::fail(HEOM_E_ARG, "operator construction: unexpected nonzero count");
        }
}

using CMat = std::vector<cd>;
CMat cmul(int n, const CMat &a, const CMat &b) {
    CMat c((size_t)n * n);
    for (int j = 0; j < n; j++)
        for (int k = 0; k < n; k++) {
            cd bkj = b[(size_t)k + (size_t)j * n];
            if (bkj == 0.0) continue;
            for (int i = 0; i < n; i++) c[(size_t)i + (size_t)j * n] += a[(size_t)i + (size_t)k * n] * bkj;
        }
    return c;
}
CMat op(const heom_model &m, int o, int s, bool dag) {  // 1-based orbital/spin
    int n = m.nrho;
    CMat a((size_t)n * n);
    const double *src = &m.amsori[((size_t)(o - 1) + (size_t)(s - 1) * m.norbs) * n * n];
    for (int j = 0; j < n; j++)
        for (int i = 0; i < n; i++) a[dag ? (size_t)j + (size_t)i * n : (size_t)i + (size_t)j * n] = src[(size_t)i + (size_t)j * n];
    return a;
}
void axpy(CMat &y, cd a, const CMat &x) { for (size_t k = 0; k < y.size(); k++) y[k] += a * x[k]; }

// ---- system Hamiltonians (role of main/calchs.f90 para1/para4 and lreadhs data) ----
void build_hs(heom_model &m) {
    const int n = m.nrho;
    const double hb = heom::kHbar;
    const heom_params &p = m.p;
    m.hs.assign((size_t)n * n, 0.0);
    m.dhs_deps.assign((size_t)n * n, 0.0);
    m.dhs_du.assign((size_t)n * n, 0.0);
    auto num = [&](int o, int s) { return cmul(n, op(m, o, s, true), op(m, o, s, false)); };
    if (p.model == 1) {
        if (m.norbs != 1 || m.nspin != 2) heom::fail(HEOM_E_ARG, "model 1 ($para1) needs norbs=1, nspin=2");
        CMat nu = num(1, 1), nd = num(1, 2), nn = cmul(n, nu, nd);
        axpy(m.hs, p.eup / hb, nu); axpy(m.hs, p.edown / hb, nd); axpy(m.hs, p.uu / hb, nn);
        axpy(m.dhs_deps, 1.0 / hb, nu); axpy(m.dhs_deps, 1.0 / hb, nd);
        axpy(m.dhs_du, 1.0 / hb, nn);
    } else if (p.model == 4) {
        if (m.norbs != 2 || m.nspin != 2) heom::fail(HEOM_E_ARG, "model 4 ($para4) needs norbs=2, nspin=2");
        CMat n1u = num(1, 1), n1d = num(1, 2), n2u = num(2, 1), n2d = num(2, 2);
        axpy(m.hs, p.e1up / hb, n1u); axpy(m.hs, p.e1down / hb, n1d);
        axpy(m.hs, p.e2up / hb, n2u); axpy(m.hs, p.e2down / hb, n2d);
        CMat d1 = cmul(n, n1u, n1d), d2 = cmul(n, n2u, n2d);
        axpy(m.hs, p.uu1 / hb, d1); axpy(m.hs, p.uu2 / hb, d2);
        CMat n1 = n1u, n2 = n2u;
        axpy(n1, 1.0, n1d); axpy(n2, 1.0, n2d);
        axpy(m.hs, p.u12 / hb, cmul(n, n1, n2));
        CMat hop((size_t)n * n);
        for (int s = 1; s <= 2; s++) {
            axpy(hop, 1.0, cmul(n, op(m, 1, s, true), op(m, 2, s, false)));
            axpy(hop, 1.0, cmul(n, op(m, 2, s, true), op(m, 1, s, false)));
        }
        axpy(m.hs, p.t12 / hb, hop);
        for (const CMat *q : {&n1u, &n1d, &n2u, &n2d}) axpy(m.dhs_deps, 1.0 / hb, *q);
        axpy(m.dhs_du, 1.0 / hb, d1); axpy(m.dhs_du, 1.0 / hb, d2);
    } else if (p.model == 5) {
        // Kanamori: eps sum n + U sum n_u n_d + U' sum_{m!=m'} n_mu n_m'd + (U'-J) sum_{m<m',s} n_ms n_m's
        //           - J sum_{m!=m'} c+_mu c_md c+_m'd c_m'u + J sum_{m!=m'} c+_mu c+_md c_m'd c_m'u,  U' = U - 2J
        const int no = m.norbs;
        double U = p.kan_u / hb, J = p.kan_j / hb, Up = U - 2 * J, eps = p.kan_eps / hb;
        for (int o = 1; o <= no; o++) {
            CMat nu = num(o, 1), nd = num(o, 2), nn = cmul(n, nu, nd);
            axpy(m.hs, eps, nu); axpy(m.hs, eps, nd); axpy(m.hs, U, nn);
            axpy(m.dhs_deps, 1.0 / hb, nu); axpy(m.dhs_deps, 1.0 / hb, nd);
            axpy(m.dhs_du, 1.0 / hb, nn);
        }
        for (int o = 1; o <= no; o++)
            for (int q = 1; q <= no; q++) {
                if (o == q) continue;
                axpy(m.hs, Up, cmul(n, num(o, 1), num(q, 2)));
                if (o < q)
                    for (int s = 1; s <= 2; s++) axpy(m.hs, Up - J, cmul(n, num(o, s), num(q, s)));
                CMat sf = cmul(n, cmul(n, cmul(n, op(m, o, 1, true), op(m, o, 2, false)), op(m, q, 2, true)), op(m, q, 1, false));
                axpy(m.hs, -J, sf);
                CMat ph = cmul(n, cmul(n, cmul(n, op(m, o, 1, true), op(m, o, 2, true)), op(m, q, 2, false)), op(m, q, 1, false));
                axpy(m.hs, J, ph);
            }
    } else if (p.model == 9) {
        if (!p.hs_in) heom::fail(HEOM_E_ARG, "model 9 needs hs_in");
        for (size_t k = 0; k < (size_t)n * n; k++) m.hs[k] = p.hs_in[k];
    } else {
        heom::fail(HEOM_E_UNSUPPORTED, "unknown model");
    }
}

// ---- bath coefficients (role of main/evaluatepara.f90:1897-2227, Lorentzian + PSD) ----
void build_coefficients(heom_model &m) {
    const heom_params &p = m.p;
    const double hb = heom::kHbar;
    const bool psf = p.npsf > 0;
    double width[2] = {p.bandwidth[0], p.bandwidth[1]};
    if (psf) {
        // psfjob (main/evaluatepara.f90:256-722, 1187-1189): the npsf fitted terms replace the
        // Drude pole and the Pade terms; the band half-width is rpsf * T, centred at 0
        if (p.npsf > 64 || !p.psf_coef || !p.psf_pole || !(p.tpsf > 0) || !(p.rpsf > 0))
            heom::fail(HEOM_E_ARG, "the Prony scheme needs 1..64 coefficients and poles, tpsf > 0 and rpsf > 0");
        const cd *zc = reinterpret_cast<const cd *>(p.psf_coef), *zp = reinterpret_cast<const cd *>(p.psf_pole);
        m.psfcoef.assign(zc, zc + p.npsf);
        m.psfpole.assign(zp, zp + p.npsf);
        m.nmats = p.npsf;
        m.ncor = m.nmats;
        for (int a = 0; a < m.nalf; a++) width[a] = p.temperature[a] * p.rpsf;
    } else {
        m.ncor = 1 + m.nmats;
        pade(m.nmats, m.cpcoef, m.cppole);
    }
    m.nopr = 2 * m.norbs * m.nspin * m.nalf;
    m.nvar = m.nopr * m.ncor;
    m.nrho = 1;
    for (int k = 0; k < m.norbs; k++) m.nrho *= 2 * m.nspin;
    std::vector<double> zxip((size_t)m.nalf * m.norbs), lw((size_t)m.nalf * m.norbs);
    for (int a = 0; a < m.nalf; a++)
        for (int o = 0; o < m.norbs; o++) {
            lw[a * m.norbs + o] = p.linewidth[a][o];
            zxip[a * m.norbs + o] = p.linewidth[a][o] * width[a] * width[a] * 0.5;
        }
    if (p.doubledot) {
        if (m.norbs != 2 || m.nalf != 2) heom::fail(HEOM_E_ARG, "doubledot needs norbs=2 and nalf=2");
        lw[0 * 2 + 1] = 0; lw[1 * 2 + 0] = 0;
        std::fill(zxip.begin(), zxip.end(), 0.0);
        zxip[0] = p.linewidth[0][0] * width[0] * width[0] * 0.5;
        zxip[1 * 2 + 1] = p.linewidth[1][1] * width[1] * width[1] * 0.5;
    }
    m.hybrid.resize(lw.size());
    for (size_t k = 0; k < lw.size(); k++) m.hybrid[k] = lw[k] / hb;
    size_t ncb = (size_t)m.norbs * m.nspin * m.ncor * m.nalf * 2;
    m.cb.assign(ncb, 0.0); m.cdd.assign(ncb, 0.0); m.cgama.assign(ncb, 0.0);
    for (int sg = 1; sg <= 2; sg++) {
        double dpm = sg == 1 ? 1.0 : -1.0;
        for (int s = 1; s <= m.nspin; s++)
            for (int o = 1; o <= m.norbs; o++)
                for (int a = 1; a <= m.nalf; a++) {
                    double T = p.temperature[a - 1], W = width[a - 1], zx = zxip[(a - 1) * m.norbs + (o - 1)];
                    for (int k = 1; k <= m.ncor; k++) {
                        size_t id = cbidx(m, o, s, k, a, sg);
                        if (psf) {      // fitted exponential k: T / tpsf (zpole, zcoef 2 zxip / W^2)
                            const double sc = T / p.tpsf;
                            m.cgama[id] = sc * m.psfpole[k - 1];
                            m.cb[id] = sc * m.psfcoef[k - 1] * (zx / (W * W) * 2.0);
                            m.cdd[id] = std::conj(m.cb[id]);
                        } else if (k == 1) {   // Drude pole of the Lorentzian band, Pade-expanded Fermi function
                            m.cgama[id] = cd(-W, 0) / hb;
                            cd f1 = fermi_pade(m, sg, cd(0, W / T));
                            cd f2 = fermi_pade(m, 3 - sg, cd(0, W / T));
                            m.cb[id] = zx / W * f1 / (hb * hb);
                            m.cdd[id] = std::conj(zx / W * f2) / (hb * hb);
                        } else {        // Pade poles
                            int im = k - 2;
                            cd pl = m.cppole[(sg - 1) * m.nmats + im], plt = m.cppole[(2 - sg) * m.nmats + im];
                            m.cgama[id] = dpm * cd(0, 1) * T * pl / hb;
                            cd num = cd(0, 2.0) * m.cpcoef[im] * zx * T;
                            m.cb[id] = num / (pl * T * pl * T + W * W) / (hb * hb);
                            m.cdd[id] = std::conj(num) / std::conj(plt * T * plt * T + W * W) / (hb * hb);
                        }
                    }
                }
    }
    m.jredex.resize(m.nopr); m.jomit.resize(m.nopr);
    int half = m.nopr / 2;
    for (int l = 1; l <= m.nopr; l++) m.jredex[l - 1] = l <= half ? l + half : l - half;
    int q = 0;
    for (int sg = 1; sg <= 2; sg++)
        for (int s = 1; s <= m.nspin; s++)
            for (int o = 1; o <= m.norbs; o++)
                for (int a = 1; a <= m.nalf; a++) m.jomit[q++] = std::fabs(zxip[(a - 1) * m.norbs + (o - 1)]) < heom::kDsmall;
    m.cgamma.resize(m.nvar); m.dipm.resize(m.nvar);
    for (auto *v : {&m.mpm, &m.morbs, &m.mspin, &m.ilead, &m.mcor, &m.mopr, &m.iredex, &m.indexdraw}) v->resize(m.nvar);
    int d = 0, kept = 0;
    for (int sg = 1; sg <= 2; sg++)
        for (int s = 1; s <= m.nspin; s++)
            for (int o = 1; o <= m.norbs; o++)
                for (int a = 1; a <= m.nalf; a++) {
                    int iopr = ((sg - 1) * m.nspin * m.norbs + (s - 1) * m.norbs + o - 1) * m.nalf + a;
                    for (int k = 1; k <= m.ncor; k++, d++) {
                        m.mopr[d] = iopr; m.mpm[d] = sg; m.dipm[d] = sg == 1 ? 1.0 : -1.0;
                        m.ilead[d] = a; m.morbs[d] = o; m.mspin[d] = s; m.mcor[d] = k;
                        m.cgamma[d] = m.cgama[cbidx(m, o, s, k, a, sg)];
                        bool screened = p.lscreen && m.jomit[iopr - 1];
                        m.indexdraw[d] = screened ? 0 : ++kept;
                    }
                }
    for (int l = 1; l <= m.nvar; l++) m.iredex[l - 1] = l <= m.nvar / 2 ? l + m.nvar / 2 : l - m.nvar / 2;
    m.eleadinfty.assign((size_t)m.nalf * m.nspin, 0.0);
    m.amps.assign((size_t)m.nalf * m.nspin, 0.0);
    m.tcharv.assign((size_t)m.nalf * m.nspin, 0.0);
    for (int a = 0; a < m.nalf; a++)
        for (int s = 0; s < m.nspin; s++) {
            m.amps[a + (size_t)s * m.nalf] = p.engyshift[a][s] / hb;
            m.eleadinfty[a + (size_t)s * m.nalf] = p.engyshift[a][s] / hb;
            m.tcharv[a + (size_t)s * m.nalf] = p.tchar[a][s];
        }
}

// ---- hierarchy tables ----
uint64_t pack(const int *v, int n) {   // <= 7 entries of < 2^9 (one map per tier, so n is implied)
    uint64_t k = 0;
    for (int i = 0; i < n; i++) k = (k << 9) | (uint64_t)v[i];
    return k;
}
// Open-addressing map from a packed drawer tuple to its ADO index (linear probing; the packed
// keys are below 2^63, so all ones marks an empty slot)
struct TupleIndex {
    std::vector<uint64_t> key;
    std::vector<int64_t> val;
    uint64_t mask = 0;
    explicit TupleIndex(size_t n = 0)
    {
        size_t cap = 16;
        while (cap < 2 * n) cap <<= 1;
        key.assign(cap, ~0ull);
        val.assign(cap, 0);
        mask = cap - 1;
    }
    static uint64_t mix(uint64_t k)
    {
        k ^= k >> 33;
        k *= 0xff51afd7ed558ccdull;
        k ^= k >> 33;
        return k;
    }
    void put(uint64_t k, int64_t v)
    {
        size_t i = mix(k) & mask;
        while (key[i] != ~0ull && key[i] != k) i = (i + 1) & mask;
        key[i] = k;
        val[i] = v;
    }
    const int64_t *get(uint64_t k) const
    {
        for (size_t i = mix(k) & mask; key[i] != ~0ull; i = (i + 1) & mask)
            if (key[i] == k) return &val[i];
        return nullptr;
    }
};

// parity of the exchange sort of the reference (swap whenever a[i] > a[j], i < j)
int exchange_sort(int *a, int n) {
    int f = 1;
    for (int i = 0; i < n - 1; i++)
        for (int j = i + 1; j < n; j++)
            if (a[i] > a[j]) { std::swap(a[i], a[j]); f = -f; }
    return f;
}

void build_tables(heom_model &m) {
    const int nopr = m.nopr, ncor = m.ncor, T = m.ntier;
    if (m.nvar >= 512) heom::fail(HEOM_E_UNSUPPORTED, "too many drawers for the table builder");
    m.nfirst.assign(T, 1); m.nlast.assign(T, 1); m.ifirst.assign(T, 1); m.ilast.assign(T, 1);
    m.indextable.assign(1, 0);
    std::vector<TupleIndex> lookup(T + 1);
    for (int it = 2; it <= T; it++) {
        int nb = it - 1;
        // operator multisets: nondecreasing tuples, keep one of each complement pair
        std::vector<std::vector<int>> ops;
        std::unordered_set<uint64_t> kept;
        std::vector<int> v(nb, 1);
        while (true) {
            bool ok = true;
            if (m.p.lscreen)
                for (int x : v) ok = ok && !m.jomit[x - 1];
            if (ok) {
                std::vector<int> c(nb);
                for (int i = 0; i < nb; i++) c[i] = m.jredex[v[nb - 1 - i] - 1];
                std::sort(c.begin(), c.end());
                if (!kept.count(pack(c.data(), nb))) { kept.insert(pack(v.data(), nb)); ops.push_back(v); }
            }
            int k = nb - 1;
            while (k >= 0 && v[k] == nopr) k--;
            if (k < 0) break;
            v[k]++;
            for (int i = k + 1; i < nb; i++) v[i] = v[k];
        }
        // drawer tuples: memory components nondecreasing within runs of equal operators
        std::vector<int> rows;
        for (const auto &o : ops) {
            std::vector<int> c(nb, 1);
            while (true) {
                bool ok = true;
                for (int i = 0; i + 1 < nb && ok; i++)
                    if (o[i] == o[i + 1] && c[i] > c[i + 1]) ok = false;
                if (ok)
                    for (int i = 0; i < nb; i++) rows.push_back((o[i] - 1) * ncor + c[i]);
                int k = nb - 1;
                while (k >= 0 && c[k] == ncor) { c[k] = 1; k--; }
                if (k < 0) break;
                c[k]++;
            }
        }
        int64_t cnt = (int64_t)rows.size() / nb;
        // lexicographic order of the tuples = numeric order of their packed keys (fixed width)
        std::vector<std::pair<uint64_t, int64_t>> keyed(cnt);
        for (int64_t r = 0; r < cnt; r++) keyed[r] = {pack(&rows[r * nb], nb), r};
        std::sort(keyed.begin(), keyed.end());
        m.nfirst[it - 1] = m.nlast[it - 2] + 1;
        m.nlast[it - 1] = m.nlast[it - 2] + cnt;
        m.ifirst[it - 1] = m.ilast[it - 2] + 1;
        m.ilast[it - 1] = m.ilast[it - 2] + cnt * nb;
        lookup[it] = TupleIndex((size_t)cnt);
        m.indextable.reserve(m.indextable.size() + (size_t)(cnt * nb));
        for (int64_t r = 0; r < cnt; r++) {
            const int *row = &rows[keyed[r].second * nb];
            m.indextable.insert(m.indextable.end(), row, row + nb);
            lookup[it].put(keyed[r].first, m.nfirst[it - 1] + r);
        }
    }
    m.nunk = m.nlast[T - 1];
    // couplings: lower tier entries, then higher tier in sgn > spin > orbs > alf > cor order
    m.index_coef_ref.assign(m.nunk, 0);
    auto find = [&](int tier, const int *rec, int n, int &fact, int &itype) -> int64_t {
        const TupleIndex &L = lookup[tier];
        const int64_t *hit = L.get(pack(rec, n));
        if (hit) { fact = 1; itype = 0; return *hit; }
        int c[16];
        for (int i = 0; i < n; i++) c[i] = m.iredex[rec[n - 1 - i] - 1];
        fact = exchange_sort(c, n);
        hit = L.get(pack(c, n));
        if (!hit) heom::fail(HEOM_E_ARG, "coupling target not found");
        itype = 1;
        return *hit;
    };
    // Every ADO's couplings sit at offsets known in advance: its nb lower-tier entries, then,
    // below the last tier, one entry per unscreened (sign, spin, orbital, lead, memory)
    // drawer.  The entries are filled in parallel over the ADOs of each tier.
    int nhigh = 0;
    for (int iopr = 1; iopr <= 2 * m.nspin * m.norbs * m.nalf; iopr++)
        if (!(m.p.lscreen && m.jomit[iopr - 1])) nhigh += ncor;
    int64_t lnl = 1;
    for (int it = 2; it <= T; it++)
        for (int64_t lni = m.nfirst[it - 1]; lni <= m.nlast[it - 1]; lni++) {
            m.index_coef_ref[lni - 1] = lnl;
            lnl += (it - 1) + (it < T ? nhigh : 0);
        }
    const size_t total = (size_t)(lnl - 1);
    m.indexcoef.assign(total, 0);
    m.itypecoef.assign(total, 0);
    m.ifactfcoef.assign(total, 0);
    m.ifactrcoef.assign(total, 0);
    auto fill = [&](int it, int64_t l0, int64_t l1) {
        const int nb = it - 1;
        for (int64_t lni = l0; lni < l1; lni++) {
            size_t q = (size_t)(m.index_coef_ref[lni - 1] - 1);
            const int *nk = &m.indextable[m.ifirst[it - 1] - 1 + (lni - m.nfirst[it - 1]) * nb];
            auto put = [&](int64_t tgt, int itype, int ff, int fr) {
                m.indexcoef[q] = tgt; m.itypecoef[q] = (int8_t)itype;
                m.ifactfcoef[q] = (int8_t)ff; m.ifactrcoef[q] = (int8_t)fr;
                q++;
            };
            for (int ni = 1; ni <= nb; ni++) {
                int64_t tgt = 1; int fact = 1, itype = 0;
                if (it > 2) {
                    int rec[16], c = 0;
                    for (int k = 0; k < nb; k++) if (k != ni - 1) rec[c++] = nk[k];
                    tgt = find(it - 1, rec, nb - 1, fact, itype);
                }
                int ff = (ni % 2 == 0) ? -1 : 1, fr = ((it - 1 - ni) % 2 == 0) ? 1 : -1;
                if (itype) { ff *= fact; fr *= fact; }
                put(tgt, itype, ff, fr);
            }
            if (it < T) {
                for (int sg = 1; sg <= 2; sg++)
                    for (int s = 1; s <= m.nspin; s++)
                        for (int o = 1; o <= m.norbs; o++)
                            for (int a = 1; a <= m.nalf; a++) {
                                int iopr = ((sg - 1) * m.nspin * m.norbs + (s - 1) * m.norbs + o - 1) * m.nalf + a;
                                if (m.p.lscreen && m.jomit[iopr - 1]) continue;
                                for (int k = 1; k <= ncor; k++) {
                                    int plus = (iopr - 1) * ncor + k;
                                    int fr_[16], rr[16];
                                    fr_[0] = plus;
                                    for (int q2 = 0; q2 < nb; q2++) fr_[q2 + 1] = nk[q2], rr[q2] = nk[q2];
                                    rr[nb] = plus;
                                    int ffact = exchange_sort(fr_, it), rfact = exchange_sort(rr, it);
                                    int fact, itype;
                                    int64_t tgt = find(it + 1, rr, it, fact, itype);
                                    put(tgt, itype, ffact * fact, rfact * fact);
                                }
                            }
            }
        }
    };
    const unsigned hw = std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
    for (int it = 2; it <= T; it++) {
        const int64_t l0 = m.nfirst[it - 1], l1 = m.nlast[it - 1] + 1, cnt = l1 - l0;
        const int64_t per = std::max<int64_t>(2048, (cnt + hw - 1) / hw);
        if (cnt <= per) { fill(it, l0, l1); continue; }
        std::vector<std::thread> pool;
        std::vector<std::exception_ptr> errs;
        std::mutex mu;
        for (int64_t a = l0; a < l1; a += per)
            pool.emplace_back([&, a] {
                try { fill(it, a, std::min(l1, a + per)); }
                catch (...) { std::lock_guard<std::mutex> g(mu); errs.push_back(std::current_exception()); }
            });
        for (auto &t : pool) t.join();
        if (!errs.empty()) std::rethrow_exception(errs.front());
    }
    m.lall = (int64_t)m.indexcoef.size();
}

// ---- sparsity: structural propagation of the pattern rule of fermion/prelude_spa.f90 ----
struct Bits {
    int n = 0;
    std::vector<uint64_t> w;
    explicit Bits(int n_ = 0) : n(n_), w(((size_t)n_ * n_ + 63) / 64, 0) {}
    bool get(int i, int j) const { size_t k = (size_t)i + (size_t)j * n; return (w[k >> 6] >> (k & 63)) & 1; }
    void set(int i, int j) { size_t k = (size_t)i + (size_t)j * n; w[k >> 6] |= 1ull << (k & 63); }
};

// Pattern of every ADO from the RDO seed by the tier rule: an ADO of tier >= 2 holds the
// structure of E0 (op(a) X_low + X_low op(a)) summed over its lower-tier couplings, and
// nothing when one of its drawers has no hybridisation.  Structural propagation stands in
// for the reference's random-coefficient products (nonzero with probability one).
struct PatternOut {
    std::vector<int32_t> nnz, irow, icol;
    std::vector<int64_t> ind;
    int64_t lunk = 0;
};

// E0 = exp(0.314 H) to Taylor order 10: pairs joined by a walk of <= 10 steps in the graph of H
Bits exp_structure(const heom_model &m) {
    const int n = m.nrho;
    Bits h(n), e(n);
    for (int j = 0; j < n; j++)
        for (int i = 0; i < n; i++)
            if (std::abs(m.hs[(size_t)i + (size_t)j * n]) >= heom::kDsmall) h.set(i, j);
    for (int i = 0; i < n; i++) e.set(i, i);
    for (int step = 0; step < 10; step++) {
        Bits nx = e;
        for (int j = 0; j < n; j++)
            for (int k = 0; k < n; k++)
                if (h.get(k, j))
                    for (int i = 0; i < n; i++)
                        if (e.get(i, k)) nx.set(i, j);
        e = nx;
    }
    return e;
}

void propagate_pattern(const heom_model &m, const Bits &e, const Bits &seed, PatternOut &out) {
    const int n = m.nrho;
    std::vector<std::vector<int>> ecol(n);   // rows of each column of E0
    for (int j = 0; j < n; j++)
        for (int i = 0; i < n; i++)
            if (e.get(i, j)) ecol[j].push_back(i);
    // operator maps: row of column / column of row, 1-based (0 = none)
    auto opmaps = [&](int o, int s, std::vector<int> &rofc, std::vector<int> &cofr) {
        rofc.assign(n + 1, 0); cofr.assign(n + 1, 0);
        size_t base = (size_t)m.nams * ((o - 1) + (size_t)(s - 1) * m.norbs);
        for (int k = 0; k < m.nams; k++) { rofc[m.colams[base + k]] = m.rowams[base + k]; cofr[m.rowams[base + k]] = m.colams[base + k]; }
    };
    std::vector<std::vector<int>> rofc(m.norbs * m.nspin), cofr(m.norbs * m.nspin);
    for (int s = 1; s <= m.nspin; s++)
        for (int o = 1; o <= m.norbs; o++) opmaps(o, s, rofc[(o - 1) + (s - 1) * m.norbs], cofr[(o - 1) + (s - 1) * m.norbs]);
    // The patterns repeat: an ADO's pattern is the union of one contribution per lower-tier
    // coupling, and a contribution depends only on the lower ADO's pattern, the operator, its
    // dagger and the coupling's transpose flag.  So every distinct pattern is kept once (a
    // class), every ADO holds its class, and every contribution is computed once.
    const size_t nw = ((size_t)n * n + 63) / 64;
    using Words = std::vector<uint64_t>;
    std::vector<Words> cls;
    std::map<Words, int> cls_id;
    auto class_of = [&](const Words &w) {
        auto it = cls_id.find(w);
        if (it != cls_id.end()) return it->second;
        const int id = (int)cls.size();
        cls.push_back(w);
        cls_id.emplace(w, id);
        return id;
    };
    auto bit = [n](const uint64_t *w, int i, int j) { size_t k = (size_t)i + (size_t)j * n; return (w[k >> 6] >> (k & 63)) & 1; };
    // E0 (op(a)(i, r) X(r, c) + X(r, c) op(a)(c, j)) on the structure of X (X^T when tr)
    std::map<std::array<int, 4>, Words> contrib;
    Bits sl(n), sr(n), acc(n);
    auto contribution = [&](int c, int oi, bool dag, bool tr) -> const Words & {
        const std::array<int, 4> key = {c, oi, dag ? 1 : 0, tr ? 1 : 0};
        auto hit = contrib.find(key);
        if (hit != contrib.end()) return hit->second;
        const uint64_t *low = cls[c].data();
        const std::vector<int> &rc = rofc[oi], &cr = cofr[oi];
        std::fill(sl.w.begin(), sl.w.end(), 0);
        std::fill(sr.w.begin(), sr.w.end(), 0);
        std::fill(acc.w.begin(), acc.w.end(), 0);
        for (int cc = 0; cc < n; cc++)
            for (int r = 0; r < n; r++) {
                if (!(tr ? bit(low, cc, r) : bit(low, r, cc))) continue;
                int i = dag ? cr[r + 1] : rc[r + 1];    // left:  op(a)(i, r)
                if (i) sl.set(i - 1, cc);
                int jj = dag ? rc[cc + 1] : cr[cc + 1];   // right: op(a)(c, jj)
                if (jj) sr.set(r, jj - 1);
            }
        for (const Bits *src : {&sl, &sr})
            for (int j = 0; j < n; j++)
                for (int k = 0; k < n; k++)
                    if (src->get(k, j))
                        for (int i : ecol[k]) acc.set(i, j);
        return contrib.emplace(key, acc.w).first->second;
    };
    std::vector<int> ado_cls((size_t)m.nunk, 0);
    ado_cls[0] = class_of(seed.w);
    const Words none(nw, 0);
    Words w(nw);
    for (int it = 2; it <= m.ntier; it++) {
        int nb = it - 1;
        for (int64_t lni = m.nfirst[it - 1]; lni <= m.nlast[it - 1]; lni++) {
            std::fill(w.begin(), w.end(), 0);
            bool empty = false;
            int64_t lnl = m.index_coef_ref[lni - 1];
            for (int b = 0; b < nb; b++, lnl++) {
                int d = m.indextable[m.ifirst[it - 1] - 1 + (lni - m.nfirst[it - 1]) * nb + b];
                int o = m.morbs[d - 1], s = m.mspin[d - 1], a = m.ilead[d - 1];
                if (std::fabs(m.hybrid[(a - 1) * m.norbs + (o - 1)]) <= heom::kDsmall) { empty = true; continue; }
                const Words &cw = contribution(ado_cls[(size_t)(m.indexcoef[lnl - 1] - 1)], (o - 1) + (s - 1) * m.norbs,
                                               m.mpm[d - 1] == 1, m.itypecoef[lnl - 1] != 0);
                for (size_t q = 0; q < nw; q++) w[q] |= cw[q];
            }
            ado_cls[(size_t)(lni - 1)] = class_of(empty ? none : w);
        }
    }
    // entries of every class in column-major order
    std::vector<std::vector<int32_t>> crow(cls.size()), ccol(cls.size());
    for (size_t c = 0; c < cls.size(); c++)
        for (int j = 0; j < n; j++)
            for (int i = 0; i < n; i++)
                if (bit(cls[c].data(), i, j)) { crow[c].push_back(i + 1); ccol[c].push_back(j + 1); }
    out = PatternOut();
    out.nnz.assign(m.nunk, 0);
    out.ind.assign(m.nunk, 0);
    int64_t total = 0;
    for (int64_t u = 0; u < m.nunk; u++) total += (int64_t)crow[ado_cls[(size_t)u]].size();
    out.irow.reserve((size_t)total);
    out.icol.reserve((size_t)total);
    int64_t off = 1;
    for (int64_t u = 0; u < m.nunk; u++) {
        const int c = ado_cls[(size_t)u];
        out.ind[u] = off;
        out.nnz[u] = (int32_t)crow[c].size();
        out.irow.insert(out.irow.end(), crow[c].begin(), crow[c].end());
        out.icol.insert(out.icol.end(), ccol[c].begin(), ccol[c].end());
        off += out.nnz[u];
    }
    out.lunk = off - 1;
}

// fermion/prelude_spa.f90:146-747: the RDO seed is E0 itself
void build_pattern(heom_model &m) {
    Bits e = exp_structure(m);
    PatternOut p;
    propagate_pattern(m, e, e, p);
    m.nnz_spa = std::move(p.nnz); m.ind_spa = std::move(p.ind);
    m.irow_spa = std::move(p.irow); m.icol_spa = std::move(p.icol);
    m.lunk = p.lunk;
}

// corrfunc/prelude_cf_spa.f90:146-760: the RDO seed is E0 a E0 + E0 a^dag E0 (the reference
// mixes the two with random weights), a = a_{iorbs,ispin}
void build_cf_pattern(heom_model &m, int iorbs, int ispin) {
    const int n = m.nrho;
    Bits e = exp_structure(m), seed(n);
    size_t base = (size_t)m.nams * ((iorbs - 1) + (size_t)(ispin - 1) * m.norbs);
    for (int q = 0; q < m.nams; q++) {
        int k = m.rowams[base + q] - 1, l = m.colams[base + q] - 1;   // a(k, l) != 0
        for (int j = 0; j < n; j++)
            for (int i = 0; i < n; i++) {
                if (e.get(i, k) && e.get(l, j)) seed.set(i, j);          // E0 a E0
                if (e.get(i, l) && e.get(k, j)) seed.set(i, j);          // E0 a^dag E0
            }
    }
    PatternOut p;
    propagate_pattern(m, e, seed, p);
    m.cf_nnz = std::move(p.nnz); m.cf_ind = std::move(p.ind);
    m.cf_irow = std::move(p.irow); m.cf_icol = std::move(p.icol);
    m.cf_lunk = p.lunk;
    m.cf_iorbs = iorbs; m.cf_ispin = ispin;
}

void fill_view(heom_model &m) {
    heom_tables &t = m.view;
    t = heom_tables{};
    t.norbs = m.norbs; t.nspin = m.nspin; t.nalf = m.nalf; t.ncor = m.ncor; t.ntier = m.ntier;
    t.nrho = m.nrho; t.nams = m.nams; t.lscreen = m.p.lscreen;
    t.nunk = m.nunk; t.lall = m.lall; t.lunk_spa = m.lunk;
    t.cgamma = reinterpret_cast<const double _Complex *>(m.cgamma.data());
    t.dipm = m.dipm.data();
    t.mpm = m.mpm.data(); t.morbs = m.morbs.data(); t.mspin = m.mspin.data(); t.ilead = m.ilead.data(); t.mcor = m.mcor.data();
    t.indexdraw = m.indexdraw.data();
    t.cb = reinterpret_cast<const double _Complex *>(m.cb.data());
    t.cd = reinterpret_cast<const double _Complex *>(m.cdd.data());
    t.eleadinfty = m.eleadinfty.data();
    t.nfirst = m.nfirst.data(); t.nlast = m.nlast.data(); t.ifirst = m.ifirst.data();
    t.indextable = m.indextable.data(); t.index_coef_ref = m.index_coef_ref.data();
    t.indexcoef = m.indexcoef.data(); t.itypecoef = m.itypecoef.data();
    t.ifactfcoef = m.ifactfcoef.data(); t.ifactrcoef = m.ifactrcoef.data();
    t.rowams = m.rowams.data(); t.colams = m.colams.data(); t.sgnams = m.sgnams.data();
    t.hs = reinterpret_cast<const double _Complex *>(m.hs.data());
    t.nnz_spa = m.nnz_spa.data(); t.ind_spa = m.ind_spa.data();
    t.irow_spa = m.irow_spa.data(); t.icol_spa = m.icol_spa.data();
}

// Hermitian Jacobi diagonalisation through the real symmetric embedding [[A,-B],[B,A]].
void sym_eig(int n, std::vector<double> &a, std::vector<double> &w, std::vector<double> &v) {
    v.assign((size_t)n * n, 0.0);
    for (int i = 0; i < n; i++) v[(size_t)i * n + i] = 1.0;
    for (int sweep = 0; sweep < 60; sweep++) {
        double off = 0;
        for (int j = 0; j < n; j++) for (int i = 0; i < j; i++) off += a[i + (size_t)j * n] * a[i + (size_t)j * n];
        if (off < 1e-28) break;
        for (int p = 0; p < n; p++)
            for (int q = p + 1; q < n; q++) {
                double apq = a[p + (size_t)q * n];
                if (std::fabs(apq) < 1e-300) continue;
                double th = (a[q + (size_t)q * n] - a[p + (size_t)p * n]) / (2 * apq);
                double t = (th >= 0 ? 1.0 : -1.0) / (std::fabs(th) + std::sqrt(th * th + 1));
                double c = 1 / std::sqrt(t * t + 1), s = t * c;
                for (int k = 0; k < n; k++) {
                    double x = a[k + (size_t)p * n], y = a[k + (size_t)q * n];
                    a[k + (size_t)p * n] = c * x - s * y; a[k + (size_t)q * n] = s * x + c * y;
                }
                for (int k = 0; k < n; k++) {
                    double x = a[p + (size_t)k * n], y = a[q + (size_t)k * n];
                    a[p + (size_t)k * n] = c * x - s * y; a[q + (size_t)k * n] = s * x + c * y;
                }
                for (int k = 0; k < n; k++) {
                    double x = v[k + (size_t)p * n], y = v[k + (size_t)q * n];
                    v[k + (size_t)p * n] = c * x - s * y; v[k + (size_t)q * n] = s * x + c * y;
                }
            }
    }
    w.resize(n);
    for (int i = 0; i < n; i++) w[i] = a[i + (size_t)i * n];
}

}  // namespace

extern "C" {

int heom_model_build(const heom_params *p, heom_model **out) {
    return heom::guarded([&] {
        if (!p || !out) heom::fail(HEOM_E_ARG, "null argument");
        *out = nullptr;
        if (p->norbs < 1 || p->norbs > 3 || (p->nspin != 1 && p->nspin != 2) || p->nalf < 1 || p->nalf > 2 ||
            p->nmats < 1 || p->nmats > 64 || p->ntier < 2 || p->ntier > 8)
            heom::fail(HEOM_E_ARG, "parameters out of the supported range");
        if (p->nspin != 2) heom::fail(HEOM_E_UNSUPPORTED, "only nspin = 2 models are supported");
        auto *m = new heom_model();
        try {
            m->p = *p;
            m->norbs = p->norbs; m->nspin = p->nspin; m->nalf = p->nalf; m->nmats = p->nmats; m->ntier = p->ntier;
            build_coefficients(*m);
            build_operators(*m);
            build_hs(*m);
            build_tables(*m);
            build_pattern(*m);
            fill_view(*m);
        } catch (...) {
            delete m;
            throw;
        }
        *out = m;
    });
}

void heom_model_destroy(heom_model *m) { delete m; }

int heom_model_cf_pattern(heom_model *m, int32_t iorbs, int32_t ispin, heom_cf_tables *out) {
    return heom::guarded([&] {
        if (!m || !out) heom::fail(HEOM_E_ARG, "null argument");
        if (iorbs < 1 || iorbs > m->norbs || ispin < 1 || ispin > m->nspin) heom::fail(HEOM_E_ARG, "invalid spin-orbital");
        if (m->cf_iorbs != iorbs || m->cf_ispin != ispin) build_cf_pattern(*m, iorbs, ispin);
        *out = heom_cf_tables{};
        out->iorbs = iorbs; out->ispin = ispin;
        out->lunkcf_spa = m->cf_lunk;
        out->nnzcf_spa = m->cf_nnz.data(); out->indcf_spa = m->cf_ind.data();
        out->irowcf_spa = m->cf_irow.data(); out->icolcf_spa = m->cf_icol.data();
    });
}

const heom_tables *heom_model_tables(const heom_model *m) { return m ? &m->view : nullptr; }

int heom_model_initial_guess(const heom_model *m, double _Complex *rho) {
    return heom::guarded([&] {
        if (!m || !rho) heom::fail(HEOM_E_ARG, "null argument");
        int n = m->nrho, n2 = 2 * n;
        std::vector<double> a((size_t)n2 * n2), w, v;
        for (int j = 0; j < n; j++)
            for (int i = 0; i < n; i++) {
                cd h = m->hs[(size_t)i + (size_t)j * n];
                a[i + (size_t)j * n2] = h.real(); a[(i + n) + (size_t)(j + n) * n2] = h.real();
                a[(i + n) + (size_t)j * n2] = h.imag(); a[i + (size_t)(j + n) * n2] = -h.imag();
            }
        sym_eig(n2, a, w, v);
        double emin = *std::min_element(w.begin(), w.end()), T = m->p.temperature[0];
        std::vector<cd> r((size_t)n * n);
        for (int k = 0; k < n2; k++) {
            double f = std::exp(-(w[k] - emin) * heom::kHbar / T);
            for (int j = 0; j < n; j++)
                for (int i = 0; i < n; i++)
                    r[i + (size_t)j * n] += f * cd(v[i + (size_t)k * n2] * v[j + (size_t)k * n2], v[(i + n) + (size_t)k * n2] * v[j + (size_t)k * n2]);
        }
        double tr = 0;
        for (int i = 0; i < n; i++) tr += r[i + (size_t)i * n].real();
        cd *out = reinterpret_cast<cd *>(rho);
        std::fill(out, out + m->lunk, cd(0, 0));
        for (int q = 0; q < m->nnz_spa[0]; q++) out[q] = r[(m->irow_spa[q] - 1) + (size_t)(m->icol_spa[q] - 1) * n] / tr;
    });
}

int heom_model_field(const heom_model *m, double *amps, double *tchar) {
    return heom::guarded([&] {
        if (!m) heom::fail(HEOM_E_ARG, "null model");
        if (amps) std::copy(m->amps.begin(), m->amps.end(), amps);
        if (tchar) std::copy(m->tcharv.begin(), m->tcharv.end(), tchar);
    });
}

int heom_model_get(const heom_model *m, const char *name, void *dst) {
    return heom::guarded([&] {
        if (!m || !name || !dst) heom::fail(HEOM_E_ARG, "null argument");
        std::string k(name);
        auto cp = [&](const void *src, size_t bytes) { std::memcpy(dst, src, bytes); };
        if (k == "hs") cp(m->hs.data(), m->hs.size() * sizeof(cd));
        else if (k == "dhs_deps") cp(m->dhs_deps.data(), m->dhs_deps.size() * sizeof(cd));
        else if (k == "dhs_du") cp(m->dhs_du.data(), m->dhs_du.size() * sizeof(cd));
        else if (k == "cpcoef") cp(m->cpcoef.data(), m->cpcoef.size() * sizeof(double));
        else if (k == "cppole") cp(m->cppole.data(), m->cppole.size() * sizeof(cd));
        else if (k == "amsori") cp(m->amsori.data(), m->amsori.size() * sizeof(double));
        else heom::fail(HEOM_E_ARG, "unknown model quantity: " + k);
    });
}

}  // extern "C"
