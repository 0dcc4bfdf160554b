// Steady-state sensitivities of the lead current by the adjoint method.
//
// The steady state solves A x = e_trace (calc_ax_tfqmr_spa_omp.f90 with the Tr rho0 row).
// A is singular: its null space holds the free trace unknown x[lunk] and anti-Hermitian
// stationary RDO directions.  The physical solution has a Hermitian RDO block and
// x[lunk] = 0, and on that subspace A equals the regularised operator A~ of the
// mixed-precision solver, which is nonsingular.  Parameter derivatives keep x on the
// subspace, so
//     dI/dtheta = -Re< lambda, (dA/dtheta) x >,   A~^H lambda = c,
// with c the current functional I = Re<c, x> (td/calcj.f90:40-85).  A~^H is the adjoint
// apply (the transpose that bicg/calc_atrx_bicg_omp.f90 defines, in the sparse layout)
// followed by the adjoint of the regularising blocks (k_reg_adjoint below).
#include <cmath>
#include <cstring>
#include <vector>

#include "context.cuh"
#include "plan.h"

namespace heom {

namespace {
constexpr int NT = 256;

// z = P_H z + s P_A y on the RDO block; z[lunk] = (s / ndiag) sum_diag Re y + i s Im y[lunk].
// P_H / P_A: Hermitian / anti-Hermitian part of the RDO block.  One block per instance; the
// few RDO entries are combined in FP64 whatever the vectors' number type.
template <typename T>
__global__ void k_reg_adjoint(const typename Num<T>::V *y, typename Num<T>::V *z, int64_t vstride, int64_t lunk, int nz0,
                              int ndiag, const int32_t *pair, double s, const int *active)
{
    using N = Num<T>;
    const int b = blockIdx.x;
    if (active && !active[b]) return;
    y += (int64_t)b * vstride;
    z += (int64_t)b * vstride;
    auto ld = [](const typename N::V &v) { const typename N::A a = N::load(v); return make_double2(N::re(a), N::im(a)); };
    auto st = [](typename N::V &v, double re, double im) { v = N::store(N::from_d(re, im)); };
    __shared__ double red[NT];
    double dsum = 0;
    for (int q = threadIdx.x; q < nz0; q += NT) {
        const int p = pair[q];
        if (p < q) continue;
        const double2 zq = ld(z[q]), zp = ld(z[p]), yq = ld(y[q]), yp = ld(y[p]);
        if (p == q) {
            st(z[q], zq.x, s * yq.y);   // Hermitian part keeps Re, anti-Hermitian part is i Im
            dsum += yq.x;
            continue;
        }
        // Hermitian part of (zq, zp) plus s times the anti-Hermitian part of (yq, yp)
        const double hx = 0.5 * (zq.x + zp.x), hy = 0.5 * (zq.y - zp.y);
        const double ax = 0.5 * (yq.x - yp.x), ay = 0.5 * (yq.y + yp.y);
        st(z[q], hx + s * ax, hy + s * ay);
        st(z[p], hx - s * ax, -hy + s * ay);
    }
    red[threadIdx.x] = dsum;
    __syncthreads();
    for (int w = NT / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) st(z[lunk], s * red[0] / ndiag, s * ld(y[lunk]).y);
}

__global__ void k_fill(double2 *x, int64_t n, double2 v)
{
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) x[i] = v;
}

int grid_for(int64_t n) { int64_t g = (n + NT - 1) / NT; return (int)(g < 1 ? 1 : (g > 4096 ? 4096 : g)); }
}  // namespace

// y = A~^H x for one instance (device, in the number type T).
template <typename T>
ApplyFn<T> regularised_adjoint(heom_ctx *c, const DevCoef<T> &Kadj)
{
    const DevPlan P = c->dadj.view;
    cudaStream_t s = c->stream;
    const int64_t N = c->lunk + 1, lunk = c->lunk;
    const int nz0 = c->nz0, ndiag = c->ndiag;
    const int32_t *pair = c->d_rdo_pair;
    const double sc = c->reg_scale;
    return [=](const typename Num<T>::V *x, typename Num<T>::V *y, const int *act) {
        launch_apply<T, true>(P, Kadj, x, y, 1, N, act, s);
        k_reg_adjoint<T><<<1, NT, 0, s>>>(x, y, N, lunk, nz0, ndiag, pair, sc, act);
    };
}

// Mixed-precision solve of A~^H x = rhs for one instance (solve_custom_mixed) with the
// adjoint plan's ADO diagonals precomputed, so that the FP32x2 applies do no FP64 arithmetic.
void solve_adjoint_mixed(heom_ctx *c, const DevCoef<double> &K64, const DevCoef<DF> &KDF, const double2 *rhs, double2 *x,
                         double crit_abs, int maxit0, heom_solve_info &info)
{
    float4 *gd = nullptr;
    CK(cudaMalloc((void **)&gd, sizeof(float4) * gdiag_elems<DF>(c->dadj.view, 1)));
    try {
        DevCoef<DF> KD = KDF;
        fill_gdiag<DF>(c->dadj.view, KD, gd, 1, c->stream);
        solve_custom_mixed(c, regularised_adjoint<double>(c, K64), regularised_adjoint<DF>(c, KD), rhs, x, crit_abs, maxit0, info);
    } catch (...) { cudaFree(gd); throw; }
    cudaFree(gd);
}

// Re<a, b> over n complex entries (device vectors, result on the host).
double device_rdot(heom_ctx *c, int64_t n, const double2 *a, const double2 *b);

}  // namespace heom

using namespace heom;

extern "C" int heom_steady_gradient(heom_ctx *c, const heom_grad_opts *o, const double _Complex *rho, int32_t which,
                                    double *dI, heom_solve_info *info)
{
    return guarded([&] {
        require_ctx(c);
        if (!o || !rho || !dI) fail(HEOM_E_ARG, "null argument");
        if (!c->has_adj) fail(HEOM_E_ARG, "the context was created without the adjoint plan");
        DeviceScope dsc(c->device);
        const int64_t N = c->lunk + 1;
        std::vector<void *> blocks;
        auto dalloc2 = [&](int64_t n) { void *p = nullptr; CK(cudaMalloc(&p, sizeof(double2) * n)); blocks.push_back(p); return (double2 *)p; };
        try {
            double2 *x = dalloc2(N), *cvec = dalloc2(N), *lam = dalloc2(N), *dax = dalloc2(N);
            // x = [rho, 0]; the physical steady state has a Hermitian RDO block
            std::vector<cd> xh(N, 0.0);
            std::memcpy(xh.data(), rho, sizeof(cd) * c->lunk);
            herm_rdo(c, xh.data());
            CK(cudaMemcpyAsync(x, xh.data(), sizeof(cd) * N, cudaMemcpyHostToDevice, c->stream));
            // current functional of lead 1: I = sum_s jt(1, s) = Re<c, x>, c_e = -2 i jconst sign
            std::vector<cd> ch(N, 0.0);
            for (const CurrentTerm &tm : c->cur_terms)
                if (tm.slot % c->nalf == 0) ch[tm.entry] += cd(0.0, -2.0 * kJconst * tm.sign);
            CK(cudaMemcpyAsync(cvec, ch.data(), sizeof(cd) * N, cudaMemcpyHostToDevice, c->stream));
            k_fill<<<grid_for(N), NT, 0, c->stream>>>(lam, N, make_double2(0, 0));
            // adjoint solve A~^H lambda = c
            double cn = 0;
            for (const cd &v : ch) cn += std::norm(v);
            cn = std::sqrt(cn);
            const double crit = (o->crit > 0 ? o->crit : 1e-10) * cn;
            heom_solve_info inf{};
            const CoefSet KA = ctx_coefs(c, true);
            if (o->precision == HEOM_PREC_MIXED)
                solve_adjoint_mixed(c, KA.k64, KA.kdf, cvec, lam, crit, o->maxit0 > 0 ? o->maxit0 : 20000, inf);
            else if (o->precision == HEOM_PREC_FP64)
                solve_custom64(c, regularised_adjoint<double>(c, KA.k64), cvec, lam, crit, o->maxit0 > 0 ? o->maxit0 : 20000, inf);
            else fail(HEOM_E_ARG, "adjoint solve precision must be HEOM_PREC_FP64 or HEOM_PREC_MIXED");
            if (info) *info = inf;
            if (!inf.converged) fail(HEOM_E_NOCONV, "adjoint solve did not converge");
            // (dA/dtheta) x for the parameters asked for
            for (int k = 0; k < 4; k++) dI[k] = 0.0;
            const DevCoef<double> base = ctx_coefs(c, false).k64;
            std::vector<void *> dblocks;
            auto upload = [&](const void *h, size_t bytes) { void *p = nullptr; CK(cudaMalloc(&p, bytes)); blocks.push_back(p); CK(cudaMemcpyAsync(p, h, bytes, cudaMemcpyHostToDevice, c->stream)); return p; };
            const size_t nh = c->hst.rows.size();
            const std::vector<double2> zeros_h(std::max<size_t>(nh, 1), make_double2(0, 0));
            const std::vector<double2> zc(std::max<size_t>(c->fwd.cl.size(), 1), make_double2(0, 0));
            const double2 *hzero = (const double2 *)upload(zeros_h.data(), sizeof(double2) * zeros_h.size());
            const double2 *czero = (const double2 *)upload(zc.data(), sizeof(double2) * zc.size());
            const double zes[4] = {0, 0, 0, 0};
            const double *eszero = (const double *)upload(zes, sizeof(zes));
            auto derivative = [&](int k) -> DevCoef<double> {
                DevCoef<double> K = base;
                K.g0_scale = 0.0;
                K.unit_on = 0;
                K.trace_on = 0;
                K.hval = hzero;
                K.eshift = eszero;
                K.cl = czero;
                K.cr = czero;
                K.h_real = 0;
                if (k == 0) {   // bias: d eshift / dV
                    if (!o->deshift) fail(HEOM_E_ARG, "deshift is needed for dI/dV");
                    double d4[4] = {0, 0, 0, 0};
                    for (int a = 0; a < c->nalf; a++)
                        for (int s = 0; s < c->nspin; s++) d4[a + s * c->nalf] = o->deshift[a + (size_t)s * c->nalf];
                    K.eshift = (const double *)upload(d4, sizeof(d4));
                } else if (k == 1) {   // linewidth: the lower-tier residues scale with Gamma
                    if (!(o->gamma > 0)) fail(HEOM_E_ARG, "gamma is needed for dI/dGamma");
                    std::vector<cd> cl, cr;
                    gamma_derivative_coefs(heom_tables{}, c->fwd, o->gamma, cl, cr);
                    std::vector<double2> l2(cl.size()), r2(cr.size());
                    for (size_t q = 0; q < cl.size(); q++) { l2[q] = make_double2(cl[q].real(), cl[q].imag()); r2[q] = make_double2(cr[q].real(), cr[q].imag()); }
                    K.cl = (const double2 *)upload(l2.data(), sizeof(double2) * std::max<size_t>(l2.size(), 1));
                    K.cr = (const double2 *)upload(r2.data(), sizeof(double2) * std::max<size_t>(r2.size(), 1));
                } else {   // U or eps: -i [dH, x] on every ADO
                    const double _Complex *dh = k == 2 ? o->dhs_du : o->dhs_deps;
                    if (!dh) fail(HEOM_E_ARG, "the H derivative is needed for dI/dU and dI/deps");
                    std::vector<double2> h64;
                    hvalues64(c, reinterpret_cast<const cd *>(dh), h64);
                    K.hval = (const double2 *)upload(h64.data(), sizeof(double2) * std::max<size_t>(h64.size(), 1));
                }
                return K;
            };
            for (int k = 0; k < 4; k++) {
                if (!(which & (1 << k))) continue;
                const DevCoef<double> K = derivative(k);
                launch_apply<double, false>(c->dfwd.view, K, x, dax, 1, N, nullptr, c->stream);
                CK(cudaGetLastError());
                dI[k] = -device_rdot(c, c->lunk, lam, dax);
            }
            CK(cudaStreamSynchronize(c->stream));
            for (void *p : blocks) cudaFree(p);
        } catch (...) { for (void *p : blocks) cudaFree(p); throw; }
    });
}
