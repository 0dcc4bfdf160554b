// Time propagation on the device: RK4 (td/intstp.f90) and Chebyshev (td/chebyshev.f90,
// td/prechebyshev.f90) over the FP64 sparse derivative apply (calcderiv_spa_omp), with
// the lead currents (td/calcj.f90) recorded at the start of every step.
//
// One step is captured once as a CUDA graph and replayed nstep times.  The lead shift of
// every stage is computed on the device from a step counter, so the captured step does
// not depend on the step index.
#include <cmath>
#include <vector>

#include "apply_entry.cuh"
#include "context.cuh"
#include "propagate.cuh"

namespace heom {

namespace {
constexpr int NT = 256;

int grid_for(int64_t n) { int64_t g = (n + NT - 1) / NT; return (int)(g < 1 ? 1 : (g > 4096 ? 4096 : g)); }

// eshift(t) of td/calcderiv_spa_omp.f90:219-223 for the step-bias / exponential-onset
// pulse: amps (1 - exp(-t / tchar)), or amps for t > 0 when tchar = 0.
__global__ void k_stage_shift(const PropClock *clk, double frac, double *es)
{
    const int k = threadIdx.x;
    if (k >= 4) return;
    const double t = clk->t0 + ((double)clk->n + frac) * clk->dt;
    const double a = clk->amp_scale * clk->amps[k], tc = clk->tchar[k];
    es[k] = tc > 0 ? a * (1.0 - exp(-t / tc)) : (t > 0 ? a : 0.0);
}

__global__ void k_advance(PropClock *clk) { clk->n += clk->dir; }

// jt(slot) = -2 Im sum sign * rho(entry) * jconst (td/calcj.f90:40-85); one block.
__global__ void k_current(const double2 *x, const CurrentTerm *terms, int nterms, int nslot, const PropClock *clk,
                          double *jt)
{
    __shared__ double part[NT][4];
    double acc[4] = {0, 0, 0, 0};
    for (int k = threadIdx.x; k < nterms; k += NT) {
        const CurrentTerm tm = terms[k];
        const double v = (double)tm.sign * x[tm.entry].y;
#pragma unroll
        for (int s = 0; s < 4; s++) acc[s] += (tm.slot == s) ? v : 0.0;
    }
    for (int s = 0; s < 4; s++) part[threadIdx.x][s] = acc[s];
    __syncthreads();
    for (int w = NT / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w)
            for (int s = 0; s < 4; s++) part[threadIdx.x][s] += part[threadIdx.x + w][s];
        __syncthreads();
    }
    if (threadIdx.x < nslot) jt[(int64_t)clk->n * nslot + threadIdx.x] = -2.0 * part[0][threadIdx.x] * kJconst;
}

// The current of an FP32x2 state (k_current on the FP64 value of every summed entry)
__global__ void k_current_df(const float4 *x, const CurrentTerm *terms, int nterms, int nslot, const PropClock *clk,
                             double *jt)
{
    __shared__ double part[NT][4];
    double acc[4] = {0, 0, 0, 0};
    for (int k = threadIdx.x; k < nterms; k += NT) {
        const CurrentTerm tm = terms[k];
        const double v = (double)tm.sign * Num<DF>::im(Num<DF>::load(x[tm.entry]));
#pragma unroll
        for (int s = 0; s < 4; s++) acc[s] += (tm.slot == s) ? v : 0.0;
    }
    for (int s = 0; s < 4; s++) part[threadIdx.x][s] = acc[s];
    __syncthreads();
    for (int w = NT / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w)
            for (int s = 0; s < 4; s++) part[threadIdx.x][s] += part[threadIdx.x + w][s];
        __syncthreads();
    }
    if (threadIdx.x < nslot) jt[(int64_t)clk->n * nslot + threadIdx.x] = -2.0 * part[0][threadIdx.x] * kJconst;
}

// One Chebyshev term in FP32x2 with the derivative apply fused in: l = A pm1, pn = pm2 + s l,
// rho += c pn (first term: l = A pm2 with pm2 the copy of rho, pn = s l, rho = c0 pm2 + c pn).
// l is renormalised as a store and reload of it would be: the terms are bit-identical to a
// separate apply followed by the update, without l's round trip through memory and one
// launch per term.
__global__ void __launch_bounds__(256, 6) k_cheb_apply_df(DevPlan P, DevCoef<DF> C, const float4 *__restrict__ src,
                                                       const float4 *__restrict__ pm2, float4 *__restrict__ pn,
                                                       float4 *__restrict__ rho, f2r s, f2r c, int first, f2r c0)
{
    using N = Num<DF>;
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P.lunk) return;
    const N::A l = N::norm(apply_entry<DF, false, false>(P, C, src, i, 0));
    const N::A p2 = N::load(pm2[i]);
    const N::A v = first ? N::scale(l, s) : N::add(p2, N::scale(l, s));
    pn[i] = N::store(v);
    const N::A r = first ? N::scale(p2, c0) : N::load(rho[i]);
    rho[i] = N::store(N::add(r, N::scale(N::norm(v), c)));
}

__global__ void k_to_df(int64_t n, const double2 *a, float4 *o)
{
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        o[i] = Num<DF>::store(Num<DF>::from_d(a[i].x, a[i].y));
}

__global__ void k_from_df(int64_t n, const float4 *a, double2 *o)
{
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const Num<DF>::A v = Num<DF>::load(a[i]);
        o[i] = make_double2(Num<DF>::re(v), Num<DF>::im(v));
    }
}

// RK4 stage update: rt = r0 + a k; acc = (first ? r0 : acc) + b k
__global__ void k_rk4(int64_t n, const double2 *r0, const double2 *k, double2 *rt, double2 *acc, double a, double b,
                      int first, int write_rt)
{
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const double2 kk = k[i], r = r0[i];
        const double2 base = first ? r : acc[i];
        acc[i] = make_double2(base.x + b * kk.x, base.y + b * kk.y);
        if (write_rt) rt[i] = make_double2(r.x + a * kk.x, r.y + a * kk.y);
    }
}

// Chebyshev term: pn = pm2 + s lp; rho += c pn  (first term: pn = s lp, rho = c0 pm2 + c pn)
__global__ void k_cheb(int64_t n, const double2 *pm2, const double2 *lp, double2 *pn, double2 *rho, double s, double c,
                       int first, double c0)
{
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const double2 l = lp[i], p2 = pm2[i];
        const double2 v = first ? make_double2(s * l.x, s * l.y) : make_double2(p2.x + s * l.x, p2.y + s * l.y);
        pn[i] = v;
        const double2 r = first ? make_double2(c0 * p2.x, c0 * p2.y) : rho[i];
        rho[i] = make_double2(r.x + c * v.x, r.y + c * v.y);
    }
}
}  // namespace

// Bessel function of the first kind J_n(x), n >= 0, by Miller's backward recurrence
// normalised with J_0 + 2 sum_k J_2k = 1 (Abramowitz & Stegun 9.1.27, 9.1.46).
double bessel_j(int n, double x)
{
    if (x == 0.0) return n == 0 ? 1.0 : 0.0;
    const double ax = std::fabs(x);
    const int top = 2 * (std::max(n, (int)ax) + 16 + (int)std::sqrt(40.0 * (n + ax + 10.0)));
    double above = 0.0, cur = 1e-300, val = 0.0, norm = 0.0;
    for (int k = top; k >= 0; k--) {
        const double below = 2.0 * (k + 1) / ax * cur - above;   // J_k from J_{k+1}, J_{k+2}
        norm += (k == 0) ? below : ((k & 1) ? 0.0 : 2.0 * below);
        if (k == n) val = below;
        above = cur;
        cur = below;
        if (std::fabs(cur) > 1e250) { cur *= 1e-250; above *= 1e-250; val *= 1e-250; norm *= 1e-250; }
    }
    double v = val / norm;
    if (x < 0 && (n & 1)) v = -v;
    return v;
}

// Spectral width of the Liouville diagonal (td/prechebyshev.f90:56-110), computed from the
// index table when the context is created.
double cheby_width(heom_ctx *c) { return c->cheby_delta; }

// Terms of the expansion: add J_n(delta dt) while |J_n| / sum_k |J_k| >= dpre
// (td/prechebyshev.f90:117-130, cheby_dpre = 1e-21).
int cheby_terms(double delta, double dt, double dpre)
{
    double s = 0.0, r = 1.0;
    int n = 0;
    while (r >= dpre && n < 100000) {
        const double b = bessel_j(n, delta * dt);
        s += std::fabs(b);
        r = std::fabs(b) / s;
        n++;
    }
    return n;
}

void stage_prepare(heom_ctx *c, PropBuffers &B, double frac, bool adj, cudaStream_t s)
{
    k_stage_shift<<<1, 32, 0, s>>>(B.clk, frac, B.es);
    DevCoef<double> K = c->dfwd.template coef<double>();
    K.eshift = B.es;
    fill_gdiag<double>(c->dfwd.view, K, B.gd, 1, s);
    if (adj) {
        DevCoef<double> KA = c->dadj.template coef<double>();
        KA.eshift = B.es;
        fill_gdiag<double>(c->dadj.view, KA, B.gda, 1, s);
    }
}

void prop_clock_init(heom_ctx *c, PropClock &h, double t0, double dt, double amp_scale)
{
    h.n = 0;
    h.dir = 1;
    h.t0 = t0;
    h.dt = dt;
    h.amp_scale = amp_scale;
    for (int k = 0; k < 4; k++) { h.amps[k] = c->amps[k]; h.tchar[k] = c->tchar[k]; }
}

PropBuffers::PropBuffers(heom_ctx *c, int nvec, int64_t njt)
{
    N = c->lunk + 1;
    // every piece starts on a 256-byte boundary; the size is the sum of the rounded pieces
    auto rounded = [](size_t b) { return (b + 255) / 256 * 256; };
    const size_t nd = (size_t)std::max<int32_t>(1, std::max(c->dfwd.view.nado, c->has_adj ? c->dadj.view.nado : 0));
    const size_t bytes = rounded(sizeof(double2) * (size_t)N) * nvec + rounded(sizeof(double) * 8) +
                         rounded(sizeof(PropClock)) + rounded(sizeof(double) * std::max<int64_t>(njt, 1)) +
                         2 * rounded(sizeof(double2) * nd);
    CK(cudaMalloc(&mem, bytes));
    char *p = (char *)mem;
    auto take = [&](size_t b) { char *q = p; p += rounded(b); return (void *)q; };
    for (int k = 0; k < nvec; k++) vec.push_back((double2 *)take(sizeof(double2) * N));
    es = (double *)take(sizeof(double) * 8);
    clk = (PropClock *)take(sizeof(PropClock));
    jt = (double *)take(sizeof(double) * std::max<int64_t>(njt, 1));
    gd = (double2 *)take(sizeof(double2) * nd);
    gda = (double2 *)take(sizeof(double2) * nd);
    CK(cudaMemsetAsync(mem, 0, bytes, c->stream));
}
PropBuffers::~PropBuffers() { if (mem) cudaFree(mem); }

// Enqueue one step (current at the start, then the step) on the context stream.
void enqueue_step(heom_ctx *c, int method, const DevCoef<double> &Kin, PropBuffers &B, double2 *rho, double delta,
                  const std::vector<double> &bes, bool record_current)
{
    const DevPlan &P = c->dfwd.view;
    DevCoef<double> K = Kin;
    K.trace_on = 0;
    K.eshift = B.es;
    K.gdiag = B.gd;   // refreshed by stage_prepare before each stage's applies
    const int64_t N = B.N, L = c->lunk;
    const int ns = c->nalf * c->nspin;
    cudaStream_t s = c->stream;
    if (record_current) k_current<<<1, NT, 0, s>>>(rho, c->d_cur_terms, c->n_cur_terms, ns, B.clk, B.jt);
    if (method == HEOM_PROP_RK4) {
        const double dt = B.dt;
        double2 *rt = B.vec[0], *k = B.vec[1], *acc = B.vec[2];
        const double fr[4] = {0.0, 0.5, 0.5, 1.0};
        const double a[4] = {dt / 2, dt / 2, dt, 0.0}, b[4] = {dt / 6, dt / 3, dt / 3, dt / 6};
        for (int st = 0; st < 4; st++) {
            stage_prepare(c, B, fr[st], false, s);
            launch_apply<double, false>(P, K, st == 0 ? rho : rt, k, 1, N, nullptr, s);
            k_rk4<<<grid_for(L), NT, 0, s>>>(L, rho, k, rt, acc, a[st], b[st], st == 0, st < 3);
        }
        CK(cudaMemcpyAsync(rho, acc, sizeof(double2) * L, cudaMemcpyDeviceToDevice, s));
    } else {
        // rho(t+dt) = J0 P0 + 2 sum_n J_n(delta dt) P_n, P1 = L P0 / delta, P_n = P_{n-2} + (2/delta) L P_{n-1}
        double2 *pm2 = B.vec[0], *pm1 = B.vec[1], *pn = B.vec[2], *lp = B.vec[3];
        stage_prepare(c, B, 0.0, false, s);
        CK(cudaMemcpyAsync(pm2, rho, sizeof(double2) * L, cudaMemcpyDeviceToDevice, s));
        launch_apply<double, false>(P, K, pm2, lp, 1, N, nullptr, s);
        k_cheb<<<grid_for(L), NT, 0, s>>>(L, pm2, lp, pm1, rho, 1.0 / delta, 2.0 * bes[1], 1, bes[0]);
        for (size_t n = 2; n < bes.size(); n++) {
            launch_apply<double, false>(P, K, pm1, lp, 1, N, nullptr, s);
            k_cheb<<<grid_for(L), NT, 0, s>>>(L, pm2, lp, pn, rho, 2.0 / delta, 2.0 * bes[n], 0, 0.0);
            double2 *t = pm2; pm2 = pm1; pm1 = pn; pn = t;
        }
    }
    k_advance<<<1, 1, 0, s>>>(B.clk);
}

// One Chebyshev step in FP32x2 (HEOM_PROP_CHEBYSHEV_MIXED): the state rho, the recurrence
// vectors v[0..3] and the applies in FP32x2; gdf receives the step's ADO diagonals.
void enqueue_step_df(heom_ctx *c, const DevCoef<DF> &Kin, PropBuffers &B, float4 *rho, float4 *const v[3], float4 *gdf,
                     double delta, const std::vector<double> &bes, bool record_current)
{
    const DevPlan &P = c->dfwd.view;
    DevCoef<DF> K = Kin;
    K.trace_on = 0;
    K.eshift = B.es;
    const int64_t L = c->lunk;
    const int ns = c->nalf * c->nspin;
    cudaStream_t s = c->stream;
    if (record_current) k_current_df<<<1, NT, 0, s>>>(rho, c->d_cur_terms, c->n_cur_terms, ns, B.clk, B.jt);
    stage_prepare(c, B, 0.0, false, s);   // the step's lead shifts in B.es
    fill_gdiag<DF>(P, K, gdf, 1, s);      // and its ADO diagonals in FP32x2 (K.gdiag = gdf)
    float4 *pm2 = v[0], *pm1 = v[1], *pn = v[2];
    const unsigned nb = (unsigned)((L + 255) / 256);
    CK(cudaMemcpyAsync(pm2, rho, sizeof(float4) * L, cudaMemcpyDeviceToDevice, s));
    k_cheb_apply_df<<<nb, 256, 0, s>>>(P, K, pm2, pm2, pm1, rho, f2r_from_d(1.0 / delta), f2r_from_d(2.0 * bes[1]), 1,
                                       f2r_from_d(bes[0]));
    for (size_t n = 2; n < bes.size(); n++) {
        k_cheb_apply_df<<<nb, 256, 0, s>>>(P, K, pm1, pm2, pn, rho, f2r_from_d(2.0 / delta), f2r_from_d(2.0 * bes[n]), 0,
                                           f2r_from_d(0.0));
        float4 *t = pm2; pm2 = pm1; pm1 = pn; pn = t;
    }
    k_advance<<<1, 1, 0, s>>>(B.clk);
}

}  // namespace heom

using namespace heom;

extern "C" {

int heom_propagate(heom_ctx *c, int32_t method, double t0, double dt, int32_t nstep, double _Complex *rho,
                   double *jt_out)
{
    return guarded([&] {
        require_ctx(c);
        if (!rho || nstep < 0 || !(dt > 0)) fail(HEOM_E_ARG, "bad propagation arguments");
        if (method != HEOM_PROP_RK4 && method != HEOM_PROP_CHEBYSHEV && method != HEOM_PROP_CHEBYSHEV_MIXED)
            fail(HEOM_E_ARG, "unknown propagation method");
        DeviceScope dsc(c->device);
        const int ns = c->nalf * c->nspin;
        PropBuffers B(c, 5, (int64_t)nstep * ns);
        B.dt = dt;
        double2 *x = B.vec[4];
        CK(cudaMemcpyAsync(x, rho, sizeof(double2) * c->lunk, cudaMemcpyHostToDevice, c->stream));
        PropClock h;
        prop_clock_init(c, h, t0, dt, 1.0);
        CK(cudaMemcpyAsync(B.clk, &h, sizeof(h), cudaMemcpyHostToDevice, c->stream));
        double delta = 0.0;
        std::vector<double> bes;
        if (method != HEOM_PROP_RK4) {
            delta = cheby_width(c);
            if (!(delta > 0)) fail(HEOM_E_ARG, "Chebyshev propagation needs a nonzero spectral width");
            const int nt = std::max(2, cheby_terms(delta, dt, 1e-21));
            for (int n = 0; n < nt; n++) bes.push_back(bessel_j(n, delta * dt));
        }
        const CoefSet K = ctx_coefs(c);
        // FP32x2 state and recurrence for HEOM_PROP_CHEBYSHEV_MIXED
        float4 *dfmem = nullptr;
        float4 *xdf = nullptr, *vdf[3] = {nullptr, nullptr, nullptr}, *gdf = nullptr;
        struct DfFree { float4 *&p; ~DfFree() { if (p) cudaFree(p); } } df_free{dfmem};
        if (method == HEOM_PROP_CHEBYSHEV_MIXED) {
            const int64_t N = c->lunk + 1, vs = (N + 63) / 64 * 64, nd = std::max<int64_t>(1, c->dfwd.view.nado);
            CK(cudaMalloc((void **)&dfmem, sizeof(float4) * (size_t)(4 * vs + nd)));
            CK(cudaMemsetAsync(dfmem, 0, sizeof(float4) * (size_t)(4 * vs + nd), c->stream));
            xdf = dfmem;
            for (int k = 0; k < 3; k++) vdf[k] = dfmem + (k + 1) * vs;
            gdf = dfmem + 4 * vs;
            k_to_df<<<grid_for(c->lunk), NT, 0, c->stream>>>(c->lunk, x, xdf);
        }
        if (nstep > 0) {
            cudaGraph_t g = nullptr;
            cudaGraphExec_t ge = nullptr;
            {
                const CapturedGraph cg = capture_graph(c->stream, [&] {
                    if (method == HEOM_PROP_CHEBYSHEV_MIXED) enqueue_step_df(c, K.kdf, B, xdf, vdf, gdf, delta, bes, true);
                    else enqueue_step(c, method, K.k64, B, x, delta, bes, true);
                });
                g = cg.graph;
                ge = cg.exec;
            }
            cudaError_t err = cudaSuccess;
            for (int n = 0; n < nstep && err == cudaSuccess; n++) err = cudaGraphLaunch(ge, c->stream);
            cudaGraphExecDestroy(ge);
            cudaGraphDestroy(g);
            CK(err);
        }
        if (method == HEOM_PROP_CHEBYSHEV_MIXED) k_from_df<<<grid_for(c->lunk), NT, 0, c->stream>>>(c->lunk, xdf, x);
        CK(cudaMemcpyAsync(rho, x, sizeof(double2) * c->lunk, cudaMemcpyDeviceToHost, c->stream));
        if (jt_out && nstep > 0)
            CK(cudaMemcpyAsync(jt_out, B.jt, sizeof(double) * (size_t)nstep * ns, cudaMemcpyDeviceToHost, c->stream));
        CK(cudaStreamSynchronize(c->stream));
        CK(cudaGetLastError());
    });
}

}  // extern "C"
