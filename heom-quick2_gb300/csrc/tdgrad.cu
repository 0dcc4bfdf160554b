// Gradient of a time integral of the lead current through the Chebyshev propagation
// (td/chebyshev.f90 steps on the sparse derivative), by a reverse pass with checkpoints.
//
// J(A) = dt sum_{n=0}^{N-1} I_1(rho_n), rho_{n+1} = U_n rho_n, where the lead shift of step
// n is A * amps * onset(t_n) and I_1 = Re<c, rho> is the lead-1 current.  One Chebyshev step
// is out = sum_k a_k Q_k with Q_0 = rho, Q_1 = L Q_0 / delta, Q_k = Q_{k-2} + (2/delta) L Q_{k-1}
// (a_0 = J_0, a_k = 2 J_k).  Backwards through it, with lambda = dJ/d(out):
//     mu_{K-1} = a_{K-1} lambda,  mu_k = a_k lambda + s_{k+1} L^H mu_{k+1} + mu_{k+2},
//     dJ/d rho = mu_0,   dJ/dA += sum_{j>=1} s_j Re<mu_j, (dL/dA) Q_{j-1}>,
// s_1 = 1/delta, s_j = 2/delta.  dL/dA is diagonal: i sum_k cnt_k(ado) amps_k onset_k(t).
// The forward pass stores rho every `checkpoint_every` steps; the reverse pass recomputes
// the states of one segment from its checkpoint, then walks it backwards.  The vectors and
// the applies are FP64 (HEOM_PROP_CHEBYSHEV) or FP32x2 (HEOM_PROP_CHEBYSHEV_MIXED, the
// streaming updates computed in FP64 from the stored values); the coefficients, the lead
// shifts and the accumulated parameter term are FP64 in both.
#include <cmath>
#include <cstring>
#include <type_traits>
#include <vector>

#include "apply_entry.cuh"
#include "context.cuh"
#include "propagate.cuh"

namespace heom {
namespace {
constexpr int NT = 256;
int grid_for(int64_t n) { int64_t g = (n + NT - 1) / NT; return (int)(g < 1 ? 1 : (g > 4096 ? 4096 : g)); }

// a stored complex value as FP64, and back (identity for FP64)
template <typename T> struct Io;
template <> struct Io<double> {
    static __device__ __forceinline__ double2 ld(const double2 &v) { return v; }
    static __device__ __forceinline__ void st(double2 &v, double2 a) { v = a; }
};
template <> struct Io<DF> {
    static __device__ __forceinline__ double2 ld(const float4 &v)
    {
        const Num<DF>::A a = Num<DF>::load(v);
        return make_double2(Num<DF>::re(a), Num<DF>::im(a));
    }
    static __device__ __forceinline__ void st(float4 &v, double2 a) { v = Num<DF>::store(Num<DF>::from_d(a.x, a.y)); }
};

// Q_k = (first ? 0 : Q_{k-2}) + s lq
template <typename T>
__global__ void k_qstep(int64_t n, const typename Num<T>::V *qm2, const typename Num<T>::V *lq, typename Num<T>::V *q,
                        double s, int first)
{
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const double2 l = Io<T>::ld(lq[i]);
        const double2 b = first ? make_double2(0, 0) : Io<T>::ld(qm2[i]);
        Io<T>::st(q[i], make_double2(b.x + s * l.x, b.y + s * l.y));
    }
}

// mu_j = a lam + s_next lh + mu_{j+2} (terms present when the pointers are non-null), then
// acc[e] += s_j d_e Re(conj(mu_j) i Q_{j-1}) with d_e = sum_k cnt_k es_k (when qprev != null)
template <typename T>
__global__ void k_mu(int64_t n, const DevPlan P, const double *es, const typename Num<T>::V *lam, double a,
                     const typename Num<T>::V *lh, double s_next, const typename Num<T>::V *mu2, typename Num<T>::V *mu,
                     const typename Num<T>::V *qprev, double s_j, double *acc)
{
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const double2 l = Io<T>::ld(lam[i]);
        double2 m = make_double2(a * l.x, a * l.y);
        if (lh) { const double2 h = Io<T>::ld(lh[i]); m.x += s_next * h.x; m.y += s_next * h.y; }
        if (mu2) { const double2 u = Io<T>::ld(mu2[i]); m.x += u.x; m.y += u.y; }
        Io<T>::st(mu[i], m);
        if (qprev) {
            const unsigned cnt = (unsigned)P.ado_cnt[P.ent_ado[i]];
            double d = 0;
            for (int k = 0; k < 4; k++) d += (double)(int8_t)(cnt >> (8 * k)) * es[k];
            const double2 q = Io<T>::ld(qprev[i]);
            // Re(conj(m) * i q) = m.x * (-q.y) + m.y * q.x
            acc[i] += s_j * d * (m.y * q.x - m.x * q.y);
        }
    }
}

// lam = dt c + mu0
template <typename T>
__global__ void k_lambda(int64_t n, const typename Num<T>::V *c, double dt, const typename Num<T>::V *mu0,
                         typename Num<T>::V *lam)
{
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const double2 cc = Io<T>::ld(c[i]), m = Io<T>::ld(mu0[i]);
        Io<T>::st(lam[i], make_double2(dt * cc.x + m.x, dt * cc.y + m.y));
    }
}

__global__ void k_set_step(PropClock *clk, int64_t n) { clk->n = n; }

// Terms with the apply fused in (one kernel per term, no round trip of the applied vector
// through memory).  In FP32x2 the applied value is renormalised in registers, as its store
// and reload would be, and then read as FP64 like the stored values.  In FP64 the threads
// take the entries in the plan's work-profile order, as the FP64 apply does.
template <typename T> __device__ __forceinline__ double2 applied(const typename Num<T>::A &a);
template <> __device__ __forceinline__ double2 applied<double>(const double2 &a) { return a; }
template <> __device__ __forceinline__ double2 applied<DF>(const f2c &a)
{
    const Num<DF>::A v = Num<DF>::norm(a);
    return make_double2(Num<DF>::re(v), Num<DF>::im(v));
}
template <typename T> __device__ __forceinline__ int64_t term_entry(const DevPlan &P, int64_t tid)
{
    return (std::is_same<T, double>::value && P.order) ? (int64_t)__ldg(P.order + tid) : tid;
}

// One term of a Chebyshev step with its Q kept, the apply fused in: Q_k = (first ? 0 :
// Q_{k-2}) + s L Q_{k-1} and out = (first ? c0 Q_0 : out) + c Q_k (the arithmetic of the
// propagation step); src = Q_{k-1}
template <typename T>
__global__ void __launch_bounds__(256, 6) k_qcheb_apply(DevPlan P, DevCoef<T> C, const typename Num<T>::V *__restrict__ src,
                                                     const typename Num<T>::V *q0, const typename Num<T>::V *qm2,
                                                     typename Num<T>::V *q, typename Num<T>::V *out, double s, double c,
                                                     int first, double c0)
{
    const int64_t tid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (tid >= P.lunk) return;
    const int64_t i = term_entry<T>(P, tid);
    const double2 l = applied<T>(apply_entry<T, false, false>(P, C, src, i, 0));
    double2 v;
    if (first) v = make_double2(s * l.x, s * l.y);
    else { const double2 p = Io<T>::ld(qm2[i]); v = make_double2(p.x + s * l.x, p.y + s * l.y); }
    Io<T>::st(q[i], v);
    double2 r;
    if (first) { const double2 z = Io<T>::ld(q0[i]); r = make_double2(c0 * z.x, c0 * z.y); }
    else r = Io<T>::ld(out[i]);
    Io<T>::st(out[i], make_double2(r.x + c * v.x, r.y + c * v.y));
}

// k_mu with lh = L^H src (src = mu_{j+1}, the adjoint plan PA)
template <typename T>
__global__ void __launch_bounds__(256, 6) k_mu_apply(DevPlan PA, DevCoef<T> CA, const typename Num<T>::V *__restrict__ src,
                                                  const DevPlan P, const double *es, const typename Num<T>::V *lam, double a,
                                                  double s_next, const typename Num<T>::V *mu2, typename Num<T>::V *mu,
                                                  const typename Num<T>::V *qprev, double s_j, double *acc)
{
    const int64_t tid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (tid >= P.lunk) return;
    const int64_t i = term_entry<T>(PA, tid);
    const double2 h = applied<T>(apply_entry<T, true, false>(PA, CA, src, i, 0));
    const double2 l = Io<T>::ld(lam[i]);
    double2 m = make_double2(a * l.x, a * l.y);
    m.x += s_next * h.x; m.y += s_next * h.y;
    if (mu2) { const double2 u = Io<T>::ld(mu2[i]); m.x += u.x; m.y += u.y; }
    Io<T>::st(mu[i], m);
    if (qprev) {
        const unsigned cnt = (unsigned)P.ado_cnt[P.ent_ado[i]];
        double d = 0;
        for (int k = 0; k < 4; k++) d += (double)(int8_t)(cnt >> (8 * k)) * es[k];
        const double2 q = Io<T>::ld(qprev[i]);
        acc[i] += s_j * d * (m.y * q.x - m.x * q.y);
    }
}

template <typename T>
__global__ void k_from_host_d(int64_t n, const double2 *a, typename Num<T>::V *o)
{
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        Io<T>::st(o[i], a[i]);
}

__global__ void k_sum(int64_t n, const double *a, double *out)
{
    __shared__ double red[NT];
    double s = 0;
    for (int64_t i = threadIdx.x; i < n; i += NT) s += a[i];
    red[threadIdx.x] = s;
    __syncthreads();
    for (int w = NT / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) *out = red[0];
}

template <typename T> DevCoef<T> pick(const CoefSet &K);
template <> DevCoef<double> pick<double>(const CoefSet &K) { return K.k64; }
template <> DevCoef<DF> pick<DF>(const CoefSet &K) { return K.kdf; }

// J and dJ/dA with vectors and applies in the number type T
template <typename T>
void td_gradient_run(heom_ctx *c, double dt, int nstep, int ck, const double _Complex *rho0, double *integral,
                     double *dintegral)
{
    using V = typename Num<T>::V;
    const int64_t N = c->lunk + 1, L = c->lunk;
    const int ns = c->nalf * c->nspin;
    const double delta = cheby_width(c);
    if (!(delta > 0)) fail(HEOM_E_ARG, "Chebyshev propagation needs a nonzero spectral width");
    const int K = std::max(2, cheby_terms(delta, dt, 1e-21));
    std::vector<double> bes(K);
    for (int k = 0; k < K; k++) bes[k] = bessel_j(k, delta * dt);
    const int ncp = (nstep + ck - 1) / ck;
    // buffers: 5 FP64 propagation vectors (FP64 forward steps) and the stage data; in T:
    // checkpoints, one segment of states, Q_0..Q_{K-1}, 3 mu, lambda, L^H output, the current
    // functional, the forward state and recurrence (FP32x2 forward steps); the per-entry
    // accumulator in FP64
    PropBuffers B(c, 5, (int64_t)nstep * ns);
    B.dt = dt;
    std::vector<void *> blocks;
    auto dalloc = [&](size_t bytes) { void *p = nullptr; CK(cudaMalloc(&p, bytes)); blocks.push_back(p); CK(cudaMemsetAsync(p, 0, bytes, c->stream)); return p; };
    try {
        const size_t vb = sizeof(V) * (size_t)N;
        const size_t nd = (size_t)std::max<int32_t>(1, std::max(c->dfwd.view.nado, c->dadj.view.nado));
        char *cps = (char *)dalloc(vb * ncp);
        char *seg = (char *)dalloc(vb * (ck + 1));
        char *qs = (char *)dalloc(vb * K);
        V *mu[3] = {(V *)dalloc(vb), (V *)dalloc(vb), (V *)dalloc(vb)};
        V *lam = (V *)dalloc(vb), *lh = (V *)dalloc(vb), *cv = (V *)dalloc(vb);
        V *x = (V *)dalloc(vb), *xv[3] = {(V *)dalloc(vb), (V *)dalloc(vb), (V *)dalloc(vb)};
        V *gdT = (V *)dalloc(sizeof(V) * nd), *gdaT = (V *)dalloc(sizeof(V) * nd);
        double *acc = (double *)dalloc(sizeof(double) * N);
        double *dsum = (double *)dalloc(sizeof(double));
        double2 *stage = (double2 *)dalloc(sizeof(double2) * N);
        auto cp = [&](int i) { return (V *)(cps + vb * i); };
        auto st = [&](int i) { return (V *)(seg + vb * i); };
        auto Q = [&](int k) { return (V *)(qs + vb * k); };
        cudaStream_t s = c->stream;
        const int gL = grid_for(L);
        const unsigned gA = (unsigned)((L + NT - 1) / NT);   // one thread per entry (the fused applies)
        std::vector<cd> ch(N, 0.0);
        for (const CurrentTerm &tm : c->cur_terms)
            if (tm.slot % c->nalf == 0) ch[tm.entry] += cd(0.0, -2.0 * kJconst * tm.sign);
        CK(cudaMemcpyAsync(stage, ch.data(), sizeof(double2) * N, cudaMemcpyHostToDevice, s));
        k_from_host_d<T><<<gL, NT, 0, s>>>(N, stage, cv);
        CK(cudaMemcpyAsync(stage, rho0, sizeof(double2) * L, cudaMemcpyHostToDevice, s));
        k_from_host_d<T><<<gL, NT, 0, s>>>(L, stage, x);
        PropClock h;
        prop_clock_init(c, h, 0.0, dt, 1.0);
        CK(cudaMemcpyAsync(B.clk, &h, sizeof(h), cudaMemcpyHostToDevice, s));
        const CoefSet Kf = ctx_coefs(c, false), Ka = ctx_coefs(c, true);
        // forward pass: checkpoints and currents
        {
            cudaGraph_t g = nullptr;
            cudaGraphExec_t ge = nullptr;
            {
                const CapturedGraph cg = capture_graph(s, [&] {
                    if constexpr (std::is_same<T, double>::value) enqueue_step(c, HEOM_PROP_CHEBYSHEV, Kf.k64, B, x, delta, bes, true);
                    else enqueue_step_df(c, Kf.kdf, B, x, xv, gdT, delta, bes, true);
                });
                g = cg.graph;
                ge = cg.exec;
            }
            cudaError_t err = cudaSuccess;
            for (int n = 0; n < nstep && err == cudaSuccess; n++) {
                if (n % ck == 0) err = cudaMemcpyAsync(cp(n / ck), x, vb, cudaMemcpyDeviceToDevice, s);
                if (err == cudaSuccess) err = cudaGraphLaunch(ge, s);
            }
            cudaGraphExecDestroy(ge);
            cudaGraphDestroy(g);
            CK(err);
        }
        std::vector<double> jt((size_t)nstep * ns);
        CK(cudaMemcpyAsync(jt.data(), B.jt, sizeof(double) * jt.size(), cudaMemcpyDeviceToHost, s));
        CK(cudaStreamSynchronize(s));
        double J = 0;
        for (int n = 0; n < nstep; n++)
            for (int k = 0; k < ns; k++)
                if (k % c->nalf == 0) J += dt * jt[(size_t)n * ns + k];
        *integral = J;
        // reverse pass
        const DevPlan &P = c->dfwd.view, &PA = c->dadj.view;
        DevCoef<T> KF = pick<T>(Kf), KA = pick<T>(Ka);
        KF.trace_on = 0; KA.trace_on = 0;
        KF.eshift = B.es; KA.eshift = B.es;
        // the step's lead shifts (stage_prepare) and ADO diagonals of both plans in T
        auto prepare = [&](bool adj) {
            stage_prepare(c, B, 0.0, false, s);
            fill_gdiag<T>(P, KF, gdT, 1, s);
            if (adj) fill_gdiag<T>(PA, KA, gdaT, 1, s);
        };
        // when a segment's Q_k (K ck vectors) fit in half the free device memory, the
        // recomputation of the segment keeps them, and the backward walk reuses them
        // instead of rebuilding them (K - 1 fewer applies per step)
        size_t mem_free = 0, mem_total = 0;
        CK(cudaMemGetInfo(&mem_free, &mem_total));
        char *qseg = nullptr;
        if ((double)vb * K * ck <= 0.5 * (double)mem_free) qseg = (char *)dalloc(vb * (size_t)K * ck);
        auto QS = [&](int i, int k) { return (V *)(qseg + vb * ((size_t)i * K + k)); };
        for (int sg = ncp - 1; sg >= 0; sg--) {
            const int n0 = sg * ck, n1 = std::min(nstep, n0 + ck);
            // recompute rho_{n0} .. rho_{n1-1} (and keep every step's Q_k when qseg is there)
            CK(cudaMemcpyAsync(st(0), cp(sg), vb, cudaMemcpyDeviceToDevice, s));
            for (int n = n0; n < (qseg ? n1 : n1 - 1); n++) {
                k_set_step<<<1, 1, 0, s>>>(B.clk, n);
                prepare(false);
                auto Qk = [&](int k) { return qseg ? QS(n - n0, k) : Q(k); };
                CK(cudaMemcpyAsync(Qk(0), st(n - n0), vb, cudaMemcpyDeviceToDevice, s));
                for (int k = 1; k < K; k++) {
                    k_qcheb_apply<T><<<gA, NT, 0, s>>>(P, KF, Qk(k - 1), Qk(0), k >= 2 ? Qk(k - 2) : nullptr, Qk(k), x,
                                                       k == 1 ? 1.0 / delta : 2.0 / delta, 2.0 * bes[k], k == 1, bes[0]);
                }
                if (n < n1 - 1) CK(cudaMemcpyAsync(st(n - n0 + 1), x, vb, cudaMemcpyDeviceToDevice, s));
            }
            for (int n = n1 - 1; n >= n0; n--) {
                k_set_step<<<1, 1, 0, s>>>(B.clk, n);
                prepare(true);
                // Q_0 = rho_n, Q_1 = L Q_0 / delta, Q_k = Q_{k-2} + (2/delta) L Q_{k-1} (kept, or rebuilt)
                auto Qn = [&](int k) { return qseg ? QS(n - n0, k) : Q(k); };
                if (!qseg) {
                    CK(cudaMemcpyAsync(Q(0), st(n - n0), vb, cudaMemcpyDeviceToDevice, s));
                    for (int k = 1; k < K; k++) {
                        launch_apply<T, false>(P, KF, Q(k - 1), lh, 1, N, nullptr, s);
                        k_qstep<T><<<gL, NT, 0, s>>>(L, k >= 2 ? Q(k - 2) : nullptr, lh, Q(k), k == 1 ? 1.0 / delta : 2.0 / delta, k == 1);
                    }
                }
                // mu recurrence, lambda = dJ/d rho_{n+1} (zero at n = nstep - 1)
                const V *m2 = nullptr, *m1 = nullptr;
                int slot = 0;
                for (int j = K - 1; j >= 0; j--) {
                    V *mj = mu[slot];
                    slot = (slot + 1) % 3;
                    const double a = j == 0 ? bes[0] : 2.0 * bes[j];
                    const double s_next = (j + 1 == 1) ? 1.0 / delta : 2.0 / delta;
                    const V *qp = j >= 1 ? Qn(j - 1) : nullptr;
                    const double sj = j == 1 ? 1.0 / delta : 2.0 / delta;
                    if (m1) k_mu_apply<T><<<gA, NT, 0, s>>>(PA, KA, m1, P, B.es, lam, a, s_next, m2, mj, qp, sj, acc);
                    else k_mu<T><<<gL, NT, 0, s>>>(L, P, B.es, lam, a, nullptr, s_next, m2, mj, qp, sj, acc);
                    m2 = m1;
                    m1 = mj;
                }
                k_lambda<T><<<gL, NT, 0, s>>>(L, cv, dt, m1, lam);
            }
            CK(cudaGetLastError());
        }
        k_sum<<<1, NT, 0, s>>>(L, acc, dsum);
        double dJ = 0;
        CK(cudaMemcpyAsync(&dJ, dsum, sizeof(double), cudaMemcpyDeviceToHost, s));
        CK(cudaStreamSynchronize(s));
        *dintegral = dJ;
        for (void *p : blocks) cudaFree(p);
    } catch (...) { for (void *p : blocks) cudaFree(p); throw; }
}
}  // namespace
}  // namespace heom

using namespace heom;

extern "C" int heom_td_gradient_ex(heom_ctx *c, int32_t method, double dt, int32_t nstep, int32_t checkpoint_every,
                                   const double _Complex *rho0, double *integral, double *dintegral)
{
    return guarded([&] {
        require_ctx(c);
        if (!rho0 || !integral || !dintegral || nstep < 1 || !(dt > 0)) fail(HEOM_E_ARG, "bad arguments");
        if (!c->has_adj) fail(HEOM_E_ARG, "the context was created without the adjoint plan");
        if (method != HEOM_PROP_CHEBYSHEV && method != HEOM_PROP_CHEBYSHEV_MIXED)
            fail(HEOM_E_ARG, "the gradient runs through HEOM_PROP_CHEBYSHEV or HEOM_PROP_CHEBYSHEV_MIXED steps");
        DeviceScope dsc(c->device);
        const int ck = checkpoint_every > 0 ? checkpoint_every : 32;
        if (method == HEOM_PROP_CHEBYSHEV) td_gradient_run<double>(c, dt, nstep, ck, rho0, integral, dintegral);
        else td_gradient_run<DF>(c, dt, nstep, ck, rho0, integral, dintegral);
    });
}

extern "C" int heom_td_gradient(heom_ctx *c, double dt, int32_t nstep, int32_t checkpoint_every,
                                const double _Complex *rho0, double *integral, double *dintegral)
{
    return heom_td_gradient_ex(c, HEOM_PROP_CHEBYSHEV, dt, nstep, checkpoint_every, rho0, integral, dintegral);
}
