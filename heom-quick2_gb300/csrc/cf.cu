// Correlation and spectral functions in the frequency domain on GB300 (corrfunc/).
//
// The operator of calc_ax_cf_spa_omp (corrfunc/calc_ax_cf_spa_omp.f90) acts on the two
// components h, a of the unknown; build_cf_plan turns it into one plan over the entries
// [h; a], so the apply is the steady apply_entry with the CF switch (real unit pairs and
// the +-omega terms between the components).  The solves are the batched FP64 TFQMR of the
// steady path: one instance per (frequency, isgnb, isgnw), all advanced by one launch per
// operator apply.  A spectral function of nfreq frequencies is one batch of 2 nfreq solves.
#include <algorithm>
#include <cmath>
#include <memory>

#include "apply_entry.cuh"
#include "context.cuh"
#include "inner.cuh"

namespace heom {

template <typename T>
__global__ void __launch_bounds__(256, 6) k_apply_cf(DevPlan P, DevCoef<T> C, const typename Num<T>::V *__restrict__ x,
                                                  typename Num<T>::V *__restrict__ y, int64_t vstride,
                                                  const int *__restrict__ active)
{
    const int b = blockIdx.y;
    if (active && !active[b]) return;
    x += (int64_t)b * vstride;
    y += (int64_t)b * vstride;
    const int64_t tid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (tid > P.lunk) return;
    const int64_t t = (tid < P.lunk && P.order) ? (int64_t)__ldg(P.order + tid) : tid;
    y[t] = Num<T>::store(apply_entry<T, false, false, true>(P, C, x, t, b));
}

namespace {

void launch_apply_cf(const DevPlan &P, const DevCoef<double> &C, const double2 *x, double2 *y, int nbatch, int64_t vstride,
                     const int *active, cudaStream_t s)
{
    dim3 grid((unsigned)((P.lunk + 1 + 255) / 256), (unsigned)nbatch);
    k_apply_cf<double><<<grid, 256, 0, s>>>(P, C, x, y, vstride, active);
}

}  // namespace
}  // namespace heom

using namespace heom;

struct heom_cf {
    heom_ctx *ctx = nullptr;
    int device = 0;   // the context's device (destroy may run after the context is gone)
    int iorbs = 0, ispin = 0, nrho = 0;
    int64_t lunkcf = 0, nunk = 0;
    // host copies: cf pattern, steady pattern (for the right-hand sides), a_{iorbs,ispin}
    std::vector<int32_t> nnzcf, irowcf, icolcf, nnz, irow, icol;
    std::vector<int64_t> indcf, ind;
    std::vector<int32_t> rofc, cofr, srofc, scofr;   // 1-based, nrho + 1 entries
    std::vector<int32_t> ar, ac, as;                 // a entries: row, col (1-based), sign
    HostPlan plan;
    PlanDev dplan;
    double *d_omega = nullptr;
    int omega_cap = 0;
    double2 *dx = nullptr, *dy = nullptr;            // 2 lunkcf + 1 scratch vectors
    std::vector<double> rt_host;
    ~heom_cf()
    {
        dplan.release();
        if (d_omega) cudaFree(d_omega);
        if (dx) cudaFree(dx);
        if (dy) cudaFree(dy);
    }
};

namespace {

void require_cf(heom_cf *cf) { if (!cf || !cf->ctx) fail(HEOM_E_ARG, "null correlation-function context"); }

// the operator's coefficient set: FP64, lead shifts as t -> infinity (igroundsteady),
// per-instance frequencies in d_omega
DevCoef<double> cf_coef(heom_cf *cf)
{
    DevCoef<double> k = cf->dplan.coef<double>();
    k.eshift = cf->ctx->es64;
    k.h_real = cf->ctx->h_real;
    k.hval = cf->ctx->hval64;
    k.trace_on = 0;
    k.cf_omega = cf->d_omega;
    k.cf_half = cf->lunkcf;
    return k;
}

void ensure_omega(heom_cf *cf, int n)
{
    if (n <= cf->omega_cap) return;
    if (cf->d_omega) { cudaFree(cf->d_omega); cf->d_omega = nullptr; cf->omega_cap = 0; }
    CK(cudaMalloc((void **)&cf->d_omega, sizeof(double) * n));
    cf->omega_cap = n;
}

// brhoh, brhoa on the cf pattern (solve_cf_tfqmr_spa.f90:136-183), returned as the right-hand
// side -(brhoh; brhoa) of the solve (lines 185-197), 2 lunkcf entries
void cf_rhs(heom_cf *cf, const cd *rho, int isgnb, std::vector<cd> &b)
{
    const int n = cf->nrho;
    const int64_t L = cf->lunkcf;
    b.assign(2 * L, cd(0, 0));
    const bool dag_l = isgnb == 1, dag_r = isgnb != 1;
    std::vector<cd> lft((size_t)n * n), rgt((size_t)n * n);
    std::vector<int32_t> touched;
    for (int64_t u = 0; u < cf->nunk; u++) {
        if (cf->nnz[u] == 0 || cf->nnzcf[u] == 0) continue;
        const int64_t st = cf->ind[u] - 1;
        for (int q = 0; q < cf->nnz[u]; q++) {
            const int r = cf->irow[st + q], c = cf->icol[st + q];
            const cd v = rho[st + q];
            // left: op_l(a)(i, r) rho(r, c)
            int i = dag_l ? cf->cofr[r] : cf->rofc[r], sg = dag_l ? cf->scofr[r] : cf->srofc[r];
            if (i) { size_t k = (size_t)(i - 1) + (size_t)(c - 1) * n; lft[k] += (double)sg * v; touched.push_back((int32_t)k); }
            // right: rho(r, c) op_r(a)(c, j)
            int j = dag_r ? cf->rofc[c] : cf->cofr[c];
            sg = dag_r ? cf->srofc[c] : cf->scofr[c];
            if (j) { size_t k = (size_t)(r - 1) + (size_t)(j - 1) * n; rgt[k] += (double)sg * v; touched.push_back((int32_t)k); }
        }
        const int64_t sc = cf->indcf[u] - 1;
        for (int q = 0; q < cf->nnzcf[u]; q++) {
            const size_t k = (size_t)(cf->irowcf[sc + q] - 1) + (size_t)(cf->icolcf[sc + q] - 1) * n;
            b[sc + q] = -(lft[k] + rgt[k]);
            b[L + sc + q] = -(cd(0, -1) * lft[k] + cd(0, 1) * rgt[k]);
        }
        for (int32_t k : touched) lft[k] = rgt[k] = 0;
        touched.clear();
    }
}

struct CfBatchResult {
    std::vector<cd> xh0, xa0;      // per instance: the RDO block (nnzcf[0] entries) of h and a
    std::vector<double> resid;     // per instance ||b - L x||
    int iters = 0, ierr = 0;
    int64_t launches = 0;
};

// Solves L(omega_b) x_b = rhs[rid_b] from x = 0 for every instance b.
// FP64 (the reference algorithm): batched TFQMR with tolerance 1e-3 crit and the true
// residual test ||b - L x|| <= crit (solve_cf_tfqmr_spa.f90:56-60, 262-290).
// MIXED: FP64 residuals refined by fused FP32x2 inner TFQMR solves (mixed_rounds) on the
// operator itself, which has no null space for omega != 0; FP64 inner solves take over for
// instances whose round fails to halve the residual.
void cf_solve_batch(heom_cf *cf, const std::vector<double> &omega, const std::vector<int> &rid,
                    const std::vector<std::vector<cd>> &rhs, double crit, int maxit0, int precision, CfBatchResult &res,
                    int bench_reps = 0, double *bench = nullptr)
{
    heom_ctx *c = cf->ctx;
    const int nb = (int)omega.size();
    const int64_t L = cf->lunkcf, N = 2 * L + 1, vs = (N + 63) / 64 * 64;
    const int nz0 = cf->nnzcf[0];
    const int nlim = std::max(1, maxit0 / 2);
    res = CfBatchResult();
    res.xh0.assign((size_t)nb * nz0, cd(0, 0));
    res.xa0.assign((size_t)nb * nz0, cd(0, 0));
    res.resid.assign(nb, 0.0);
    ensure_omega(cf, nb);
    CK(cudaMemcpyAsync(cf->d_omega, omega.data(), sizeof(double) * nb, cudaMemcpyHostToDevice, c->stream));
    std::vector<void *> tmp;
    auto cleanup = [&] { for (void *p : tmp) cudaFree(p); tmp.clear(); };
    auto dmalloc = [&](size_t bytes) { void *p = nullptr; CK(cudaMalloc(&p, bytes)); tmp.push_back(p); return p; };
    TfqWork<double> W;
    try {
        // B: the right-hand sides, X: the solutions, R: residual scratch (stride vs)
        double2 *B = (double2 *)dmalloc(sizeof(double2) * (size_t)vs * nb);
        double2 *X = (double2 *)dmalloc(sizeof(double2) * (size_t)vs * nb);
        double2 *R = (double2 *)dmalloc(sizeof(double2) * (size_t)vs * nb);
        CK(cudaMemsetAsync(B, 0, sizeof(double2) * (size_t)vs * nb, c->stream));
        CK(cudaMemsetAsync(X, 0, sizeof(double2) * (size_t)vs * nb, c->stream));
        double2 *drhs = (double2 *)dmalloc(sizeof(double2) * (size_t)N * rhs.size());
        for (size_t k = 0; k < rhs.size(); k++)
            CK(cudaMemcpyAsync(drhs + k * N, rhs[k].data(), sizeof(double2) * 2 * L, cudaMemcpyHostToDevice, c->stream));
        for (int b = 0; b < nb; b++)
            CK(cudaMemcpyAsync(B + (int64_t)b * vs, drhs + (size_t)rid[b] * N, sizeof(double2) * 2 * L,
                               cudaMemcpyDeviceToDevice, c->stream));
        // per-instance parameter arrays (the kernels index H values and lead shifts by
        // instance): the context's single set replicated nb times
        DevCoef<double> K = cf_coef(cf);
        const DevPlan P = cf->dplan.view;
        double2 *hv = (double2 *)dmalloc(sizeof(double2) * (size_t)std::max(1, P.nh) * nb);
        double *es = (double *)dmalloc(sizeof(double) * 4 * (size_t)nb);
        double es_host[4];
        CK(cudaMemcpyAsync(es_host, c->es64, sizeof es_host, cudaMemcpyDeviceToHost, c->stream));
        CK(cudaStreamSynchronize(c->stream));
        std::vector<double> es_rep(4 * (size_t)nb);
        for (int b = 0; b < nb; b++) std::copy(es_host, es_host + 4, es_rep.begin() + 4 * (size_t)b);
        CK(cudaMemcpyAsync(es, es_rep.data(), sizeof(double) * es_rep.size(), cudaMemcpyHostToDevice, c->stream));
        for (int b = 0; b < nb; b++)
            CK(cudaMemcpyAsync(hv + (size_t)b * P.nh, c->hval64, sizeof(double2) * P.nh, cudaMemcpyDeviceToDevice, c->stream));
        CK(cudaStreamSynchronize(c->stream));
        K.hval = hv;
        K.eshift = es;
        // per-instance ADO diagonals: keeps the lead-shift sums out of the per-entry work
        double2 *gd = (double2 *)dmalloc(sizeof(double2) * (size_t)P.nado * nb);
        fill_gdiag<double>(P, K, gd, nb, c->stream);
        cudaStream_t s = c->stream;
        ApplyFn<double> op = [P, K, nb, vs, s](const double2 *x, double2 *y, const int *act) {
            launch_apply_cf(P, K, x, y, nb, vs, act, s);
        };
        // true residuals B - L X (the reference's final norm) into R and res.resid
        auto residuals = [&] {
            op(X, R, nullptr);
            vec_axpby<double>(vs * nb, R, 1.0, B, -1.0, R, c->stream);
            double worst = 0;
            for (int b = 0; b < nb; b++) {
                res.resid[b] = device_norm2(N, R + (int64_t)b * vs, c->dscratch, c->stream);
                worst = std::max(worst, res.resid[b]);
            }
            res.launches += 2 + nb;
            return worst;
        };
        if (precision == HEOM_PREC_MIXED) {
            DevCoef<DF> KD = cf->dplan.coef<DF>();
            float4 *hvd = (float4 *)dmalloc(sizeof(float4) * (size_t)std::max(1, P.nh) * nb);
            for (int b = 0; b < nb; b++)
                CK(cudaMemcpyAsync(hvd + (size_t)b * P.nh, c->hvaldf, sizeof(float4) * P.nh, cudaMemcpyDeviceToDevice, c->stream));
            KD.hval = hvd;
            KD.eshift = es;
            KD.h_real = c->h_real;
            KD.trace_on = 0;
            KD.cf_omega = cf->d_omega;
            KD.cf_half = L;
            if (bench_reps > 0) {
                // measurement: the two fused inner kernels (B: apply of w with the first half of
                // the vector updates; A: apply of v with the second half) over the batch
                InnerWork<DF> IW;
                inner_alloc<DF>(IW, nb, N, c->stream, 2, 2);   // the layout of the solves
                float4 *gdd = nullptr;
                try {
                    std::vector<float4> rt(N);
                    for (int64_t i = 0; i < N; i++)
                        rt[i] = Num<DF>::store_host(Num<DF>::from_d(cf->rt_host[2 * i], cf->rt_host[2 * i + 1]));
                    CK(cudaMemcpyAsync(IW.rt, rt.data(), sizeof(float4) * N, cudaMemcpyHostToDevice, c->stream));
                    CK(cudaMalloc((void **)&gdd, sizeof(float4) * (size_t)gdiag_elems<DF>(P, nb)));
                    fill_gdiag<DF>(P, KD, gdd, nb, c->stream);
                    // with the inner preconditioner of the mixed solves
                    float *pre = (float *)dmalloc(sizeof(float) * std::max(1, P.nado));
                    fill_pre(P, K.g0, hs_inf_norm(c), pre, c->stream);
                    KD.pre = pre;
                    CK(cudaStreamSynchronize(c->stream));
                    float mb = 0, ma = 0;
                    inner_time<DF>(IW, P, KD, bench_reps, c->stream, mb, ma);
                    const double v = (double)N * sizeof(float4), pb = plan_read_bytes(cf->plan);
                    bench[0] = mb * 1e-3;
                    bench[1] = ma * 1e-3;
                    bench[2] = nb * (2.0 + 10.0) * v + v + pb;
                    bench[3] = nb * (2.0 + 3.0) * v + v + pb;
                } catch (...) { inner_free(IW); if (gdd) cudaFree(gdd); throw; }
                inner_free(IW);
                cudaFree(gdd);
                cleanup();
                return;
            }
            heom_solve_opts mo{};
            mo.crit = crit;
            mo.maxit0 = maxit0;
            // frequencies converge at different rates: pairs of instances sharing a lane (the
            // iterates of one instance per group, the plan decoded once per pair; a pair with one
            // instance left runs it alone)
            mo.interleave = 2;
            mo.lane_instances = 2;
            std::vector<double> norms(nb, 0.0);
            std::function<void(const double2 *, double2 *)> residual = [&](const double2 *xx, double2 *r) {
                op(xx, r, nullptr);
                vec_axpby<double>(vs * nb, r, 1.0, B, -1.0, r, c->stream);
            };
            std::function<void(const double2 *)> batch_norms = [&](const double2 *v) {
                for (int b = 0; b < nb; b++) norms[b] = device_norm2(N, v + (int64_t)b * vs, c->dscratch, c->stream);
            };
            bool stalled = false, conv = false, unused = false;
            int total = 0, ierr = 0, rounds = 0, more = 0;
            int64_t aux = 0;
            mixed_rounds<DF>(c, mo, X, nb, vs, B, K, KD, R, norms, nlim, 8, true, stalled, total, ierr, conv, rounds,
                             res.launches, aux, residual, batch_norms, P, N);
            if (stalled && !conv)
                mixed_rounds<double>(c, mo, X, nb, vs, B, K, K, R, norms, nlim, 8, false, unused, total, ierr, conv, more,
                                     res.launches, aux, residual, batch_norms, P, N);
            res.iters = total;
            res.ierr = ierr;
            res.launches += aux;
            residuals();
        } else {
            tfq_alloc<double>(W, nb, N, c->stream);
            std::vector<double2> rt(N);
            for (int64_t i = 0; i < N; i++) rt[i] = make_double2(cf->rt_host[2 * i], cf->rt_host[2 * i + 1]);
            CK(cudaMemcpyAsync(W.rt, rt.data(), sizeof(double2) * N, cudaMemcpyHostToDevice, c->stream));
            ApplyFn<double> opw = [P, K, nb, s, &W](const double2 *x, double2 *y, const int *act) {
                launch_apply_cf(P, K, x, y, nb, W.vstride, act, s);
            };
            for (int b = 0; b < nb; b++)
                CK(cudaMemcpyAsync(W.b + (int64_t)b * W.vstride, B + (int64_t)b * vs, sizeof(double2) * N,
                                   cudaMemcpyDeviceToDevice, c->stream));
            // The reference runs one TFQMR and reports whatever it reached.  TFQMR can stop early
            // on an exact zero of rho or sigma (ierr 8), which happens on small hierarchies whose
            // Krylov space closes, so unconverged instances restart from their residual: every
            // round solves L d = B - L X from d = 0 and adds d to X; converged instances leave at
            // the round's first residual test.
            int total = 0;
            for (int round = 0; round < 8 && total < 2 * nlim; round++) {
                if (round > 0)
                    for (int b = 0; b < nb; b++)
                        CK(cudaMemcpyAsync(W.b + (int64_t)b * W.vstride, R + (int64_t)b * vs, sizeof(double2) * N,
                                           cudaMemcpyDeviceToDevice, c->stream));
                tfq_start<double>(W, crit * 1e-3, nlim, crit, 0.0, 0, c->stream);
                int it = 0;
                run_tfqmr64(c, W, opw, nlim, it, res.launches);
                for (int b = 0; b < nb; b++)
                    vec_axpby<double>(N, X + (int64_t)b * vs, 1.0, X + (int64_t)b * vs, 1.0, W.x + (int64_t)b * W.vstride, c->stream);
                std::vector<TfqState> st(nb);
                CK(cudaMemcpyAsync(st.data(), W.st, sizeof(TfqState) * nb, cudaMemcpyDeviceToHost, c->stream));
                CK(cudaStreamSynchronize(c->stream));
                int axb = 0;
                res.ierr = 0;   // of the last round
                for (auto &sv : st) { axb = std::max(axb, sv.axb); res.ierr = std::max(res.ierr, sv.ierr); }
                total += axb;
                res.launches += kTfqStartLaunches + 2 * nb;
                if (residuals() <= crit) break;
            }
            res.iters = total;
        }
        for (int b = 0; b < nb; b++) {
            CK(cudaMemcpyAsync(res.xh0.data() + (size_t)b * nz0, X + (int64_t)b * vs, sizeof(double2) * nz0,
                               cudaMemcpyDeviceToHost, c->stream));
            CK(cudaMemcpyAsync(res.xa0.data() + (size_t)b * nz0, X + (int64_t)b * vs + L, sizeof(double2) * nz0,
                               cudaMemcpyDeviceToHost, c->stream));
        }
        CK(cudaStreamSynchronize(c->stream));
    } catch (...) { tfq_free(W); cleanup(); throw; }
    tfq_free(W);
    cleanup();
}

// dense nrho x nrho matrix of an RDO block on the cf pattern
void rdo_dense(heom_cf *cf, const cd *x0, std::vector<cd> &out)
{
    const int n = cf->nrho;
    out.assign((size_t)n * n, cd(0, 0));
    for (int q = 0; q < cf->nnzcf[0]; q++) out[(size_t)(cf->irowcf[q] - 1) + (size_t)(cf->icolcf[q] - 1) * n] = x0[q];
}

// Tr[op(a) M] for op = a (dag = false) or a^dag
cd trace_op(heom_cf *cf, const std::vector<cd> &m, bool dag)
{
    const int n = cf->nrho;
    cd s(0, 0);
    for (size_t k = 0; k < cf->ar.size(); k++) {
        const int r = cf->ar[k] - 1, c = cf->ac[k] - 1;   // a(r, c) = sign
        // Tr[a M] = sum a(r, c) M(c, r); Tr[a^dag M] = sum a(r, c) M(r, c)
        s += (double)cf->as[k] * (dag ? m[(size_t)r + (size_t)c * n] : m[(size_t)c + (size_t)r * n]);
    }
    return s;
}

template <class F>
void timed(heom_cf *cf, heom_solve_info *info, F &&f)
{
    cudaEvent_t e0, e1;
    CK(cudaEventCreate(&e0)); CK(cudaEventCreate(&e1));
    CK(cudaEventRecord(e0, cf->ctx->stream));
    try { f(); } catch (...) { cudaEventDestroy(e0); cudaEventDestroy(e1); throw; }
    CK(cudaEventRecord(e1, cf->ctx->stream));
    CK(cudaEventSynchronize(e1));
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0); cudaEventDestroy(e1);
    if (info) info->seconds = ms * 1e-3;
}

void fill_info(const CfBatchResult &r, double crit, heom_solve_info *info)
{
    if (!info) return;
    double w = 0;
    for (double v : r.resid) w = std::max(w, v);
    info->iters = r.iters;
    info->ierr = r.ierr;
    info->refinements = 0;
    info->resid = w;
    info->converged = w <= crit;
    info->launches = r.launches;
}

// frequencies per batch: the TFQMR workspace holds ten vectors per instance
int batch_cap(heom_cf *cf)
{
    const double per = 10.0 * 16.0 * (double)(2 * cf->lunkcf + 64);
    size_t fr = 0, tot = 0;
    if (cudaMemGetInfo(&fr, &tot) != cudaSuccess) fr = (size_t)8 << 30;
    const double room = std::min(0.5 * (double)fr, 64.0 * (1ull << 30));
    return (int)std::max(2.0, std::min(256.0, std::floor(room / per)));
}

}  // namespace

extern "C" {

int heom_cf_create(heom_ctx *ctx, const heom_tables *t, const heom_cf_tables *cft, heom_cf **out)
{
    return guarded([&] {
        require_ctx(ctx);
        if (!t || !cft || !out) fail(HEOM_E_ARG, "null argument");
        *out = nullptr;
        if (t->lunk_spa != ctx->lunk || t->nunk != ctx->nunk || t->nrho != ctx->nrho)
            fail(HEOM_E_ARG, "tables do not belong to this context");
        if (cft->iorbs < 1 || cft->iorbs > t->norbs || cft->ispin < 1 || cft->ispin > t->nspin)
            fail(HEOM_E_ARG, "invalid spin-orbital");
        DeviceScope dsc(ctx->device);
        std::unique_ptr<heom_cf> cf(new heom_cf());
        cf->ctx = ctx;
        cf->device = ctx->device;
        cf->iorbs = cft->iorbs; cf->ispin = cft->ispin; cf->nrho = t->nrho;
        cf->lunkcf = cft->lunkcf_spa; cf->nunk = t->nunk;
        const int64_t nu = t->nunk, L = cft->lunkcf_spa;
        for (int64_t u = 0; u < nu; u++) {
            if (cft->nnzcf_spa[u] < 0 || cft->indcf_spa[u] < 1 || cft->indcf_spa[u] - 1 + cft->nnzcf_spa[u] > L)
                fail(HEOM_E_ARG, "nnzcf_spa / indcf_spa out of range");
        }
        cf->nnzcf.assign(cft->nnzcf_spa, cft->nnzcf_spa + nu);
        cf->indcf.assign(cft->indcf_spa, cft->indcf_spa + nu);
        cf->irowcf.assign(cft->irowcf_spa, cft->irowcf_spa + L);
        cf->icolcf.assign(cft->icolcf_spa, cft->icolcf_spa + L);
        cf->nnz.assign(t->nnz_spa, t->nnz_spa + nu);
        cf->ind.assign(t->ind_spa, t->ind_spa + nu);
        cf->irow.assign(t->irow_spa, t->irow_spa + t->lunk_spa);
        cf->icol.assign(t->icol_spa, t->icol_spa + t->lunk_spa);
        const int n = t->nrho;
        cf->rofc.assign(n + 1, 0); cf->cofr = cf->rofc; cf->srofc = cf->rofc; cf->scofr = cf->rofc;
        const size_t base = (size_t)t->nams * ((cf->iorbs - 1) + (size_t)(cf->ispin - 1) * t->norbs);
        for (int k = 0; k < t->nams; k++) {
            const int r = t->rowams[base + k], c = t->colams[base + k], sg = t->sgnams[base + k] ? -1 : 1;
            cf->rofc[c] = r; cf->srofc[c] = sg; cf->cofr[r] = c; cf->scofr[r] = sg;
            cf->ar.push_back(r); cf->ac.push_back(c); cf->as.push_back(sg);
        }
        build_cf_plan(*t, *cft, ctx->hst, cf->plan);
        cf->dplan.upload(cf->plan);
        const int64_t N = 2 * L + 1;
        CK(cudaMalloc((void **)&cf->dx, sizeof(double2) * N));
        CK(cudaMalloc((void **)&cf->dy, sizeof(double2) * N));
        CK(cudaMemsetAsync(cf->dx, 0, sizeof(double2) * N, ctx->stream));
        ensure_omega(cf.get(), 2);
        drandn_host(2 * N, cf->rt_host);
        CK(cudaDeviceSynchronize());   // the plan's pageable set-up copies, before any kernel reads them
        *out = cf.release();
    });
}

void heom_cf_destroy(heom_cf *cf)
{
    if (!cf) return;
    try { heom::DeviceScope dsc(cf->device); delete cf; } catch (...) { delete cf; }
}

int64_t heom_cf_lunk(const heom_cf *cf) { return cf ? cf->lunkcf : -1; }

int heom_cf_calc_ax(heom_cf *cf, double dfreq, int32_t isgnw, int64_t ldim, const double _Complex *rcga,
                    const double _Complex *rcgb, double _Complex *rhsa, double _Complex *rhsb)
{
    return guarded([&] {
        require_cf(cf);
        DeviceScope dsc(cf->ctx->device);
        if (ldim != cf->lunkcf) fail(HEOM_E_ARG, "ldim does not match lunkcf_spa");
        if (!rcga || !rcgb || !rhsa || !rhsb) fail(HEOM_E_ARG, "null vector");
        if (isgnw != 1 && isgnw != 2) fail(HEOM_E_ARG, "isgnw must be 1 or 2");
        heom_ctx *c = cf->ctx;
        const int64_t L = cf->lunkcf;
        const double w = isgnw == 1 ? dfreq : -dfreq;
        CK(cudaMemcpyAsync(cf->d_omega, &w, sizeof(double), cudaMemcpyHostToDevice, c->stream));
        CK(cudaMemcpyAsync(cf->dx, rcga, sizeof(double2) * L, cudaMemcpyHostToDevice, c->stream));
        CK(cudaMemcpyAsync(cf->dx + L, rcgb, sizeof(double2) * L, cudaMemcpyHostToDevice, c->stream));
        launch_apply_cf(cf->dplan.view, cf_coef(cf), cf->dx, cf->dy, 1, 2 * L + 1, nullptr, c->stream);
        CK(cudaGetLastError());
        CK(cudaMemcpyAsync(rhsa, cf->dy, sizeof(double2) * L, cudaMemcpyDeviceToHost, c->stream));
        CK(cudaMemcpyAsync(rhsb, cf->dy + L, sizeof(double2) * L, cudaMemcpyDeviceToHost, c->stream));
        CK(cudaStreamSynchronize(c->stream));
    });
}

int heom_cf_solve(heom_cf *cf, const double _Complex *rho, int32_t isgnb, int32_t isgnw, int32_t nfreq,
                  const double *dfreq, const heom_solve_opts *o, double _Complex *zouth, double _Complex *zouta,
                  heom_solve_info *info)
{
    return guarded([&] {
        require_cf(cf);
        DeviceScope dsc(cf->ctx->device);
        if (!rho || !dfreq || !o || nfreq < 1) fail(HEOM_E_ARG, "null argument or no frequency");
        if (isgnb != 1 && isgnb != 2) fail(HEOM_E_ARG, "isgnb must be 1 or 2");
        if (isgnw != 1 && isgnw != 2) fail(HEOM_E_ARG, "isgnw must be 1 or 2");
        if (o->precision != HEOM_PREC_FP64 && o->precision != HEOM_PREC_MIXED)
            fail(HEOM_E_UNSUPPORTED, "correlation-function solves run in FP64 or MIXED precision");
        if (info) *info = heom_solve_info{};
        const int n = cf->nrho, nz0 = cf->nnzcf[0];
        std::vector<std::vector<cd>> rhs(1);
        cf_rhs(cf, reinterpret_cast<const cd *>(rho), isgnb, rhs[0]);
        const int cap = batch_cap(cf);
        CfBatchResult all;
        timed(cf, info, [&] {
            for (int f0 = 0; f0 < nfreq; f0 += cap) {
                const int nb = std::min(cap, nfreq - f0);
                std::vector<double> w(nb);
                for (int k = 0; k < nb; k++) w[k] = isgnw == 1 ? dfreq[f0 + k] : -dfreq[f0 + k];
                CfBatchResult r;
                cf_solve_batch(cf, w, std::vector<int>(nb, 0), rhs, o->crit, o->maxit0, o->precision, r);
                for (int k = 0; k < nb; k++) {
                    std::vector<cd> m;
                    if (zouth) {
                        rdo_dense(cf, r.xh0.data() + (size_t)k * nz0, m);
                        std::copy(m.begin(), m.end(), reinterpret_cast<cd *>(zouth) + (size_t)(f0 + k) * n * n);
                    }
                    if (zouta) {
                        rdo_dense(cf, r.xa0.data() + (size_t)k * nz0, m);
                        std::copy(m.begin(), m.end(), reinterpret_cast<cd *>(zouta) + (size_t)(f0 + k) * n * n);
                    }
                }
                all.resid.insert(all.resid.end(), r.resid.begin(), r.resid.end());
                all.iters = std::max(all.iters, r.iters);
                all.ierr = std::max(all.ierr, r.ierr);
                all.launches += r.launches;
            }
        });
        fill_info(all, o->crit, info);
    });
}

int heom_cf_dos(heom_cf *cf, const double _Complex *rho, int32_t nfreq, const double *freq_ev, const heom_solve_opts *o,
                double *out, heom_solve_info *info)
{
    return guarded([&] {
        require_cf(cf);
        DeviceScope dsc(cf->ctx->device);
        if (!rho || !freq_ev || !o || !out || nfreq < 1) fail(HEOM_E_ARG, "null argument or no frequency");
        if (o->precision != HEOM_PREC_FP64 && o->precision != HEOM_PREC_MIXED)
            fail(HEOM_E_UNSUPPORTED, "correlation-function solves run in FP64 or MIXED precision");
        if (info) *info = heom_solve_info{};
        const int nz0 = cf->nnzcf[0];
        // instance 2k: isgnb = 2, isgnw = 2 (C_{B^dag B}); 2k+1: isgnb = 1, isgnw = 1 (C_{B B^dag})
        std::vector<std::vector<cd>> rhs(2);
        cf_rhs(cf, reinterpret_cast<const cd *>(rho), 2, rhs[0]);
        cf_rhs(cf, reinterpret_cast<const cd *>(rho), 1, rhs[1]);
        const int capf = std::max(1, batch_cap(cf) / 2);
        CfBatchResult all;
        timed(cf, info, [&] {
            for (int f0 = 0; f0 < nfreq; f0 += capf) {
                const int nf = std::min(capf, nfreq - f0);
                std::vector<double> w(2 * nf);
                std::vector<int> rid(2 * nf);
                for (int k = 0; k < nf; k++) {
                    const double wi = freq_ev[f0 + k] / kHbar;
                    w[2 * k] = -wi; rid[2 * k] = 0;
                    w[2 * k + 1] = wi; rid[2 * k + 1] = 1;
                }
                CfBatchResult r;
                cf_solve_batch(cf, w, rid, rhs, o->crit, o->maxit0, o->precision, r);
                for (int k = 0; k < nf; k++) {
                    cd tr[2];
                    for (int h = 0; h < 2; h++) {
                        const size_t b = (size_t)(2 * k + h) * nz0;
                        std::vector<cd> c5(nz0);
                        for (int q = 0; q < nz0; q++) c5[q] = 0.5 * r.xh0[b + q] + cd(0, 0.5) * r.xa0[b + q];
                        std::vector<cd> m;
                        rdo_dense(cf, c5.data(), m);
                        tr[h] = trace_op(cf, m, h == 0);
                    }
                    double *o5 = out + 5 * (size_t)(f0 + k);
                    o5[1] = tr[0].real() / kPi / kHbar;
                    o5[2] = tr[1].real() / kPi / kHbar;
                    o5[0] = o5[1] + o5[2];
                    const cd g = cd(0, -1) * (std::conj(tr[0]) + tr[1]) / kHbar;
                    o5[3] = g.real(); o5[4] = g.imag();
                }
                all.resid.insert(all.resid.end(), r.resid.begin(), r.resid.end());
                all.iters = std::max(all.iters, r.iters);
                all.ierr = std::max(all.ierr, r.ierr);
                all.launches += r.launches;
            }
        });
        fill_info(all, o->crit, info);
    });
}

int heom_cf_propagate(heom_cf *cf, const double _Complex *rho, double dt, int32_t nstep, int32_t ljw,
                      double _Complex *corr, double _Complex *rdo_h, double _Complex *rdo_a)
{
    return guarded([&] {
        require_cf(cf);
        DeviceScope dsc(cf->ctx->device);
        if (!rho || !corr || nstep < 0 || !(dt > 0)) fail(HEOM_E_ARG, "null argument, nstep < 0 or dt <= 0");
        heom_ctx *c = cf->ctx;
        const int nb = ljw ? 2 : 1, n = cf->nrho, nz0 = cf->nnzcf[0];
        const int64_t L = cf->lunkcf, N = 2 * L + 1, vs = (N + 63) / 64 * 64;
        // initial values (initialize_cf.f90:40-170, b_ams_isgn = 2): instance 0 holds B rho
        // (a rho + rho a^dag), instance 1 B^dag rho (a^dag rho + rho a); cf_rhs returns -(B rho)
        std::vector<std::vector<cd>> b0(nb);
        cf_rhs(cf, reinterpret_cast<const cd *>(rho), 2, b0[0]);
        if (ljw) cf_rhs(cf, reinterpret_cast<const cd *>(rho), 1, b0[1]);
        std::vector<void *> tmp;
        auto cleanup = [&] { for (void *p : tmp) cudaFree(p); tmp.clear(); };
        auto dmalloc = [&](size_t bytes) { void *p = nullptr; CK(cudaMalloc(&p, bytes)); tmp.push_back(p); return p; };
        try {
            const size_t vb = sizeof(double2) * (size_t)vs * nb;
            double2 *x = (double2 *)dmalloc(vb), *acc = (double2 *)dmalloc(vb), *stg = (double2 *)dmalloc(vb), *k = (double2 *)dmalloc(vb);
            double2 *hist = (double2 *)dmalloc(sizeof(double2) * 2 * (size_t)nz0 * nb * (nstep + 1));
            CK(cudaMemsetAsync(x, 0, vb, c->stream));
            for (int b = 0; b < nb; b++) {
                std::vector<cd> pos(b0[b].size());
                for (size_t q = 0; q < pos.size(); q++) pos[q] = -b0[b][q];
                CK(cudaMemcpyAsync(x + (int64_t)b * vs, pos.data(), sizeof(double2) * 2 * L, cudaMemcpyHostToDevice, c->stream));
                CK(cudaStreamSynchronize(c->stream));
            }
            // the operator without frequency terms (lfreq = F), per-instance parameter copies
            ensure_omega(cf, nb);
            const double zero[2] = {0.0, 0.0};
            CK(cudaMemcpyAsync(cf->d_omega, zero, sizeof(double) * nb, cudaMemcpyHostToDevice, c->stream));
            DevCoef<double> K = cf_coef(cf);
            const DevPlan P = cf->dplan.view;
            double2 *hv = (double2 *)dmalloc(sizeof(double2) * (size_t)std::max(1, P.nh) * nb);
            double *es = (double *)dmalloc(sizeof(double) * 4 * (size_t)nb);
            double2 *gd = (double2 *)dmalloc(sizeof(double2) * (size_t)P.nado * nb);
            for (int b = 0; b < nb; b++) {
                CK(cudaMemcpyAsync(hv + (size_t)b * P.nh, c->hval64, sizeof(double2) * P.nh, cudaMemcpyDeviceToDevice, c->stream));
                CK(cudaMemcpyAsync(es + 4 * (size_t)b, c->es64, sizeof(double) * 4, cudaMemcpyDeviceToDevice, c->stream));
            }
            K.hval = hv;
            K.eshift = es;
            fill_gdiag<double>(P, K, gd, nb, c->stream);
            K.gdiag = gd;
            const int64_t nv = vs * nb;
            auto record = [&](int step) {
                for (int b = 0; b < nb; b++)
                    for (int h = 0; h < 2; h++)
                        CK(cudaMemcpyAsync(hist + ((size_t)step * nb * 2 + (size_t)b * 2 + h) * nz0, x + (int64_t)b * vs + h * L,
                                           sizeof(double2) * nz0, cudaMemcpyDeviceToDevice, c->stream));
            };
            // classical RK4 (corrfunc.f90:430-610): x <- x + dt (k1 + 2 k2 + 2 k3 + k4) / 6
            record(0);
            for (int step = 1; step <= nstep; step++) {
                launch_apply_cf(P, K, x, k, nb, vs, nullptr, c->stream);                 // k1
                vec_axpby<double>(nv, acc, 1.0, x, dt / 6.0, k, c->stream);
                vec_axpby<double>(nv, stg, 1.0, x, dt / 2.0, k, c->stream);
                launch_apply_cf(P, K, stg, k, nb, vs, nullptr, c->stream);               // k2
                vec_axpby<double>(nv, acc, 1.0, acc, dt / 3.0, k, c->stream);
                vec_axpby<double>(nv, stg, 1.0, x, dt / 2.0, k, c->stream);
                launch_apply_cf(P, K, stg, k, nb, vs, nullptr, c->stream);               // k3
                vec_axpby<double>(nv, acc, 1.0, acc, dt / 3.0, k, c->stream);
                vec_axpby<double>(nv, stg, 1.0, x, dt, k, c->stream);
                launch_apply_cf(P, K, stg, k, nb, vs, nullptr, c->stream);               // k4
                vec_axpby<double>(nv, x, 1.0, acc, dt / 6.0, k, c->stream);
                record(step);
            }
            CK(cudaGetLastError());
            std::vector<cd> hh((size_t)2 * nz0 * nb * (nstep + 1));
            CK(cudaMemcpyAsync(hh.data(), hist, sizeof(double2) * hh.size(), cudaMemcpyDeviceToHost, c->stream));
            CK(cudaStreamSynchronize(c->stream));
            // C(t) = Tr[A (X_h + i X_a) / 2] and, with ljw, conj(Tr[A^dag (Y_h + i Y_a) / 2]) with
            // A = a^dag (a_ams_isgn = 1, initialize_cf.f90:211-217; corrfunc.f90:378-416)
            std::vector<cd> z(nz0), m;
            for (int step = 0; step <= nstep; step++) {
                for (int b = 0; b < 2; b++) {
                    cd val(0, 0);
                    if (b < nb) {
                        const cd *xh = hh.data() + ((size_t)step * nb * 2 + (size_t)b * 2) * nz0, *xa = xh + nz0;
                        for (int q = 0; q < nz0; q++) z[q] = 0.5 * xh[q] + cd(0, 0.5) * xa[q];
                        rdo_dense(cf, z.data(), m);
                        val = b == 0 ? trace_op(cf, m, true) : std::conj(trace_op(cf, m, false));
                    }
                    reinterpret_cast<cd *>(corr)[2 * (size_t)step + b] = val;
                }
                if (rdo_h || rdo_a) {
                    const cd *xh = hh.data() + ((size_t)step * nb * 2) * nz0, *xa = xh + nz0;
                    if (rdo_h) { rdo_dense(cf, xh, m); std::copy(m.begin(), m.end(), reinterpret_cast<cd *>(rdo_h) + (size_t)step * n * n); }
                    if (rdo_a) { rdo_dense(cf, xa, m); std::copy(m.begin(), m.end(), reinterpret_cast<cd *>(rdo_a) + (size_t)step * n * n); }
                }
            }
        } catch (...) { cleanup(); throw; }
        cleanup();
    });
}

int heom_cf_bench_inner(heom_cf *cf, int32_t nbatch, int32_t reps, double *out)
{
    return guarded([&] {
        require_cf(cf);
        DeviceScope dsc(cf->ctx->device);
        if (nbatch < 1 || reps < 1 || !out) fail(HEOM_E_ARG, "nbatch and reps must be positive");
        std::vector<double> w(nbatch);
        for (int b = 0; b < nbatch; b++) w[b] = (b % 2 ? 1.0 : -1.0) * (0.1 + 0.01 * b) / kHbar;
        std::vector<std::vector<cd>> rhs(1, std::vector<cd>(2 * cf->lunkcf, cd(1e-3, 0)));
        CfBatchResult r;
        cf_solve_batch(cf, w, std::vector<int>(nbatch, 0), rhs, 1e-8, 100, HEOM_PREC_MIXED, r, reps, out);
    });
}

int heom_cf_bench_apply(heom_cf *cf, int32_t nbatch, int32_t reps, double *seconds, double *bytes)
{
    return guarded([&] {
        require_cf(cf);
        DeviceScope dsc(cf->ctx->device);
        if (nbatch < 1 || reps < 1) fail(HEOM_E_ARG, "nbatch and reps must be positive");
        heom_ctx *c = cf->ctx;
        const int64_t N = 2 * cf->lunkcf + 1, vs = (N + 63) / 64 * 64;
        std::vector<void *> tmp;
        auto cleanup = [&] { for (void *p : tmp) cudaFree(p); tmp.clear(); };
        cudaEvent_t e0 = nullptr, e1 = nullptr;
        try {
            ensure_omega(cf, nbatch);
            std::vector<double> w(nbatch);
            for (int b = 0; b < nbatch; b++) w[b] = (b % 2 ? 1.0 : -1.0) * (0.1 + 0.01 * b) / kHbar;
            CK(cudaMemcpyAsync(cf->d_omega, w.data(), sizeof(double) * nbatch, cudaMemcpyHostToDevice, c->stream));
            double2 *x = nullptr, *y = nullptr, *hv = nullptr, *gd = nullptr;
            double *es = nullptr;
            CK(cudaMalloc((void **)&x, sizeof(double2) * (size_t)vs * nbatch)); tmp.push_back(x);
            CK(cudaMalloc((void **)&y, sizeof(double2) * (size_t)vs * nbatch)); tmp.push_back(y);
            const DevPlan P = cf->dplan.view;
            CK(cudaMalloc((void **)&hv, sizeof(double2) * (size_t)std::max(1, P.nh) * nbatch)); tmp.push_back(hv);
            CK(cudaMalloc((void **)&es, sizeof(double) * 4 * (size_t)nbatch)); tmp.push_back(es);
            CK(cudaMalloc((void **)&gd, sizeof(double2) * (size_t)P.nado * nbatch)); tmp.push_back(gd);
            // x = 1e-3 (1 + i) everywhere: the timing does not depend on the values
            std::vector<double2> ones((size_t)vs, make_double2(1e-3, 1e-3));
            for (int b = 0; b < nbatch; b++) {
                CK(cudaMemcpyAsync(x + (size_t)b * vs, ones.data(), sizeof(double2) * vs, cudaMemcpyHostToDevice, c->stream));
                CK(cudaMemcpyAsync(hv + (size_t)b * P.nh, c->hval64, sizeof(double2) * P.nh, cudaMemcpyDeviceToDevice, c->stream));
                CK(cudaMemcpyAsync(es + 4 * (size_t)b, c->es64, sizeof(double) * 4, cudaMemcpyDeviceToDevice, c->stream));
            }
            DevCoef<double> K = cf_coef(cf);
            K.hval = hv;
            K.eshift = es;
            fill_gdiag<double>(P, K, gd, nbatch, c->stream);
            K.gdiag = gd;
            for (int r = 0; r < 3; r++) launch_apply_cf(P, K, x, y, nbatch, vs, nullptr, c->stream);
            CK(cudaEventCreate(&e0)); CK(cudaEventCreate(&e1));
            CK(cudaEventRecord(e0, c->stream));
            for (int r = 0; r < reps; r++) launch_apply_cf(P, K, r % 2 ? y : x, r % 2 ? x : y, nbatch, vs, nullptr, c->stream);
            CK(cudaEventRecord(e1, c->stream));
            CK(cudaEventSynchronize(e1));
            CK(cudaGetLastError());
            float ms = 0;
            cudaEventElapsedTime(&ms, e0, e1);
            if (seconds) *seconds = ms * 1e-3 / reps;
            if (bytes) *bytes = nbatch * 2.0 * (double)N * sizeof(double2) + plan_read_bytes(cf->plan);
        } catch (...) {
            if (e0) cudaEventDestroy(e0);
            if (e1) cudaEventDestroy(e1);
            cleanup();
            throw;
        }
        cudaEventDestroy(e0); cudaEventDestroy(e1);
        cleanup();
    });
}

}  // extern "C"
