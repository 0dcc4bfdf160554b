// extern "C" entry points of the GB300 HEOM library (declared in include/heom_gb300.h).
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <mutex>

#include <type_traits>

#include "context.cuh"
#include "inner.cuh"

namespace heom {

static thread_local std::string g_error;
void set_error(const std::string &msg) { g_error = msg; }
void fail(int code, const std::string &msg) { throw HeomError{code, msg}; }
void cuda_check(cudaError_t e, const char *what)
{
    if (e != cudaSuccess) fail(HEOM_E_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

template <typename T>
static T *dalloc(std::vector<void *> &blocks, size_t n)
{
    T *p = nullptr;
    if (n == 0) n = 1;
    if (cudaMalloc((void **)&p, sizeof(T) * n) != cudaSuccess) fail(HEOM_E_NOMEM, "device allocation failed");
    blocks.push_back(p);
    return p;
}
template <typename T>
static T *upload_vec(std::vector<void *> &blocks, const std::vector<T> &v)
{
    T *p = dalloc<T>(blocks, v.size());
    if (!v.empty()) CK(cudaMemcpy(p, v.data(), sizeof(T) * v.size(), cudaMemcpyHostToDevice));
    return p;
}

void PlanDev::upload(const HostPlan &P)
{
    view = DevPlan();
    view.lunk = P.lunk; view.nado = P.nado; view.nslots = P.nslots; view.nh = P.nh;
    view.ntrace = (int32_t)P.trace_idx.size();
    view.ent_ado = upload_vec(blocks, P.ent_ado);
    view.ado_off = upload_vec(blocks, P.ado_off);
    view.ado_cls = upload_vec(blocks, P.ado_cls);
    view.ado_cnt = upload_vec(blocks, P.ado_cnt);
    view.coup_ptr = upload_vec(blocks, P.coup_ptr);
    view.coup_mid = upload_vec(blocks, P.coup_mid);
    view.cls_tptr = upload_vec(blocks, P.cls_tptr);
    view.term_ptr = upload_vec(blocks, P.term_ptr);
    view.trace_idx = upload_vec(blocks, P.trace_idx);
    view.terms = upload_vec(blocks, P.terms);
    view.maps = upload_vec(blocks, P.maps);
    std::vector<int4> coup(P.coup.size());
    for (size_t k = 0; k < coup.size(); k++) coup[k] = make_int4(P.coup[k].src_off, P.coup[k].map_base, P.coup[k].cid, 0);
    view.coup = upload_vec(blocks, coup);
    {
        // work profile of every entry: couplings of its ADO, nonzero gather words, same-tier
        // terms; a stable sort by profile (then class and position) makes warps uniform
        std::vector<uint64_t> key(P.lunk);
        for (int64_t e = 0; e < P.lunk; e++) {
            const int32_t a = P.ent_ado[e], p = (int32_t)(e - P.ado_off[a]), c = P.ado_cls[a];
            const int32_t ncp = P.coup_ptr[a + 1] - P.coup_ptr[a];
            int32_t used = 0;
            for (int32_t k = P.coup_ptr[a]; k < P.coup_ptr[a + 1]; k++) used += P.maps[P.coup[k].map_base + p] != 0;
            const int32_t tb = P.cls_tptr[c] + p;
            const int32_t nt = P.term_ptr[tb + 1] - P.term_ptr[tb];
            key[e] = ((uint64_t)std::min(ncp, 255) << 56) | ((uint64_t)std::min(used, 255) << 48) |
                     ((uint64_t)std::min(nt, 255) << 40) | ((uint64_t)std::min(c, 65535) << 24) | (uint64_t)std::min(p, 16777215);
        }
        std::vector<int32_t> order(P.lunk);
        for (int64_t e = 0; e < P.lunk; e++) order[e] = (int32_t)e;
        std::stable_sort(order.begin(), order.end(), [&](int32_t a, int32_t b) { return key[a] < key[b]; });
        view.order = upload_vec(blocks, order);
    }
    auto to64 = [](const std::vector<cd> &v) { std::vector<double2> o(v.size()); for (size_t k = 0; k < v.size(); k++) o[k] = make_double2(v[k].real(), v[k].imag()); return o; };
    auto to32 = [](const std::vector<cd> &v) { std::vector<float2> o(v.size()); for (size_t k = 0; k < v.size(); k++) o[k] = make_float2((float)v[k].real(), (float)v[k].imag()); return o; };
    g0_64 = upload_vec(blocks, to64(P.g0)); cl_64 = upload_vec(blocks, to64(P.cl)); cr_64 = upload_vec(blocks, to64(P.cr));
    g0_32 = upload_vec(blocks, to32(P.g0)); cl_32 = upload_vec(blocks, to32(P.cl)); cr_32 = upload_vec(blocks, to32(P.cr));
    auto todf = [](const std::vector<cd> &v) { std::vector<float4> o(v.size()); for (size_t k = 0; k < v.size(); k++) o[k] = Num<DF>::store_host(Num<DF>::from_d(v[k].real(), v[k].imag())); return o; };
    g0_df = upload_vec(blocks, todf(P.g0)); cl_df = upload_vec(blocks, todf(P.cl)); cr_df = upload_vec(blocks, todf(P.cr));
    ncoef = (int64_t)P.cl.size();
}

void PlanDev::release()
{
    for (void *p : blocks) cudaFree(p);
    blocks.clear();
}

template <> DevCoef<double> PlanDev::coef<double>() const { DevCoef<double> c; c.g0 = g0_64; c.cl = cl_64; c.cr = cr_64; return c; }
template <> DevCoef<float> PlanDev::coef<float>() const { DevCoef<float> c; c.g0 = g0_32; c.cl = cl_32; c.cr = cr_32; return c; }
template <> DevCoef<DF> PlanDev::coef<DF>() const
{
    DevCoef<DF> c;
    c.g0 = g0_df; c.cl = cl_df; c.cr = cr_df;
    return c;
}

}  // namespace heom

using namespace heom;

heom_ctx::~heom_ctx()
{
    dfwd.release();
    dadj.release();
    void *ptrs[] = {hval64, hval32, hvaldf, es64, d_cur_terms, dx, dy, dz, fx, fy, dscratch, d_rdo_pair, d_rdo_upper, d_ent_rc};
    for (void *p : ptrs) if (p) cudaFree(p);
    if (stream) cudaStreamDestroy(stream);
}

struct heom_batch {
    heom_ctx *ctx = nullptr;
    int device = 0;   // the context's device (destroy may run after the context is gone)
    int nbatch = 0;
    int64_t vs = 0;
    double2 *h64 = nullptr;
    float4 *hdf = nullptr;
    float2 *h32 = nullptr;
    double *e64 = nullptr;
    int h_real = 0;
    // truncated instances (heom_batch_set_tiers): per instance (first entry of its last kept
    // tier, one past its last kept entry); nullptr = all at the context's depth
    int2 *tier_lim = nullptr;
    std::vector<int2> tier_lim_host;
    ~heom_batch()
    {
        if (h64) cudaFree(h64);
        if (hdf) cudaFree(hdf);
        if (h32) cudaFree(h32);
        if (e64) cudaFree(e64);
        if (tier_lim) cudaFree(tier_lim);
    }
};

namespace heom {

// H values of the context's structure from a dense hs, in the three number types
void hvalues(heom_ctx *c, const cd *hs, std::vector<double2> &h64, std::vector<float2> &h32, std::vector<float4> &hdf, int &real)
{
    size_t nh = c->hst.rows.size();
    h64.resize(nh); h32.resize(nh); hdf.resize(nh);
    real = 1;
    for (size_t k = 0; k < nh; k++) {
        cd v = hs[(size_t)c->hst.rows[k] + (size_t)c->hst.cols[k] * c->nrho];
        h64[k] = make_double2(v.real(), v.imag());
        h32[k] = make_float2((float)v.real(), (float)v.imag());
        hdf[k] = Num<DF>::store_host(Num<DF>::from_d(v.real(), v.imag()));
        if (v.imag() != 0.0) real = 0;
    }
}

void set_params(heom_ctx *c, const std::vector<cd> &hs, const double *es)
{
    std::vector<double2> h64; std::vector<float2> h32; std::vector<float4> hdf;
    hvalues(c, hs.data(), h64, h32, hdf, c->h_real);
    CK(cudaMemcpyAsync(c->hval64, h64.data(), sizeof(double2) * h64.size(), cudaMemcpyHostToDevice, c->stream));
    CK(cudaMemcpyAsync(c->hval32, h32.data(), sizeof(float2) * h32.size(), cudaMemcpyHostToDevice, c->stream));
    CK(cudaMemcpyAsync(c->hvaldf, hdf.data(), sizeof(float4) * hdf.size(), cudaMemcpyHostToDevice, c->stream));
    double e4[4] = {0, 0, 0, 0};
    for (int k = 0; k < 4; k++) e4[k] = es[k];
    CK(cudaMemcpyAsync(c->es64, e4, sizeof e4, cudaMemcpyHostToDevice, c->stream));
    CK(cudaStreamSynchronize(c->stream));
}

template <typename T> DevCoef<T> main_coef(heom_ctx *c, bool adj)
{
    DevCoef<T> k = (adj ? c->dadj : c->dfwd).template coef<T>();
    k.eshift = c->es64;
    k.h_real = c->h_real;
    return k;
}
template <typename T> void set_hval(DevCoef<T> &k, heom_ctx *c);
template <> void set_hval<double>(DevCoef<double> &k, heom_ctx *c) { k.hval = c->hval64; }
template <> void set_hval<float>(DevCoef<float> &k, heom_ctx *c) { k.hval = c->hval32; }
template <> void set_hval<DF>(DevCoef<DF> &k, heom_ctx *c) { k.hval = c->hvaldf; }
template <typename T> DevCoef<T> ctx_coef(heom_ctx *c, bool adj)
{
    DevCoef<T> k = main_coef<T>(c, adj);
    set_hval<T>(k, c);
    return k;
}

CoefSet ctx_coefs(heom_ctx *c, bool adj)
{
    return CoefSet{ctx_coef<double>(c, adj), ctx_coef<float>(c, adj), ctx_coef<DF>(c, adj)};
}

void require_ctx(heom_ctx *c) { if (!c) fail(HEOM_E_ARG, "null context"); }

// Hermitise the RDO part of a host rho: upper triangle defines the lower one and the
// diagonal is made real (utility/zmat_herm_coo.f90 with uplo = 'u').
void herm_rdo(heom_ctx *c, cd *rho)
{
    int n = c->nrho;
    std::vector<cd> t((size_t)n * n, 0.0);
    for (size_t q = 0; q < c->rdo_rows.size(); q++) {
        int r = c->rdo_rows[q], cc = c->rdo_cols[q];
        if (cc > r) { t[(r - 1) + (size_t)(cc - 1) * n] = rho[q]; t[(cc - 1) + (size_t)(r - 1) * n] = std::conj(rho[q]); }
        if (cc == r) t[(r - 1) + (size_t)(cc - 1) * n] = rho[q].real();
    }
    for (size_t q = 0; q < c->rdo_rows.size(); q++) rho[q] = t[(c->rdo_rows[q] - 1) + (size_t)(c->rdo_cols[q] - 1) * n];
}

__global__ void k_add_real(double2 *p, double v) { p->x += v; }

// Replace the RDO block of every instance by its Hermitian part and clear the free trace
// unknown x[lunk]; thread q handles the pair (q, q') with q <= q', so the update is in place.
__global__ void k_herm_rdo(double2 *x, int64_t vstride, int64_t lunk, int nz0, const int32_t *pair)
{
    double2 *xb = x + (int64_t)blockIdx.y * vstride;
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < nz0; q += gridDim.x * blockDim.x) {
        const int p = pair[q];
        if (p < q) continue;
        const double2 a = xb[q], b = xb[p];
        if (p == q) { xb[q].y = 0.0; continue; }
        const double2 h = make_double2(0.5 * (a.x + b.x), 0.5 * (a.y - b.y));
        xb[q] = h;
        xb[p] = make_double2(h.x, -h.y);
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) xb[lunk] = make_double2(0.0, 0.0);
}

// The reference's hermitisation of an input RDO block (utility/zmat_herm_coo.f90, uplo 'u'):
// the upper triangle defines the lower one and the diagonal is made real.
__global__ void k_herm_rdo_upper(double2 *x, int64_t vstride, int nz0, const int32_t *pair, const int32_t *upper)
{
    double2 *xb = x + (int64_t)blockIdx.y * vstride;
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < nz0; q += gridDim.x * blockDim.x) {
        const int p = pair[q];
        if (p == q) xb[q].y = 0.0;
        else if (upper[q]) xb[p] = make_double2(xb[q].x, -xb[q].y);
    }
}

void herm_rdo_upper_dev(heom_ctx *c, double2 *x, int nbatch, int64_t vstride)
{
    dim3 g((unsigned)std::max(1, std::min(64, (c->nz0 + 255) / 256)), (unsigned)nbatch);
    k_herm_rdo_upper<<<g, 256, 0, c->stream>>>(x, vstride, c->nz0, c->d_rdo_pair, c->d_rdo_upper);
}

void herm_rdo_dev(heom_ctx *c, double2 *x, int nbatch, int64_t vstride)
{
    dim3 g((unsigned)std::max(1, std::min(64, (c->nz0 + 255) / 256)), (unsigned)nbatch);
    k_herm_rdo<<<g, 256, 0, c->stream>>>(x, vstride, c->lunk, c->nz0, c->d_rdo_pair);
}

template <typename T> DevCoef<T> regularised(heom_ctx *c, DevCoef<T> K)
{
    K.reg = 1;
    K.nz0 = c->nz0;
    K.ndiag = c->ndiag;
    K.rdo_pair = c->d_rdo_pair;
    K.reg_scale = c->reg_scale;
    return K;
}

void drandn_stream(int64_t n, std::vector<double> &out)
{
    // tfqmr_double/drandn.f90 with SEED = 1: multiplicative congruential generator with
    // multiplier 2^29 + 5 modulo 2^31 - 1 on 32-bit wrapping integers
    out.resize(n);
    int32_t im = (1 << 29) + 5, imax = 2147483647, is = 1;
    for (int64_t i = 0; i < n; i++) {
        out[i] = (double)is / (double)imax;
        int32_t prod = (int32_t)((uint32_t)im * (uint32_t)is);
        int32_t r = prod % imax;
        is = r < 0 ? -r : r;
    }
}

template <typename T>
void upload_rt_to(heom_ctx *c, typename Num<T>::V *dst, int64_t n, const double *src = nullptr)
{
    using V = typename Num<T>::V;
    if (!src) src = c->rt_host.data();
    std::vector<V> rt(n);
    for (int64_t i = 0; i < n; i++) rt[i] = Num<T>::store_host(Num<T>::from_d(src[2 * i], src[2 * i + 1]));
    CK(cudaMemcpyAsync(dst, rt.data(), sizeof(V) * n, cudaMemcpyHostToDevice, c->stream));
    CK(cudaStreamSynchronize(c->stream));
}

template <typename T>
void upload_rt(heom_ctx *c, TfqWork<T> &W) { upload_rt_to<T>(c, W.rt, W.N); }

// Run TFQMR iterations until every instance finished; graph-captured chunks of `chunk`
// iterations, host polls the done flags between chunks.
template <typename T>
void tfq_run(heom_ctx *c, TfqWork<T> &W, const ApplyFn<T> &apply, int nlim, int &iters_out, int64_t &launches)
{
    const int chunk = 25;
    cudaGraph_t g = nullptr;
    cudaGraphExec_t ge = nullptr;
    {
        const CapturedGraph cg = capture_graph(c->stream, [&] { for (int k = 0; k < chunk; k++) tfq_iteration<T>(W, apply, c->stream); });
        g = cg.graph;
        ge = cg.exec;
    }
    std::vector<int> act(W.nbatch);
    int launched = 0;
    while (true) {
        CK(cudaGraphLaunch(ge, c->stream));
        launched += chunk;
        CK(cudaMemcpyAsync(act.data(), W.act_main, sizeof(int) * W.nbatch, cudaMemcpyDeviceToHost, c->stream));
        CK(cudaStreamSynchronize(c->stream));
        bool any = false;
        for (int a : act) any = any || a;
        if (!any || launched > nlim + chunk) break;
    }
    cudaGraphExecDestroy(ge);
    cudaGraphDestroy(g);
    iters_out = launched;
    launches += (int64_t)launched * kTfqIterationLaunches;
}

template <typename T>
ApplyFn<T> make_apply(heom_ctx *c, const DevCoef<T> &K, int nbatch, int64_t vstride, bool adj)
{
    const DevPlan P = adj ? c->dadj.view : c->dfwd.view;
    cudaStream_t s = c->stream;
    return [P, K, nbatch, vstride, s, adj](const typename Num<T>::V *x, typename Num<T>::V *y, const int *act) {
        if (adj) launch_apply<T, true>(P, K, x, y, nbatch, vstride, act, s);
        else launch_apply<T, false>(P, K, x, y, nbatch, vstride, act, s);
    };
}

// y = e_trace - A x  (FP64, device)
void residual64(heom_ctx *c, const DevCoef<double> &K, const double2 *x, double2 *r, int nbatch, int64_t vstride, bool adj,
                const double2 *rhs = nullptr)
{
    const DevPlan &P = adj ? c->dadj.view : c->dfwd.view;
    if (adj) launch_apply<double, true>(P, K, x, r, nbatch, vstride, nullptr, c->stream);
    else launch_apply<double, false>(P, K, x, r, nbatch, vstride, nullptr, c->stream);
    if (rhs) vec_axpby<double>(vstride * nbatch, r, -1.0, r, 1.0, rhs, c->stream);
    else {
        vec_axpby<double>(vstride * nbatch, r, -1.0, r, 0.0, r, c->stream);
        for (int b = 0; b < nbatch; b++) k_add_real<<<1, 1, 0, c->stream>>>(r + (int64_t)b * vstride + c->lunk, 1.0);
    }
}

}  // namespace

// ----------------------------------------------------------------------------
namespace heom {

void hvalues64(heom_ctx *c, const cd *hs, std::vector<double2> &h64)
{
    std::vector<float2> a;
    std::vector<float4> b;
    int r;
    hvalues(c, hs, h64, a, b, r);
}

double device_rdot(heom_ctx *c, int64_t n, const double2 *a, const double2 *b)
{
    return device_dot(n, a, b, c->dscratch, c->stream);
}

void run_tfqmr64(heom_ctx *c, TfqWork<double> &W, const ApplyFn<double> &apply, int nlim, int &iters, int64_t &launches)
{
    tfq_run<double>(c, W, apply, nlim, iters, launches);
}

void drandn_host(int64_t n, std::vector<double> &out) { drandn_stream(n, out); }

void solve_custom64(heom_ctx *c, const ApplyFn<double> &op, const double2 *rhs, double2 *x, double crit_abs, int maxit0,
                    heom_solve_info &info)
{
    const int64_t N = c->lunk + 1;
    const int nlim = std::max(1, maxit0 / 2);
    info = heom_solve_info{};
    cudaEvent_t e0, e1;
    CK(cudaEventCreate(&e0)); CK(cudaEventCreate(&e1));
    CK(cudaEventRecord(e0, c->stream));
    TfqWork<double> W;
    tfq_alloc<double>(W, 1, N, c->stream);
    double resid = 0;
    try {
        upload_rt(c, W);
        // restarted TFQMR: each round solves op d = rhs - op(x) from d = 0 and adds d to x;
        // a restart clears the drift between TFQMR's recursive and true residuals
        for (int round = 0;; round++) {
            op(x, W.s, nullptr);
            vec_axpby<double>(N, W.b, 1.0, rhs, -1.0, W.s, c->stream);
            resid = device_norm2(N, W.b, c->dscratch, c->stream);
            if (resid <= crit_abs || round == 8 || info.iters >= 2 * nlim) break;
            tfq_start<double>(W, crit_abs / resid, nlim, crit_abs, 0.0, 8, c->stream);
            int it = 0;
            tfq_run<double>(c, W, op, nlim, it, info.launches);
            vec_axpby<double>(N, x, 1.0, x, 1.0, W.x, c->stream);
            TfqState st;
            CK(cudaMemcpyAsync(&st, W.st, sizeof(TfqState), cudaMemcpyDeviceToHost, c->stream));
            CK(cudaStreamSynchronize(c->stream));
            info.iters += st.axb;
            info.ierr = st.ierr;
            info.refinements = round + 1;
        }
    } catch (...) { tfq_free(W); cudaEventDestroy(e0); cudaEventDestroy(e1); throw; }
    tfq_free(W);
    CK(cudaEventRecord(e1, c->stream));
    CK(cudaEventSynchronize(e1));
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0); cudaEventDestroy(e1);
    info.resid = resid;
    info.converged = resid <= crit_abs;
    info.seconds = ms * 1e-3;
}

void solve_custom_mixed(heom_ctx *c, const ApplyFn<double> &op64, const ApplyFn<DF> &opdf, const double2 *rhs, double2 *x,
                        double crit_abs, int maxit0, heom_solve_info &info)
{
    const int64_t N = c->lunk + 1;
    const int nlim = std::max(1, maxit0 / 2);
    info = heom_solve_info{};
    cudaEvent_t e0, e1;
    CK(cudaEventCreate(&e0)); CK(cudaEventCreate(&e1));
    CK(cudaEventRecord(e0, c->stream));
    TfqWork<DF> W;
    tfq_alloc<DF>(W, 1, N, c->stream);
    double2 *r = nullptr;
    double resid = 0, prev = 0;
    bool stalled = false;
    try {
        CK(cudaMalloc((void **)&r, sizeof(double2) * N));
        upload_rt_to<DF>(c, W.rt, N);
        for (int round = 0; round < 16; round++) {
            op64(x, r, nullptr);
            vec_axpby<double>(N, r, 1.0, rhs, -1.0, r, c->stream);   // r = rhs - op64(x)
            resid = device_norm2(N, r, c->dscratch, c->stream);
            if (resid <= crit_abs) break;
            if (round > 0 && resid > 0.5 * prev) { stalled = true; break; }
            prev = resid;
            vec_from_d<DF>(N, r, W.b, 1.0 / resid, c->stream);
            const double tgt = std::max(crit_abs / resid, 1e-10);
            tfq_start<DF>(W, tgt * 1e-3, nlim, tgt, 0.0, 40, c->stream);
            int it = 0;
            tfq_run<DF>(c, W, opdf, nlim, it, info.launches);
            vec_axpy_to_d<DF>(N, x, resid, W.x, c->stream);
            TfqState st;
            CK(cudaMemcpyAsync(&st, W.st, sizeof(TfqState), cudaMemcpyDeviceToHost, c->stream));
            CK(cudaStreamSynchronize(c->stream));
            info.iters += st.axb;
            info.refinements = round + 1;
        }
    } catch (...) { tfq_free(W); if (r) cudaFree(r); cudaEventDestroy(e0); cudaEventDestroy(e1); throw; }
    tfq_free(W);
    cudaFree(r);
    CK(cudaEventRecord(e1, c->stream));
    CK(cudaEventSynchronize(e1));
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0); cudaEventDestroy(e1);
    info.resid = resid;
    info.converged = resid <= crit_abs;
    info.seconds = ms * 1e-3;
    if (stalled && !info.converged) {   // the rest with the restarted FP64 solve
        heom_solve_info more{};
        solve_custom64(c, op64, rhs, x, crit_abs, maxit0, more);
        info.iters += more.iters;
        info.refinements += more.refinements;
        info.launches += more.launches;
        info.resid = more.resid;
        info.converged = more.converged;
        info.seconds += more.seconds;
    }
}

// ||H||_inf of the context's Hamiltonian (the scale of the inner preconditioner)
double hs_inf_norm(heom_ctx *c)
{
    double hn = 0;
    for (int i = 0; i < c->nrho; i++) {
        double rs = 0;
        for (int j = 0; j < c->nrho; j++) rs += std::abs(c->hs_host[i + (size_t)j * c->nrho]);
        hn = std::max(hn, rs);
    }
    return std::max(hn, 1e-300);
}

// Mixed-precision refinement: rounds of (hermitise x, FP64 residual r = rhs - A x, inner
// TFQMR on A~ d = r / ||r|| in the number type T, x += ||r|| d) until ||r|| <= crit.  A~ is
// the regularised operator (DevCoef::reg): it agrees with A on vectors whose RDO block is
// Hermitian and whose trace unknown is zero, and is nonsingular where A has the null space
// spanned by the free trace unknown and the anti-Hermitian stationary RDO directions; the
// inner Krylov solves then stay well conditioned in low precision.  The inner solves run
// the fused TFQMR of inner.cuh from one CUDA graph of kInnerChunk iterations plus a
// residual check, instantiated once and replayed for every round.
template <typename T>
void mixed_rounds(heom_ctx *c, const heom_solve_opts &o, double2 *x, int nbatch, int64_t vstride, const double2 *rhs,
                  const DevCoef<double> &K64, const DevCoef<T> &KT, double2 *r64, std::vector<double> &norms,
                  int nlim, int max_rounds, bool stall_exit, bool &stalled,
                  int &total_iters, int &last_ierr, bool &converged, int &rounds, int64_t &launches, int64_t &aux,
                  const std::function<void(const double2 *, double2 *)> &residual,
                  const std::function<void(const double2 *)> &batch_norms,
                  const DevPlan &PV, int64_t N)
{
    constexpr int kInnerChunk = 25;   // 50 applies between residual checks, as in the reference driver
    const double itol = o.inner_tol > 0 ? o.inner_tol : (std::is_same<T, float>::value ? 1e-2 : 1e-10);
    InnerWork<T> W;
    inner_alloc<T>(W, nbatch, N, c->stream, o.interleave, o.lane_instances > 0 ? o.lane_instances : 1);
    typename Num<T>::V *gd = nullptr;
    float *pre = nullptr;
    double pre_kappa = 1.0, pre_max = 1.0;
    // one graph of a chunk per lane configuration (W.GE, W.ipl), instantiated on first use
    std::map<int, std::pair<cudaGraph_t, cudaGraphExec_t>> graphs;
    auto release = [&] {
        for (auto &g : graphs) {
            if (g.second.second) cudaGraphExecDestroy(g.second.second);
            if (g.second.first) cudaGraphDestroy(g.second.first);
        }
        inner_free(W);
        if (gd) cudaFree(gd);
        if (pre) cudaFree(pre);
    };
    try {
        inner_shadow<T>(W, 0, c->stream);   // sign-symmetric; another one after a round without progress
        aux++;
        // with a given right-hand side the operator is used as it is; the steady problem
        // (rhs == nullptr) is solved on the regularised operator
        DevCoef<T> KI = rhs ? KT : regularised<T>(c, KT);
        // per-instance ADO diagonals, so the inner applies do no FP64 arithmetic
        CK(cudaMalloc((void **)&gd, sizeof(typename Num<T>::V) * gdiag_elems<T>(PV, nbatch)));
        fill_gdiag<T>(PV, KI, gd, nbatch, c->stream);
        aux++;
        // left diagonal preconditioning: the inner problem M A d = M r with M = diag(1 / (|g0_n|
        // + ||H||_inf)) per ADO evens out the rows of the hierarchy's tiers (about half the
        // Krylov iterations on the double dot); the FP64 refinement still tests A x = b
        // (the FP64 inner solves of FP64_REFINED and of the stall fallback stay unscaled: there
        // the divided target would ask for more than FP64 TFQMR reaches on some models)
        if (o.inner_precond >= 0 && !std::is_same<T, double>::value) {
            CK(cudaMalloc((void **)&pre, sizeof(float) * std::max(1, PV.nado)));
            fill_pre(PV, K64.g0, hs_inf_norm(c), pre, c->stream);
            KI.pre = pre;
            aux++;
            // the inner solve measures M (b - A d): ||b - A d|| <= ||M^-1|| ||M (b - A d)||, so
            // its target is divided by the condition number of M relative to the scaling of b
            // (c->stream is non-blocking: the read is queued behind fill_pre on that stream)
            std::vector<float> ph(std::max(1, PV.nado));
            CK(cudaMemcpyAsync(ph.data(), pre, sizeof(float) * ph.size(), cudaMemcpyDeviceToHost, c->stream));
            CK(cudaStreamSynchronize(c->stream));
            const float lo = *std::min_element(ph.begin(), ph.end()), hi = *std::max_element(ph.begin(), ph.end());
            pre_kappa = lo > 0 ? (double)hi / lo : 1.0;
            pre_max = hi;
        }
        W.tier_lim = KI.tier_lim;
        if (W.ipl_max > 1 && (KI.tier_lim || (KI.cf_half && W.G != 2)))
            fail(HEOM_E_ARG, "two instances per lane: whole hierarchies only, and correlation functions in groups of two");
        KI = inner_layout_coef<T>(W, PV, KI, c->stream);   // the workspace's instance-interleaved layout
        auto chunk_graph = [&]() -> cudaGraphExec_t {
            const int key = 4 * W.GE + W.ipl;
            auto it = graphs.find(key);
            if (it != graphs.end()) return it->second.second;
            const CapturedGraph cg = capture_graph(c->stream, [&] { inner_chunk<T>(W, PV, KI, kInnerChunk, c->stream); });
            graphs[key] = {cg.graph, cg.exec};
            return cg.exec;
        };
        std::vector<InnerState> st(nbatch);
        std::vector<int> amap;
        int round = 0;
        std::vector<double> prev;
        for (; round < std::max(1, max_rounds); round++) {
            if (!rhs) { herm_rdo_dev(c, x, nbatch, vstride); aux++; }
            residual(x, r64);
            batch_norms(r64);
            bool all_ok = true;
            for (double v : norms) all_ok = all_ok && v <= o.crit;
            if (all_ok) { converged = true; break; }
            // a round that did not halve some instance's residual: with stall_exit the inner
            // arithmetic cannot resolve what is left, and the caller continues with FP64 inner
            // solves; otherwise the next round's inner solves change their shadow vector
            if (!prev.empty()) {
                bool stuck = false;
                for (int b = 0; b < nbatch; b++) stuck = stuck || (norms[b] > o.crit && norms[b] > 0.5 * prev[b]);
                if (stuck && stall_exit) { stalled = true; break; }
                if (stuck) { inner_shadow<T>(W, round, c->stream); aux++; }   // the next inner solve
            }
            prev = norms;
            for (int b = 0; b < nbatch; b++)   // instances already below crit get b = 0 and stop at once
                inner_rhs<T>(W, PV, r64 + (int64_t)b * vstride, b, norms[b] <= o.crit ? 0.0 : 1.0 / norms[b], pre, c->stream);
            aux += nbatch;
            // the scaled inner problem has ||b|| = 1: stop at max(itol, crit / ||r||) (the most
            // demanding instance sets it), or at the arithmetic's floor
            double tgt = 1.0;
            for (double v : norms) if (v > o.crit) tgt = std::min(tgt, o.crit / v);
            tgt = std::max(tgt, itol);
            if (pre) tgt *= pre_max / pre_kappa;   // b = M r / ||r|| has ||b|| <= max m
            inner_start<T>(W, tgt, nlim, o.stag_window > 0 ? o.stag_window : 40, c->stream);
            aux += kInnerStartLaunches;
            CK(cudaMemcpyAsync(st.data(), W.st, sizeof(InnerState) * nbatch, cudaMemcpyDeviceToHost, c->stream));
            CK(cudaStreamSynchronize(c->stream));
            for (int iters = 0;;) {
                bool any = false;
                for (const auto &sv : st) any = any || !sv.done;
                if (!any) break;
                // the running instances of each group on as few lanes as hold them
                inner_lanes<T>(W, st.data(), amap, c->stream);
                CK(cudaGraphLaunch(chunk_graph(), c->stream));
                iters += kInnerChunk;
                launches += (int64_t)kInnerChunk * kInnerIterationLaunches + kInnerCheckLaunches;
                CK(cudaMemcpyAsync(st.data(), W.st, sizeof(InnerState) * nbatch, cudaMemcpyDeviceToHost, c->stream));
                CK(cudaStreamSynchronize(c->stream));
                if (iters > nlim + kInnerChunk) break;
            }
            int applies = 0;
            for (const auto &sv : st) { applies = std::max(applies, 2 * sv.n + sv.checks); last_ierr = sv.ierr; }
            total_iters += applies;
            for (int b = 0; b < nbatch; b++)
                if (norms[b] > o.crit)
                    inner_add_solution<T>(W, x + (int64_t)b * vstride, b, norms[b], st[b].best_slot, c->stream), aux++;
        }
        if (!rhs) { herm_rdo_dev(c, x, nbatch, vstride); aux++; }
        rounds = round;
    } catch (...) { release(); throw; }
    release();
}

#define HEOM_MIXED_ROUNDS(T)                                                                                       \
    template void mixed_rounds<T>(heom_ctx *, const heom_solve_opts &, double2 *, int, int64_t, const double2 *,     \
                                  const DevCoef<double> &, const DevCoef<T> &, double2 *, std::vector<double> &, int, \
                                  int, bool, bool &, int &, int &, bool &, int &, int64_t &, int64_t &,               \
                                  const std::function<void(const double2 *, double2 *)> &,                            \
                                  const std::function<void(const double2 *)> &, const DevPlan &, int64_t);
HEOM_MIXED_ROUNDS(DF)
HEOM_MIXED_ROUNDS(double)
#undef HEOM_MIXED_ROUNDS

// The layouts (interleave, instances per lane) the automatic choice of the mixed batch
// solves compares: one instance per group; two instances per lane in groups of two (the
// iterates of the first, with the plan decoded once for two instances; not for truncated
// batches); the largest interleave with one and with two instances per lane.
std::vector<std::pair<int, int>> layout_candidates(int nbatch, bool truncated)
{
    const int g = inner_default_interleave(nbatch);
    std::vector<std::pair<int, int>> c = {{1, 1}};
    if (g == 1) return c;
    if (!truncated) c.push_back({2, 2});
    if (g > 2 || truncated) c.push_back({g, 1});
    if (g > 2 && !truncated) c.push_back({g, 2});
    return c;
}

// Solve A x = rhs (rhs = e_trace when rhs == nullptr) for nbatch instances, in FP64 or
// mixed precision.  x: device FP64, nbatch vectors with stride vstride (vstride >= lunk+1),
// holding the initial guess on entry.
void solve_device(heom_ctx *c, const heom_solve_opts &o, double2 *x, int nbatch, int64_t vstride, bool adj,
                  const double2 *rhs, heom_solve_info &info, const CoefSet &K)
{
    const int64_t N = c->lunk + 1;
    int nlim = o.maxit0 / 2;
    if (nlim < 1) nlim = 1;
    if (o.lane_instances < 0 || o.lane_instances > 2) fail(HEOM_E_ARG, "lane_instances must be 0, 1 or 2");
    if (o.precision == HEOM_PREC_MIXED && o.lane_instances == 2 && o.interleave == 1)
        fail(HEOM_E_ARG, "two instances per lane need an interleave of at least 2");
    info = heom_solve_info{};
    cudaEvent_t e0, e1;
    CK(cudaEventCreate(&e0)); CK(cudaEventCreate(&e1));
    CK(cudaEventRecord(e0, c->stream));
    std::vector<void *> tmp;
    double2 *r64 = nullptr;
    CK(cudaMalloc((void **)&r64, sizeof(double2) * (size_t)vstride * nbatch));
    tmp.push_back(r64);
    DevCoef<double> k64 = K.k64;   // gets the per-instance ADO diagonals below
    int total_iters = 0, last_ierr = 0;
    bool converged = false;
    std::vector<double> norms(nbatch, 0.0);
    int64_t aux = 0;   // launches outside the TFQMR graphs
    std::function<void(const double2 *)> batch_norms = [&](const double2 *v) {
        for (int b = 0; b < nbatch; b++) norms[b] = device_norm2(N, v + (int64_t)b * vstride, c->dscratch, c->stream);
        aux += nbatch;
    };
    std::function<void(const double2 *, double2 *)> residual = [&](const double2 *xx, double2 *r) {
        residual64(c, k64, xx, r, nbatch, vstride, adj, rhs);
        aux += rhs ? 2 : 2 + nbatch;
    };
    try {
        // per-instance ADO diagonals of the FP64 applies, so they do no per-entry lead-shift sums
        const DevPlan &PV = adj ? c->dadj.view : c->dfwd.view;
        double2 *gd64 = nullptr;
        CK(cudaMalloc((void **)&gd64, sizeof(double2) * std::max<int64_t>(1, (int64_t)PV.nado * nbatch)));
        tmp.push_back(gd64);
        fill_gdiag<double>(PV, k64, gd64, nbatch, c->stream);
        aux++;
        if (o.precision == HEOM_PREC_FP64) {
            TfqWork<double> W;
            tfq_alloc<double>(W, nbatch, N, c->stream);
            W.tier_lim = k64.tier_lim;
            try {
                upload_rt(c, W);
                // b = rhs - A x0 per instance, stored with the workspace stride
                residual(x, r64);
                for (int b = 0; b < nbatch; b++)
                    CK(cudaMemcpyAsync(W.b + (int64_t)b * W.vstride, r64 + (int64_t)b * vstride, sizeof(double2) * N, cudaMemcpyDeviceToDevice, c->stream));
                tfq_start<double>(W, o.crit * 1e-3, nlim, o.crit, 0.0, 0, c->stream);
                aux += kTfqStartLaunches;
                int it = 0;
                tfq_run<double>(c, W, make_apply<double>(c, k64, nbatch, W.vstride, adj), nlim, it, info.launches);
                for (int b = 0; b < nbatch; b++)
                    vec_axpby<double>(N, x + (int64_t)b * vstride, 1.0, x + (int64_t)b * vstride, 1.0, W.x + (int64_t)b * W.vstride, c->stream), aux++;
                std::vector<TfqState> st(nbatch);
                CK(cudaMemcpyAsync(st.data(), W.st, sizeof(TfqState) * nbatch, cudaMemcpyDeviceToHost, c->stream));
                CK(cudaStreamSynchronize(c->stream));
                int axb = 0;
                for (auto &sv : st) { axb = std::max(axb, sv.axb); last_ierr = sv.ierr; }
                total_iters = axb;
            } catch (...) { tfq_free(W); throw; }
            tfq_free(W);
        } else {
            if (adj) fail(HEOM_E_UNSUPPORTED, "mixed precision is implemented for the forward operator");
            bool stalled = false, unused = false;
            if (o.precision == HEOM_PREC_MIXED)
                mixed_rounds<DF>(c, o, x, nbatch, vstride, rhs, k64, K.kdf, r64, norms, nlim, o.max_refine, true, stalled,
                                 total_iters, last_ierr, converged, info.refinements, info.launches, aux, residual, batch_norms,
                                 c->dfwd.view, N);
            else if (o.precision == HEOM_PREC_FP64_REFINED)
                mixed_rounds<double>(c, o, x, nbatch, vstride, rhs, k64, K.k64, r64, norms, nlim, o.max_refine, false, unused,
                                     total_iters, last_ierr, converged, info.refinements, info.launches, aux, residual, batch_norms,
                                 c->dfwd.view, N);
            else if (o.precision == HEOM_PREC_MIXED_FP32)
                mixed_rounds<float>(c, o, x, nbatch, vstride, rhs, k64, K.k32, r64, norms, nlim, o.max_refine, true, stalled,
                                    total_iters, last_ierr, converged, info.refinements, info.launches, aux, residual, batch_norms,
                                 c->dfwd.view, N);
            else fail(HEOM_E_ARG, "unknown precision");
            if (stalled && !converged) {
                // up to max_refine rounds with FP64 inner solves on the same regularised operator
                int more = 0;
                mixed_rounds<double>(c, o, x, nbatch, vstride, rhs, k64, K.k64, r64, norms, nlim,
                                     std::max(1, o.max_refine), false, unused, total_iters, last_ierr,
                                     converged, more, info.launches, aux, residual, batch_norms, c->dfwd.view, N);
                info.refinements += more;
            }
        }
    } catch (...) { for (void *p : tmp) cudaFree(p); cudaEventDestroy(e0); cudaEventDestroy(e1); throw; }
    // final FP64 residual
    residual(x, r64);
    batch_norms(r64);
    double worst = 0;
    for (double v : norms) worst = std::max(worst, v);
    CK(cudaEventRecord(e1, c->stream));
    CK(cudaEventSynchronize(e1));
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0); cudaEventDestroy(e1);
    for (void *p : tmp) cudaFree(p);
    info.iters = total_iters;
    info.ierr = last_ierr;
    info.resid = worst;
    info.converged = worst <= o.crit || converged;
    info.seconds = ms * 1e-3;
    info.launches += aux;
}

}  // namespace heom

extern "C" {

const char *heom_last_error(void) { return heom::g_error.c_str(); }

int heom_ctx_create(const heom_tables *t, const heom_ctx_opts *opts, heom_ctx **out)
{
    return guarded([&] {
        if (!t || !out) fail(HEOM_E_ARG, "null argument");
        *out = nullptr;
        int dev = opts ? opts->device : 0;
        int ndev = 0;
        if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) fail(HEOM_E_CUDA, "no CUDA device available");
        DeviceScope dsc(dev);
        std::unique_ptr<heom_ctx> c(new heom_ctx());
        c->device = dev;
        CK(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
        c->norbs = t->norbs; c->nspin = t->nspin; c->nalf = t->nalf; c->ncor = t->ncor; c->nrho = t->nrho; c->ntier = t->ntier;
        c->lunk = t->lunk_spa; c->nunk = t->nunk;
        std::vector<const double _Complex *> extra;
        if (opts) for (auto *d : opts->dhs) if (d) extra.push_back(d);
        c->hst = make_hstructure(*t, extra);
        build_forward_plan(*t, c->hst, c->fwd);
        c->dfwd.upload(c->fwd);
        bool want_adj = !opts || opts->build_adjoint;
        if (want_adj) {
            build_adjoint_plan(*t, c->fwd, c->adj);
            c->dadj.upload(c->adj);
            c->has_adj = true;
        }
        size_t nh = c->hst.rows.size();
        CK(cudaMalloc((void **)&c->hval64, sizeof(double2) * nh));
        CK(cudaMalloc((void **)&c->hval32, sizeof(float2) * nh));
        CK(cudaMalloc((void **)&c->hvaldf, sizeof(float4) * nh));
        CK(cudaMalloc((void **)&c->es64, sizeof(double) * 4));
        const cd *hs = reinterpret_cast<const cd *>(t->hs);
        c->hs_host.assign(hs, hs + (size_t)c->nrho * c->nrho);
        if (opts) for (auto *d : opts->dhs) if (d) c->dhs_host.emplace_back(reinterpret_cast<const cd *>(d), reinterpret_cast<const cd *>(d) + (size_t)c->nrho * c->nrho);
        for (int a = 0; a < t->nalf; a++)
            for (int s = 0; s < t->nspin; s++) {
                int slot = a + s * t->nalf;
                c->eleadinfty[slot] = t->eleadinfty[a + (size_t)s * t->nalf];
                c->amps[slot] = opts && opts->amps ? opts->amps[a + (size_t)s * t->nalf] : c->eleadinfty[slot];
                c->tchar[slot] = opts && opts->tchar ? opts->tchar[a + (size_t)s * t->nalf] : 0.0;
            }
        set_params(c.get(), c->hs_host, c->eleadinfty);
        // observables
        int nz0 = t->nnz_spa[0];
        c->rdo_rows.assign(t->irow_spa, t->irow_spa + nz0);
        c->rdo_cols.assign(t->icol_spa, t->icol_spa + nz0);
        {
            // transposed partner of every RDO entry (the pattern of exp(-0.314 H) is symmetric)
            std::vector<int32_t> pos((size_t)t->nrho * t->nrho, -1), pair(nz0);
            for (int q = 0; q < nz0; q++) pos[(t->irow_spa[q] - 1) + (size_t)(t->icol_spa[q] - 1) * t->nrho] = q;
            for (int q = 0; q < nz0; q++) {
                pair[q] = pos[(t->icol_spa[q] - 1) + (size_t)(t->irow_spa[q] - 1) * t->nrho];
                if (pair[q] < 0) fail(HEOM_E_ARG, "RDO sparsity pattern is not symmetric");
                if (pair[q] == q) c->ndiag++;
            }
            c->nz0 = nz0;
            std::vector<int32_t> upper(nz0);
            for (int q = 0; q < nz0; q++) upper[q] = t->icol_spa[q] > t->irow_spa[q];
            CK(cudaMalloc((void **)&c->d_rdo_pair, sizeof(int32_t) * std::max(1, nz0)));
            CK(cudaMemcpy(c->d_rdo_pair, pair.data(), sizeof(int32_t) * nz0, cudaMemcpyHostToDevice));
            CK(cudaMalloc((void **)&c->d_rdo_upper, sizeof(int32_t) * std::max(1, nz0)));
            CK(cudaMemcpy(c->d_rdo_upper, upper.data(), sizeof(int32_t) * nz0, cudaMemcpyHostToDevice));
            // regularising weight: minus the largest bath decay rate |Re cgamma|, a typical
            // diagonal magnitude of the operator; the negative sign puts the regularised
            // directions on the decaying side of the spectrum with the physical ones (about
            // 12 % fewer inner applies than the positive sign on the double-dot models)
            int nvar = 2 * t->norbs * t->nspin * t->nalf * t->ncor;
            const cd *cg = reinterpret_cast<const cd *>(t->cgamma);
            double m = 0;
            for (int k = 0; k < nvar; k++) m = std::max(m, std::abs(cg[k].real()));
            c->reg_scale = m > 0 ? -m : -1.0;
            // Chebyshev spectral width (td/prechebyshev.f90:56-110): spread of Re(sum of the
            // drawers' cgamma) over every ADO of the index table, the RDO (0) included
            double lo = 0.0, hi = 0.0;
            for (int it = 2; it <= t->ntier; it++) {
                const int nb = it - 1;
                for (int64_t a = t->nfirst[it - 1]; a <= t->nlast[it - 1]; a++) {
                    const int32_t *row = t->indextable + (t->ifirst[it - 1] - 1) + (a - t->nfirst[it - 1]) * nb;
                    double g = 0;
                    for (int k = 0; k < nb; k++) g += cg[row[k] - 1].real();
                    lo = std::min(lo, g); hi = std::max(hi, g);
                }
            }
            c->cheby_delta = hi - lo;
        }
        const int n = t->nrho;
        for (int s = 1; s <= t->nspin; s++)
            for (int o = 1; o <= t->norbs; o++) {
                size_t base = (size_t)t->nams * ((o - 1) + (size_t)(s - 1) * t->norbs);
                std::vector<int> cofr(n + 1, 0), sg(n + 1, 0);
                for (int k = 0; k < t->nams; k++) { cofr[t->rowams[base + k]] = t->colams[base + k]; sg[t->rowams[base + k]] = t->sgnams[base + k] ? -1 : 1; }
                // occupation: n_ms = a^+ a is diagonal with ones on the columns holding an element
                std::vector<char> occupied(n + 1, 0);
                for (int k = 0; k < t->nams; k++) occupied[t->colams[base + k]] = 1;
                for (int q = 0; q < nz0; q++)
                    if (t->irow_spa[q] == t->icol_spa[q] && occupied[t->irow_spa[q]]) { c->occ_entry.push_back(q); c->occ_slot.push_back((o - 1) + (s - 1) * t->norbs); }
                // current: tr(a_{ms} rho+) over the first-tier ADOs of every lead and memory component
                for (int al = 1; al <= t->nalf; al++)
                    for (int k = 1; k <= t->ncor; k++) {
                        int iopr = ((s - 1) * t->norbs + o - 1) * t->nalf + al;
                        int d = (iopr - 1) * t->ncor + k;
                        int64_t u = t->nfirst[1] - 1 + t->indexdraw[d - 1];
                        int64_t st = t->ind_spa[u - 1] - 1;
                        for (int q = 0; q < t->nnz_spa[u - 1]; q++) {
                            int r = t->irow_spa[st + q], cc = t->icol_spa[st + q];
                            if (cofr[cc] == r) c->cur_terms.push_back(CurrentTerm{(int32_t)(st + q), (al - 1) + (s - 1) * t->nalf, (float)sg[cc]});
                        }
                    }
            }
        c->n_cur_terms = (int32_t)c->cur_terms.size();
        CK(cudaMalloc((void **)&c->d_cur_terms, sizeof(CurrentTerm) * std::max<size_t>(1, c->cur_terms.size())));
        if (!c->cur_terms.empty()) CK(cudaMemcpy(c->d_cur_terms, c->cur_terms.data(), sizeof(CurrentTerm) * c->cur_terms.size(), cudaMemcpyHostToDevice));
        int64_t N = c->lunk + 1;
        CK(cudaMalloc((void **)&c->dx, sizeof(double2) * N));
        CK(cudaMalloc((void **)&c->dy, sizeof(double2) * N));
        CK(cudaMalloc((void **)&c->dz, sizeof(double2) * N));
        CK(cudaMalloc((void **)&c->fx, sizeof(float2) * N));
        CK(cudaMalloc((void **)&c->fy, sizeof(float2) * N));
        CK(cudaMalloc((void **)&c->dscratch, sizeof(double) * 2048));
        drandn_stream(2 * N, c->rt_host);
        {
            // stored entries before each tier's first ADO (ADOs that store nothing count zero)
            c->tier_entry.assign((size_t)t->ntier + 1, c->lunk);
            int64_t acc = 0, u = 1;
            for (int it = 1; it <= t->ntier; it++) {
                for (; u < t->nfirst[it - 1]; u++) acc += t->nnz_spa[u - 1];
                c->tier_entry[it - 1] = acc;
            }
        }
        // (row, col) of every stored entry, 0-based in one byte each, for the per-ADO dense
        // transforms of the Jacobi sweep; the largest |cb| for its shift
        if (c->nrho <= 256) {
            std::vector<uint16_t> rc((size_t)std::max<int64_t>(1, c->lunk));
            for (int64_t e = 0; e < c->lunk; e++) rc[e] = (uint16_t)((t->irow_spa[e] - 1) | ((t->icol_spa[e] - 1) << 8));
            CK(cudaMalloc((void **)&c->d_ent_rc, sizeof(uint16_t) * rc.size()));
            CK(cudaMemcpy(c->d_ent_rc, rc.data(), sizeof(uint16_t) * rc.size(), cudaMemcpyHostToDevice));
        }
        {
            const size_t ncb = (size_t)t->norbs * t->nspin * t->ncor * t->nalf * 2;
            const cd *cbv = reinterpret_cast<const cd *>(t->cb);
            for (size_t k = 0; k < ncb; k++) c->cb_abs_max = std::max(c->cb_abs_max, std::abs(cbv[k]));
        }
        // the set-up copies above are synchronous copies from pageable memory, whose DMA may
        // still be in flight on return; kernels on the non-blocking stream are not ordered
        // after them, so wait for the whole device once here
        CK(cudaDeviceSynchronize());
        *out = c.release();
    });
}

void heom_ctx_destroy(heom_ctx *ctx)
{
    if (!ctx) return;
    try { heom::DeviceScope dsc(ctx->device); delete ctx; } catch (...) { delete ctx; }
}

int64_t heom_ctx_lunk(const heom_ctx *ctx) { return ctx ? ctx->lunk : -1; }

int heom_calc_ax(heom_ctx *c, int64_t ldim, const double _Complex *x, double _Complex *y)
{
    return guarded([&] {
        require_ctx(c);
        DeviceScope dsc(c->device);
        if (ldim != c->lunk) fail(HEOM_E_ARG, "ldim does not match lunk_spa");
        if (!x || !y) fail(HEOM_E_ARG, "null vector");
        int64_t N = c->lunk + 1;
        CK(cudaMemcpyAsync(c->dx, x, sizeof(double2) * N, cudaMemcpyHostToDevice, c->stream));
        launch_apply<double, false>(c->dfwd.view, ctx_coef<double>(c, false), c->dx, c->dy, 1, N, nullptr, c->stream);
        CK(cudaGetLastError());
        CK(cudaMemcpyAsync(y, c->dy, sizeof(double2) * N, cudaMemcpyDeviceToHost, c->stream));
        CK(cudaStreamSynchronize(c->stream));
    });
}

int heom_calc_ax_dev(heom_ctx *c, const void *dx, void *dy)
{
    return guarded([&] {
        require_ctx(c);
        DeviceScope dsc(c->device);
        launch_apply<double, false>(c->dfwd.view, ctx_coef<double>(c, false), (const double2 *)dx, (double2 *)dy, 1, c->lunk + 1, nullptr, c->stream);
        CK(cudaGetLastError());
        CK(cudaStreamSynchronize(c->stream));
    });
}

int heom_calc_ax_fp32_dev(heom_ctx *c, const void *dx, void *dy)
{
    return guarded([&] {
        require_ctx(c);
        DeviceScope dsc(c->device);
        launch_apply<float, false>(c->dfwd.view, ctx_coef<float>(c, false), (const float2 *)dx, (float2 *)dy, 1, c->lunk + 1, nullptr, c->stream);
        CK(cudaGetLastError());
        CK(cudaStreamSynchronize(c->stream));
    });
}

}  // extern "C"

namespace {
// y = the operator of the mixed-precision inner solves (regularised; rows scaled by the inner
// preconditioner when precond) in the number type T, on device vectors of lunk + 1 values
template <typename T>
void inner_operator(heom_ctx *c, bool precond, const void *dx, void *dy)
{
    const DevPlan &P = c->dfwd.view;
    DevCoef<T> K = regularised<T>(c, ctx_coef<T>(c, false));
    typename Num<T>::V *ws = nullptr;
    float *pre = nullptr;
    CK(cudaMalloc((void **)&ws, sizeof(typename Num<T>::V) * gdiag_elems<T>(P, 1)));
    try {
        fill_gdiag<T>(P, K, ws, 1, c->stream);
        if (precond) {
            CK(cudaMalloc((void **)&pre, sizeof(float) * std::max(1, P.nado)));
            fill_pre(P, c->dfwd.g0_64, hs_inf_norm(c), pre, c->stream);
            K.pre = pre;
        }
        launch_apply<T, false>(P, K, (const typename Num<T>::V *)dx, (typename Num<T>::V *)dy, 1, c->lunk + 1, nullptr,
                               c->stream);
        CK(cudaGetLastError());
        CK(cudaStreamSynchronize(c->stream));
    } catch (...) { cudaFree(ws); if (pre) cudaFree(pre); throw; }
    CK(cudaFree(ws));
    if (pre) CK(cudaFree(pre));
}
}  // namespace

extern "C" {

int heom_calc_ax_inner_dev(heom_ctx *c, int32_t precision, int32_t precond, const void *dx, void *dy)
{
    return guarded([&] {
        require_ctx(c);
        DeviceScope dsc(c->device);
        if (!dx || !dy) fail(HEOM_E_ARG, "null vector");
        if (precision == HEOM_PREC_MIXED) inner_operator<DF>(c, precond != 0, dx, dy);
        else if (precision == HEOM_PREC_MIXED_FP32) inner_operator<float>(c, precond != 0, dx, dy);
        else if (precision == HEOM_PREC_FP64_REFINED || precision == HEOM_PREC_FP64) inner_operator<double>(c, precond != 0, dx, dy);
        else fail(HEOM_E_ARG, "unknown precision");
    });
}

int heom_calc_ax_fp32x2_dev(heom_ctx *c, const void *dx, void *dy)
{
    return guarded([&] {
        require_ctx(c);
        DeviceScope dsc(c->device);
        DevCoef<DF> K = ctx_coef<DF>(c, false);
        float4 *ws = nullptr;
        CK(cudaMalloc((void **)&ws, sizeof(float4) * gdiag_elems<DF>(c->dfwd.view, 1)));
        try {
            fill_gdiag<DF>(c->dfwd.view, K, ws, 1, c->stream);
            launch_apply<DF, false>(c->dfwd.view, K, (const float4 *)dx, (float4 *)dy, 1, c->lunk + 1, nullptr, c->stream);
            CK(cudaGetLastError());
            CK(cudaStreamSynchronize(c->stream));
        } catch (...) { cudaFree(ws); throw; }
        CK(cudaFree(ws));
    });
}

int heom_calc_atrx(heom_ctx *c, int64_t ldim, const double _Complex *x, double _Complex *y)
{
    return guarded([&] {
        require_ctx(c);
        DeviceScope dsc(c->device);
        if (!c->has_adj) fail(HEOM_E_ARG, "context built without the adjoint plan");
        if (ldim != c->lunk) fail(HEOM_E_ARG, "ldim does not match lunk_spa");
        int64_t N = c->lunk + 1;
        CK(cudaMemcpyAsync(c->dx, x, sizeof(double2) * N, cudaMemcpyHostToDevice, c->stream));
        launch_apply<double, true>(c->dadj.view, ctx_coef<double>(c, true), c->dx, c->dy, 1, N, nullptr, c->stream);
        CK(cudaGetLastError());
        CK(cudaMemcpyAsync(y, c->dy, sizeof(double2) * N, cudaMemcpyDeviceToHost, c->stream));
        CK(cudaStreamSynchronize(c->stream));
    });
}

int heom_calc_atrx_dev(heom_ctx *c, const void *dx, void *dy)
{
    return guarded([&] {
        require_ctx(c);
        DeviceScope dsc(c->device);
        if (!c->has_adj) fail(HEOM_E_ARG, "context built without the adjoint plan");
        launch_apply<double, true>(c->dadj.view, ctx_coef<double>(c, true), (const double2 *)dx, (double2 *)dy, 1, c->lunk + 1, nullptr, c->stream);
        CK(cudaGetLastError());
        CK(cudaStreamSynchronize(c->stream));
    });
}

int heom_calcderiv(heom_ctx *c, double t, const double _Complex *x, double _Complex *y)
{
    return guarded([&] {
        require_ctx(c);
        DeviceScope dsc(c->device);
        if (!x || !y) fail(HEOM_E_ARG, "null vector");
        double es[4];
        for (int k = 0; k < 4; k++) {
            double tc = c->tchar[k];
            es[k] = tc > 0 ? c->amps[k] * (1.0 - std::exp(-t / tc)) : (t > 0 ? c->amps[k] : 0.0);
        }
        set_params(c, c->hs_host, es);
        int64_t N = c->lunk + 1;
        CK(cudaMemsetAsync(c->dx, 0, sizeof(double2) * N, c->stream));
        CK(cudaMemcpyAsync(c->dx, x, sizeof(double2) * c->lunk, cudaMemcpyHostToDevice, c->stream));
        DevCoef<double> K = ctx_coef<double>(c, false);
        K.trace_on = 0;
        launch_apply<double, false>(c->dfwd.view, K, c->dx, c->dy, 1, N, nullptr, c->stream);
        CK(cudaGetLastError());
        CK(cudaMemcpyAsync(y, c->dy, sizeof(double2) * c->lunk, cudaMemcpyDeviceToHost, c->stream));
        CK(cudaStreamSynchronize(c->stream));
        set_params(c, c->hs_host, c->eleadinfty);
    });
}

int heom_solve_tfqmr(heom_ctx *c, const heom_solve_opts *o, double _Complex *rho, heom_solve_info *info)
{
    return guarded([&] {
        require_ctx(c);
        DeviceScope dsc(c->device);
        if (!o || !rho) fail(HEOM_E_ARG, "null argument");
        int64_t N = c->lunk + 1;
        std::vector<cd> x(N, 0.0);
        std::memcpy(x.data(), rho, sizeof(cd) * c->lunk);
        herm_rdo(c, x.data());
        CK(cudaMemcpyAsync(c->dz, x.data(), sizeof(double2) * N, cudaMemcpyHostToDevice, c->stream));
        heom_solve_info inf;
        solve_device(c, *o, c->dz, 1, N, false, nullptr, inf, ctx_coefs(c));
        CK(cudaMemcpyAsync(rho, c->dz, sizeof(double2) * c->lunk, cudaMemcpyDeviceToHost, c->stream));
        CK(cudaStreamSynchronize(c->stream));
        if (info) *info = inf;
        if (!inf.converged) fail(inf.ierr == 8 ? HEOM_E_BREAKDOWN : HEOM_E_NOCONV, "TFQMR did not reach crit");
    });
}

int heom_current(heom_ctx *c, const double _Complex *rho, double *jt)
{
    return guarded([&] {
        require_ctx(c);
        const cd *r = reinterpret_cast<const cd *>(rho);
        int ns = c->nalf * c->nspin;
        for (int k = 0; k < ns; k++) jt[k] = 0;
        std::vector<cd> acc(ns, 0.0);
        for (auto &tm : c->cur_terms) acc[tm.slot] += (double)tm.sign * r[tm.entry];
        for (int k = 0; k < ns; k++) jt[k] = -2.0 * acc[k].imag() * kJconst;
    });
}

int heom_occupation(heom_ctx *c, const double _Complex *rho, double *occ)
{
    return guarded([&] {
        require_ctx(c);
        const cd *r = reinterpret_cast<const cd *>(rho);
        for (int k = 0; k < c->norbs * c->nspin; k++) occ[k] = 0;
        for (size_t k = 0; k < c->occ_entry.size(); k++) occ[c->occ_slot[k]] += r[c->occ_entry[k]].real();
    });
}

int heom_batch_create(heom_ctx *c, int32_t nbatch, const double _Complex *hs_batch, const double *eshift_batch,
                      heom_batch **out)
{
    return guarded([&] {
        require_ctx(c);
        DeviceScope dsc(c->device);
        if (nbatch < 1 || !out) fail(HEOM_E_ARG, "bad batch arguments");
        *out = nullptr;
        std::unique_ptr<heom_batch> B(new heom_batch());
        B->ctx = c;
        B->device = c->device;
        B->nbatch = nbatch;
        int64_t N = c->lunk + 1;
        B->vs = (N + 63) / 64 * 64;
        size_t nh = c->hst.rows.size();
        std::vector<double2> h64(nh * nbatch);
        std::vector<float4> hdf(nh * nbatch);
        std::vector<float2> h32(nh * nbatch);
        std::vector<double> e64(4 * (size_t)nbatch, 0.0);
        int all_real = 1;
        for (int b = 0; b < nbatch; b++) {
            const cd *hs = hs_batch ? reinterpret_cast<const cd *>(hs_batch) + (size_t)b * c->nrho * c->nrho : c->hs_host.data();
            std::vector<double2> a64; std::vector<float2> a32; std::vector<float4> adf; int real;
            hvalues(c, hs, a64, a32, adf, real);
            all_real = all_real && real;
            std::copy(a64.begin(), a64.end(), h64.begin() + b * nh);
            std::copy(adf.begin(), adf.end(), hdf.begin() + b * nh);
            std::copy(a32.begin(), a32.end(), h32.begin() + b * nh);
            for (int a = 0; a < c->nalf; a++)
                for (int s = 0; s < c->nspin; s++) {
                    int slot = a + s * c->nalf;
                    e64[4 * b + slot] = eshift_batch ? eshift_batch[(size_t)b * c->nalf * c->nspin + a + (size_t)s * c->nalf] : c->eleadinfty[slot];
                }
        }
        CK(cudaMalloc((void **)&B->h64, sizeof(double2) * h64.size()));
        CK(cudaMalloc((void **)&B->hdf, sizeof(float4) * hdf.size()));
        CK(cudaMalloc((void **)&B->h32, sizeof(float2) * h32.size()));
        CK(cudaMemcpy(B->h32, h32.data(), sizeof(float2) * h32.size(), cudaMemcpyHostToDevice));
        CK(cudaMalloc((void **)&B->e64, sizeof(double) * e64.size()));
        CK(cudaMemcpy(B->h64, h64.data(), sizeof(double2) * h64.size(), cudaMemcpyHostToDevice));
        CK(cudaMemcpy(B->hdf, hdf.data(), sizeof(float4) * hdf.size(), cudaMemcpyHostToDevice));
        CK(cudaMemcpy(B->e64, e64.data(), sizeof(double) * e64.size(), cudaMemcpyHostToDevice));
        B->h_real = all_real;
        CK(cudaDeviceSynchronize());   // the pageable copies above, before any kernel reads them
        *out = B.release();
    });
}

int64_t heom_batch_stride(const heom_batch *b) { return b ? b->vs : -1; }

void heom_batch_destroy(heom_batch *b)
{
    if (!b) return;
    try { heom::DeviceScope dsc(b->device); delete b; } catch (...) { delete b; }
}

int heom_batch_set_tiers(heom_batch *B, const int32_t *ntier)
{
    return guarded([&] {
        if (!B) fail(HEOM_E_ARG, "null batch");
        heom_ctx *c = B->ctx;
        require_ctx(c);
        DeviceScope dsc(c->device);
        if (!ntier) {   // back to the whole hierarchy for every instance
            if (B->tier_lim) cudaFree(B->tier_lim);
            B->tier_lim = nullptr;
            B->tier_lim_host.clear();
            return;
        }
        std::vector<int2> lim(B->nbatch);
        for (int b = 0; b < B->nbatch; b++) {
            const int nt = ntier[b];
            if (nt < 1 || nt > c->ntier)
                fail(HEOM_E_ARG, "instance tier count outside 1 .. the context's ntier");
            lim[b] = make_int2((int)c->tier_entry[nt - 1], (int)c->tier_entry[nt]);
        }
        if (!B->tier_lim) CK(cudaMalloc((void **)&B->tier_lim, sizeof(int2) * B->nbatch));
        CK(cudaMemcpyAsync(B->tier_lim, lim.data(), sizeof(int2) * B->nbatch, cudaMemcpyHostToDevice, c->stream));
        CK(cudaStreamSynchronize(c->stream));
        B->tier_lim_host = lim;
    });
}

int heom_batch_solve_dev(heom_batch *B, const heom_solve_opts *o, void *x_dev, heom_solve_info *info)
{
    return guarded([&] {
        if (!B || !o || !x_dev) fail(HEOM_E_ARG, "null argument");
        heom_ctx *c = B->ctx;
        DeviceScope dsc(c->device);
        DevCoef<double> K64 = c->dfwd.coef<double>(); K64.hval = B->h64; K64.eshift = B->e64; K64.h_real = B->h_real;
        DevCoef<DF> KDF = c->dfwd.coef<DF>(); KDF.hval = B->hdf; KDF.eshift = B->e64; KDF.h_real = B->h_real;
        DevCoef<float> K32 = c->dfwd.coef<float>(); K32.hval = B->h32; K32.eshift = B->e64; K32.h_real = B->h_real;
        if (B->tier_lim) {
            K64.tier_lim = KDF.tier_lim = K32.tier_lim = B->tier_lim;
            // a truncated instance's entries beyond its tier start (and stay) zero
            for (int b = 0; b < B->nbatch; b++) {
                const int64_t y = B->tier_lim_host[b].y;
                if (y < c->lunk)
                    CK(cudaMemsetAsync((double2 *)x_dev + (int64_t)b * B->vs + y, 0, sizeof(double2) * (size_t)(c->lunk - y), c->stream));
            }
        }
        heom_solve_info inf;
        // automatic layout of the mixed solves' inner kernels: the context's first mixed
        // solves of a batch of this size and kind run with each candidate layout; later ones
        // keep the fastest
        heom_solve_opts oo = *o;
        heom_ctx::LayoutTune *tu = nullptr;
        if (oo.precision == HEOM_PREC_MIXED && oo.interleave == 0) {
            tu = &c->il_tune[{B->nbatch, B->tier_lim ? 1 : 0}];
            if (tu->cand.empty()) tu->cand = layout_candidates(B->nbatch, B->tier_lim != nullptr);
            const std::pair<int, int> l = tu->done() ? tu->best() : tu->cand[tu->seconds.size()];
            oo.interleave = l.first;
            oo.lane_instances = l.second;
            if (tu->done()) tu = nullptr;
        }
        solve_device(c, oo, (double2 *)x_dev, B->nbatch, B->vs, false, nullptr, inf, CoefSet{K64, K32, KDF});
        if (tu) tu->seconds.push_back(inf.seconds);
        if (info) *info = inf;
        if (!inf.converged) fail(HEOM_E_NOCONV, "batched TFQMR did not reach crit");
    });
}

int heom_solve_batch(heom_ctx *c, int32_t nbatch, const double _Complex *hs_batch, const double *eshift_batch,
                     const heom_solve_opts *o, double _Complex *rho_batch, heom_solve_info *info)
{
    heom_batch *B = nullptr;
    int rc = heom_batch_create(c, nbatch, hs_batch, eshift_batch, &B);
    if (rc) return rc;
    void *dxb = nullptr;
    rc = guarded([&] {
        if (!o || !rho_batch) fail(HEOM_E_ARG, "null argument");
        DeviceScope dsc(c->device);
        const int64_t vs = B->vs;
        CK(cudaMalloc(&dxb, sizeof(double2) * (size_t)vs * nbatch));
        CK(cudaMemsetAsync(dxb, 0, sizeof(double2) * (size_t)vs * nbatch, c->stream));
        // one strided copy straight from the caller's buffer (DMA at full speed when it is
        // pinned), then the reference's hermitisation of the RDO block on the device
        CK(cudaMemcpy2DAsync(dxb, sizeof(double2) * vs, rho_batch, sizeof(double2) * c->lunk, sizeof(double2) * c->lunk,
                             nbatch, cudaMemcpyHostToDevice, c->stream));
        herm_rdo_upper_dev(c, (double2 *)dxb, nbatch, vs);
        CK(cudaStreamSynchronize(c->stream));
    });
    if (rc == 0) rc = heom_batch_solve_dev(B, o, dxb, info);
    if (rc == 0 || rc == HEOM_E_NOCONV) {
        int rc2 = guarded([&] {
            DeviceScope dsc(c->device);
            CK(cudaMemcpy2DAsync(rho_batch, sizeof(double2) * c->lunk, dxb, sizeof(double2) * B->vs, sizeof(double2) * c->lunk,
                                 nbatch, cudaMemcpyDeviceToHost, c->stream));
            CK(cudaStreamSynchronize(c->stream));
        });
        if (rc == 0) rc = rc2;
    }
    if (dxb) guarded([&] { DeviceScope dsc(c->device); cudaFree(dxb); });
    heom_batch_destroy(B);
    return rc;
}

}  // extern "C"

namespace {

// Device inputs of the measurement hooks: nbatch copies of the context's H values and lead
// shifts, and the matching ADO diagonals of the FP32 / FP32x2 applies.
struct BenchInputs {
    std::vector<void *> blocks;
    void *hv = nullptr, *gdiag = nullptr;
    double *es = nullptr;
    float *pre = nullptr;   // the inner preconditioner of the mixed solves
    ~BenchInputs() { for (void *p : blocks) cudaFree(p); }
    void *alloc(size_t n) { void *p = nullptr; CK(cudaMalloc(&p, n)); blocks.push_back(p); return p; }
};

void bench_inputs(heom_ctx *c, int precision, int nbatch, BenchInputs &I)
{
    const size_t nh = c->hst.rows.size();
    I.hv = I.alloc(16 * std::max<size_t>(1, nh) * nbatch);
    I.es = (double *)I.alloc(sizeof(double) * 4 * nbatch);
    std::vector<double> e(4 * (size_t)nbatch);
    for (int b = 0; b < nbatch; b++) for (int k = 0; k < 4; k++) e[4 * b + k] = c->eleadinfty[k];
    CK(cudaMemcpyAsync(I.es, e.data(), sizeof(double) * e.size(), cudaMemcpyHostToDevice, c->stream));
    std::vector<double2> h64; std::vector<float2> h32; std::vector<float4> hdf; int real;
    hvalues(c, c->hs_host.data(), h64, h32, hdf, real);
    for (int b = 0; b < nbatch; b++) {
        if (precision == HEOM_PREC_FP64 || precision == HEOM_PREC_FP64_REFINED)
            CK(cudaMemcpyAsync((double2 *)I.hv + b * nh, h64.data(), 16 * nh, cudaMemcpyHostToDevice, c->stream));
        else if (precision == HEOM_PREC_MIXED) CK(cudaMemcpyAsync((float4 *)I.hv + b * nh, hdf.data(), 16 * nh, cudaMemcpyHostToDevice, c->stream));
        else CK(cudaMemcpyAsync((float2 *)I.hv + b * nh, h32.data(), 8 * nh, cudaMemcpyHostToDevice, c->stream));
    }
    I.gdiag = I.alloc(16 * (size_t)gdiag_elems<DF>(c->dfwd.view, nbatch));
    if (precision == HEOM_PREC_MIXED || precision == HEOM_PREC_MIXED_FP32) {
        I.pre = (float *)I.alloc(sizeof(float) * std::max(1, c->dfwd.view.nado));
        fill_pre(c->dfwd.view, c->dfwd.g0_64, hs_inf_norm(c), I.pre, c->stream);
    }
    if (precision == HEOM_PREC_MIXED) {
        DevCoef<DF> K = main_coef<DF>(c, false); K.eshift = I.es; K.hval = (const float4 *)I.hv;
        fill_gdiag<DF>(c->dfwd.view, K, (float4 *)I.gdiag, nbatch, c->stream);
    } else if (precision == HEOM_PREC_MIXED_FP32) {
        DevCoef<float> K = main_coef<float>(c, false); K.eshift = I.es;
        fill_gdiag<float>(c->dfwd.view, K, (float2 *)I.gdiag, nbatch, c->stream);
    } else if (precision == HEOM_PREC_FP64_REFINED || precision == HEOM_PREC_FP64) {
        DevCoef<double> K = main_coef<double>(c, false); K.eshift = I.es;
        fill_gdiag<double>(c->dfwd.view, K, (double2 *)I.gdiag, nbatch, c->stream);
    }
    CK(cudaStreamSynchronize(c->stream));
}

// the regularised coefficient set of an inner solve over the measurement inputs
template <typename T> DevCoef<T> bench_coef(heom_ctx *c, const BenchInputs &I)
{
    DevCoef<T> K = regularised<T>(c, main_coef<T>(c, false));
    K.hval = (const typename Num<T>::V *)I.hv;
    K.eshift = I.es;
    K.gdiag = (const typename Num<T>::V *)I.gdiag;
    K.pre = I.pre;
    return K;
}

// the plan's bytes (heom_ctx_stats entry 8)
double plan_bytes(heom_ctx *c)
{
    double st[9];
    heom_ctx_stats(c, st);
    return st[8];
}

// layout (interleave G, instances per lane) of the inner kernels: G = 0 selects the one the
// batch solves of this size use (the tuned one once tuned, else the largest interleave)
template <typename T>
void time_inner(heom_ctx *c, const BenchInputs &I, int nbatch, int reps, double *seconds, double *bytes, int G = 0,
                int ipl = 1)
{
    const int64_t N = c->lunk + 1;
    InnerWork<T> W;
    if (G == 0) {
        ipl = 1;
        auto it = c->il_tune.find({nbatch, 0});
        if (it != c->il_tune.end() && it->second.done()) std::tie(G, ipl) = it->second.best();
    }
    inner_alloc<T>(W, nbatch, N, c->stream, G, ipl);
    try {
        upload_rt_to<T>(c, W.rt, N);
        float mb = 0, ma = 0;
        inner_time<T>(W, c->dfwd.view, bench_coef<T>(c, I), reps, c->stream, mb, ma);
        if (seconds) { seconds[0] = mb * 1e-3; seconds[1] = ma * 1e-3; }
        // algorithmic bytes per launch: the apply's (source read once, result written once per
        // instance, plus the plan), the epilogue's vectors once per instance, r~ once
        const double v = (double)N * sizeof(typename Num<T>::V), pb = plan_bytes(c);
        if (bytes) {
            bytes[0] = nbatch * (2.0 + 10.0) * v + v + pb;   // B: reads u2 y v d x, writes y v d x
            bytes[1] = nbatch * (2.0 + 3.0) * v + v + pb;    // A: reads u1 w, writes w
        }
    } catch (...) { inner_free(W); throw; }
    inner_free(W);
}

}  // namespace

extern "C" {

int heom_bench_apply(heom_ctx *c, int32_t precision, int32_t nbatch, int32_t reps, double *seconds, double *bytes)
{
    return guarded([&] {
        require_ctx(c);
        DeviceScope dsc(c->device);
        if (reps < 1) reps = 1;
        if (nbatch < 1) nbatch = 1;
        const int64_t N = c->lunk + 1, vs = (N + 63) / 64 * 64;
        BenchInputs I;
        bench_inputs(c, precision, nbatch, I);
        void *xin = I.alloc(16 * (size_t)vs * nbatch), *yout = I.alloc(16 * (size_t)vs * nbatch);
        CK(cudaMemsetAsync(xin, 0, 16 * (size_t)vs * nbatch, c->stream));
        // the apply of each solver precision: FP64, and the regularised FP32 / FP32x2 applies
        // of the mixed-precision inner solves
        auto run = [&] {
            if (precision == HEOM_PREC_FP64) {
                DevCoef<double> K = main_coef<double>(c, false); K.hval = (double2 *)I.hv; K.eshift = I.es;
                K.gdiag = (const double2 *)I.gdiag;
                launch_apply<double, false>(c->dfwd.view, K, (double2 *)xin, (double2 *)yout, nbatch, vs, nullptr, c->stream);
            } else if (precision == HEOM_PREC_MIXED) {
                launch_apply<DF, false>(c->dfwd.view, bench_coef<DF>(c, I), (float4 *)xin, (float4 *)yout, nbatch, vs, nullptr, c->stream);
            } else if (precision == HEOM_PREC_MIXED_FP32) {
                launch_apply<float, false>(c->dfwd.view, bench_coef<float>(c, I), (float2 *)xin, (float2 *)yout, nbatch, vs, nullptr, c->stream);
            } else fail(HEOM_E_ARG, "unknown precision");
        };
        cudaEvent_t e0, e1;
        CK(cudaEventCreate(&e0)); CK(cudaEventCreate(&e1));
        for (int w = 0; w < 3; w++) run();
        CK(cudaEventRecord(e0, c->stream));
        for (int r = 0; r < reps; r++) run();
        CK(cudaEventRecord(e1, c->stream));
        CK(cudaEventSynchronize(e1));
        CK(cudaGetLastError());
        float ms = 0;
        cudaEventElapsedTime(&ms, e0, e1);
        cudaEventDestroy(e0); cudaEventDestroy(e1);
        if (seconds) *seconds = ms * 1e-3 / reps;
        const double s = precision == HEOM_PREC_MIXED_FP32 ? 8.0 : 16.0;
        // algorithmic bytes of one launch: x read once, y written once per instance, plus the plan
        if (bytes) *bytes = nbatch * 2.0 * (double)N * s + plan_bytes(c);
    });
}

int heom_bench_inner(heom_ctx *c, int32_t precision, int32_t nbatch, int32_t reps, double *seconds, double *bytes)
{
    return guarded([&] {
        require_ctx(c);
        DeviceScope dsc(c->device);
        if (reps < 1) reps = 1;
        if (nbatch < 1) nbatch = 1;
        BenchInputs I;
        bench_inputs(c, precision, nbatch, I);
        if (precision == HEOM_PREC_MIXED) time_inner<DF>(c, I, nbatch, reps, seconds, bytes);
        else if (precision == HEOM_PREC_MIXED_FP32) time_inner<float>(c, I, nbatch, reps, seconds, bytes);
        else if (precision == HEOM_PREC_FP64_REFINED) time_inner<double>(c, I, nbatch, reps, seconds, bytes);
        else fail(HEOM_E_ARG, "heom_bench_inner: precision must be one of the refined (inner-solve) precisions");
    });
}

int heom_bench_inner_layout(heom_ctx *c, int32_t nbatch, int32_t reps, int32_t interleave, int32_t lane_instances,
                            double *seconds, double *bytes)
{
    return guarded([&] {
        require_ctx(c);
        DeviceScope dsc(c->device);
        if (reps < 1) reps = 1;
        if (nbatch < 1) nbatch = 1;
        if (interleave < 1) fail(HEOM_E_ARG, "heom_bench_inner_layout: interleave must be 1 or a power of two up to 32");
        if (lane_instances == 2 && interleave < 2) fail(HEOM_E_ARG, "two instances per lane need interleave >= 2");
        BenchInputs I;
        bench_inputs(c, HEOM_PREC_MIXED, nbatch, I);
        time_inner<DF>(c, I, nbatch, reps, seconds, bytes, interleave, lane_instances);
    });
}

int heom_tuned_layout(heom_ctx *c, int32_t nbatch, int32_t truncated, int32_t *interleave, int32_t *lane_instances)
{
    return guarded([&] {
        require_ctx(c);
        if (!interleave || !lane_instances) fail(HEOM_E_ARG, "null argument");
        *interleave = 0;
        *lane_instances = 0;
        const auto cand = layout_candidates(nbatch, truncated != 0);
        if (cand.size() == 1) { *interleave = cand[0].first; *lane_instances = cand[0].second; return; }
        auto it = c->il_tune.find({nbatch, truncated ? 1 : 0});
        if (it != c->il_tune.end() && it->second.done()) std::tie(*interleave, *lane_instances) = it->second.best();
    });
}

int heom_ctx_stats(const heom_ctx *c, double *out)
{
    return guarded([&] {
        if (!c || !out) fail(HEOM_E_ARG, "null argument");
        const HostPlan &P = c->fwd;
        double lower = 0;
        for (int32_t a = 0; a < P.nado; a++) {
            int nz = P.ado_off[a + 1] - P.ado_off[a];
            for (int e = P.coup_ptr[a]; e < P.coup_ptr[a + 1]; e++) {
                if (P.coup[e].cid & kCoefUnit) continue;
                for (int p = 0; p < nz; p++) {
                    uint32_t w = P.maps[P.coup[e].map_base + p];
                    lower += ((w & 0xFFFFu) != 0) + ((w >> 16) != 0);
                }
            }
        }
        out[0] = (double)(P.lunk + 1);
        out[1] = P.nado;
        out[2] = (double)P.n_classes;
        out[3] = (double)P.n_couplings;
        out[4] = (double)P.n_maps;
        out[5] = P.gather_hits;
        out[6] = (double)P.n_terms_same;
        out[7] = lower;
        out[8] = plan_read_bytes(P);
    });
}

}  // extern "C"
