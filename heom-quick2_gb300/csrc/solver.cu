// Batched TFQMR on the device.
//
// The vector updates, inner products and stopping tests are those of the TFQMR
// algorithm of R. W. Freund (SIAM J. Sci. Comput. 14 (1993) 470) in the column
// roles and tolerances of tfqmr_double/dutfx.f90: 1 x, 2 b, 3 shadow r~, 4 v, 5 w,
// 6 y, 7 d, 8 A y (u), 9 scratch (t).  Vector arithmetic runs in the number type T
// (FP64, FP32 or FP32x2); inner products are summed in FP64 across threads.  A reduction
// kernel writes one partial per block; a one-block-per-instance finaliser (k_*_fin) sums
// them in a fixed order (deterministic) and updates that instance's scalars.  Vector
// kernels skip instances that have finished, so one launch sequence serves a batch of
// independent solves and can be captured in a CUDA graph.
#include <cstdio>

#include "solver.cuh"

namespace heom {

namespace {

constexpr int NT = 256;

__device__ __forceinline__ double2 block_sum2(double a, double c)
{
    __shared__ double sa[NT / 32], sc[NT / 32];
    for (int o = 16; o > 0; o >>= 1) {
        a += __shfl_down_sync(0xffffffffu, a, o);
        c += __shfl_down_sync(0xffffffffu, c, o);
    }
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) { sa[wid] = a; sc[wid] = c; }
    __syncthreads();
    double2 r = make_double2(0, 0);
    if (wid == 0) {
        a = lane < NT / 32 ? sa[lane] : 0.0;
        c = lane < NT / 32 ? sc[lane] : 0.0;
        for (int o = 16; o > 0; o >>= 1) {
            a += __shfl_down_sync(0xffffffffu, a, o);
            c += __shfl_down_sync(0xffffffffu, c, o);
        }
        r = make_double2(a, c);
    }
    return r;   // valid in thread 0
}

// Per-block partial sums of a reduction (written by thread 0; no atomics, no fences).
template <typename T>
__device__ void write_partial(const TfqWork<T> &W, int b, double a, double c)
{
    const double2 r = block_sum2(a, c);
    if (threadIdx.x == 0) {
        double *pp = W.part + 2 * ((size_t)b * W.nblk + blockIdx.x);
        pp[0] = r.x;
        pp[1] = r.y;
    }
}

// In the one-block-per-instance kernel that follows a reduction: the grand totals, summed
// in a fixed order (deterministic), valid in thread 0.
template <typename T>
__device__ bool gather_partials(const TfqWork<T> &W, int b, double &ta, double &tc)
{
    double sa = 0, sc = 0;
    for (int k = threadIdx.x; k < W.nblk; k += NT) {
        sa += W.part[2 * ((size_t)b * W.nblk + k)];
        sc += W.part[2 * ((size_t)b * W.nblk + k) + 1];
    }
    const double2 r = block_sum2(sa, sc);
    if (threadIdx.x == 0) { ta = r.x; tc = r.y; return true; }
    return false;
}

__device__ void set_flags(const TfqState &S, int *am, int *at, int *ac, int b)
{
    am[b] = !S.done;
    at[b] = S.tres && !S.done;
    ac[b] = S.chk && !S.done;
}

// Before apply number k the reference driver tests ||A x - b|| <= crit when k % 50 == 0
// (solve_tfqmr.f90:200-217); the test is taken at the start of the iteration holding k.
__device__ void schedule_check(TfqState &S)
{
    int a = S.axb % 50;
    S.chk = (a == 0 || a == 49);
}

__device__ void advance(TfqState &S)
{
    S.n += 1;
    S.beta = S.rho_next / S.rho;
    S.rho = S.rho_next;
    schedule_check(S);
}

// Per-thread accumulation of the real inner product Re(a^H b): FP64 for FP64 vectors,
// FP32 for FP32 vectors, FP32x2 (on the FP32 pipe) for FP32x2 vectors; the per-thread
// values are summed in FP64 across the grid.
template <typename T> struct DotAcc {
    double v = 0;
    __device__ __forceinline__ void add(typename Num<T>::A a, typename Num<T>::A b)
    { v += Num<T>::re(a) * Num<T>::re(b) + Num<T>::im(a) * Num<T>::im(b); }
    __device__ __forceinline__ double val() const { return v; }
};
template <> struct DotAcc<float> {   // a few elements per thread: FP32 partial sums
    float v = 0.f;
    __device__ __forceinline__ void add(float2 a, float2 b) { v = fmaf(a.x, b.x, fmaf(a.y, b.y, v)); }
    __device__ __forceinline__ double val() const { return (double)v; }
};
template <> struct DotAcc<DF> {
    f2r v{0.f, 0.f};
    // operands normalised first: lazy sums may carry |lo| >= |hi| after cancellation
    __device__ __forceinline__ void add(f2c a, f2c b)
    {
        a = Num<DF>::norm(a);
        b = Num<DF>::norm(b);
        v = f2r_add(v, f2r_add(f2r_mul(a.re, b.re), f2r_mul(a.im, b.im)));
    }
    __device__ __forceinline__ double val() const { return (double)v.hi + (double)v.lo; }
};

#define INST_SETUP                                  \
    using NN = Num<T>;                              \
    using AA = typename NN::A;                      \
    const int b = blockIdx.y;                       \
    TfqState *S = W.st + b;                         \
    const int64_t o = (int64_t)b * W.vstride;       \
    const int64_t i0 = (int64_t)blockIdx.x * NT + threadIdx.x, di = (int64_t)W.nblk * NT;

// restrict-qualified views of this instance's vectors: lets the compiler overlap the loads
// of successive elements with the stores of earlier ones
#define VIEWS                                                               \
    using VV = typename NN::V;                                              \
    VV *__restrict__ x_ = W.x + o, *__restrict__ v_ = W.v + o, *__restrict__ w_ = W.w + o; \
    VV *__restrict__ y_ = W.y + o, *__restrict__ d_ = W.d + o, *__restrict__ s_ = W.s + o; \
    const VV *__restrict__ u_ = W.u + o, *__restrict__ t_ = W.t + o;      \
    const VV *__restrict__ b_ = W.b + o, *__restrict__ rt_ = W.rt;        \
    (void)x_; (void)v_; (void)w_; (void)y_; (void)d_; (void)s_; (void)u_; (void)t_; (void)b_; (void)rt_;

template <typename T>
__global__ void k_init(TfqWork<T> W, double tol, int nlim, double crit, double rel_crit, int stag_window)
{
    INST_SETUP
    DotAcc<T> bb, rb;
    for (int64_t i = i0; i < W.N; i += di) {
        const AA bv = NN::load(W.b[o + i]), r = NN::load(W.rt[shadow_index(W.tier_lim, b, i, W.N)]);
        const typename NN::V z = NN::store(NN::zero());
        W.x[o + i] = z; W.v[o + i] = z; W.y[o + i] = z; W.d[o + i] = z; W.u[o + i] = z;
        W.w[o + i] = NN::store(bv);
        bb.add(bv, bv);
        rb.add(r, bv);
    }
    write_partial(W, b, bb.val(), rb.val());
}

template <typename T>
__global__ void k_init_fin(TfqWork<T> W, double tol, int nlim, double crit, double rel_crit, int stag_window)
{
    const int b = blockIdx.x;
    TfqState *S = W.st + b;
    (void)S;
    double tb, trb;
    if (gather_partials(W, b, tb, trb)) {
        TfqState s = {};
        s.r0 = sqrt(tb);
        s.tol = tol; s.nlim = nlim; s.stag_window = stag_window;
        s.crit = fmax(crit, rel_crit * s.r0);
        s.ext_resid = s.r0;
        s.best = s.r0;
        if (tol >= 1.0 || s.r0 == 0.0) { s.done = 1; s.ierr = 0; }
        else {
            s.n = 1; s.resn = 1; s.rho = 1; s.var = 0; s.eta = 0; s.tau = s.r0 * s.r0; s.ierr = 8;
            s.rho_next = trb; s.beta = trb / s.rho; s.rho = trb;
            s.axb = 0;
            schedule_check(s);
        }
        *S = s;
        set_flags(s, W.act_main, W.act_tres, W.act_chk, b);
    }
}

// x += xpend d; y = w + beta y   (the v update of this half step is done in k_p2)
template <typename T>
__global__ void k_p1(TfqWork<T> W)
{
    INST_SETUP
    if (S->done) return;
    VIEWS
    const auto beta = NN::sc(S->beta), xe = NN::sc(S->xpend);
#pragma unroll 2
    for (int64_t i = i0; i < W.N; i += di) {
        const AA d = NN::load(d_[i]);
        x_[i] = NN::store(NN::add(NN::load(x_[i]), NN::scale(d, xe)));
        y_[i] = NN::store(NN::add(NN::load(w_[i]), NN::scale(NN::load(y_[i]), beta)));
    }
}

// every-50-applies check: ||s - b||, s = A x
template <typename T>
__global__ void k_chk(TfqWork<T> W)
{
    INST_SETUP
    if (!W.act_chk[b]) return;
    DotAcc<T> ss;
    for (int64_t i = i0; i < W.N; i += di) {
        const AA e = NN::sub(NN::load(W.s[o + i]), NN::load(W.b[o + i]));
        ss.add(e, e);
    }
    write_partial(W, b, ss.val(), 0.0);
}

template <typename T>
__global__ void k_chk_fin(TfqWork<T> W)
{
    const int b = blockIdx.x;
    TfqState *S = W.st + b;
    (void)S;
    if (!W.act_chk[b]) return;
    double t, dummy;
    if (gather_partials(W, b, t, dummy)) {
        TfqState st = *S;
        st.ext_resid = sqrt(t);
        st.chk = 0;
        if (st.ext_resid <= st.crit) { st.done = 1; st.conv_ext = 1; }
        else if (st.stag_window) {
            // inner solve of a refinement: hand back to the FP64 refinement once the arithmetic's
            // floor is reached, seen either as the true residual running 10x above TFQMR's own
            // bound sqrt(2n+1) tau (the recursion has drifted from the true residual), or as
            // stag_window consecutive tests that fail to halve the best true residual
            if (st.n > 2 && st.ext_resid > 10.0 * st.unrm * st.r0) { st.done = 1; st.ierr = 4; }
            else if (st.ext_resid < 0.5 * st.best) { st.best = st.ext_resid; st.stag = 0; }
            else if (++st.stag >= st.stag_window) { st.done = 1; st.ierr = 4; }
        }
        *S = st;
        set_flags(st, W.act_main, W.act_tres, W.act_chk, b);
    }
}

// v = beta (beta v + u) + t; sigma = <r~, v>   (u = A y of the previous half step)
template <typename T>
__global__ void k_p2(TfqWork<T> W)
{
    INST_SETUP
    if (S->done) return;
    VIEWS
    const auto beta = NN::sc(S->beta);
    DotAcc<T> sg;
#pragma unroll 2
    for (int64_t i = i0; i < W.N; i += di) {
        const AA vu = NN::add(NN::scale(NN::load(v_[i]), beta), NN::load(u_[i]));
        const AA v = NN::add(NN::scale(vu, beta), NN::load(t_[i]));
        v_[i] = NN::store(v);
        sg.add(NN::load(rt_[shadow_index(W.tier_lim, b, i, W.N)]), v);
    }
    write_partial(W, b, sg.val(), 0.0);
}

template <typename T>
__global__ void k_p2_fin(TfqWork<T> W)
{
    const int b = blockIdx.x;
    TfqState *S = W.st + b;
    (void)S;
    if (S->done) return;
    double sigma, dummy;
    if (gather_partials(W, b, sigma, dummy)) {
        TfqState s = *S;
        s.axb += 1;
        if (sigma == 0.0 || s.rho == 0.0) { s.ierr = 8; s.done = 1; }
        else { s.alpha = s.rho / sigma; s.dd = s.var * s.eta / s.alpha; s.xpend = 0; }
        *S = s;
        set_flags(s, W.act_main, W.act_tres, W.act_chk, b);
    }
}

// d = y + dd d; w = w - alpha t; ||w||^2  -> var, cos, tau, eta, unrm
template <typename T>
__global__ void k_p3(TfqWork<T> W)
{
    INST_SETUP
    if (S->done) return;
    VIEWS
    const auto dd = NN::sc(S->dd), al = NN::sc(S->alpha);
    DotAcc<T> ww;
#pragma unroll 2
    for (int64_t i = i0; i < W.N; i += di) {
        d_[i] = NN::store(NN::add(NN::load(y_[i]), NN::scale(NN::load(d_[i]), dd)));
        const AA w = NN::sub(NN::load(w_[i]), NN::scale(NN::load(t_[i]), al));
        w_[i] = NN::store(w);
        ww.add(w, w);
    }
    write_partial(W, b, ww.val(), 0.0);
}

template <typename T>
__global__ void k_p3_fin(TfqWork<T> W)
{
    const int b = blockIdx.x;
    TfqState *S = W.st + b;
    (void)S;
    if (S->done) return;
    double tw, dummy;
    if (gather_partials(W, b, tw, dummy)) {
        TfqState s = *S;
        s.var = tw / s.tau; s.cosv = 1.0 / (1.0 + s.var); s.tau = tw * s.cosv; s.eta = s.alpha * s.cosv;
        s.xpend = s.eta;
        s.unrm = sqrt((double)(2 * s.n) * s.tau) / s.r0;
        s.uchk = s.unrm;
        s.tres = !(s.unrm / s.tol > 10.0);
        if (!s.tres && s.resn <= s.tol) { s.ierr = 0; s.done = 1; }
        *S = s;
        set_flags(s, W.act_main, W.act_tres, W.act_chk, b);
    }
}

// true residual path: x += xpend d
template <typename T>
__global__ void k_tx(TfqWork<T> W)
{
    INST_SETUP
    if (!W.act_tres[b]) return;
    const auto xe = NN::sc(S->xpend);
    for (int64_t i = i0; i < W.N; i += di)
        W.x[o + i] = NN::store(NN::add(NN::load(W.x[o + i]), NN::scale(NN::load(W.d[o + i]), xe)));
}

// s = b - A x; resn = ||s|| / r0, then the stopping tests of the half step
template <typename T>
__global__ void k_tr(TfqWork<T> W, int second_half)
{
    INST_SETUP
    if (!W.act_tres[b]) return;
    DotAcc<T> ss;
    for (int64_t i = i0; i < W.N; i += di) {
        const AA s = NN::sub(NN::load(W.b[o + i]), NN::load(W.s[o + i]));
        W.s[o + i] = NN::store(s);
        ss.add(s, s);
    }
    write_partial(W, b, ss.val(), 0.0);
}

template <typename T>
__global__ void k_tr_fin(TfqWork<T> W, int second_half)
{
    const int b = blockIdx.x;
    TfqState *S = W.st + b;
    (void)S;
    if (!W.act_tres[b]) return;
    double t, dummy;
    if (gather_partials(W, b, t, dummy)) {
        TfqState st = *S;
        st.xpend = 0; st.axb += 1; st.tres = 0;
        st.resn = sqrt(t) / st.r0;
        st.uchk = second_half ? st.unrm : st.resn;
        if (st.resn <= st.tol) { st.ierr = 0; st.done = 1; }
        else if (st.unrm < st.uchk / 100.0) { st.ierr = 4; st.done = 1; }
        else if (second_half && st.n >= st.nlim) { st.ierr = 4; st.done = 1; }
        else if (second_half) advance(st);
        *S = st;
        set_flags(st, W.act_main, W.act_tres, W.act_chk, b);
    }
}

// x += xpend d (old d); y = y - alpha v; d = y + var cos d
template <typename T>
__global__ void k_p4(TfqWork<T> W)
{
    INST_SETUP
    if (S->done) return;
    VIEWS
    const auto xe = NN::sc(S->xpend), al = NN::sc(S->alpha), vc = NN::sc(S->var * S->cosv);
#pragma unroll 2
    for (int64_t i = i0; i < W.N; i += di) {
        const AA d = NN::load(d_[i]);
        x_[i] = NN::store(NN::add(NN::load(x_[i]), NN::scale(d, xe)));
        const AA y = NN::sub(NN::load(y_[i]), NN::scale(NN::load(v_[i]), al));
        y_[i] = NN::store(y);
        d_[i] = NN::store(NN::add(y, NN::scale(d, vc)));
    }
}

// w = w - alpha u; ||w||^2 and <r~, w>
template <typename T>
__global__ void k_p5(TfqWork<T> W)
{
    INST_SETUP
    if (S->done) return;
    VIEWS
    const auto al = NN::sc(S->alpha);
    DotAcc<T> ww, rw;
#pragma unroll 2
    for (int64_t i = i0; i < W.N; i += di) {
        const AA w = NN::sub(NN::load(w_[i]), NN::scale(NN::load(u_[i]), al));
        w_[i] = NN::store(w);
        ww.add(w, w);
        rw.add(NN::load(rt_[shadow_index(W.tier_lim, b, i, W.N)]), w);
    }
    write_partial(W, b, ww.val(), rw.val());
}

template <typename T>
__global__ void k_p5_fin(TfqWork<T> W)
{
    const int b = blockIdx.x;
    TfqState *S = W.st + b;
    (void)S;
    if (S->done) return;
    double tw, trw;
    if (gather_partials(W, b, tw, trw)) {
        TfqState s = *S;
        s.axb += 1;
        s.var = tw / s.tau; s.cosv = 1.0 / (1.0 + s.var); s.tau = tw * s.cosv; s.eta = s.alpha * s.cosv;
        s.xpend = s.eta;
        s.unrm = sqrt((double)(2 * s.n + 1) * s.tau) / s.r0;
        s.uchk = s.unrm;
        s.rho_next = trw;
        s.tres = !((s.unrm / s.tol > 10.0) && (s.n < s.nlim));
        if (!s.tres) {
            if (s.resn <= s.tol) { s.ierr = 0; s.done = 1; }
            else advance(s);
        }
        *S = s;
        set_flags(s, W.act_main, W.act_tres, W.act_chk, b);
    }
}

template <typename T>
__global__ void k_axpby(int64_t n, typename Num<T>::V *z, double a, const typename Num<T>::V *x, double bb,
                        const typename Num<T>::V *y)
{
    using NN = Num<T>;
    const auto as = NN::sc(a), bs = NN::sc(bb);
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        z[i] = NN::store(NN::add(NN::scale(NN::load(x[i]), as), NN::scale(NN::load(y[i]), bs)));
}

// conversions between FP64 vectors and the number type of a solver
template <typename T>
__global__ void k_from_d(int64_t n, const double2 *in, typename Num<T>::V *out, double scale)
{
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        out[i] = Num<T>::store(Num<T>::from_d(in[i].x * scale, in[i].y * scale));
}
template <typename T>
__global__ void k_axpy_to_d(int64_t n, double2 *y, double a, const typename Num<T>::V *x)
{
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const typename Num<T>::A v = Num<T>::load(x[i]);
        y[i].x += a * Num<T>::re(v);
        y[i].y += a * Num<T>::im(v);
    }
}

__global__ void k_norm2(int64_t n, const double2 *x, double *out)
{
    double s = 0;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        s += x[i].x * x[i].x + x[i].y * x[i].y;
    double2 r = block_sum2(s, 0.0);
    if (threadIdx.x == 0) out[blockIdx.x] = r.x;
}

__global__ void k_dot(int64_t n, const double2 *a, const double2 *b, double *out)
{
    double s = 0;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        s += a[i].x * b[i].x + a[i].y * b[i].y;
    double2 r = block_sum2(s, 0.0);
    if (threadIdx.x == 0) out[blockIdx.x] = r.x;
}

int grid_for(int64_t n) { int64_t g = (n + NT - 1) / NT; return (int)(g < 1 ? 1 : (g > 1216 ? 1216 : g)); }

}  // namespace

template <typename T>
void tfq_alloc(TfqWork<T> &W, int nbatch, int64_t N, cudaStream_t s)
{
    using V = typename Num<T>::V;
    W.nbatch = nbatch;
    W.N = N;
    W.vstride = (N + 63) / 64 * 64;
    // about four elements per thread and instance, at most 296 blocks (2 per SM) per instance
    int64_t nb = (N + 4 * NT - 1) / (4 * NT);
    W.nblk = (int)(nb < 1 ? 1 : (nb > 296 ? 296 : nb));
    size_t vbytes = sizeof(V) * (size_t)W.vstride * nbatch;
    // every piece starts on a 256-byte boundary; the size is the sum of the rounded pieces
    auto rounded = [](size_t b) { return (b + 255) / 256 * 256; };
    const size_t total = rounded(vbytes) * 9 + rounded(sizeof(V) * (size_t)W.vstride) + rounded(sizeof(TfqState) * nbatch) +
                         rounded(sizeof(double) * 2 * (size_t)nbatch * W.nblk) +
                         3 * rounded(sizeof(int) * nbatch);
    char *p = nullptr;
    if (cudaMalloc((void **)&p, total) != cudaSuccess) fail(HEOM_E_NOMEM, "device allocation of the TFQMR workspace failed");
    // cleared on the solver's stream (no device-wide synchronisation, which would collide with
    // graph captures of other contexts), finished before first use
    if (cudaMemsetAsync(p, 0, total, s) != cudaSuccess || cudaStreamSynchronize(s) != cudaSuccess) {
        cudaFree(p);
        fail(HEOM_E_CUDA, "clearing the TFQMR workspace failed");
    }
    W.mem = p;
    auto take = [&](size_t bytes) { char *q = p; p += rounded(bytes); return q; };
    W.x = (V *)take(vbytes); W.b = (V *)take(vbytes); W.v = (V *)take(vbytes); W.w = (V *)take(vbytes);
    W.y = (V *)take(vbytes); W.d = (V *)take(vbytes); W.u = (V *)take(vbytes); W.t = (V *)take(vbytes);
    W.s = (V *)take(vbytes);
    W.rt = (V *)take(sizeof(V) * (size_t)W.vstride);
    W.st = (TfqState *)take(sizeof(TfqState) * nbatch);
    W.part = (double *)take(sizeof(double) * 2 * (size_t)nbatch * W.nblk);
    W.act_main = (int *)take(sizeof(int) * nbatch);
    W.act_tres = (int *)take(sizeof(int) * nbatch);
    W.act_chk = (int *)take(sizeof(int) * nbatch);
}

template <typename T>
void tfq_free(TfqWork<T> &W)
{
    if (W.mem) cudaFree(W.mem);
    W = TfqWork<T>();
}

template <typename T>
void tfq_start(TfqWork<T> &W, double tol, int nlim, double crit, double rel_crit, int stag_window, cudaStream_t s)
{
    dim3 g(W.nblk, W.nbatch);
    k_init<T><<<g, NT, 0, s>>>(W, tol, nlim, crit, rel_crit, stag_window);
    k_init_fin<T><<<W.nbatch, NT, 0, s>>>(W, tol, nlim, crit, rel_crit, stag_window);
}

template <typename T>
void tfq_iteration(TfqWork<T> &W, const ApplyFn<T> &apply, cudaStream_t s)
{
    dim3 g(W.nblk, W.nbatch);
    const unsigned nb = (unsigned)W.nbatch;
    k_p1<T><<<g, NT, 0, s>>>(W);
    apply(W.x, W.s, W.act_chk);            // residual test every 50 applies
    k_chk<T><<<g, NT, 0, s>>>(W);
    k_chk_fin<T><<<nb, NT, 0, s>>>(W);
    apply(W.y, W.t, W.act_main);           // t = A y_{2n-1}
    k_p2<T><<<g, NT, 0, s>>>(W);
    k_p2_fin<T><<<nb, NT, 0, s>>>(W);
    k_p3<T><<<g, NT, 0, s>>>(W);
    k_p3_fin<T><<<nb, NT, 0, s>>>(W);
    k_tx<T><<<g, NT, 0, s>>>(W);
    apply(W.x, W.s, W.act_tres);
    k_tr<T><<<g, NT, 0, s>>>(W, 0);
    k_tr_fin<T><<<nb, NT, 0, s>>>(W, 0);
    k_p4<T><<<g, NT, 0, s>>>(W);
    apply(W.y, W.u, W.act_main);           // u = A y_{2n}
    k_p5<T><<<g, NT, 0, s>>>(W);
    k_p5_fin<T><<<nb, NT, 0, s>>>(W);
    k_tx<T><<<g, NT, 0, s>>>(W);
    apply(W.x, W.s, W.act_tres);
    k_tr<T><<<g, NT, 0, s>>>(W, 1);
    k_tr_fin<T><<<nb, NT, 0, s>>>(W, 1);
}

template <typename T>
void vec_axpby(int64_t n, typename Num<T>::V *z, double a, const typename Num<T>::V *x, double bb,
               const typename Num<T>::V *y, cudaStream_t s)
{
    k_axpby<T><<<grid_for(n), NT, 0, s>>>(n, z, a, x, bb, y);
}

template <typename T>
void vec_from_d(int64_t n, const double2 *in, typename Num<T>::V *out, double scale, cudaStream_t s)
{
    k_from_d<T><<<grid_for(n), NT, 0, s>>>(n, in, out, scale);
}

template <typename T>
void vec_axpy_to_d(int64_t n, double2 *y, double a, const typename Num<T>::V *x, cudaStream_t s)
{
    k_axpy_to_d<T><<<grid_for(n), NT, 0, s>>>(n, y, a, x);
}

double device_norm2(int64_t n, const double2 *x, double *scratch, cudaStream_t s)
{
    int g = grid_for(n);
    if (g > 1024) g = 1024;
    k_norm2<<<g, NT, 0, s>>>(n, x, scratch);
    std::vector<double> h(g);
    cudaMemcpyAsync(h.data(), scratch, sizeof(double) * g, cudaMemcpyDeviceToHost, s);
    cudaStreamSynchronize(s);
    double t = 0;
    for (double v : h) t += v;
    return std::sqrt(t);
}

double device_dot(int64_t n, const double2 *a, const double2 *b, double *scratch, cudaStream_t s)
{
    int g = grid_for(n);
    if (g > 1024) g = 1024;
    k_dot<<<g, NT, 0, s>>>(n, a, b, scratch);
    std::vector<double> h(g);
    cudaMemcpyAsync(h.data(), scratch, sizeof(double) * g, cudaMemcpyDeviceToHost, s);
    cudaStreamSynchronize(s);
    double t = 0;
    for (double v : h) t += v;
    return t;
}

#define INST(T)                                                                                                 \
    template void tfq_alloc<T>(TfqWork<T> &, int, int64_t, cudaStream_t);                                      \
    template void tfq_free<T>(TfqWork<T> &);                                                                    \
    template void tfq_start<T>(TfqWork<T> &, double, int, double, double, int, cudaStream_t);                   \
    template void tfq_iteration<T>(TfqWork<T> &, const ApplyFn<T> &, cudaStream_t);                             \
    template void vec_axpby<T>(int64_t, Num<T>::V *, double, const Num<T>::V *, double, const Num<T>::V *,      \
                               cudaStream_t);                                                                   \
    template void vec_from_d<T>(int64_t, const double2 *, Num<T>::V *, double, cudaStream_t);                   \
    template void vec_axpy_to_d<T>(int64_t, double2 *, double, const Num<T>::V *, cudaStream_t);
INST(double)
INST(float)
INST(DF)

}  // namespace heom
