// Fused batched TFQMR for the inner solves of mixed-precision refinement (see inner.cuh
// for the arrangement of the iteration).
#include <cmath>
#include <functional>
#include <string>

#include "apply_entry.cuh"
#include "inner.cuh"

namespace heom {

namespace {

constexpr int NT = 256;
// entries per thread: the per-thread fixed costs (flags, scalars, the warp reductions of the
// inner products) are shared by kEPT entries, NT apart (coalesced)
constexpr int kEPT = 1;

// Per-thread accumulation of Re(a^H b) in the vectors' number type (for FP32x2 at least one
// operand of each product must be normalised; see f2r_mul).  warp_sum() adds the 32
// lanes (every lane must call it; the result is valid on every lane) in the same type;
// add() and to_double() combine and convert warp sums.  FP64 appears only in to_double,
// called once per block: the FP64 pipe of GB300 runs at 1/64 of the FP32 rate.
template <typename T> struct WarpAcc;
template <> struct WarpAcc<double> {
    using R = double;
    double v = 0;
    __device__ __forceinline__ void add(double2 a, double2 b) { v = fma(a.x, b.x, fma(a.y, b.y, v)); }
    __device__ __forceinline__ R warp_sum() const
    {
        double s = v;
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        return s;
    }
    static __device__ __forceinline__ R add(R a, R b) { return a + b; }
    static __device__ __forceinline__ double to_double(R a) { return a; }
};
template <> struct WarpAcc<float> {
    using R = float;
    float v = 0.f;
    __device__ __forceinline__ void add(float2 a, float2 b) { v = fmaf(a.x, b.x, fmaf(a.y, b.y, v)); }
    __device__ __forceinline__ R warp_sum() const
    {
        float s = v;
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        return s;
    }
    static __device__ __forceinline__ R add(R a, R b) { return a + b; }
    static __device__ __forceinline__ double to_double(R a) { return (double)a; }
};
template <> struct WarpAcc<DF> {
    using R = f2r;
    f2r v{0.f, 0.f};
    __device__ __forceinline__ void add(f2c a, f2c b) { v = f2r_add(v, f2r_add(f2r_mul(a.re, b.re), f2r_mul(a.im, b.im))); }
    __device__ __forceinline__ R warp_sum() const
    {
        f2r s = f2r_norm(v);
        for (int o = 16; o > 0; o >>= 1) {
            const f2r q{__shfl_xor_sync(0xffffffffu, s.hi, o), __shfl_xor_sync(0xffffffffu, s.lo, o)};
            s = f2r_add(s, q);
        }
        return s;
    }
    static __device__ __forceinline__ R add(R a, R b) { return f2r_add(a, b); }
    static __device__ __forceinline__ double to_double(R a) { return (double)a.hi + (double)a.lo; }
};

// K warp sums -> one FP64 partial per block, written to part[(3 b + k) nblk + block].
// Warps 1..7 leave their sums in shared memory, arrive at named barrier 1 and retire at
// once; warp 0 waits there (bar.sync), then its lane 0 adds the eight sums in warp order
// (deterministic).  Every thread of the block must reach this call.
constexpr int kWarps = NT / 32;
template <typename T, int K>
__device__ __forceinline__ void block_partials(const typename WarpAcc<T>::R (&ws)[K], double *part, int nblk, int b)
{
    using R = typename WarpAcc<T>::R;
    __shared__ R sh[K][kWarps];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (wid != 0) {
        if (lane == 0)
#pragma unroll
            for (int k = 0; k < K; k++) sh[k][wid] = ws[k];
        asm volatile("bar.arrive 1, %0;" ::"r"(NT) : "memory");
        return;
    }
    asm volatile("bar.sync 1, %0;" ::"r"(NT) : "memory");
    if (lane == 0)
#pragma unroll
        for (int k = 0; k < K; k++) {
            R s = ws[k];
            for (int w = 1; w < kWarps; w++) s = WarpAcc<T>::add(s, sh[k][w]);
            part[(3 * (size_t)b + k) * nblk + blockIdx.x] = WarpAcc<T>::to_double(s);
        }
}

// In the one-block-per-instance finalisers (NTF threads): the grand totals of the K
// partials of instance b, summed in a fixed order, valid in thread 0.
constexpr int NTF = 1024;
template <int K>
__device__ __forceinline__ void grand_totals(const double *part, int nblk, int b, double (&tot)[K])
{
    __shared__ double sh[K][NTF / 32];
    double s[K];
#pragma unroll
    for (int k = 0; k < K; k++) {
        s[k] = 0;
        const double *run = part + (3 * (size_t)b + k) * nblk;
        for (int i = threadIdx.x; i < nblk; i += NTF) s[k] += run[i];
    }
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int k = 0; k < K; k++) {
        for (int o = 16; o > 0; o >>= 1) s[k] += __shfl_down_sync(0xffffffffu, s[k], o);
        if (lane == 0) sh[k][wid] = s[k];
    }
    __syncthreads();
    if (threadIdx.x == 0)
#pragma unroll
        for (int k = 0; k < K; k++) {
            double a = 0;
            for (int w = 0; w < NTF / 32; w++) a += sh[k][w];
            tot[k] = a;
        }
}

// Truncated batches: true (after writing the block's K partials as zero) when every entry
// of this block lies at or beyond instance b's last kept entry and the block does not hold
// the trace slot; such a block has nothing to do (the decision is uniform over the block).
template <typename T, int K>
__device__ __forceinline__ bool masked_block(const InnerWork<T> &W, int b)
{
    if (!W.tier_lim) return false;
    const int64_t first = (int64_t)blockIdx.x * NT * kEPT, last = first + NT * kEPT - 1;
    if (first < (int64_t)__ldg(&W.tier_lim[b].y) || last >= W.N - 1) return false;
    if (threadIdx.x < K) W.part[(3 * (size_t)b + threadIdx.x) * W.nblk + blockIdx.x] = 0.0;
    return true;
}

#define FUSED_SETUP(K)                                         \
    using N = Num<T>;                                          \
    using A = typename N::A;                                   \
    const int b = blockIdx.y;                                  \
    if (W.st[b].done) return;                                  \
    if (masked_block<T, K>(W, b)) return;                      \
    const int64_t o = (int64_t)b * W.vstride;                  \
    const int64_t t0 = (int64_t)blockIdx.x * NT * kEPT + threadIdx.x;

// w = b, other vectors 0; partials ||b||^2, <r~, b>
template <typename T>
__global__ void k_in_init(InnerWork<T> W)
{
    using N = Num<T>;
    using A = typename N::A;
    const int b = blockIdx.y;
    const int64_t o = (int64_t)b * W.vstride;
    const int64_t t0 = (int64_t)blockIdx.x * NT * kEPT + threadIdx.x;
    WarpAcc<T> bb, rb;
#pragma unroll 1
    for (int e = 0; e < kEPT; e++) {
        const int64_t t = t0 + (int64_t)e * NT;
        if (t >= W.N) break;
        const A bv = N::load(W.b[o + t]);
        const typename N::V z = N::store(N::zero());
        W.w[o + t] = N::store(bv);
        W.x[o + t] = z; W.xs[o + t] = z; W.xs2[o + t] = z; W.y[o + t] = z; W.d[o + t] = z; W.v[o + t] = z; W.u2[o + t] = z;
        bb.add(bv, bv);
        rb.add(N::load(W.rt[shadow_index(W.tier_lim, b, t, W.N)]), bv);
    }
    const typename WarpAcc<T>::R ws[2] = {bb.warp_sum(), rb.warp_sum()};
    block_partials<T, 2>(ws, W.part, W.nblk, b);
}

template <typename T>
__global__ void __launch_bounds__(NTF) k_in_init_fin(InnerWork<T> W, double crit, int nlim, int stag_window)
{
    const int b = blockIdx.x;
    double tot[2];
    grand_totals<2>(W.part, W.nblk, b, tot);
    if (threadIdx.x != 0) return;
    InnerState s = {};
    s.r0 = sqrt(tot[0]);
    s.tau = tot[0];
    s.rho = tot[1];
    s.crit = crit; s.nlim = nlim; s.stag_window = stag_window;
    s.best = s.r0; s.ext_resid = s.r0;
    s.best_e = s.r0; s.best_slot = 0;   // slot 0 holds x = 0
    if (s.r0 <= crit) { s.done = 1; s.conv = 1; }
    else if (s.rho == 0.0) { s.done = 1; s.ierr = 8; }
    W.st[b] = s;
    InnerCoef<T> k;
    k.beta = k.alpha = k.alpha_prev = k.dd1 = k.eta1 = k.dd2 = k.eta2 = Num<T>::sc(0.0);
    W.cf[b] = k;
}

// B: u1 = A w + beta u2, the pending x / d updates, y = w + beta y2, v = u1 + beta (u2 + beta v)
template <typename T, bool REG, bool CF = false>
__global__ void __launch_bounds__(NT, 6) k_in_b(DevPlan P, DevCoef<T> C, InnerWork<T> W)
{
    FUSED_SETUP(1)
    WarpAcc<T> sg;
#pragma unroll 1
    for (int e = 0; e < kEPT; e++) {
        const int64_t t = t0 + (int64_t)e * NT;
        if (t >= W.N) break;
        const A aw = apply_entry<T, false, REG, CF>(P, C, W.w + o, t, b);
        const InnerCoef<T> &k = W.cf[b];
        const A u2 = N::load(W.u2[o + t]), vo = N::load(W.v[o + t]), yo = N::load(W.y[o + t]);
        const A u1 = N::add(aw, N::scale(u2, k.beta));
        W.u1[o + t] = N::store(u1);
        const A d1 = N::add(yo, N::scale(N::load(W.d[o + t]), k.dd1));
        const A y2 = N::sub(yo, N::scale(vo, k.alpha_prev));
        const A d2 = N::add(y2, N::scale(d1, k.dd2));
        W.d[o + t] = N::store(d2);
        W.x[o + t] = N::store(N::add(N::load(W.x[o + t]), N::add(N::scale(d1, k.eta1), N::scale(d2, k.eta2))));
        W.y[o + t] = N::store(N::add(N::load(W.w[o + t]), N::scale(y2, k.beta)));
        const A vn = N::add(u1, N::scale(N::add(u2, N::scale(vo, k.beta)), k.beta));
        W.v[o + t] = N::store(vn);
        sg.add(N::load(W.rt[shadow_index(W.tier_lim, b, t, W.N)]), vn);
    }
    const typename WarpAcc<T>::R ws[1] = {sg.warp_sum()};
    block_partials<T, 1>(ws, W.part, W.nblk, b);
}

template <typename T>
__global__ void __launch_bounds__(NTF) k_in_b_fin(InnerWork<T> W)
{
    const int b = blockIdx.x;
    if (W.st[b].done) return;
    double tot[1];
    grand_totals<1>(W.part, W.nblk, b, tot);
    if (threadIdx.x != 0) return;
    InnerState s = W.st[b];
    const double sigma = tot[0];
    if (sigma == 0.0 || !isfinite(sigma)) { s.done = 1; s.ierr = 8; }
    else {
        s.alpha = s.rho / sigma;
        W.cf[b].alpha = Num<T>::sc(s.alpha);
    }
    W.st[b] = s;
}

// A: u2 = u1 - alpha A v, w1 = w - alpha u1, w = w1 - alpha u2
template <typename T, bool REG, bool CF = false>
__global__ void __launch_bounds__(NT, 6) k_in_a(DevPlan P, DevCoef<T> C, InnerWork<T> W)
{
    FUSED_SETUP(3)
    WarpAcc<T> a1, a2, a3;
#pragma unroll 1
    for (int e = 0; e < kEPT; e++) {
        const int64_t t = t0 + (int64_t)e * NT;
        if (t >= W.N) break;
        const A av = apply_entry<T, false, REG, CF>(P, C, W.v + o, t, b);
        const typename N::S al = W.cf[b].alpha;
        const A u1 = N::load(W.u1[o + t]);
        const A u2 = N::sub(u1, N::scale(av, al));
        W.u2[o + t] = N::store(u2);
        // normalised before the squared norms (the lazy differences cancel near convergence)
        const A w1 = N::norm(N::sub(N::load(W.w[o + t]), N::scale(u1, al)));
        const A w2 = N::norm(N::sub(w1, N::scale(u2, al)));
        W.w[o + t] = N::pack(w2);
        a1.add(w1, w1);
        a2.add(w2, w2);
        a3.add(N::load(W.rt[shadow_index(W.tier_lim, b, t, W.N)]), w2);
    }
    const typename WarpAcc<T>::R ws[3] = {a1.warp_sum(), a2.warp_sum(), a3.warp_sum()};
    block_partials<T, 3>(ws, W.part, W.nblk, b);
}

template <typename T>
__global__ void __launch_bounds__(NTF) k_in_a_fin(InnerWork<T> W)
{
    const int b = blockIdx.x;
    if (W.st[b].done) return;
    double tot[3];
    grand_totals<3>(W.part, W.nblk, b, tot);
    if (threadIdx.x != 0) return;
    InnerState s = W.st[b];
    const double al = s.alpha;
    const double dd1 = s.var * s.eta / al;
    s.var = tot[0] / s.tau;
    double cs = 1.0 / (1.0 + s.var);
    s.tau = tot[0] * cs;
    s.eta = al * cs;
    const double eta1 = s.eta;
    const double dd2 = s.var * s.eta / al;
    s.var = tot[1] / s.tau;
    cs = 1.0 / (1.0 + s.var);
    s.tau = tot[1] * cs;
    s.eta = al * cs;
    s.n += 1;
    s.unrm = sqrt((double)(2 * s.n + 1) * s.tau) / s.r0;
    s.beta = tot[2] / s.rho;
    s.rho = tot[2];
    if (tot[2] == 0.0 || !isfinite(s.beta)) { s.done = 1; s.ierr = 8; }
    // predicted true residual below a third of the target: stop here, measured at the next check
    else if (s.ratio > 0.0 && s.unrm * s.r0 * s.ratio <= s.crit / 3.0) { s.done = 1; s.finishing = 1; }
    W.st[b] = s;
    using N = Num<T>;
    InnerCoef<T> k = W.cf[b];
    k.beta = N::sc(s.beta);
    k.alpha_prev = N::sc(al);
    k.dd1 = N::sc(dd1);
    k.eta1 = N::sc(eta1);
    k.dd2 = N::sc(dd2);
    k.eta2 = N::sc(s.eta);
    W.cf[b] = k;
}

// xs = x + the pending updates of the last iteration
template <typename T>
__global__ void k_in_x(InnerWork<T> W)
{
    using N = Num<T>;
    using A = typename N::A;
    const int b = blockIdx.y;
    if (W.st[b].done && !W.st[b].finishing) return;
    const int64_t o = (int64_t)b * W.vstride;
    const int64_t t0 = (int64_t)blockIdx.x * NT * kEPT + threadIdx.x;
    const InnerCoef<T> &k = W.cf[b];
    typename N::V *xo = W.slot(1 - W.st[b].best_slot);   // keep the best checked iterate
    for (int e = 0; e < kEPT; e++) {
        const int64_t t = t0 + (int64_t)e * NT;
        if (t >= W.N) break;
        const A yo = N::load(W.y[o + t]);
        const A d1 = N::add(yo, N::scale(N::load(W.d[o + t]), k.dd1));
        const A d2 = N::add(N::sub(yo, N::scale(N::load(W.v[o + t]), k.alpha_prev)), N::scale(d1, k.dd2));
        xo[o + t] = N::store(N::add(N::load(W.x[o + t]), N::add(N::scale(d1, k.eta1), N::scale(d2, k.eta2))));
    }
}

// partial ||b - A xs||^2
template <typename T, bool REG, bool CF = false>
__global__ void __launch_bounds__(NT, 6) k_in_chk(DevPlan P, DevCoef<T> C, InnerWork<T> W)
{
    using N = Num<T>;
    using A = typename N::A;
    const int b = blockIdx.y;
    if (W.st[b].done && !W.st[b].finishing) return;
    if (masked_block<T, 1>(W, b)) return;
    const int64_t o = (int64_t)b * W.vstride;
    const int64_t t0 = (int64_t)blockIdx.x * NT * kEPT + threadIdx.x;
    const typename N::V *xc = W.slot(1 - W.st[b].best_slot);
    WarpAcc<T> ee;
#pragma unroll 1
    for (int e = 0; e < kEPT; e++) {
        const int64_t t = t0 + (int64_t)e * NT;
        if (t >= W.N) break;
        const A r = N::norm(N::sub(N::load(W.b[o + t]), apply_entry<T, false, REG, CF>(P, C, xc + o, t, b)));
        ee.add(r, r);
    }
    const typename WarpAcc<T>::R ws[1] = {ee.warp_sum()};
    block_partials<T, 1>(ws, W.part, W.nblk, b);
}

template <typename T>
__global__ void __launch_bounds__(NTF) k_in_chk_fin(InnerWork<T> W)
{
    const int b = blockIdx.x;
    if (W.st[b].done && !W.st[b].finishing) return;
    double tot[1];
    grand_totals<1>(W.part, W.nblk, b, tot);
    if (threadIdx.x != 0) return;
    InnerState s = W.st[b];
    const double e = sqrt(tot[0]);
    s.ext_resid = e;
    s.checks += 1;
    if (s.unrm > 0.0) s.ratio = e / (s.unrm * s.r0);
    if (e < s.best_e) { s.best_e = e; s.best_slot = 1 - s.best_slot; }
    if (s.finishing) {   // stopped on the prediction: record what the check found
        s.finishing = 0;
        s.conv = e <= s.crit;
        s.ierr = isfinite(e) ? (s.conv ? 0 : 4) : 8;
        W.st[b] = s;
        return;
    }
    if (e <= s.crit) { s.done = 1; s.conv = 1; s.ierr = 0; }
    else if (s.n >= s.nlim) { s.done = 1; s.ierr = 4; }
    else if (s.stag_window) {
        // the arithmetic's floor: the true residual 10x above TFQMR's bound, or
        // stag_window checks without halving the best true residual
        if (s.n > 2 && e > 10.0 * s.unrm * s.r0) { s.done = 1; s.ierr = 4; }
        else if (e < 0.5 * s.best) { s.best = e; s.stag = 0; }
        else if (++s.stag >= s.stag_window) { s.done = 1; s.ierr = 4; }
    }
    if (!isfinite(e)) { s.done = 1; s.ierr = 8; }
    W.st[b] = s;
}

// measurement pattern: every vector = (1 + k/8) r~, finite scalars, no instance done
template <typename T>
__global__ void k_in_fill(InnerWork<T> W)
{
    using N = Num<T>;
    const int b = blockIdx.y;
    const int64_t o = (int64_t)b * W.vstride;
    const int64_t t0 = (int64_t)blockIdx.x * NT * kEPT + threadIdx.x;
#pragma unroll 1
    for (int e = 0; e < kEPT; e++) {
        const int64_t t = t0 + (int64_t)e * NT;
        if (t >= W.N) break;
        const typename N::V r = W.rt[t];
        typename N::V *vec[10] = {W.x, W.xs, W.b, W.w, W.y, W.d, W.v, W.u1, W.u2, W.xs2};
        for (int k = 0; k < 10; k++)
            vec[k][o + t] = N::store(N::scale(N::load(r), N::sc(1.0 + 0.125 * k)));
    }
    if (t0 == 0) {
        InnerState st = {};
        st.r0 = 1; st.tau = 1; st.rho = 1; st.nlim = 1 << 30;
        W.st[b] = st;
        InnerCoef<T> k;
        k.beta = k.alpha = k.alpha_prev = k.dd1 = k.eta1 = k.dd2 = k.eta2 = N::sc(0.5);
        W.cf[b] = k;
    }
}

}  // namespace

template <typename T>
void inner_time(InnerWork<T> &W, const DevPlan &P, const DevCoef<T> &C, int reps, cudaStream_t s, float &ms_b, float &ms_a)
{
    dim3 g((unsigned)W.nblk, (unsigned)W.nbatch);
    DevPlan Q = P;
    Q.order = nullptr;
    k_in_fill<T><<<g, NT, 0, s>>>(W);
    auto run_b = [&] {
        if (C.cf_half) k_in_b<T, false, true><<<g, NT, 0, s>>>(Q, C, W);
        else if (C.reg) k_in_b<T, true><<<g, NT, 0, s>>>(Q, C, W);
        else k_in_b<T, false><<<g, NT, 0, s>>>(Q, C, W);
    };
    auto run_a = [&] {
        if (C.cf_half) k_in_a<T, false, true><<<g, NT, 0, s>>>(Q, C, W);
        else if (C.reg) k_in_a<T, true><<<g, NT, 0, s>>>(Q, C, W);
        else k_in_a<T, false><<<g, NT, 0, s>>>(Q, C, W);
    };
    cudaEvent_t e0, e1;
    if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) fail(HEOM_E_CUDA, "cudaEventCreate failed");
    auto timed = [&](const std::function<void()> &f) {
        for (int w = 0; w < 3; w++) f();
        cudaEventRecord(e0, s);
        for (int r = 0; r < reps; r++) f();
        cudaEventRecord(e1, s);
        cudaEventSynchronize(e1);
        float ms = 0;
        cudaEventElapsedTime(&ms, e0, e1);
        return ms / reps;
    };
    ms_b = timed(run_b);
    ms_a = timed(run_a);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) fail(HEOM_E_CUDA, std::string("fused inner kernels: ") + cudaGetErrorString(e));
}

template <typename T>
void inner_alloc(InnerWork<T> &W, int nbatch, int64_t N, cudaStream_t s)
{
    using V = typename Num<T>::V;
    W.nbatch = nbatch;
    W.N = N;
    W.vstride = (N + 63) / 64 * 64;
    W.nblk = (int)((N + (int64_t)NT * kEPT - 1) / ((int64_t)NT * kEPT));
    const size_t vbytes = sizeof(V) * (size_t)W.vstride * nbatch;
    // every piece starts on a 256-byte boundary; the size is the sum of the rounded pieces
    auto rounded = [](size_t b) { return (b + 255) / 256 * 256; };
    const size_t total = rounded(vbytes) * 10 + rounded(sizeof(V) * (size_t)W.vstride) + rounded(sizeof(InnerState) * nbatch) +
                         rounded(sizeof(InnerCoef<T>) * nbatch) + rounded(sizeof(double) * 3 * (size_t)nbatch * W.nblk);
    char *p = nullptr;
    if (cudaMalloc((void **)&p, total) != cudaSuccess) fail(HEOM_E_NOMEM, "device allocation of the inner-solver workspace failed");
    if (cudaMemsetAsync(p, 0, total, s) != cudaSuccess || cudaStreamSynchronize(s) != cudaSuccess) {
        cudaFree(p);
        fail(HEOM_E_CUDA, "clearing the inner-solver workspace failed");
    }
    W.mem = p;
    auto take = [&](size_t bytes) { char *q = p; p += rounded(bytes); return q; };
    W.x = (V *)take(vbytes); W.xs = (V *)take(vbytes); W.b = (V *)take(vbytes); W.w = (V *)take(vbytes);
    W.y = (V *)take(vbytes); W.d = (V *)take(vbytes); W.v = (V *)take(vbytes); W.u1 = (V *)take(vbytes);
    W.u2 = (V *)take(vbytes); W.xs2 = (V *)take(vbytes);
    W.rt = (V *)take(sizeof(V) * (size_t)W.vstride);
    W.st = (InnerState *)take(sizeof(InnerState) * nbatch);
    W.cf = (InnerCoef<T> *)take(sizeof(InnerCoef<T>) * nbatch);
    W.part = (double *)take(sizeof(double) * 3 * (size_t)nbatch * W.nblk);
}

template <typename T>
void inner_free(InnerWork<T> &W)
{
    if (W.mem) cudaFree(W.mem);
    W = InnerWork<T>();
}

template <typename T>
void inner_start(InnerWork<T> &W, double crit, int nlim, int stag_window, cudaStream_t s)
{
    dim3 g((unsigned)W.nblk, (unsigned)W.nbatch);
    k_in_init<T><<<g, NT, 0, s>>>(W);
    k_in_init_fin<T><<<W.nbatch, NTF, 0, s>>>(W, crit, nlim, stag_window);
}

template <typename T>
void inner_chunk(InnerWork<T> &W, const DevPlan &P, const DevCoef<T> &C, int iters, cudaStream_t s)
{
    dim3 g((unsigned)W.nblk, (unsigned)W.nbatch);
    const unsigned nb = (unsigned)W.nbatch;
    DevPlan Q = P;
    Q.order = nullptr;   // entry order: coalesced epilogue access
    for (int i = 0; i < iters; i++) {
        if (C.cf_half) k_in_b<T, false, true><<<g, NT, 0, s>>>(Q, C, W);
        else if (C.reg) k_in_b<T, true><<<g, NT, 0, s>>>(Q, C, W);
        else k_in_b<T, false><<<g, NT, 0, s>>>(Q, C, W);
        k_in_b_fin<T><<<nb, NTF, 0, s>>>(W);
        if (C.cf_half) k_in_a<T, false, true><<<g, NT, 0, s>>>(Q, C, W);
        else if (C.reg) k_in_a<T, true><<<g, NT, 0, s>>>(Q, C, W);
        else k_in_a<T, false><<<g, NT, 0, s>>>(Q, C, W);
        k_in_a_fin<T><<<nb, NTF, 0, s>>>(W);
    }
    k_in_x<T><<<g, NT, 0, s>>>(W);
    if (C.cf_half) k_in_chk<T, false, true><<<g, NT, 0, s>>>(Q, C, W);
    else if (C.reg) k_in_chk<T, true><<<g, NT, 0, s>>>(Q, C, W);
    else k_in_chk<T, false><<<g, NT, 0, s>>>(Q, C, W);
    k_in_chk_fin<T><<<nb, NTF, 0, s>>>(W);
}

#define INST(T)                                                                              \
    template void inner_alloc<T>(InnerWork<T> &, int, int64_t, cudaStream_t);                \
    template void inner_free<T>(InnerWork<T> &);                                              \
    template void inner_start<T>(InnerWork<T> &, double, int, int, cudaStream_t);             \
    template void inner_chunk<T>(InnerWork<T> &, const DevPlan &, const DevCoef<T> &, int, cudaStream_t);    \
    template void inner_time<T>(InnerWork<T> &, const DevPlan &, const DevCoef<T> &, int, cudaStream_t, float &, float &);
INST(double)
INST(float)
INST(DF)

}  // namespace heom
