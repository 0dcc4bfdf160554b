// Kernels of the fused inner TFQMR (see inner.cuh), shared by the translation units that
// instantiate them: inner.cu (one instance per group, every number type), inner_il.cu
// (FP32x2, every position of a group served, stride known at compile time) and
// inner_ilc.cu (FP32x2, a group's running instances compacted onto fewer lanes, stride read
// at run time).  Template parameters of the kernels: GE lanes per entry (0: one instance
// per group), CMP (lanes map to positions through the lane map) and IPL instances per lane
// (2: a lane serves two adjacent positions of its group and decodes the plan once for both).
#pragma once
#include <cmath>
#include <functional>
#include <string>

#include "apply_entry.cuh"
#include "inner.cuh"

namespace heom {
namespace inner_detail {
namespace {   // every translation unit launches its own instantiations


constexpr int NT = 256;

// Per-thread accumulation of Re(a^H b) in the vectors' number type (for FP32x2 at least one
// operand of each product must be normalised; see f2r_mul).  warp_sum<G>() adds, in the same
// type, the lanes that hold one instance (lanes equal modulo G; every lane must call it;
// lanes 0 .. G-1 hold the sums of the warp's G instances); add() and to_double() combine
// and convert warp sums.  FP64 appears only in to_double, called once per block and
// instance: the FP64 pipe of GB300 runs at 1/64 of the FP32 rate.
template <typename T> struct WarpAcc;
template <> struct WarpAcc<double> {
    using R = double;
    double v = 0;
    __device__ __forceinline__ void add(double2 a, double2 b) { v = fma(a.x, b.x, fma(a.y, b.y, v)); }
    template <int G> __device__ __forceinline__ R warp_sum() const
    {
        double s = v;
        for (int o = 16; o >= G; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        return s;
    }
    static __device__ __forceinline__ R add(R a, R b) { return a + b; }
    static __device__ __forceinline__ double to_double(R a) { return a; }
};
template <> struct WarpAcc<float> {
    using R = float;
    float v = 0.f;
    __device__ __forceinline__ void add(float2 a, float2 b) { v = fmaf(a.x, b.x, fmaf(a.y, b.y, v)); }
    template <int G> __device__ __forceinline__ R warp_sum() const
    {
        float s = v;
        for (int o = 16; o >= G; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        return s;
    }
    static __device__ __forceinline__ R add(R a, R b) { return a + b; }
    static __device__ __forceinline__ double to_double(R a) { return (double)a; }
};
template <> struct WarpAcc<DF> {
    using R = f2r;
    f2r v{0.f, 0.f};
    __device__ __forceinline__ void add(f2c a, f2c b) { v = f2r_add(v, f2r_add(f2r_mul(a.re, b.re), f2r_mul(a.im, b.im))); }
    template <int G> __device__ __forceinline__ R warp_sum() const
    {
        f2r s = f2r_norm(v);
        for (int o = 16; o >= G; o >>= 1) {
            const f2r q{__shfl_xor_sync(0xffffffffu, s.hi, o), __shfl_xor_sync(0xffffffffu, s.lo, o)};
            s = f2r_add(s, q);
        }
        return s;
    }
    static __device__ __forceinline__ R add(R a, R b) { return f2r_add(a, b); }
    static __device__ __forceinline__ double to_double(R a) { return (double)a.hi + (double)a.lo; }
};

// In the one-block-per-instance finalisers (NTF threads): the grand totals of the K
// partials of instance b, summed in a fixed order, valid in thread 0.
constexpr int NTF = 1024;
template <int K>
__device__ __forceinline__ void grand_totals(const double *part, int nblk, int b, double (&tot)[K])
{
    __shared__ double sh[K][NTF / 32];
    double s[K];
    // four independent running sums per thread keep four loads in flight (the interleaved
    // layout gives G times more blocks, hence partials, per instance), added in a fixed order
#pragma unroll
    for (int k = 0; k < K; k++) {
        const double *run = part + (3 * (size_t)b + k) * nblk;
        double q0 = 0, q1 = 0, q2 = 0, q3 = 0;
        int i = threadIdx.x;
        for (; i + 3 * NTF < nblk; i += 4 * NTF) {
            q0 += run[i];
            q1 += run[i + NTF];
            q2 += run[i + 2 * NTF];
            q3 += run[i + 3 * NTF];
        }
        for (; i < nblk; i += NTF) q0 += run[i];
        s[k] = (q0 + q1) + (q2 + q3);
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

// Lane geometry of the fused kernels.  GE lanes serve one entry (GE = 0: the plain layout,
// one instance per group, stride 1 known at compile time), each lane IPL instances.  Slot
// j < GE IPL of group blockIdx.y serves the instance at position p of the group: p = j when
// every position is served (GE IPL == G), else p = amap[G blockIdx.y + j] (-1: no
// instance), so that a group whose instances have partly finished runs on fewer lanes and
// fewer blocks.  Lane l serves slots l IPL .. l IPL + IPL - 1.  The instance is
// b = G blockIdx.y + p, and its entry t sits at o + t stride.
template <int GE> constexpr int lanes_of() { return GE == 0 ? 1 : GE; }

template <typename T, int GE, bool CMP>
__device__ __forceinline__ int slot_pos(const InnerWork<T> &W, int j)
{
    if constexpr (GE == 0) return 0;
    else if constexpr (!CMP) return j;
    else return __ldg(&W.amap[(int)blockIdx.y * W.G + j]);
}

template <int IPL>
struct Lane {
    int b[IPL];         // instances
    bool on[IPL];       // the slot serves an instance
    int64_t t;          // entry
    int64_t o[IPL];     // base of the instances' vectors
};
template <typename T, int GE, bool CMP, int IPL>
__device__ __forceinline__ Lane<IPL> lane_of(const InnerWork<T> &W)
{
    static_assert(IPL == 1 || (GE > 0 && !CMP), "two instances per lane: every position of the group served");
    constexpr int NL = lanes_of<GE>();
    Lane<IPL> L;
    const int l = (int)(threadIdx.x & (NL - 1));
#pragma unroll
    for (int i = 0; i < IPL; i++) {
        const int p = slot_pos<T, GE, CMP>(W, l * IPL + i);
        L.b[i] = (int)blockIdx.y * W.G + p;
        L.on[i] = p >= 0 && L.b[i] < W.nbatch;
        L.o[i] = (int64_t)blockIdx.y * W.gstride + (p < 0 ? 0 : p);
    }
    L.t = (int64_t)blockIdx.x * (NT / NL) + threadIdx.x / NL;
    return L;
}
template <typename T, int GE, bool CMP, int IPL>
__device__ __forceinline__ int64_t stride_of(const InnerWork<T> &W) { return GE == 0 ? 1 : CMP ? W.G : GE * IPL; }

// the applies of the lane's instances to their entry L.t, instance i on the vector at x[i]
// (an instance's element stride); with two instances per lane, one whose slot serves no
// instance is computed on the group's zero padding and not used
template <typename T, bool REG, bool CF, int GE, bool CMP, int IPL>
__device__ __forceinline__ void apply_lane(const DevPlan &P, const DevCoef<T> &C, const InnerWork<T> &W,
                                           const typename Num<T>::V *const (&x)[IPL], const Lane<IPL> &L,
                                           typename Num<T>::A (&y)[IPL])
{
    const typename Num<T>::V *xv[IPL];
#pragma unroll
    for (int i = 0; i < IPL; i++) xv[i] = x[i] + L.o[i];
    apply_entries<T, false, REG, CF, GE == 0 ? 1 : CMP ? 0 : GE * IPL, IPL>(P, C, xv, L.t, L.b, y, W.G);
}

// K warp sums per slot -> one FP64 partial per block and instance, written to
// part[(3 b + k) nblk + block] for the instances the slots serve.  Warps 1..7 leave their
// sums in shared memory, arrive at named barrier 1 and retire at once; warp 0 waits there
// (bar.sync), then its lanes 0 .. GE-1 add the eight sums of each of their slots in warp
// order (deterministic).  Every thread of the block must reach this call.
constexpr int kWarps = NT / 32;
template <typename T, int K, int GE, bool CMP, int IPL>
__device__ __forceinline__ void block_partials(const typename WarpAcc<T>::R (&ws)[K][IPL], const InnerWork<T> &W)
{
    using R = typename WarpAcc<T>::R;
    constexpr int NL = lanes_of<GE>();
    __shared__ R sh[K][IPL][kWarps][NL];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (wid != 0) {
        if (lane < NL)
#pragma unroll
            for (int k = 0; k < K; k++)
#pragma unroll
                for (int i = 0; i < IPL; i++) sh[k][i][wid][lane] = ws[k][i];
        asm volatile("bar.arrive 1, %0;" ::"r"(NT) : "memory");
        return;
    }
    asm volatile("bar.sync 1, %0;" ::"r"(NT) : "memory");
    if (lane >= NL) return;
#pragma unroll
    for (int i = 0; i < IPL; i++) {
        const int p = slot_pos<T, GE, CMP>(W, lane * IPL + i), b = (int)blockIdx.y * W.G + p;
        if (p < 0 || b >= W.nbatch) continue;
#pragma unroll
        for (int k = 0; k < K; k++) {
            R s = ws[k][i];
            for (int w = 1; w < kWarps; w++) s = WarpAcc<T>::add(s, sh[k][i][w][lane]);
            W.part[(3 * (size_t)b + k) * W.nblk + blockIdx.x] = WarpAcc<T>::to_double(s);
        }
    }
}

// Whether the block has work for the lane's i-th instance: the slot serves one, it runs
// (`run`), and, in a truncated batch (tier_lim), the block's entries are not all beyond its
// tier (a block that holds the trace slot always has work).
template <typename T, int GE, bool CMP, int IPL>
__device__ __forceinline__ bool block_work(const InnerWork<T> &W, const Lane<IPL> &L, int i, bool run)
{
    constexpr int NL = lanes_of<GE>();
    if (!L.on[i] || !run) return false;
    if (!W.tier_lim) return true;
    const int64_t first = (int64_t)blockIdx.x * (NT / NL), last = first + NT / NL - 1;
    return first < (int64_t)__ldg(&W.tier_lim[L.b[i]].y) || last >= W.N - 1;
}

// Programmatic dependent launch: `k_in_b` and `k_in_a` are launched while the preceding
// finaliser still runs (it calls allow_dependents first).  Their applies read only vectors
// that the fused kernel before the finaliser wrote; they wait for the finaliser
// (wait_prior_grid, griddepcontrol.wait: the whole preceding grid has finished and its
// writes are visible) before they read the instances' states and coefficients it writes, or
// write partial sums it may still be reading.  Without the launch attribute the wait returns
// at once.
__device__ __forceinline__ void wait_prior_grid() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void allow_dependents() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

// Entry of the fused kernels with K partials: false (after writing the K partials of this
// block as zero for the instances its slots serve) when no lane of the block has work; the
// decision is uniform over the block.  `work`: whether this lane has work for any of its
// instances.
template <typename T, int K, int GE, bool CMP, int IPL>
__device__ __forceinline__ bool block_enter(const InnerWork<T> &W, bool work)
{
    constexpr int NS = lanes_of<GE>() * IPL;   // slots of a block
    bool any;
    if constexpr (GE == 0) any = work;   // one instance per block
    else any = __syncthreads_or(work) != 0;
    if (any) return true;
    wait_prior_grid();
    if (threadIdx.x < K * NS) {
        const int p = slot_pos<T, GE, CMP>(W, (int)(threadIdx.x % NS)), k = (int)(threadIdx.x / NS);
        const int b = (int)blockIdx.y * W.G + p;
        if (p >= 0 && b < W.nbatch) W.part[(3 * (size_t)b + k) * W.nblk + blockIdx.x] = 0.0;
    }
    return false;
}

// w = b, other vectors 0; partials ||b||^2, <r~, b>
template <typename T, int GE, bool CMP, int IPL>
__global__ void k_in_init(InnerWork<T> W)
{
    using N = Num<T>;
    using A = typename N::A;
    constexpr int NL = lanes_of<GE>();
    const Lane<IPL> L = lane_of<T, GE, CMP, IPL>(W);
    WarpAcc<T> bb[IPL], rb[IPL];
#pragma unroll
    for (int i = 0; i < IPL; i++)
        if (L.on[i] && L.t < W.N) {
            const int64_t e = L.o[i] + L.t * stride_of<T, GE, CMP, IPL>(W);
            const A bv = N::load(W.b[e]);
            const typename N::V z = N::store(N::zero());
            W.w[e] = N::store(bv);
            W.x[e] = z; W.xs[e] = z; W.xs2[e] = z; W.y[e] = z; W.d[e] = z; W.v[e] = z; W.u2[e] = z;
            bb[i].add(bv, bv);
            rb[i].add(N::load(W.rt[shadow_index(W.tier_lim, L.b[i], L.t, W.N)]), bv);
        }
    typename WarpAcc<T>::R ws[2][IPL];
#pragma unroll
    for (int i = 0; i < IPL; i++) {
        ws[0][i] = bb[i].template warp_sum<NL>();
        ws[1][i] = rb[i].template warp_sum<NL>();
    }
    block_partials<T, 2, GE, CMP, IPL>(ws, W);
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

// Resident blocks per SM of the apply kernels: six (at most 40 registers) with one instance
// per lane; five (48 registers, 8-24 bytes of spills) with two, whose accumulators double.
// Measured on the double dot at tier 4, batch 8, two instances per lane in groups of two
// (k_in_b + k_in_a): 403 us at five blocks; 430 us at six (40 registers, 40-110 bytes of
// spills); at four (64 registers, no spills) too few warps hide the gathers' latency (437 us,
// issue slots 66 % busy).
template <int IPL> constexpr int apply_blocks_per_sm() { return IPL == 1 ? 6 : 5; }

// B: u1 = A w + beta u2, the pending x / d updates, y = w + beta y2, v = u1 + beta (u2 + beta v)
template <typename T, bool REG, bool CF, int GE, bool CMP, int IPL>
__global__ void __launch_bounds__(NT, apply_blocks_per_sm<IPL>()) k_in_b(DevPlan P, DevCoef<T> C, InnerWork<T> W)
{
    using N = Num<T>;
    using A = typename N::A;
    constexpr int NL = lanes_of<GE>();
    const Lane<IPL> L = lane_of<T, GE, CMP, IPL>(W);
    // an instance finished before the preceding finaliser stays finished within the round
    bool work[IPL], any = false;
#pragma unroll
    for (int i = 0; i < IPL; i++) {
        work[i] = block_work<T, GE, CMP, IPL>(W, L, i, L.on[i] && !W.st[L.b[i]].done);
        any = any || work[i];
    }
    if (!block_enter<T, 1, GE, CMP, IPL>(W, any)) return;
    WarpAcc<T> sg[IPL];
    A aw[IPL];
    if (any && L.t < W.N) {
        const typename N::V *xv[IPL];
#pragma unroll
        for (int i = 0; i < IPL; i++) xv[i] = W.w;
        apply_lane<T, REG, CF, GE, CMP, IPL>(P, C, W, xv, L, aw);
    }
    wait_prior_grid();
#pragma unroll
    for (int i = 0; i < IPL; i++)
        if (work[i] && L.t < W.N && !W.st[L.b[i]].done) {
            const int64_t e = L.o[i] + L.t * stride_of<T, GE, CMP, IPL>(W);
            const InnerCoef<T> &k = W.cf[L.b[i]];
            const A u2 = N::load(W.u2[e]), vo = N::load(W.v[e]), yo = N::load(W.y[e]);
            const A u1 = N::add(aw[i], N::scale(u2, k.beta));
            W.u1[e] = N::store(u1);
            const A d1 = N::add(yo, N::scale(N::load(W.d[e]), k.dd1));
            const A y2 = N::sub(yo, N::scale(vo, k.alpha_prev));
            const A d2 = N::add(y2, N::scale(d1, k.dd2));
            W.d[e] = N::store(d2);
            W.x[e] = N::store(N::add(N::load(W.x[e]), N::add(N::scale(d1, k.eta1), N::scale(d2, k.eta2))));
            W.y[e] = N::store(N::add(N::load(W.w[e]), N::scale(y2, k.beta)));
            const A vn = N::add(u1, N::scale(N::add(u2, N::scale(vo, k.beta)), k.beta));
            W.v[e] = N::store(vn);
            sg[i].add(N::load(W.rt[shadow_index(W.tier_lim, L.b[i], L.t, W.N)]), vn);
        }
    typename WarpAcc<T>::R ws[1][IPL];
#pragma unroll
    for (int i = 0; i < IPL; i++) ws[0][i] = sg[i].template warp_sum<NL>();
    block_partials<T, 1, GE, CMP, IPL>(ws, W);
}

template <typename T>
__global__ void __launch_bounds__(NTF) k_in_b_fin(InnerWork<T> W)
{
    allow_dependents();
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
template <typename T, bool REG, bool CF, int GE, bool CMP, int IPL>
__global__ void __launch_bounds__(NT, apply_blocks_per_sm<IPL>()) k_in_a(DevPlan P, DevCoef<T> C, InnerWork<T> W)
{
    using N = Num<T>;
    using A = typename N::A;
    constexpr int NL = lanes_of<GE>();
    const Lane<IPL> L = lane_of<T, GE, CMP, IPL>(W);
    bool work[IPL], any = false;
#pragma unroll
    for (int i = 0; i < IPL; i++) {
        work[i] = block_work<T, GE, CMP, IPL>(W, L, i, L.on[i] && !W.st[L.b[i]].done);
        any = any || work[i];
    }
    if (!block_enter<T, 3, GE, CMP, IPL>(W, any)) return;
    WarpAcc<T> a1[IPL], a2[IPL], a3[IPL];
    A av[IPL];
    if (any && L.t < W.N) {
        const typename N::V *xv[IPL];
#pragma unroll
        for (int i = 0; i < IPL; i++) xv[i] = W.v;
        apply_lane<T, REG, CF, GE, CMP, IPL>(P, C, W, xv, L, av);
    }
    wait_prior_grid();
#pragma unroll
    for (int i = 0; i < IPL; i++)
        if (work[i] && L.t < W.N && !W.st[L.b[i]].done) {
            const int64_t e = L.o[i] + L.t * stride_of<T, GE, CMP, IPL>(W);
            const typename N::S al = W.cf[L.b[i]].alpha;
            const A u1 = N::load(W.u1[e]);
            const A u2 = N::sub(u1, N::scale(av[i], al));
            W.u2[e] = N::store(u2);
            // normalised before the squared norms (the lazy differences cancel near convergence)
            const A w1 = N::norm(N::sub(N::load(W.w[e]), N::scale(u1, al)));
            const A w2 = N::norm(N::sub(w1, N::scale(u2, al)));
            W.w[e] = N::pack(w2);
            a1[i].add(w1, w1);
            a2[i].add(w2, w2);
            a3[i].add(N::load(W.rt[shadow_index(W.tier_lim, L.b[i], L.t, W.N)]), w2);
        }
    typename WarpAcc<T>::R ws[3][IPL];
#pragma unroll
    for (int i = 0; i < IPL; i++) {
        ws[0][i] = a1[i].template warp_sum<NL>();
        ws[1][i] = a2[i].template warp_sum<NL>();
        ws[2][i] = a3[i].template warp_sum<NL>();
    }
    block_partials<T, 3, GE, CMP, IPL>(ws, W);
}

template <typename T>
__global__ void __launch_bounds__(NTF) k_in_a_fin(InnerWork<T> W)
{
    allow_dependents();
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


// xs = x + the pending updates of the last iteration (into the slot that does not hold the
// best checked iterate)
template <typename T, int GE, bool CMP, int IPL>
__global__ void k_in_x(InnerWork<T> W)
{
    using N = Num<T>;
    using A = typename N::A;
    const Lane<IPL> L = lane_of<T, GE, CMP, IPL>(W);
    if (L.t >= W.N) return;
#pragma unroll
    for (int i = 0; i < IPL; i++) {
        if (!L.on[i]) continue;
        const InnerState &st = W.st[L.b[i]];
        if (st.done && !st.finishing) continue;
        const int64_t e = L.o[i] + L.t * stride_of<T, GE, CMP, IPL>(W);
        const InnerCoef<T> &k = W.cf[L.b[i]];
        typename N::V *xo = W.slot(1 - st.best_slot);
        const A yo = N::load(W.y[e]);
        const A d1 = N::add(yo, N::scale(N::load(W.d[e]), k.dd1));
        const A d2 = N::add(N::sub(yo, N::scale(N::load(W.v[e]), k.alpha_prev)), N::scale(d1, k.dd2));
        xo[e] = N::store(N::add(N::load(W.x[e]), N::add(N::scale(d1, k.eta1), N::scale(d2, k.eta2))));
    }
}

// partial ||b - A xs||^2
template <typename T, bool REG, bool CF, int GE, bool CMP, int IPL>
__global__ void __launch_bounds__(NT, apply_blocks_per_sm<IPL>()) k_in_chk(DevPlan P, DevCoef<T> C, InnerWork<T> W)
{
    using N = Num<T>;
    using A = typename N::A;
    constexpr int NL = lanes_of<GE>();
    const Lane<IPL> L = lane_of<T, GE, CMP, IPL>(W);
    bool work[IPL], any = false;
#pragma unroll
    for (int i = 0; i < IPL; i++) {
        const bool run = L.on[i] && (!W.st[L.b[i]].done || W.st[L.b[i]].finishing);
        work[i] = block_work<T, GE, CMP, IPL>(W, L, i, run);
        any = any || work[i];
    }
    if (!block_enter<T, 1, GE, CMP, IPL>(W, any)) return;
    WarpAcc<T> ee[IPL];
    if (any && L.t < W.N) {
        const typename N::V *xc[IPL];
#pragma unroll
        for (int i = 0; i < IPL; i++) xc[i] = W.slot(L.on[i] ? 1 - W.st[L.b[i]].best_slot : 0);
        A ax[IPL];
        apply_lane<T, REG, CF, GE, CMP, IPL>(P, C, W, xc, L, ax);
#pragma unroll
        for (int i = 0; i < IPL; i++)
            if (work[i]) {
                const A r = N::norm(N::sub(N::load(W.b[L.o[i] + L.t * stride_of<T, GE, CMP, IPL>(W)]), ax[i]));
                ee[i].add(r, r);
            }
    }
    typename WarpAcc<T>::R ws[1][IPL];
#pragma unroll
    for (int i = 0; i < IPL; i++) ws[0][i] = ee[i].template warp_sum<NL>();
    block_partials<T, 1, GE, CMP, IPL>(ws, W);
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
template <typename T, int GE, bool CMP, int IPL>
__global__ void k_in_fill(InnerWork<T> W)
{
    using N = Num<T>;
    const Lane<IPL> L = lane_of<T, GE, CMP, IPL>(W);
    if (L.t >= W.N) return;
#pragma unroll
    for (int i = 0; i < IPL; i++) {
        if (!L.on[i]) continue;
        const int64_t e = L.o[i] + L.t * stride_of<T, GE, CMP, IPL>(W);
        const typename N::V r = W.rt[L.t];
        typename N::V *vec[10] = {W.x, W.xs, W.b, W.w, W.y, W.d, W.v, W.u1, W.u2, W.xs2};
        for (int k = 0; k < 10; k++) vec[k][e] = N::store(N::scale(N::load(r), N::sc(1.0 + 0.125 * k)));
        if (L.t == 0) {
            InnerState st = {};
            st.r0 = 1; st.tau = 1; st.rho = 1; st.nlim = 1 << 30;
            W.st[L.b[i]] = st;
            InnerCoef<T> k;
            k.beta = k.alpha = k.alpha_prev = k.dd1 = k.eta1 = k.dd2 = k.eta2 = N::sc(0.5);
            W.cf[L.b[i]] = k;
        }
    }
}

// The launches of one chunk (`iters` iterations and a check) in configuration (GE, CMP,
// IPL).  With two instances per lane the correlation-function operator is instantiated for
// groups of two only (the layout of its solves), and truncated batches are refused.
template <int GE, int IPL> constexpr bool cf_variant() { return IPL == 1 || GE == 1; }

template <typename T, int GE, bool CMP, int IPL>
void check_layout(const DevCoef<T> &C)
{
    if (IPL > 1 && C.tier_lim) fail(HEOM_E_ARG, "two instances per lane: whole hierarchies only");
    if (!cf_variant<GE, IPL>() && C.cf_half)
        fail(HEOM_E_ARG, "two instances per lane: the correlation-function operator in groups of two only");
}

template <typename T, int GE, bool CMP, int IPL>
void chunk_ge(InnerWork<T> &W, const DevPlan &Q, const DevCoef<T> &C, int iters, cudaStream_t s)
{
    dim3 g((unsigned)W.nblk, (unsigned)W.ngroups);
    const unsigned nb = (unsigned)W.nbatch;
    // the fused kernels as programmatic dependents of the finaliser before them
    auto dependent = [&](auto kernel) {
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = g;
        cfg.blockDim = dim3(NT);
        cfg.dynamicSmemBytes = 0;
        cfg.stream = s;
        cudaLaunchAttribute at[1];
        at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
        at[0].val.programmaticStreamSerializationAllowed = 1;
        cfg.attrs = at;
        cfg.numAttrs = 1;
        if (cudaLaunchKernelEx(&cfg, kernel, Q, C, W) != cudaSuccess) fail(HEOM_E_CUDA, "launch of a fused inner kernel failed");
    };
    check_layout<T, GE, CMP, IPL>(C);
    for (int i = 0; i < iters; i++) {
        if constexpr (cf_variant<GE, IPL>())
            if (C.cf_half) dependent(k_in_b<T, false, true, GE, CMP, IPL>);
        if (!C.cf_half) {
            if (C.reg) dependent(k_in_b<T, true, false, GE, CMP, IPL>);
            else dependent(k_in_b<T, false, false, GE, CMP, IPL>);
        }
        k_in_b_fin<T><<<nb, NTF, 0, s>>>(W);
        if constexpr (cf_variant<GE, IPL>())
            if (C.cf_half) dependent(k_in_a<T, false, true, GE, CMP, IPL>);
        if (!C.cf_half) {
            if (C.reg) dependent(k_in_a<T, true, false, GE, CMP, IPL>);
            else dependent(k_in_a<T, false, false, GE, CMP, IPL>);
        }
        k_in_a_fin<T><<<nb, NTF, 0, s>>>(W);
    }
    k_in_x<T, GE, CMP, IPL><<<g, NT, 0, s>>>(W);
    if constexpr (cf_variant<GE, IPL>())
        if (C.cf_half) k_in_chk<T, false, true, GE, CMP, IPL><<<g, NT, 0, s>>>(Q, C, W);
    if (!C.cf_half) {
        if (C.reg) k_in_chk<T, true, false, GE, CMP, IPL><<<g, NT, 0, s>>>(Q, C, W);
        else k_in_chk<T, false, false, GE, CMP, IPL><<<g, NT, 0, s>>>(Q, C, W);
    }
    k_in_chk_fin<T><<<nb, NTF, 0, s>>>(W);
}

template <typename T, int GE, bool CMP, int IPL>
void time_ge(InnerWork<T> &W, const DevPlan &Q, const DevCoef<T> &C, int reps, cudaStream_t s, float &ms_b, float &ms_a)
{
    dim3 g((unsigned)W.nblk, (unsigned)W.ngroups);
    check_layout<T, GE, CMP, IPL>(C);
    k_in_fill<T, GE, CMP, IPL><<<g, NT, 0, s>>>(W);
    auto run_b = [&] {
        if constexpr (cf_variant<GE, IPL>())
            if (C.cf_half) { k_in_b<T, false, true, GE, CMP, IPL><<<g, NT, 0, s>>>(Q, C, W); return; }
        if (C.reg) k_in_b<T, true, false, GE, CMP, IPL><<<g, NT, 0, s>>>(Q, C, W);
        else k_in_b<T, false, false, GE, CMP, IPL><<<g, NT, 0, s>>>(Q, C, W);
    };
    auto run_a = [&] {
        if constexpr (cf_variant<GE, IPL>())
            if (C.cf_half) { k_in_a<T, false, true, GE, CMP, IPL><<<g, NT, 0, s>>>(Q, C, W); return; }
        if (C.reg) k_in_a<T, true, false, GE, CMP, IPL><<<g, NT, 0, s>>>(Q, C, W);
        else k_in_a<T, false, false, GE, CMP, IPL><<<g, NT, 0, s>>>(Q, C, W);
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
}


}  // namespace

// blocks per group with `ge` lanes per entry
inline int blocks_per_group(int64_t N, int ge)
{
    const int per = NT / (ge == 0 ? 1 : ge);
    return (int)((N + per - 1) / per);
}

// FP32x2 configurations with more than one instance per group (inner_il.cu: every position
// served, GE = W.G; inner_ilc.cu: compacted, GE = W.GE < W.G)
void df_init_full(const InnerWork<DF> &F, cudaStream_t s);
void df_chunk_full(InnerWork<DF> &W, const DevPlan &Q, const DevCoef<DF> &C, int iters, cudaStream_t s);
void df_time_full(InnerWork<DF> &F, const DevPlan &Q, const DevCoef<DF> &C, int reps, cudaStream_t s, float &ms_b, float &ms_a);
void df_chunk_compact(InnerWork<DF> &W, const DevPlan &Q, const DevCoef<DF> &C, int iters, cudaStream_t s);
// two instances per lane, every position served (inner_ilp.cu: GE = W.G / 2)
void df_init_pair(const InnerWork<DF> &F, cudaStream_t s);
void df_chunk_pair(InnerWork<DF> &W, const DevPlan &Q, const DevCoef<DF> &C, int iters, cudaStream_t s);
void df_time_pair(InnerWork<DF> &F, const DevPlan &Q, const DevCoef<DF> &C, int reps, cudaStream_t s, float &ms_b, float &ms_a);

}  // namespace inner_detail
}  // namespace heom
