// Fused batched TFQMR for the inner solves of mixed-precision refinement (see inner.cuh
// for the arrangement of the iteration).
#include <cmath>
#include <functional>
#include <string>
#include <type_traits>
#include <vector>

#include "inner_kernels.cuh"

namespace heom {

namespace {

using namespace inner_detail;

// Shadow vector of round `round`: 2 N reals uniform in [-1, 1) from the splitmix64 sequence
// (Steele, Lea, Flood, OOPSLA 2014) z_k = 0x9E3779B97F4A7C15 (round + 2 + k), element i
// taking k = 2 i (real part) and 2 i + 1 (imaginary part).
__device__ __forceinline__ double splitmix_uniform(uint64_t z)
{
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z ^= z >> 31;
    return 2.0 * ((double)(z >> 11) * (1.0 / 9007199254740992.0)) - 1.0;
}

template <typename T>
__global__ void k_in_shadow(typename Num<T>::V *rt, int64_t n, int round)
{
    const uint64_t g = 0x9E3779B97F4A7C15ull;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const uint64_t k = 2 * (uint64_t)i + (uint64_t)round + 2;
        rt[i] = Num<T>::store(Num<T>::from_d(splitmix_uniform(g * k), splitmix_uniform(g * (k + 1))));
    }
}

// instance-major values (n per instance) -> the interleaved layout of groups of G
template <typename V>
__global__ void k_interleave(const V *__restrict__ src, V *__restrict__ dst, int64_t n, int nbatch, int G)
{
    const int b = blockIdx.y;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        dst[(int64_t)(b / G) * n * G + i * G + b % G] = src[(int64_t)b * n + i];
}

template <typename T>
__global__ void k_in_rhs(DevPlan P, const double2 *__restrict__ r, InnerWork<T> W, int inst, double scale, const float *pre)
{
    using N = Num<T>;
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < W.N; t += (int64_t)gridDim.x * blockDim.x) {
        double f = scale;
        if (pre && t < P.lunk) f *= (double)pre[__ldg(P.ent_ado + t)];
        W.b[W.at(inst, t)] = N::store(N::from_d(r[t].x * f, r[t].y * f));
    }
}

template <typename T>
__global__ void k_in_add_solution(double2 *__restrict__ x, InnerWork<T> W, int inst, double a, int slot)
{
    using N = Num<T>;
    const typename N::V *src = W.slot(slot);
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < W.N; t += (int64_t)gridDim.x * blockDim.x) {
        const typename N::A v = N::load(src[W.at(inst, t)]);
        x[t].x += a * N::re(v);
        x[t].y += a * N::im(v);
    }
}

// G > 1 only for FP32x2 (the mixed solves); FP64 and FP32 keep one instance per group
template <typename T> constexpr bool kInterleaves = std::is_same<T, DF>::value;

// W configured for every position of every group (GE = G / ipl_max; 0 for the plain layout)
template <typename T>
InnerWork<T> full_lanes(const InnerWork<T> &W)
{
    InnerWork<T> F = W;
    F.ipl = W.ipl_max;
    F.GE = W.G == 1 ? 0 : W.G / W.ipl_max;
    F.nblk = blocks_per_group(W.N, F.GE);
    return F;
}

}  // namespace

template <typename T>
void inner_time(InnerWork<T> &W, const DevPlan &P, const DevCoef<T> &C, int reps, cudaStream_t s, float &ms_b, float &ms_a)
{
    DevPlan Q = P;
    Q.order = nullptr;
    const DevCoef<T> K = inner_layout_coef<T>(W, P, C, s);
    InnerWork<T> F = full_lanes(W);
    if (F.GE == 0) time_ge<T, 0, false, 1>(F, Q, K, reps, s, ms_b, ms_a);
    else if constexpr (kInterleaves<T>) {
        if (F.ipl == 2) df_time_pair(F, Q, K, reps, s, ms_b, ms_a);
        else df_time_full(F, Q, K, reps, s, ms_b, ms_a);
    }
    else fail(HEOM_E_ARG, "inner workspace: interleave of a non-FP32x2 type");
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) fail(HEOM_E_CUDA, std::string("fused inner kernels: ") + cudaGetErrorString(e));
}

template <typename T>
void inner_alloc(InnerWork<T> &W, int nbatch, int64_t N, cudaStream_t s, int G, int ipl)
{
    using V = typename Num<T>::V;
    if (G < 0 || G > 32 || (G & (G - 1))) fail(HEOM_E_ARG, "interleave must be 0 or a power of two up to 32");
    if (ipl != 1 && ipl != 2) fail(HEOM_E_ARG, "instances per lane must be 1 or 2");
    W.nbatch = nbatch;
    W.N = N;
    W.G = !kInterleaves<T> ? 1 : G > 0 ? G : inner_default_interleave(nbatch);
    W.ipl_max = W.G > 1 ? ipl : 1;
    W.ipl = 1;
    W.ngroups = (nbatch + W.G - 1) / W.G;
    W.vstride = (N + 63) / 64 * 64;
    W.gstride = W.vstride * W.G;
    W.GE = W.G == 1 ? 0 : W.G;
    W.nblk = blocks_per_group(N, W.GE);   // the most blocks per group (every position served)
    const int npad = W.ngroups * W.G;
    const size_t vbytes = sizeof(V) * (size_t)W.gstride * W.ngroups;
    // every piece starts on a 256-byte boundary; the size is the sum of the rounded pieces
    auto rounded = [](size_t b) { return (b + 255) / 256 * 256; };
    const size_t total = rounded(vbytes) * 10 + rounded(sizeof(V) * (size_t)W.vstride) + rounded(sizeof(InnerState) * nbatch) +
                         rounded(sizeof(InnerCoef<T>) * nbatch) + rounded(sizeof(double) * 3 * (size_t)npad * W.nblk) +
                         rounded(sizeof(int) * (size_t)npad);
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
    W.part = (double *)take(sizeof(double) * 3 * (size_t)npad * W.nblk);
    W.amap = (int *)take(sizeof(int) * (size_t)npad);
}

template <typename T>
void inner_free(InnerWork<T> &W)
{
    if (W.mem) cudaFree(W.mem);
    if (W.coef_mem) cudaFree(W.coef_mem);
    W = InnerWork<T>();
}

template <typename T>
DevCoef<T> inner_layout_coef(InnerWork<T> &W, const DevPlan &P, const DevCoef<T> &C, cudaStream_t s)
{
    using V = typename Num<T>::V;
    if (W.G == 1) return C;
    if (!C.hval || !C.gdiag) fail(HEOM_E_ARG, "inner coefficients: per-instance H values and ADO diagonals required");
    const int npad = W.ngroups * W.G;
    const int64_t nh = std::max(1, P.nh), nd = std::max(1, P.nado);
    const size_t bytes = sizeof(V) * (size_t)(nh + nd) * npad;
    if (W.coef_mem) { cudaFree(W.coef_mem); W.coef_mem = nullptr; }
    if (cudaMalloc(&W.coef_mem, bytes) != cudaSuccess) fail(HEOM_E_NOMEM, "device allocation of the interleaved coefficients failed");
    if (cudaMemsetAsync(W.coef_mem, 0, bytes, s) != cudaSuccess) fail(HEOM_E_CUDA, "clearing the interleaved coefficients failed");
    V *hv = (V *)W.coef_mem, *gd = hv + nh * npad;
    k_interleave<V><<<dim3((unsigned)std::min<int64_t>(64, (nh + 255) / 256), (unsigned)W.nbatch), 256, 0, s>>>(C.hval, hv, P.nh, W.nbatch, W.G);
    k_interleave<V><<<dim3((unsigned)std::min<int64_t>(256, (nd + 255) / 256), (unsigned)W.nbatch), 256, 0, s>>>(C.gdiag, gd, P.nado, W.nbatch, W.G);
    DevCoef<T> K = C;
    K.hval = hv;
    K.gdiag = gd;
    return K;
}

template <typename T>
void inner_rhs(InnerWork<T> &W, const DevPlan &P, const double2 *r, int inst, double scale, const float *pre, cudaStream_t s)
{
    k_in_rhs<T><<<(unsigned)std::min<int64_t>(2048, (W.N + 255) / 256), 256, 0, s>>>(P, r, W, inst, scale, pre);
}

template <typename T>
void inner_add_solution(InnerWork<T> &W, double2 *x, int inst, double a, int slot, cudaStream_t s)
{
    k_in_add_solution<T><<<(unsigned)std::min<int64_t>(2048, (W.N + 255) / 256), 256, 0, s>>>(x, W, inst, a, slot);
}

template <typename T>
void inner_shadow(InnerWork<T> &W, int round, cudaStream_t s)
{
    k_in_shadow<T><<<(unsigned)std::min<int64_t>(1024, (W.N + 255) / 256), 256, 0, s>>>(W.rt, W.N, round);
}

template <typename T>
void inner_start(InnerWork<T> &W, double crit, int nlim, int stag_window, cudaStream_t s)
{
    const InnerWork<T> F = full_lanes(W);
    dim3 g((unsigned)F.nblk, (unsigned)F.ngroups);
    if (F.GE == 0) k_in_init<T, 0, false, 1><<<g, NT, 0, s>>>(F);
    else if constexpr (kInterleaves<T>) {
        if (F.ipl == 2) df_init_pair(F, s);
        else df_init_full(F, s);
    }
    else fail(HEOM_E_ARG, "inner workspace: interleave of a non-FP32x2 type");
    k_in_init_fin<T><<<F.nbatch, NTF, 0, s>>>(F, crit, nlim, stag_window);
}

template <typename T>
void inner_lanes(InnerWork<T> &W, const InnerState *st, std::vector<int> &amap_host, cudaStream_t s)
{
    if (W.G == 1) { W.GE = 0; W.ipl = 1; W.nblk = blocks_per_group(W.N, 0); return; }
    int most = 0;
    amap_host.assign((size_t)W.ngroups * W.G, -1);
    for (int g = 0; g < W.ngroups; g++) {
        int n = 0;
        for (int p = 0; p < W.G; p++) {
            const int b = g * W.G + p;
            if (b < W.nbatch && !st[b].done) amap_host[(size_t)g * W.G + n++] = p;
        }
        most = std::max(most, n);
    }
    if (W.ipl_max == 2 && 2 * most > W.G) {   // every position, two per lane
        W.ipl = 2;
        W.GE = W.G / 2;
        W.nblk = blocks_per_group(W.N, W.GE);
        return;
    }
    int ge = 1;
    while (ge < most) ge *= 2;
    W.ipl = 1;
    W.GE = ge;
    W.nblk = blocks_per_group(W.N, ge);
    if (ge < W.G && cudaMemcpyAsync(W.amap, amap_host.data(), sizeof(int) * amap_host.size(), cudaMemcpyHostToDevice, s) != cudaSuccess)
        fail(HEOM_E_CUDA, "copying the inner lane map failed");
}

template <typename T>
void inner_chunk(InnerWork<T> &W, const DevPlan &P, const DevCoef<T> &C, int iters, cudaStream_t s)
{
    DevPlan Q = P;
    Q.order = nullptr;   // entry order: coalesced epilogue access
    if (W.GE == 0) chunk_ge<T, 0, false, 1>(W, Q, C, iters, s);
    else if constexpr (kInterleaves<T>) {
        if (W.ipl == 2) df_chunk_pair(W, Q, C, iters, s);
        else if (W.GE == W.G) df_chunk_full(W, Q, C, iters, s);
        else df_chunk_compact(W, Q, C, iters, s);
    } else fail(HEOM_E_ARG, "inner workspace: interleave of a non-FP32x2 type");
}

#define INST(T)                                                                              \
    template void inner_alloc<T>(InnerWork<T> &, int, int64_t, cudaStream_t, int, int);      \
    template void inner_free<T>(InnerWork<T> &);                                              \
    template DevCoef<T> inner_layout_coef<T>(InnerWork<T> &, const DevPlan &, const DevCoef<T> &, cudaStream_t); \
    template void inner_rhs<T>(InnerWork<T> &, const DevPlan &, const double2 *, int, double, const float *, cudaStream_t); \
    template void inner_add_solution<T>(InnerWork<T> &, double2 *, int, double, int, cudaStream_t); \
    template void inner_shadow<T>(InnerWork<T> &, int, cudaStream_t);                          \
    template void inner_lanes<T>(InnerWork<T> &, const InnerState *, std::vector<int> &, cudaStream_t); \
    template void inner_start<T>(InnerWork<T> &, double, int, int, cudaStream_t);             \
    template void inner_chunk<T>(InnerWork<T> &, const DevPlan &, const DevCoef<T> &, int, cudaStream_t);    \
    template void inner_time<T>(InnerWork<T> &, const DevPlan &, const DevCoef<T> &, int, cudaStream_t, float &, float &);
INST(double)
INST(float)
INST(DF)

}  // namespace heom
