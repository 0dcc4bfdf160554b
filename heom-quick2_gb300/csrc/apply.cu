// The sparse HEOM Liouvillian apply on GB300 (sm_103a), one thread per stored entry
// (the per-entry arithmetic is apply_entry).  In FP64 the kernel is bounded by the FP64
// pipe; in FP32x2 by instruction issue on the FP32 / ALU pipes (double-float arithmetic,
// about 1 400 instructions per entry); in FP32 by gather latency.
#include <algorithm>
#include <type_traits>

#include "apply_entry.cuh"

namespace heom {

// __launch_bounds__(256, 6): at most 40 registers, six resident blocks per SM (measured 8 %
// faster than the unconstrained 46-register build for the FP32x2 apply, no spills)
template <typename T, bool ADJ, bool REG>
__global__ void __launch_bounds__(256, 6) k_apply(DevPlan P, DevCoef<T> C, const typename Num<T>::V *__restrict__ x,
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
    y[t] = Num<T>::store(apply_entry<T, ADJ, REG>(P, C, x, t, b));
}

template <typename T>
__global__ void k_fill_gdiag(DevPlan P, DevCoef<T> C, typename Num<T>::V *gdiag)
{
    using N = Num<T>;
    const int b = blockIdx.y;
    for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < P.nado; n += gridDim.x * blockDim.x) {
        const unsigned cnt = (unsigned)__ldg(P.ado_cnt + n);
        double es = 0;
        for (int k = 0; k < 4; k++) es += (double)(int8_t)(cnt >> (8 * k)) * C.eshift[b * 4 + k];
        const typename N::A g0 = N::load(C.g0[n]);
        gdiag[(int64_t)b * P.nado + n] = N::store(N::from_d(C.g0_scale * N::re(g0), C.g0_scale * N::im(g0) + es));
    }
}

template <typename T>
void fill_gdiag(const DevPlan &P, DevCoef<T> &C, typename Num<T>::V *ws, int nbatch, cudaStream_t s)
{
    dim3 grid((unsigned)std::max(1, std::min(1024, (P.nado + 255) / 256)), (unsigned)nbatch);
    DevCoef<T> K = C;
    K.gdiag = nullptr;
    k_fill_gdiag<T><<<grid, 256, 0, s>>>(P, K, ws);
    C.gdiag = ws;
}

template <typename T, bool ADJ>
void launch_apply(const DevPlan &P, const DevCoef<T> &C, const typename Num<T>::V *x, typename Num<T>::V *y,
                  int nbatch, int64_t vstride, const int *active, cudaStream_t s)
{
    dim3 grid((unsigned)((P.lunk + 1 + 255) / 256), (unsigned)nbatch);
    // the work-profile order pays in FP64 (FP64-pipe bound: divergence costs issue slots);
    // the FP32 / FP32x2 kernels keep entry order for coalesced entry, map and output access
    DevPlan Q = P;
    if (!std::is_same<T, double>::value) Q.order = nullptr;
    if (!ADJ && C.reg) k_apply<T, false, true><<<grid, 256, 0, s>>>(Q, C, x, y, vstride, active);
    else k_apply<T, ADJ, false><<<grid, 256, 0, s>>>(Q, C, x, y, vstride, active);
}

__global__ void k_fill_pre(DevPlan P, const double2 *__restrict__ g0, double hnorm, float *__restrict__ pre)
{
    for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < P.nado; n += gridDim.x * blockDim.x)
        pre[n] = (float)(1.0 / (sqrt(g0[n].x * g0[n].x + g0[n].y * g0[n].y) + hnorm));
}

void fill_pre(const DevPlan &P, const double2 *g0, double hnorm, float *pre, cudaStream_t s)
{
    k_fill_pre<<<std::max(1, std::min(1024, (P.nado + 255) / 256)), 256, 0, s>>>(P, g0, hnorm, pre);
}

template void fill_gdiag<double>(const DevPlan &, DevCoef<double> &, double2 *, int, cudaStream_t);
template void fill_gdiag<float>(const DevPlan &, DevCoef<float> &, float2 *, int, cudaStream_t);
template void fill_gdiag<DF>(const DevPlan &, DevCoef<DF> &, float4 *, int, cudaStream_t);
template void launch_apply<double, false>(const DevPlan &, const DevCoef<double> &, const double2 *, double2 *, int, int64_t, const int *, cudaStream_t);
template void launch_apply<double, true>(const DevPlan &, const DevCoef<double> &, const double2 *, double2 *, int, int64_t, const int *, cudaStream_t);
template void launch_apply<float, false>(const DevPlan &, const DevCoef<float> &, const float2 *, float2 *, int, int64_t, const int *, cudaStream_t);
template void launch_apply<float, true>(const DevPlan &, const DevCoef<float> &, const float2 *, float2 *, int, int64_t, const int *, cudaStream_t);
template void launch_apply<DF, false>(const DevPlan &, const DevCoef<DF> &, const float4 *, float4 *, int, int64_t, const int *, cudaStream_t);
template void launch_apply<DF, true>(const DevPlan &, const DevCoef<DF> &, const float4 *, float4 *, int, int64_t, const int *, cudaStream_t);

}  // namespace heom
