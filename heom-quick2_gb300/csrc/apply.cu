// The sparse HEOM Liouvillian apply on GB300 (sm_103a), one thread per stored entry.
//
// Role: tfqmr_double/calc_ax_tfqmr_spa_omp.f90 (steady, with the Tr rho0 row),
// td/calcderiv_spa_omp.f90 (time-dependent lead shifts, no trace row) and the
// adjoint of the former.  Per output entry the thread accumulates
//   g x  +  same-tier commutator terms of its pattern class  +  one or two signed
//   gathers per coupled ADO (left and right operator products),
// where every gather is a precomputed index into the source ADO's stored entries.
// The higher-tier couplings have coefficients +-i and cost only additions; the
// lower-tier ones multiply by the bath residues cb, cd.  In FP64 the kernel is
// bounded by the FP64 pipe; in FP32x2 by instruction issue on the FP32 / ALU pipes
// (double-float arithmetic, about 1 400 instructions per entry); in FP32 by gather latency.
//
// REG selects the regularised operator of the mixed-precision inner solves (see DevCoef):
// reads of RDO entries (source offset 0) see the Hermitian part (x_q + conj x_q')/2.
#include <algorithm>
#include <type_traits>

#include "device.cuh"

namespace heom {

template <typename T>
__device__ __forceinline__ typename Num<T>::A herm_part(const typename Num<T>::V *__restrict__ x, const int32_t *pair, int q)
{
    using N = Num<T>;
    return N::half(N::add(N::load(x[q]), N::conj(N::load(x[__ldg(pair + q)]))));
}

// __launch_bounds__(256, 6): at most 40 registers, six resident blocks per SM (measured 8 %
// faster than the unconstrained 46-register build for the FP32x2 apply, no spills)
template <typename T, bool ADJ, bool REG>
__global__ void __launch_bounds__(256, 6) k_apply(DevPlan P, DevCoef<T> C, const typename Num<T>::V *__restrict__ x,
                                               typename Num<T>::V *__restrict__ y, int64_t vstride,
                                               const int *__restrict__ active)
{
    using N = Num<T>;
    using A = typename N::A;
    const int b = blockIdx.y;
    if (active && !active[b]) return;
    x += (int64_t)b * vstride;
    y += (int64_t)b * vstride;
    const int64_t tid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (tid > P.lunk) return;
    const int64_t t = (tid < P.lunk && P.order) ? (int64_t)__ldg(P.order + tid) : tid;
    if (t == P.lunk) {   // the trace slot
        A s = N::zero();
        if (!ADJ && C.trace_on)
            for (int k = 0; k < P.ntrace; k++)
                s = N::add(s, REG ? herm_part<T>(x, C.rdo_pair, P.trace_idx[k]) : N::load(x[P.trace_idx[k]]));
        if (REG) s = N::add(s, N::from_d(0.0, C.reg_scale * N::im(N::load(x[t]))));
        y[t] = N::store(s);
        return;
    }
    const int n = __ldg(P.ent_ado + t);
    const int off = __ldg(P.ado_off + n);
    const int p = (int)(t - off);
    const int c = __ldg(P.ado_cls + n);
    const typename N::V *hv = C.hval + (int64_t)b * P.nh;

    // g = sum over the drawers of (cgamma + i dipm eshift)
    A g;
    if (C.gdiag) g = N::load(C.gdiag[(int64_t)b * P.nado + n]);
    else {
        const unsigned cnt = (unsigned)__ldg(P.ado_cnt + n);
        double es = 0;
#pragma unroll
        for (int k = 0; k < 4; k++) es += (double)(int8_t)(cnt >> (8 * k)) * C.eshift[b * 4 + k];
        g = N::add(N::scale(N::load(C.g0[n]), N::sc(C.g0_scale)), N::from_d(0.0, es));
    }
    if (ADJ) g = N::conj(g);
    const bool rdo = REG && off == 0;   // output row and same-tier sources in the RDO block
    A acc = N::mul(g, rdo ? herm_part<T>(x, C.rdo_pair, (int)t) : N::load(x[t]));
    if (rdo) {
        const int q = (int)t, qp = __ldg(C.rdo_pair + q);
        const A xq = N::load(x[q]);
        acc = N::add(acc, N::scale(N::sub(xq, N::conj(N::load(x[qp]))), N::sc(0.5 * C.reg_scale)));
        if (qp == q) acc = N::add(acc, N::from_d(C.reg_scale * N::re(N::load(x[P.lunk])) / C.ndiag, 0.0));
    }

    // same tier: -i H X + i X H restricted to the class pattern (adjoint: conj'ed coefficients)
    const int tb = __ldg(P.cls_tptr + c) + p;
    const int k0 = __ldg(P.term_ptr + tb), k1 = __ldg(P.term_ptr + tb + 1);
    // one signed sum: right terms (x H) count +, left terms (H x) count - (no divergent branch)
    A sd = N::zero();
    for (int k = k0; k < k1; k++) {
        const uint32_t w = __ldg(P.terms + k);
        A h = N::load(hv[(w >> 16) & 0x7FFF]);
        if (ADJ) h = N::conj(h);
        const A xs = rdo ? herm_part<T>(x, C.rdo_pair, (int)(w & 0xFFFF)) : N::load(x[off + (int)(w & 0xFFFF)]);
        const A hx = C.h_real ? N::scale(xs, N::re_s(h)) : N::mul(h, xs);
        sd = N::add(sd, (w >> 31) ? hx : N::neg(hx));
    }
    // forward: acc += i (sum_right - sum_left); adjoint: acc += -i (...)
    const A dlt = N::mul_i(N::norm(sd));
    acc = N::add(acc, ADJ ? N::neg(dlt) : dlt);

    // couplings to the neighbouring tiers
    const int e0 = __ldg(P.coup_ptr + n), e1 = __ldg(P.coup_ptr + n + 1);
    A ua = N::zero();   // sum of unit-coefficient contributions (times -i at the end)
    for (int e = e0; e < e1; e++) {
        const int4 rec = __ldg(P.coup + e);
        const uint32_t mw = __ldg(P.maps + rec.y + p);
        if (!mw) continue;
        const bool cj = rec.z < 0;
        const uint32_t lo = mw & 0xFFFFu, hi = mw >> 16;
        A vl = N::zero(), vr = N::zero();
        const bool src_rdo = REG && rec.x == 0;
        if (lo) {
            vl = src_rdo ? herm_part<T>(x, C.rdo_pair, (int)(lo & 0x7FFF) - 1) : N::load(x[rec.x + (int)(lo & 0x7FFF) - 1]);
            if (cj) vl = N::conj(vl);
            if (lo & 0x8000u) vl = N::neg(vl);
        }
        if (hi) {
            vr = src_rdo ? herm_part<T>(x, C.rdo_pair, (int)(hi & 0x7FFF) - 1) : N::load(x[rec.x + (int)(hi & 0x7FFF) - 1]);
            if (cj) vr = N::conj(vr);
            if (hi & 0x8000u) vr = N::neg(vr);
        }
        if (rec.z & kCoefUnit) {
            // cL v + cR v' with cL = i sL, cR = i sR: accumulate sL v + sR v', times i below
            if (C.unit_on) {
                ua = N::add(ua, (rec.z & 1) ? N::neg(vl) : vl);
                ua = N::add(ua, (rec.z & 2) ? N::neg(vr) : vr);
            }
        } else {
            const int cid = rec.z & 0x3FFFFFFF;
            if (lo) acc = N::add(acc, N::mul(N::load(C.cl[cid]), vl));
            if (hi) acc = N::add(acc, N::mul(N::load(C.cr[cid]), vr));
            if ((e - e0) & 1) acc = N::norm(acc);
        }
        if (((e - e0) & 3) == 3) ua = N::norm(ua);
    }
    acc = N::add(acc, N::mul_i(ua));
    y[t] = N::store(acc);
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
void fill_gdiag(const DevPlan &P, const DevCoef<T> &C, typename Num<T>::V *gdiag, int nbatch, cudaStream_t s)
{
    dim3 grid((unsigned)std::max(1, std::min(1024, (P.nado + 255) / 256)), (unsigned)nbatch);
    DevCoef<T> K = C;
    K.gdiag = nullptr;
    k_fill_gdiag<T><<<grid, 256, 0, s>>>(P, K, gdiag);
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

template void fill_gdiag<double>(const DevPlan &, const DevCoef<double> &, double2 *, int, cudaStream_t);
template void fill_gdiag<float>(const DevPlan &, const DevCoef<float> &, float2 *, int, cudaStream_t);
template void fill_gdiag<DF>(const DevPlan &, const DevCoef<DF> &, float4 *, int, cudaStream_t);
template void launch_apply<double, false>(const DevPlan &, const DevCoef<double> &, const double2 *, double2 *, int, int64_t, const int *, cudaStream_t);
template void launch_apply<double, true>(const DevPlan &, const DevCoef<double> &, const double2 *, double2 *, int, int64_t, const int *, cudaStream_t);
template void launch_apply<float, false>(const DevPlan &, const DevCoef<float> &, const float2 *, float2 *, int, int64_t, const int *, cudaStream_t);
template void launch_apply<float, true>(const DevPlan &, const DevCoef<float> &, const float2 *, float2 *, int, int64_t, const int *, cudaStream_t);
template void launch_apply<DF, false>(const DevPlan &, const DevCoef<DF> &, const float4 *, float4 *, int, int64_t, const int *, cudaStream_t);
template void launch_apply<DF, true>(const DevPlan &, const DevCoef<DF> &, const float4 *, float4 *, int, int64_t, const int *, cudaStream_t);

}  // namespace heom
