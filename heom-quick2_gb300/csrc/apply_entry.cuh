// One output entry of the sparse HEOM Liouvillian apply, shared by the plain apply kernel
// and by the fused inner-solver kernels.
//
// Role: tfqmr_double/calc_ax_tfqmr_spa_omp.f90 (steady, with the Tr rho0 row),
// td/calcderiv_spa_omp.f90 (time-dependent lead shifts, no trace row) and the
// adjoint of the former.  For entry t the value is
//   g x  +  same-tier commutator terms of its pattern class  +  one or two signed
//   gathers per coupled ADO (left and right operator products),
// where every gather is a precomputed index into the source ADO's stored entries.
// The higher-tier couplings have coefficients +-i and cost only additions; the
// lower-tier ones multiply by the bath residues cb, cd.
//
// REG selects the regularised operator of the mixed-precision inner solves (see DevCoef):
// reads of RDO entries (source offset 0) see the Hermitian part (x_q + conj x_q')/2.
// CF selects the correlation-function operator (corrfunc/calc_ax_cf_spa_omp.f90) on a plan
// of build_cf_plan: its unit pairs are real (no factor i), and every entry adds the
// frequency term -w x[t + half] (h rows) or +w x[t - half] (a rows).
#pragma once
#include "device.cuh"

namespace heom {

template <typename T>
__device__ __forceinline__ typename Num<T>::A herm_part(const typename Num<T>::V *__restrict__ x, const int32_t *pair, int q,
                                                      int xs)
{
    using N = Num<T>;
    return N::half(N::add(N::load(x[(int64_t)q * xs]), N::conj(N::load(x[(int64_t)__ldg(pair + q) * xs]))));
}

// y[t] of NI instances b[0 .. NI) (x[i]: instance b[i]'s vector); t in [0, lunk], lunk = the
// trace slot.  Interleaved layout (the fused inner solves): with XS = 0 the stride xs_rt (a
// power of two) applies: instances interleaved entry by entry in groups of xs_rt, element k
// of instance b[i] at x[i][k xs_rt], and the per-instance ADO diagonals and H values
// interleaved the same way within each group.  XS = 1: one instance per vector (the plain
// applies).  NI > 1: the instances sit in one interleaved group (XS != 1) and share the
// decode of the plan (entry, pattern class, coupling records, map words, coefficients);
// only the loads of their values and their arithmetic are per instance.  Truncated batches
// (C.tier_lim) use NI = 1.
template <typename T, bool ADJ, bool REG, bool CF = false, int XS = 1, int NI = 1>
__device__ __forceinline__ void apply_entries(const DevPlan &P, const DevCoef<T> &C,
                                              const typename Num<T>::V *const (&x)[NI], int64_t t, const int (&b)[NI],
                                              typename Num<T>::A (&y)[NI], int xs_rt = 1)
{
    using N = Num<T>;
    using A = typename N::A;
    static_assert(NI == 1 || XS != 1, "instances sharing a thread sit in one interleaved group");
    const int xs = XS > 0 ? XS : xs_rt;
    const int bg = XS == 1 ? b[0] : b[0] / xs;   // the group of the instances
    int bl[NI];                                  // their lanes in the group
#pragma unroll
    for (int i = 0; i < NI; i++) bl[i] = XS == 1 ? 0 : b[i] - bg * xs;
    if (t == P.lunk) {   // the trace slot
#pragma unroll
        for (int i = 0; i < NI; i++) {
            A s = N::zero();
            if (!ADJ && C.trace_on)
                for (int k = 0; k < P.ntrace; k++)
                    s = N::add(s, REG ? herm_part<T>(x[i], C.rdo_pair, P.trace_idx[k], xs) : N::load(x[i][(int64_t)P.trace_idx[k] * xs]));
            if (REG) s = N::add(s, N::from_d(0.0, C.reg_scale * N::im(N::load(x[i][(int64_t)(t) * xs]))));
            y[i] = s;
        }
        return;
    }
    if (NI == 1 && C.tier_lim && t >= __ldg(&C.tier_lim[b[0]].y)) {   // beyond the instance's tier
        y[0] = N::zero();
        return;
    }
    const int n = __ldg(P.ent_ado + t);
    const int off = __ldg(P.ado_off + n);
    const int p = (int)(t - off);
    const int c = __ldg(P.ado_cls + n);
    const typename N::V *hv[NI];
#pragma unroll
    for (int i = 0; i < NI; i++) hv[i] = C.hval + (int64_t)bg * P.nh * xs + bl[i];

    // g = sum over the drawers of (cgamma + i dipm eshift)
    A acc[NI];
    const bool rdo = REG && off == 0;   // output row and same-tier sources in the RDO block
#pragma unroll
    for (int i = 0; i < NI; i++) {
        A g;
        if (C.gdiag) g = N::load(C.gdiag[(int64_t)bg * P.nado * xs + (int64_t)n * xs + bl[i]]);
        else {
            const unsigned cnt = (unsigned)__ldg(P.ado_cnt + n);
            double es = 0;
#pragma unroll
            for (int k = 0; k < 4; k++) es += (double)(int8_t)(cnt >> (8 * k)) * C.eshift[b[i] * 4 + k];
            g = N::add(N::scale(N::load(C.g0[n]), N::sc(C.g0_scale)), N::from_d(0.0, es));
        }
        if (ADJ) g = N::conj(g);
        acc[i] = N::mul(g, rdo ? herm_part<T>(x[i], C.rdo_pair, (int)t, xs) : N::load(x[i][(int64_t)(t) * xs]));
    }
    if (rdo) {
        const int q = (int)t, qp = __ldg(C.rdo_pair + q);
#pragma unroll
        for (int i = 0; i < NI; i++) {
            const A xq = N::load(x[i][(int64_t)(q) * xs]);
            acc[i] = N::add(acc[i], N::scale(N::sub(xq, N::conj(N::load(x[i][(int64_t)(qp) * xs]))), N::sc(0.5 * C.reg_scale)));
            if (qp == q) acc[i] = N::add(acc[i], N::from_d(C.reg_scale * N::re(N::load(x[i][(int64_t)(P.lunk) * xs])) / C.ndiag, 0.0));
        }
    }
    if (CF) {   // dfacta = -s, dfactb = +s (calc_ax_cf_spa_omp.f90:96-105); cf_omega[b] = s w
        const bool hrow = t < C.cf_half;
        const int64_t u = hrow ? t + C.cf_half : t - C.cf_half;
#pragma unroll
        for (int i = 0; i < NI; i++) {
            const double w = hrow ? -C.cf_omega[b[i]] : C.cf_omega[b[i]];
            acc[i] = N::add(acc[i], N::scale(N::load(x[i][u * xs]), N::sc(w)));
        }
    }

    // same tier: -i H X + i X H restricted to the class pattern (adjoint: conj'ed coefficients)
    const int tb = __ldg(P.cls_tptr + c) + p;
    const int k0 = __ldg(P.term_ptr + tb), k1 = __ldg(P.term_ptr + tb + 1);
    // one signed sum: right terms (x H) count +, left terms (H x) count - (no divergent branch)
    A sd[NI];
#pragma unroll
    for (int i = 0; i < NI; i++) sd[i] = N::zero();
    for (int k = k0; k < k1; k++) {
        const uint32_t w = __ldg(P.terms + k);
        const int hq = (int)((w >> 16) & 0x7FFF), q = (int)(w & 0xFFFF);
#pragma unroll
        for (int i = 0; i < NI; i++) {
            A h = N::load(hv[i][(int64_t)hq * xs]);
            if (ADJ) h = N::conj(h);
            const A xv = rdo ? herm_part<T>(x[i], C.rdo_pair, q, xs) : N::load(x[i][(int64_t)(off + q) * xs]);
            const A hx = C.h_real ? N::scale(xv, N::re_s(h)) : N::mul(h, xv);
            sd[i] = N::add(sd[i], N::flip(hx, (w >> 31) ^ 1u, 0u));
        }
    }
    // forward: acc += i (sum_right - sum_left); adjoint: acc += -i (...)
#pragma unroll
    for (int i = 0; i < NI; i++) {
        const A dlt = N::mul_i(N::norm(sd[i]));
        acc[i] = N::add(acc[i], ADJ ? N::neg(dlt) : dlt);
    }

    // couplings to the neighbouring tiers: coefficient pairs (lower tier) first, then the
    // unit pairs (higher tier / RDO); a map word holds the left and right source entries
    // (q + 1, 0 = none) with their signs in bit 15
    const int e0 = __ldg(P.coup_ptr + n), em = __ldg(P.coup_mid + n), e1 = __ldg(P.coup_ptr + n + 1);
    for (int e = e0; e < em; e++) {
        const int4 rec = __ldg(P.coup + e);
        const uint32_t mw = __ldg(P.maps + rec.y + p);
        const uint32_t cj = (uint32_t)rec.z >> 31, lo = mw & 0xFFFFu, hi = mw >> 16;
        const bool src_rdo = REG && rec.x == 0;
        const int cid = rec.z & 0x3FFFFFFF;
        if (lo) {
            const A cl = N::load(C.cl[cid]);
            const int q = (int)(lo & 0x7FFF) - 1;
#pragma unroll
            for (int i = 0; i < NI; i++) {
                const A v = src_rdo ? herm_part<T>(x[i], C.rdo_pair, q, xs) : N::load(x[i][(int64_t)(rec.x + q) * xs]);
                acc[i] = N::add(acc[i], N::mul(cl, N::flip(v, lo >> 15, cj)));
            }
        }
        if (hi) {
            const A cr = N::load(C.cr[cid]);
            const int q = (int)(hi & 0x7FFF) - 1;
#pragma unroll
            for (int i = 0; i < NI; i++) {
                const A v = src_rdo ? herm_part<T>(x[i], C.rdo_pair, q, xs) : N::load(x[i][(int64_t)(rec.x + q) * xs]);
                acc[i] = N::add(acc[i], N::mul(cr, N::flip(v, hi >> 15, cj)));
            }
        }
        if ((e - e0) & 1)
#pragma unroll
            for (int i = 0; i < NI; i++) acc[i] = N::norm(acc[i]);
    }
    // cL v + cR v' with cL = i sL, cR = i sR: accumulate sL v + sR v', times i below
    A ua[NI];
#pragma unroll
    for (int i = 0; i < NI; i++) ua[i] = N::zero();
    // the last kept tier of a truncated instance has no higher-tier couplings
    const int eu = (C.unit_on && (ADJ || !C.tier_lim || off < __ldg(&C.tier_lim[b[0]].x))) ? e1 : em;
    for (int e = em; e < eu; e++) {
        const int4 rec = __ldg(P.coup + e);
        const uint32_t mw = __ldg(P.maps + rec.y + p);
        const uint32_t cj = (uint32_t)rec.z >> 31, lo = mw & 0xFFFFu, hi = mw >> 16;
        const bool src_rdo = REG && rec.x == 0;
        if (lo) {
            const int q = (int)(lo & 0x7FFF) - 1;
            const uint32_t ng = ((lo >> 15) ^ (uint32_t)rec.z) & 1u;
#pragma unroll
            for (int i = 0; i < NI; i++) {
                const A v = src_rdo ? herm_part<T>(x[i], C.rdo_pair, q, xs) : N::load(x[i][(int64_t)(rec.x + q) * xs]);
                ua[i] = N::add(ua[i], N::flip(v, ng, cj));
            }
        }
        if (hi) {
            const int q = (int)(hi & 0x7FFF) - 1;
            const uint32_t ng = ((hi >> 15) ^ ((uint32_t)rec.z >> 1)) & 1u;
#pragma unroll
            for (int i = 0; i < NI; i++) {
                const A v = src_rdo ? herm_part<T>(x[i], C.rdo_pair, q, xs) : N::load(x[i][(int64_t)(rec.x + q) * xs]);
                ua[i] = N::add(ua[i], N::flip(v, ng, cj));
            }
        }
        if (((e - e0) & 3) == 3)
#pragma unroll
            for (int i = 0; i < NI; i++) ua[i] = N::norm(ua[i]);
    }
    const float pre = C.pre ? __ldg(C.pre + n) : 1.f;
#pragma unroll
    for (int i = 0; i < NI; i++) {
        acc[i] = N::add(acc[i], CF ? ua[i] : N::mul_i(ua[i]));
        if (C.pre) acc[i] = N::scale(acc[i], N::sc((double)pre));
        y[i] = acc[i];
    }
}

// One instance: y[t] of instance b, x its vector (see apply_entries).
template <typename T, bool ADJ, bool REG, bool CF = false, int XS = 1>
__device__ __forceinline__ typename Num<T>::A apply_entry(const DevPlan &P, const DevCoef<T> &C,
                                                          const typename Num<T>::V *__restrict__ x, int64_t t, int b,
                                                          int xs_rt = 1)
{
    const typename Num<T>::V *const xv[1] = {x};
    const int bv[1] = {b};
    typename Num<T>::A y[1];
    apply_entries<T, ADJ, REG, CF, XS, 1>(P, C, xv, t, bv, y, xs_rt);
    return y[0];
}


}  // namespace heom
