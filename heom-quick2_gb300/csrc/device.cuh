// Device-side views shared by the CUDA translation units.
#pragma once
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>

#include "numeric.cuh"
#include "plan.h"

namespace heom {

template <typename R> struct VT { using v2 = typename Num<R>::V; };

// Read-only device view of one plan.
struct DevPlan {
    int64_t lunk = 0;
    int32_t nado = 0, nslots = 0, nh = 0, ntrace = 0;
    const int32_t *ent_ado = nullptr, *ado_off = nullptr, *ado_cls = nullptr, *ado_cnt = nullptr;
    const int32_t *coup_ptr = nullptr, *coup_mid = nullptr, *cls_tptr = nullptr, *term_ptr = nullptr, *trace_idx = nullptr;
    const int4 *coup = nullptr;
    const uint32_t *maps = nullptr, *terms = nullptr;
    // thread -> entry order: entries grouped by their work profile (couplings, useful
    // gathers, same-tier terms) so that the threads of a warp follow the same trip counts
    const int32_t *order = nullptr;
};

// Parameter set of one apply: coefficient tables, per-instance H values and lead shifts.
template <typename T>
struct DevCoef {
    using V = typename Num<T>::V;
    const V *g0 = nullptr, *cl = nullptr, *cr = nullptr;
    const V *hval = nullptr;        // nh values per instance (instance stride nh)
    const double *eshift = nullptr; // 4 lead-shift slots per instance (FP64, converted in-kernel)
    // optional per-instance ADO diagonal g (nado per instance) precomputed from g0, g0_scale
    // and eshift: keeps FP64 arithmetic out of the FP32 / FP32x2 kernels
    const V *gdiag = nullptr;
    double g0_scale = 1;            // 0 switches the sum of damping rates off (derivative applies)
    int unit_on = 1;                // 0 drops the unit (higher-tier / RDO) couplings (derivative applies)
    int trace_on = 1;               // forward plan: write Tr(rho0) into the trace slot
    int h_real = 0;                 // all H values real: cheaper same-tier products
    // Regularised operator of the inner solves of mixed precision (forward plan only):
    // A acts on the Hermitian part of the RDO block (entries 0 .. nz0-1); its anti-Hermitian
    // part, scaled by reg_scale, goes to the anti-Hermitian part of the RDO output, and the
    // free trace unknown x[lunk] goes to the RDO diagonal (real part) and to Im y[lunk].
    int reg = 0;
    int32_t nz0 = 0, ndiag = 0;
    const int32_t *rdo_pair = nullptr;   // index of the transposed RDO entry
    double reg_scale = 0;
    // correlation-function operator: entries [h; a] of cf_half each, signed frequency per instance
    const double *cf_omega = nullptr;
    int64_t cf_half = 0;
    // left diagonal preconditioner of the inner solves: every row of ADO n is scaled by
    // pre[n] (the trace slot is not); nullptr = none
    const float *pre = nullptr;
    // truncated batches (instances of one table family at different hierarchy depths, on the
    // deepest member's tables): per instance, x = first stored entry of its last kept tier,
    // y = one past its last kept entry.  Rows from y on are zero, and the rows of the last
    // kept tier skip their couplings to the next tier (whose entries the caller keeps zero).
    // nullptr = every instance uses the whole hierarchy.
    const int2 *tier_lim = nullptr;
};

// Index of the shadow-vector component that instance b pairs with its entry i (N = lunk + 1
// elements per vector).  A truncated instance (tier_lim) pairs its trace slot with the
// component at its own hierarchy's trace index, tier_lim[b].y: its shadow vector is then the
// one a solve on its own tables uses (the prefix of the same drandn stream), and its Krylov
// iterates are those of that solve.
__device__ __forceinline__ int64_t shadow_index(const int2 *tier_lim, int b, int64_t i, int64_t N)
{
    return (tier_lim && i == N - 1) ? (int64_t)__ldg(&tier_lim[b].y) : i;
}

// Elements of type Num<T>::V that fill_gdiag needs for nbatch instances (the ADO diagonals).
template <typename T>
inline int64_t gdiag_elems(const DevPlan &P, int nbatch) { return std::max<int64_t>(1, (int64_t)P.nado * nbatch); }

// pre[n] = 1 / (|g0[n]| + hnorm): the inverse size of ADO n's diagonal block
void fill_pre(const DevPlan &P, const double2 *g0, double hnorm, float *pre, cudaStream_t s);

// y = A x (ADJ = false) or y = A^H x (ADJ = true) for nbatch instances (gridDim.y);
// vstride = complex elements between instance vectors; active[b] == 0 skips instance b.
// fill_gdiag writes into ws (gdiag_elems<T> elements) the per-instance ADO diagonals
// g[b][n] = g0_scale g0[n] + i sum_k cnt_k(n) eshift[b][k] and points C.gdiag at them.
template <typename T>
void fill_gdiag(const DevPlan &P, DevCoef<T> &C, typename Num<T>::V *ws, int nbatch, cudaStream_t s);

template <typename T, bool ADJ>
void launch_apply(const DevPlan &P, const DevCoef<T> &C, const typename Num<T>::V *x, typename Num<T>::V *y,
                  int nbatch, int64_t vstride, const int *active, cudaStream_t s);

}  // namespace heom
