// Device-side views shared by the CUDA translation units.
#pragma once
#include <cuda_runtime.h>

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
    const int32_t *coup_ptr = nullptr, *cls_tptr = nullptr, *term_ptr = nullptr, *trace_idx = nullptr;
    const int4 *coup = nullptr;
    const uint32_t *maps = nullptr, *terms = nullptr;
};

// Parameter set of one apply: coefficient tables, per-instance H values and lead shifts.
template <typename T>
struct DevCoef {
    using V = typename Num<T>::V;
    const V *g0 = nullptr, *cl = nullptr, *cr = nullptr;
    const V *hval = nullptr;        // nh values per instance (instance stride nh)
    const double *eshift = nullptr; // 4 lead-shift slots per instance (FP64, converted in-kernel)
    double g0_scale = 1;            // 0 switches the sum of damping rates off (derivative applies)
    int unit_on = 1;                // 0 drops the unit (higher-tier / RDO) couplings (derivative applies)
    int trace_on = 1;               // forward plan: write Tr(rho0) into the trace slot
    int h_real = 0;                 // all H values real: cheaper same-tier products
};

// y = A x (ADJ = false) or y = A^H x (ADJ = true) for nbatch instances (gridDim.y);
// vstride = complex elements between instance vectors; active[b] == 0 skips instance b.
template <typename T, bool ADJ>
void launch_apply(const DevPlan &P, const DevCoef<T> &C, const typename Num<T>::V *x, typename Num<T>::V *y,
                  int nbatch, int64_t vstride, const int *active, cudaStream_t s);

}  // namespace heom
