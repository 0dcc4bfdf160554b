// Fused batched TFQMR for the inner solves of mixed-precision refinement.
//
// Same Krylov method as solver.cuh (R. W. Freund, SIAM J. Sci. Comput. 14 (1993) 470),
// rearranged so that every vector update and inner product of an iteration runs inside
// the two operator applies of that iteration: the apply is bounded by instruction issue
// and leaves HBM mostly idle, so the streaming work rides along in its epilogue.
// Per iteration n (alpha = alpha_n, beta = beta_n):
//   B: u1 = A w + beta u2       (A applied to w, so y1 = w + beta y2 needs no pass of its own)
//      pending updates of iteration n-1: d1 = y1 + dd1 d, x += eta1 d1, y2 = y1 - alpha' v,
//      d2 = y2 + dd2 d1, x += eta2 d2, d = d2;  y1 = w + beta y2;  v = u1 + beta (u2 + beta v);
//      partial <r~, v>
//   B_fin: alpha = rho / sigma
//   A: u2 = u1 - alpha A v;  w1 = w - alpha u1;  w2 = w1 - alpha u2;  w = w2;
//      partials ||w1||^2, ||w2||^2, <r~, w2>
//   A_fin: the two half steps' var, cos, tau, eta; the pending coefficients; beta, rho
// Every `chunk` iterations a check forms xs = x + pending updates and ||b - A xs||; the
// solve of an instance ends at a check (converged, floor reached or iteration limit), or
// at the iteration where TFQMR's bound times the bound-to-true ratio of the last check
// predicts a residual of a third of the target; such an instance skips the rest of the
// chunk and the next check forms and measures its xs.  Checked iterates alternate between
// two slots so that the best one is kept: it is the result, also when an instance stops
// at its arithmetic's floor after the residual has begun to drift up.  Inner products are summed per thread and per warp in the vectors'
// number type and across warps and blocks in FP64, in a fixed order (deterministic).
// Launches per iteration: 4 (no guarded no-ops).  The FP64 reference solver keeps the
// unfused form of solver.cuh, whose iterates follow the reference driver step by step.
#pragma once
#include "device.cuh"

namespace heom {

struct InnerState {
    double r0, tau, var, eta, rho, beta, alpha, crit, best, ext_resid, unrm;
    double ratio;      // true residual / TFQMR's bound sqrt(2n+1) tau at the last check (0 before it)
    double best_e;     // smallest checked residual, held by iterate slot best_slot
    int n, nlim, done, ierr, stag, stag_window, checks, conv;
    int finishing;     // stopped on the predicted residual: the next check forms and measures xs
    int best_slot;     // 0 or 1: which xs slot holds the best checked iterate (the result)
};

// Per-instance scalars in the number type of the vectors, written by the finalisers so
// that the fused kernels do no FP64 arithmetic.
template <typename T>
struct InnerCoef {
    typename Num<T>::S beta, alpha, alpha_prev, dd1, eta1, dd2, eta2;
};

template <typename T>
struct InnerWork {
    using V = typename Num<T>::V;
    int nbatch = 0, nblk = 0;   // nblk: blocks of 256 per instance, one entry per thread
    int64_t N = 0;              // complex elements per instance (lunk + 1)
    int64_t vstride = 0;        // complex elements between instances
    V *x = nullptr, *xs = nullptr, *b = nullptr, *w = nullptr, *y = nullptr, *d = nullptr, *v = nullptr,
      *u1 = nullptr, *u2 = nullptr, *rt = nullptr;
    V *xs2 = nullptr;           // second iterate slot (xs is slot 0)
    __host__ __device__ V *slot(int s) const { return s ? xs2 : xs; }
    InnerState *st = nullptr;
    InnerCoef<T> *cf = nullptr;
    double *part = nullptr;     // per-block partials: 3 runs of nblk per instance
    // truncated batches (DevCoef::tier_lim): the apply kernels skip blocks wholly beyond an
    // instance's last kept entry (their entries stay zero in every vector) and leave zero partials
    const int2 *tier_lim = nullptr;
    void *mem = nullptr;        // single allocation backing everything above
};

template <typename T> void inner_alloc(InnerWork<T> &W, int nbatch, int64_t N, cudaStream_t s);
template <typename T> void inner_free(InnerWork<T> &W);

// Start a solve: W.b holds the right-hand sides and W.rt the shadow vector.  An instance
// stops at the first check with ||b - A xs|| <= crit; with stag_window > 0 also at the
// arithmetic's floor (the true residual 10x above TFQMR's bound sqrt(2n+1) tau, or
// stag_window checks that fail to halve the best residual); or once nlim iterations ran.
template <typename T>
void inner_start(InnerWork<T> &W, double crit, int nlim, int stag_window, cudaStream_t s);
// Enqueue `iters` iterations and one check (capturable in a CUDA graph).
template <typename T>
void inner_chunk(InnerWork<T> &W, const DevPlan &P, const DevCoef<T> &C, int iters, cudaStream_t s);

// Measurement: fill the workspace with a fixed pattern (no instance done), then time `reps`
// launches of the B kernel and of the A kernel; milliseconds per launch.
template <typename T>
void inner_time(InnerWork<T> &W, const DevPlan &P, const DevCoef<T> &C, int reps, cudaStream_t s, float &ms_b, float &ms_a);

constexpr int kInnerStartLaunches = 2;
constexpr int kInnerIterationLaunches = 4;
constexpr int kInnerCheckLaunches = 3;

}  // namespace heom
