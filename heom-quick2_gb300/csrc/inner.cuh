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
#include <vector>

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

// Vector layout: instances are interleaved entry by entry in groups of G (G = 1 for FP64
// and FP32; for FP32x2 the smallest power of two >= nbatch, at most 32).  Element t of
// instance b sits at (b / G) gstride + t G + b % G.  A warp then holds 32 / G entries of G
// instances: lanes of one entry share the plan's records, map words and loop trip counts
// (one control flow per entry, plan reads broadcast to G lanes), and the gathered values of
// the G instances are adjacent in memory.
template <typename T>
struct InnerWork {
    using V = typename Num<T>::V;
    int nbatch = 0, nblk = 0;   // nblk: blocks of 256 threads per group in the current configuration
    int G = 1, ngroups = 0;     // instances per group, groups
    // current launch configuration: GE lanes per entry (0: G == 1, one instance per group);
    // when GE < G, slot j of group g serves position amap[g G + j] (-1: none), so that the
    // running instances of a group share fewer lanes and blocks (inner_lanes)
    int GE = 0;
    int *amap = nullptr;
    // instances per lane: ipl_max = 2 lets a lane serve two adjacent positions of its group
    // (GE = G / 2 lanes per entry; the plan is decoded once for both) while more than half of
    // a group's instances run; ipl is the current configuration's
    int ipl_max = 1, ipl = 1;
    int64_t N = 0;              // complex elements per instance (lunk + 1)
    int64_t vstride = 0;        // N rounded up to a multiple of 64
    int64_t gstride = 0;        // complex elements between groups (vstride G)
    V *x = nullptr, *xs = nullptr, *b = nullptr, *w = nullptr, *y = nullptr, *d = nullptr, *v = nullptr,
      *u1 = nullptr, *u2 = nullptr, *rt = nullptr;
    V *xs2 = nullptr;           // second iterate slot (xs is slot 0)
    __host__ __device__ V *slot(int s) const { return s ? xs2 : xs; }
    __host__ __device__ int64_t at(int inst, int64_t t) const
    {
        return (int64_t)(inst / G) * gstride + t * G + inst % G;
    }
    InnerState *st = nullptr;
    InnerCoef<T> *cf = nullptr;
    double *part = nullptr;     // per-block partials: 3 runs of nblk per instance (G ngroups instances)
    // truncated batches (DevCoef::tier_lim): the apply kernels skip blocks wholly beyond an
    // instance's last kept entry (their entries stay zero in every vector) and leave zero partials
    const int2 *tier_lim = nullptr;
    void *mem = nullptr;        // single allocation backing everything above
    void *coef_mem = nullptr;   // interleaved H values and ADO diagonals (inner_layout_coef)
};

// G: instances per entry group (a power of two <= 32; 0 = inner_default_interleave; FP64
// and FP32 workspaces always use 1); ipl: instances per lane (1, or 2 for FP32x2 with G > 1)
template <typename T> void inner_alloc(InnerWork<T> &W, int nbatch, int64_t N, cudaStream_t s, int G = 0, int ipl = 1);
// the smallest power of two >= nbatch, at most 32
inline int inner_default_interleave(int nbatch)
{
    int g = 1;
    while (g < nbatch && g < 32) g *= 2;
    return g;
}
template <typename T> void inner_free(InnerWork<T> &W);
// The coefficient set in the workspace's layout: C.hval (P.nh values per instance) and
// C.gdiag (P.nado per instance), both instance-major, copied into W's interleaved layout
// (W.coef_mem) when G > 1; C itself when G == 1.
template <typename T>
DevCoef<T> inner_layout_coef(InnerWork<T> &W, const DevPlan &P, const DevCoef<T> &C, cudaStream_t s);
// Right-hand side of instance `inst`: W.b = scale r (FP64, N elements), rows of ADO n times
// pre[n] when pre is given (the trace slot is not scaled).
template <typename T>
void inner_rhs(InnerWork<T> &W, const DevPlan &P, const double2 *r, int inst, double scale, const float *pre, cudaStream_t s);
// The shadow vector W.rt of the inner solves: sign-symmetric pseudo-random entries, a
// different vector for every `round`.  The reference's stream (all positive) left the inner
// solves of the Kanamori model at T = 0.1 without progress round after round: restarted on
// the same normalised residual with the same shadow vector, TFQMR repeats the same iterates.
template <typename T>
void inner_shadow(InnerWork<T> &W, int round, cudaStream_t s);
// x += a W.slot(slot) of instance `inst` (x: FP64, N elements).
template <typename T>
void inner_add_solution(InnerWork<T> &W, double2 *x, int inst, double a, int slot, cudaStream_t s);

// Start a solve: W.b holds the right-hand sides and W.rt the shadow vector.  An instance
// stops at the first check with ||b - A xs|| <= crit; with stag_window > 0 also at the
// arithmetic's floor (the true residual 10x above TFQMR's bound sqrt(2n+1) tau, or
// stag_window checks that fail to halve the best residual); or once nlim iterations ran.
template <typename T>
void inner_start(InnerWork<T> &W, double crit, int nlim, int stag_window, cudaStream_t s);
// Configure W for the next chunk from the instances' states (host copy): with two instances
// per lane allowed and more than half of some group's instances running, every position on
// G / 2 lanes of two instances; else GE = the smallest power of two >= the most running
// instances of any group, and their positions in the lane map (copied with cudaMemcpyAsync
// from amap_host, which must stay unchanged until the stream has passed the copy).
template <typename T>
void inner_lanes(InnerWork<T> &W, const InnerState *st, std::vector<int> &amap_host, cudaStream_t s);
// Enqueue `iters` iterations and one check in W's current configuration (capturable in a
// CUDA graph; W is captured by value).
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
