// Batched TFQMR on the device (role of tfqmr_double/dutfx.f90 + solve_tfqmr.f90).
#pragma once
#include <functional>

#include "device.cuh"

namespace heom {

// Scalars of one TFQMR instance (dutfx.f90 SAVE variables plus driver state).
struct TfqState {
    double rho, beta, alpha, var, eta, tau, cosv, r0, tol, resn, unrm, uchk, crit, xpend, dd, rho_next, ext_resid, best;
    int n, nlim, ierr, done, tres, axb, chk, conv_ext, stag, stag_window;
};

template <typename T>
struct TfqWork {
    using V = typename Num<T>::V;
    int nbatch = 0, nblk = 0;
    int64_t N = 0;          // complex elements per instance (lunk + 1)
    int64_t vstride = 0;    // complex elements between instances
    V *x = nullptr, *b = nullptr, *rt = nullptr, *v = nullptr, *w = nullptr, *y = nullptr, *d = nullptr, *u = nullptr,
      *t = nullptr, *s = nullptr;
    TfqState *st = nullptr;       // device, nbatch
    double *part = nullptr;       // nbatch * nblk * 2
    int *act_main = nullptr, *act_tres = nullptr, *act_chk = nullptr;
    const int2 *tier_lim = nullptr;   // truncated batches (DevCoef::tier_lim): shadow_index
    void *mem = nullptr;          // single allocation backing everything above
};

template <typename T> void tfq_alloc(TfqWork<T> &W, int nbatch, int64_t N, cudaStream_t s);
template <typename T> void tfq_free(TfqWork<T> &W);

// apply(x, y, active): y = A x for the instances whose active flag is set
template <typename T>
using ApplyFn = std::function<void(const typename Num<T>::V *, typename Num<T>::V *, const int *)>;

// Kernel launches of tfq_start and of one tfq_iteration (including guarded no-op launches).
constexpr int kTfqStartLaunches = 2;
constexpr int kTfqIterationLaunches = 21;

// Initialise the solve: expects W.b filled (right-hand side), W.rt filled (drandn stream).
// The every-50-applies test stops an instance at ||A x - b|| <= max(crit, rel_crit ||b||);
// stag_window > 0 also stops it after that many tests without halving the best residual.
template <typename T>
void tfq_start(TfqWork<T> &W, double tol, int nlim, double crit, double rel_crit, int stag_window, cudaStream_t s);
// Enqueue one TFQMR iteration (two operator applies plus the optional true-residual
// and every-50-applies residual checks, all guarded by device flags).
template <typename T> void tfq_iteration(TfqWork<T> &W, const ApplyFn<T> &apply, cudaStream_t s);
template <typename T> void vec_axpby(int64_t n, typename Num<T>::V *z, double a, const typename Num<T>::V *x, double bb,
                                     const typename Num<T>::V *y, cudaStream_t s);
template <typename T> void vec_from_d(int64_t n, const double2 *in, typename Num<T>::V *out, double scale, cudaStream_t s);
template <typename T> void vec_axpy_to_d(int64_t n, double2 *y, double a, const typename Num<T>::V *x, cudaStream_t s);
double device_norm2(int64_t n, const double2 *x, double *scratch, cudaStream_t s);
// Re(a^H b) (FP64, result on the host)
double device_dot(int64_t n, const double2 *a, const double2 *b, double *scratch, cudaStream_t s);

}  // namespace heom
