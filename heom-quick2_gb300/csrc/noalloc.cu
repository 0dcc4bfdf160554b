// Allocation-free lead currents of a batch of device-resident states.
//
// The currents of td/calcj.f90:40-85 for nbatch instances whose vectors already sit on the
// device (for instance the states a heom_batch_solve_dev call leaves behind).  The per-
// instance sums land in a file-scope device array instead of a buffer allocated per call,
// so the entry point makes no cudaMalloc / cudaFree: a caller that polls the currents
// between solver rounds or time steps does not pay the device-wide synchronisation that
// cudaFree implies, and a caller that reserves all device memory up front keeps working.
//
// The scratch holds kMaxBatch x 4 doubles (128 KiB).  Every call writes every slot it
// reads back, so nothing has to start at zero.  The first call on a device looks up the
// array's device address (cudaGetSymbolAddress, with that device current); make that
// first call before any stream capture.  Two calls that overlap in time (two host threads,
// or two contexts on one device) share the scratch and race: serialise them.  The kernel
// runs on the context's non-blocking stream, which is not ordered after the caller's
// streams, so the states must be complete when the call is made.
#include <mutex>

#include "context.cuh"

namespace heom {
namespace {

constexpr int kMaxBatch = 4096;   // instances per call
constexpr int kSlots = 4;         // nalf * nspin <= 4
constexpr int kThreads = 256;
constexpr int kMaxDevices = 64;

static __device__ __align__(256) double g_current_scratch[kMaxBatch * kSlots];

std::mutex g_sym_mutex;
double *g_sym_addr[kMaxDevices] = {nullptr};

double *scratch_on(int device)
{
    if (device < 0 || device >= kMaxDevices) fail(HEOM_E_ARG, "device ordinal out of range");
    std::lock_guard<std::mutex> lock(g_sym_mutex);
    if (!g_sym_addr[device]) {
        void *p = nullptr;
        CK(cudaGetSymbolAddress(&p, g_current_scratch));   // the caller made `device` current
        if (!p) fail(HEOM_E_CUDA, "no device address for the current scratch");
        g_sym_addr[device] = (double *)p;
    }
    return g_sym_addr[device];
}

// One block per instance: jt[b][slot] = -2 jconst Im sum_terms sign * x_b[entry].
__global__ void k_batch_current(const double2 *x, int64_t vstride, const CurrentTerm *terms, int nterms, int nslot,
                                double *out)
{
    __shared__ double part[kThreads][kSlots];
    const double2 *xb = x + (int64_t)blockIdx.x * vstride;
    double acc[kSlots] = {0, 0, 0, 0};
    for (int k = threadIdx.x; k < nterms; k += kThreads) {
        const CurrentTerm tm = terms[k];
        const double v = (double)tm.sign * xb[tm.entry].y;
#pragma unroll
        for (int s = 0; s < kSlots; s++) acc[s] += (tm.slot == s) ? v : 0.0;
    }
    for (int s = 0; s < kSlots; s++) part[threadIdx.x][s] = acc[s];
    __syncthreads();
    for (int w = kThreads / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w)
            for (int s = 0; s < kSlots; s++) part[threadIdx.x][s] += part[threadIdx.x + w][s];
        __syncthreads();
    }
    if (threadIdx.x < nslot) out[(int64_t)blockIdx.x * nslot + threadIdx.x] = -2.0 * part[0][threadIdx.x] * kJconst;
}

}  // namespace
}  // namespace heom

using namespace heom;

extern "C" int heom_batch_current_static(heom_ctx *c, const void *x_dev, int32_t nbatch, int64_t vstride, double *jt)
{
    return guarded([&] {
        require_ctx(c);
        if (!x_dev || !jt) fail(HEOM_E_ARG, "null argument");
        if (nbatch < 1 || nbatch > kMaxBatch) fail(HEOM_E_ARG, "nbatch must be in 1..4096");
        if (vstride < c->lunk + 1) fail(HEOM_E_ARG, "vstride is shorter than lunk + 1");
        const int ns = c->nalf * c->nspin;
        if (ns > kSlots) fail(HEOM_E_ARG, "more than 4 lead/spin slots");
        DeviceScope dsc(c->device);
        double *scr = scratch_on(c->device);
        k_batch_current<<<nbatch, kThreads, 0, c->stream>>>((const double2 *)x_dev, vstride, c->d_cur_terms,
                                                            c->n_cur_terms, ns, scr);
        CK(cudaGetLastError());
        CK(cudaMemcpyAsync(jt, scr, sizeof(double) * (size_t)nbatch * ns, cudaMemcpyDeviceToHost, c->stream));
        CK(cudaStreamSynchronize(c->stream));
    });
}
