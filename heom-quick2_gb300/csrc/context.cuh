// The opaque heom_ctx: device plans, coefficient sets and work buffers of one model.
#pragma once
#include <map>
#include <memory>

#include "solver.cuh"

namespace heom {

void cuda_check(cudaError_t e, const char *what);
#define CK(call) ::heom::cuda_check((call), #call)

// Makes device `dev` current for the lifetime of the object and gives the caller's current
// device back on exit: an entry point called with a context of another device neither
// launches on the wrong device nor leaves the caller's device selection changed.
struct DeviceScope {
    int prev = -1;
    explicit DeviceScope(int dev)
    {
        if (cudaGetDevice(&prev) != cudaSuccess) prev = -1;
        if (prev != dev) CK(cudaSetDevice(dev));
    }
    ~DeviceScope()
    {
        if (prev >= 0) cudaSetDevice(prev);
    }
    DeviceScope(const DeviceScope &) = delete;
    DeviceScope &operator=(const DeviceScope &) = delete;
};

// The launches that `enqueue` makes on stream s, captured into a graph and instantiated.
// When enqueue or the capture fails, the capture is ended and the partial graph released
// before the exception propagates, so that the context's stream stays usable.
struct CapturedGraph {
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    void release()
    {
        if (exec) cudaGraphExecDestroy(exec);
        if (graph) cudaGraphDestroy(graph);
        exec = nullptr;
        graph = nullptr;
    }
};
template <typename F>
CapturedGraph capture_graph(cudaStream_t s, F &&enqueue)
{
    CapturedGraph cg;
    CK(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
    try {
        enqueue();
    } catch (...) {
        cudaStreamEndCapture(s, &cg.graph);
        cg.release();
        throw;
    }
    CK(cudaStreamEndCapture(s, &cg.graph));
    const cudaError_t e = cudaGraphInstantiate(&cg.exec, cg.graph, 0);
    if (e != cudaSuccess) {
        cg.release();
        CK(e);
    }
    return cg;
}

// Device copy of one HostPlan plus its coefficient tables in both precisions.
struct PlanDev {
    DevPlan view;
    std::vector<void *> blocks;
    double2 *g0_64 = nullptr, *cl_64 = nullptr, *cr_64 = nullptr;
    float2 *g0_32 = nullptr, *cl_32 = nullptr, *cr_32 = nullptr;
    float4 *g0_df = nullptr, *cl_df = nullptr, *cr_df = nullptr;
    int64_t ncoef = 0;
    void upload(const HostPlan &P);
    void release();
    template <typename R> DevCoef<R> coef() const;
};

// Extra per-entry data used by observables.
struct CurrentTerm {
    int32_t entry;   // global entry of a first-tier + ADO
    int32_t slot;    // ialf-1 + (ispin-1)*nalf
    float sign;      // sign of the a_{ms} element
};

// The coefficient sets of one operator in the three number types.
struct CoefSet {
    DevCoef<double> k64;
    DevCoef<float> k32;
    DevCoef<DF> kdf;
};

}  // namespace heom

struct heom_ctx;

namespace heom {
// Shared host helpers of the C-ABI translation units.
CoefSet ctx_coefs(heom_ctx *c, bool adj = false);
void require_ctx(heom_ctx *c);
void herm_rdo(heom_ctx *c, cd *rho);
void set_params(heom_ctx *c, const std::vector<cd> &hs, const double *es);
void solve_device(heom_ctx *c, const heom_solve_opts &o, double2 *x, int nbatch, int64_t vstride, bool adj,
                  const double2 *rhs, heom_solve_info &info, const CoefSet &K);
// FP64 TFQMR on op(x) = rhs for one instance (x: initial guess in, solution out), stopping
// at ||rhs - op(x)|| <= crit_abs.
void solve_custom64(heom_ctx *c, const ApplyFn<double> &op, const double2 *rhs, double2 *x, double crit_abs, int maxit0,
                    heom_solve_info &info);
// Mixed-precision solve of op(x) = rhs for one instance (x: initial guess in, solution out):
// rounds of FP64 residual r = rhs - op64(x), FP32x2 TFQMR on opdf(d) = r / ||r|| to
// max(crit_abs / ||r||, 1e-10) or its floor, x += ||r|| d, until ||r|| <= crit_abs; a round
// that fails to halve ||r|| hands the rest to solve_custom64.
void solve_custom_mixed(heom_ctx *c, const ApplyFn<double> &op64, const ApplyFn<DF> &opdf, const double2 *rhs, double2 *x,
                        double crit_abs, int maxit0, heom_solve_info &info);
// Values of a full nrho x nrho matrix on the context's H structure (FP64).
void hvalues64(heom_ctx *c, const cd *hs, std::vector<double2> &h64);
double device_rdot(heom_ctx *c, int64_t n, const double2 *a, const double2 *b);
// Batched FP64 TFQMR iterations until every instance of W has finished (graph-captured
// chunks on the context's stream); iters: iterations launched.
void run_tfqmr64(heom_ctx *c, TfqWork<double> &W, const ApplyFn<double> &apply, int nlim, int &iters, int64_t &launches);
// Mixed-precision refinement of A x = rhs (rhs == nullptr: the steady problem on the
// regularised operator) for nbatch instances of N elements on the plan PV: rounds of FP64
// residual (residual(x, r64)), per-instance norms (batch_norms), and a fused inner TFQMR in
// the number type T on rhs / ||rhs||, until every norm is <= o.crit.
template <typename T>
void mixed_rounds(heom_ctx *c, const heom_solve_opts &o, double2 *x, int nbatch, int64_t vstride, const double2 *rhs,
                  const DevCoef<double> &K64, const DevCoef<T> &KT, double2 *r64, std::vector<double> &norms,
                  int nlim, int max_rounds, bool stall_exit, bool &stalled,
                  int &total_iters, int &last_ierr, bool &converged, int &rounds, int64_t &launches, int64_t &aux,
                  const std::function<void(const double2 *, double2 *)> &residual,
                  const std::function<void(const double2 *)> &batch_norms,
                  const DevPlan &PV, int64_t N);
// ||H||_inf of the context's Hamiltonian (the scale of the inner preconditioner)
double hs_inf_norm(heom_ctx *c);
// The reference's shadow-vector stream (tfqmr_double/drandn.f90, SEED = 1): n reals.
void drandn_host(int64_t n, std::vector<double> &out);
}  // namespace heom

struct heom_ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    int norbs = 0, nspin = 0, nalf = 0, ncor = 0, nrho = 0, ntier = 0;
    int64_t lunk = 0, nunk = 0;
    heom::HStructure hst;
    heom::HostPlan fwd, adj;
    heom::PlanDev dfwd, dadj;
    bool has_adj = false;
    // parameter sets: H structure values (nh) in both precisions
    double2 *hval64 = nullptr;
    float2 *hval32 = nullptr;
    float4 *hvaldf = nullptr;
    double *es64 = nullptr;   // 4 lead-shift slots
    int h_real = 0;
    double eleadinfty[4] = {0, 0, 0, 0};
    double amps[4] = {0, 0, 0, 0}, tchar[4] = {0, 0, 0, 0};
    std::vector<heom::cd> hs_host;
    std::vector<std::vector<heom::cd>> dhs_host;   // optional parameter derivatives of hs
    // host copies for observables
    std::vector<heom::CurrentTerm> cur_terms;
    std::vector<int32_t> occ_entry, occ_slot;       // RDO diagonal entries contributing to occ(m,s)
    std::vector<int32_t> rdo_rows, rdo_cols;        // RDO pattern (1-based)
    int32_t *d_rdo_pair = nullptr;                  // transposed RDO entry (device)
    int32_t *d_rdo_upper = nullptr;                 // 1 for entries above the diagonal (device)
    int32_t nz0 = 0, ndiag = 0;
    double reg_scale = 1.0;                         // weight of the regularising blocks
    double cheby_delta = 0.0;                       // spectral width of the Liouville diagonal
    uint16_t *d_ent_rc = nullptr;                   // 0-based (row | col << 8) of every stored entry
    double cb_abs_max = 0.0;                        // largest |cb| (the Jacobi shift rule)
    heom::CurrentTerm *d_cur_terms = nullptr;
    int32_t n_cur_terms = 0;
    // scratch vectors (lunk + 1 complex)
    double2 *dx = nullptr, *dy = nullptr, *dz = nullptr;
    float2 *fx = nullptr, *fy = nullptr;
    double *dscratch = nullptr;
    std::vector<double> rt_host;                    // drandn stream (2*(lunk+1) reals)
    // first stored entry of every tier (1-based tier k at index k-1; lunk at index ntier):
    // the tables are tier-major, so a hierarchy truncated at tier k is the prefix up to
    // tier_entry[k]
    std::vector<int64_t> tier_entry;
    // automatic layout of the FP32x2 inner kernels of the mixed batch solves, per batch size
    // and kind (whole hierarchies 0, truncated 1): the candidate layouts (interleave,
    // instances per lane) and the device seconds of one solve with each, timed on the
    // context's first solves of that size and kind; then the fastest is kept
    struct LayoutTune {
        std::vector<std::pair<int, int>> cand;
        std::vector<double> seconds;   // of the candidates timed so far, in order
        bool done() const { return seconds.size() >= cand.size(); }
        std::pair<int, int> best() const
        {
            size_t k = 0;
            for (size_t i = 1; i < seconds.size(); i++)
                if (seconds[i] < seconds[k]) k = i;
            return cand[k];
        }
    };
    std::map<std::pair<int, int>, LayoutTune> il_tune;
    ~heom_ctx();
};
