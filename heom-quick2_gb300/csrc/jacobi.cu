// Jacobi steady-state iteration on GB300 (jacobi/: prelude_jacobi, calc_ax_jacobi_spa_omp,
// solve_jacobi).
//
// One sweep maps x to x' with, for every ADO n (drawers summing to g_n),
//     x'_n = P_n (ejac - g_n + i L)^-1 (ejac x_n + C_n x),
// where C_n x are the couplings of n to the neighbouring tiers on the pattern P_n of n and
// L = [H, .] is the system Liouvillian; its fixed point solves A x = 0 with the trace kept.
// The reference diagonalises L in Liouville space (nrho^2 x nrho^2) and applies its
// eigenvectors by two matrix-vector products per ADO.  Here H = U diag(E) U^H is diagonalised
// once and (ejac - g + i L)^-1 Y = U [(U^H Y U)_ab / (ejac - g + i (E_a - E_b))] U^H: three
// products per ADO on one thread block, from shared memory, each summing only over the
// sector block of H its index lies in.  The couplings come from the steady apply:
// C_n x = (A x)_n - g_n x_n + i P_n [H, x_n].
#include <algorithm>
#include <cmath>
#include <complex>
#include <memory>

#include "context.cuh"

namespace heom {

namespace {

constexpr int kJacThreads = 256;
constexpr double kDpico = 1e-12;

__device__ __forceinline__ double2 cmul(double2 a, double2 b) { return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x); }
__device__ __forceinline__ double2 cmulc(double2 a, double2 b) { return make_double2(a.x * b.x + a.y * b.y, a.x * b.y - a.y * b.x); }  // conj(a) b
__device__ __forceinline__ double2 cadd(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }

// a persistent block walks the ADOs blockIdx.x, blockIdx.x + gridDim.x, ... of instance blockIdx.y
// States are renumbered so that the connected components of the graph of H (its conserved
// sectors) are contiguous: H, and with it U, are then block diagonal, and every product below
// runs over the block [lo(i), hi(i)) of the index it sums against.  perm maps a state to
// its new number; H, U, E arrive in the new numbering.
__global__ void __launch_bounds__(kJacThreads) k_jacobi(DevPlan P, const uint16_t *__restrict__ rc,
                                                       const double2 *__restrict__ x, const double2 *__restrict__ y,
                                                       double2 *__restrict__ xn, const double2 *__restrict__ gdiag,
                                                       const double2 *__restrict__ U, const double *__restrict__ E,
                                                       const double2 *__restrict__ H, const uint8_t *__restrict__ perm,
                                                       const uint8_t *__restrict__ blo, const uint8_t *__restrict__ bhi,
                                                       double ejac, int n, int64_t vstride)
{
    extern __shared__ double2 sm[];
    const int nn = n * n;
    double2 *sU = sm, *sH = sm + nn, *sX = sm + 2 * nn, *sY = sm + 3 * nn, *sT = sm + 4 * nn;
    double *sE = reinterpret_cast<double *>(sm + 5 * nn);
    uint8_t *sP = reinterpret_cast<uint8_t *>(sE + n), *sLo = sP + n, *sHi = sLo + n;
    const int b = blockIdx.y;
    x += (int64_t)b * vstride;
    y += (int64_t)b * vstride;
    xn += (int64_t)b * vstride;
    U += (int64_t)b * nn;
    H += (int64_t)b * nn;
    E += (int64_t)b * n;
    // the instance's H, U and E stay in shared memory while the block walks its ADOs
    for (int k = threadIdx.x; k < nn; k += blockDim.x) { sU[k] = U[k]; sH[k] = H[k]; }
    for (int k = threadIdx.x; k < n; k += blockDim.x) { sE[k] = E[k]; sP[k] = perm[k]; sLo[k] = blo[k]; sHi[k] = bhi[k]; }
    for (int a = blockIdx.x; a < P.nado; a += gridDim.x) {
    const int off = __ldg(P.ado_off + a), nz = __ldg(P.ado_off + a + 1) - off;
    for (int k = threadIdx.x; k < nn; k += blockDim.x) {
        sX[k] = make_double2(0, 0);
        sY[k] = make_double2(0, 0);
    }
    __syncthreads();
    for (int q = threadIdx.x; q < nz; q += blockDim.x) {
        const unsigned w = rc[off + q];
        sX[sP[w & 0xFF] + sP[w >> 8] * n] = x[off + q];
    }
    __syncthreads();
    const double2 g = gdiag[(int64_t)b * P.nado + a];
    const double2 d = make_double2(ejac - g.x, -g.y);
    // Y = ejac x + C x = (ejac - g) x + A x + i P[H, x] on the pattern
    for (int q = threadIdx.x; q < nz; q += blockDim.x) {
        const unsigned w = rc[off + q];
        const int r = sP[w & 0xFF], c = sP[w >> 8];
        double2 comm = make_double2(0, 0);
        for (int k = sLo[r]; k < sHi[r]; k++) comm = cadd(comm, cmul(sH[r + k * n], sX[k + c * n]));
        for (int k = sLo[c]; k < sHi[c]; k++) {
            const double2 xh = cmul(sX[r + k * n], sH[k + c * n]);
            comm = make_double2(comm.x - xh.x, comm.y - xh.y);
        }
        const double2 v = cadd(cadd(cmul(d, x[off + q]), y[off + q]), make_double2(-comm.y, comm.x));
        sY[r + c * n] = v;
    }
    __syncthreads();
    // T = U^H Y
    for (int k = threadIdx.x; k < nn; k += blockDim.x) {
        const int i = k % n, j = k / n;
        double2 s = make_double2(0, 0);
        for (int l = sLo[i]; l < sHi[i]; l++) s = cadd(s, cmulc(sU[l + i * n], sY[l + j * n]));
        sT[k] = s;
    }
    __syncthreads();
    // W = (T U) / (ejac - g + i (E_i - E_j)), into Y
    const bool dsmall = sqrt(d.x * d.x + d.y * d.y) <= kDpico;
    for (int k = threadIdx.x; k < nn; k += blockDim.x) {
        const int i = k % n, j = k / n;
        double2 s = make_double2(0, 0);
        for (int l = sLo[j]; l < sHi[j]; l++) s = cadd(s, cmul(sT[i + l * n], sU[l + j * n]));
        const double lam = sE[i] - sE[j];
        double2 den = make_double2(d.x, d.y + lam);
        if (dsmall) den = make_double2(0.0, lam);
        double2 f = make_double2(0, 0);
        if (!dsmall || fabs(lam) > kDpico) {
            const double inv = 1.0 / (den.x * den.x + den.y * den.y);
            f = make_double2(den.x * inv, -den.y * inv);
        }
        sY[k] = cmul(s, f);
    }
    __syncthreads();
    // T = U W
    for (int k = threadIdx.x; k < nn; k += blockDim.x) {
        const int i = k % n, j = k / n;
        double2 s = make_double2(0, 0);
        for (int l = sLo[i]; l < sHi[i]; l++) s = cadd(s, cmul(sU[i + l * n], sY[l + j * n]));
        sT[k] = s;
    }
    __syncthreads();
    // x'(r, c) = (T U^H)(r, c) on the pattern
    for (int q = threadIdx.x; q < nz; q += blockDim.x) {
        const unsigned w = rc[off + q];
        const int r = sP[w & 0xFF], c = sP[w >> 8];
        double2 s = make_double2(0, 0);
        for (int l = sLo[c]; l < sHi[c]; l++) {
            const double2 u = sU[c + l * n];
            s = cadd(s, cmul(sT[r + l * n], make_double2(u.x, -u.y)));
        }
        xn[off + q] = s;
    }
    __syncthreads();   // the next ADO clears sX and sY
    }
}

// Hermitian eigen-decomposition by cyclic Jacobi rotations (a phase on column q makes a_pq
// real, then a real plane rotation removes it): a (column-major) is destroyed, v receives
// the eigenvectors as columns.
void herm_eig(int n, std::vector<cd> &a, std::vector<double> &w, std::vector<cd> &v)
{
    v.assign((size_t)n * n, cd(0, 0));
    for (int i = 0; i < n; i++) v[i + (size_t)i * n] = 1.0;
    auto A = [&](int i, int j) -> cd & { return a[i + (size_t)j * n]; };
    for (int sweep = 0; sweep < 100; sweep++) {
        double off = 0, tot = 0;
        for (int j = 0; j < n; j++)
            for (int i = 0; i < n; i++) { double t = std::norm(A(i, j)); tot += t; if (i != j) off += t; }
        if (off <= 1e-30 * std::max(tot, 1e-300)) break;
        for (int p = 0; p < n; p++)
            for (int q = p + 1; q < n; q++) {
                const double r = std::abs(A(p, q));
                if (r < 1e-300) continue;
                const cd ph = A(p, q) / r;
                for (int k = 0; k < n; k++) { A(k, q) *= std::conj(ph); v[k + (size_t)q * n] *= std::conj(ph); }
                for (int k = 0; k < n; k++) A(q, k) *= ph;
                const double th = (A(q, q).real() - A(p, p).real()) / (2 * r);
                const double t = (th >= 0 ? 1.0 : -1.0) / (std::fabs(th) + std::sqrt(th * th + 1));
                const double c = 1 / std::sqrt(t * t + 1), s = t * c;
                for (int k = 0; k < n; k++) { cd x = A(k, p), y = A(k, q); A(k, p) = c * x - s * y; A(k, q) = s * x + c * y; }
                for (int k = 0; k < n; k++) { cd x = A(p, k), y = A(q, k); A(p, k) = c * x - s * y; A(q, k) = s * x + c * y; }
                for (int k = 0; k < n; k++) {
                    cd x = v[k + (size_t)p * n], y = v[k + (size_t)q * n];
                    v[k + (size_t)p * n] = c * x - s * y; v[k + (size_t)q * n] = s * x + c * y;
                }
            }
    }
    w.resize(n);
    for (int i = 0; i < n; i++) w[i] = A(i, i).real();
}

}  // namespace
}  // namespace heom

using namespace heom;

extern "C" {

int heom_jacobi_shift(heom_ctx *c, double *ejac)
{
    return guarded([&] {
        require_ctx(c);
        DeviceScope dsc(c->device);
        if (!ejac) fail(HEOM_E_ARG, "null argument");
        std::vector<cd> a = c->hs_host, v;
        std::vector<double> e;
        herm_eig(c->nrho, a, e, v);
        const double lo = *std::min_element(e.begin(), e.end()), hi = *std::max_element(e.begin(), e.end());
        // the nonzero eigenvalues of L = [H, .] are the differences E_a - E_b; their span
        const double gap = hi - lo > kDpico ? 2 * (hi - lo) : 0.0;
        *ejac = std::max(gap, std::sqrt((double)(c->ntier - 1) * c->cb_abs_max));
    });
}

}  // extern "C"

namespace {

// The solve, or with bench_reps > 0 a measurement of its two kernels instead:
// bench[0..1] = seconds per launch of the sector transform and of the apply,
// bench[2..3] = the transform's algorithmic bytes and complex multiply-adds per launch.
void jacobi_run(heom_ctx *c, const heom_solve_opts *o, double ejac, double _Complex *rho, heom_solve_info *info,
                int bench_reps, double *bench)
{
    {
        if (!o || !rho) fail(HEOM_E_ARG, "null argument");
        const int n = c->nrho, nn = n * n;
        if (n > 32) fail(HEOM_E_UNSUPPORTED, "the Jacobi sweep keeps five nrho x nrho matrices in shared memory: nrho <= 32");
        if (!c->d_ent_rc) fail(HEOM_E_UNSUPPORTED, "entry coordinates missing");
        if (ejac <= 0) heom_jacobi_shift(c, &ejac);
        if (info) *info = heom_solve_info{};
        const int64_t N = c->lunk + 1;
        std::vector<cd> h(reinterpret_cast<cd *>(rho), reinterpret_cast<cd *>(rho) + c->lunk);
        herm_rdo(c, h.data());
        // sectors: connected components of the graph of H, numbered contiguously
        std::vector<int> comp(n, -1), order;
        for (int s0 = 0, nc = 0; s0 < n; s0++) {
            if (comp[s0] >= 0) continue;
            std::vector<int> stack{s0};
            comp[s0] = nc;
            while (!stack.empty()) {
                const int i = stack.back();
                stack.pop_back();
                for (int j = 0; j < n; j++)
                    if (comp[j] < 0 && (std::abs(c->hs_host[i + (size_t)j * n]) >= kDsmall || std::abs(c->hs_host[j + (size_t)i * n]) >= kDsmall)) {
                        comp[j] = nc;
                        stack.push_back(j);
                    }
            }
            nc++;
        }
        for (int cc = 0; cc < n; cc++)
            for (int i = 0; i < n; i++) if (comp[i] == cc) order.push_back(i);   // new number -> state
        std::vector<uint8_t> perm(n), blo(n), bhi(n);
        for (int k = 0; k < n; k++) perm[order[k]] = (uint8_t)k;
        for (int k = 0; k < n; k++) {
            int lo = k, hi = k + 1;
            while (lo > 0 && comp[order[lo - 1]] == comp[order[k]]) lo--;
            while (hi < n && comp[order[hi]] == comp[order[k]]) hi++;
            blo[k] = (uint8_t)lo; bhi[k] = (uint8_t)hi;
        }
        std::vector<cd> hp((size_t)nn);
        for (int j = 0; j < n; j++)
            for (int i = 0; i < n; i++) hp[i + (size_t)j * n] = c->hs_host[order[i] + (size_t)order[j] * n];
        std::vector<cd> a = hp, v;
        std::vector<double> e;
        herm_eig(n, a, e, v);
        std::vector<void *> tmp;
        auto cleanup = [&] { for (void *p : tmp) cudaFree(p); tmp.clear(); };
        cudaEvent_t e0 = nullptr, e1 = nullptr;
        try {
            double2 *x = nullptr, *xn = nullptr, *y = nullptr, *gd = nullptr, *dU = nullptr, *dH = nullptr;
            double *dE = nullptr;
            CK(cudaMalloc((void **)&x, sizeof(double2) * N)); tmp.push_back(x);
            CK(cudaMalloc((void **)&xn, sizeof(double2) * N)); tmp.push_back(xn);
            CK(cudaMalloc((void **)&y, sizeof(double2) * N)); tmp.push_back(y);
            const DevPlan &P = c->dfwd.view;
            CK(cudaMalloc((void **)&gd, sizeof(double2) * std::max(1, P.nado))); tmp.push_back(gd);
            CK(cudaMalloc((void **)&dU, sizeof(double2) * nn)); tmp.push_back(dU);
            CK(cudaMalloc((void **)&dH, sizeof(double2) * nn)); tmp.push_back(dH);
            CK(cudaMalloc((void **)&dE, sizeof(double) * n)); tmp.push_back(dE);
            uint8_t *dperm = nullptr;
            CK(cudaMalloc((void **)&dperm, 3 * (size_t)n)); tmp.push_back(dperm);
            std::vector<uint8_t> pb(perm);
            pb.insert(pb.end(), blo.begin(), blo.end());
            pb.insert(pb.end(), bhi.begin(), bhi.end());
            CK(cudaMemcpyAsync(dperm, pb.data(), 3 * (size_t)n, cudaMemcpyHostToDevice, c->stream));
            CK(cudaMemsetAsync(x, 0, sizeof(double2) * N, c->stream));
            CK(cudaMemsetAsync(xn, 0, sizeof(double2) * N, c->stream));
            CK(cudaMemcpyAsync(x, h.data(), sizeof(double2) * c->lunk, cudaMemcpyHostToDevice, c->stream));
            CK(cudaMemcpyAsync(dU, v.data(), sizeof(double2) * nn, cudaMemcpyHostToDevice, c->stream));
            CK(cudaMemcpyAsync(dH, hp.data(), sizeof(double2) * nn, cudaMemcpyHostToDevice, c->stream));
            CK(cudaMemcpyAsync(dE, e.data(), sizeof(double) * n, cudaMemcpyHostToDevice, c->stream));
            CK(cudaStreamSynchronize(c->stream));
            DevCoef<double> K = ctx_coefs(c).k64;
            fill_gdiag<double>(P, K, gd, 1, c->stream);
            K.gdiag = gd;
            const size_t smem = sizeof(double2) * 5 * nn + sizeof(double) * n + 3 * (size_t)n;
            if (smem > 48 * 1024)
                CK(cudaFuncSetAttribute(k_jacobi, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
            // a persistent grid: as many resident blocks as the SMs hold, each walking ADOs
            int nsm = 0, per_sm = 0;
            CK(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, c->device));
            CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_jacobi, kJacThreads, smem));
            const unsigned jgrid = (unsigned)std::max(1, std::min(P.nado, nsm * std::max(1, per_sm)));
            auto sweep = [&](double2 *from, double2 *to) {
                launch_apply<double, false>(P, K, from, y, 1, N, nullptr, c->stream);
                k_jacobi<<<dim3(jgrid, 1), kJacThreads, smem, c->stream>>>(P, c->d_ent_rc, from, y, to, gd, dU, dE,
                                                                                   dH, dperm, dperm + n, dperm + 2 * n,
                                                                                   ejac, n, N);
            };
            // ||A x - e_trace|| (solve_jacobi.f90:183-190)
            auto residual = [&](double2 *from) {
                launch_apply<double, false>(P, K, from, y, 1, N, nullptr, c->stream);
                std::vector<double2> last(1);
                CK(cudaMemcpyAsync(last.data(), y + c->lunk, sizeof(double2), cudaMemcpyDeviceToHost, c->stream));
                CK(cudaStreamSynchronize(c->stream));
                last[0].x -= 1.0;
                CK(cudaMemcpyAsync(y + c->lunk, last.data(), sizeof(double2), cudaMemcpyHostToDevice, c->stream));
                return device_norm2(N, y, c->dscratch, c->stream);
            };
            if (bench_reps > 0) {
                cudaEvent_t b0, b1, b2;
                CK(cudaEventCreate(&b0)); CK(cudaEventCreate(&b1)); CK(cudaEventCreate(&b2));
                sweep(x, xn);
                CK(cudaEventRecord(b0, c->stream));
                for (int r = 0; r < bench_reps; r++)
                    k_jacobi<<<dim3(jgrid, 1), kJacThreads, smem, c->stream>>>(P, c->d_ent_rc, x, y, xn, gd, dU, dE, dH, dperm,
                                                                                       dperm + n, dperm + 2 * n, ejac, n, N);
                CK(cudaEventRecord(b1, c->stream));
                for (int r = 0; r < bench_reps; r++) launch_apply<double, false>(P, K, x, y, 1, N, nullptr, c->stream);
                CK(cudaEventRecord(b2, c->stream));
                CK(cudaEventSynchronize(b2));
                CK(cudaGetLastError());
                float m1 = 0, m2 = 0;
                cudaEventElapsedTime(&m1, b0, b1);
                cudaEventElapsedTime(&m2, b1, b2);
                cudaEventDestroy(b0); cudaEventDestroy(b1); cudaEventDestroy(b2);
                // per ADO: x, A x read and x' written (16 B each per entry) plus the entry's
                // coordinates (2 B); the per-instance U, H, E and the ADO diagonal come from L2
                double s2 = 0;
                for (int k = 0; k < n; k++) s2 += bhi[k] - blo[k];
                bench[0] = m1 * 1e-3 / bench_reps;
                bench[1] = m2 * 1e-3 / bench_reps;
                bench[2] = (double)c->lunk * (3 * 16 + 2) + (double)P.nado * 16;
                // complex multiply-adds: three products over the blocks (n * sum_i |block(i)|
                // each) and, per stored entry, the commutator and the extraction
                double entries_blk = 0;
                {
                    std::vector<uint16_t> rcv((size_t)c->lunk);
                    CK(cudaMemcpy(rcv.data(), c->d_ent_rc, sizeof(uint16_t) * rcv.size(), cudaMemcpyDeviceToHost));
                    for (uint16_t w : rcv) {
                        const int r = perm[w & 0xFF], cc = perm[w >> 8];
                        entries_blk += (double)(bhi[r] - blo[r]) + 2.0 * (bhi[cc] - blo[cc]);
                    }
                }
                bench[3] = (double)P.nado * 3.0 * n * s2 + entries_blk;
                cleanup();
                return;
            }
            // sweeps 50 at a time in one graph: an even count leaves the iterate in x
            constexpr int kChunk = 50;
            cudaGraph_t g = nullptr;
            cudaGraphExec_t ge = nullptr;
            {
                const CapturedGraph cg = capture_graph(c->stream, [&] { for (int k = 0; k < kChunk; k += 2) { sweep(x, xn); sweep(xn, x); } });
                g = cg.graph;
                ge = cg.exec;
            }
            CK(cudaEventCreate(&e0)); CK(cudaEventCreate(&e1));
            CK(cudaEventRecord(e0, c->stream));
            // iteration 0, then chunks of 50; the residual test follows iterations 0, 50, 100, ...
            sweep(x, xn);
            CK(cudaMemcpyAsync(x, xn, sizeof(double2) * N, cudaMemcpyDeviceToDevice, c->stream));
            int iter = 0;
            double res = residual(x);
            int64_t launches = 3;
            while (res > o->crit && iter + kChunk <= std::max(0, o->maxit0)) {
                CK(cudaGraphLaunch(ge, c->stream));
                iter += kChunk;
                launches += 2 * kChunk + 1;
                res = residual(x);
            }
            CK(cudaEventRecord(e1, c->stream));
            CK(cudaEventSynchronize(e1));
            float ms = 0;
            cudaEventElapsedTime(&ms, e0, e1);
            cudaGraphExecDestroy(ge);
            cudaGraphDestroy(g);
            CK(cudaMemcpyAsync(rho, x, sizeof(double2) * c->lunk, cudaMemcpyDeviceToHost, c->stream));
            CK(cudaStreamSynchronize(c->stream));
            CK(cudaGetLastError());
            if (info) {
                info->iters = iter;
                info->resid = res;
                info->converged = res <= o->crit;
                info->ierr = info->converged ? 0 : 1;
                info->seconds = ms * 1e-3;
                info->launches = launches;
            }
        } catch (...) {
            if (e0) cudaEventDestroy(e0);
            if (e1) cudaEventDestroy(e1);
            cleanup();
            throw;
        }
        cudaEventDestroy(e0); cudaEventDestroy(e1);
        cleanup();
    }
}

}  // namespace

extern "C" {

int heom_solve_jacobi(heom_ctx *c, const heom_solve_opts *o, double ejac, double _Complex *rho, heom_solve_info *info)
{
    return guarded([&] {
        require_ctx(c);
        DeviceScope dsc(c->device);
        jacobi_run(c, o, ejac, rho, info, 0, nullptr);
    });
}

int heom_bench_jacobi(heom_ctx *c, double ejac, int32_t reps, double *out)
{
    return guarded([&] {
        require_ctx(c);
        DeviceScope dsc(c->device);
        if (!out || reps < 1) fail(HEOM_E_ARG, "null output or reps < 1");
        heom_solve_opts o{};
        o.crit = 1.0;
        std::vector<cd> rho((size_t)c->lunk, cd(0, 0));
        jacobi_run(c, &o, ejac, reinterpret_cast<double _Complex *>(rho.data()), nullptr, reps, out);
    });
}

}  // extern "C"
