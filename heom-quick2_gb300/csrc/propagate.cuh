// Device time propagation: shared pieces of the forward steps and the reverse pass.
#pragma once
#include <vector>

#include "context.cuh"

namespace heom {

// Step counter and pulse parameters read by the device at every stage.
struct PropClock {
    int64_t n;          // step index (forward: 0, 1, ...; reverse: counts down)
    int64_t dir;        // +1 forward, -1 reverse
    double t0, dt;
    double amp_scale;   // bias amplitude scale A (eshift = A * amps * onset(t))
    double amps[4], tchar[4];
};

struct PropBuffers {
    int64_t N = 0;
    double dt = 0;
    void *mem = nullptr;
    std::vector<double2 *> vec;   // nvec FP64 vectors of lunk + 1 elements
    double *es = nullptr;         // 4 lead shifts of the current stage (+4 spare)
    double2 *gd = nullptr;        // ADO diagonals of the forward plan at the current stage
    double2 *gda = nullptr;       // ADO diagonals of the adjoint plan at the current stage
    PropClock *clk = nullptr;
    double *jt = nullptr;         // recorded currents
    PropBuffers(heom_ctx *c, int nvec, int64_t njt);
    ~PropBuffers();
    PropBuffers(const PropBuffers &) = delete;
    PropBuffers &operator=(const PropBuffers &) = delete;
};

// es = the lead shifts at the stage (frac of a step) and the matching ADO diagonals in B.gd
// (and B.gda for the adjoint plan when adj is set), so the stage's FP64 applies read g
// instead of summing the lead shifts per entry
void stage_prepare(heom_ctx *c, PropBuffers &B, double frac, bool adj, cudaStream_t s);

double bessel_j(int n, double x);
double cheby_width(heom_ctx *c);
int cheby_terms(double delta, double dt, double dpre);
void prop_clock_init(heom_ctx *c, PropClock &h, double t0, double dt, double amp_scale);
void enqueue_step(heom_ctx *c, int method, const DevCoef<double> &K, PropBuffers &B, double2 *rho, double delta,
                  const std::vector<double> &bes, bool record_current);
// One Chebyshev step in FP32x2: state rho, recurrence vectors v[0..2], the step's ADO
// diagonals written to gdf (HEOM_PROP_CHEBYSHEV_MIXED)
void enqueue_step_df(heom_ctx *c, const DevCoef<DF> &K, PropBuffers &B, float4 *rho, float4 *const v[3], float4 *gdf,
                     double delta, const std::vector<double> &bes, bool record_current);

}  // namespace heom
