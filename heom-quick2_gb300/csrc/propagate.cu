// Time propagation and sensitivities (filled in below).
#include "context.cuh"

extern "C" {
int heom_propagate(heom_ctx *, int32_t, double, double, int32_t, double _Complex *, double *) { heom::set_error("not built yet"); return HEOM_E_UNSUPPORTED; }
int heom_steady_gradient(heom_ctx *, const heom_grad_opts *, const double _Complex *, int32_t, double *, heom_solve_info *) { heom::set_error("not built yet"); return HEOM_E_UNSUPPORTED; }
int heom_td_gradient(heom_ctx *, double, int32_t, int32_t, const double _Complex *, double *, double *) { heom::set_error("not built yet"); return HEOM_E_UNSUPPORTED; }
}
