// The fused inner kernels in FP32x2 with a group's running instances compacted onto GE < G
// lanes per entry (the lane map of inner_lanes; the element stride G is read at run time).
#include "inner_kernels.cuh"

namespace heom {
namespace inner_detail {

void df_chunk_compact(InnerWork<DF> &W, const DevPlan &Q, const DevCoef<DF> &C, int iters, cudaStream_t s)
{
    switch (W.GE) {
    case 1: chunk_ge<DF, 1, true, 1>(W, Q, C, iters, s); break;
    case 2: chunk_ge<DF, 2, true, 1>(W, Q, C, iters, s); break;
    case 4: chunk_ge<DF, 4, true, 1>(W, Q, C, iters, s); break;
    case 8: chunk_ge<DF, 8, true, 1>(W, Q, C, iters, s); break;
    case 16: chunk_ge<DF, 16, true, 1>(W, Q, C, iters, s); break;
    default: fail(HEOM_E_ARG, "inner workspace: unsupported lanes per entry");
    }
}

}  // namespace inner_detail
}  // namespace heom
