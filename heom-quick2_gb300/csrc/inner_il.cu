// The fused inner kernels in FP32x2 with G > 1 instances per group, every position served:
// the stride of an instance's elements (G) is known at compile time.
#include "inner_kernels.cuh"

namespace heom {
namespace inner_detail {

#define HEOM_FULL_G(CALL)                                                     \
    switch (F.G) {                                                            \
    case 2: { constexpr int G = 2; CALL; } break;                             \
    case 4: { constexpr int G = 4; CALL; } break;                             \
    case 8: { constexpr int G = 8; CALL; } break;                             \
    case 16: { constexpr int G = 16; CALL; } break;                           \
    case 32: { constexpr int G = 32; CALL; } break;                           \
    default: fail(HEOM_E_ARG, "inner workspace: unsupported interleave");     \
    }

void df_init_full(const InnerWork<DF> &F, cudaStream_t s)
{
    dim3 g((unsigned)F.nblk, (unsigned)F.ngroups);
    HEOM_FULL_G((k_in_init<DF, G, false, 1><<<g, NT, 0, s>>>(F)))
}

void df_chunk_full(InnerWork<DF> &F, const DevPlan &Q, const DevCoef<DF> &C, int iters, cudaStream_t s)
{
    HEOM_FULL_G((chunk_ge<DF, G, false, 1>(F, Q, C, iters, s)))
}

void df_time_full(InnerWork<DF> &F, const DevPlan &Q, const DevCoef<DF> &C, int reps, cudaStream_t s, float &ms_b, float &ms_a)
{
    HEOM_FULL_G((time_ge<DF, G, false, 1>(F, Q, C, reps, s, ms_b, ms_a)))
}

#undef HEOM_FULL_G

}  // namespace inner_detail
}  // namespace heom
