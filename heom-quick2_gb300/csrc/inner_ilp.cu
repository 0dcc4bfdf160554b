// The fused inner kernels in FP32x2 with two instances per lane: a group of G instances on
// G / 2 lanes per entry, each lane serving two adjacent positions, so that the plan's
// records, map words and coefficients are decoded once for two instances.  With G = 2 a
// block covers the same 256 entries of each instance as the plain layout and sums them in
// the same order, so the iterates are those of one instance per group.
#include "inner_kernels.cuh"

namespace heom {
namespace inner_detail {

#define HEOM_PAIR_G(CALL)                                                      \
    switch (F.G) {                                                             \
    case 2: { constexpr int GE = 1; CALL; } break;                             \
    case 4: { constexpr int GE = 2; CALL; } break;                             \
    case 8: { constexpr int GE = 4; CALL; } break;                             \
    case 16: { constexpr int GE = 8; CALL; } break;                            \
    case 32: { constexpr int GE = 16; CALL; } break;                           \
    default: fail(HEOM_E_ARG, "inner workspace: unsupported interleave");      \
    }

void df_init_pair(const InnerWork<DF> &F, cudaStream_t s)
{
    dim3 g((unsigned)F.nblk, (unsigned)F.ngroups);
    HEOM_PAIR_G((k_in_init<DF, GE, false, 2><<<g, NT, 0, s>>>(F)))
}

void df_chunk_pair(InnerWork<DF> &F, const DevPlan &Q, const DevCoef<DF> &C, int iters, cudaStream_t s)
{
    HEOM_PAIR_G((chunk_ge<DF, GE, false, 2>(F, Q, C, iters, s)))
}

void df_time_pair(InnerWork<DF> &F, const DevPlan &Q, const DevCoef<DF> &C, int reps, cudaStream_t s, float &ms_b, float &ms_a)
{
    HEOM_PAIR_G((time_ge<DF, GE, false, 2>(F, Q, C, reps, s, ms_b, ms_a)))
}

#undef HEOM_PAIR_G

}  // namespace inner_detail
}  // namespace heom
