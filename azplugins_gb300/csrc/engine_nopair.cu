// engine_nopair.cu -- fused step kernels of the resident engine for pair evaluator
// NoPair (one translation unit per evaluator so the instantiations compile in parallel).
#include "engine_kernels.cuh"

namespace azp
{
int launch_md_nopair(int bond_kind, int precision, int integ, const MDArgs& a, cudaStream_t s)
{
    return launch_md_pe<NoPair>(bond_kind, precision, integ, a, s);
}
}  // namespace azp
