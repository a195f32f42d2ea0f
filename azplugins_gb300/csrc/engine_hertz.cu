// engine_hertz.cu -- fused step kernels of the resident engine for pair evaluator
// Hertz (one translation unit per evaluator so the instantiations compile in parallel).
#include "engine_kernels.cuh"

namespace azp
{
int launch_md_hertz(int bond_kind, int precision, int integ, const MDArgs& a, cudaStream_t s)
{
    return launch_md_pe<Hertz>(bond_kind, precision, integ, a, s);
}
}  // namespace azp
