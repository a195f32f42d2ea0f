// engine_dpd.cu -- fused step kernels of the resident engine for the DPD pair
// force with a general weight (src/DPDPairEvaluatorGeneralWeight.h:165-255).
#include "engine_kernels.cuh"

namespace azp
{
int launch_md_dpd(int bond_kind, int precision, int integ, const MDArgs& a, cudaStream_t s)
{
    // a DPD thermostat needs velocities: Langevin-type integration (the
    // noiseless, drag-free Langevin step is velocity Verlet) or forces alone
    if (integ == MD_INTEG_BROWNIAN) return AZP_ERR_UNSUPPORTED;
    return launch_md_pe<DpdEngine>(bond_kind, precision, integ, a, s);
}
}  // namespace azp
