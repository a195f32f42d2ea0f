// Prints sizeof(param_type) of the reference's pair, bond and wall evaluators as
// JSON, compiled in place from the azplugins source tree against the
// hoomd/HOOMDMath.h stand-in. Built twice by oracle/build_ref.sh: Scalar = double
// (HOOMD_LONGREAL_SIZE 64, the default HOOMD build) and, with AZP_REF_SINGLE,
// Scalar = float (HOOMD_LONGREAL_SIZE 32). The C ABI's record strides are pinned
// against these numbers (tests/golden/ref_vectors.json "record_bytes").
// Test infrastructure only.
#include <cstdio>

#include "BondEvaluatorDoubleWell.h"
#include "BondEvaluatorQuartic.h"
#include "DPDPairEvaluatorGeneralWeight.h"
#include "PairEvaluatorColloid.h"
#include "PairEvaluatorExpandedYukawa.h"
#include "PairEvaluatorHertz.h"
#include "PairEvaluatorPerturbedLennardJones.h"
#include "WallEvaluatorColloid.h"
#include "WallEvaluatorLJ93.h"

namespace azd = hoomd::azplugins::detail;

int main()
    {
    std::printf("{\"scalar_bytes\": %zu, \"pair\": {", sizeof(hoomd::Scalar));
    std::printf("\"PerturbedLennardJones\": %zu, ", sizeof(azd::PairParametersPerturbedLennardJones));
    std::printf("\"ExpandedYukawa\": %zu, ", sizeof(azd::PairParametersExpandedYukawa));
    std::printf("\"Hertz\": %zu, ", sizeof(azd::PairParametersHertz));
    std::printf("\"Colloid\": %zu, ", sizeof(azd::PairParametersColloid));
    std::printf("\"DPDGeneralWeight\": %zu}, ", sizeof(azd::PairParametersDPDGeneralWeight));
    std::printf("\"bond\": {\"Quartic\": %zu, ", sizeof(azd::BondParametersQuartic));
    std::printf("\"DoubleWell\": %zu}, ", sizeof(azd::BondParametersDoubleWell));
    std::printf("\"wall\": {\"LJ93\": %zu, ", sizeof(azd::WallParametersLJ93));
    std::printf("\"Colloid\": %zu}}\n", sizeof(azd::WallParametersColloid));
    return 0;
    }
