// bond.cuh -- bond-force kernel arguments and launcher.
#pragma once

#include "common.cuh"

namespace azp
{
struct BondArgs {
    const double4_32a* pos;
    const uint4* fixed;      // FP32 mode
    uint32_t N;
    uint32_t nbondtypes;
    double L[3], Linv[3];
    float sfix[3];
    const uint32_t* n_bonds; // [N]
    const uint2* table;      // [height][N] (partner index, bond type)
    const double* params;    // [nbondtypes] reference param records (Eval::REC_DOUBLES each)
    void* force;             // accumulated: double4_32a / float4 [N]
    void* virial;            // accumulated: [6][pitch] or null
    uint32_t pitch;
    uint32_t* err;           // AZP_EBIT_BOND on refusal, may be null
    const int* image;        // [N][3]: image-unwrapped displacements, else null (minimum image)
};

int launch_bond(int kind, int precision, const BondArgs& a, cudaStream_t s);

}  // namespace azp
