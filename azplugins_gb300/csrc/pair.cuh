// pair.cuh -- pair-force kernels over the column-major full neighbour list.
//
// Loop semantics follow HOOMD's PotentialPair as observed by the reference tests
// (src/pytest/test_pair.py:351-363): for every listed j with rsq < r_cut^2 the
// evaluator gives force/r and energy; F_i += dx f/r, U_i += U/2,
// W_i += dx (x) dx f/(2r) with components xx, xy, xz, yy, yz, zz
// (src/ImagePotentialBondGPU.cuh:228-234). Modes none / shift / xplor.
#pragma once

#include "common.cuh"
#include "evaluators.cuh"

namespace azp
{
constexpr uint32_t MAX_PAIR_TYPES = 16;

// Per type pair table in global memory: PAIR_REC + CUT_REC doubles each.
constexpr int PAIR_TBL = PAIR_REC + CUT_REC;

struct PairArgs {
    const double4_32a* pos;    // FP64 positions (always, for the exact cutoff decision)
    const uint4* fixed;    // FP32 mode: fixed-point shadow
    uint32_t N;
    uint32_t ntypes;
    double L[3], Linv[3];
    float sfix[3];
    const uint32_t* counts;
    const uint32_t* nbrs;
    uint32_t max_nn;       // rows allocated: reads stop there even if a count overflowed
    const double* table;   // [ntypes^2][PAIR_TBL]
    void* force;           // double4_32a / float4 [N]
    void* virial;          // [6][pitch] or null
    uint32_t pitch;
};

// host: fill table for one evaluator kind from reference param records
int build_pair_table(int kind, const double* params, const double* r_cut, const double* r_on, int mode,
                     uint32_t ntypes, double* table_out);
// device: the same table from device params / r_cut / r_on (r_on may be null)
int launch_pair_table(int kind, const double* params, const double* r_cut, const double* r_on, int mode,
                      uint32_t ntypes, double* table_out, cudaStream_t s);

// launch the kernel for (kind, precision, tpp)
int launch_pair(int kind, int precision, int tpp, const PairArgs& a, cudaStream_t s);

}  // namespace azp
