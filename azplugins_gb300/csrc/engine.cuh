// engine.cuh -- device side of the resident MD engine (azp_md).
#pragma once

#include "common.cuh"
#include "fixed64.cuh"
#include "integrate.cuh"
#include "walls.cuh"

namespace azp
{
// sizes of the FP32 records carried in MDArgs (PAIR_TBL and BOND_F of
// evaluators.cuh / pair.cuh; checked there)
constexpr int MD_PAIR_TBL = 12;
constexpr int MD_BOND_F = 12;

struct MDArgs {
    const double4_32a* pos;     // current positions
    double4_32a* pos_next;      // written when integrating
    const uint4* fix;           // fixed-point shadow of pos
    uint4* fix_next;
    const uint4* fix_build;     // shadow at the last list build
    double4_32a* vel;
    double* accel;              // [N][3]
    int* image;                 // [N][3]
    const uint32_t* tag;
    const double* diameter;
    uint32_t N, ntypes;
    double L[3], Linv[3], lo[3], hi[3];
    double fscale[3];           // 2^32 / L
    float sfix[3];
    // pair
    const uint32_t* counts;
    const uint32_t* nbrs;
    uint32_t max_nn;            // rows allocated: reads stop there even if a count overflowed
    const double* pair_table;   // [ntypes^2][12]
    // bonds (index order)
    const uint32_t* bt_n;
    const uint2* bt;
    const double* bond_params;
    uint32_t nbondtypes;
    // integrator
    double dt, kT;
    const unsigned long long* d_timestep;
    uint32_t seed;
    int noiseless;
    const double* gamma;
    const double* noise;        // per type sqrt(6 gamma kT / dt), 0 when noiseless
    int use_lambda;
    double lambda;
    FlowD flow;
    double max_disp;
    double fcap;                // > 0: per-pair force magnitude cap
    float disp_thresh2;         // (r_buff / 2)^2, slightly reduced
    uint32_t* flags;            // [0] rebuild request, [1] error bits, [2] builds, [4] ticket
    unsigned long long* d_timestep_rw;
    // outputs (M_OUT / M_FORCES)
    double4_32a* out_force;     // fx, fy, fz, energy
    double* out_virial;         // [6][N]
    // graph conditional of the next rebuild (set_cond == 0: none)
    cudaGraphConditionalHandle next_cond;
    int set_cond;
    int next;                   // Langevin: also do step one of the next timestep
    int out;                    // write out_force / out_virial
    int tpp;                    // threads per particle (1, 2, 4, 8, 16, 32)
    int tpp_shift;              // log2(tpp)
    // FP32-force state (fixed64.cuh): fix holds the high words, these the rest
    const uint4* flo;           // low words of the 64-bit fixed positions (x, y, z)
    uint4* flo_next;
    VelFF* velf;                // float-float velocities and 1/m (in the vel buffer)
    float s64h[3], s64l[3];     // 2^32 / L as a float pair
    int cubic;                  // Lx == Ly == Lz: r^2 from the exact integer displacement (fx_rsq)
    float s2h, s2l;             // (L / 2^32)^2 as a float pair (cubic boxes)
    // cubic boxes, per type pair in the units of the integer r^2, c^2 2^64 / L^2:
    // the colloid gap forms' contact distance (0: no gap form), the DPD cutoff
    const long long* contact_q;
    double l64[3];              // L * 2^-64 (exact cutoff decisions near r_cut)
    float dtf, kTf, lambdaf, fcapf, max_dispf;
    FlowF flowf;
    // single-type systems (one particle type, at most one bond type): the FP32
    // records of type pair 0 and bond type 0, r_cut^2 and the drag / noise of
    // type 0 as kernel arguments, read from the constant bank in the step
    int one_type;
    float rec0[MD_PAIR_TBL];
    float bond0[MD_BOND_F];
    double rc2_0;
    float gamma0, noise0;
    // harmonic barrier added to the net force (bar_geom -1: none). bar_tab holds
    // one record per (row, type): FP64 steps double2 (c = location + offset, k),
    // FP32 steps BarrierRecF; row r belongs to timestep bar_hdr[0] + r (clamped to
    // the bar_hdr[1] rows). A Langevin step at timestep t evaluates the forces of
    // the positions of t + 1, a Brownian step and a forces-only launch those of t.
    int bar_geom;
    const void* bar_tab;
    const unsigned long long* bar_hdr;
    // wall potential added to the net force (wall_kind -1: none); wall_tab per
    // type: record (4), r_cut^2, r_extrap, r_cut, - ; walls in device memory
    int wall_kind;
    const WallField* walls;
    const double* wall_tab;
    float wall_tol;             // FP32 screening margin (FP32-force step)
    // FP32-force step: each particle's wall force and energy, written by
    // k_walls_fx right before the step (an out-of-line wall call inside the step
    // would cost it a stack frame and spills even with the walls off)
    const float4* wall_f;
    // DPD: the velocities of the step's start (a snapshot taken right before the
    // step, so that neighbours are read while their owners update them):
    // double4 (v, mass) in FP64 steps, float4 (v, 1/m) in FP32-force steps
    const void* dvel;
    // ImageHarmonic bonds: the image counts of the step's start ([N][3], a
    // snapshot for the same reason: the step updates image[] in place)
    const int* img0;
    // integration group by type (bit t: type t moves); 0xffffffff: every particle
    uint32_t group_types;
    // temperature table (kT_hdr null: the constant kT and noise above): row r
    // holds timestep kT_hdr[0] + r, clamped to the kT_hdr[1] rows
    const unsigned long long* kT_hdr;
    const double* kT_tab;       // [rows] kT
    const double* noise_tab;    // [rows][ntypes] sqrt(6 gamma kT / dt), 0 when noiseless
    // shared-memory neighbour tiles (celllist.cuh): block records, or null when
    // the list holds plain particle indices
    const uint32_t* tile;
};

// does the method move particles of type t?
AZP_D bool in_group(const MDArgs& a, uint32_t t)
{
    return a.group_types == 0xffffffffu || (t < 32u && ((a.group_types >> t) & 1u));
}

// row of timestep ts in the temperature table
AZP_D size_t kT_row(const MDArgs& a, unsigned long long ts)
{
    const unsigned long long t0 = a.kT_hdr[0], rows = a.kT_hdr[1];
    return (size_t)(ts <= t0 ? 0ull : min(ts - t0, rows - 1ull));
}

constexpr int MD_INTEG_LANGEVIN = 0;
constexpr int MD_INTEG_BROWNIAN = 1;
constexpr int MD_FORCES_ONLY = 2;

// one launcher per pair evaluator (engine_<pair>.cu); pair_kind -1 = no pair force
int launch_md_step(int pair_kind, int bond_kind, int precision, int integ, const MDArgs& a, cudaStream_t s);

}  // namespace azp
