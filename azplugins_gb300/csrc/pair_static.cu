// pair_static.cu -- azp_pair_forces_static: the pair-force driver for callers
// that cannot allocate device memory.
//
// azp_pair_forces keeps its scratch (the derived type-pair table and the FP32
// fixed-point position shadow) in an azp_nlist workspace that azp_nlist_create
// allocates. Some host programs cannot hand out such a workspace: a simulation
// code that reserves its whole device-memory budget at start-up and lets plugins
// touch only the buffers it owns, or a caller on a path where cudaMalloc's
// implicit device synchronisation is not acceptable. For them this variant keeps
// the same scratch in one fixed array of this library (g_pair_scratch below),
// sized for at most AZP_STATIC_MAX_N particles and MAX_PAIR_TYPES types. Every
// GPU that loads the library holds that array until the process exits.
//
// The caller passes the neighbour list as plain device arrays (counts[N],
// column-major neighbors[k * N + i]), the parameter tables and the outputs, as
// for azp_pair_forces. The kernels are the ones azp_pair_forces launches, with
// the same threads per particle, so the results are identical.
#include <string>

#include "celllist.cuh"
#include "pair.cuh"

namespace azp
{
namespace
{
// threads per particle: the default of azp_pair_forces (azp_nlist::tpp)
constexpr int kStaticTpp = 4;
constexpr size_t kTableBytes = (size_t)MAX_PAIR_TYPES * MAX_PAIR_TYPES * PAIR_TBL * sizeof(double);
constexpr size_t kFixedOffset = (kTableBytes + 255) & ~(size_t)255;
constexpr size_t kScratchBytes = kFixedOffset + (size_t)AZP_STATIC_MAX_N * sizeof(uint4);

bool box_valid(const azp_box& b)
{
    for (int d = 0; d < 3; ++d)
        if (!(b.L[d] > 0.0) || !(b.L[d] < 1e300)) return false;
    return true;
}
}  // namespace

// [0, kFixedOffset): type-pair table, [kFixedOffset, ...): uint4 shadow [N].
// Shared by every call in the process on a given device.
static __device__ __align__(256) unsigned char g_pair_scratch[kScratchBytes];

// Device address of g_pair_scratch on the current device, looked up on every
// call with the caller's device current. The host symbol g_pair_scratch itself is
// not a device address and is never passed on. The lookup enqueues no work; no
// address is kept between calls, so a context torn down and created again
// (cudaDeviceReset) gets the array's new address on its next call.
static int scratch_address(unsigned char** out)
{
    void* p = nullptr;
    AZP_CUDA_TRY(cudaGetSymbolAddress(&p, g_pair_scratch));
    if (!p) return record_error(AZP_ERR_CUDA, "azp_pair_forces_static: cudaGetSymbolAddress returned NULL");
    *out = static_cast<unsigned char*>(p);
    return AZP_OK;
}

}  // namespace azp

extern "C" int azp_pair_forces_static(const azp_system* sys, const uint32_t* counts, const uint32_t* neighbors,
                                      uint32_t max_neighbors, int kind, const double* params, const double* r_cut,
                                      const double* r_on, int shift_mode, const azp_forces* out, void* stream)
{
    using namespace azp;
    if (!sys || !params || !r_cut || !out || !out->force) return AZP_ERR_INVALID;
    if (!box_valid(sys->box) || sys->ntypes == 0 || sys->ntypes > MAX_PAIR_TYPES) return AZP_ERR_INVALID;
    if (out->precision != AZP_FP64 && out->precision != AZP_FP32) return AZP_ERR_INVALID;
    if (sys->N > AZP_STATIC_MAX_N) {
        const std::string msg = "azp_pair_forces_static: N = " + std::to_string(sys->N) +
                                " exceeds the static scratch limit of " + std::to_string(AZP_STATIC_MAX_N) +
                                " particles (use azp_pair_forces with an azp_nlist workspace)";
        return record_error(AZP_ERR_TOO_LARGE, msg.c_str());
    }
    if (sys->N == 0) return AZP_OK;
    if (!sys->pos || !counts || (max_neighbors > 0 && !neighbors)) return AZP_ERR_INVALID;
    unsigned char* base = nullptr;
    int st = scratch_address(&base);
    if (st) return st;
    double* table = reinterpret_cast<double*>(base);
    uint4* fixed = reinterpret_cast<uint4*>(base + kFixedOffset);
    cudaStream_t s = as_stream(stream);
    // both scratch regions are fully rewritten before they are read: the table
    // for all ntypes^2 pairs, the shadow for all N particles (FP32 only)
    st = launch_pair_table(kind, params, r_cut, r_on, shift_mode, sys->ntypes, table, s);
    if (st) return st;
    if (out->precision == AZP_FP32)
        launch_to_fixed(reinterpret_cast<const double4_32a*>(sys->pos), fixed, sys->N, sys->box, s);
    PairArgs a;
    a.pos = reinterpret_cast<const double4_32a*>(sys->pos);
    a.fixed = fixed;
    a.N = sys->N;
    a.ntypes = sys->ntypes;
    for (int d = 0; d < 3; ++d) {
        a.L[d] = sys->box.L[d];
        a.Linv[d] = 1.0 / sys->box.L[d];
        a.sfix[d] = (float)(sys->box.L[d] * 2.3283064365386963e-10);
    }
    a.counts = counts;
    a.nbrs = neighbors;
    a.max_nn = max_neighbors;
    a.table = table;
    a.force = out->force;
    a.virial = out->virial;
    a.pitch = out->virial_pitch ? out->virial_pitch : sys->N;
    return launch_pair(kind, out->precision, kStaticTpp, a, s);
}
