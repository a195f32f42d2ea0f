// capi.cu -- extern "C" entry points of the standalone drivers: parameter
// builders (the param_type dict constructors / asDict), pair / bond force
// drivers and the integrator drivers. The resident engine lives in engine.cu.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "bond.cuh"
#include "celllist.cuh"
#include "integrate.cuh"
#include "nlist_impl.cuh"
#include "pair.cuh"

namespace azp
{
static thread_local std::string g_last_error;

int record_cuda_error(cudaError_t e, const char* what)
{
    g_last_error = std::string(what) + ": " + cudaGetErrorString(e);
    return AZP_ERR_CUDA;
}

int record_error(int status, const char* msg)
{
    g_last_error = msg;
    return status;
}

}  // namespace azp

namespace
{
int n_pair_values(int kind)
{
    switch (kind) {
    case AZP_PAIR_PERTURBED_LJ: return 3;
    case AZP_PAIR_EXPANDED_YUKAWA: return 3;
    case AZP_PAIR_HERTZ: return 1;
    case AZP_PAIR_COLLOID: return 4;
    case AZP_PAIR_DPD_GENERAL_WEIGHT: return 3;
    default: return -1;
    }
}

int n_bond_values(int kind)
{
    switch (kind) {
    case AZP_BOND_QUARTIC: return 8;
    case AZP_BOND_DOUBLE_WELL: return 4;
    case AZP_BOND_IMAGE_HARMONIC: return 2;
    default: return -1;
    }
}

void fill_box(const azp_box& b, double* L, double* Linv, float* sfix)
{
    for (int d = 0; d < 3; ++d) {
        L[d] = b.L[d];
        Linv[d] = 1.0 / b.L[d];
        sfix[d] = (float)(b.L[d] * 2.3283064365386963e-10);
    }
}

bool box_ok(const azp_box& b)
{
    for (int d = 0; d < 3; ++d)
        if (!(b.L[d] > 0.0) || !std::isfinite(b.L[d])) return false;
    return true;
}

}  // namespace

extern "C" {

int azp_abi_version(void) { return AZP_ABI_VERSION; }

int azp_device_count(void)
{
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return n;
}

const char* azp_last_error(void) { return azp::g_last_error.c_str(); }

int azp_pair_num_values(int kind) { return n_pair_values(kind); }
int azp_bond_num_values(int kind) { return n_bond_values(kind); }

// Scalars declared by each param_type (src/PairEvaluatorPerturbedLennardJones.h:57-60,
// src/PairEvaluatorExpandedYukawa.h:45-47, src/PairEvaluatorHertz.h:41,
// src/PairEvaluatorColloid.h:48-51, src/DPDPairEvaluatorGeneralWeight.h:54-56,
// src/BondEvaluatorQuartic.h:69-76, src/BondEvaluatorDoubleWell.h:52-55, HOOMD's
// harmonic bond {k, r_0}, src/WallEvaluatorLJ93.h:50-51, src/WallEvaluatorColloid.h:58-60)
// and the record alignment of the single-precision build (the aligned(...)
// branch for HOOMD_LONGREAL_SIZE == 32); 0 for an unknown kind
static int record_fields(int cls, int kind, int* align_single)
{
    *align_single = 16;
    if (cls == AZP_RECORD_PAIR) {
        switch (kind) {
        case AZP_PAIR_PERTURBED_LJ: return 4;
        case AZP_PAIR_EXPANDED_YUKAWA: return 3;
        case AZP_PAIR_HERTZ: *align_single = 4; return 1;
        case AZP_PAIR_COLLOID: return 4;
        case AZP_PAIR_DPD_GENERAL_WEIGHT: return 3;
        default: return 0;
        }
    }
    if (cls == AZP_RECORD_BOND) {
        switch (kind) {
        case AZP_BOND_QUARTIC: return 8;
        case AZP_BOND_DOUBLE_WELL: return 4;
        case AZP_BOND_IMAGE_HARMONIC: *align_single = 8; return 2;
        default: return 0;
        }
    }
    if (cls == AZP_RECORD_WALL) {
        *align_single = 8;
        if (kind == AZP_WALL_LJ93) return 2;
        if (kind == AZP_WALL_COLLOID) return 3;
    }
    return 0;
}

int azp_record_size(int cls, int kind, int single)
{
    int align = 0;
    const int n = record_fields(cls, kind, &align);
    if (n == 0) return AZP_ERR_INVALID;
    if (single) return ((n * 4 + align - 1) / align) * align;
    const int d = cls == AZP_RECORD_PAIR ? azp::pair_record_doubles(kind)
                                         : (cls == AZP_RECORD_BOND ? azp::bond_record_doubles(kind)
                                                                   : azp::wall_record_doubles(kind));
    return 8 * d;
}

int azp_params_from_single(int cls, int kind, const void* src, uint32_t n, double* dst)
{
    int align = 0;
    const int fields = record_fields(cls, kind, &align);
    if (fields == 0 || (n && (!src || !dst))) return AZP_ERR_INVALID;
    const int sb = azp_record_size(cls, kind, 1), dd = azp_record_size(cls, kind, 0) / 8;
    const unsigned char* in = static_cast<const unsigned char*>(src);
    for (uint32_t r = 0; r < n; ++r) {
        float f[8];
        std::memcpy(f, in + (size_t)r * sb, sizeof(float) * fields);
        for (int k = 0; k < dd; ++k) dst[(size_t)r * dd + k] = k < fields ? (double)f[k] : 0.0;
    }
    return AZP_OK;
}

// PairParameters*(pybind11::dict) -- src/PairEvaluatorPerturbedLennardJones.h:33-45,
// src/PairEvaluatorExpandedYukawa.h:28-33, src/PairEvaluatorHertz.h:28-31,
// src/PairEvaluatorColloid.h:28-35
int azp_pair_params_from_values(int kind, const double* v, double* rec)
{
    if (!v || !rec) return AZP_ERR_INVALID;
    if (n_pair_values(kind) <= 0) return AZP_ERR_INVALID;
    for (int k = 0; k < azp::pair_record_doubles(kind); ++k) rec[k] = 0.0;
    switch (kind) {
    case AZP_PAIR_PERTURBED_LJ: {
        const double sigma = v[1], s2 = sigma * sigma, s4 = s2 * s2;
        rec[0] = s2 * s4;                              // sigma_6
        rec[1] = 4.0 * v[0];                           // epsilon_x_4
        rec[2] = v[2];                                 // attraction_scale_factor
        rec[3] = std::pow(2.0, 1.0 / 3.0) * s2;        // rwcasq
        return AZP_OK;
    }
    case AZP_PAIR_EXPANDED_YUKAWA: rec[0] = v[0]; rec[1] = v[1]; rec[2] = v[2]; return AZP_OK;
    case AZP_PAIR_HERTZ: rec[0] = v[0]; return AZP_OK;
    case AZP_PAIR_COLLOID: rec[0] = v[0]; rec[1] = v[1]; rec[2] = v[2]; rec[3] = v[3] * v[3] * v[3]; return AZP_OK;
    // PairParametersDPDGeneralWeight(pybind11::dict), src/DPDPairEvaluatorGeneralWeight.h:37-42
    case AZP_PAIR_DPD_GENERAL_WEIGHT: rec[0] = v[0]; rec[1] = v[1]; rec[2] = v[2]; return AZP_OK;
    default: return AZP_ERR_INVALID;
    }
}

// asDict() of the same structs (:47-54 etc.)
int azp_pair_params_to_values(int kind, const double* rec, double* v)
{
    if (!v || !rec) return AZP_ERR_INVALID;
    switch (kind) {
    case AZP_PAIR_PERTURBED_LJ:
        v[0] = rec[1] / 4.0;
        v[1] = std::pow(rec[0], 1.0 / 6.0);
        v[2] = rec[2];
        return AZP_OK;
    case AZP_PAIR_EXPANDED_YUKAWA: v[0] = rec[0]; v[1] = rec[1]; v[2] = rec[2]; return AZP_OK;
    case AZP_PAIR_HERTZ: v[0] = rec[0]; return AZP_OK;
    case AZP_PAIR_COLLOID: v[0] = rec[0]; v[1] = rec[1]; v[2] = rec[2]; v[3] = std::cbrt(rec[3]); return AZP_OK;
    case AZP_PAIR_DPD_GENERAL_WEIGHT: v[0] = rec[0]; v[1] = rec[1]; v[2] = rec[2]; return AZP_OK;
    default: return AZP_ERR_INVALID;
    }
}

// BondParametersQuartic(pybind11::dict) src/BondEvaluatorQuartic.h:37-55,
// BondParametersDoubleWell(pybind11::dict) src/BondEvaluatorDoubleWell.h:33-39
int azp_bond_params_from_values(int kind, const double* v, double* rec)
{
    if (!v || !rec) return AZP_ERR_INVALID;
    if (n_bond_values(kind) <= 0) return AZP_ERR_INVALID;
    for (int k = 0; k < azp::bond_record_doubles(kind); ++k) rec[k] = 0.0;
    switch (kind) {
    case AZP_BOND_QUARTIC: {
        const double sigma = v[5], s2 = sigma * sigma, s4 = s2 * s2;
        rec[0] = v[0];   // k
        rec[1] = v[1];   // r_0
        rec[2] = v[2];   // b_1
        rec[3] = v[3];   // b_2
        rec[4] = v[4];   // U_0
        rec[5] = s2 * s4;        // sigma_6
        rec[6] = 4.0 * v[6];     // epsilon_x_4
        rec[7] = v[7];   // delta
        return AZP_OK;
    }
    case AZP_BOND_DOUBLE_WELL:
        rec[0] = v[1];          // r_1
        rec[1] = v[1] - v[0];   // r_diff = r_1 - r_0
        rec[2] = v[2];          // U_1
        rec[3] = v[3];          // U_tilt
        return AZP_OK;
    case AZP_BOND_IMAGE_HARMONIC:
        // HOOMD's harmonic bond parameters {k, r0} (src/bond.py:160-192)
        rec[0] = v[0];
        rec[1] = v[1];
        return AZP_OK;
    default: return AZP_ERR_INVALID;
    }
}

int azp_bond_params_to_values(int kind, const double* rec, double* v)
{
    if (!v || !rec) return AZP_ERR_INVALID;
    switch (kind) {
    case AZP_BOND_QUARTIC:
        v[0] = rec[0]; v[1] = rec[1]; v[2] = rec[2]; v[3] = rec[3]; v[4] = rec[4];
        v[5] = std::pow(rec[5], 1.0 / 6.0);
        v[6] = rec[6] / 4.0;
        v[7] = rec[7];
        return AZP_OK;
    case AZP_BOND_DOUBLE_WELL:
        v[0] = rec[0] - rec[1];
        v[1] = rec[0];
        v[2] = rec[2];
        v[3] = rec[3];
        return AZP_OK;
    case AZP_BOND_IMAGE_HARMONIC:
        v[0] = rec[0];
        v[1] = rec[1];
        return AZP_OK;
    default: return AZP_ERR_INVALID;
    }
}

int azp_pair_forces(const azp_system* sys, azp_nlist* nl, int kind, const double* params, const double* r_cut,
                    const double* r_on, int shift_mode, const azp_forces* out, void* stream)
{
    if (!sys || !nl || !params || !r_cut || !out || !out->force) return AZP_ERR_INVALID;
    if (!box_ok(sys->box) || sys->ntypes == 0 || sys->ntypes > azp::MAX_PAIR_TYPES) return AZP_ERR_INVALID;
    if (out->precision != AZP_FP64 && out->precision != AZP_FP32) return AZP_ERR_INVALID;
    if (sys->N != nl->N || sys->ntypes != nl->ntypes) return AZP_ERR_INVALID;
    if (sys->N == 0) return AZP_OK;
    cudaStream_t s = azp::as_stream(stream);
    int st = azp::launch_pair_table(kind, params, r_cut, r_on, shift_mode, sys->ntypes, nl->table, s);
    if (st) return st;
    if (out->precision == AZP_FP32)
        azp::launch_to_fixed(reinterpret_cast<const double4_32a*>(sys->pos), nl->fixed, sys->N, sys->box, s);
    azp::PairArgs a;
    a.pos = reinterpret_cast<const double4_32a*>(sys->pos);
    a.fixed = nl->fixed;
    a.N = sys->N;
    a.ntypes = sys->ntypes;
    fill_box(sys->box, a.L, a.Linv, a.sfix);
    a.counts = nl->counts;
    a.nbrs = nl->nbrs;
    a.max_nn = nl->max_nn;
    a.table = nl->table;
    a.force = out->force;
    a.virial = out->virial;
    a.pitch = out->virial_pitch ? out->virial_pitch : sys->N;
    return azp::launch_pair(kind, out->precision, nl->tpp, a, s);
}

int azp_bond_forces(const azp_system* sys, const uint32_t* n_bonds, const uint32_t* table, uint32_t table_height,
                    int kind, const double* params, uint32_t nbondtypes, const azp_forces* out, uint32_t* err,
                    void* stream)
{
    (void)table_height;
    if (!sys || !n_bonds || !table || !params || !out || !out->force) return AZP_ERR_INVALID;
    if (!box_ok(sys->box) || nbondtypes == 0) return AZP_ERR_INVALID;
    if (sys->N == 0) return AZP_OK;
    azp::BondArgs a;
    a.pos = reinterpret_cast<const double4_32a*>(sys->pos);
    a.fixed = nullptr;
    a.N = sys->N;
    a.nbondtypes = nbondtypes;
    fill_box(sys->box, a.L, a.Linv, a.sfix);
    a.n_bonds = n_bonds;
    a.table = reinterpret_cast<const uint2*>(table);
    a.params = params;
    a.force = out->force;
    a.virial = out->virial;
    a.pitch = out->virial_pitch ? out->virial_pitch : sys->N;
    a.err = err;
    // the ImageHarmonic bond measures the image-unwrapped distance (src/ImagePotentialBond.h:136-140)
    a.image = kind == AZP_BOND_IMAGE_HARMONIC ? sys->image : nullptr;
    if (kind == AZP_BOND_IMAGE_HARMONIC && !sys->image) return AZP_ERR_INVALID;
    return azp::launch_bond(kind, out->precision, a, azp::as_stream(stream));
}

static int fill_step(const azp_system* sys, const uint32_t* group, uint32_t n_group, azp::StepArgs& a)
{
    if (!sys || !sys->pos || !box_ok(sys->box)) return AZP_ERR_INVALID;
    a = azp::StepArgs();
    a.pos = reinterpret_cast<double4_32a*>(sys->pos);
    a.vel = reinterpret_cast<double4_32a*>(sys->vel);
    a.accel = sys->accel;
    a.image = sys->image;
    a.tag = sys->tag;
    a.diameter = sys->diameter;
    a.group = group;
    a.n = group ? n_group : sys->N;
    a.ntypes = sys->ntypes;
    for (int d = 0; d < 3; ++d) {
        a.L[d] = sys->box.L[d];
        a.lo[d] = -0.5 * sys->box.L[d];
        a.hi[d] = 0.5 * sys->box.L[d];
    }
    return AZP_OK;
}

int azp_langevin_step1(const azp_system* sys, const uint32_t* group, uint32_t n_group, double dt, void* stream)
{
    azp::StepArgs a;
    int st = fill_step(sys, group, n_group, a);
    if (st) return st;
    if (!sys->vel || !sys->accel || !sys->image) return AZP_ERR_INVALID;
    a.dt = dt;
    return azp::launch_step1(a, azp::as_stream(stream));
}

int azp_langevin_step2(const azp_system* sys, const uint32_t* group, uint32_t n_group, const void* net_force,
                       int net_precision, const double* gamma, int use_lambda, double lambda, azp_flow flow,
                       double dt, double kT, uint64_t timestep, uint32_t seed, int noiseless, void* stream)
{
    azp::StepArgs a;
    int st = fill_step(sys, group, n_group, a);
    if (st) return st;
    if (!sys->vel || !sys->accel || !sys->tag || !net_force) return AZP_ERR_INVALID;
    if (use_lambda ? !sys->diameter : !gamma) return AZP_ERR_INVALID;
    a.net_force = net_force;
    a.net_precision = net_precision;
    a.gamma = gamma;
    a.use_lambda = use_lambda;
    a.lambda = lambda;
    a.flow = azp::make_flow(flow);
    a.dt = dt;
    a.kT = kT;
    a.timestep = timestep;
    a.seed = seed;
    a.noiseless = noiseless;
    return azp::launch_step2(a, azp::as_stream(stream));
}

int azp_brownian_step(const azp_system* sys, const uint32_t* group, uint32_t n_group, const void* net_force,
                      int net_precision, const double* gamma, int use_lambda, double lambda, azp_flow flow, double dt,
                      double kT, uint64_t timestep, uint32_t seed, int noiseless, double max_displacement,
                      void* stream)
{
    azp::StepArgs a;
    int st = fill_step(sys, group, n_group, a);
    if (st) return st;
    if (!sys->image || !sys->tag || !net_force) return AZP_ERR_INVALID;
    if (use_lambda ? !sys->diameter : !gamma) return AZP_ERR_INVALID;
    a.net_force = net_force;
    a.net_precision = net_precision;
    a.gamma = gamma;
    a.use_lambda = use_lambda;
    a.lambda = lambda;
    a.flow = azp::make_flow(flow);
    a.dt = dt;
    a.kT = kT;
    a.timestep = timestep;
    a.seed = seed;
    a.noiseless = noiseless;
    a.max_disp = max_displacement;
    return azp::launch_brownian(a, azp::as_stream(stream));
}

int azp_uniform3(uint32_t rng_id, uint64_t timestep, uint32_t seed, const uint32_t* tags, uint32_t n, double lo,
                 double hi, double* out, void* stream)
{
    if (!tags || !out) return AZP_ERR_INVALID;
    return azp::launch_uniform3(rng_id, timestep, seed, tags, n, lo, hi, out, azp::as_stream(stream));
}

}  // extern "C"
