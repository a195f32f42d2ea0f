// external.cu -- azp_harmonic_barrier_forces: the moving harmonic barriers of
// src/HarmonicBarrier.h (planar and spherical evaluators) as a drop-in driver.
//
// One thread per particle, as HOOMD's ForceCompute contract has it: the force
// and energy of the barrier alone are written (overwritten) per particle and the
// virial is zeroed, because the reference does not compute it
// (src/HarmonicBarrier.h:177-179). FP64 output: FP64 arithmetic with every
// product and sum rounded as the FP64 oracle rounds it (no FMA contraction), so
// the results are bit-identical to the oracle's. FP32 output: FP32 arithmetic
// after the FP64 wrap and the one difference that cancels near the barrier (FP64
// runs at about 1/64 of the FP32 rate; its operations, not HBM, bounded the
// FP64 form).
#include <string>

#include "barrier.cuh"
#include "common.cuh"
#include "integrate.cuh"

namespace azp
{
namespace
{
constexpr int kBlock = 256;

template<int GEOM, typename T>
__global__ void __launch_bounds__(kBlock) k_harmonic_barrier(const double4_32a* __restrict__ pos,
                                                              const double2* __restrict__ params, BoxD box,
                                                              double location, uint32_t N, T* __restrict__ force,
                                                              T* __restrict__ virial, uint32_t pitch)
{
    const uint32_t i = blockIdx.x * kBlock + threadIdx.x;
    if (i >= N) return;
    const double4_32a p = pos[i];
    double x[3] = {p.x, p.y, p.z};
    // wrap into the box in case a particle drifted out (src/HarmonicBarrier.h:168-170);
    // the planar form reads y only, so only y is wrapped (FP64 is the cost here)
    int img = 0;
    if constexpr (GEOM == AZP_BARRIER_PLANAR)
        wrap1(x[1], img, box.L[1], box.lo[1], box.hi[1]);
    else
        for (int d = 0; d < 3; ++d) wrap1(x[d], img, box.L[d], box.lo[d], box.hi[d]);
    const double2 kp = __ldg(&params[type_of(p.w)]);
    const double c = __dadd_rn(location, kp.y);
    if constexpr (sizeof(T) == 8) {
        double f[3] = {0.0, 0.0, 0.0}, e = 0.0;
        if constexpr (GEOM == AZP_BARRIER_PLANAR)
            planar_barrier(x, c, kp.x, f, e);
        else
            spherical_barrier(x, c, kp.x, f, e);
        reinterpret_cast<double4_32a*>(force)[i] = make_double4_32a(f[0], f[1], f[2], e);
    } else {
        // FP32 output: FP64 for the wrap and the one difference that cancels
        // (y - c; r^2 - c^2 for the sphere, so that r - c = (r^2 - c^2) / (r + c)
        // keeps FP32 relative accuracy without an FP64 square root), FP32 after
        float f[3] = {0.0f, 0.0f, 0.0f}, e = 0.0f;
        const float k = (float)kp.x;
        if constexpr (GEOM == AZP_BARRIER_PLANAR) {
            const float dy = (float)(x[1] - c);
            if (dy > 0.0f) {
                f[1] = -k * dy;
                e = -0.5f * f[1] * dy;
            }
        } else {
            const double r2 = x[0] * x[0] + x[1] * x[1] + x[2] * x[2];
            const float rf = sqrtf((float)r2);
            // c <= 0 (an offset below -R): r - c does not cancel
            const float dr = c > 0.0 ? (float)(r2 - c * c) / (rf + (float)c) : rf - (float)c;
            if (dr > 0.0f && rf > 0.0f) {
                const float k_dr = k * dr;
                const float sc = -k_dr / rf;
                f[0] = sc * (float)x[0];
                f[1] = sc * (float)x[1];
                f[2] = sc * (float)x[2];
                e = 0.5f * k_dr * dr;
            }
        }
        reinterpret_cast<float4*>(force)[i] = make_float4(f[0], f[1], f[2], e);
    }
    if (virial)
        for (int c = 0; c < 6; ++c) virial[(size_t)c * pitch + i] = T(0);
}

template<int GEOM>
void launch_barrier(const azp_system* sys, double location, const double* params, const azp_forces* out,
                    cudaStream_t s)
{
    const BoxD box = make_box(sys->box);
    const uint32_t grid = (sys->N + kBlock - 1) / kBlock;
    const uint32_t pitch = out->virial_pitch ? out->virial_pitch : sys->N;
    const auto* pos = reinterpret_cast<const double4_32a*>(sys->pos);
    const auto* par = reinterpret_cast<const double2*>(params);
    if (out->precision == AZP_FP64)
        k_harmonic_barrier<GEOM, double><<<grid, kBlock, 0, s>>>(pos, par, box, location, sys->N,
                                                                 static_cast<double*>(out->force),
                                                                 static_cast<double*>(out->virial), pitch);
    else
        k_harmonic_barrier<GEOM, float><<<grid, kBlock, 0, s>>>(pos, par, box, location, sys->N,
                                                                static_cast<float*>(out->force),
                                                                static_cast<float*>(out->virial), pitch);
}
}  // namespace

}  // namespace azp

extern "C" int azp_harmonic_barrier_forces(const azp_system* sys, int geometry, double location, const double* params,
                                           const azp_forces* out, void* stream)
{
    using namespace azp;
    if (!sys || !out || !out->force) return AZP_ERR_INVALID;
    if (geometry != AZP_BARRIER_PLANAR && geometry != AZP_BARRIER_SPHERICAL) return AZP_ERR_INVALID;
    if (out->precision != AZP_FP64 && out->precision != AZP_FP32) return AZP_ERR_INVALID;
    for (int d = 0; d < 3; ++d)
        if (!(sys->box.L[d] > 0.0) || !(sys->box.L[d] < 1e300)) return AZP_ERR_INVALID;
    if (!barrier_location_valid(geometry, location, sys->box))
        return record_error(AZP_ERR_INVALID, "Barrier position is invalid");
    if (sys->N == 0) return AZP_OK;
    if (!sys->pos || !params) return AZP_ERR_INVALID;
    cudaStream_t s = as_stream(stream);
    if (geometry == AZP_BARRIER_PLANAR)
        launch_barrier<AZP_BARRIER_PLANAR>(sys, location, params, out, s);
    else
        launch_barrier<AZP_BARRIER_SPHERICAL>(sys, location, params, out, s);
    AZP_CHECK_LAUNCH("k_harmonic_barrier");
    return AZP_OK;
}
