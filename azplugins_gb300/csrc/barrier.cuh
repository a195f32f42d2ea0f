// barrier.cuh -- harmonic barrier evaluators (src/PlanarBarrierEvaluator.h,
// src/SphericalBarrierEvaluator.h), shared by the drop-in driver
// (azp_harmonic_barrier_forces) and the engine's fused step.
//
// The evaluators take c = location + offset, formed once: by the driver's
// kernel, or by the engine's host code when it tabulates a run's locations
// (the same double addition, so both give the same c).
#pragma once

#include <cmath>
#include <cstdint>

#include "common.cuh"

namespace azp
{
// src/PlanarBarrierEvaluator.h:36-47: U = k/2 (y - c)^2 above y = c, F = -k (y - c) y_hat.
// Every product and sum is rounded separately, as in the FP64 oracle.
AZP_D void planar_barrier(const double* x, double c, double k, double* f, double& e)
{
    const double dy = __dsub_rn(x[1], c);
    if (dy <= 0.0) return;
    f[1] = -__dmul_rn(k, dy);
    e = __dmul_rn(__dmul_rn(-0.5, f[1]), dy);
}

// src/SphericalBarrierEvaluator.h:36-51: U = k/2 (r - c)^2 beyond r = c, F = -k (r - c) r_hat
AZP_D void spherical_barrier(const double* x, double c, double k, double* f, double& e)
{
    const double r = sqrt(rsq_exact(x[0], x[1], x[2]));
    const double dr = __dsub_rn(r, c);
    if (dr <= 0.0) return;
    const double k_dr = __dmul_rn(k, dr);
    const double s = -__ddiv_rn(k_dr, r);
    for (int d = 0; d < 3; ++d) f[d] = __dmul_rn(s, x[d]);
    e = __dmul_rn(__dmul_rn(0.5, k_dr), dr);
}

// Record of one (timestep, type) for the FP32-force engine, whose positions are
// fixed point (hi word = x / L * 2^32, rounded). Planar: q = c / L * 2^32 rounded
// to an integer (int64, so offsets reaching beyond the box stay exact); the
// barrier acts when hi_y > q, with y - c = (hi_y - q) L 2^-32. Spherical: c as a
// float, r from the hi words.
struct BarrierRecF {
    long long q;
    float c;
    float k;
};
static_assert(sizeof(BarrierRecF) == 16, "BarrierRecF is one 16-byte load");

// FP32 evaluation on the fixed-point shadow (hi words, sfix = L 2^-32 per axis)
AZP_D void planar_barrier_fx(const uint4& hi, const BarrierRecF& r, float sfix_y, float* f, float& e)
{
    const long long d = (long long)(int32_t)hi.y - r.q;
    if (d <= 0) return;
    const float dy = __ll2float_rn(d) * sfix_y;
    f[1] = -r.k * dy;
    e = -0.5f * f[1] * dy;
}

AZP_D void spherical_barrier_fx(const uint4& hi, const BarrierRecF& r, const float* sfix, float* f, float& e)
{
    const float x = (float)(int32_t)hi.x * sfix[0];
    const float y = (float)(int32_t)hi.y * sfix[1];
    const float z = (float)(int32_t)hi.z * sfix[2];
    const float rr = sqrtf(x * x + y * y + z * z);
    const float dr = rr - r.c;
    if (dr <= 0.0f) return;
    const float k_dr = r.k * dr;
    const float s = -__fdiv_rn(k_dr, rr);
    f[0] = s * x;
    f[1] = s * y;
    f[2] = s * z;
    e = 0.5f * k_dr * dr;
}

// src/PlanarBarrierEvaluator.h:50-56 (lo.y <= H < hi.y) and
// src/SphericalBarrierEvaluator.h:54-61 (R >= 0 and 2R within the nearest plane
// distances, which are the edge lengths of an orthorhombic box)
inline bool barrier_location_valid(int geometry, double location, const azp_box& b)
{
    if (geometry == AZP_BARRIER_PLANAR) return location >= -0.5 * b.L[1] && location < 0.5 * b.L[1];
    const double two_R = 2.0 * location;
    return location >= 0.0 && b.L[0] >= two_R && b.L[1] >= two_R && b.L[2] >= two_R;
}

// FP32 record of c = location + offset for a box edge Ly (planar) on the host
inline BarrierRecF barrier_rec_f(int geometry, double c, double k, double Ly)
{
    BarrierRecF r;
    r.k = (float)k;
    if (geometry == AZP_BARRIER_PLANAR) {
        r.q = (long long)std::llrint(c / Ly * 4294967296.0);
        r.c = 0.0f;
    } else {
        r.q = 0;
        r.c = (float)c;
    }
    return r;
}

}  // namespace azp
