// fixed64.cuh -- state of the FP32-force engine: 64-bit fixed-point positions
// and float-float velocities, advanced without FP64 instructions.
//
// GB300 issues FP64 at about 1/64 of its FP32 rate, so an FP64 add per
// coordinate per step costs more than the whole FP32 force loop. The FP32-force
// engine therefore keeps positions and velocities in forms that accumulate at
// least as precisely as FP64 with FP32 and integer instructions only:
//
//  * position component x in [-L/2, L/2) as the signed 64-bit integer
//    q = x / L * 2^64 (resolution L * 2^-64, about 6e-18 sigma at L = 100),
//    stored as hi = round(q / 2^32) -- the 16-byte shadow that neighbours gather,
//    whose int32 differences are exact minimum images -- and the low word
//    lo = q - hi * 2^32 in [-2^31, 2^31) (private to the particle). Periodic
//    wrapping is the two's complement wrap of q; an image crossing is a signed
//    overflow of the add.
//  * velocity component as an unevaluated float pair v = h + l (about 48
//    significant bits), updated by an error-free two-sum.
//
// A step's increments (kicks, displacements) are FP32, as accurate as the FP32
// forces they come from; their accumulation loses nothing (positions) or
// 2^-48 relative (velocities).
#pragma once

#include <cmath>

#include "common.cuh"

namespace azp
{
// velocity record of the FP32-force engine: h = (vx, vy, vz, 1/m) leading
// floats, l = (vx, vy, vz) trailing floats (l.w unused)
struct __align__(32) VelFF {
    float4 h;
    float4 l;
};

AZP_HD int64_t fx_join(uint32_t hi, uint32_t lo)
{
    return (int64_t)(((uint64_t)hi << 32) + (uint64_t)(int64_t)(int32_t)lo);
}

AZP_HD void fx_split(int64_t q, uint32_t& hi, uint32_t& lo)
{
    lo = (uint32_t)(uint64_t)q;
    hi = (uint32_t)(((uint64_t)q - (uint64_t)(int64_t)(int32_t)lo) >> 32);
}

// x = q * (L 2^-64): one rounding in the conversion, one in the product
AZP_HD double fx_to_double(int64_t q, double l64) { return (double)q * l64; }

// q = round(x / L * 2^64) for any x (wrapped into [-L/2, L/2) first)
AZP_HD int64_t fx_from_double(double x, double Linv)
{
    double t = x * Linv;
    t -= floor(t + 0.5);  // [-1/2, 1/2)
    if (t >= 0.5) t -= 1.0;
    const double s = t * 18446744073709551616.0;  // exact power-of-two scaling
#ifdef __CUDA_ARCH__
    return __double2ll_rn(s);
#else
    return (int64_t)llrint(s);
#endif
}

// float-float accumulation: (h, l) += k, error-free two-sum then renormalise
AZP_D void ff_add(float& h, float& l, float k)
{
    const float s = __fadd_rn(h, k);
    const float bb = __fsub_rn(s, h);
    const float err = __fadd_rn(__fsub_rn(h, __fsub_rn(s, bb)), __fsub_rn(k, bb));
    const float t = __fadd_rn(l, err);
    h = __fadd_rn(s, t);
    l = __fsub_rn(t, __fsub_rn(h, s));
}

// Adds the displacement dx (float, in length units) to the fixed-point
// component (hi, lo). s_hi + s_lo = 2^32 / L as a float pair, so dx * 2^32 / L is
// formed to float-float accuracy (the FMA gives the product's rounding error
// exactly). Returns the image change (+1, -1 or 0). Sets bad (and leaves the
// component unchanged) when dx is not finite or moves half a box or more in one
// step (a move the minimum-image convention cannot represent).
AZP_D int fx_advance(uint32_t& hi, uint32_t& lo, float dx, float s_hi, float s_lo, bool& bad)
{
    const float p = __fmul_rn(dx, s_hi);                               // units of L 2^-32
    const float e = __fadd_rn(__fmaf_rn(dx, s_hi, -p), __fmul_rn(dx, s_lo));
    const bool ok = fabsf(p) < 2147483392.0f;                          // |dx| < L / 2; false for NaN
    bad |= !ok;
    const float ip = rintf(p);
    const float t = __fadd_rn(__fsub_rn(p, ip), e);                     // p - ip is exact
    const float it = rintf(t);
    const float fr = __fsub_rn(t, it);                                   // exact, |fr| <= 1/2
    const int64_t ih = ok ? (int64_t)__float2int_rn(ip) + __float2int_rn(it) : 0;
    const int32_t il = ok ? __float2int_rn(__fmul_rn(fr, 2147483648.0f)) : 0;  // units of L 2^-63
    const int64_t dq = (int64_t)((uint64_t)ih << 32) + (int64_t)il * 2;
    const int64_t q0 = fx_join(hi, lo);
    const int64_t q1 = (int64_t)((uint64_t)q0 + (uint64_t)dq);
    fx_split(q1, hi, lo);
    // signed overflow of q0 + dq: the component crossed the +L/2 or -L/2 face
    return ((q0 ^ q1) & (dq ^ q1)) < 0 ? (dq > 0 ? 1 : -1) : 0;
}

// FP32 flow field: CONSTANT u = (a, b, c); PARABOLIC u_x = a (1 - (y b)^2) with
// a = Umax and b = 1 / half-width (src/ConstantFlow.h:48-51, src/ParabolicFlow.h:69-73)
struct FlowF {
    int kind;
    float a, b, c;
};

AZP_D void flow_at_ff(const FlowF& f, float y, float& ux, float& uy, float& uz)
{
    if (f.kind == AZP_FLOW_PARABOLIC) {
        const float yr = y * f.b;
        ux = f.a * (1.0f - yr * yr);
        uy = 0.0f;
        uz = 0.0f;
    } else {
        ux = f.a;
        uy = f.b;
        uz = f.c;
    }
}

}  // namespace azp
