// Minimal stand-in for HOOMD-blue's hoomd/HOOMDMath.h, used ONLY to compile the
// reference's header-only evaluator and flow-field functors on the host for the
// oracle pin (oracle/_ref). Test infrastructure; never linked into the product.
//
// Scalar is double (HOOMD_LONGREAL_SIZE == 64); with AZP_REF_SINGLE defined it is
// float (HOOMD_LONGREAL_SIZE == 32, HOOMD's single-precision build), used only to
// take sizeof of the param_type records (oracle/ref_sizes.cpp). __host__/__device__
// expand to nothing because ConstantFlow.h / ParabolicFlow.h emit them in host builds.
#ifndef AZP_REF_SHIM_HOOMDMATH_H_
#define AZP_REF_SHIM_HOOMDMATH_H_

#include <cmath>
#include <cstdint>

#ifdef AZP_REF_SINGLE
#define HOOMD_LONGREAL_SIZE 32
#else
#define HOOMD_LONGREAL_SIZE 64
#endif
#ifndef __host__
#define __host__
#endif
#ifndef __device__
#define __device__
#endif

namespace hoomd
    {
#ifdef AZP_REF_SINGLE
typedef float Scalar;
#else
typedef double Scalar;
#endif
struct Scalar3
    {
    Scalar x, y, z;
    };
struct Scalar4
    {
    Scalar x, y, z, w;
    };
inline Scalar3 make_scalar3(Scalar x, Scalar y, Scalar z)
    {
    return Scalar3 {x, y, z};
    }
namespace fast
    {
inline double sqrt(double x)
    {
    return std::sqrt(x);
    }
inline double rsqrt(double x)
    {
    return 1.0 / std::sqrt(x);
    }
inline double exp(double x)
    {
    return std::exp(x);
    }
inline double pow(double x, double y)
    {
    return std::pow(x, y);
    }
inline float sqrt(float x)
    {
    return std::sqrt(x);
    }
inline float rsqrt(float x)
    {
    return 1.0f / std::sqrt(x);
    }
inline float exp(float x)
    {
    return std::exp(x);
    }
inline float pow(float x, float y)
    {
    return std::pow(x, y);
    }
    } // namespace fast
    } // namespace hoomd

#endif
