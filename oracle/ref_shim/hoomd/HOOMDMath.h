// Minimal stand-in for HOOMD-blue's hoomd/HOOMDMath.h, used ONLY to compile the
// reference's header-only evaluator and flow-field functors on the host for the
// oracle pin (oracle/_ref). Test infrastructure; never linked into the product.
//
// Scalar is double (HOOMD_LONGREAL_SIZE == 64). __host__/__device__ expand to
// nothing because ConstantFlow.h / ParabolicFlow.h emit them in host builds.
#ifndef AZP_REF_SHIM_HOOMDMATH_H_
#define AZP_REF_SHIM_HOOMDMATH_H_

#include <cmath>
#include <cstdint>

#define HOOMD_LONGREAL_SIZE 64
#ifndef __host__
#define __host__
#endif
#ifndef __device__
#define __device__
#endif

namespace hoomd
    {
typedef double Scalar;
struct Scalar3
    {
    double x, y, z;
    };
struct Scalar4
    {
    double x, y, z, w;
    };
inline Scalar3 make_scalar3(double x, double y, double z)
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
    } // namespace fast
    } // namespace hoomd

#endif
