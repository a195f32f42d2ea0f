// common.cuh -- shared device/host helpers of the azplugins_gb300 library.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/azplugins_gb300.h"

#define AZP_HD __host__ __device__ __forceinline__
#define AZP_D __device__ __forceinline__

namespace azp
{
// ---------------------------------------------------------------- error handling
// Records the last failing CUDA call for azp_last_error(); returns AZP_ERR_CUDA.
int record_cuda_error(cudaError_t e, const char* what);
// Records a message for azp_last_error(); returns status.
int record_error(int status, const char* msg);

#define AZP_CUDA_TRY(call)                                        \
    do {                                                          \
        cudaError_t e_ = (call);                                  \
        if (e_ != cudaSuccess) return azp::record_cuda_error(e_, #call); \
    } while (0)

#define AZP_CHECK_LAUNCH(what)                                    \
    do {                                                          \
        cudaError_t e_ = cudaGetLastError();                      \
        if (e_ != cudaSuccess) return azp::record_cuda_error(e_, what); \
    } while (0)

inline cudaStream_t as_stream(void* s) { return reinterpret_cast<cudaStream_t>(s); }

// Rebuild kernels take a pointer to the engine's flag words: [0] the rebuild
// request, [1] the error bits. They do nothing unless a rebuild was requested
// and no error has been raised (a system that produced non-finite positions is
// not re-binned: the run ends with the error instead). NULL: always run.
AZP_D bool gated_off(const uint32_t* gate) { return gate && (gate[0] == 0u || gate[1] != 0u); }

// ---------------------------------------------------------------- param_type strides
// doubles of one param_type record in the reference's double-precision layout
// (sizeof / 8): every table argument of the C ABI is an array at this stride
AZP_HD int pair_record_doubles(int kind) { return kind == AZP_PAIR_HERTZ ? 1 : 4; }
AZP_HD int bond_record_doubles(int kind)
{
    return kind == AZP_BOND_QUARTIC ? 8 : (kind == AZP_BOND_DOUBLE_WELL ? 4 : 2);
}
AZP_HD int wall_record_doubles(int kind) { return kind == AZP_WALL_LJ93 ? 2 : 4; }

// ---------------------------------------------------------------- type bits
// The type lives in the low 32 bits of pos.w's bit pattern (HOOMD __int_as_scalar).
AZP_HD uint32_t type_of(double w)
{
#ifdef __CUDA_ARCH__
    return (uint32_t)__double_as_longlong(w);
#else
    union { double d; uint64_t u; } v;
    v.d = w;
    return (uint32_t)v.u;
#endif
}

AZP_HD double type_as_double(uint32_t t)
{
#ifdef __CUDA_ARCH__
    return __longlong_as_double((long long)t);
#else
    union { double d; uint64_t u; } v;
    v.u = (uint64_t)t;
    return v.d;
#endif
}

// ---------------------------------------------------------------- box
struct BoxD {
    double L[3], Linv[3], lo[3], hi[3];
};

inline BoxD make_box(const azp_box& b)
{
    BoxD r;
    for (int d = 0; d < 3; ++d) {
        r.L[d] = b.L[d];
        r.Linv[d] = 1.0 / b.L[d];
        r.lo[d] = -0.5 * b.L[d];
        r.hi[d] = 0.5 * b.L[d];
    }
    return r;
}

// minimum image, same operation order as the oracle (v -= L * rint(v / L) with a
// precomputed 1/L); L * rint(...) is exact for |rint| <= 1 so FMA contraction
// cannot change the result.
AZP_D double min_image1(double v, double L, double Linv) { return v - L * rint(v * Linv); }

// |v|^2 with every product and sum rounded separately (no FMA), bit-identical to
// the oracle compiled with -ffp-contract=off.
AZP_D double rsq_exact(double x, double y, double z)
{
    return __dadd_rn(__dadd_rn(__dmul_rn(x, x), __dmul_rn(y, y)), __dmul_rn(z, z));
}

// ---------------------------------------------------------------- fixed point
// FP32 mode keeps a 16-byte shadow of every position: x, y, z as 32-bit fixed
// point fractions of the box (x / L * 2^32, two's complement wrap) and the type.
// A difference of two fixed values, read as int32, is the minimum image exactly;
// converting it to float costs one rounding (2^-24 relative).
AZP_D uint32_t to_fixed(double x, double Linv)
{
    // x / L in [-1/2, 1/2); scale to [-2^31, 2^31)
    const double s = x * Linv * 4294967296.0;
    return (uint32_t)(int32_t)__double2ll_rn(s);
}

// ---------------------------------------------------------------- compensated sums
// Knuth two-sum: (s, c) += b with the rounding error of s carried in c.
struct Comp {
    float s, c;
    AZP_D void add(float b)
    {
        const float t = s + b;
        const float bp = t - s;
        const float err = (s - (t - bp)) + (b - bp);
        s = t;
        c += err;
    }
    AZP_D float value() const { return s + c; }
};

}  // namespace azp
