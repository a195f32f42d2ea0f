// dual.cuh -- forward-mode dual numbers (value + K partial derivatives) so the
// templated evaluators of evaluators.cuh give exact derivatives of force/r and
// energy with respect to rsq and to the parameter-record fields, for the adjoint
// kernels of the potentials without a hand-written derivative.
#pragma once

#include "common.cuh"
#include <math.h>

namespace azp
{
template<int K> struct Dual {
    double v;
    double d[K];
    AZP_HD Dual() : v(0.0)
    {
#pragma unroll
        for (int k = 0; k < K; ++k) d[k] = 0.0;
    }
    AZP_HD Dual(double x) : v(x)  // NOLINT: implicit from constants, as R(2.5) in the evaluators
    {
#pragma unroll
        for (int k = 0; k < K; ++k) d[k] = 0.0;
    }
    AZP_HD explicit operator int() const { return (int)v; }
    AZP_HD Dual& operator+=(const Dual& b)
    {
        v += b.v;
#pragma unroll
        for (int k = 0; k < K; ++k) d[k] += b.d[k];
        return *this;
    }
    AZP_HD Dual& operator-=(const Dual& b)
    {
        v -= b.v;
#pragma unroll
        for (int k = 0; k < K; ++k) d[k] -= b.d[k];
        return *this;
    }
    AZP_HD Dual& operator*=(const Dual& b)
    {
#pragma unroll
        for (int k = 0; k < K; ++k) d[k] = d[k] * b.v + v * b.d[k];
        v *= b.v;
        return *this;
    }
    AZP_HD Dual& operator/=(const Dual& b)
    {
        const double q = v / b.v;
#pragma unroll
        for (int k = 0; k < K; ++k) d[k] = (d[k] - q * b.d[k]) / b.v;
        v = q;
        return *this;
    }
    // friends (not templates): implicit conversion from double works on either side
    friend AZP_HD Dual operator+(Dual a, const Dual& b) { return a += b; }
    friend AZP_HD Dual operator-(Dual a, const Dual& b) { return a -= b; }
    friend AZP_HD Dual operator*(Dual a, const Dual& b) { return a *= b; }
    friend AZP_HD Dual operator/(Dual a, const Dual& b) { return a /= b; }
    friend AZP_HD Dual operator-(const Dual& a)
    {
        Dual r;
        r.v = -a.v;
#pragma unroll
        for (int k = 0; k < K; ++k) r.d[k] = -a.d[k];
        return r;
    }
    friend AZP_HD bool operator<(const Dual& a, const Dual& b) { return a.v < b.v; }
    friend AZP_HD bool operator>(const Dual& a, const Dual& b) { return a.v > b.v; }
    friend AZP_HD bool operator<=(const Dual& a, const Dual& b) { return a.v <= b.v; }
    friend AZP_HD bool operator>=(const Dual& a, const Dual& b) { return a.v >= b.v; }
    friend AZP_HD bool operator==(const Dual& a, const Dual& b) { return a.v == b.v; }
    friend AZP_HD bool operator!=(const Dual& a, const Dual& b) { return a.v != b.v; }
};

// the global overloads stay visible next to the Dual ones below
using ::exp;
using ::log;
using ::sqrt;


template<int K> AZP_HD Dual<K> chain(const Dual<K>& a, double f, double df)
{
    Dual<K> r;
    r.v = f;
#pragma unroll
    for (int k = 0; k < K; ++k) r.d[k] = df * a.d[k];
    return r;
}
template<int K> AZP_HD Dual<K> sqrt(const Dual<K>& a)
{
    const double s = ::sqrt(a.v);
    return chain(a, s, 0.5 / s);
}
template<int K> AZP_HD Dual<K> exp(const Dual<K>& a)
{
    const double e = ::exp(a.v);
    return chain(a, e, e);
}
template<int K> AZP_HD Dual<K> log(const Dual<K>& a) { return chain(a, ::log(a.v), 1.0 / a.v); }
template<int K> AZP_HD Dual<K> rcp(const Dual<K>& a)
{
    const double r = 1.0 / a.v;
    return chain(a, r, -r * r);
}
template<int K> AZP_HD double value_of(const Dual<K>& a) { return a.v; }
AZP_HD double value_of(double a) { return a; }
AZP_HD double value_of(float a) { return a; }

}  // namespace azp
