// Declarations-only stand-in for HOOMD-blue's hoomd/RandomNumbers.h, enough for
// the reference's DPD evaluator header to parse when oracle/ref_sizes.cpp takes
// sizeof of its param_type. Nothing here is ever called. Test infrastructure.
#ifndef AZP_REF_SHIM_RANDOMNUMBERS_H_
#define AZP_REF_SHIM_RANDOMNUMBERS_H_
#include <cstdint>
namespace hoomd
    {
struct Seed
    {
    Seed(unsigned int, uint64_t, uint16_t) { }
    };
struct Counter
    {
    Counter(unsigned int = 0, unsigned int = 0, unsigned int = 0, unsigned int = 0) { }
    };
struct RandomGenerator
    {
    RandomGenerator(const Seed&, const Counter&) { }
    };
template<typename T> struct UniformDistribution
    {
    UniformDistribution(T, T) { }
    T operator()(RandomGenerator&)
        {
        return T(0);
        }
    };
    } // namespace hoomd
#endif
