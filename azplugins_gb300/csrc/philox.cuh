// philox.cuh -- Philox4x32-10 counter-based generator (Salmon, Moraes, Dror &
// Shaw, "Parallel random numbers: as easy as 1, 2, 3", SC'11) and the uniform
// draws of the flow integrators.
//
// Stream layout (the same in the oracle): the reference keys its integrator
// streams as RandomGenerator(RNGIdentifier, seed, tag, timestep)
// (src/TwoStepLangevinFlow.h:216-219, src/TwoStepBrownianFlow.h:161-164) with
// ids from src/RNGIdentifiers.h:20-27; azplugins_gb300 packs them as
//   key = { id << 24 | (seed & 0xffff) << 8 | (timestep >> 32) & 0xff,
//           timestep & 0xffffffff }
//   ctr = { call index, tag, 0, 0 }
// and maps each 64-bit word w to a double in (0, 1) as ((w >> 11) + 0.5) 2^-53.
#pragma once

#include "common.cuh"

namespace azp
{
struct Philox4 {
    uint32_t v[4];
};

AZP_HD void philox_round(uint32_t& c0, uint32_t& c1, uint32_t& c2, uint32_t& c3, uint32_t k0, uint32_t k1)
{
#ifdef __CUDA_ARCH__
    const uint32_t lo0 = 0xD2511F53u * c0;
    const uint32_t hi0 = __umulhi(0xD2511F53u, c0);
    const uint32_t lo1 = 0xCD9E8D57u * c2;
    const uint32_t hi1 = __umulhi(0xCD9E8D57u, c2);
#else
    const uint64_t p0 = (uint64_t)0xD2511F53u * c0;
    const uint64_t p1 = (uint64_t)0xCD9E8D57u * c2;
    const uint32_t lo0 = (uint32_t)p0, hi0 = (uint32_t)(p0 >> 32);
    const uint32_t lo1 = (uint32_t)p1, hi1 = (uint32_t)(p1 >> 32);
#endif
    const uint32_t n0 = hi1 ^ c1 ^ k0;
    const uint32_t n2 = hi0 ^ c3 ^ k1;
    c0 = n0;
    c1 = lo1;
    c2 = n2;
    c3 = lo0;
}

AZP_HD Philox4 philox4x32_10(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3, uint32_t k0, uint32_t k1)
{
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        philox_round(c0, c1, c2, c3, k0, k1);
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    Philox4 o;
    o.v[0] = c0;
    o.v[1] = c1;
    o.v[2] = c2;
    o.v[3] = c3;
    return o;
}

AZP_HD void stream_key(uint32_t id, uint64_t timestep, uint32_t seed, uint32_t& k0, uint32_t& k1)
{
    k0 = (id << 24) | ((seed & 0xffffu) << 8) | (uint32_t)((timestep >> 32) & 0xffu);
    k1 = (uint32_t)(timestep & 0xffffffffu);
}

AZP_HD double open01(uint32_t hi, uint32_t lo)
{
    const uint64_t w = ((uint64_t)hi << 32) | lo;
    // (w >> 11) + 0.5 and the power-of-two scale are exact
    return ((double)(w >> 11) + 0.5) * (1.0 / 9007199254740992.0);
}

// three uniform doubles in (lo, lo + width): two Philox calls
AZP_HD void uniform3(uint32_t id, uint64_t timestep, uint32_t seed, uint32_t tag, double lo, double width,
                     double& r0, double& r1, double& r2)
{
    uint32_t k0, k1;
    stream_key(id, timestep, seed, k0, k1);
    const Philox4 a = philox4x32_10(0u, tag, 0u, 0u, k0, k1);
    const Philox4 b = philox4x32_10(1u, tag, 0u, 0u, k0, k1);
#ifdef __CUDA_ARCH__
    // two roundings, no FMA: the same doubles as the oracle
    r0 = __dadd_rn(lo, __dmul_rn(width, open01(a.v[0], a.v[1])));
    r1 = __dadd_rn(lo, __dmul_rn(width, open01(a.v[2], a.v[3])));
    r2 = __dadd_rn(lo, __dmul_rn(width, open01(b.v[0], b.v[1])));
#else
    r0 = lo + width * open01(a.v[0], a.v[1]);
    r1 = lo + width * open01(a.v[2], a.v[3]);
    r2 = lo + width * open01(b.v[0], b.v[1]);
#endif
}

// The same three draws at 24-bit resolution for the FP32-force integrator: the
// top 24 bits of each 64-bit word above, as a float in (0, 1).
AZP_HD float open01f(uint32_t hi) { return ((float)(hi >> 8) + 0.5f) * (1.0f / 16777216.0f); }

AZP_HD void uniform3f(uint32_t id, uint64_t timestep, uint32_t seed, uint32_t tag, float lo, float width, float& r0,
                      float& r1, float& r2)
{
    uint32_t k0, k1;
    stream_key(id, timestep, seed, k0, k1);
    const Philox4 a = philox4x32_10(0u, tag, 0u, 0u, k0, k1);
    const Philox4 b = philox4x32_10(1u, tag, 0u, 0u, k0, k1);
    r0 = lo + width * open01f(a.v[0]);
    r1 = lo + width * open01f(a.v[2]);
    r2 = lo + width * open01f(b.v[0]);
}

}  // namespace azp
