// azp_oracle.cpp -- CPU restatement of the azplugins short-range
// force-and-integrate path, in FP64. TEST INFRASTRUCTURE ONLY: the tests, the
// smoke check and the bench's CPU-baseline leg load it to check and time the
// GPU results against; the product (azplugins_gb300) never links, imports or
// calls it.
//
// What is restated, and from where (paths relative to the azplugins tree):
//   * pair evaluators   src/PairEvaluatorPerturbedLennardJones.h:117-155,
//                       src/PairEvaluatorExpandedYukawa.h:92-115,
//                       src/PairEvaluatorHertz.h:93-110,
//                       src/PairEvaluatorColloid.h:101-269
//   * pair parameters   the dict constructors of the same headers (:25-66 etc.)
//   * bond evaluators   src/BondEvaluatorQuartic.h:129-200,
//                       src/BondEvaluatorDoubleWell.h:96-113
//   * flow fields       src/ConstantFlow.h:48-51, src/ParabolicFlow.h:69-93
//   * Langevin flow     src/TwoStepLangevinFlow.h:128-153 (step one),
//                       :194-245 (step two)
//   * Brownian flow     src/TwoStepBrownianFlow.h:136-178 (type bits kept)
//   * RNG stream ids    src/RNGIdentifiers.h:20-27
//   * pair loop         HOOMD PotentialPair (not in the tree); observable
//                       contract src/pytest/test_pair.py:351-363 (half energy per
//                       particle, equal and opposite forces), virial order
//                       src/ImagePotentialBondGPU.cuh:228-234
//   * bond loop         src/ImagePotentialBond.h:142-194 with minimum image
//   * neighbour list    HOOMD NeighborListBinned (not in the tree): all j != i
//                       with |dx|^2 < (r_cut_ij + r_buff)^2, r_cut_ij > 0,
//                       minus exclusions; rebuilt when a particle moved more
//                       than r_buff/2 since the last build.
//   * wall potentials   src/WallEvaluatorLJ93.h:100-133, src/WallEvaluatorColloid.h:118-183
//                       (HOOMD's EvaluatorWalls restated from its documentation)
//   * velocity field    src/VelocityFieldCompute.h:196-344, src/*BinningOperation.h
//   * harmonic barrier  src/HarmonicBarrier.h:149-180,
//                       src/PlanarBarrierEvaluator.h:36-56,
//                       src/SphericalBarrierEvaluator.h:36-61
//   * Philox4x32-10     Salmon, Moraes, Dror, Shaw, SC'11 (published algorithm)
//
// Compiled with -ffp-contract=off so that x86 and Arm builds round alike.
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <vector>
#include <algorithm>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace
{
// ---------------------------------------------------------------- evaluators
enum PairKind { PAIR_PLJ = 0, PAIR_EYUK = 1, PAIR_HERTZ = 2, PAIR_COLLOID = 3, PAIR_DPD = 4 };
enum BondKind { BOND_QUARTIC = 0, BOND_DOUBLEWELL = 1, BOND_IMAGE_HARMONIC = 2 };
enum ShiftMode { MODE_NONE = 0, MODE_SHIFT = 1, MODE_XPLOR = 2 };

// Perturbed LJ: p = {sigma^6, 4 eps, lambda, 2^(1/3) sigma^2}
inline double plj_energy_raw(double r6inv, double lj1, double lj2) { return r6inv * (lj1 * r6inv - lj2); }

bool eval_plj(const double* p, double rsq, double rcutsq, bool shift, double& fdr, double& e)
{
    const double lj1 = p[1] * p[0] * p[0];
    const double lj2 = p[1] * p[0];
    const double lam = p[2];
    const double rwcasq = p[3];
    if (!(rsq < rcutsq) || lj1 == 0.0) return false;
    const double wca_shift = p[1] * (1.0 - lam) / 4.0;
    const double r2inv = 1.0 / rsq;
    const double r6inv = r2inv * r2inv * r2inv;
    double f = r2inv * r6inv * (12.0 * lj1 * r6inv - 6.0 * lj2);
    double u = plj_energy_raw(r6inv, lj1, lj2);
    if (rsq < rwcasq) {
        u += wca_shift;
    } else {
        f *= lam;
        u *= lam;
    }
    if (shift) {
        const double rc2inv = 1.0 / rcutsq;
        const double rc6inv = rc2inv * rc2inv * rc2inv;
        double uc = plj_energy_raw(rc6inv, lj1, lj2);
        if (rcutsq < rwcasq) uc += wca_shift; else uc *= lam;
        u -= uc;
    }
    fdr = f;
    e = u;
    return true;
}

// Expanded Yukawa: p = {eps, kappa, delta}
bool eval_eyuk(const double* p, double rsq, double rcutsq, bool shift, double& fdr, double& e)
{
    const double eps = p[0], kap = p[1], del = p[2];
    if (!(rsq < rcutsq) || eps == 0.0) return false;
    const double r = std::sqrt(rsq);
    const double s = r - del;
    const double sinv = 1.0 / s;
    double u = eps * std::exp(-kap * s) * sinv;
    fdr = u * (kap + sinv) / r;
    if (shift) {
        const double sc = std::sqrt(rcutsq) - del;
        u -= eps * std::exp(-kap * sc) / sc;
    }
    e = u;
    return true;
}

// Hertz: p = {eps}; never shifted (goes to zero at r_cut)
bool eval_hertz(const double* p, double rsq, double rcutsq, bool, double& fdr, double& e)
{
    const double eps = p[0];
    if (!(rsq < rcutsq) || eps == 0.0) return false;
    const double r = std::sqrt(rsq);
    const double rc = std::sqrt(rcutsq);
    const double x = 1.0 - r / rc;
    const double ex32 = eps * x * std::sqrt(x);
    fdr = 2.5 * ex32 / (r * rc);
    e = ex32 * x;
    return true;
}

// Colloid (Everaers-Ejtehadi integrated LJ): p = {A, a_1, a_2, sigma^3}
double colloid_ss(double A, double s6, double rsq, double* fdr)
{
    const double r2inv = 1.0 / rsq;
    const double r6inv = r2inv * r2inv * r2inv;
    const double c = A * s6 / 36.0;
    if (fdr) *fdr = 6.0 * c * r2inv * r6inv * (2.0 * s6 * r6inv - 1.0);
    return c * r6inv * (s6 * r6inv - 1.0);
}

double colloid_cs(double A, double s3, double s6, double a, double rsq, double* fdr)
{
    const double a2 = a * a;
    const double d = a2 - rsq;           // a^2 - r^2
    const double d3 = d * d * d;
    const double d6 = d3 * d3;
    const double r4 = rsq * rsq;
    const double pre = s3 * A * a * a2 / d3;
    if (fdr) {
        const double poly = 2.0 * (a2 + rsq) * (a2 * (5.0 * a2 + 22.0 * rsq) + 5.0 * r4);
        *fdr = (4.0 / 15.0) * pre * (poly * s6 / d6 - 5.0) / d;
    }
    const double poly_e = a2 * (a2 * (a2 / 3.0 + 3.0 * rsq) + 4.2 * r4) + rsq * r4;
    return (2.0 / 9.0) * pre * (1.0 - poly_e * s6 / d6);
}

inline double inv7(double x)
{
    const double xi = 1.0 / x;
    double g = xi * xi;
    g = g * g * g;
    return g * xi;
}

double colloid_cc(double A, double s6, double ai, double aj, double rsq, double* fdr)
{
    const double r = std::sqrt(rsq);
    const double prod = ai * aj;
    const double sum = ai + aj;
    const double dif = ai - aj;
    const double sp = sum + r, sm = sum - r, dp = dif + r, dm = dif - r;
    const double q7 = 1.0 / (sp * sm);
    const double q8 = 1.0 / (dp * dm);
    double g0 = inv7(sp), g1 = inv7(sm), g2 = inv7(dp), g3 = inv7(dm);
    const double h0 = ((sp + 5.0 * sum) * sp + 30.0 * prod) * g0;
    const double h1 = ((sm + 5.0 * sum) * sm + 30.0 * prod) * g1;
    const double h2 = ((dp + 5.0 * dif) * dp - 30.0 * prod) * g2;
    const double h3 = ((dm + 5.0 * dif) * dm - 30.0 * prod) * g3;
    const double pre = A * s6 / r / 37800.0;
    double u = pre * (h0 - h1 - h2 + h3);
    if (fdr) {
        g0 *= 42.0 * prod / sp + 6.0 * sum + sp;
        g1 *= 42.0 * prod / sm + 6.0 * sum + sm;
        g2 *= -42.0 * prod / dp + 6.0 * dif + dp;
        g3 *= -42.0 * prod / dm + 6.0 * dif + dm;
        const double dur = u / r + 5.0 * pre * (g0 + g1 - g2 - g3);
        const double dua = -A / 3.0 * r * ((2.0 * prod * q7 + 1.0) * q7 + (2.0 * prod * q8 - 1.0) * q8);
        *fdr = (dur + dua) / r;
    }
    u += A / 6.0 * (2.0 * prod * (q7 + q8) - std::log(q8 / q7));
    return u;
}

bool eval_colloid(const double* p, double rsq, double rcutsq, bool shift, double& fdr, double& e)
{
    const double A = p[0], a1 = p[1], a2 = p[2], s3 = p[3];
    if (!(rsq < rcutsq) || A == 0.0) return false;
    const double s6 = s3 * s3;
    double u;
    if (a1 == 0.0 && a2 == 0.0) {
        u = colloid_ss(A, s6, rsq, &fdr);
        if (shift) u -= colloid_ss(A, s6, rcutsq, nullptr);
    } else if (a1 != 0.0 && a2 != 0.0) {
        u = colloid_cc(A, s6, a1, a2, rsq, &fdr);
        if (shift) u -= colloid_cc(A, s6, a1, a2, rcutsq, nullptr);
    } else {
        const double a = a1 > a2 ? a1 : a2;
        u = colloid_cs(A, s3, s6, a, rsq, &fdr);
        if (shift) u -= colloid_cs(A, s3, s6, a, rcutsq, nullptr);
    }
    e = u;
    return true;
}

// DPD general weight, conservative part only: p = {A, gamma, s}
bool eval_dpd_cons(const double* p, double rsq, double rcutsq, bool, double& fdr, double& e)
{
    if (!(rsq < rcutsq)) return false;
    const double A = p[0];
    const double rinv = 1.0 / std::sqrt(rsq);
    const double r = 1.0 / rinv;
    const double rcinv = 1.0 / std::sqrt(rcutsq);
    const double rc = 1.0 / rcinv;
    fdr = A * (rinv - rcinv);
    e = A * (rc - r) - 0.5 * A * rcinv * (rcutsq - rsq);
    return true;
}

bool eval_pair(int kind, const double* p, double rsq, double rcutsq, bool shift, double& f, double& e)
{
    switch (kind) {
    case PAIR_PLJ: return eval_plj(p, rsq, rcutsq, shift, f, e);
    case PAIR_EYUK: return eval_eyuk(p, rsq, rcutsq, shift, f, e);
    case PAIR_HERTZ: return eval_hertz(p, rsq, rcutsq, shift, f, e);
    case PAIR_COLLOID: return eval_colloid(p, rsq, rcutsq, shift, f, e);
    case PAIR_DPD: return eval_dpd_cons(p, rsq, rcutsq, shift, f, e);
    default: return false;
    }
}

// Quartic bond: p = {k, r_0, b_1, b_2, U_0, sigma^6, 4 eps, delta}
bool eval_quartic(const double* p, double rsq, double& fdr, double& e)
{
    const double k = p[0], r0 = p[1], b1 = p[2], b2 = p[3], U0 = p[4];
    const double lj1 = p[6] * p[5] * p[5];
    const double lj2 = p[6] * p[5];
    const double del = p[7];
    fdr = 0.0;
    e = 0.0;
    if (r0 == 0.0) return false;
    double rr = 1.0;  // (reduced distance) - r_0, positive means "beyond r_0"
    if (del == 0.0) {
        const double r2inv = 1.0 / rsq;
        const double r6inv = r2inv * r2inv * r2inv;
        if (lj1 != 0.0 && r6inv > (lj2 / lj1) / 2.0) {
            fdr += r2inv * r6inv * (12.0 * lj1 * r6inv - 6.0 * lj2);
            e += r6inv * (lj1 * r6inv - lj2) + lj2 * lj2 / 4.0 / lj1;
        }
        if (rsq < r0 * r0) rr = std::sqrt(rsq) - r0;
    } else {
        const double rs = std::sqrt(rsq) - del;
        const double r2inv = 1.0 / rs / rs;
        const double r6inv = r2inv * r2inv * r2inv;
        if (lj1 != 0.0 && r6inv > (lj2 / lj1) / 2.0) {
            fdr += r6inv * (12.0 * lj1 * r6inv - 6.0 * lj2) / rs / (rs + del);
            e += r6inv * (lj1 * r6inv - lj2) + p[6] / 4.0;
        }
        if (rs < r0) rr = rs - r0;
    }
    if (rr < 0.0) {
        fdr += -k * rr * (4.0 * rr * rr - 3.0 * (b1 + b2) * rr + 2.0 * b1 * b2) / (rr + r0 + del);
        e += k * (rr - b1) * (rr - b2) * rr * rr + U0;
    } else {
        e += U0;
    }
    return true;
}

// Double well bond: p = {r_1, r_1 - r_0, U_1, U_tilt}
bool eval_doublewell(const double* p, double rsq, double& fdr, double& e)
{
    const double r1 = p[0], rd = p[1], U1 = p[2], Ut = p[3];
    fdr = 0.0;
    e = 0.0;
    if (rd == 0.0) return false;
    const double r = std::sqrt(rsq);
    const double x = (r1 - r) / rd;
    const double y = 1.0 - x * x;
    e = U1 * y * y + Ut * (1.0 - x - y * y);
    fdr = (4.0 * x * y * (Ut - U1) - Ut) / (rd * r);
    return true;
}

// harmonic bond (HOOMD's EvaluatorBondHarmonic, applied by src/ImagePotentialBond.h:
// 144-152): p = {k, r_0}; U = k/2 (r - r_0)^2, F/r = k (r_0/r - 1) (0 at r = 0)
bool eval_harmonic(const double* p, double rsq, double& f, double& e)
{
    const double k = p[0], r0 = p[1];
    const double r = std::sqrt(rsq);
    f = r > 0.0 ? k * (r0 / r - 1.0) : 0.0;
    e = 0.5 * k * (r0 - r) * (r0 - r);
    return true;
}

bool eval_bond(int kind, const double* p, double rsq, double& f, double& e)
{
    switch (kind) {
    case BOND_QUARTIC: return eval_quartic(p, rsq, f, e);
    case BOND_DOUBLEWELL: return eval_doublewell(p, rsq, f, e);
    case BOND_IMAGE_HARMONIC: return eval_harmonic(p, rsq, f, e);
    default: return false;
    }
}

// RNG stream ids, src/RNGIdentifiers.h:20-27
constexpr uint8_t RNG_DPD = 200, RNG_BROWNIAN = 201, RNG_LANGEVIN = 202;

// ---------------------------------------------------------------- Philox4x32-10
inline void mulhilo(uint32_t a, uint32_t b, uint32_t& hi, uint32_t& lo)
{
    const uint64_t p = (uint64_t)a * (uint64_t)b;
    hi = (uint32_t)(p >> 32);
    lo = (uint32_t)p;
}

void philox(const uint32_t in[4], const uint32_t key_in[2], uint32_t out[4])
{
    uint32_t c0 = in[0], c1 = in[1], c2 = in[2], c3 = in[3];
    uint32_t k0 = key_in[0], k1 = key_in[1];
    for (int round = 0; round < 10; ++round) {
        uint32_t hi0, lo0, hi1, lo1;
        mulhilo(0xD2511F53u, c0, hi0, lo0);
        mulhilo(0xCD9E8D57u, c2, hi1, lo1);
        const uint32_t n0 = hi1 ^ c1 ^ k0;
        const uint32_t n1 = lo1;
        const uint32_t n2 = hi0 ^ c3 ^ k1;
        const uint32_t n3 = lo0;
        c0 = n0; c1 = n1; c2 = n2; c3 = n3;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

// Stream layout used here and on the GPU (mirrors HOOMD's Seed(id, timestep, seed) +
// Counter(tag) structure; HOOMD's exact packing is not available to pin):
//   key = { id<<24 | (seed & 0xffff)<<8 | (timestep>>32 & 0xff), timestep & 0xffffffff }
//   ctr = { call index, tag, 0, 0 }
// Each Philox call yields two 64-bit words (w0<<32|w1, w2<<32|w3); a uniform
// double in (0,1) is ((u64 >> 11) + 0.5) * 2^-53. Three draws use two calls.
inline void stream_key(uint8_t id, uint64_t timestep, uint32_t seed, uint32_t key[2])
{
    key[0] = ((uint32_t)id << 24) | ((seed & 0xffffu) << 8) | (uint32_t)((timestep >> 32) & 0xffu);
    key[1] = (uint32_t)(timestep & 0xffffffffu);
}

inline double u64_to_open01(uint64_t u) { return ((double)(u >> 11) + 0.5) * (1.0 / 9007199254740992.0); }

void uniform3(uint8_t id, uint64_t timestep, uint32_t seed, uint32_t tag, double lo, double hi, double r[3])
{
    uint32_t key[2];
    stream_key(id, timestep, seed, key);
    uint32_t c0[4] = {0u, tag, 0u, 0u}, c1[4] = {1u, tag, 0u, 0u};
    uint32_t o0[4], o1[4];
    philox(c0, key, o0);
    philox(c1, key, o1);
    const uint64_t u0 = ((uint64_t)o0[0] << 32) | o0[1];
    const uint64_t u1 = ((uint64_t)o0[2] << 32) | o0[3];
    const uint64_t u2 = ((uint64_t)o1[0] << 32) | o1[1];
    const double w = hi - lo;
    r[0] = lo + w * u64_to_open01(u0);
    r[1] = lo + w * u64_to_open01(u1);
    r[2] = lo + w * u64_to_open01(u2);
}

// ---------------------------------------------------------------- box
struct Box {
    double L[3], Linv[3], lo[3], hi[3];
};

inline Box make_box(const double* L)
{
    Box b;
    for (int d = 0; d < 3; ++d) {
        b.L[d] = L[d];
        b.Linv[d] = 1.0 / L[d];
        b.lo[d] = -0.5 * L[d];
        b.hi[d] = 0.5 * L[d];
    }
    return b;
}

inline void min_image(const Box& b, double* v)
{
    for (int d = 0; d < 3; ++d) v[d] -= b.L[d] * std::rint(v[d] * b.Linv[d]);
}

inline void wrap(const Box& b, double* x, int* img)
{
    for (int d = 0; d < 3; ++d) {
        if (x[d] >= b.hi[d]) { x[d] -= b.L[d]; img[d] += 1; }
        else if (x[d] < b.lo[d]) { x[d] += b.L[d]; img[d] -= 1; }
    }
}

inline double rsq_of(const double* v) { return v[0] * v[0] + v[1] * v[1] + v[2] * v[2]; }

// ---------------------------------------------------------------- neighbour list
struct Excl {
    const int32_t* start;  // [N+1] CSR of excluded partner indices
    const int32_t* idx;
};

inline bool excluded(const Excl& ex, int i, int j)
{
    if (!ex.start) return false;
    for (int k = ex.start[i]; k < ex.start[i + 1]; ++k)
        if (ex.idx[k] == j) return true;
    return false;
}

inline bool listed(const Box& b, const double* pos, const int32_t* type, int ntypes,
                   const double* rlistsq, int i, int j)
{
    double v[3] = {pos[4 * i] - pos[4 * j], pos[4 * i + 1] - pos[4 * j + 1], pos[4 * i + 2] - pos[4 * j + 2]};
    min_image(b, v);
    const double rs = rsq_of(v);
    return rs < rlistsq[type[i] * ntypes + type[j]];
}

}  // namespace

extern "C" {

// ---- version / identity
int orc_version() { return 3; }

// ---- threads used by every parallel phase (1 = the scalar oracle)
int orc_set_threads(int n)
{
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
    return omp_get_max_threads();
#else
    (void)n;
    return 1;
#endif
}

// ---- parameter construction (the dict constructors), in param_type field order
// PLJ in: {epsilon, sigma, attraction_scale_factor} -> {sigma_6, epsilon_x_4, lambda, rwcasq}
// EYUK in: {epsilon, kappa, delta} -> same
// HERTZ in: {epsilon} -> same
// COLLOID in: {A, a_1, a_2, sigma} -> {A, a_1, a_2, sigma_3}
// DPD in: {A, gamma, s} -> same
int orc_pair_params(int kind, const double* in, double* out)
{
    switch (kind) {
    case PAIR_PLJ: {
        const double s2 = in[1] * in[1];
        out[0] = s2 * (s2 * s2);
        out[1] = 4.0 * in[0];
        out[2] = in[2];
        out[3] = std::pow(2.0, 1.0 / 3.0) * s2;
        return 0;
    }
    case PAIR_EYUK: out[0] = in[0]; out[1] = in[1]; out[2] = in[2]; return 0;
    case PAIR_HERTZ: out[0] = in[0]; return 0;
    case PAIR_COLLOID: out[0] = in[0]; out[1] = in[1]; out[2] = in[2]; out[3] = in[3] * in[3] * in[3]; return 0;
    case PAIR_DPD: out[0] = in[0]; out[1] = in[1]; out[2] = in[2]; return 0;
    default: return -1;
    }
}

// Quartic in: {k, r_0, b_1, b_2, U_0, sigma, epsilon, delta}
// DoubleWell in: {r_0, r_1, U_1, U_tilt} -> {r_1, r_1 - r_0, U_1, U_tilt}
int orc_bond_params(int kind, const double* in, double* out)
{
    switch (kind) {
    case BOND_QUARTIC: {
        const double s2 = in[5] * in[5];
        out[0] = in[0]; out[1] = in[1]; out[2] = in[2]; out[3] = in[3]; out[4] = in[4];
        out[5] = s2 * (s2 * s2);
        out[6] = 4.0 * in[6];
        out[7] = in[7];
        return 0;
    }
    case BOND_DOUBLEWELL:
        out[0] = in[1]; out[1] = in[1] - in[0]; out[2] = in[2]; out[3] = in[3];
        return 0;
    case BOND_IMAGE_HARMONIC:
        out[0] = in[0]; out[1] = in[1];
        return 0;
    default: return -1;
    }
}

int orc_pair_eval(int kind, const double* p, double rsq, double rcutsq, int shift, double* f, double* e)
{
    double ff = 0.0, ee = 0.0;
    const bool ok = eval_pair(kind, p, rsq, rcutsq, shift != 0, ff, ee);
    *f = ok ? ff : 0.0;
    *e = ok ? ee : 0.0;
    return ok ? 1 : 0;
}

int orc_bond_eval(int kind, const double* p, double rsq, double* f, double* e)
{
    double ff = 0.0, ee = 0.0;
    const bool ok = eval_bond(kind, p, rsq, ff, ee);
    *f = ff;
    *e = ee;
    return ok ? 1 : 0;
}

// flow: kind 0 = ConstantFlow {Ux,Uy,Uz}; kind 1 = ParabolicFlow {mean_velocity, separation}
void orc_flow(int kind, const double* fp, const double* r, double* u)
{
    if (kind == 0) {
        u[0] = fp[0]; u[1] = fp[1]; u[2] = fp[2];
    } else {
        const double umax = 1.5 * fp[0];
        const double half = 0.5 * fp[1];
        const double yr = r[1] / half;
        u[0] = umax * (1.0 - yr * yr);
        u[1] = 0.0;
        u[2] = 0.0;
    }
}

void orc_philox4x32_10(const uint32_t* ctr, const uint32_t* key, uint32_t* out) { philox(ctr, key, out); }

void orc_uniform3(int id, uint64_t timestep, uint32_t seed, uint32_t tag, double lo, double hi, double* r)
{
    uniform3((uint8_t)id, timestep, seed, tag, lo, hi, r);
}

// ---- neighbour list (CSR output: start[N+1], idx[], each row ascending)
// Brute force O(N^2). rlistsq[ti*ntypes+tj] = (r_cut + r_buff)^2, or 0 to skip.
// Returns the number of entries written, or -(needed) if cap is too small.
long orc_nlist_brute(int N, const double* pos, const int32_t* type, int ntypes, const double* L,
                     const double* rlistsq, const int32_t* ex_start, const int32_t* ex_idx,
                     int32_t* start, int32_t* idx, long cap)
{
    const Box b = make_box(L);
    const Excl ex{ex_start, ex_idx};
    long n = 0;
    for (int i = 0; i < N; ++i) {
        start[i] = (int32_t)std::min<long>(n, cap);
        for (int j = 0; j < N; ++j) {
            if (j == i) continue;
            if (!listed(b, pos, type, ntypes, rlistsq, i, j)) continue;
            if (excluded(ex, i, j)) continue;
            if (n < cap) idx[n] = j;
            ++n;
        }
    }
    start[N] = (int32_t)std::min<long>(n, cap);
    return n <= cap ? n : -n;
}

// Cell-list build, same contract as orc_nlist_brute (cells of width >= r_list_max).
// Parallel over particles: count pass, prefix sum, write pass; rows ascending.
long orc_nlist_cell(int N, const double* pos, const int32_t* type, int ntypes, const double* L,
                    const double* rlistsq, const int32_t* ex_start, const int32_t* ex_idx,
                    int32_t* start, int32_t* idx, long cap)
{
    const Box b = make_box(L);
    const Excl ex{ex_start, ex_idx};
    double rmax = 0.0;
    for (int t = 0; t < ntypes * ntypes; ++t) rmax = std::max(rmax, std::sqrt(rlistsq[t]));
    int dim[3];
    for (int d = 0; d < 3; ++d) {
        dim[d] = rmax > 0.0 ? (int)std::floor(L[d] / rmax) : 1;
        if (dim[d] < 3) dim[d] = 1;  // too few cells: scan everything along d
    }
    const int ncell = dim[0] * dim[1] * dim[2];
    std::vector<int> cell_of(N), head(ncell + 1, 0), order(N);
    for (int i = 0; i < N; ++i) {
        int c[3];
        for (int d = 0; d < 3; ++d) {
            const double f = (pos[4 * i + d] - b.lo[d]) * b.Linv[d];
            int ci = (int)std::floor(f * dim[d]);
            ci = ((ci % dim[d]) + dim[d]) % dim[d];
            c[d] = ci;
        }
        cell_of[i] = (c[2] * dim[1] + c[1]) * dim[0] + c[0];
        head[cell_of[i] + 1]++;
    }
    for (int c = 0; c < ncell; ++c) head[c + 1] += head[c];
    {
        std::vector<int> fill(head.begin(), head.end() - 1);
        for (int i = 0; i < N; ++i) order[fill[cell_of[i]]++] = i;
    }
    const int rx = dim[0] >= 3 ? 1 : 0, ry = dim[1] >= 3 ? 1 : 0, rz = dim[2] >= 3 ? 1 : 0;
    auto gather_row = [&](int i, std::vector<int>& row) {
        row.clear();
        const int c = cell_of[i];
        const int cx = c % dim[0], cy = (c / dim[0]) % dim[1], cz = c / (dim[0] * dim[1]);
        for (int oz = -rz; oz <= rz; ++oz)
            for (int oy = -ry; oy <= ry; ++oy)
                for (int ox = -rx; ox <= rx; ++ox) {
                    const int nx = (cx + ox + dim[0]) % dim[0];
                    const int ny = (cy + oy + dim[1]) % dim[1];
                    const int nz = (cz + oz + dim[2]) % dim[2];
                    const int nc = (nz * dim[1] + ny) * dim[0] + nx;
                    for (int s = head[nc]; s < head[nc + 1]; ++s) {
                        const int j = order[s];
                        if (j == i) continue;
                        if (!listed(b, pos, type, ntypes, rlistsq, i, j)) continue;
                        if (excluded(ex, i, j)) continue;
                        row.push_back(j);
                    }
                }
        std::sort(row.begin(), row.end());
        row.erase(std::unique(row.begin(), row.end()), row.end());
    };
    std::vector<long> cnt(N + 1, 0);
#ifdef _OPENMP
#pragma omp parallel
#endif
    {
        std::vector<int> row;
#ifdef _OPENMP
#pragma omp for schedule(dynamic, 512)
#endif
        for (int i = 0; i < N; ++i) {
            gather_row(i, row);
            cnt[i + 1] = (long)row.size();
        }
    }
    for (int i = 0; i < N; ++i) cnt[i + 1] += cnt[i];
    if (cnt[N] > cap) return -cnt[N];
    for (int i = 0; i <= N; ++i) start[i] = (int32_t)cnt[i];
#ifdef _OPENMP
#pragma omp parallel
#endif
    {
        std::vector<int> row;
#ifdef _OPENMP
#pragma omp for schedule(dynamic, 512)
#endif
        for (int i = 0; i < N; ++i) {
            gather_row(i, row);
            std::copy(row.begin(), row.end(), idx + cnt[i]);
        }
    }
    return cnt[N];
}

// ---- pair forces over a CSR full list.
// params[(ti*ntypes+tj)*pstride ...], rcutsq / ronsq per type pair.
// Outputs are OVERWRITTEN: force[N*3], energy[N], virial[N*6] (xx,xy,xz,yy,yz,zz).
void orc_pair_forces(int N, const double* pos, const int32_t* type, int ntypes, const double* L,
                     const int32_t* start, const int32_t* idx, int kind, const double* params, int pstride,
                     const double* rcutsq, const double* ronsq, int mode, double* force, double* energy,
                     double* virial, double fcap)
{
    const Box b = make_box(L);
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 256)
#endif
    for (int i = 0; i < N; ++i) {
        double F[3] = {0, 0, 0}, U = 0.0, W[6] = {0, 0, 0, 0, 0, 0};
        const int ti = type[i];
        for (int k = start[i]; k < start[i + 1]; ++k) {
            const int j = idx[k];
            double v[3] = {pos[4 * i] - pos[4 * j], pos[4 * i + 1] - pos[4 * j + 1], pos[4 * i + 2] - pos[4 * j + 2]};
            min_image(b, v);
            const double rs = rsq_of(v);
            const int tp = ti * ntypes + type[j];
            const double rc2 = rcutsq[tp];
            const double ro2 = ronsq ? ronsq[tp] : 0.0;
            bool shift = (mode == MODE_SHIFT);
            if (mode == MODE_XPLOR && ro2 > rc2) shift = true;
            double fdr = 0.0, e = 0.0;
            if (!eval_pair(kind, params + (size_t)tp * pstride, rs, rc2, shift, fdr, e)) continue;
            if (mode == MODE_XPLOR && rs >= ro2 && rs < rc2) {
                // XPLOR smoothing S(r) between r_on and r_cut
                const double den = (rc2 - ro2) * (rc2 - ro2) * (rc2 - ro2);
                const double a = rs - rc2;
                const double s = a * a * (rc2 + 2.0 * rs - 3.0 * ro2) / den;
                const double dsdr_r = 12.0 * (rs - ro2) * a / den;
                fdr = s * fdr - dsdr_r * e;
                e = e * s;
            }
            // optional per-pair force cap (overlap relaxation of generated systems)
            if (fcap > 0.0 && fdr * fdr * rs > fcap * fcap) fdr = std::copysign(fcap / std::sqrt(rs), fdr);
            F[0] += v[0] * fdr;
            F[1] += v[1] * fdr;
            F[2] += v[2] * fdr;
            U += 0.5 * e;
            const double h = 0.5 * fdr;
            W[0] += h * v[0] * v[0];
            W[1] += h * v[0] * v[1];
            W[2] += h * v[0] * v[2];
            W[3] += h * v[1] * v[1];
            W[4] += h * v[1] * v[2];
            W[5] += h * v[2] * v[2];
        }
        for (int d = 0; d < 3; ++d) force[3 * i + d] = F[d];
        energy[i] = U;
        if (virial)
            for (int c = 0; c < 6; ++c) virial[6 * i + c] = W[c];
    }
}

// ---- DPD with general weight, full thermostat (src/DPDPairEvaluatorGeneralWeight.h:165-255):
// conservative A (1/r - 1/r_cut), dissipative -gamma w(r) (dx . dv) / r^2 with
// w = (1 - r/r_cut)^s, random sqrt(6 kT gamma / dt) sqrt(w) alpha / r with alpha
// uniform in (-1, 1) drawn once per pair from the stream
// (RNG id 200, timestep, seed) at counter {0, min(tag_i, tag_j), max(...), 0}
// (the reference's Seed(id, timestep, seed) + Counter(i, j) at :227-233). Energy
// and virial: conservative part only (:203-204, :249-250). params [ntypes^2][4]:
// A, gamma, s, -; vel [N][4] (v, mass).
double dpd_alpha(uint64_t timestep, uint32_t seed, uint32_t ti, uint32_t tj)
{
    uint32_t key[2];
    stream_key(RNG_DPD, timestep, seed, key);
    const uint32_t oi = ti < tj ? ti : tj, oj = ti < tj ? tj : ti;
    uint32_t c[4] = {0u, oi, oj, 0u}, o[4];
    philox(c, key, o);
    const uint64_t u = ((uint64_t)o[0] << 32) | o[1];
    return -1.0 + 2.0 * u64_to_open01(u);
}

void orc_dpd_forces(int N, const double* pos, const double* vel, const int32_t* type, const uint32_t* tag,
                    int ntypes, const double* L, const int32_t* start, const int32_t* idx, const double* params,
                    const double* rcutsq, double kT, double dt, uint64_t timestep, uint32_t seed, double* force,
                    double* energy, double* virial)
{
    const Box b = make_box(L);
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 256)
#endif
    for (int i = 0; i < N; ++i) {
        double F[3] = {0, 0, 0}, U = 0.0, W[6] = {0, 0, 0, 0, 0, 0};
        const int ti = type[i];
        for (int k = start[i]; k < start[i + 1]; ++k) {
            const int j = idx[k];
            double v[3] = {pos[4 * i] - pos[4 * j], pos[4 * i + 1] - pos[4 * j + 1], pos[4 * i + 2] - pos[4 * j + 2]};
            min_image(b, v);
            const double rs = rsq_of(v);
            const int tp = ti * ntypes + type[j];
            const double rc2 = rcutsq[tp];
            if (!(rs < rc2)) continue;
            const double* p = params + (size_t)tp * 4;
            const double A = p[0], gamma = p[1], s = p[2];
            const double rinv = 1.0 / std::sqrt(rs);
            const double r = 1.0 / rinv;
            const double rcinv = 1.0 / std::sqrt(rc2);
            const double rc = 1.0 / rcinv;
            const double dot = v[0] * (vel[4 * i] - vel[4 * j]) + v[1] * (vel[4 * i + 1] - vel[4 * j + 1]) +
                               v[2] * (vel[4 * i + 2] - vel[4 * j + 2]);
            const double fc = A * (rinv - rcinv);
            // r < r_cut, but 1 - r / r_cut can round below 0 right at the cutoff, where the
            // reference's pow would return NaN: clamped to 0
            const double wR = std::pow(std::fmax(1.0 - r * rcinv, 0.0), 0.5 * s) * rinv;
            const double alpha = dpd_alpha(timestep, seed, tag[i], tag[j]);
            const double fdr = fc - gamma * wR * wR * dot + std::sqrt(6.0 * kT * gamma / dt) * wR * alpha;
            const double e = A * (rc - r) - 0.5 * A * rcinv * (rc2 - rs);
            F[0] += v[0] * fdr;
            F[1] += v[1] * fdr;
            F[2] += v[2] * fdr;
            U += 0.5 * e;
            const double h = 0.5 * fc;
            W[0] += h * v[0] * v[0];
            W[1] += h * v[0] * v[1];
            W[2] += h * v[0] * v[2];
            W[3] += h * v[1] * v[1];
            W[4] += h * v[1] * v[2];
            W[5] += h * v[2] * v[2];
        }
        for (int d = 0; d < 3; ++d) force[3 * i + d] = F[d];
        energy[i] = U;
        if (virial)
            for (int c = 0; c < 6; ++c) virial[6 * i + c] = W[c];
    }
}

// ---- bond forces. bonds[2*b] = {a, b} particle indices; btype[b]; params[t*8...].
// ACCUMULATES into force/energy/virial. Returns 0, or 1 + index of the first
// bond whose evaluator refused (r_0 == 0 / r_1 == r_0), like the device flag.
long orc_bond_forces(int N, const double* pos, const double* L, long nbonds, const int32_t* bonds,
                     const int32_t* btype, int kind, const double* params, int pstride, double* force,
                     double* energy, double* virial)
{
    (void)N;
    const Box b = make_box(L);
    for (long k = 0; k < nbonds; ++k) {
        const int ia = bonds[2 * k], ib = bonds[2 * k + 1];
        double v[3] = {pos[4 * ib] - pos[4 * ia], pos[4 * ib + 1] - pos[4 * ia + 1], pos[4 * ib + 2] - pos[4 * ia + 2]};
        min_image(b, v);
        const double rs = rsq_of(v);
        double fdr = 0.0, e = 0.0;
        if (!eval_bond(kind, params + (size_t)btype[k] * pstride, rs, fdr, e)) return 1 + k;
        e *= 0.5;
        const double h = 0.5 * fdr;
        const double w[6] = {h * v[0] * v[0], h * v[0] * v[1], h * v[0] * v[2], h * v[1] * v[1], h * v[1] * v[2], h * v[2] * v[2]};
        for (int d = 0; d < 3; ++d) {
            force[3 * ib + d] += fdr * v[d];
            force[3 * ia + d] -= fdr * v[d];
        }
        energy[ia] += e;
        energy[ib] += e;
        if (virial)
            for (int c = 0; c < 6; ++c) {
                virial[6 * ia + c] += w[c];
                virial[6 * ib + c] += w[c];
            }
    }
    return 0;
}

// ---- bond forces from a per-particle table (each bond listed on both ends):
// bt_start[N+1], bt_partner[], bt_type[]. For particle i and partner j,
// dx = x_i - x_j (minimum image) and F_i += dx * f/r, U_i += U/2, W_i += dx dx f/(2r).
// ACCUMULATES. Parallel over particles. Returns 0, or 1 + the first failing particle.
long orc_bond_forces_pp(int N, const double* pos, const double* L, const int32_t* bt_start,
                        const int32_t* bt_partner, const int32_t* bt_type, int kind, const double* params,
                        int pstride, double* force, double* energy, double* virial)
{
    const Box b = make_box(L);
    long fail = 0;
#ifdef _OPENMP
#pragma omp parallel for schedule(static) reduction(max : fail)
#endif
    for (int i = 0; i < N; ++i) {
        for (int k = bt_start[i]; k < bt_start[i + 1]; ++k) {
            const int j = bt_partner[k];
            double v[3] = {pos[4 * i] - pos[4 * j], pos[4 * i + 1] - pos[4 * j + 1], pos[4 * i + 2] - pos[4 * j + 2]};
            min_image(b, v);
            const double rs = rsq_of(v);
            double fdr = 0.0, e = 0.0;
            if (!eval_bond(kind, params + (size_t)bt_type[k] * pstride, rs, fdr, e)) {
                fail = std::max<long>(fail, 1 + i);
                continue;
            }
            for (int d = 0; d < 3; ++d) force[3 * i + d] += fdr * v[d];
            energy[i] += 0.5 * e;
            if (virial) {
                const double h = 0.5 * fdr;
                virial[6 * i + 0] += h * v[0] * v[0];
                virial[6 * i + 1] += h * v[0] * v[1];
                virial[6 * i + 2] += h * v[0] * v[2];
                virial[6 * i + 3] += h * v[1] * v[1];
                virial[6 * i + 4] += h * v[1] * v[2];
                virial[6 * i + 5] += h * v[2] * v[2];
            }
        }
    }
    return fail;
}

// ---- integrators. pos[N*4] (w ignored), vel[N*4] (w = mass), accel[N*3], image[N*3].
void orc_langevin_step1(int N, double* pos, int32_t* image, double* vel, const double* accel, const double* L,
                        double dt)
{
    const Box b = make_box(L);
#ifdef _OPENMP
#pragma omp parallel for schedule(static)
#endif
    for (int i = 0; i < N; ++i) {
        double x[3], v[3];
        for (int d = 0; d < 3; ++d) {
            x[d] = pos[4 * i + d];
            v[d] = vel[4 * i + d];
        }
        for (int d = 0; d < 3; ++d) x[d] += (v[d] + 0.5 * dt * accel[3 * i + d]) * dt;
        wrap(b, x, image + 3 * i);
        for (int d = 0; d < 3; ++d) v[d] += 0.5 * dt * accel[3 * i + d];
        for (int d = 0; d < 3; ++d) {
            pos[4 * i + d] = x[d];
            vel[4 * i + d] = v[d];
        }
    }
}

// gamma: per-type table (use_lambda == 0) or lambda * diameter[i].
void orc_langevin_step2(int N, const double* pos, const int32_t* type, double* vel, double* accel,
                        const double* net_force, const uint32_t* tag, const double* diameter,
                        const double* gamma, int use_lambda, double lambda, int flow_kind, const double* flow_p,
                        double kT, double dt, uint64_t timestep, uint32_t seed, int noiseless)
{
#ifdef _OPENMP
#pragma omp parallel for schedule(static)
#endif
    for (int i = 0; i < N; ++i) {
        const double g = use_lambda ? lambda * diameter[i] : gamma[type[i]];
        double u[3];
        orc_flow(flow_kind, flow_p, pos + 4 * i, u);
        double c = std::sqrt(6.0 * g * kT / dt);
        if (noiseless) c = 0.0;
        double R[3];
        uniform3(RNG_LANGEVIN, timestep, seed, tag[i], -c, c, R);
        const double m = vel[4 * i + 3];
        const double minv = 1.0 / m;
        for (int d = 0; d < 3; ++d) {
            const double bd = R[d] - g * (vel[4 * i + d] - u[d]);
            const double a = (net_force[3 * i + d] + bd) * minv;
            vel[4 * i + d] += 0.5 * dt * a;
            accel[3 * i + d] = a;
        }
    }
}

void orc_brownian(int N, double* pos, int32_t* image, const int32_t* type, const double* net_force,
                  const uint32_t* tag, const double* diameter, const double* gamma, int use_lambda, double lambda,
                  int flow_kind, const double* flow_p, const double* L, double kT, double dt, uint64_t timestep,
                  uint32_t seed, int noiseless, double max_disp)
{
    const Box b = make_box(L);
#ifdef _OPENMP
#pragma omp parallel for schedule(static)
#endif
    for (int i = 0; i < N; ++i) {
        const double g = use_lambda ? lambda * diameter[i] : gamma[type[i]];
        double x[3] = {pos[4 * i], pos[4 * i + 1], pos[4 * i + 2]};
        double u[3];
        orc_flow(flow_kind, flow_p, x, u);
        double c = std::sqrt(6.0 * g * kT / dt);
        if (noiseless) c = 0.0;
        double R[3];
        uniform3(RNG_BROWNIAN, timestep, seed, tag[i], -c, c, R);
        for (int d = 0; d < 3; ++d) {
            double dd = (u[d] + (net_force[3 * i + d] + R[d]) / g) * dt;
            if (max_disp > 0.0) dd = std::fmin(std::fmax(dd, -max_disp), max_disp);
            x[d] += dd;
        }
        wrap(b, x, image + 3 * i);
        for (int d = 0; d < 3; ++d) pos[4 * i + d] = x[d];
    }
}

// ---- harmonic barriers (src/HarmonicBarrier.h:149-180: wrap each position into
// the box, then the evaluator with the type's (k, offset); the virial is not
// computed). geometry 0: src/PlanarBarrierEvaluator.h:36-47 (push -y above
// y = H + offset); 1: src/SphericalBarrierEvaluator.h:36-51 (push inward beyond
// r = R + offset). params[2 * type] = {k, offset}. Writes force[3N], energy[N].
// Returns 0, or -1 when the location fails the evaluator's valid(box)
// (PlanarBarrierEvaluator.h:50-56, SphericalBarrierEvaluator.h:54-61).
int orc_barrier_valid(int geometry, double location, const double* L)
{
    if (geometry == 0) return (location >= -0.5 * L[1] && location < 0.5 * L[1]) ? 0 : -1;
    const double two_R = 2.0 * location;
    // nearest plane distances of an orthorhombic box are its edge lengths
    return (location >= 0.0 && L[0] >= two_R && L[1] >= two_R && L[2] >= two_R) ? 0 : -1;
}

int orc_harmonic_barrier(int N, const double* pos, const int32_t* type, const double* L, int geometry,
                         double location, const double* params, double* force, double* energy)
{
    if (orc_barrier_valid(geometry, location, L)) return -1;
    const Box b = make_box(L);
    for (int i = 0; i < N; ++i) {
        double x[3] = {pos[4 * i], pos[4 * i + 1], pos[4 * i + 2]};
        int img[3] = {0, 0, 0};
        wrap(b, x, img);
        const double k = params[2 * type[i]], offset = params[2 * type[i] + 1];
        double f[3] = {0.0, 0.0, 0.0}, e = 0.0;
        if (geometry == 0) {
            const double dy = x[1] - (location + offset);
            if (dy > 0.0) {
                f[1] = -k * dy;
                e = -0.5 * f[1] * dy;
            }
        } else {
            const double r = std::sqrt(x[0] * x[0] + x[1] * x[1] + x[2] * x[2]);
            const double dr = r - (location + offset);
            if (dr > 0.0) {
                const double k_dr = k * dr;
                for (int d = 0; d < 3; ++d) f[d] = -(k_dr / r) * x[d];
                e = 0.5 * k_dr * dr;
            }
        }
        for (int d = 0; d < 3; ++d) force[3 * i + d] = f[d];
        energy[i] = e;
    }
    return 0;
}

// ---- wall potentials (src/WallEvaluatorLJ93.h:100-133, src/WallEvaluatorColloid.h:
// 118-183) applied through HOOMD's EvaluatorWalls (not in the tree; restated from
// its documented behaviour): for every wall, the vector from the nearest point of
// the wall surface to the particle and whether the particle is on the wall's
// active side; standard mode (r_extrap = 0): the shifted pair form of the
// distance d on the active side only; extrapolated mode (r_extrap > 0): that form
// for d >= r_extrap on the active side, else the linear continuation
// U(r_extrap) + F(r_extrap) (r_extrap - d_signed) with the constant force
// F(r_extrap) pushing towards the active side. Full energy per particle; virial
// F_a x_b. Walls are visited spheres, cylinders, planes.
//   params[4 * type]: LJ93 {sigma^3, A, -, -}; Colloid {c_1, c_2, a, -}
//   spheres  [ns][6]: r, origin xyz, inside, open
//   cylinders[nc][9]: r, origin xyz, unit axis xyz, inside, open
//   planes   [np][7]: origin xyz, unit normal xyz, open
enum WallKind { WALL_LJ93 = 0, WALL_COLLOID = 1 };

// energy-shifted evaluator at squared distance rsq; false when not evaluated
bool wall_eval(int kind, const double* p, double rsq, double rcutsq, double& fdr, double& e)
{
    if (kind == WALL_LJ93) {
        const double lj1 = (2.0 / 15.0) * p[1] * p[0] * p[0] * p[0];
        const double lj2 = p[1] * p[0];
        if (!(rsq < rcutsq) || lj1 == 0.0) return false;
        const double r2inv = 1.0 / rsq;
        const double r3inv = r2inv * std::sqrt(r2inv);
        const double r6inv = r3inv * r3inv;
        fdr = r2inv * r3inv * (9.0 * lj1 * r6inv - 3.0 * lj2);
        e = r3inv * (lj1 * r6inv - lj2);
        const double rc2inv = 1.0 / rcutsq;
        const double rc3inv = rc2inv * std::sqrt(rc2inv);
        const double rc6inv = rc3inv * rc3inv;
        e -= rc3inv * (lj1 * rc6inv - lj2);
        return true;
    }
    const double c1 = p[0], c2 = p[1], a = p[2];
    if (!(rsq < rcutsq) || c1 == 0.0 || !(a > 0.0)) return false;
    auto potential = [&](double r2, bool force, double& f) {
        const double r = std::sqrt(r2);
        const double arinv = a / r;
        const double rma = 1.0 / (r - a), rpa = 1.0 / (r + a);
        const double r2ma2 = rma * rpa;
        const double rma2 = rma * rma, rma6 = rma2 * rma2 * rma2;
        const double rpa2 = rpa * rpa, rpa6 = rpa2 * rpa2 * rpa2;
        if (force) {
            const double arinv8 = 8.0 * arinv;
            f = 6.0 * c1 * ((arinv8 - 1.0) * rma2 * rma6 + (arinv8 + 1.0) * rpa2 * rpa6);
            f -= c2 * (4.0 * a * a * arinv * r2ma2 * r2ma2);
        }
        const double a7 = 7.0 * a;
        double en = c1 * ((a7 - r) * rma * rma6 + (a7 + r) * rpa * rpa6);
        en -= c2 * (2.0 * a * r * r2ma2 + std::log(rpa / rma));
        return en;
    };
    double dummy = 0.0;
    e = potential(rsq, true, fdr);
    e -= potential(rcutsq, false, dummy);
    return true;
}

// dr = particle - nearest wall point (the reference's dr = -drv), inside flag
void wall_sphere(const double* w, const double* x, double* dr, bool& inside)
{
    const double t[3] = {x[0] - w[1], x[1] - w[2], x[2] - w[3]};
    const double rxyz = std::sqrt(t[0] * t[0] + t[1] * t[1] + t[2] * t[2]);
    const double R = w[0];
    const bool win = w[4] != 0.0, open = w[5] != 0.0;
    if (rxyz > 0.0) {
        inside = (win ? rxyz < R : rxyz > R) || (rxyz == R && !open);
        const double s = R / rxyz;
        for (int d = 0; d < 3; ++d) dr[d] = t[d] - t[d] * s;
    } else {
        // at the centre every surface point is nearest: the one along +x
        inside = win;
        dr[0] = -R;
        dr[1] = dr[2] = 0.0;
    }
}

void wall_cylinder(const double* w, const double* x, double* dr, bool& inside)
{
    const double t[3] = {x[0] - w[1], x[1] - w[2], x[2] - w[3]};
    const double* ax = w + 4;
    const double along = t[0] * ax[0] + t[1] * ax[1] + t[2] * ax[2];
    const double perp[3] = {t[0] - along * ax[0], t[1] - along * ax[1], t[2] - along * ax[2]};
    const double rxy = std::sqrt(perp[0] * perp[0] + perp[1] * perp[1] + perp[2] * perp[2]);
    const double R = w[0];
    const bool win = w[7] != 0.0, open = w[8] != 0.0;
    if (rxy > 0.0) {
        inside = (win ? rxy < R : rxy > R) || (rxy == R && !open);
        const double s = R / rxy;
        for (int d = 0; d < 3; ++d) dr[d] = perp[d] - perp[d] * s;
    } else {
        // on the axis: the surface point along the first direction normal to the axis
        inside = win;
        double u[3];
        if (std::fabs(ax[0]) < 0.9) {
            u[0] = 0.0; u[1] = ax[2]; u[2] = -ax[1];
        } else {
            u[0] = -ax[2]; u[1] = 0.0; u[2] = ax[0];
        }
        const double un = std::sqrt(u[0] * u[0] + u[1] * u[1] + u[2] * u[2]);
        for (int d = 0; d < 3; ++d) dr[d] = -R * u[d] / un;
    }
}

void wall_plane(const double* w, const double* x, double* dr, bool& inside)
{
    const double* n = w + 3;
    const double d = (x[0] - w[0]) * n[0] + (x[1] - w[1]) * n[1] + (x[2] - w[2]) * n[2];
    const bool open = w[6] != 0.0;
    inside = d > 0.0 || (d == 0.0 && !open);
    for (int k = 0; k < 3; ++k) dr[k] = d * n[k];
}

// one wall's contribution; nrm = the wall normal used when the particle lies on the surface
void wall_apply(int kind, const double* p, double rcutsq, double rextrap, const double* dr, bool inside,
                const double* nrm, double* F, double& U)
{
    const double rsq = dr[0] * dr[0] + dr[1] * dr[1] + dr[2] * dr[2];
    if (rextrap > 0.0) {
        const double rextrapsq = rextrap * rextrap;
        if (inside && rsq >= rextrapsq) {
            double fdr = 0.0, e = 0.0;
            if (wall_eval(kind, p, rsq, rcutsq, fdr, e)) {
                for (int d = 0; d < 3; ++d) F[d] += dr[d] * fdr;
                U += e;
            }
            return;
        }
        // unit vector from the wall towards the active side
        double u[3];
        const double r = std::sqrt(rsq);
        if (rsq > 0.0) {
            const double sgn = inside ? 1.0 : -1.0;
            for (int d = 0; d < 3; ++d) u[d] = sgn * dr[d] / r;
        } else {
            for (int d = 0; d < 3; ++d) u[d] = nrm[d];
        }
        const double rp = inside ? rextrap - r : rextrap + r;  // r_extrap - signed distance
        double fdr = 0.0, e = 0.0;
        if (wall_eval(kind, p, rextrapsq, rcutsq, fdr, e)) {
            const double fmag = fdr * rextrap;
            for (int d = 0; d < 3; ++d) F[d] += u[d] * fmag;
            U += e + fmag * rp;
        }
        return;
    }
    if (!inside) return;
    double fdr = 0.0, e = 0.0;
    if (wall_eval(kind, p, rsq, rcutsq, fdr, e)) {
        for (int d = 0; d < 3; ++d) F[d] += dr[d] * fdr;
        U += e;
    }
}

void orc_wall_forces(int N, const double* pos, const int32_t* type, int kind, const double* params,
                     const double* rcut, const double* rextrap, int ns, const double* spheres, int nc,
                     const double* cylinders, int np, const double* planes, double* force, double* energy,
                     double* virial)
{
    for (int i = 0; i < N; ++i) {
        const double x[3] = {pos[4 * i], pos[4 * i + 1], pos[4 * i + 2]};
        const int t = type[i];
        const double* p = params + 4 * t;
        const double rcutsq = rcut[t] * rcut[t];
        double F[3] = {0.0, 0.0, 0.0}, U = 0.0;
        double dr[3], nrm[3];
        bool inside = false;
        for (int k = 0; k < ns; ++k) {
            const double* w = spheres + 6 * k;
            wall_sphere(w, x, dr, inside);
            // on the surface: towards the centre for an inside wall, outwards otherwise
            const double t0[3] = {x[0] - w[1], x[1] - w[2], x[2] - w[3]};
            const double tn = std::sqrt(t0[0] * t0[0] + t0[1] * t0[1] + t0[2] * t0[2]);
            for (int d = 0; d < 3; ++d) nrm[d] = tn > 0.0 ? (w[4] != 0.0 ? -t0[d] / tn : t0[d] / tn) : 0.0;
            wall_apply(kind, p, rcutsq, rextrap[t], dr, inside, nrm, F, U);
        }
        for (int k = 0; k < nc; ++k) {
            const double* w = cylinders + 9 * k;
            wall_cylinder(w, x, dr, inside);
            const double t0[3] = {x[0] - w[1], x[1] - w[2], x[2] - w[3]};
            const double along = t0[0] * w[4] + t0[1] * w[5] + t0[2] * w[6];
            const double pp[3] = {t0[0] - along * w[4], t0[1] - along * w[5], t0[2] - along * w[6]};
            const double pn = std::sqrt(pp[0] * pp[0] + pp[1] * pp[1] + pp[2] * pp[2]);
            for (int d = 0; d < 3; ++d) nrm[d] = pn > 0.0 ? (w[7] != 0.0 ? -pp[d] / pn : pp[d] / pn) : 0.0;
            wall_apply(kind, p, rcutsq, rextrap[t], dr, inside, nrm, F, U);
        }
        for (int k = 0; k < np; ++k) {
            const double* w = planes + 7 * k;
            wall_plane(w, x, dr, inside);
            wall_apply(kind, p, rcutsq, rextrap[t], dr, inside, w + 3, F, U);
        }
        for (int d = 0; d < 3; ++d) force[3 * i + d] = F[d];
        energy[i] = U;
        if (virial) {
            double* v = virial + 6 * i;
            v[0] = F[0] * x[0];
            v[1] = F[0] * x[1];
            v[2] = F[0] * x[2];
            v[3] = F[1] * x[1];
            v[4] = F[1] * x[2];
            v[5] = F[2] * x[2];
        }
    }
}

// param_type dict constructors (src/WallEvaluatorLJ93.h:31-45, src/WallEvaluatorColloid.h:31-53)
// LJ93 values {A, sigma} -> {sigma^3, A}; Colloid values {A, a, sigma} -> {c_1, c_2, a}
int orc_wall_params(int kind, const double* v, double* out)
{
    out[0] = out[1] = out[2] = out[3] = 0.0;
    if (kind == WALL_LJ93) {
        const double A = v[0], sigma = v[1];
        out[0] = sigma * sigma * sigma;
        out[1] = A;
        return 0;
    }
    if (kind == WALL_COLLOID) {
        const double A = v[0], a = v[1], sigma = v[2];
        const double sigma_3 = sigma * sigma * sigma;
        out[0] = A * sigma_3 * sigma_3 / 7560.0;
        out[1] = A / 6.0;
        out[2] = a;
        return 0;
    }
    return -1;
}

// ---- velocity field (src/VelocityFieldCompute.h:196-205 addParticleToBin and
// :292-344 binParticles, src/BinningOperation.h:71-87 bin1D,
// src/CartesianBinningOperation.h:27-52, src/CylindricalBinningOperation.h:27-76):
// each member's position wrapped into the box, binned, its momentum m v (turned
// into (v_r, v_theta, v_z) for cylindrical bins) and mass summed per bin in
// member order; velocity = momentum / mass (0 in an empty bin). kind 0
// Cartesian, 1 cylindrical; num_bins 0 ignores a coordinate. members: index
// list or NULL for all N. Outputs mass[nb], momentum[3 nb], velocity[3 nb].
static bool bin1d(double x, double lo, double hi, unsigned n, unsigned& b)
{
    const int k = (int)std::floor(((x - lo) / (hi - lo)) * n);
    if (k >= 0 && k < (int)n) {
        b = (unsigned)k;
        return true;
    }
    return false;
}

void orc_velocity_field(int N, const double* pos, const double* vel, const double* L, const int32_t* members,
                        int n_members, int kind, const uint32_t* num_bins, const double* lo, const double* hi,
                        double* mass, double* momentum, double* velocity)
{
    const Box b = make_box(L);
    unsigned nb[3];
    bool use[3];
    for (int d = 0; d < 3; ++d) {
        use[d] = num_bins[d] > 0;
        nb[d] = use[d] ? num_bins[d] : 1u;
    }
    const size_t total = (size_t)nb[0] * nb[1] * nb[2];
    for (size_t k = 0; k < total; ++k) {
        mass[k] = 0.0;
        momentum[3 * k] = momentum[3 * k + 1] = momentum[3 * k + 2] = 0.0;
    }
    const int n = members ? n_members : N;
    for (int m = 0; m < n; ++m) {
        const int i = members ? members[m] : m;
        double x[3] = {pos[4 * i], pos[4 * i + 1], pos[4 * i + 2]};
        int img[3] = {0, 0, 0};
        wrap(b, x, img);
        const double mi = vel[4 * i + 3];
        const double p[3] = {vel[4 * i] * mi, vel[4 * i + 1] * mi, vel[4 * i + 2] * mi};
        unsigned bin[3] = {0, 0, 0};
        double t[3];
        if (kind == 0) {
            bool ok = true;
            for (int d = 0; d < 3 && ok; ++d)
                if (use[d]) ok = bin1d(x[d], lo[d], hi[d], nb[d], bin[d]);
            if (!ok) continue;
            t[0] = p[0];
            t[1] = p[1];
            t[2] = p[2];
        } else {
            if (use[2] && !bin1d(x[2], lo[2], hi[2], nb[2], bin[2])) continue;
            if (use[1]) {
                double theta = std::atan2(x[1], x[0]);
                if (theta < 0.0) theta += 2.0 * M_PI;
                if (!bin1d(theta, lo[1], hi[1], nb[1], bin[1])) continue;
            }
            const double r = std::sqrt(x[0] * x[0] + x[1] * x[1]);
            if (use[0] && !bin1d(r, lo[0], hi[0], nb[0], bin[0])) continue;
            double c = 1.0, s = 0.0;
            if (r > 0.0) {
                c = x[0] / r;
                s = x[1] / r;
            }
            t[0] = c * p[0] + s * p[1];
            t[1] = -s * p[0] + c * p[1];
            t[2] = p[2];
        }
        const size_t k = (size_t)bin[2] + nb[2] * ((size_t)bin[1] + nb[1] * (size_t)bin[0]);
        mass[k] += mi;
        for (int d = 0; d < 3; ++d) momentum[3 * k + d] += t[d];
    }
    for (size_t k = 0; k < total; ++k)
        for (int d = 0; d < 3; ++d) velocity[3 * k + d] = mass[k] > 0.0 ? momentum[3 * k + d] / mass[k] : 0.0;
}

// ---- image-unwrapped bonds (src/ImagePotentialBond.h:57-204): for bond (a, b)
// the vector dx = (x_b - x_a) + (img_b - img_a) L, F_b += f/r dx, F_a -= f/r dx,
// half the energy and the virial dx (x) dx f/(2r) to each particle, bonds in list
// order. ACCUMULATES. Returns 0, or 1 + the first refused bond.
long orc_image_bond_forces(int N, const double* pos, const int32_t* image, const double* L, long nbonds,
                           const int32_t* bonds, const int32_t* btype, int kind, const double* params, int pstride,
                           double* force, double* energy, double* virial)
{
    (void)N;
    long bad = 0;
    for (long k = 0; k < nbonds; ++k) {
        const int ia = bonds[2 * k], ib = bonds[2 * k + 1];
        double dx[3];
        for (int d = 0; d < 3; ++d)
            dx[d] = (pos[4 * ib + d] - pos[4 * ia + d]) + (double)(image[3 * ib + d] - image[3 * ia + d]) * L[d];
        const double rsq = dx[0] * dx[0] + dx[1] * dx[1] + dx[2] * dx[2];
        double fdr = 0.0, e = 0.0;
        if (!eval_bond(kind, params + (size_t)btype[k] * pstride, rsq, fdr, e)) {
            if (!bad) bad = k + 1;
            continue;
        }
        e *= 0.5;
        const double h = 0.5 * fdr;
        const double w[6] = {dx[0] * dx[0] * h, dx[0] * dx[1] * h, dx[0] * dx[2] * h,
                             dx[1] * dx[1] * h, dx[1] * dx[2] * h, dx[2] * dx[2] * h};
        for (int d = 0; d < 3; ++d) {
            force[3 * ib + d] += fdr * dx[d];
            force[3 * ia + d] -= fdr * dx[d];
        }
        energy[ib] += e;
        energy[ia] += e;
        if (virial)
            for (int c = 0; c < 6; ++c) {
                virial[6 * ib + c] += w[c];
                virial[6 * ia + c] += w[c];
            }
    }
    return bad;
}

// ---- the same per particle (each bond on both ends, the MD loop's table):
// dx = (x_i - x_j) + (img_i - img_j) L, F_i += dx f/r, U_i += U/2, W_i += dx dx f/2r
// (src/ImagePotentialBond.h:144-190 seen from each end)
long orc_image_bond_forces_pp(int N, const double* pos, const int32_t* image, const double* L,
                              const int32_t* bt_start, const int32_t* bt_partner, const int32_t* bt_type, int kind,
                              const double* params, int pstride, double* force, double* energy, double* virial)
{
    long fail = 0;
#ifdef _OPENMP
#pragma omp parallel for schedule(static) reduction(max : fail)
#endif
    for (int i = 0; i < N; ++i) {
        for (int k = bt_start[i]; k < bt_start[i + 1]; ++k) {
            const int j = bt_partner[k];
            double v[3];
            for (int d = 0; d < 3; ++d)
                v[d] = (pos[4 * i + d] - pos[4 * j + d]) + (double)(image[3 * i + d] - image[3 * j + d]) * L[d];
            const double rs = rsq_of(v);
            double fdr = 0.0, e = 0.0;
            if (!eval_bond(kind, params + (size_t)bt_type[k] * pstride, rs, fdr, e)) {
                fail = std::max<long>(fail, 1 + i);
                continue;
            }
            for (int d = 0; d < 3; ++d) force[3 * i + d] += fdr * v[d];
            energy[i] += 0.5 * e;
            if (virial) {
                const double h = 0.5 * fdr;
                virial[6 * i + 0] += h * v[0] * v[0];
                virial[6 * i + 1] += h * v[0] * v[1];
                virial[6 * i + 2] += h * v[0] * v[2];
                virial[6 * i + 3] += h * v[1] * v[1];
                virial[6 * i + 4] += h * v[1] * v[2];
                virial[6 * i + 5] += h * v[2] * v[2];
            }
        }
    }
    return fail;
}

// ---- maximum squared displacement since the last list build
double orc_max_disp2(int N, const double* pos, const double* pos_build, const double* L)
{
    const Box b = make_box(L);
    double m = 0.0;
#ifdef _OPENMP
#pragma omp parallel for schedule(static) reduction(max : m)
#endif
    for (int i = 0; i < N; ++i) {
        double v[3] = {pos[4 * i] - pos_build[4 * i], pos[4 * i + 1] - pos_build[4 * i + 1], pos[4 * i + 2] - pos_build[4 * i + 2]};
        min_image(b, v);
        m = std::max(m, rsq_of(v));
    }
    return m;
}

}  // extern "C"
