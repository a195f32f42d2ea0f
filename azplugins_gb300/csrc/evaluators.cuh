// evaluators.cuh -- azplugins pair and bond potentials as device functors,
// templated on the arithmetic type (float for AZP_FP32, double for AZP_FP64).
//
// Each pair potential works on an 8-value "kernel record" derived on the host
// from the reference's param_type fields (prepare_*), so per-pair work holds no
// parameter arithmetic. The formulas are those of the reference evaluators:
//   PerturbedLennardJones  src/PairEvaluatorPerturbedLennardJones.h:117-155
//   ExpandedYukawa         src/PairEvaluatorExpandedYukawa.h:92-115
//   Hertz                  src/PairEvaluatorHertz.h:93-110
//   Colloid                src/PairEvaluatorColloid.h:101-269
//   Quartic bond           src/BondEvaluatorQuartic.h:129-200
//   DoubleWell bond        src/BondEvaluatorDoubleWell.h:96-113
#pragma once

#include "common.cuh"
#include <math.h>
#include <type_traits>

namespace azp
{
constexpr int PAIR_REC = 8;   // values per pair kernel record
constexpr int CUT_REC = 4;    // rcutsq, ronsq, 1/(rcutsq-ronsq)^3, xplor flag

// correctly rounded reciprocal; the FP32 form maps to the hardware-assisted
// rounded reciprocal instead of a full division (an approximate reciprocal's
// extra ulp, raised to the 12th power by the LJ core, costs too much of the
// FP32 force budget at overlapped pairs)
AZP_HD double rcp(double x) { return 1.0 / x; }
AZP_HD float rcp(float x)
{
#ifdef __CUDA_ARCH__
    return __frcp_rn(x);
#else
    return 1.0f / x;
#endif
}

// ================================================================ pair potentials
// Interface: enabled(rec) -- the reference's "lj1 != 0" / "epsilon != 0" test;
// eval(rec, rsq, fdr, e) -- force/r and energy at rsq < rcutsq, unshifted.
// The energy shift at r_cut is rec[SHIFT_SLOT], subtracted by the caller.

struct PerturbedLJ {
    // rec: lj1, lj2, lambda, rwcasq, wca_shift, 12 lj1, 6 lj2, (shift)
    static constexpr int SHIFT_SLOT = 7;
    static constexpr int REC_DOUBLES = 4;  // param_type: sigma_6, epsilon_x_4, attraction_scale_factor, rwcasq
    template<typename R> AZP_HD static void prepare(const R* p, R* rec)
    {
        const R s6 = p[0], e4 = p[1], lam = p[2];
        rec[0] = e4 * s6 * s6;
        rec[1] = e4 * s6;
        rec[2] = lam;
        rec[3] = p[3];
        rec[4] = e4 * (R(1) - lam) / R(4);
        rec[5] = R(12) * rec[0];
        rec[6] = R(6) * rec[1];
        rec[7] = R(0);
    }
    template<typename R> AZP_HD static bool enabled(const R* rec) { return rec[0] != R(0); }
    template<typename R> AZP_HD static void eval(const R* rec, R rsq, R& fdr, R& e)
    {
        const R r2inv = rcp(rsq);
        const R r6inv = r2inv * r2inv * r2inv;
        R f = r2inv * r6inv * (rec[5] * r6inv - rec[6]);
        R u = r6inv * (rec[0] * r6inv - rec[1]);
        if (rsq < rec[3]) {
            u += rec[4];
        } else {
            f *= rec[2];
            u *= rec[2];
        }
        fdr = f;
        e = u;
    }
};

struct ExpandedYukawa {
    // rec: epsilon, kappa, delta, (shift)
    static constexpr int SHIFT_SLOT = 3;
    static constexpr int REC_DOUBLES = 4;  // param_type: epsilon, kappa, delta (aligned(32))
    template<typename R> AZP_HD static void prepare(const R* p, R* rec)
    {
        rec[0] = p[0];
        rec[1] = p[1];
        rec[2] = p[2];
        for (int k = 3; k < PAIR_REC; ++k) rec[k] = R(0);
    }
    template<typename R> AZP_HD static bool enabled(const R* rec) { return rec[0] != R(0); }
    template<typename R> AZP_HD static void eval(const R* rec, R rsq, R& fdr, R& e)
    {
        const R r = sqrt(rsq);
        const R s = r - rec[2];
        const R sinv = rcp(s);
        const R u = rec[0] * exp(-rec[1] * s) * sinv;
        fdr = u * (rec[1] + sinv) / r;
        e = u;
    }
};

struct Hertz {
    // rec: epsilon, r_cut, (shift, never set: the reference has no shift branch)
    static constexpr int SHIFT_SLOT = 7;
    static constexpr int REC_DOUBLES = 1;  // param_type: epsilon (aligned(8))
    template<typename R> AZP_HD static void prepare(const R* p, R* rec)
    {
        rec[0] = p[0];
        for (int k = 1; k < PAIR_REC; ++k) rec[k] = R(0);
    }
    template<typename R> AZP_HD static bool enabled(const R* rec) { return rec[0] != R(0); }
    template<typename R> AZP_HD static void eval(const R* rec, R rsq, R& fdr, R& e)
    {
        const R r = sqrt(rsq);
        const R rc = rec[1];
        const R x = R(1) - r / rc;
        const R ex32 = rec[0] * x * sqrt(x);
        fdr = R(2.5) * ex32 / (r * rc);
        e = ex32 * x;
    }
};

struct Colloid {
    // rec: A, a_1, a_2, sigma^3, sigma^6, form (0 SS, 1 CS, 2 CC), max(a_1,a_2), (shift)
    static constexpr int SHIFT_SLOT = 7;
    static constexpr int REC_DOUBLES = 4;  // param_type: A, a_1, a_2, sigma_3
    template<typename R> AZP_HD static void prepare(const R* p, R* rec)
    {
        rec[0] = p[0];
        rec[1] = p[1];
        rec[2] = p[2];
        rec[3] = p[3];
        rec[4] = p[3] * p[3];
        rec[5] = (p[1] == R(0) && p[2] == R(0)) ? R(0) : ((p[1] != R(0) && p[2] != R(0)) ? R(2) : R(1));
        rec[6] = p[1] > p[2] ? p[1] : p[2];
        rec[7] = R(0);
    }
    template<typename R> AZP_HD static bool enabled(const R* rec) { return rec[0] != R(0); }

    template<typename R> AZP_HD static R inv7(R x)
    {
        const R xi = rcp(x);
        R g = xi * xi;
        g = g * g * g;
        return g * xi;
    }

    // point -- sphere of radius a, with d = a^2 - rsq supplied
    template<typename R> AZP_HD static void cs_form(const R* rec, R rsq, R d, R& fdr, R& e)
    {
        const R A = rec[0], s3 = rec[3], s6 = rec[4];
        const R a = rec[6];
        const R a2 = a * a;
        const R d3 = d * d * d;
        const R d6 = d3 * d3;
        const R r4 = rsq * rsq;
        const R pre = s3 * A * a * a2 / d3;
        const R poly = R(2) * (a2 + rsq) * (a2 * (R(5) * a2 + R(22) * rsq) + R(5) * r4);
        fdr = R(4.0 / 15.0) * pre * (poly * s6 / d6 - R(5)) / d;
        const R poly_e = a2 * (a2 * (a2 / R(3) + R(3) * rsq) + R(4.2) * r4) + rsq * r4;
        e = R(2.0 / 9.0) * pre * (R(1) - poly_e * s6 / d6);
    }

    // sphere -- sphere (Everaers & Ejtehadi, PRE 67, 041710), with r = sqrt(rsq)
    // and the surface gap sm = (a_1 + a_2) - r supplied
    template<typename R> AZP_HD static void cc_form(const R* rec, R r, R sm, R& fdr, R& e)
    {
        const R A = rec[0], s6 = rec[4];
        const R ai = rec[1], aj = rec[2];
        const R prod = ai * aj, sum = ai + aj, dif = ai - aj;
        const R sp = sum + r, dp = dif + r, dm = dif - r;
        const R q7 = rcp(sp * sm);
        const R q8 = rcp(dp * dm);
        R g0 = inv7(sp), g1 = inv7(sm), g2 = inv7(dp), g3 = inv7(dm);
        const R h0 = ((sp + R(5) * sum) * sp + R(30) * prod) * g0;
        const R h1 = ((sm + R(5) * sum) * sm + R(30) * prod) * g1;
        const R h2 = ((dp + R(5) * dif) * dp - R(30) * prod) * g2;
        const R h3 = ((dm + R(5) * dif) * dm - R(30) * prod) * g3;
        const R pre = A * s6 / r / R(37800);
        R u = pre * (h0 - h1 - h2 + h3);
        g0 *= R(42) * prod / sp + R(6) * sum + sp;
        g1 *= R(42) * prod / sm + R(6) * sum + sm;
        g2 *= R(-42) * prod / dp + R(6) * dif + dp;
        g3 *= R(-42) * prod / dm + R(6) * dif + dm;
        const R dur = u / r + R(5) * pre * (g0 + g1 - g2 - g3);
        const R dua = -A / R(3) * r * ((R(2) * prod * q7 + R(1)) * q7 + (R(2) * prod * q8 - R(1)) * q8);
        fdr = (dur + dua) / r;
        u += A / R(6) * (R(2) * prod * (q7 + q8) - log(q8 / q7));
        e = u;
    }

    template<typename R> AZP_HD static void eval(const R* rec, R rsq, R& fdr, R& e)
    {
        const R A = rec[0], s6 = rec[4];
        const int form = (int)rec[5];
        if (form == 0) {
            // integrated over no sphere: LJ with prefactor A/36
            const R r2inv = rcp(rsq);
            const R r6inv = r2inv * r2inv * r2inv;
            const R c = A * s6 / R(36);
            fdr = R(6) * c * r2inv * r6inv * (R(2) * s6 * r6inv - R(1));
            e = c * r6inv * (s6 * r6inv - R(1));
        } else if (form == 1) {
            const R a = rec[6];
            cs_form(rec, rsq, a * a - rsq, fdr, e);
        } else {
            const R r = sqrt(rsq);
            cc_form(rec, r, (rec[1] + rec[2]) - r, fdr, e);
        }
    }

    // Forms whose arguments cancel near contact: point-sphere (a^2 - r^2) and
    // sphere-sphere ((a_1 + a_2) - r). Their forces fall off like the ninth or
    // higher power of that difference, so in FP32 a difference formed from a
    // rounded r^2 loses the force budget a fraction of sigma from contact.
    template<typename R> AZP_HD static bool gap_form(const R* rec) { return rec[5] != R(0); }
    // squared contact distance of the form, from the FP64 record: a^2 or (a_1 + a_2)^2
    AZP_HD static double contact2(const double* rec_d)
    {
        const double c = rec_d[5] == 1.0 ? rec_d[6] : rec_d[1] + rec_d[2];
        return c * c;
    }
    // FP32 evaluation of a gap form with rsq and dq = contact^2 - rsq formed by
    // the caller from an exact displacement, each rounded once to FP32: the
    // point-sphere d is dq, the sphere-sphere gap is dq / (a_1 + a_2 + r).
    AZP_D static void eval_gap(const float* rec, float rsq, float dq, float& fdr, float& e)
    {
        if (rec[5] == 1.0f) {
            cs_form(rec, rsq, dq, fdr, e);
        } else {
            const float r = sqrtf(rsq);
            cc_form(rec, r, dq / ((rec[1] + rec[2]) + r), fdr, e);
        }
    }
    // squared contact distance of the form from the FP32 record
    AZP_D static float contact2_f(const float* rec)
    {
        const float c = rec[5] == 1.0f ? rec[6] : rec[1] + rec[2];
        return c * c;
    }
    // one evaluation per pair whatever its form: the LJ form (solvent pairs) on
    // rsq, the gap forms on (rsq, dq) as eval_gap
    AZP_D static void eval_any(const float* rec, float rsq, float dq, float& fdr, float& e)
    {
        if (rec[5] == 0.0f) eval(rec, rsq, fdr, e);
        else eval_gap(rec, rsq, dq, fdr, e);
    }
};

template<class E> struct has_gap_form {
    static constexpr bool value = false;
};
template<> struct has_gap_form<Colloid> {
    static constexpr bool value = true;
};

// Host: fill the kernel record and cut record of one type pair.
// p: the reference param_type zero-padded to 4 doubles; mode: azp_shift_mode.
template<class Eval, typename R>
AZP_HD void prepare_pair_t(const R* p, double rcut, double ron, int mode, R* rec, R* cut)
{
    Eval::prepare(p, rec);
    const double rcutsq = rcut * rcut;
    const double ronsq = ron * ron;
    if (std::is_same<Eval, Hertz>::value) rec[1] = R(rcut);
    cut[0] = R(rcutsq);
    cut[1] = R(ronsq);
    cut[2] = R((mode == AZP_MODE_XPLOR && ronsq < rcutsq) ? 1.0 / ((rcutsq - ronsq) * (rcutsq - ronsq) * (rcutsq - ronsq))
                                                          : 0.0);
    cut[3] = R((mode == AZP_MODE_XPLOR && ronsq < rcutsq) ? 1.0 : 0.0);
    const bool shift = (mode == AZP_MODE_SHIFT) || (mode == AZP_MODE_XPLOR && ronsq > rcutsq);
    if (shift && rcut > 0.0 && Eval::enabled(rec) && !std::is_same<Eval, Hertz>::value) {
        R f = R(0), e = R(0);
        Eval::eval(rec, R(rcutsq), f, e);
        rec[Eval::SHIFT_SLOT] = e;
    }
    if (!(rcut > 0.0)) cut[0] = R(0);  // r_cut 0: the type pair is never evaluated
}

template<class Eval>
AZP_HD void prepare_pair(const double* p, double rcut, double ron, int mode, double* rec, double* cut)
{
    prepare_pair_t<Eval, double>(p, rcut, ron, mode, rec, cut);
}

// one record of a caller's table (Eval::REC_DOUBLES doubles at p) zero-padded to 4
template<class Eval> AZP_HD void load_pair_record(const double* p, double* q)
{
    for (int k = 0; k < 4; ++k) q[k] = k < Eval::REC_DOUBLES ? p[k] : 0.0;
}
// the same for a bond record, padded to AZP_BOND_PARAM_DOUBLES
template<class Eval> AZP_HD void load_bond_record(const double* p, double* q)
{
    for (int k = 0; k < AZP_BOND_PARAM_DOUBLES; ++k) q[k] = k < Eval::REC_DOUBLES ? p[k] : 0.0;
}

// XPLOR smoothing of (fdr, e) for ronsq <= rsq < rcutsq (HOOMD pair.Pair mode
// "xplor"): S = (rc2 - r2)^2 (rc2 + 2 r2 - 3 ro2) / (rc2 - ro2)^3.
template<typename R> AZP_HD void xplor(const R* cut, R rsq, R& fdr, R& e)
{
    if (cut[3] != R(0) && rsq >= cut[1]) {
        const R a = rsq - cut[0];
        const R s = a * a * (cut[0] + R(2) * rsq - R(3) * cut[1]) * cut[2];
        const R dsdr_r = R(12) * (rsq - cut[1]) * a * cut[2];
        fdr = s * fdr - dsdr_r * e;
        e = e * s;
    }
}

// ================================================================ bond potentials
// rec = the reference param_type, zero-padded to 8 doubles (load_bond_record).
// eval returns false when the
// evaluator refuses (the reference's "invalid parameters" returns).
// The FP32-force engine step uses FP32 records of BOND_F floats per bond type
// instead, with the per-type constants of eval precomputed (prepare_f), so its
// eval_f holds no parameter division.
constexpr int BOND_F = 12;

struct QuarticBond {
    static constexpr int REC_DOUBLES = 8;  // param_type: k, r_0, b_1, b_2, U_0, sigma_6, epsilon_x_4, delta
    template<typename R> AZP_HD static bool eval(const R* p, R rsq, R& fdr, R& e)
    {
        const R k = p[0], r0 = p[1], b1 = p[2], b2 = p[3], U0 = p[4];
        const R lj1 = p[6] * p[5] * p[5];
        const R lj2 = p[6] * p[5];
        const R del = p[7];
        fdr = R(0);
        e = R(0);
        if (r0 == R(0)) return false;
        R rr = R(1);
        if (del == R(0)) {
            const R r2inv = rcp(rsq);
            const R r6inv = r2inv * r2inv * r2inv;
            if (lj1 != R(0) && r6inv > (lj2 / lj1) / R(2)) {
                fdr += r2inv * r6inv * (R(12) * lj1 * r6inv - R(6) * lj2);
                e += r6inv * (lj1 * r6inv - lj2) + lj2 * lj2 / R(4) / lj1;
            }
            if (rsq < r0 * r0) rr = sqrt(rsq) - r0;
        } else {
            const R rs = sqrt(rsq) - del;
            const R r2inv = R(1) / rs / rs;
            const R r6inv = r2inv * r2inv * r2inv;
            if (lj1 != R(0) && r6inv > (lj2 / lj1) / R(2)) {
                fdr += r6inv * (R(12) * lj1 * r6inv - R(6) * lj2) / rs / (rs + del);
                e += r6inv * (lj1 * r6inv - lj2) + p[6] / R(4);
            }
            if (rs < r0) rr = rs - r0;
        }
        if (rr < R(0)) {
            fdr += -k * rr * (R(4) * rr * rr - R(3) * (b1 + b2) * rr + R(2) * b1 * b2) / (rr + r0 + del);
            e += k * (rr - b1) * (rr - b2) * rr * rr + U0;
        } else {
            e += U0;
        }
        return true;
    }
    // q: k, r_0, b_1, b_2, U_0, lj1, lj2, delta, WCA r^-6 threshold, WCA energy
    // shift, 3 (b_1 + b_2), 2 b_1 b_2
    AZP_HD static void prepare_f(const double* p, float* q)
    {
        const double lj1 = p[6] * p[5] * p[5], lj2 = p[6] * p[5];
        for (int k = 0; k < 5; ++k) q[k] = (float)p[k];
        q[5] = (float)lj1;
        q[6] = (float)lj2;
        q[7] = (float)p[7];
        q[8] = lj1 != 0.0 ? (float)((lj2 / lj1) / 2.0) : 0.0f;
        q[9] = p[7] == 0.0 ? (lj1 != 0.0 ? (float)(lj2 * lj2 / 4.0 / lj1) : 0.0f) : (float)(p[6] / 4.0);
        q[10] = (float)(3.0 * (p[2] + p[3]));
        q[11] = (float)(2.0 * p[2] * p[3]);
    }
    AZP_D static bool eval_f(const float* q, float rsq, float& fdr, float& e)
    {
        const float k = q[0], r0 = q[1], b1 = q[2], b2 = q[3], lj1 = q[5], lj2 = q[6], del = q[7];
        fdr = 0.0f;
        e = 0.0f;
        if (r0 == 0.0f) return false;
        float rr = 1.0f;
        if (del == 0.0f) {
            const float r2inv = rcp(rsq);
            const float r6inv = r2inv * r2inv * r2inv;
            if (lj1 != 0.0f && r6inv > q[8]) {
                fdr += r2inv * r6inv * (12.0f * lj1 * r6inv - 6.0f * lj2);
                e += r6inv * (lj1 * r6inv - lj2) + q[9];
            }
            if (rsq < r0 * r0) rr = sqrtf(rsq) - r0;
        } else {
            const float rs = sqrtf(rsq) - del;
            const float r2inv = rcp(rs * rs);
            const float r6inv = r2inv * r2inv * r2inv;
            if (lj1 != 0.0f && r6inv > q[8]) {
                fdr += r6inv * (12.0f * lj1 * r6inv - 6.0f * lj2) / (rs * (rs + del));
                e += r6inv * (lj1 * r6inv - lj2) + q[9];
            }
            if (rs < r0) rr = rs - r0;
        }
        if (rr < 0.0f) {
            fdr += -k * rr * (4.0f * rr * rr - q[10] * rr + q[11]) / (rr + r0 + del);
            e += k * (rr - b1) * (rr - b2) * rr * rr + q[4];
        } else {
            e += q[4];
        }
        return true;
    }
};

struct DoubleWellBond {
    static constexpr int REC_DOUBLES = 4;  // param_type: r_1, r_diff, U_1, U_tilt
    template<typename R> AZP_HD static bool eval(const R* p, R rsq, R& fdr, R& e)
    {
        const R r1 = p[0], rd = p[1], U1 = p[2], Ut = p[3];
        fdr = R(0);
        e = R(0);
        if (rd == R(0)) return false;
        const R r = sqrt(rsq);
        const R x = (r1 - r) / rd;
        const R y = R(1) - x * x;
        e = U1 * y * y + Ut * (R(1) - x - y * y);
        fdr = (R(4) * x * y * (Ut - U1) - Ut) / (rd * r);
        return true;
    }
    AZP_HD static void prepare_f(const double* p, float* q)
    {
        for (int k = 0; k < BOND_F; ++k) q[k] = k < AZP_BOND_PARAM_DOUBLES ? (float)p[k] : 0.0f;
    }
    AZP_D static bool eval_f(const float* q, float rsq, float& fdr, float& e) { return eval(q, rsq, fdr, e); }
};

// DPD with a general weight function inside the resident engine
// (src/DPDPairEvaluatorGeneralWeight.h:165-255). The fused step evaluates it
// in its own pair term (velocities and a per-pair Philox draw), not through
// eval(); the kernel record, built by the engine on the host, holds
// rec = {1/r_cut, r_cut, A, gamma, s/2, sigma_R = sqrt(6 kT gamma / dt), -, -}
// and the cut record's r_cut^2.
struct DpdEngine {
    static constexpr int SHIFT_SLOT = 7;
    template<typename R> AZP_HD static bool enabled(const R* rec) { return rec[1] > R(0); }
    template<typename R> AZP_HD static void eval(const R*, R, R& fdr, R& e)
    {
        fdr = R(0);
        e = R(0);
    }
};

// Harmonic bond U = k/2 (r - r_0)^2 (HOOMD's EvaluatorBondHarmonic, which
// src/ImagePotentialBond.h:144-152 applies to the image-unwrapped distance):
// p = {k, r_0}. At r = 0 the force is set to 0 (its direction is undefined).
struct HarmonicBond {
    static constexpr int REC_DOUBLES = 2;  // HOOMD harmonic bond param_type: k, r_0
    template<typename R> AZP_HD static bool eval(const R* p, R rsq, R& fdr, R& e)
    {
        const R k = p[0], r0 = p[1];
        const R r = sqrt(rsq);
        fdr = r > R(0) ? k * (r0 / r - R(1)) : R(0);
        e = R(0.5) * k * (r0 - r) * (r0 - r);
        return true;
    }
    // FP32 record of the fused step: q = k, r_0
    AZP_HD static void prepare_f(const double* p, float* q)
    {
        for (int c = 0; c < BOND_F; ++c) q[c] = 0.0f;
        q[0] = (float)p[0];
        q[1] = (float)p[1];
    }
    AZP_D static bool eval_f(const float* q, float rsq, float& fdr, float& e)
    {
        const float k = q[0], r0 = q[1];
        const float r = sqrtf(rsq);
        fdr = r > 0.0f ? k * (r0 / r - 1.0f) : 0.0f;
        e = 0.5f * k * (r0 - r) * (r0 - r);
        return true;
    }
};

// bond evaluators measured between image-unwrapped positions (x + img L)
// instead of the minimum image: the ImageHarmonic bond
template<class BE> struct bond_uses_image {
    static constexpr bool value = false;
};
template<> struct bond_uses_image<HarmonicBond> {
    static constexpr bool value = true;
};

}  // namespace azp
