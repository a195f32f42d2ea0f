// engine_kernels.cuh -- the fused force-and-integrate step of the resident engine.
//
// One launch per timestep: pair forces over the column-major list + bond forces
// from the per-particle table (TPP threads per particle, warp-shuffle reduction),
// then, by the group's first lane, Langevin step two at timestep t followed by
// step one of timestep t + 1 (or the Brownian move at t), writing the next
// position buffer and its fixed-point shadow, and the list-rebuild request.
// Arithmetic of each phase follows the standalone kernels (pair.cu, bond.cu,
// integrate.cu) and through them the reference lines cited there.
#pragma once

#include "barrier.cuh"
#include "celllist.cuh"
#include "engine.cuh"
#include "philox.cuh"
#include "evaluators.cuh"
#include "pair.cuh"

namespace azp
{
static_assert(MD_PAIR_TBL == PAIR_TBL && MD_BOND_F == BOND_F, "record sizes of MDArgs");
constexpr int MD_BLOCK = 256;
// threads per block of the FP32-force step
#ifndef AZP_FX_BLOCK
#define AZP_FX_BLOCK 256
#endif
constexpr int FX_BLOCK = AZP_FX_BLOCK;
constexpr uint32_t MD_MAX_BOND_TYPES = 32;

struct NoPair {
    static constexpr int SHIFT_SLOT = 7;
    template<typename R> AZP_HD static bool enabled(const R*) { return false; }
    template<typename R> AZP_HD static void eval(const R*, R, R& f, R& e) { f = e = R(0); }
};
struct NoBond {
    template<typename R> AZP_HD static bool eval(const R*, R, R& f, R& e)
    {
        f = e = R(0);
        return true;
    }
    AZP_HD static void prepare_f(const double*, float*) {}
    AZP_D static bool eval_f(const float*, float, float& f, float& e)
    {
        f = e = 0.0f;
        return true;
    }
};

// accumulator: compensated force / energy in FP32, plain in FP64
template<typename R> struct Acc;
template<> struct Acc<double> {
    double fx = 0, fy = 0, fz = 0, u = 0, w[6] = {0, 0, 0, 0, 0, 0};
    AZP_D void add(double dx, double dy, double dz, double fdr, double e, bool vir)
    {
        fx += dx * fdr;
        fy += dy * fdr;
        fz += dz * fdr;
        u += 0.5 * e;
        if (vir) {
            const double h = 0.5 * fdr;
            w[0] += h * dx * dx;
            w[1] += h * dx * dy;
            w[2] += h * dx * dz;
            w[3] += h * dy * dy;
            w[4] += h * dy * dz;
            w[5] += h * dz * dz;
        }
    }
    // force from fdr, virial from fvir (DPD: the conservative part only)
    AZP_D void add_split(double dx, double dy, double dz, double fdr, double fvir, double e, bool vir)
    {
        fx += dx * fdr;
        fy += dy * fdr;
        fz += dz * fdr;
        u += 0.5 * e;
        if (vir) {
            const double h = 0.5 * fvir;
            w[0] += h * dx * dx;
            w[1] += h * dx * dy;
            w[2] += h * dx * dz;
            w[3] += h * dy * dy;
            w[4] += h * dy * dz;
            w[5] += h * dz * dz;
        }
    }
    AZP_D void reduce(int tpp, bool vir)
    {
        for (int m = tpp >> 1; m > 0; m >>= 1) {
            fx += __shfl_xor_sync(0xffffffffu, fx, m);
            fy += __shfl_xor_sync(0xffffffffu, fy, m);
            fz += __shfl_xor_sync(0xffffffffu, fz, m);
            u += __shfl_xor_sync(0xffffffffu, u, m);
            if (vir)
                for (int c = 0; c < 6; ++c) w[c] += __shfl_xor_sync(0xffffffffu, w[c], m);
        }
    }
    AZP_D double Fx() const { return fx; }
    AZP_D double Fy() const { return fy; }
    AZP_D double Fz() const { return fz; }
    AZP_D double U() const { return u; }
};
template<> struct Acc<float> {
    Comp fx{0.f, 0.f}, fy{0.f, 0.f}, fz{0.f, 0.f}, u{0.f, 0.f};
    float w[6] = {0, 0, 0, 0, 0, 0};
    AZP_D void add(float dx, float dy, float dz, float fdr, float e, bool vir)
    {
        fx.add(dx * fdr);
        fy.add(dy * fdr);
        fz.add(dz * fdr);
        u.add(0.5f * e);
        if (vir) {
            const float h = 0.5f * fdr;
            w[0] += h * dx * dx;
            w[1] += h * dx * dy;
            w[2] += h * dx * dz;
            w[3] += h * dy * dy;
            w[4] += h * dy * dz;
            w[5] += h * dz * dz;
        }
    }
    AZP_D static void comb(Comp& c, int m)
    {
        const float s2 = __shfl_xor_sync(0xffffffffu, c.s, m);
        const float c2 = __shfl_xor_sync(0xffffffffu, c.c, m);
        c.add(s2);
        c.c += c2;
    }
    AZP_D void reduce(int tpp, bool vir)
    {
        for (int m = tpp >> 1; m > 0; m >>= 1) {
            comb(fx, m);
            comb(fy, m);
            comb(fz, m);
            comb(u, m);
            if (vir)
                for (int c = 0; c < 6; ++c) w[c] += __shfl_xor_sync(0xffffffffu, w[c], m);
        }
    }
    // sum and carry converted separately: the FP64 result keeps the compensation
    AZP_D double Fx() const { return (double)fx.s + (double)fx.c; }
    AZP_D double Fy() const { return (double)fy.s + (double)fy.c; }
    AZP_D double Fz() const { return (double)fz.s + (double)fz.c; }
    AZP_D double U() const { return (double)u.s + (double)u.c; }
};

// Accumulator of the FP32-force step. The terms of one gather batch (at most
// FX_BATCH pairs, or the bonds) are summed in plain FP32, and each batch sum
// enters the per-particle force with two-sum compensation, so the rounding error
// does not grow with the neighbour count. Energy and virial are accumulated only
// when the step writes them (the integrator needs forces alone).
struct AccFx {
    Comp fx{0.f, 0.f}, fy{0.f, 0.f}, fz{0.f, 0.f}, u{0.f, 0.f};
    float w[6] = {0, 0, 0, 0, 0, 0};
    float bx = 0.f, by = 0.f, bz = 0.f, bu = 0.f;
    AZP_D void add(float dx, float dy, float dz, float fdr, float e, bool out)
    {
        bx += dx * fdr;
        by += dy * fdr;
        bz += dz * fdr;
        if (out) {
            bu += 0.5f * e;
            const float h = 0.5f * fdr;
            w[0] += h * dx * dx;
            w[1] += h * dx * dy;
            w[2] += h * dx * dz;
            w[3] += h * dy * dy;
            w[4] += h * dy * dz;
            w[5] += h * dz * dz;
        }
    }
    // force from fdr, virial from fvir (DPD: the conservative part only)
    AZP_D void add_split(float dx, float dy, float dz, float fdr, float fvir, float e, bool out)
    {
        bx += dx * fdr;
        by += dy * fdr;
        bz += dz * fdr;
        if (out) {
            bu += 0.5f * e;
            const float h = 0.5f * fvir;
            w[0] += h * dx * dx;
            w[1] += h * dx * dy;
            w[2] += h * dx * dz;
            w[3] += h * dy * dy;
            w[4] += h * dy * dz;
            w[5] += h * dz * dz;
        }
    }
    // close a batch: its sums enter the compensated totals
    AZP_D void commit(bool out)
    {
        fx.add(bx);
        fy.add(by);
        fz.add(bz);
        if (out) u.add(bu);
        bx = by = bz = bu = 0.f;
    }
    AZP_D void reduce(int tpp, bool out)
    {
        for (int m = tpp >> 1; m > 0; m >>= 1) {
            Acc<float>::comb(fx, m);
            Acc<float>::comb(fy, m);
            Acc<float>::comb(fz, m);
            if (out) {
                Acc<float>::comb(u, m);
                for (int c = 0; c < 6; ++c) w[c] += __shfl_xor_sync(0xffffffffu, w[c], m);
            }
        }
    }
    AZP_D double Fx() const { return (double)fx.s + (double)fx.c; }
    AZP_D double Fy() const { return (double)fy.s + (double)fy.c; }
    AZP_D double Fz() const { return (double)fz.s + (double)fz.c; }
    AZP_D double U() const { return (double)u.s + (double)u.c; }
};

// ---------------------------------------------------------------- harmonic barrier
// record offset of (timestep ts, type ti) in the barrier table (rows clamped)
AZP_D size_t barrier_slot(const MDArgs& a, unsigned long long ts, uint32_t ti)
{
    const unsigned long long t0 = a.bar_hdr[0], rows = a.bar_hdr[1];
    const unsigned long long r = ts <= t0 ? 0ull : min(ts - t0, rows - 1ull);
    return (size_t)r * a.ntypes + ti;
}

// FP64: the barrier force and energy of particle i (position p) at timestep ts
AZP_D void barrier_fp64(const MDArgs& a, const double4_32a& p, unsigned long long ts, double* f, double& e)
{
    const double2 ck = __ldg(reinterpret_cast<const double2*>(a.bar_tab) + barrier_slot(a, ts, type_of(p.w)));
    const double x[3] = {p.x, p.y, p.z};
    if (a.bar_geom == AZP_BARRIER_PLANAR)
        planar_barrier(x, ck.x, ck.y, f, e);
    else
        spherical_barrier(x, ck.x, ck.y, f, e);
}

// FP32: the same on the fixed-point shadow fi (hi words, type in w)
AZP_D void barrier_fx(const MDArgs& a, const uint4& fi, unsigned long long ts, float* f, float& e)
{
    const BarrierRecF* tab = reinterpret_cast<const BarrierRecF*>(a.bar_tab);
    const size_t k = barrier_slot(a, ts, fi.w);
    BarrierRecF r;
    const int4 raw = __ldg(reinterpret_cast<const int4*>(tab + k));
    r.q = (long long)(((unsigned long long)(uint32_t)raw.y << 32) | (uint32_t)raw.x);
    r.c = __int_as_float(raw.z);
    r.k = __int_as_float(raw.w);
    if (a.bar_geom == AZP_BARRIER_PLANAR)
        planar_barrier_fx(fi, r, a.sfix[1], f, e);
    else
        spherical_barrier_fx(fi, r, a.sfix, f, e);
}

// ---------------------------------------------------------------- walls
// wall_tab row of a type: record (4 doubles), r_cut^2, r_extrap, r_cut, -
constexpr int WALL_TAB = 8;

// FP64 force and energy of every wall on a particle at x (type t), added to
// F[0..2] and F[3]. Out of line: its registers and stack do not count against
// the step's neighbour loop.
static __device__ __noinline__ void engine_walls(int kind, const WallField* __restrict__ wf, const double* __restrict__ tab,
                                          double x0, double x1, double x2, uint32_t t, double* F)
{
    const double* row = tab + (size_t)t * WALL_TAB;
    const double p[4] = {row[0], row[1], row[2], row[3]};
    const double x[3] = {x0, x1, x2};
    double f[3] = {0.0, 0.0, 0.0}, u = 0.0;
    if (kind == AZP_WALL_LJ93)
        walls_force<WallLJ93>(*wf, p, row[4], row[5], x, f, u);
    else
        walls_force<WallColloid>(*wf, p, row[4], row[5], x, f, u);
    F[0] += f[0];
    F[1] += f[1];
    F[2] += f[2];
    F[3] += u;
}

// FP32 screen of the FP32-force step: could any wall act on a particle at
// (x, y, z) (positions good to about L 2^-24, covered by tol)? A wall acts within
// r_cut on its active side, and anywhere on its inactive side with r_extrap > 0.
AZP_D bool walls_near_f(const WallField* __restrict__ wf, const double* __restrict__ tab, uint32_t t, float x,
                        float y, float z, float tol)
{
    const double* row = tab + (size_t)t * WALL_TAB;
    return walls_near(*wf, (float)row[6] + tol, row[5] > 0.0, x, y, z, tol);
}

// |fixed - fixed at the last build|^2 > threshold, in FP32 on exact integer differences
AZP_D bool displaced(const uint4& f, const uint4& fb, const float* sfix, float thresh2)
{
    const float dx = (float)(int32_t)(f.x - fb.x) * sfix[0];
    const float dy = (float)(int32_t)(f.y - fb.y) * sfix[1];
    const float dz = (float)(int32_t)(f.z - fb.z) * sfix[2];
    return dx * dx + dy * dy + dz * dz > thresh2;
}

// ---------------------------------------------------------------- DPD in the step
// The timestep whose forces a step evaluates (the DPD draw's timestep): a
// Langevin step at t evaluates t + 1 (HOOMD computes the net force of t + 1
// between the halves), a forces-only launch its own timestep.
template<int INTEG> AZP_D unsigned long long force_timestep(const MDArgs& a)
{
    return *a.d_timestep + (INTEG == MD_INTEG_LANGEVIN ? 1ull : 0ull);
}

// alpha in (-1, 1) of the pair (tags ti, tj): the first 64-bit word of the
// pair's Philox block, stream (AZP_RNG_DPD_GENERAL_WEIGHT, timestep, seed),
// counter {0, min tag, max tag, 0}, as azp_dpd_forces draws it
AZP_D void dpd_key(const MDArgs& a, unsigned long long ts, uint32_t& k0, uint32_t& k1)
{
    stream_key(AZP_RNG_DPD_GENERAL_WEIGHT, ts, a.seed, k0, k1);
}

AZP_D double dpd_weight_engine(double x, double h)
{
    if (h == 0.5) return sqrt(x);
    if (h == 0.25) return sqrt(sqrt(x));
    if (h == 1.0) return x;
    return pow(x, h);
}

AZP_D float dpd_weight_engine_f(float x, float h)
{
    if (h == 0.5f) return sqrtf(x);
    if (h == 0.25f) return sqrtf(sqrtf(x));
    if (h == 1.0f) return x;
    return powf(x, h);
}

// one pair in FP64: dx = x_i - x_j, dv = v_i - v_j; rec as in DpdEngine.
// Returns false outside r_cut (rsq >= rcutsq).
AZP_D bool dpd_term_fp64(const double* rec, double rcutsq, double dx, double dy, double dz, double dvx, double dvy,
                         double dvz, uint32_t k0, uint32_t k1, uint32_t tgi, uint32_t tgj, double& fdr, double& fc,
                         double& e)
{
    const double rs = rsq_exact(dx, dy, dz);
    if (!(rs < rcutsq)) return false;
    const double rcinv = rec[0], rc = rec[1], A = rec[2], gamma = rec[3];
    const double rinv = 1.0 / sqrt(rs);
    const double r = 1.0 / rinv;
    const double dot = dx * dvx + dy * dvy + dz * dvz;
    fc = A * (rinv - rcinv);
    const double wR = dpd_weight_engine(fmax(1.0 - r * rcinv, 0.0), rec[4]) * rinv;
    const Philox4 ph = philox4x32_10(0u, min(tgi, tgj), max(tgi, tgj), 0u, k0, k1);
    const double alpha = -1.0 + 2.0 * open01(ph.v[0], ph.v[1]);
    fdr = fc - gamma * wR * wR * dot + rec[5] * wR * alpha;
    e = A * (rc - r) - 0.5 * A * rcinv * (rcutsq - rs);
    return true;
}

// FP64 step: FP64 positions, forces and integration, the oracle's rounding for
// every decision.
template<class PE, class BE, typename R, int INTEG>
__global__ void __launch_bounds__(MD_BLOCK) k_md_step(MDArgs a)
{
    static_assert(std::is_same<R, double>::value, "k_md_step is the FP64 step; FP32 forces use k_md_step_fx");
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const uint32_t nt2 = a.ntypes * a.ntypes;
    double* s_rc2 = reinterpret_cast<double*>(smem_raw);
    double* s_gamma = s_rc2 + nt2;
    double* s_noise = s_gamma + a.ntypes;
    R* s_rec = reinterpret_cast<R*>(s_noise + a.ntypes);
    R* s_bond = s_rec + nt2 * PAIR_TBL;
    if (!std::is_same<PE, NoPair>::value)
        for (uint32_t t = threadIdx.x; t < nt2 * PAIR_TBL; t += blockDim.x) {
            s_rec[t] = (R)a.pair_table[t];
            if (t % PAIR_TBL == PAIR_REC) s_rc2[t / PAIR_TBL] = a.pair_table[t];
        }
    if (!std::is_same<BE, NoBond>::value)
        for (uint32_t t = threadIdx.x; t < a.nbondtypes * AZP_BOND_PARAM_DOUBLES; t += blockDim.x)
            s_bond[t] = (R)a.bond_params[t];
    if (INTEG != MD_FORCES_ONLY && !a.use_lambda)
        for (uint32_t t = threadIdx.x; t < a.ntypes; t += blockDim.x) {
            s_gamma[t] = a.gamma[t];
            s_noise[t] = a.noise[t];
        }
    __syncthreads();

    const int tpp = a.tpp;
    const uint32_t gid = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t i = gid / tpp;
    const uint32_t sub = gid % tpp;
    const bool active = i < a.N;
    const bool vir = a.out != 0;
    Acc<R> acc;
    if (active) {
        // ---------------------------------------------------------------- pair
        if constexpr (!std::is_same<PE, NoPair>::value) {
            const uint32_t n = min(a.counts[i], a.max_nn);
            {
                const double4_32a pi = a.pos[i];
                const uint32_t ti = type_of(pi.w);
                uint32_t k0 = 0, k1 = 0, tgi = 0;
                double4_32a vi{};
                if constexpr (std::is_same<PE, DpdEngine>::value) {
                    dpd_key(a, force_timestep<INTEG>(a), k0, k1);
                    tgi = a.tag[i];
                    vi = reinterpret_cast<const double4_32a*>(a.dvel)[i];
                }
                for (uint32_t k = sub; k < n; k += tpp) {
                    const uint32_t j = a.nbrs[(size_t)k * a.N + i];
                    const double4_32a pj = a.pos[j];
                    const double dx = min_image1(pi.x - pj.x, a.L[0], a.Linv[0]);
                    const double dy = min_image1(pi.y - pj.y, a.L[1], a.Linv[1]);
                    const double dz = min_image1(pi.z - pj.z, a.L[2], a.Linv[2]);
                    const double rsq = rsq_exact(dx, dy, dz);
                    const uint32_t tp = ti * a.ntypes + type_of(pj.w);
                    const R* rec = s_rec + (size_t)tp * PAIR_TBL;
                    const R* cut = rec + PAIR_REC;
                    if constexpr (std::is_same<PE, DpdEngine>::value) {
                        const double4_32a vj = reinterpret_cast<const double4_32a*>(a.dvel)[j];
                        double fdr, fc, e;
                        if (dpd_term_fp64(rec, cut[0], dx, dy, dz, vi.x - vj.x, vi.y - vj.y, vi.z - vj.z, k0, k1, tgi,
                                          a.tag[j], fdr, fc, e))
                            acc.add_split(dx, dy, dz, fdr, fc, e, vir);
                        continue;
                    }
                    if (!(rsq < cut[0]) || !PE::enabled(rec)) continue;
                    R fdr, e;
                    PE::eval(rec, rsq, fdr, e);
                    e -= rec[PE::SHIFT_SLOT];
                    xplor(cut, rsq, fdr, e);
                    if (a.fcap > 0.0 && (double)fdr * fdr * rsq > a.fcap * a.fcap)
                        fdr = (R)copysign(a.fcap / sqrt((double)rsq), (double)fdr);
                    acc.add(dx, dy, dz, fdr, e, vir);
                }
            }
        }
        // ---------------------------------------------------------------- bonds
        if constexpr (!std::is_same<BE, NoBond>::value) {
            const uint32_t nb = a.bt_n[i];
            for (uint32_t k = sub; k < nb; k += tpp) {
                const uint2 e2 = a.bt[(size_t)k * a.N + i];
                const double4_32a pi = a.pos[i];
                const double4_32a pj = a.pos[e2.x];
                double dx, dy, dz;
                if constexpr (bond_uses_image<BE>::value) {
                    // (x_i - x_j) + (img_i - img_j) L (src/ImagePotentialBond.h:144-152)
                    const int* gi = a.img0 + 3 * (size_t)i;
                    const int* gj = a.img0 + 3 * (size_t)e2.x;
                    dx = __dadd_rn(pi.x - pj.x, __dmul_rn((double)(gi[0] - gj[0]), a.L[0]));
                    dy = __dadd_rn(pi.y - pj.y, __dmul_rn((double)(gi[1] - gj[1]), a.L[1]));
                    dz = __dadd_rn(pi.z - pj.z, __dmul_rn((double)(gi[2] - gj[2]), a.L[2]));
                } else {
                    dx = min_image1(pi.x - pj.x, a.L[0], a.Linv[0]);
                    dy = min_image1(pi.y - pj.y, a.L[1], a.Linv[1]);
                    dz = min_image1(pi.z - pj.z, a.L[2], a.Linv[2]);
                }
                const double rsq = rsq_exact(dx, dy, dz);
                double fdr, en;
                if (!BE::eval(s_bond + e2.y * AZP_BOND_PARAM_DOUBLES, rsq, fdr, en)) {
                    atomicOr(&a.flags[1], AZP_EBIT_BOND);
                    continue;
                }
                acc.add(dx, dy, dz, fdr, en, vir);
            }
        }
    }
    if (tpp > 1) acc.reduce(tpp, vir);

    bool want_rebuild = false;
    if (active && sub == 0) {
        double Fx = acc.Fx(), Fy = acc.Fy(), Fz = acc.Fz();
        double Ub = 0.0;
        if (a.bar_geom >= 0) {
            // the barrier's force joins the net force (src/HarmonicBarrier.h:149-180)
            double fb[3] = {0.0, 0.0, 0.0};
            barrier_fp64(a, a.pos[i], *a.d_timestep + (INTEG == MD_INTEG_LANGEVIN ? 1ull : 0ull), fb, Ub);
            Fx += fb[0];
            Fy += fb[1];
            Fz += fb[2];
        }
        double fw[4] = {0.0, 0.0, 0.0, 0.0};
        double4_32a pw;
        if (a.wall_kind >= 0) {
            // the wall potential's force joins the net force (HOOMD adds the
            // external wall compute into net_force)
            pw = a.pos[i];
            engine_walls(a.wall_kind, a.walls, a.wall_tab, pw.x, pw.y, pw.z, type_of(pw.w), fw);
            Fx += fw[0];
            Fy += fw[1];
            Fz += fw[2];
            Ub += fw[3];
        }
        if (a.out) {
            a.out_force[i] = make_double4_32a(Fx, Fy, Fz, acc.U() + Ub);
            double wv[6] = {(double)acc.w[0], (double)acc.w[1], (double)acc.w[2],
                            (double)acc.w[3], (double)acc.w[4], (double)acc.w[5]};
            if (a.wall_kind >= 0) {
                wv[0] += fw[0] * pw.x;
                wv[1] += fw[0] * pw.y;
                wv[2] += fw[0] * pw.z;
                wv[3] += fw[1] * pw.y;
                wv[4] += fw[1] * pw.z;
                wv[5] += fw[2] * pw.z;
            }
            for (int c = 0; c < 6; ++c) a.out_virial[(size_t)c * a.N + i] = wv[c];
        }
        if constexpr (INTEG != MD_FORCES_ONLY) {
            const unsigned long long ts = *a.d_timestep;
            double4_32a p = a.pos[i];
            const uint32_t ti = type_of(p.w);
            const uint32_t tg = a.tag[i];
            bool moved = false;
            {
                // FP64 path: the reference arithmetic throughout; the per-type noise
                // amplitude sqrt(6 gamma kT / dt) comes from a host table built with
                // the same double operations, so the draws stay bit-exact
                const double gam = a.use_lambda ? a.lambda * a.diameter[i] : s_gamma[ti];
                // the method's temperature at this timestep (a table when it varies)
                double kTv = a.kT, nz = a.use_lambda ? 0.0 : s_noise[ti];
                if (a.kT_hdr) {
                    const size_t r = kT_row(a, ts);
                    kTv = a.kT_tab[r];
                    nz = a.noise_tab[r * a.ntypes + ti];
                }
                const double c = a.noiseless ? 0.0 : (a.use_lambda ? sqrt(6.0 * gam * kTv / a.dt) : nz);
                const bool mover = in_group(a, ti);
                double ux, uy, uz;
                flow_at(a.flow, p.y, ux, uy, uz);
                double r0, r1, r2;
                if constexpr (INTEG == MD_INTEG_LANGEVIN) {
                    uniform3(AZP_RNG_LANGEVIN_FLOW, ts, a.seed, tg, -c, c - (-c), r0, r1, r2);
                    double4_32a v = a.vel[i];
                    const double minv = 1.0 / v.w;
                    const double ax = (Fx + (r0 - gam * (v.x - ux))) * minv;
                    const double ay = (Fy + (r1 - gam * (v.y - uy))) * minv;
                    const double az = (Fz + (r2 - gam * (v.z - uz))) * minv;
                    const double h = 0.5 * a.dt;
                    if (mover) {
                        v.x += h * ax;
                        v.y += h * ay;
                        v.z += h * az;
                    }
                    if (a.next) {
                        // step one of the next timestep with the acceleration just computed
                        if (mover) {
                            p.x += (v.x + h * ax) * a.dt;
                            p.y += (v.y + h * ay) * a.dt;
                            p.z += (v.z + h * az) * a.dt;
                            v.x += h * ax;
                            v.y += h * ay;
                            v.z += h * az;
                        }
                        moved = true;
                    } else if (mover) {
                        a.accel[3 * i] = ax;
                        a.accel[3 * i + 1] = ay;
                        a.accel[3 * i + 2] = az;
                    }
                    a.vel[i] = v;
                } else {
                    uniform3(AZP_RNG_BROWNIAN_FLOW, ts, a.seed, tg, -c, c - (-c), r0, r1, r2);
                    double dx = (ux + (Fx + r0) / gam) * a.dt;
                    double dy = (uy + (Fy + r1) / gam) * a.dt;
                    double dz = (uz + (Fz + r2) / gam) * a.dt;
                    if (a.max_disp > 0.0) {
                        dx = fmin(fmax(dx, -a.max_disp), a.max_disp);
                        dy = fmin(fmax(dy, -a.max_disp), a.max_disp);
                        dz = fmin(fmax(dz, -a.max_disp), a.max_disp);
                    }
                    if (mover) {
                        p.x += dx;
                        p.y += dy;
                        p.z += dz;
                    }
                    moved = true;
                }
                if (moved) {
                    int wx = 0, wy = 0, wz = 0;
                    wrap1(p.x, wx, a.L[0], a.lo[0], a.hi[0]);
                    wrap1(p.y, wy, a.L[1], a.lo[1], a.hi[1]);
                    wrap1(p.z, wz, a.L[2], a.lo[2], a.hi[2]);
                    if (wx | wy | wz) {
                        a.image[3 * i] += wx;
                        a.image[3 * i + 1] += wy;
                        a.image[3 * i + 2] += wz;
                    }
                    a.pos_next[i] = p;
                    uint4 f;
                    f.x = to_fixed(p.x, a.Linv[0]);
                    f.y = to_fixed(p.y, a.Linv[1]);
                    f.z = to_fixed(p.z, a.Linv[2]);
                    f.w = ti;
                    a.fix_next[i] = f;
                    want_rebuild = displaced(f, a.fix_build[i], a.sfix, a.disp_thresh2);
                    if (!(isfinite(p.x) && isfinite(p.y) && isfinite(p.z))) atomicOr(&a.flags[1], AZP_EBIT_NONFINITE);
                }
            }
        }
    }
    if constexpr (INTEG != MD_FORCES_ONLY) {
        if (__any_sync(0xffffffffu, want_rebuild) && (threadIdx.x & 31) == 0) atomicOr(&a.flags[0], 1u);
        // the last block to finish advances the timestep and arms the next rebuild
        __syncthreads();
        if (threadIdx.x == 0) {
            __threadfence();
            const uint32_t t = atomicAdd(&a.flags[4], 1u);
            if (t == gridDim.x - 1) {
                __threadfence();
                const uint32_t req = atomicAdd(&a.flags[0], 0u) && !atomicAdd(&a.flags[1], 0u);
                if (a.set_cond) cudaGraphSetConditional(a.next_cond, req ? 1u : 0u);
                a.flags[4] = 0u;
                *a.d_timestep_rw = *a.d_timestep_rw + 1ull;
            }
        }
    }
}

// ---------------------------------------------------------------- FP32-force step
// State: 64-bit fixed positions (fix = high words, lo = low words) and
// float-float velocities (fixed64.cuh). Pair and bond arithmetic in FP32 on the
// exact integer displacement of the high words, compensated force / energy sums;
// the r_cut decision is the oracle's FP64 one within 4e-6 of r_cut^2, on the
// full 64-bit positions. Integration with FP32 increments accumulated exactly
// (positions) or in float-float (velocities): no FP64 instruction per particle.

// |x_i - x_j|^2 < rc2 exactly as the FP64 oracle decides it, on the 64-bit positions
AZP_D bool inside_exact(const MDArgs& a, uint32_t i, uint32_t j, double rc2)
{
    const uint4 hi = a.fix[i], hj = a.fix[j];
    const uint4 li = a.flo[i], lj = a.flo[j];
    const double vx = min_image1(fx_to_double(fx_join(hi.x, li.x), a.l64[0]) - fx_to_double(fx_join(hj.x, lj.x), a.l64[0]),
                                 a.L[0], a.Linv[0]);
    const double vy = min_image1(fx_to_double(fx_join(hi.y, li.y), a.l64[1]) - fx_to_double(fx_join(hj.y, lj.y), a.l64[1]),
                                 a.L[1], a.Linv[1]);
    const double vz = min_image1(fx_to_double(fx_join(hi.z, li.z), a.l64[2]) - fx_to_double(fx_join(hj.z, lj.z), a.l64[2]),
                                 a.L[2], a.Linv[2]);
    return rsq_exact(vx, vy, vz) < rc2;
}

// exact minimum-image displacement of one axis from the 64-bit fixed positions
// (the wrapping 64-bit difference), in FP64 (one rounding)
AZP_D double fx_disp(uint32_t hi_i, uint32_t lo_i, uint32_t hi_j, uint32_t lo_j, double l64)
{
    const long long d = (long long)((unsigned long long)fx_join(hi_i, lo_i) - (unsigned long long)fx_join(hi_j, lo_j));
    return (double)d * l64;
}

// r^2 of the displacement between two fixed-point positions (high words): in a
// cubic box (AZP_FX_IRSQ=1, the default) the exact integer sum of squares of the
// int32 differences (each below 2^62, the sum below 2^64) rounded once to FP32
// and scaled by (L / 2^32)^2 held as a float pair; otherwise the sum of squares of
// the FP32 components. The integer form's r^2 is about three times closer (1.2e-7
// against 3.4e-7 relative), which r^-14 and the bond polynomial amplify: on the
// melt at N = 1M the force error against the FP64 oracle was 8.2e-6 to 1.07e-5
// over the end states of the bench runs with the FP32 components (over the 1e-5
// budget once) and 5.8-6.1e-6 with the integer form, for a step kernel about
// 9 % longer (0.090 -> 0.098 ms).
#ifndef AZP_FX_IRSQ
#define AZP_FX_IRSQ 1
#endif
AZP_D float fx_rsq(const MDArgs& a, const uint4& fi, const uint4& fj, float dx, float dy, float dz)
{
#if AZP_FX_IRSQ
    if (a.cubic) {
        const long long ix = (int32_t)(fi.x - fj.x), iy = (int32_t)(fi.y - fj.y), iz = (int32_t)(fi.z - fj.z);
        const unsigned long long q = (unsigned long long)(ix * ix) + (unsigned long long)(iy * iy) +
                                     (unsigned long long)(iz * iz);
        // (the conversion runs on the FP64 pipe, 32 % busy; a shifted 32-bit
        // conversion on other pipes measured slower, 0.102 against 0.098 ms)
        const float qf = __ull2float_rn(q);
        return fmaf(qf, a.s2h, qf * a.s2l);
    }
#endif
    return dx * dx + dy * dy + dz * dz;
}

// r^2 and the contact difference dq = c^2 - r^2 of a colloid point-sphere or
// sphere-sphere pair, each rounded once to FP32, for PE::eval_gap.
// AZP_COLLOID_GAP 2 (default; cubic boxes): from the 64-bit displacement rounded
// to 2^-32 L, whose integer sum of squares q (below 2^62 for a pair inside the
// half box) is exact, with c^2 held in the same units as the 64-bit integer
// contact_q (c^2 2^64 / L^2): dq = contact_q - q is an exact integer difference,
// so the cancellation costs nothing and no FP64 instruction runs. Other boxes, and
// AZP_COLLOID_GAP 1: in FP64 from the exact 64-bit displacement. Measured on the
// colloid mixture (N = 262,144, 5000 Brownian steps): FP64 841 timesteps/s, force
// error 6.7e-6; integer 968, 7.2e-6; the FP32 forms on the FP32 r^2 (0) 1,399 but
// 1.1e-5, over the 1e-5 budget; the exact difference only for r^2 < 2 c^2 1,015,
// 8.2e-6.
#ifndef AZP_COLLOID_GAP
#define AZP_COLLOID_GAP 2
#endif
// the integer r^2, in units of (L / 2^32)^2, of the 64-bit fixed-point
// displacement rounded to 2^-32 L per axis; exact, and below 2^62 for a pair
// inside the half box
AZP_D long long fx_rsq_rounded(const uint4& fi, const uint4& li, const uint4& fj, const uint4& lj)
{
    const auto axis = [](uint32_t hi_i, uint32_t lo_i, uint32_t hi_j, uint32_t lo_j) -> long long {
        const unsigned long long d = (unsigned long long)fx_join(hi_i, lo_i) - (unsigned long long)fx_join(hi_j, lo_j);
        return (long long)(d + 0x80000000ull) >> 32;
    };
    const long long ix = axis(fi.x, li.x, fj.x, lj.x), iy = axis(fi.y, li.y, fj.y, lj.y),
                    iz = axis(fi.z, li.z, fj.z, lj.z);
    return ix * ix + iy * iy + iz * iz;
}
template<class PE>
AZP_D void gap_args(const MDArgs& a, const uint4& fi, const uint4& fj, uint32_t i, uint32_t j, uint32_t tp,
                    float& rsq, float& dq)
{
    const uint4 li = __ldg(a.flo + i), lj = __ldg(a.flo + j);
#if AZP_COLLOID_GAP == 2
    if (a.contact_q) {
        const long long q = fx_rsq_rounded(fi, li, fj, lj);
        const long long dqi = __ldg(a.contact_q + tp) - q;
        const float qf = __ll2float_rn(q), df = __ll2float_rn(dqi);
        rsq = fmaf(qf, a.s2h, qf * a.s2l);
        dq = fmaf(df, a.s2h, df * a.s2l);
        return;
    }
#endif
    const double vx = fx_disp(fi.x, li.x, fj.x, lj.x, a.l64[0]);
    const double vy = fx_disp(fi.y, li.y, fj.y, lj.y, a.l64[1]);
    const double vz = fx_disp(fi.z, li.z, fj.z, lj.z, a.l64[2]);
    const double rsq_d = vx * vx + vy * vy + vz * vz;
    rsq = (float)rsq_d;
    dq = (float)(PE::contact2(a.pair_table + (size_t)tp * PAIR_TBL) - rsq_d);
}

// ONE: a single-type system; the type pair is 0 at compile time, so the record
// lookups resolve to the caller's registers
template<class PE, bool ONE = false>
AZP_D void pair_term_fx(const MDArgs& a, const uint4& fi, const uint4& fj, uint32_t i, uint32_t j,
                        const float* s_rec, const double* s_rc2, AccFx& acc, bool vir)
{
    const float dx = (float)(int32_t)(fi.x - fj.x) * a.sfix[0];
    const float dy = (float)(int32_t)(fi.y - fj.y) * a.sfix[1];
    const float dz = (float)(int32_t)(fi.z - fj.z) * a.sfix[2];
    const float rsq = fx_rsq(a, fi, fj, dx, dy, dz);
    const uint32_t tp = ONE ? 0u : fi.w * a.ntypes + fj.w;
    const float* rec = s_rec + (size_t)tp * PAIR_TBL;
    const float* cut = rec + PAIR_REC;
    const float rc2 = cut[0];
    if (rsq >= rc2 * 1.000004f || !PE::enabled(rec)) return;
    if (rsq >= rc2 * 0.999996f && !inside_exact(a, i, j, s_rc2[tp])) return;
    float fdr, e;
    if constexpr (has_gap_form<PE>::value) {
        if (AZP_COLLOID_GAP && PE::gap_form(rec)) {
            // the cancelling contact difference (colloid point-sphere and
            // sphere-sphere forms) formed exactly
            float rg, dq;
            gap_args<PE>(a, fi, fj, i, j, tp, rg, dq);
            PE::eval_gap(rec, rg, dq, fdr, e);
        } else {
            PE::eval(rec, rsq, fdr, e);
        }
    } else {
        PE::eval(rec, rsq, fdr, e);
    }
    e -= rec[PE::SHIFT_SLOT];
    xplor(cut, rsq, fdr, e);
    if (a.fcapf > 0.0f && fdr * fdr * rsq > a.fcapf * a.fcapf) fdr = copysignf(a.fcapf * rsqrtf(rsq), fdr);
    acc.add(dx, dy, dz, fdr, e, vir);
}

// pair_term_fx for a candidate that may be a padding slot (ok false) or lie
// outside r_cut: the evaluator runs on every lane (at r_cut where the pair does
// not count) and the pair's terms are masked, so a batch has no per-lane exits;
// only the rare candidate in the band around r_cut takes the exact FP64 branch
template<class PE, bool TILE = false, bool ONE = false>
AZP_D void pair_term_fx_masked(const MDArgs& a, const uint4& fi, const uint4& fj, uint32_t i, uint32_t ent, bool ok,
                               const float* s_rec, const double* s_rc2, AccFx& acc, bool vir,
                               const uint32_t* trec = nullptr)
{
    // the particle index of the entry, needed only on the rare exact paths
    const auto jof = [&]() -> uint32_t {
        if constexpr (TILE) return tile_decode(trec, ent);
        return ent;
    };
    const float dx = (float)(int32_t)(fi.x - fj.x) * a.sfix[0];
    const float dy = (float)(int32_t)(fi.y - fj.y) * a.sfix[1];
    const float dz = (float)(int32_t)(fi.z - fj.z) * a.sfix[2];
    const float rsq = fx_rsq(a, fi, fj, dx, dy, dz);
    const uint32_t tp = ONE ? 0u : fi.w * a.ntypes + fj.w;
    const float* rec = s_rec + (size_t)tp * PAIR_TBL;
    const float* cut = rec + PAIR_REC;
    const float rc2 = cut[0];
    const bool on = ok && PE::enabled(rec);
    bool in = on && rsq < rc2 * 0.999996f;
    if (on && !in && rsq < rc2 * 1.000004f) in = inside_exact(a, i, jof(), s_rc2[tp]);
    const float rs = in ? rsq : rc2;
    float fdr, e;
    if constexpr (has_gap_form<PE>::value && AZP_COLLOID_GAP != 0) {
        // the cancelling contact difference of the colloid point-sphere and
        // sphere-sphere forms formed exactly for a pair inside r_cut (a masked
        // slot takes any finite gap); every lane then runs one evaluation of its
        // own form, so a warp never runs a gap form twice
        float rg = rs, dq = 0.0f;
        if (PE::gap_form(rec)) {
            dq = PE::contact2_f(rec) - rs;
            if (in) gap_args<PE>(a, fi, fj, i, jof(), tp, rg, dq);
        }
        PE::eval_any(rec, rg, dq, fdr, e);
    } else {
        PE::eval(rec, rs, fdr, e);
    }
    e -= rec[PE::SHIFT_SLOT];
    xplor(cut, rs, fdr, e);
    if (a.fcapf > 0.0f && fdr * fdr * rs > a.fcapf * a.fcapf) fdr = copysignf(a.fcapf * rsqrtf(rs), fdr);
    acc.add(dx, dy, dz, in ? fdr : 0.0f, in ? e : 0.0f, vir);
}

// DPD pair in the FP32-force step: FP32 on the exact fixed-point displacement,
// FP64 from the full 64-bit positions within 0.2 % of r_cut^2 (the weight
// (1 - r / r_cut)^(s/2) is steep there, and the cutoff decision is the oracle's);
// velocities from the step's snapshot (float4: v, 1/m)
template<bool ONE = false>
AZP_D void pair_term_dpd_fx(const MDArgs& a, const uint4& fi, const uint4& fj, uint32_t i, uint32_t j,
                            const float* s_rec, const double* s_rc2, AccFx& acc, bool vir, const float4& vi,
                            uint32_t tgi, uint32_t k0, uint32_t k1)
{
    const float dx = (float)(int32_t)(fi.x - fj.x) * a.sfix[0];
    const float dy = (float)(int32_t)(fi.y - fj.y) * a.sfix[1];
    const float dz = (float)(int32_t)(fi.z - fj.z) * a.sfix[2];
    const float rs = fx_rsq(a, fi, fj, dx, dy, dz);
    const uint32_t tp = ONE ? 0u : fi.w * a.ntypes + fj.w;
    const float* rec = s_rec + (size_t)tp * PAIR_TBL;
    const float rc2 = rec[PAIR_REC];
    if (!(rc2 > 0.0f) || rs >= rc2 * 1.000004f) return;
    const float4 vj = reinterpret_cast<const float4*>(a.dvel)[j];
    const uint32_t tgj = a.tag[j];
    if (rs >= rc2 * 0.998f && a.contact_q) {
        // within 0.2 % of r_cut^2 in a cubic box: the cutoff decided and 1 - r / r_cut
        // formed from the exact integer difference r_cut^2 - r^2, the rest in FP32
        const long long q = fx_rsq_rounded(fi, a.flo[i], fj, a.flo[j]);
        const long long dqi = __ldg(a.contact_q + tp) - q;
        if (dqi <= 0) return;
        const float qf = __ll2float_rn(q), df = __ll2float_rn(dqi);
        const float r2 = fmaf(qf, a.s2h, qf * a.s2l), dq = fmaf(df, a.s2h, df * a.s2l);
        const float rcinv = rec[0], rc = rec[1], A = rec[2];
        const float rinv = rsqrtf(r2);
        const float x = dq * rcinv / (rc + r2 * rinv);  // 1 - r / r_cut = (r_cut^2 - r^2) / (r_cut (r_cut + r))
        const float dot = dx * (vi.x - vj.x) + dy * (vi.y - vj.y) + dz * (vi.z - vj.z);
        const float fc = A * x * rinv;
        const float wR = dpd_weight_engine_f(x, rec[4]) * rinv;
        const Philox4 ph = philox4x32_10(0u, min(tgi, tgj), max(tgi, tgj), 0u, k0, k1);
        const float alpha = -1.0f + 2.0f * open01f(ph.v[0]);
        const float fdr = fc - rec[3] * wR * wR * dot + rec[5] * wR * alpha;
        const float e = A * rc * x - 0.5f * A * rcinv * dq;
        acc.add_split(dx, dy, dz, fdr, fc, e, vir);
        return;
    }
    if (rs >= rc2 * 0.998f) {
        const uint4 li = a.flo[i], lj = a.flo[j];
        const double ddx = min_image1(fx_to_double(fx_join(fi.x, li.x), a.l64[0]) - fx_to_double(fx_join(fj.x, lj.x), a.l64[0]),
                                      a.L[0], a.Linv[0]);
        const double ddy = min_image1(fx_to_double(fx_join(fi.y, li.y), a.l64[1]) - fx_to_double(fx_join(fj.y, lj.y), a.l64[1]),
                                      a.L[1], a.Linv[1]);
        const double ddz = min_image1(fx_to_double(fx_join(fi.z, li.z), a.l64[2]) - fx_to_double(fx_join(fj.z, lj.z), a.l64[2]),
                                      a.L[2], a.Linv[2]);
        double fdr, fc, e;
        if (dpd_term_fp64(a.pair_table + (size_t)tp * PAIR_TBL, s_rc2[tp], ddx, ddy, ddz, (double)(vi.x - vj.x),
                          (double)(vi.y - vj.y), (double)(vi.z - vj.z), k0, k1, tgi, tgj, fdr, fc, e))
            acc.add_split((float)ddx, (float)ddy, (float)ddz, (float)fdr, (float)fc, (float)e, vir);
        return;
    }
    const float rcinv = rec[0], A = rec[2];
    const float rinv = rsqrtf(rs);
    const float r = rs * rinv;
    const float dot = dx * (vi.x - vj.x) + dy * (vi.y - vj.y) + dz * (vi.z - vj.z);
    const float fc = A * (rinv - rcinv);
    const float wR = dpd_weight_engine_f(fmaxf(1.0f - r * rcinv, 0.0f), rec[4]) * rinv;
    const Philox4 ph = philox4x32_10(0u, min(tgi, tgj), max(tgi, tgj), 0u, k0, k1);
    const float alpha = -1.0f + 2.0f * open01f(ph.v[0]);
    const float fdr = fc - rec[3] * wR * wR * dot + rec[5] * wR * alpha;
    const float e = A * (rec[1] - r) - 0.5f * A * rcinv * (rc2 - rs);
    acc.add_split(dx, dy, dz, fdr, fc, e, vir);
}

template<class BE, bool ONE = false>
AZP_D void bond_term_fx(const MDArgs& a, const uint4& fi, const uint4& fj, uint32_t btype, const float* s_bond,
                        AccFx& acc, bool vir)
{
    const float dx = (float)(int32_t)(fi.x - fj.x) * a.sfix[0];
    const float dy = (float)(int32_t)(fi.y - fj.y) * a.sfix[1];
    const float dz = (float)(int32_t)(fi.z - fj.z) * a.sfix[2];
    const float rsq = fx_rsq(a, fi, fj, dx, dy, dz);
    float fdr, en;
    if (!BE::eval_f(s_bond + (ONE ? 0u : btype) * BOND_F, rsq, fdr, en)) {
        atomicOr(&a.flags[1], AZP_EBIT_BOND);
        return;
    }
    acc.add(dx, dy, dz, fdr, en, vir);
}

// image-unwrapped displacement of one axis from the 64-bit fixed positions
// (hi, lo words) and the image difference: the wrapping 64-bit difference is
// the minimum image; w = +-1 where the exact difference overflowed it; the
// result is (minimum image) + (img_i - img_j + w) L, in FP32
AZP_D float unwrapped_fx(uint32_t hi_i, uint32_t lo_i, uint32_t hi_j, uint32_t lo_j, int dimg, float sfix)
{
    const long long qi = fx_join(hi_i, lo_i), qj = fx_join(hi_j, lo_j);
    const long long dq = (long long)((unsigned long long)qi - (unsigned long long)qj);
    const int w = (qi >= 0 && qj < 0 && dq < 0) ? 1 : ((qi < 0 && qj >= 0 && dq >= 0) ? -1 : 0);
    const float dmin =
        ((float)(int)(dq >> 32) + (float)(unsigned)((unsigned long long)dq & 0xffffffffull) * 2.3283064365386963e-10f) *
        sfix;
    // sfix = L 2^-32 rounded to float, so sfix 2^32 is L rounded to float
    return dmin + (float)(dimg + w) * (sfix * 4294967296.0f);
}

// one ImageHarmonic bond of particle i (fixed words fi / li, images g[3] of the
// step's start) with partner j in the FP32-force step
template<class BE, bool ONE = false>
AZP_D void bond_term_fx_image(const MDArgs& a, const uint4& fi, const uint4& li, const int* g, uint32_t j,
                              uint32_t btype, const float* s_bond, AccFx& acc, bool vir)
{
    const uint4 fj = __ldg(a.fix + j);
    const uint4 lj = __ldg(a.flo + j);
    const int* gj = a.img0 + 3 * (size_t)j;
    const float dx = unwrapped_fx(fi.x, li.x, fj.x, lj.x, g[0] - __ldg(gj), a.sfix[0]);
    const float dy = unwrapped_fx(fi.y, li.y, fj.y, lj.y, g[1] - __ldg(gj + 1), a.sfix[1]);
    const float dz = unwrapped_fx(fi.z, li.z, fj.z, lj.z, g[2] - __ldg(gj + 2), a.sfix[2]);
    const float rsq = dx * dx + dy * dy + dz * dz;
    float fdr, en;
    if (!BE::eval_f(s_bond + (ONE ? 0u : btype) * BOND_F, rsq, fdr, en)) {
        atomicOr(&a.flags[1], AZP_EBIT_BOND);
        return;
    }
    acc.add(dx, dy, dz, fdr, en, vir);
}

// the last block to finish advances the timestep and arms the next rebuild
AZP_D void finish_step(const MDArgs& a, bool want_rebuild)
{
    if (__any_sync(0xffffffffu, want_rebuild) && (threadIdx.x & 31) == 0) atomicOr(&a.flags[0], 1u);
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        const uint32_t t = atomicAdd(&a.flags[4], 1u);
        if (t == gridDim.x - 1) {
            __threadfence();
            const uint32_t req = atomicAdd(&a.flags[0], 0u) && !atomicAdd(&a.flags[1], 0u);
            if (a.set_cond) cudaGraphSetConditional(a.next_cond, req ? 1u : 0u);
            a.flags[4] = 0u;
            *a.d_timestep_rw = *a.d_timestep_rw + 1ull;
        }
    }
}

// neighbours gathered per batch: the list indices of a batch are loaded first,
// then their positions, so each thread keeps this many gathers in flight
#ifndef AZP_FX_BATCH
#define AZP_FX_BATCH 4
#endif
constexpr int FX_BATCH = AZP_FX_BATCH;
// Resident blocks per SM the FP32-force step is compiled for (the register cap):
// with the FP32-component r^2, 5 (48 registers) for the plain single-type step of
// the light evaluators, whose few spilled bytes cost less than the extra resident
// warps gain (measured on the melt at N = 1M: 0.0946 -> 0.0897 ms); 4 (64
// registers) for the rest, which would spill hundreds of bytes at 48 (Colloid,
// DPD, energy-writing launches), and for every step with the integer r^2.
// AZP_FX_MIN_BLOCKS overrides both.
template<class PE> struct fx_light : std::false_type {};
template<> struct fx_light<PerturbedLJ> : std::true_type {};
template<> struct fx_light<ExpandedYukawa> : std::true_type {};
template<> struct fx_light<Hertz> : std::true_type {};
template<> struct fx_light<NoPair> : std::true_type {};
template<class PE, bool OUT, bool ONE>
constexpr int fx_min_blocks()
{
#ifdef AZP_FX_MIN_BLOCKS
    return AZP_FX_MIN_BLOCKS;
#else
    // with the integer r^2 (more registers live) 4 blocks measured faster
    return (ONE && !OUT && fx_light<PE>::value && FX_BLOCK == 256 && !AZP_FX_IRSQ) ? 5 : 4;
#endif
}

// neighbour list entries of the next batch loaded while the current batch is
// evaluated (1), or at the top of each batch (0)
#ifndef AZP_FX_PIPE
#define AZP_FX_PIPE 0
#endif

// prefetch of the DRAM rows a warp's particles read (0 off, 1 into L1, 2 into L2)
#ifndef AZP_FX_PREFETCH
#define AZP_FX_PREFETCH 1
#endif
// neighbour batches walked to the warp's longest row with masked lanes instead of
// per-lane loop exits and early returns
#ifndef AZP_FX_UNIFORM
#define AZP_FX_UNIFORM 1
#endif

// the per-particle rows of step two / step one (velocity record, low position
// words, build shadow, tag) copied into shared memory by cp.async at the start of
// the step, so that their DRAM latency passes while the neighbour loop runs (1),
// or loaded where they are used (0)
#ifndef AZP_FX_STAGE
#define AZP_FX_STAGE 1
#endif

// per-thread asynchronous global -> shared copies (completed by cp_async_wait_all
// in the issuing thread, which alone reads what it copied)
AZP_D void cp_async16(void* smem, const void* g)
{
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"((uint32_t)__cvta_generic_to_shared(smem)), "l"(g)
                 : "memory");
}
AZP_D void cp_async4(void* smem, const void* g)
{
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"((uint32_t)__cvta_generic_to_shared(smem)), "l"(g)
                 : "memory");
}
AZP_D void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
AZP_D void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;" ::: "memory"); }

AZP_D void prefetch_line(const void* p)
{
#if AZP_FX_PREFETCH == 1
    asm volatile("prefetch.L1 [%0];" ::"l"(p));
#elif AZP_FX_PREFETCH == 2
    asm volatile("prefetch.L2 [%0];" ::"l"(p));
#else
    (void)p;
#endif
}

// Prefetch, by one instruction per lane, the lines of the warp's particles
// [i0, i_last] that the step reads from DRAM (velocities, low position words,
// build shadow, tags, bond counts, the first two bond-table columns) and the
// first nmax columns of their list rows, so that those latencies overlap at
// the start instead of chaining behind the neighbour loop. Addresses stay
// inside the arrays: every one is clamped to the warp's last particle.
AZP_D void prefetch_warp_rows(const MDArgs& a, uint32_t i0, uint32_t i_last, uint32_t nmax, bool bonds, bool rows)
{
    const uint32_t lane = threadIdx.x & 31u;
    if (lane < nmax) {
        prefetch_line(a.nbrs + (size_t)lane * a.N + i0);
        prefetch_line(a.nbrs + (size_t)lane * a.N + i_last);
    }
    const void* p = nullptr;
    if (!rows && lane < 18u) {
        // the integration rows are staged in shared memory instead
    } else if (lane < 8u) {
        p = a.velf + min(i0 + lane * 4u, i_last);
    } else if (lane < 12u) {
        p = a.flo + min(i0 + (lane - 8u) * 8u, i_last);
    } else if (lane < 16u) {
        p = a.fix_build + min(i0 + (lane - 12u) * 8u, i_last);
    } else if (lane < 18u) {
        p = a.tag + (lane == 16u ? i0 : i_last);
    } else if (bonds && lane < 20u) {
        p = a.bt_n + (lane == 18u ? i0 : i_last);
    } else if (bonds && lane < 26u) {
        const uint32_t c = (lane - 20u) / 3u, part = (lane - 20u) % 3u;
        p = a.bt + (size_t)c * a.N + min(i0 + part * 16u, i_last);
    }
    if (p) prefetch_line(p);
}

// ONE: single-type system, records from the kernel arguments (no shared-memory
// tables, no block barrier before the work)
// TILE (single-type systems, TILE_P particles per block, one thread each): the
// block's neighbour ranges are staged in shared memory first and the list
// entries address them there (celllist.cuh, TILE_GLOBAL entries are gathered)
template<class PE, class BE, int INTEG, bool OUT, bool ONE, bool TILE = false>
__global__ void __launch_bounds__(FX_BLOCK, (fx_min_blocks<PE, OUT, ONE>())) k_md_step_fx(MDArgs a)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const uint32_t nt2 = a.ntypes * a.ntypes;
    double* s_rc2 = reinterpret_cast<double*>(smem_raw);
    float* s_rec = reinterpret_cast<float*>(s_rc2 + nt2);
    float* s_bond = s_rec + nt2 * PAIR_TBL;
    float* s_gamma = s_bond + a.nbondtypes * BOND_F;
    float* s_noise = s_gamma + a.ntypes;
    const uint4* s_tile = reinterpret_cast<const uint4*>(smem_raw);
    const uint32_t* trec = nullptr;
    // single-type systems: the records copied from the kernel arguments into
    // registers (every lookup below has a compile-time index; no address of the
    // kernel argument is taken, so it is not copied to local memory)
    float one_rec[ONE ? PAIR_TBL : 1], one_bond[ONE ? BOND_F : 1], one_gamma = 0.0f, one_noise = 0.0f;
    double one_rc2 = 0.0;
    if constexpr (ONE) {
#pragma unroll
        for (int k = 0; k < PAIR_TBL; ++k) one_rec[k] = a.rec0[k];
#pragma unroll
        for (int k = 0; k < BOND_F; ++k) one_bond[k] = a.bond0[k];
        one_rc2 = a.rc2_0;
        one_gamma = a.gamma0;
        one_noise = a.noise0;
        s_rc2 = &one_rc2;
        s_rec = one_rec;
        s_bond = one_bond;
        s_gamma = &one_gamma;
        s_noise = &one_noise;
        if constexpr (TILE) {
            // stage the block's neighbour ranges: coalesced 16-byte copies
            trec = a.tile + (size_t)blockIdx.x * TILE_REC;
            const uint32_t nr = __ldg(trec);
            uint4* st = reinterpret_cast<uint4*>(smem_raw);
            for (uint32_t k = 0; k < nr; ++k) {
                const uint32_t b = __ldg(trec + 2 + 3 * k), e = __ldg(trec + 3 + 3 * k), off = __ldg(trec + 4 + 3 * k);
                for (uint32_t q = threadIdx.x; q < e - b; q += blockDim.x) st[off + q] = __ldg(a.fix + b + q);
            }
            __syncthreads();
        }
    } else {
        if (!std::is_same<PE, NoPair>::value)
            for (uint32_t t = threadIdx.x; t < nt2 * PAIR_TBL; t += blockDim.x) {
                s_rec[t] = (float)a.pair_table[t];
                if (t % PAIR_TBL == PAIR_REC) s_rc2[t / PAIR_TBL] = a.pair_table[t];
            }
        if (!std::is_same<BE, NoBond>::value)
            for (uint32_t t = threadIdx.x; t < a.nbondtypes; t += blockDim.x)
                BE::prepare_f(a.bond_params + (size_t)t * AZP_BOND_PARAM_DOUBLES, s_bond + (size_t)t * BOND_F);
        if (INTEG != MD_FORCES_ONLY && !a.use_lambda)
            for (uint32_t t = threadIdx.x; t < a.ntypes; t += blockDim.x) {
                s_gamma[t] = (float)a.gamma[t];
                s_noise[t] = (float)a.noise[t];
            }
        __syncthreads();
    }

    const uint32_t tpp = (uint32_t)a.tpp;
    const uint32_t gid = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t i = gid >> a.tpp_shift;
    const uint32_t sub = gid & (tpp - 1u);
    const bool active = i < a.N;
    constexpr bool vir = OUT;
#if AZP_FX_STAGE
    constexpr bool STAGE = INTEG != MD_FORCES_ONLY;
    constexpr bool STAGE_V = INTEG == MD_INTEG_LANGEVIN;
#else
    constexpr bool STAGE = false, STAGE_V = false;
#endif
    __shared__ __align__(32) VelFF st_vel[STAGE_V ? FX_BLOCK : 1];
    __shared__ __align__(16) uint4 st_lo[STAGE ? FX_BLOCK : 1];
    __shared__ __align__(16) uint4 st_fb[STAGE ? FX_BLOCK : 1];
    __shared__ uint32_t st_tag[STAGE ? FX_BLOCK : 1];
    if constexpr (STAGE) {
        if (active && sub == 0) {
            if constexpr (STAGE_V) {
                cp_async16(&st_vel[threadIdx.x].h, &a.velf[i].h);
                cp_async16(&st_vel[threadIdx.x].l, &a.velf[i].l);
            }
            cp_async16(&st_lo[threadIdx.x], a.flo + i);
            cp_async16(&st_fb[threadIdx.x], a.fix_build + i);
            cp_async4(&st_tag[threadIdx.x], a.tag + i);
            cp_async_commit();
        }
    }
    AccFx acc;
    uint4 fi = make_uint4(0u, 0u, 0u, 0u);
    uint32_t n = 0u;
    if constexpr (!std::is_same<PE, NoPair>::value) n = active ? min(__ldg(a.counts + i), a.max_nn) : 0u;
#if AZP_FX_PREFETCH || AZP_FX_UNIFORM
    // the warp's longest list row
    const uint32_t nmax = __reduce_max_sync(0xffffffffu, n);
#endif
#if AZP_FX_PREFETCH
    {
        const uint32_t i0 = (blockIdx.x * blockDim.x + (threadIdx.x & ~31u)) >> a.tpp_shift;
        if (i0 < a.N) {
            const uint32_t i_last = min(i0 + (32u >> a.tpp_shift) - 1u, a.N - 1u);
            prefetch_warp_rows(a, i0, i_last, std::is_same<PE, NoPair>::value ? 0u : nmax,
                               !std::is_same<BE, NoBond>::value, !AZP_FX_STAGE || INTEG == MD_FORCES_ONLY);
        }
    }
#endif
    if (active) {
        fi = __ldg(a.fix + i);
        // ---------------------------------------------------------------- pair
        if constexpr (!std::is_same<PE, NoPair>::value) {
            const uint32_t* col = a.nbrs + i;
            uint32_t k0 = 0, k1 = 0, tgi = 0;
            float4 vi = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            if constexpr (std::is_same<PE, DpdEngine>::value) {
                dpd_key(a, force_timestep<INTEG>(a), k0, k1);
                tgi = __ldg(a.tag + i);
                vi = reinterpret_cast<const float4*>(a.dvel)[i];
            }
#if AZP_FX_UNIFORM
            // every lane walks to the warp's longest row; slots past a lane's own
            // row are masked (no per-lane loop exit)
            const uint32_t kend = std::is_same<PE, DpdEngine>::value ? n : nmax;
#else
            const uint32_t kend = n;
#endif
#if AZP_FX_PIPE
            // the list entries of the first batch; each later batch's entries are
            // loaded while the current batch is evaluated
            uint32_t jn[FX_BATCH];
#pragma unroll
            for (int u = 0; u < FX_BATCH; ++u) {
                const uint32_t k = sub + u * tpp;
                jn[u] = k < n ? __ldg(col + (size_t)k * a.N) : (TILE ? (TILE_GLOBAL | i) : i);
            }
#endif
            for (uint32_t kb = sub; kb < kend; kb += FX_BATCH * tpp) {
                uint32_t jj[FX_BATCH];
                uint4 fj[FX_BATCH];
#if AZP_FX_PIPE
#pragma unroll
                for (int u = 0; u < FX_BATCH; ++u) jj[u] = jn[u];
#else
#pragma unroll
                for (int u = 0; u < FX_BATCH; ++u) {
                    const uint32_t k = kb + u * tpp;
                    jj[u] = k < n ? __ldg(col + (size_t)k * a.N) : (TILE ? (TILE_GLOBAL | i) : i);
                }
#endif
                if constexpr (TILE) {
#pragma unroll
                    for (int u = 0; u < FX_BATCH; ++u)
                        fj[u] = (jj[u] & TILE_GLOBAL) ? __ldg(a.fix + (jj[u] & ~TILE_GLOBAL)) : s_tile[jj[u]];
                } else {
#pragma unroll
                    for (int u = 0; u < FX_BATCH; ++u) fj[u] = __ldg(a.fix + jj[u]);
                }
#if AZP_FX_PIPE
#pragma unroll
                for (int u = 0; u < FX_BATCH; ++u) {
                    const uint32_t k = kb + (FX_BATCH + u) * tpp;
                    jn[u] = k < n ? __ldg(col + (size_t)k * a.N) : (TILE ? (TILE_GLOBAL | i) : i);
                }
#endif
#pragma unroll
                for (int u = 0; u < FX_BATCH; ++u) {
                    if constexpr (std::is_same<PE, DpdEngine>::value) {
                        if (kb + u * tpp < n)
                            pair_term_dpd_fx<ONE>(a, fi, fj[u], i, jj[u], s_rec, s_rc2, acc, vir, vi, tgi, k0, k1);
                    } else {
#if AZP_FX_UNIFORM
                        pair_term_fx_masked<PE, TILE, ONE>(a, fi, fj[u], i, jj[u], kb + u * tpp < n, s_rec, s_rc2,
                                                           acc, vir, trec);
#else
                        if (kb + u * tpp < n) pair_term_fx<PE, ONE>(a, fi, fj[u], i, jj[u], s_rec, s_rc2, acc, vir);
#endif
                    }
                }
                acc.commit(vir);
            }
        }
        // ---------------------------------------------------------------- bonds
        if constexpr (bond_uses_image<BE>::value) {
            const uint32_t nb = __ldg(a.bt_n + i);
            const uint4 li = __ldg(a.flo + i);
            const int g[3] = {__ldg(a.img0 + 3 * (size_t)i), __ldg(a.img0 + 3 * (size_t)i + 1),
                              __ldg(a.img0 + 3 * (size_t)i + 2)};
            for (uint32_t k = sub; k < nb; k += tpp) {
                const uint2 e = __ldg(a.bt + (size_t)k * a.N + i);
                bond_term_fx_image<BE, ONE>(a, fi, li, g, e.x, e.y, s_bond, acc, vir);
                acc.commit(vir);
            }
        } else if constexpr (!std::is_same<BE, NoBond>::value) {
            const uint32_t nb = __ldg(a.bt_n + i);
            for (uint32_t k0 = sub; k0 < nb; k0 += 2u * tpp) {
                const uint32_t k1 = k0 + tpp;
                const uint2 e0 = __ldg(a.bt + (size_t)k0 * a.N + i);
                const uint2 e1 = k1 < nb ? __ldg(a.bt + (size_t)k1 * a.N + i) : make_uint2(i, 0u);
                const uint4 f0 = __ldg(a.fix + e0.x);
                const uint4 f1 = __ldg(a.fix + e1.x);
                bond_term_fx<BE, ONE>(a, fi, f0, e0.y, s_bond, acc, vir);
                if (k1 < nb) bond_term_fx<BE, ONE>(a, fi, f1, e1.y, s_bond, acc, vir);
                acc.commit(vir);
            }
        }
    }
    if (tpp > 1) acc.reduce((int)tpp, vir);

    bool want_rebuild = false;
    if (active && sub == 0) {
        float fb[3] = {0.0f, 0.0f, 0.0f}, ub = 0.0f;
        if (a.bar_geom >= 0)
            // the barrier's force joins the net force (src/HarmonicBarrier.h:149-180)
            barrier_fx(a, fi, *a.d_timestep + (INTEG == MD_INTEG_LANGEVIN ? 1ull : 0ull), fb, ub);
        // the walls' force and energy (k_walls_fx, launched right before the step)
        const float4 fw = a.wall_kind >= 0 ? a.wall_f[i] : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        if constexpr (OUT) {
            a.out_force[i] = make_double4_32a(acc.Fx() + fb[0] + fw.x, acc.Fy() + fb[1] + fw.y,
                                              acc.Fz() + fb[2] + fw.z, acc.U() + ub + fw.w);
            double wv[6];
            for (int c = 0; c < 6; ++c) wv[c] = (double)acc.w[c];
            if (a.wall_kind >= 0) {
                // the wall virial F_a x_b (FP32 position: 2^-24 relative)
                const float x = (float)(int32_t)fi.x * a.sfix[0], y = (float)(int32_t)fi.y * a.sfix[1],
                            z = (float)(int32_t)fi.z * a.sfix[2];
                wv[0] += fw.x * x;
                wv[1] += fw.x * y;
                wv[2] += fw.x * z;
                wv[3] += fw.y * y;
                wv[4] += fw.y * z;
                wv[5] += fw.z * z;
            }
            for (int c = 0; c < 6; ++c) a.out_virial[(size_t)c * a.N + i] = wv[c];
        }
        if constexpr (INTEG != MD_FORCES_ONLY) {
            if constexpr (STAGE) cp_async_wait_all();
            const unsigned long long ts = *a.d_timestep;
            const uint32_t ti = fi.w;
            const uint32_t tg = STAGE ? st_tag[threadIdx.x] : __ldg(a.tag + i);
            const float fx = acc.fx.s + (acc.fx.c + (fb[0] + fw.x));
            const float fy = acc.fy.s + (acc.fy.c + (fb[1] + fw.y));
            const float fz = acc.fz.s + (acc.fz.c + (fb[2] + fw.z));
            const uint32_t tix = ONE ? 0u : ti;
            const float gam = a.use_lambda ? a.lambdaf * (float)a.diameter[i] : s_gamma[tix];
            // the method's temperature at this timestep (a table when it varies)
            float kTv = a.kTf, nz = a.use_lambda ? 0.0f : s_noise[tix];
            if (a.kT_hdr) {
                const size_t r = kT_row(a, ts);
                kTv = (float)a.kT_tab[r];
                nz = (float)a.noise_tab[r * a.ntypes + ti];
            }
            const float c = a.noiseless ? 0.0f : (a.use_lambda ? sqrtf(6.0f * gam * kTv / a.dtf) : nz);
            const bool mover = in_group(a, ti);
            float ux, uy, uz;
            flow_at_ff(a.flowf, (float)(int32_t)fi.y * a.sfix[1], ux, uy, uz);
            const float dt = a.dtf;
            float r0, r1, r2, ddx = 0.0f, ddy = 0.0f, ddz = 0.0f;
            bool moved = false;
            if constexpr (INTEG == MD_INTEG_LANGEVIN) {
                uniform3f(AZP_RNG_LANGEVIN_FLOW, ts, a.seed, tg, -c, 2.0f * c, r0, r1, r2);
                VelFF v = STAGE_V ? st_vel[threadIdx.x] : a.velf[i];
                const float minv = mover ? v.h.w : 0.0f;  // a particle outside the group keeps its velocity
                const float ax = (fx + (r0 - gam * (v.h.x - ux))) * minv;
                const float ay = (fy + (r1 - gam * (v.h.y - uy))) * minv;
                const float az = (fz + (r2 - gam * (v.h.z - uz))) * minv;
                if (a.next) {
                    // v(t + dt/2) = v(t - dt/2) + dt a: the half kick of step two and of
                    // step one; then x += v(t + dt/2) dt
                    const float kx = dt * ax, ky = dt * ay, kz = dt * az;
                    const float mdt = mover ? dt : 0.0f;
                    ddx = (v.h.x + kx) * mdt;
                    ddy = (v.h.y + ky) * mdt;
                    ddz = (v.h.z + kz) * mdt;
                    ff_add(v.h.x, v.l.x, kx);
                    ff_add(v.h.y, v.l.y, ky);
                    ff_add(v.h.z, v.l.z, kz);
                    moved = true;
                } else {
                    const float h = 0.5f * dt;
                    ff_add(v.h.x, v.l.x, h * ax);
                    ff_add(v.h.y, v.l.y, h * ay);
                    ff_add(v.h.z, v.l.z, h * az);
                    a.accel[3 * i] = ax;
                    a.accel[3 * i + 1] = ay;
                    a.accel[3 * i + 2] = az;
                }
                a.velf[i] = v;
            } else {
                uniform3f(AZP_RNG_BROWNIAN_FLOW, ts, a.seed, tg, -c, 2.0f * c, r0, r1, r2);
                const float gi = 1.0f / gam;
                const float mdt = mover ? dt : 0.0f;
                ddx = (ux + (fx + r0) * gi) * mdt;
                ddy = (uy + (fy + r1) * gi) * mdt;
                ddz = (uz + (fz + r2) * gi) * mdt;
                if (a.max_dispf > 0.0f) {
                    const float m = a.max_dispf;
                    ddx = fminf(fmaxf(ddx, -m), m);
                    ddy = fminf(fmaxf(ddy, -m), m);
                    ddz = fminf(fmaxf(ddz, -m), m);
                }
                moved = true;
            }
            if (moved) {
                uint4 lo = STAGE ? st_lo[threadIdx.x] : a.flo[i];
                bool bad = false;
                const int wx = fx_advance(fi.x, lo.x, ddx, a.s64h[0], a.s64l[0], bad);
                const int wy = fx_advance(fi.y, lo.y, ddy, a.s64h[1], a.s64l[1], bad);
                const int wz = fx_advance(fi.z, lo.z, ddz, a.s64h[2], a.s64l[2], bad);
                if (wx | wy | wz) {
                    a.image[3 * i] += wx;
                    a.image[3 * i + 1] += wy;
                    a.image[3 * i + 2] += wz;
                }
                a.fix_next[i] = fi;
                a.flo_next[i] = lo;
                want_rebuild = displaced(fi, STAGE ? st_fb[threadIdx.x] : a.fix_build[i], a.sfix, a.disp_thresh2);
                if (bad) atomicOr(&a.flags[1], AZP_EBIT_NONFINITE);
            }
        }
    }
    if constexpr (INTEG != MD_FORCES_ONLY) finish_step(a, want_rebuild);
}

template<class PE, class BE, typename R, int INTEG>
int launch_md_t(const MDArgs& a, cudaStream_t s)
{
    const size_t threads = (size_t)a.N * a.tpp;
    const int bs = std::is_same<R, float>::value ? FX_BLOCK : MD_BLOCK;
    const uint32_t blocks = (uint32_t)((threads + bs - 1) / bs);
    if (blocks == 0) return AZP_OK;
    const size_t nt2 = (size_t)a.ntypes * a.ntypes;
    if constexpr (std::is_same<R, float>::value) {
        const size_t smem = nt2 * sizeof(double) + nt2 * PAIR_TBL * sizeof(float) +
                            (size_t)a.nbondtypes * BOND_F * sizeof(float) + 2 * a.ntypes * sizeof(float);
        constexpr bool can_tile = !std::is_same<PE, NoPair>::value && !std::is_same<PE, DpdEngine>::value &&
                                  !bond_uses_image<BE>::value;
        auto k = a.out ? (a.one_type ? k_md_step_fx<PE, BE, INTEG, true, true> : k_md_step_fx<PE, BE, INTEG, true, false>)
                       : (a.one_type ? k_md_step_fx<PE, BE, INTEG, false, true>
                                     : k_md_step_fx<PE, BE, INTEG, false, false>);
        size_t smem_k = smem;
        if (a.tile && (FX_BLOCK != (int)TILE_P || a.tpp != 1 || !a.one_type || !can_tile))
            return record_error(AZP_ERR_UNSUPPORTED, "k_md_step_fx: tiles need one type, 256-thread blocks, tpp 1");
        if constexpr (can_tile) {
            if (a.tile) {
                k = a.out ? k_md_step_fx<PE, BE, INTEG, true, true, true> : k_md_step_fx<PE, BE, INTEG, false, true, true>;
                smem_k = (size_t)TILE_CAP * sizeof(uint4);
            }
        }
        if (smem_k > 32 * 1024)
            AZP_CUDA_TRY(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_k));
        k<<<blocks, FX_BLOCK, smem_k, s>>>(a);
        AZP_CHECK_LAUNCH("k_md_step_fx");
    } else {
        const size_t smem = nt2 * sizeof(double) + 2 * a.ntypes * sizeof(double) + nt2 * PAIR_TBL * sizeof(R) +
                            (size_t)a.nbondtypes * AZP_BOND_PARAM_DOUBLES * sizeof(R);
        auto k = k_md_step<PE, BE, R, INTEG>;
        if (smem > 48 * 1024) AZP_CUDA_TRY(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        k<<<blocks, MD_BLOCK, smem, s>>>(a);
        AZP_CHECK_LAUNCH("k_md_step");
    }
    return AZP_OK;
}

template<class PE, class BE, typename R>
int launch_md_integ(int integ, const MDArgs& a, cudaStream_t s)
{
    switch (integ) {
    case MD_INTEG_LANGEVIN: return launch_md_t<PE, BE, R, MD_INTEG_LANGEVIN>(a, s);
    case MD_INTEG_BROWNIAN: return launch_md_t<PE, BE, R, MD_INTEG_BROWNIAN>(a, s);
    case MD_FORCES_ONLY: return launch_md_t<PE, BE, R, MD_FORCES_ONLY>(a, s);
    default: return AZP_ERR_INVALID;
    }
}

template<class PE>
int launch_md_pe(int bond_kind, int precision, int integ, const MDArgs& a, cudaStream_t s)
{
    if (precision == AZP_FP32) {
        switch (bond_kind) {
        case -1: return launch_md_integ<PE, NoBond, float>(integ, a, s);
        case AZP_BOND_QUARTIC: return launch_md_integ<PE, QuarticBond, float>(integ, a, s);
        case AZP_BOND_DOUBLE_WELL: return launch_md_integ<PE, DoubleWellBond, float>(integ, a, s);
        case AZP_BOND_IMAGE_HARMONIC: return launch_md_integ<PE, HarmonicBond, float>(integ, a, s);
        default: return AZP_ERR_INVALID;
        }
    }
    switch (bond_kind) {
    case -1: return launch_md_integ<PE, NoBond, double>(integ, a, s);
    case AZP_BOND_QUARTIC: return launch_md_integ<PE, QuarticBond, double>(integ, a, s);
    case AZP_BOND_DOUBLE_WELL: return launch_md_integ<PE, DoubleWellBond, double>(integ, a, s);
    case AZP_BOND_IMAGE_HARMONIC: return launch_md_integ<PE, HarmonicBond, double>(integ, a, s);
    default: return AZP_ERR_INVALID;
    }
}

// per-evaluator entry points, one per translation unit
int launch_md_nopair(int bond_kind, int precision, int integ, const MDArgs& a, cudaStream_t s);
int launch_md_plj(int bond_kind, int precision, int integ, const MDArgs& a, cudaStream_t s);
int launch_md_eyuk(int bond_kind, int precision, int integ, const MDArgs& a, cudaStream_t s);
int launch_md_hertz(int bond_kind, int precision, int integ, const MDArgs& a, cudaStream_t s);
int launch_md_colloid(int bond_kind, int precision, int integ, const MDArgs& a, cudaStream_t s);
int launch_md_dpd(int bond_kind, int precision, int integ, const MDArgs& a, cudaStream_t s);

}  // namespace azp
