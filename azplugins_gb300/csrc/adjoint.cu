// adjoint.cu -- reverse-mode (vector-Jacobian) kernels of the pair and bond
// forces, FP64: given dL/dF_i and dL/dU_i, the gradient of L with respect to
// the positions and to the parameter-record fields.
//
// For a listed pair (i, j) with d = x_i - x_j (minimum image), s = |d|^2, force
// F_i += phi(s) d, F_j -= phi(s) d and energy e(s) split in halves:
//   dL/dx_i += phi (G_i - G_j) + 2 phi'(s) ((G_i - G_j) . d) d - g phi d,
//   dL/dp   += 1/2 [ ((G_i - G_j) . d) dphi/dp + g de/dp ]      (per ordered pair)
// with G = dL/dF, g = (dL/dU_i + dL/dU_j) / 2 and e'(s) = -phi / 2. Each thread
// owns one particle of the full list, so no atomics; the parameter gradient is
// written per particle and summed by the caller (deterministic).
//
// PerturbedLennardJones has its derivatives written out (the fast path of the
// gradient workload); every other evaluator is differentiated exactly by
// evaluating its own templated code on forward-mode dual numbers (dual.cuh),
// seeded on rsq and on the four parameter-record fields.
#include "dual.cuh"
#include "evaluators.cuh"
#include "nlist_impl.cuh"
#include "pair.cuh"

namespace azp
{
using D5 = Dual<5>;  // d/ds, d/dp[0..3]
using D9 = Dual<9>;  // d/ds, d/dp[0..7] (bond records)

constexpr int ADJ_BLOCK = 128;

// dual records of every type pair: rec[PAIR_REC] then cut[CUT_REC], seeded on p
template<class Eval>
__global__ void k_pair_adj_table(const double* __restrict__ params, const double* __restrict__ r_cut,
                                 const double* __restrict__ r_on, int mode, uint32_t ntypes, D5* __restrict__ out)
{
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= ntypes * ntypes) return;
    D5 p[AZP_PAIR_PARAM_DOUBLES];
    for (int m = 0; m < AZP_PAIR_PARAM_DOUBLES; ++m) {
        p[m] = D5(m < Eval::REC_DOUBLES ? params[(size_t)t * Eval::REC_DOUBLES + m] : 0.0);
        p[m].d[1 + m] = 1.0;
    }
    D5* rec = out + (size_t)t * PAIR_TBL;
    prepare_pair_t<Eval, D5>(p, r_cut[t], r_on ? r_on[t] : 0.0, mode, rec, rec + PAIR_REC);
}

struct AdjArgs {
    const double4_32a* pos;
    const double4_32a* grad;  // dL/dF (x, y, z), dL/dU_i (w)
    uint32_t N, ntypes;
    double L[3], Linv[3];
    const uint32_t* counts;
    const uint32_t* nbrs;
    uint32_t max_nn;
    const D5* table;
    double* grad_pos;         // [N][3]
    double* grad_params;      // [N][4]
    int tpp;
    int xplor;                // smoothing active: every evaluator takes the dual path
};

// phi, phi' = dphi/ds, dphi/dp[m], de/dp[m] of one pair
struct PairDerivs {
    double phi, dphi_ds, dphi_dp[4], de_dp[4];
};

// PerturbedLennardJones, written out. p = (sigma_6, epsilon_x_4, lambda, rwcasq).
AZP_D PairDerivs plj_derivs(const D5* rec, double s)
{
    PairDerivs r;
    const double lj1 = rec[0].v, lj2 = rec[1].v, lam = rec[2].v, rwcasq = rec[3].v;
    // dlj/dp from the dual record: lj1 = e4 s6^2, lj2 = e4 s6
    const double dlj1_ds6 = rec[0].d[1], dlj1_de4 = rec[0].d[2];
    const double dlj2_ds6 = rec[1].d[1], dlj2_de4 = rec[1].d[2];
    const double x2 = 1.0 / s;
    const double r6 = x2 * x2 * x2;
    const double phi_lj = x2 * r6 * (12.0 * lj1 * r6 - 6.0 * lj2);
    const double e_lj = r6 * (lj1 * r6 - lj2);
    const double dphi_lj = x2 * x2 * r6 * (-84.0 * lj1 * r6 + 24.0 * lj2);
    const double dphi_dlj1 = 12.0 * x2 * r6 * r6, dphi_dlj2 = -6.0 * x2 * r6;
    const double de_dlj1 = r6 * r6, de_dlj2 = -r6;
    const double dphi_lj_ds6 = dphi_dlj1 * dlj1_ds6 + dphi_dlj2 * dlj2_ds6;
    const double dphi_lj_de4 = dphi_dlj1 * dlj1_de4 + dphi_dlj2 * dlj2_de4;
    const double de_lj_ds6 = de_dlj1 * dlj1_ds6 + de_dlj2 * dlj2_ds6;
    const double de_lj_de4 = de_dlj1 * dlj1_de4 + de_dlj2 * dlj2_de4;
    if (s < rwcasq) {
        // WCA core: U_LJ + eps (1 - lambda), eps = e4 / 4
        r.phi = phi_lj;
        r.dphi_ds = dphi_lj;
        r.dphi_dp[0] = dphi_lj_ds6;
        r.dphi_dp[1] = dphi_lj_de4;
        r.dphi_dp[2] = 0.0;
        r.de_dp[0] = de_lj_ds6;
        r.de_dp[1] = de_lj_de4 + rec[4].d[2];   // d wca_shift / d e4
        r.de_dp[2] = rec[4].d[3];               // d wca_shift / d lambda
    } else {
        r.phi = lam * phi_lj;
        r.dphi_ds = lam * dphi_lj;
        r.dphi_dp[0] = lam * dphi_lj_ds6;
        r.dphi_dp[1] = lam * dphi_lj_de4;
        r.dphi_dp[2] = phi_lj;
        r.de_dp[0] = lam * de_lj_ds6;
        r.de_dp[1] = lam * de_lj_de4;
        r.de_dp[2] = e_lj;
    }
    r.dphi_dp[3] = 0.0;  // rwcasq only moves the (continuous) branch point
    r.de_dp[3] = 0.0;
    // energy shift at r_cut (zero unless shifting)
    const D5& sh = rec[PerturbedLJ::SHIFT_SLOT];
    for (int m = 0; m < 4; ++m) r.de_dp[m] -= sh.d[1 + m];
    return r;
}

template<class Eval> AZP_D PairDerivs dual_derivs(const D5* rec, double s)
{
    PairDerivs r;
    D5 x(s);
    x.d[0] = 1.0;
    D5 f, e;
    Eval::eval(rec, x, f, e);
    e -= rec[Eval::SHIFT_SLOT];
    xplor(rec + PAIR_REC, x, f, e);  // no-op unless the type pair is smoothed
    r.phi = f.v;
    r.dphi_ds = f.d[0];
    for (int m = 0; m < 4; ++m) {
        r.dphi_dp[m] = f.d[1 + m];
        r.de_dp[m] = e.d[1 + m];
    }
    return r;
}

// WRITTEN: the hand-written PerturbedLennardJones derivatives (no smoothing);
// otherwise the dual-number path. Separate instantiations keep the dual
// records' registers out of the hand-written kernel.
template<class Eval, bool WRITTEN>
__global__ void __launch_bounds__(ADJ_BLOCK) k_pair_adjoint(AdjArgs a)
{
    const uint32_t gid = blockIdx.x * blockDim.x + threadIdx.x;
    const int tpp = a.tpp;
    const uint32_t i = gid / tpp;
    const uint32_t sub = gid % tpp;
    const bool active = i < a.N;
    double gx = 0, gy = 0, gz = 0, gp[4] = {0, 0, 0, 0};
    if (active) {
        const double4_32a pi = a.pos[i];
        const double4_32a Gi = a.grad[i];
        const uint32_t ti = type_of(pi.w);
        const uint32_t n = min(a.counts[i], a.max_nn);
        for (uint32_t k = sub; k < n; k += tpp) {
            const uint32_t j = a.nbrs[(size_t)k * a.N + i];
            const double4_32a pj = a.pos[j];
            const double dx = min_image1(pi.x - pj.x, a.L[0], a.Linv[0]);
            const double dy = min_image1(pi.y - pj.y, a.L[1], a.Linv[1]);
            const double dz = min_image1(pi.z - pj.z, a.L[2], a.Linv[2]);
            const double s = rsq_exact(dx, dy, dz);
            const uint32_t tp = ti * a.ntypes + type_of(pj.w);
            const D5* rec = a.table + (size_t)tp * PAIR_TBL;
            const D5* cut = rec + PAIR_REC;
            if (!(s < cut[0].v) || !Eval::enabled(rec)) continue;
            PairDerivs q;
            if constexpr (WRITTEN)
                q = plj_derivs(rec, s);
            else
                q = dual_derivs<Eval>(rec, s);
            const double4_32a Gj = a.grad[j];
            const double Gx = Gi.x - Gj.x, Gy = Gi.y - Gj.y, Gz = Gi.z - Gj.z;
            const double g = 0.5 * (Gi.w + Gj.w);
            const double Gdd = Gx * dx + Gy * dy + Gz * dz;
            const double c2 = 2.0 * q.dphi_ds * Gdd - g * q.phi;
            gx += q.phi * Gx + c2 * dx;
            gy += q.phi * Gy + c2 * dy;
            gz += q.phi * Gz + c2 * dz;
#pragma unroll
            for (int m = 0; m < 4; ++m) gp[m] += 0.5 * (Gdd * q.dphi_dp[m] + g * q.de_dp[m]);
        }
    }
    for (int m = tpp >> 1; m > 0; m >>= 1) {
        gx += __shfl_xor_sync(0xffffffffu, gx, m);
        gy += __shfl_xor_sync(0xffffffffu, gy, m);
        gz += __shfl_xor_sync(0xffffffffu, gz, m);
#pragma unroll
        for (int c = 0; c < 4; ++c) gp[c] += __shfl_xor_sync(0xffffffffu, gp[c], m);
    }
    if (active && sub == 0) {
        a.grad_pos[3 * (size_t)i] = gx;
        a.grad_pos[3 * (size_t)i + 1] = gy;
        a.grad_pos[3 * (size_t)i + 2] = gz;
        if (a.grad_params)
            for (int c = 0; c < 4; ++c) a.grad_params[4 * (size_t)i + c] = gp[c];
    }
}

// ---------------------------------------------------------------- bonds
struct BondAdjArgs {
    const double4_32a* pos;
    const double4_32a* grad;
    uint32_t N, nbondtypes;
    double L[3], Linv[3];
    const uint32_t* n_bonds;
    const uint2* table;
    const double* params;
    double* grad_pos;     // [N][3]
    double* grad_params;  // [N][8]
    uint32_t* err;
};

template<class Eval>
__global__ void __launch_bounds__(ADJ_BLOCK) k_bond_adjoint(BondAdjArgs a)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.N) return;
    const double4_32a pi = a.pos[i];
    const double4_32a Gi = a.grad[i];
    double gx = 0, gy = 0, gz = 0, gp[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    const uint32_t nb = a.n_bonds[i];
    for (uint32_t k = 0; k < nb; ++k) {
        const uint2 e2 = a.table[(size_t)k * a.N + i];
        const double4_32a pj = a.pos[e2.x];
        const double dx = min_image1(pi.x - pj.x, a.L[0], a.Linv[0]);
        const double dy = min_image1(pi.y - pj.y, a.L[1], a.Linv[1]);
        const double dz = min_image1(pi.z - pj.z, a.L[2], a.Linv[2]);
        D9 p[8];
        for (int m = 0; m < 8; ++m) {
            p[m] = D9(m < Eval::REC_DOUBLES ? a.params[(size_t)e2.y * Eval::REC_DOUBLES + m] : 0.0);
            p[m].d[1 + m] = 1.0;
        }
        D9 x(rsq_exact(dx, dy, dz));
        x.d[0] = 1.0;
        D9 f, e;
        if (!Eval::eval(p, x, f, e)) {
            if (a.err) atomicOr(a.err, AZP_EBIT_BOND);
            continue;
        }
        const double4_32a Gj = a.grad[e2.x];
        const double Gx = Gi.x - Gj.x, Gy = Gi.y - Gj.y, Gz = Gi.z - Gj.z;
        const double g = 0.5 * (Gi.w + Gj.w);
        const double Gdd = Gx * dx + Gy * dy + Gz * dz;
        const double c2 = 2.0 * f.d[0] * Gdd - g * f.v;
        gx += f.v * Gx + c2 * dx;
        gy += f.v * Gy + c2 * dy;
        gz += f.v * Gz + c2 * dz;
        for (int m = 0; m < 8; ++m) gp[m] += 0.5 * (Gdd * f.d[1 + m] + g * e.d[1 + m]);
    }
    a.grad_pos[3 * (size_t)i] = gx;
    a.grad_pos[3 * (size_t)i + 1] = gy;
    a.grad_pos[3 * (size_t)i + 2] = gz;
    if (a.grad_params)
        for (int m = 0; m < 8; ++m) a.grad_params[8 * (size_t)i + m] = gp[m];
}

template<class Eval>
int launch_adj(const azp_system* sys, azp_nlist* nl, const double* params, const double* r_cut, const double* r_on,
               int mode, const double* grad, double* grad_pos, double* grad_params, cudaStream_t s)
{
    const uint32_t nt2 = sys->ntypes * sys->ntypes;
    D5* table = reinterpret_cast<D5*>(nl->adj_table);
    k_pair_adj_table<Eval><<<(nt2 + 63) / 64, 64, 0, s>>>(params, r_cut, r_on, mode, sys->ntypes, table);
    AdjArgs a;
    a.pos = reinterpret_cast<const double4_32a*>(sys->pos);
    a.grad = reinterpret_cast<const double4_32a*>(grad);
    a.N = sys->N;
    a.ntypes = sys->ntypes;
    for (int d = 0; d < 3; ++d) {
        a.L[d] = sys->box.L[d];
        a.Linv[d] = 1.0 / sys->box.L[d];
    }
    a.counts = nl->counts;
    a.nbrs = nl->nbrs;
    a.max_nn = nl->max_nn;
    a.table = table;
    a.grad_pos = grad_pos;
    a.grad_params = grad_params;
    a.tpp = nl->tpp;
    a.xplor = mode == AZP_MODE_XPLOR;
    const size_t threads = (size_t)sys->N * a.tpp;
    const uint32_t blocks = (uint32_t)((threads + ADJ_BLOCK - 1) / ADJ_BLOCK);
    if (std::is_same<Eval, PerturbedLJ>::value && !a.xplor)
        k_pair_adjoint<PerturbedLJ, true><<<blocks, ADJ_BLOCK, 0, s>>>(a);
    else
        k_pair_adjoint<Eval, false><<<blocks, ADJ_BLOCK, 0, s>>>(a);
    AZP_CHECK_LAUNCH("k_pair_adjoint");
    return AZP_OK;
}

}  // namespace azp

extern "C" {

int azp_pair_adjoint(const azp_system* sys, azp_nlist* nl, int kind, const double* params, const double* r_cut,
                     const double* r_on, int shift_mode, const double* grad, double* grad_pos, double* grad_params,
                     void* stream)
{
    if (!sys || !nl || !params || !r_cut || !grad || !grad_pos) return AZP_ERR_INVALID;
    if (sys->N != nl->N || sys->ntypes != nl->ntypes || sys->ntypes == 0 || sys->ntypes > azp::MAX_PAIR_TYPES)
        return AZP_ERR_INVALID;
    if (shift_mode < AZP_MODE_NONE || shift_mode > AZP_MODE_XPLOR) return AZP_ERR_INVALID;
    if (sys->N == 0) return AZP_OK;
    cudaStream_t s = azp::as_stream(stream);
    switch (kind) {
    case AZP_PAIR_PERTURBED_LJ:
        return azp::launch_adj<azp::PerturbedLJ>(sys, nl, params, r_cut, r_on, shift_mode, grad, grad_pos, grad_params, s);
    case AZP_PAIR_EXPANDED_YUKAWA:
        return azp::launch_adj<azp::ExpandedYukawa>(sys, nl, params, r_cut, r_on, shift_mode, grad, grad_pos, grad_params, s);
    case AZP_PAIR_HERTZ:
        return azp::launch_adj<azp::Hertz>(sys, nl, params, r_cut, r_on, shift_mode, grad, grad_pos, grad_params, s);
    case AZP_PAIR_COLLOID:
        return azp::launch_adj<azp::Colloid>(sys, nl, params, r_cut, r_on, shift_mode, grad, grad_pos, grad_params, s);
    default: return AZP_ERR_INVALID;
    }
}

int azp_bond_adjoint(const azp_system* sys, const uint32_t* n_bonds, const uint32_t* table, int kind,
                     const double* params, uint32_t nbondtypes, const double* grad, double* grad_pos,
                     double* grad_params, uint32_t* err, void* stream)
{
    if (!sys || !n_bonds || !table || !params || !grad || !grad_pos || nbondtypes == 0) return AZP_ERR_INVALID;
    if (sys->N == 0) return AZP_OK;
    azp::BondAdjArgs a;
    a.pos = reinterpret_cast<const double4_32a*>(sys->pos);
    a.grad = reinterpret_cast<const double4_32a*>(grad);
    a.N = sys->N;
    a.nbondtypes = nbondtypes;
    for (int d = 0; d < 3; ++d) {
        a.L[d] = sys->box.L[d];
        a.Linv[d] = 1.0 / sys->box.L[d];
    }
    a.n_bonds = n_bonds;
    a.table = reinterpret_cast<const uint2*>(table);
    a.params = params;
    a.grad_pos = grad_pos;
    a.grad_params = grad_params;
    a.err = err;
    cudaStream_t s = azp::as_stream(stream);
    const uint32_t blocks = (sys->N + azp::ADJ_BLOCK - 1) / azp::ADJ_BLOCK;
    switch (kind) {
    case AZP_BOND_QUARTIC: azp::k_bond_adjoint<azp::QuarticBond><<<blocks, azp::ADJ_BLOCK, 0, s>>>(a); break;
    case AZP_BOND_DOUBLE_WELL: azp::k_bond_adjoint<azp::DoubleWellBond><<<blocks, azp::ADJ_BLOCK, 0, s>>>(a); break;
    default: return AZP_ERR_INVALID;
    }
    AZP_CHECK_LAUNCH("k_bond_adjoint");
    return AZP_OK;
}

}  // extern "C"
