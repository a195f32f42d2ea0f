// bond.cu -- bond forces from a per-particle bond table (replaces HOOMD's
// gpu_compute_bond_forces<Evaluator, 2> instantiated in
// src/PotentialBondGPUKernel.cu.inc:25-29).
//
// One thread per particle walks its own bonds (each bond appears on both of its
// particles): dx = x_i - x_j (minimum image), F_i += dx f/r, U_i += U/2,
// W_i += dx (x) dx f/(2r) -- the convention of src/ImagePotentialBondGPU.cuh:
// 180-244 with the minimum image instead of the image shift. With an image array
// (the ImageHarmonic bond, src/ImagePotentialBond.h:136-140) the displacement is
// the unwrapped one instead: dx = (x_i - x_j) + (img_i - img_j) L. A refusing
// evaluator sets AZP_EBIT_BOND in the error word (the reference sets *d_flags = 1).
#include "bond.cuh"
#include "evaluators.cuh"

namespace azp
{
constexpr int BOND_BLOCK = 256;
constexpr uint32_t MAX_BOND_TYPES = 64;

template<class Eval, typename R>
__global__ void __launch_bounds__(BOND_BLOCK) k_bond(BondArgs a)
{
    __shared__ R s_p[MAX_BOND_TYPES * AZP_BOND_PARAM_DOUBLES];
    // the caller's records (Eval::REC_DOUBLES each) zero-padded to 8 values
    for (uint32_t t = threadIdx.x; t < a.nbondtypes * AZP_BOND_PARAM_DOUBLES; t += blockDim.x) {
        const uint32_t b = t / AZP_BOND_PARAM_DOUBLES, m = t % AZP_BOND_PARAM_DOUBLES;
        s_p[t] = m < (uint32_t)Eval::REC_DOUBLES ? (R)a.params[(size_t)b * Eval::REC_DOUBLES + m] : R(0);
    }
    __syncthreads();
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.N) return;
    const uint32_t nb = a.n_bonds[i];
    if (nb == 0) return;
    R fx = 0, fy = 0, fz = 0, u = 0, w[6] = {0, 0, 0, 0, 0, 0};
    bool bad = false;
    if constexpr (std::is_same<R, double>::value) {
        const double4_32a pi = a.pos[i];
        for (uint32_t k = 0; k < nb; ++k) {
            const uint2 e = a.table[(size_t)k * a.N + i];
            const double4_32a pj = a.pos[e.x];
            double dx, dy, dz;
            if (a.image) {
                dx = (pi.x - pj.x) + (double)(a.image[3 * i] - a.image[3 * e.x]) * a.L[0];
                dy = (pi.y - pj.y) + (double)(a.image[3 * i + 1] - a.image[3 * e.x + 1]) * a.L[1];
                dz = (pi.z - pj.z) + (double)(a.image[3 * i + 2] - a.image[3 * e.x + 2]) * a.L[2];
            } else {
                dx = min_image1(pi.x - pj.x, a.L[0], a.Linv[0]);
                dy = min_image1(pi.y - pj.y, a.L[1], a.Linv[1]);
                dz = min_image1(pi.z - pj.z, a.L[2], a.Linv[2]);
            }
            const double rsq = rsq_exact(dx, dy, dz);
            double fdr, en;
            if (!Eval::eval(s_p + e.y * AZP_BOND_PARAM_DOUBLES, rsq, fdr, en)) {
                bad = true;
                continue;
            }
            fx += dx * fdr;
            fy += dy * fdr;
            fz += dz * fdr;
            u += 0.5 * en;
            const double h = 0.5 * fdr;
            w[0] += h * dx * dx;
            w[1] += h * dx * dy;
            w[2] += h * dx * dz;
            w[3] += h * dy * dy;
            w[4] += h * dy * dz;
            w[5] += h * dz * dz;
        }
    } else {
        // FP32 evaluation; displacement from the fixed-point shadow when the
        // caller has one, else from the FP64 minimum image
        const uint4 fi = a.fixed ? a.fixed[i] : make_uint4(0, 0, 0, 0);
        const double4_32a pi = (a.fixed && !a.image) ? make_double4_32a(0, 0, 0, 0) : a.pos[i];
        for (uint32_t k = 0; k < nb; ++k) {
            const uint2 e = a.table[(size_t)k * a.N + i];
            float dx, dy, dz;
            if (a.image) {
                const double4_32a pj = a.pos[e.x];
                dx = (float)((pi.x - pj.x) + (double)(a.image[3 * i] - a.image[3 * e.x]) * a.L[0]);
                dy = (float)((pi.y - pj.y) + (double)(a.image[3 * i + 1] - a.image[3 * e.x + 1]) * a.L[1]);
                dz = (float)((pi.z - pj.z) + (double)(a.image[3 * i + 2] - a.image[3 * e.x + 2]) * a.L[2]);
            } else if (a.fixed) {
                const uint4 fj = a.fixed[e.x];
                dx = (float)(int32_t)(fi.x - fj.x) * a.sfix[0];
                dy = (float)(int32_t)(fi.y - fj.y) * a.sfix[1];
                dz = (float)(int32_t)(fi.z - fj.z) * a.sfix[2];
            } else {
                const double4_32a pj = a.pos[e.x];
                dx = (float)min_image1(pi.x - pj.x, a.L[0], a.Linv[0]);
                dy = (float)min_image1(pi.y - pj.y, a.L[1], a.Linv[1]);
                dz = (float)min_image1(pi.z - pj.z, a.L[2], a.Linv[2]);
            }
            const float rsq = dx * dx + dy * dy + dz * dz;
            float fdr, en;
            if (!Eval::eval(s_p + e.y * AZP_BOND_PARAM_DOUBLES, rsq, fdr, en)) {
                bad = true;
                continue;
            }
            fx += dx * fdr;
            fy += dy * fdr;
            fz += dz * fdr;
            u += 0.5f * en;
            const float h = 0.5f * fdr;
            w[0] += h * dx * dx;
            w[1] += h * dx * dy;
            w[2] += h * dx * dz;
            w[3] += h * dy * dy;
            w[4] += h * dy * dz;
            w[5] += h * dz * dz;
        }
    }
    if (bad && a.err) atomicOr(a.err, AZP_EBIT_BOND);
    if constexpr (std::is_same<R, double>::value) {
        double4_32a* f = reinterpret_cast<double4_32a*>(a.force);
        double4_32a o = f[i];
        o.x += fx;
        o.y += fy;
        o.z += fz;
        o.w += u;
        f[i] = o;
        if (a.virial) {
            double* v = reinterpret_cast<double*>(a.virial);
            for (int c = 0; c < 6; ++c) v[(size_t)c * a.pitch + i] += w[c];
        }
    } else {
        float4* f = reinterpret_cast<float4*>(a.force);
        float4 o = f[i];
        o.x += fx;
        o.y += fy;
        o.z += fz;
        o.w += u;
        f[i] = o;
        if (a.virial) {
            float* v = reinterpret_cast<float*>(a.virial);
            for (int c = 0; c < 6; ++c) v[(size_t)c * a.pitch + i] += w[c];
        }
    }
}

template<class Eval>
int launch_b(int precision, const BondArgs& a, cudaStream_t s)
{
    const uint32_t blocks = (a.N + BOND_BLOCK - 1) / BOND_BLOCK;
    if (blocks == 0) return AZP_OK;
    if (precision == AZP_FP32)
        k_bond<Eval, float><<<blocks, BOND_BLOCK, 0, s>>>(a);
    else
        k_bond<Eval, double><<<blocks, BOND_BLOCK, 0, s>>>(a);
    AZP_CHECK_LAUNCH("k_bond");
    return AZP_OK;
}

int launch_bond(int kind, int precision, const BondArgs& a, cudaStream_t s)
{
    if (a.nbondtypes > MAX_BOND_TYPES) return AZP_ERR_INVALID;
    switch (kind) {
    case AZP_BOND_QUARTIC: return launch_b<QuarticBond>(precision, a, s);
    case AZP_BOND_DOUBLE_WELL: return launch_b<DoubleWellBond>(precision, a, s);
    case AZP_BOND_IMAGE_HARMONIC: return a.image ? launch_b<HarmonicBond>(precision, a, s) : AZP_ERR_INVALID;
    default: return AZP_ERR_INVALID;
    }
}

}  // namespace azp
