// pair.cu -- pair forces (replaces HOOMD's gpu_compute_pair_forces<Evaluator>
// that src/PotentialPairGPUKernel.cu.inc:25-28 instantiates per evaluator).
//
// TPP threads share one particle (TPP | 32); each walks every TPP-th neighbour and
// the group reduces force, energy and virial with warp shuffles. FP64 mode: FP64
// positions, minimum image by rint, FP64 evaluator. FP32 mode: the exact integer
// displacement of the fixed-point shadow converted once to float, FP32 evaluator,
// compensated force / energy sums, and the r_cut decision made in FP64 (same
// rounding as the oracle) whenever the FP32 rsq lies within 4e-6 of r_cut^2.
#include <cstring>
#include <vector>

#include "pair.cuh"

namespace azp
{
template<typename R> struct Vec4;
template<> struct Vec4<double> { using T = double4_32a; };
template<> struct Vec4<float> { using T = float4; };

template<class Eval, typename R> struct PairAccum;

// FP64 accumulator
template<class Eval> struct PairAccum<Eval, double> {
    double fx = 0, fy = 0, fz = 0, u = 0, w[6] = {0, 0, 0, 0, 0, 0};
    AZP_D void add(double dx, double dy, double dz, double fdr, double e)
    {
        fx += dx * fdr;
        fy += dy * fdr;
        fz += dz * fdr;
        u += 0.5 * e;
        const double h = 0.5 * fdr;
        w[0] += h * dx * dx;
        w[1] += h * dx * dy;
        w[2] += h * dx * dz;
        w[3] += h * dy * dy;
        w[4] += h * dy * dz;
        w[5] += h * dz * dz;
    }
    AZP_D void reduce(int tpp)
    {
        for (int m = tpp >> 1; m > 0; m >>= 1) {
            fx += __shfl_xor_sync(0xffffffffu, fx, m);
            fy += __shfl_xor_sync(0xffffffffu, fy, m);
            fz += __shfl_xor_sync(0xffffffffu, fz, m);
            u += __shfl_xor_sync(0xffffffffu, u, m);
#pragma unroll
            for (int c = 0; c < 6; ++c) w[c] += __shfl_xor_sync(0xffffffffu, w[c], m);
        }
    }
    AZP_D void store(const PairArgs& a, uint32_t i, bool virial)
    {
        reinterpret_cast<double4_32a*>(a.force)[i] = make_double4_32a(fx, fy, fz, u);
        if (virial) {
            double* v = reinterpret_cast<double*>(a.virial);
#pragma unroll
            for (int c = 0; c < 6; ++c) v[(size_t)c * a.pitch + i] = w[c];
        }
    }
};

// FP32 accumulator: force and energy compensated, virial plain
template<class Eval> struct PairAccum<Eval, float> {
    Comp fx{0.f, 0.f}, fy{0.f, 0.f}, fz{0.f, 0.f}, u{0.f, 0.f};
    float w[6] = {0, 0, 0, 0, 0, 0};
    AZP_D void add(float dx, float dy, float dz, float fdr, float e)
    {
        fx.add(dx * fdr);
        fy.add(dy * fdr);
        fz.add(dz * fdr);
        u.add(0.5f * e);
        const float h = 0.5f * fdr;
        w[0] += h * dx * dx;
        w[1] += h * dx * dy;
        w[2] += h * dx * dz;
        w[3] += h * dy * dy;
        w[4] += h * dy * dz;
        w[5] += h * dz * dz;
    }
    AZP_D static void comp_reduce(Comp& c, int m)
    {
        // combine two compensated partials: (s1 + c1) + (s2 + c2)
        const float s2 = __shfl_xor_sync(0xffffffffu, c.s, m);
        const float c2 = __shfl_xor_sync(0xffffffffu, c.c, m);
        c.add(s2);
        c.c += c2;
    }
    AZP_D void reduce(int tpp)
    {
        for (int m = tpp >> 1; m > 0; m >>= 1) {
            comp_reduce(fx, m);
            comp_reduce(fy, m);
            comp_reduce(fz, m);
            comp_reduce(u, m);
#pragma unroll
            for (int c = 0; c < 6; ++c) w[c] += __shfl_xor_sync(0xffffffffu, w[c], m);
        }
    }
    AZP_D void store(const PairArgs& a, uint32_t i, bool virial)
    {
        reinterpret_cast<float4*>(a.force)[i] = make_float4(fx.value(), fy.value(), fz.value(), u.value());
        if (virial) {
            float* v = reinterpret_cast<float*>(a.virial);
#pragma unroll
            for (int c = 0; c < 6; ++c) v[(size_t)c * a.pitch + i] = w[c];
        }
    }
};

constexpr int PAIR_BLOCK = 256;

// dynamic shared memory: the FP64 r_cut^2 of every type pair (exact decision),
// then the type-pair table converted to the arithmetic type R
template<typename R> inline size_t pair_smem_bytes(uint32_t ntypes)
{
    const size_t nt2 = (size_t)ntypes * ntypes;
    return nt2 * sizeof(double) + nt2 * PAIR_TBL * sizeof(R);
}

template<class Eval, typename R, int TPP, bool VIRIAL>
__global__ void __launch_bounds__(PAIR_BLOCK) k_pair(PairArgs a)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const uint32_t nt2 = a.ntypes * a.ntypes;
    double* s_rc2 = reinterpret_cast<double*>(smem_raw);
    R* s_rec = reinterpret_cast<R*>(smem_raw + nt2 * sizeof(double));
    for (uint32_t t = threadIdx.x; t < nt2 * PAIR_TBL; t += blockDim.x) {
        s_rec[t] = (R)a.table[t];
        if (t % PAIR_TBL == PAIR_REC) s_rc2[t / PAIR_TBL] = a.table[t];
    }
    __syncthreads();

    const uint32_t gid = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t i = gid / TPP;
    const uint32_t sub = gid % TPP;
    const bool active = i < a.N;
    PairAccum<Eval, R> acc;
    if (active) {
        const uint32_t n = min(a.counts[i], a.max_nn);
        if constexpr (std::is_same<R, double>::value) {
            const double4_32a pi = a.pos[i];
            const uint32_t ti = type_of(pi.w);
            for (uint32_t k = sub; k < n; k += TPP) {
                const uint32_t j = a.nbrs[(size_t)k * a.N + i];
                const double4_32a pj = a.pos[j];
                const double dx = min_image1(pi.x - pj.x, a.L[0], a.Linv[0]);
                const double dy = min_image1(pi.y - pj.y, a.L[1], a.Linv[1]);
                const double dz = min_image1(pi.z - pj.z, a.L[2], a.Linv[2]);
                // rounded like the oracle, so the r_cut decision is exact
                const double rsq = rsq_exact(dx, dy, dz);
                const uint32_t tp = ti * a.ntypes + type_of(pj.w);
                const R* rec = s_rec + (size_t)tp * PAIR_TBL;
                const R* cut = rec + PAIR_REC;
                if (!(rsq < (double)cut[0]) || !Eval::enabled(rec)) continue;
                R fdr, e;
                Eval::eval(rec, (R)rsq, fdr, e);
                e -= rec[Eval::SHIFT_SLOT];
                xplor(cut, (R)rsq, fdr, e);
                acc.add((R)dx, (R)dy, (R)dz, fdr, e);
            }
        } else {
            const uint4 fi = a.fixed[i];
            const uint32_t ti = fi.w;
            for (uint32_t k = sub; k < n; k += TPP) {
                const uint32_t j = a.nbrs[(size_t)k * a.N + i];
                const uint4 fj = a.fixed[j];
                const float dx = (float)(int32_t)(fi.x - fj.x) * a.sfix[0];
                const float dy = (float)(int32_t)(fi.y - fj.y) * a.sfix[1];
                const float dz = (float)(int32_t)(fi.z - fj.z) * a.sfix[2];
                const float rsq = dx * dx + dy * dy + dz * dz;
                const uint32_t tp = ti * a.ntypes + fj.w;
                const R* rec = s_rec + (size_t)tp * PAIR_TBL;
                const R* cut = rec + PAIR_REC;
                const float rc2 = (float)cut[0];
                if (rsq >= rc2 * 1.000004f || !Eval::enabled(rec)) continue;
                if (rsq >= rc2 * 0.999996f) {
                    // near r_cut: decide exactly as the FP64 oracle does
                    const double4_32a pi = a.pos[i];
                    const double4_32a pj = a.pos[j];
                    const double vx = min_image1(pi.x - pj.x, a.L[0], a.Linv[0]);
                    const double vy = min_image1(pi.y - pj.y, a.L[1], a.Linv[1]);
                    const double vz = min_image1(pi.z - pj.z, a.L[2], a.Linv[2]);
                    if (!(rsq_exact(vx, vy, vz) < s_rc2[tp])) continue;
                }
                R fdr, e;
                if constexpr (has_gap_form<Eval>::value) {
                    if (Eval::gap_form(rec)) {
                        // the cancelling contact difference from the FP64
                        // positions, rounded once (colloid point-sphere and
                        // sphere-sphere forms)
                        const double4_32a pi = a.pos[i];
                        const double4_32a pj = a.pos[j];
                        const double vx = min_image1(pi.x - pj.x, a.L[0], a.Linv[0]);
                        const double vy = min_image1(pi.y - pj.y, a.L[1], a.Linv[1]);
                        const double vz = min_image1(pi.z - pj.z, a.L[2], a.Linv[2]);
                        const double rsq_d = vx * vx + vy * vy + vz * vz;
                        const double dq = Eval::contact2(a.table + (size_t)tp * PAIR_TBL) - rsq_d;
                        Eval::eval_gap(rec, (float)rsq_d, (float)dq, fdr, e);
                    } else {
                        Eval::eval(rec, (R)rsq, fdr, e);
                    }
                } else {
                    Eval::eval(rec, (R)rsq, fdr, e);
                }
                e -= rec[Eval::SHIFT_SLOT];
                xplor(cut, (R)rsq, fdr, e);
                acc.add((R)dx, (R)dy, (R)dz, fdr, e);
            }
        }
    }
    if (TPP > 1) acc.reduce(TPP);
    if (active && sub == 0) acc.store(a, i, VIRIAL);
}

template<class Eval>
void fill_table(const double* params, const double* r_cut, const double* r_on, int mode, uint32_t ntypes,
                double* out)
{
    for (uint32_t t = 0; t < ntypes * ntypes; ++t) {
        double* rec = out + (size_t)t * PAIR_TBL;
        double p[4];
        load_pair_record<Eval>(params + (size_t)t * Eval::REC_DOUBLES, p);
        prepare_pair<Eval>(p, r_cut[t], r_on ? r_on[t] : 0.0, mode, rec, rec + PAIR_REC);
    }
}

template<class Eval>
__global__ void k_pair_table(const double* __restrict__ params, const double* __restrict__ r_cut,
                             const double* __restrict__ r_on, int mode, uint32_t ntypes, double* __restrict__ out)
{
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= ntypes * ntypes) return;
    double* rec = out + (size_t)t * PAIR_TBL;
    double p[4];
    load_pair_record<Eval>(params + (size_t)t * Eval::REC_DOUBLES, p);
    prepare_pair<Eval>(p, r_cut[t], r_on ? r_on[t] : 0.0, mode, rec, rec + PAIR_REC);
}

int launch_pair_table(int kind, const double* params, const double* r_cut, const double* r_on, int mode,
                      uint32_t ntypes, double* out, cudaStream_t s)
{
    if (ntypes == 0 || ntypes > MAX_PAIR_TYPES || mode < 0 || mode > 2) return AZP_ERR_INVALID;
    const uint32_t nt2 = ntypes * ntypes;
    const uint32_t b = (nt2 + 127) / 128;
    switch (kind) {
    case AZP_PAIR_PERTURBED_LJ: k_pair_table<PerturbedLJ><<<b, 128, 0, s>>>(params, r_cut, r_on, mode, ntypes, out); break;
    case AZP_PAIR_EXPANDED_YUKAWA: k_pair_table<ExpandedYukawa><<<b, 128, 0, s>>>(params, r_cut, r_on, mode, ntypes, out); break;
    case AZP_PAIR_HERTZ: k_pair_table<Hertz><<<b, 128, 0, s>>>(params, r_cut, r_on, mode, ntypes, out); break;
    case AZP_PAIR_COLLOID: k_pair_table<Colloid><<<b, 128, 0, s>>>(params, r_cut, r_on, mode, ntypes, out); break;
    default: return AZP_ERR_INVALID;
    }
    AZP_CHECK_LAUNCH("k_pair_table");
    return AZP_OK;
}

int build_pair_table(int kind, const double* params, const double* r_cut, const double* r_on, int mode,
                     uint32_t ntypes, double* out)
{
    if (ntypes == 0 || ntypes > MAX_PAIR_TYPES || mode < 0 || mode > 2) return AZP_ERR_INVALID;
    switch (kind) {
    case AZP_PAIR_PERTURBED_LJ: fill_table<PerturbedLJ>(params, r_cut, r_on, mode, ntypes, out); break;
    case AZP_PAIR_EXPANDED_YUKAWA: fill_table<ExpandedYukawa>(params, r_cut, r_on, mode, ntypes, out); break;
    case AZP_PAIR_HERTZ: fill_table<Hertz>(params, r_cut, r_on, mode, ntypes, out); break;
    case AZP_PAIR_COLLOID: fill_table<Colloid>(params, r_cut, r_on, mode, ntypes, out); break;
    default: return AZP_ERR_INVALID;
    }
    return AZP_OK;
}

template<class Eval, typename R, int TPP>
int launch_t(const PairArgs& a, cudaStream_t s)
{
    const size_t threads = (size_t)a.N * TPP;
    const uint32_t blocks = (uint32_t)((threads + PAIR_BLOCK - 1) / PAIR_BLOCK);
    const size_t smem = pair_smem_bytes<R>(a.ntypes);
    if (blocks == 0) return AZP_OK;
    if (a.virial) {
        auto k = k_pair<Eval, R, TPP, true>;
        AZP_CUDA_TRY(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        k<<<blocks, PAIR_BLOCK, smem, s>>>(a);
    } else {
        auto k = k_pair<Eval, R, TPP, false>;
        AZP_CUDA_TRY(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        k<<<blocks, PAIR_BLOCK, smem, s>>>(a);
    }
    AZP_CHECK_LAUNCH("k_pair");
    return AZP_OK;
}

template<class Eval, typename R>
int launch_tpp(int tpp, const PairArgs& a, cudaStream_t s)
{
    switch (tpp) {
    case 1: return launch_t<Eval, R, 1>(a, s);
    case 2: return launch_t<Eval, R, 2>(a, s);
    case 4: return launch_t<Eval, R, 4>(a, s);
    case 8: return launch_t<Eval, R, 8>(a, s);
    case 16: return launch_t<Eval, R, 16>(a, s);
    case 32: return launch_t<Eval, R, 32>(a, s);
    default: return AZP_ERR_INVALID;
    }
}

template<class Eval>
int launch_prec(int precision, int tpp, const PairArgs& a, cudaStream_t s)
{
    return precision == AZP_FP32 ? launch_tpp<Eval, float>(tpp, a, s) : launch_tpp<Eval, double>(tpp, a, s);
}

int launch_pair(int kind, int precision, int tpp, const PairArgs& a, cudaStream_t s)
{
    switch (kind) {
    case AZP_PAIR_PERTURBED_LJ: return launch_prec<PerturbedLJ>(precision, tpp, a, s);
    case AZP_PAIR_EXPANDED_YUKAWA: return launch_prec<ExpandedYukawa>(precision, tpp, a, s);
    case AZP_PAIR_HERTZ: return launch_prec<Hertz>(precision, tpp, a, s);
    case AZP_PAIR_COLLOID: return launch_prec<Colloid>(precision, tpp, a, s);
    default: return AZP_ERR_INVALID;
    }
}

}  // namespace azp
