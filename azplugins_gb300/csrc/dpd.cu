// dpd.cu -- DPD with a general weight function: conservative, dissipative and
// random pair forces over the full list (replaces HOOMD's gpu_compute_dpd_forces
// instantiated for the evaluator in src/PotentialPairDPDThermoGPUKernel.cu.inc:21-24).
//
// Per listed pair with r < r_cut (src/DPDPairEvaluatorGeneralWeight.h:165-255):
//   F_C / r = A (1/r - 1/r_cut)
//   F_D / r = -gamma w(r) (dx . dv) / r^2,          w = (1 - r / r_cut)^s
//   F_R / r = sqrt(6 kT gamma / dt) sqrt(w) alpha / r, alpha uniform in (-1, 1)
//   U       = A (r_cut - r) - A (r_cut^2 - r^2) / (2 r_cut), halved per particle
// with dx = x_i - x_j (minimum image), dv = v_i - v_j; the virial takes the
// conservative force only. alpha is one draw per pair from the Philox stream
// (AZP_RNG_DPD_GENERAL_WEIGHT, timestep, seed) at counter {0, min tag, max tag, 0}
// (the reference's Seed(id, timestep, seed) + Counter(i, j), :227-233), so i and
// j draw the same number and the pair forces are equal and opposite.
//
// FP64 mode follows the oracle's operation order. FP32 mode: displacement from
// the fixed-point shadow (exact integer difference), velocities from an FP32
// shadow, FP32 arithmetic, the draw at 24-bit resolution, compensated force and
// energy sums; pairs within 0.2 % of r_cut^2 in FP64 (see the kernel).
#include "nlist_impl.cuh"
#include "pair.cuh"
#include "philox.cuh"

namespace azp
{
namespace
{
constexpr int DPD_BLOCK = 256;
// per type pair: rcutsq, rcinv, rc, A, gamma, s/2, sigma_R = sqrt(6 kT gamma / dt), -
constexpr int DPD_TBL = 8;
// in-range partners a thread queues before evaluating them (FP32 path)
constexpr uint32_t DPD_QUEUE = 16;

struct DpdArgs {
    const double4_32a* pos;
    const uint4* fixed;
    const double4_32a* vel;
    const float4* vel_f;
    const uint32_t* tag;
    uint32_t N, ntypes;
    double L[3], Linv[3];
    float sfix[3];
    float s2h, s2l;       // (L / 2^32)^2 as a float pair (cubic boxes)
    const uint32_t* counts;
    const uint32_t* nbrs;
    uint32_t max_nn;
    const double* table;  // [ntypes^2][DPD_TBL]
    uint32_t k0, k1;      // Philox key of (id, timestep, seed)
    void* force;
    void* virial;
    uint32_t pitch;
};

// o[7]: r_cut^2 in the units of the integer r^2 of the fixed-point words,
// (2^32 / L)^2 (u2 > 0: a cubic box), as the bits of a 64-bit integer; 0 without
__global__ void k_dpd_table(const double* __restrict__ params, const double* __restrict__ r_cut, uint32_t nt2,
                            double kT, double dt, double u2, double* __restrict__ out)
{
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nt2) return;
    const double rc2 = r_cut[t] * r_cut[t];
    const double rcinv = 1.0 / sqrt(rc2);
    const double A = params[4 * t], gamma = params[4 * t + 1], s = params[4 * t + 2];
    double* o = out + (size_t)t * DPD_TBL;
    o[0] = r_cut[t] > 0.0 ? rc2 : 0.0;
    o[1] = rcinv;
    o[2] = 1.0 / rcinv;
    o[3] = A;
    o[4] = gamma;
    o[5] = 0.5 * s;
    o[6] = sqrt(6.0 * kT * gamma / dt);
    o[7] = __longlong_as_double(u2 > 0.0 && r_cut[t] > 0.0 ? __double2ll_rn(rc2 * u2) : 0ll);
}

__global__ void k_vel_f(const double4_32a* __restrict__ vel, uint32_t N, float4* __restrict__ out)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= N) return;
    const double4_32a v = vel[i];
    out[i] = make_float4((float)v.x, (float)v.y, (float)v.z, 0.0f);
}

// (1 - r / r_cut)^(s/2): the exponents s/2 = 1/4, 1/2, 1 (s = 1/2, 1, 2, the
// usual choices) as square roots, which agree with pow to an ulp or two and
// avoid its cost (in FP64 a pow costs as much as the rest of the pair); any
// other exponent through pow
AZP_D double dpd_weight(double x, double h)
{
    if (h == 0.5) return sqrt(x);
    if (h == 0.25) return sqrt(sqrt(x));
    if (h == 1.0) return x;
    return pow(x, h);
}

AZP_D float dpd_weight_f(float x, float h)
{
    if (h == 0.5f) return sqrtf(x);
    if (h == 0.25f) return sqrtf(sqrtf(x));
    if (h == 1.0f) return x;
    return powf(x, h);
}

// alpha of a pair, FP64: the first 64-bit word of the pair's Philox block
AZP_D double dpd_alpha(uint32_t k0, uint32_t k1, uint32_t ti, uint32_t tj)
{
    const uint32_t oi = min(ti, tj), oj = max(ti, tj);
    const Philox4 r = philox4x32_10(0u, oi, oj, 0u, k0, k1);
    return -1.0 + 2.0 * open01(r.v[0], r.v[1]);
}

// the same draw at 24-bit resolution (the top 24 bits of the word)
AZP_D float dpd_alpha_f(uint32_t k0, uint32_t k1, uint32_t ti, uint32_t tj)
{
    const uint32_t oi = min(ti, tj), oj = max(ti, tj);
    const Philox4 r = philox4x32_10(0u, oi, oj, 0u, k0, k1);
    return -1.0f + 2.0f * open01f(r.v[0]);
}

// One pair in FP64 from the FP64 positions and velocities, the oracle's
// operation order. Returns false outside r_cut.
AZP_D bool dpd_pair_fp64(const DpdArgs& a, const double* c, const double4_32a& pi, const double4_32a& pj,
                         const double4_32a& vi, const double4_32a& vj, uint32_t tgi, uint32_t tgj, double& dx,
                         double& dy, double& dz, double& fdr, double& fc, double& e)
{
    dx = min_image1(pi.x - pj.x, a.L[0], a.Linv[0]);
    dy = min_image1(pi.y - pj.y, a.L[1], a.Linv[1]);
    dz = min_image1(pi.z - pj.z, a.L[2], a.Linv[2]);
    const double rs = rsq_exact(dx, dy, dz);
    if (!(rs < c[0])) return false;
    const double rinv = 1.0 / sqrt(rs);
    const double r = 1.0 / rinv;
    const double dot = dx * (vi.x - vj.x) + dy * (vi.y - vj.y) + dz * (vi.z - vj.z);
    fc = c[3] * (rinv - c[1]);
    const double wR = dpd_weight(fmax(1.0 - r * c[1], 0.0), c[5]) * rinv;  // never below 0 (r < r_cut)
    const double alpha = dpd_alpha(a.k0, a.k1, tgi, tgj);
    fdr = fc - c[4] * wR * wR * dot + c[6] * wR * alpha;
    e = c[3] * (c[2] - r) - 0.5 * c[3] * c[1] * (c[0] - rs);
    return true;
}

template<typename R> struct DpdAcc;
template<> struct DpdAcc<double> {
    double fx = 0, fy = 0, fz = 0, u = 0, w[6] = {0, 0, 0, 0, 0, 0};
    AZP_D void add(double dx, double dy, double dz, double fdr, double fc, double e)
    {
        fx += dx * fdr;
        fy += dy * fdr;
        fz += dz * fdr;
        u += 0.5 * e;
        const double h = 0.5 * fc;
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
            for (int c = 0; c < 6; ++c) w[c] += __shfl_xor_sync(0xffffffffu, w[c], m);
        }
    }
    AZP_D void store(const DpdArgs& a, uint32_t i)
    {
        reinterpret_cast<double4_32a*>(a.force)[i] = make_double4_32a(fx, fy, fz, u);
        if (a.virial)
            for (int c = 0; c < 6; ++c) reinterpret_cast<double*>(a.virial)[(size_t)c * a.pitch + i] = w[c];
    }
};
template<> struct DpdAcc<float> {
    Comp fx{0.f, 0.f}, fy{0.f, 0.f}, fz{0.f, 0.f}, u{0.f, 0.f};
    float w[6] = {0, 0, 0, 0, 0, 0};
    AZP_D void add(float dx, float dy, float dz, float fdr, float fc, float e)
    {
        fx.add(dx * fdr);
        fy.add(dy * fdr);
        fz.add(dz * fdr);
        u.add(0.5f * e);
        const float h = 0.5f * fc;
        w[0] += h * dx * dx;
        w[1] += h * dx * dy;
        w[2] += h * dx * dz;
        w[3] += h * dy * dy;
        w[4] += h * dy * dz;
        w[5] += h * dz * dz;
    }
    AZP_D static void comb(Comp& c, int m)
    {
        const float s2 = __shfl_xor_sync(0xffffffffu, c.s, m);
        const float c2 = __shfl_xor_sync(0xffffffffu, c.c, m);
        c.add(s2);
        c.c += c2;
    }
    AZP_D void reduce(int tpp)
    {
        for (int m = tpp >> 1; m > 0; m >>= 1) {
            comb(fx, m);
            comb(fy, m);
            comb(fz, m);
            comb(u, m);
            for (int c = 0; c < 6; ++c) w[c] += __shfl_xor_sync(0xffffffffu, w[c], m);
        }
    }
    AZP_D void store(const DpdArgs& a, uint32_t i)
    {
        reinterpret_cast<float4*>(a.force)[i] = make_float4(fx.value(), fy.value(), fz.value(), u.value());
        if (a.virial)
            for (int c = 0; c < 6; ++c) reinterpret_cast<float*>(a.virial)[(size_t)c * a.pitch + i] = w[c];
    }
};

// FP32: at most 64 registers a thread (4 blocks an SM): the kernel is latency
// bound and gains more from resident warps than from registers
template<typename R, int TPP>
__global__ void __launch_bounds__(DPD_BLOCK, std::is_same<R, float>::value ? 4 : 1) k_dpd(DpdArgs a)
{
    // the type-pair table in FP64 (FP64 pairs) and, for the FP32 path, as floats
    // (converted once per block, not per pair)
    extern __shared__ __align__(16) double s_tbl[];
    const uint32_t nt2 = a.ntypes * a.ntypes;
    float* s_tf = reinterpret_cast<float*>(s_tbl + (size_t)nt2 * DPD_TBL);
    uint32_t* s_queue = reinterpret_cast<uint32_t*>(s_tf + (size_t)nt2 * DPD_TBL);
    for (uint32_t t = threadIdx.x; t < nt2 * DPD_TBL; t += blockDim.x) {
        s_tbl[t] = a.table[t];
        if constexpr (std::is_same<R, float>::value) s_tf[t] = (float)a.table[t];
    }
    __syncthreads();
    const uint32_t gid = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t i = gid / TPP;
    const uint32_t sub = gid % TPP;
    const bool active = i < a.N;
    DpdAcc<R> acc;
    if (active) {
        const uint32_t n = min(a.counts[i], a.max_nn);
        const uint32_t tgi = a.tag[i];
        if constexpr (std::is_same<R, double>::value) {
            const double4_32a pi = a.pos[i];
            const double4_32a vi = a.vel[i];
            const uint32_t ti = type_of(pi.w);
            for (uint32_t k = sub; k < n; k += TPP) {
                const uint32_t j = a.nbrs[(size_t)k * a.N + i];
                const double4_32a pj = a.pos[j];
                const double* c = s_tbl + (size_t)(ti * a.ntypes + type_of(pj.w)) * DPD_TBL;
                double dx, dy, dz, fdr, fc, e;
                if (!dpd_pair_fp64(a, c, pi, pj, vi, a.vel[j], tgi, a.tag[j], dx, dy, dz, fdr, fc, e)) continue;
                acc.add(dx, dy, dz, fdr, fc, e);
            }
        } else {
            const uint4 fi = a.fixed[i];
            const float4 vi = a.vel_f[i];
            const uint32_t ti = fi.w;
            // Two phases per thread: the candidate scan (a gather and a distance)
            // queues the partners inside r_cut in this thread's shared-memory
            // slots, then the queue is evaluated (a Philox draw and the weight per
            // pair), so the warp runs the costly part with its lanes together
            // instead of once per lane whose candidate happens to be in range.
            uint32_t* q = s_queue + threadIdx.x * DPD_QUEUE;
            uint32_t nq = 0;
            auto flush = [&]() {
                for (uint32_t m = 0; m < nq; ++m) {
                    const uint32_t j = q[m];
                    const uint4 fj = a.fixed[j];
                    const float dx = (float)(int32_t)(fi.x - fj.x) * a.sfix[0];
                    const float dy = (float)(int32_t)(fi.y - fj.y) * a.sfix[1];
                    const float dz = (float)(int32_t)(fi.z - fj.z) * a.sfix[2];
                    const float rs = dx * dx + dy * dy + dz * dz;
                    const float* cf = s_tf + (size_t)(ti * a.ntypes + fj.w) * DPD_TBL;
                    const float rc2 = cf[0];
                    const float4 vj = a.vel_f[j];
                    const float rcinv = cf[1];
                    const float A = cf[3];
                    const float rinv = rsqrtf(rs);
                    const float r = rs * rinv;
                    const float dot = dx * (vi.x - vj.x) + dy * (vi.y - vj.y) + dz * (vi.z - vj.z);
                    const float fc = A * (rinv - rcinv);
                    const float wR = dpd_weight_f(fmaxf(1.0f - r * rcinv, 0.0f), cf[5]) * rinv;
                    const float alpha = dpd_alpha_f(a.k0, a.k1, tgi, a.tag[j]);
                    const float fdr = fc - cf[4] * wR * wR * dot + cf[6] * wR * alpha;
                    const float e = A * (cf[2] - r) - 0.5f * A * rcinv * (rc2 - rs);
                    acc.add(dx, dy, dz, fdr, fc, e);
                }
                nq = 0;
            };
            for (uint32_t k = sub; k < n; k += TPP) {
                const uint32_t j = a.nbrs[(size_t)k * a.N + i];
                const uint4 fj = a.fixed[j];
                const float dx = (float)(int32_t)(fi.x - fj.x) * a.sfix[0];
                const float dy = (float)(int32_t)(fi.y - fj.y) * a.sfix[1];
                const float dz = (float)(int32_t)(fi.z - fj.z) * a.sfix[2];
                const float rs = dx * dx + dy * dy + dz * dz;
                const size_t tp = (size_t)(ti * a.ntypes + fj.w) * DPD_TBL;
                const float* cf = s_tf + tp;
                const float rc2 = cf[0];
                if (rs >= rc2 * 1.000004f) continue;
                if (rs < rc2 * 0.998f) {
                    q[nq++] = j;
                    if (nq == DPD_QUEUE) flush();
                    continue;
                }
                {
                    const double* c = s_tbl + tp;
                    // Near r_cut the random weight (1 - r / r_cut)^(s/2) is steep
                    // (infinitely so at r_cut for s < 2): 1 - r / r_cut formed from a
                    // rounded FP32 r would cost percents of this pair's force. In a
                    // cubic box it comes from the exact integer difference
                    // r_cut^2 - r^2 of the fixed-point words, which also decides the
                    // cutoff; the rest of the pair in FP32.
                    const long long rcq = __double_as_longlong(c[7]);
                    if (rcq > 0) {
                        const long long ix = (int32_t)(fi.x - fj.x), iy = (int32_t)(fi.y - fj.y),
                                        iz = (int32_t)(fi.z - fj.z);
                        const long long qq = ix * ix + iy * iy + iz * iz;
                        const long long dqi = rcq - qq;
                        if (dqi > 0) {
                            const float qf = __ll2float_rn(qq), df = __ll2float_rn(dqi);
                            const float r2 = fmaf(qf, a.s2h, qf * a.s2l), dq = fmaf(df, a.s2h, df * a.s2l);
                            const float rinv = rsqrtf(r2);
                            const float x = dq * cf[1] / (cf[2] + r2 * rinv);  // 1 - r / r_cut
                            const float4 vj = a.vel_f[j];
                            const float dot = dx * (vi.x - vj.x) + dy * (vi.y - vj.y) + dz * (vi.z - vj.z);
                            const float fc = cf[3] * x * rinv;
                            const float wR = dpd_weight_f(x, cf[5]) * rinv;
                            const float alpha = dpd_alpha_f(a.k0, a.k1, tgi, a.tag[j]);
                            const float fdr = fc - cf[4] * wR * wR * dot + cf[6] * wR * alpha;
                            const float e = cf[3] * cf[2] * x - 0.5f * cf[3] * cf[1] * dq;
                            acc.add(dx, dy, dz, fdr, fc, e);
                        }
                        continue;
                    }
                    // other boxes: such pairs (about 0.3 % of them) in FP64 from the
                    // FP64 state, which also decides the cutoff as the oracle does
                    double ddx, ddy, ddz, dfdr, dfc, de;
                    if (dpd_pair_fp64(a, c, a.pos[i], a.pos[j], a.vel[i], a.vel[j], tgi, a.tag[j], ddx, ddy, ddz, dfdr,
                                      dfc, de))
                        acc.add((float)ddx, (float)ddy, (float)ddz, (float)dfdr, (float)dfc, (float)de);
                }
            }
            flush();
        }
    }
    if (TPP > 1) acc.reduce(TPP);
    if (active && sub == 0) acc.store(a, i);
}

template<typename R>
int launch_dpd(int tpp, const DpdArgs& a, size_t smem, cudaStream_t s)
{
    const uint32_t blocks = (uint32_t)(((size_t)a.N * tpp + DPD_BLOCK - 1) / DPD_BLOCK);
    switch (tpp) {
    case 1: k_dpd<R, 1><<<blocks, DPD_BLOCK, smem, s>>>(a); break;
    case 2: k_dpd<R, 2><<<blocks, DPD_BLOCK, smem, s>>>(a); break;
    case 4: k_dpd<R, 4><<<blocks, DPD_BLOCK, smem, s>>>(a); break;
    case 8: k_dpd<R, 8><<<blocks, DPD_BLOCK, smem, s>>>(a); break;
    case 16: k_dpd<R, 16><<<blocks, DPD_BLOCK, smem, s>>>(a); break;
    case 32: k_dpd<R, 32><<<blocks, DPD_BLOCK, smem, s>>>(a); break;
    default: return AZP_ERR_INVALID;
    }
    AZP_CHECK_LAUNCH("k_dpd");
    return AZP_OK;
}
}  // namespace
}  // namespace azp

extern "C" int azp_dpd_forces(const azp_system* sys, azp_nlist* nl, const double* params, const double* r_cut,
                              double kT, double dt, uint64_t timestep, uint32_t seed, const azp_forces* out,
                              void* stream)
{
    using namespace azp;
    if (!sys || !nl || !params || !r_cut || !out || !out->force) return AZP_ERR_INVALID;
    if (out->precision != AZP_FP64 && out->precision != AZP_FP32) return AZP_ERR_INVALID;
    if (sys->N != nl->N || sys->ntypes != nl->ntypes || sys->ntypes == 0 || sys->ntypes > MAX_PAIR_TYPES)
        return AZP_ERR_INVALID;
    if (!(dt > 0.0) || !(kT >= 0.0)) return AZP_ERR_INVALID;
    for (int d = 0; d < 3; ++d)
        if (!(sys->box.L[d] > 0.0)) return AZP_ERR_INVALID;
    if (sys->N == 0) return AZP_OK;
    if (!sys->pos || !sys->vel || !sys->tag) return AZP_ERR_INVALID;
    cudaStream_t s = as_stream(stream);
    const uint32_t nt2 = sys->ntypes * sys->ntypes;
    const bool cubic = sys->box.L[0] == sys->box.L[1] && sys->box.L[1] == sys->box.L[2];
    const double u = 4294967296.0 / sys->box.L[0];
    k_dpd_table<<<(nt2 + 63) / 64, 64, 0, s>>>(params, r_cut, nt2, kT, dt, cubic ? u * u : 0.0, nl->dpd_table);
    DpdArgs a;
    a.pos = reinterpret_cast<const double4_32a*>(sys->pos);
    a.vel = reinterpret_cast<const double4_32a*>(sys->vel);
    a.fixed = nl->fixed;
    a.vel_f = nl->vel_f;
    a.tag = sys->tag;
    a.N = sys->N;
    a.ntypes = sys->ntypes;
    for (int d = 0; d < 3; ++d) {
        a.L[d] = sys->box.L[d];
        a.Linv[d] = 1.0 / sys->box.L[d];
        a.sfix[d] = (float)(sys->box.L[d] * 2.3283064365386963e-10);
    }
    {
        const double q = sys->box.L[0] * 2.3283064365386963e-10, q2 = q * q;
        a.s2h = (float)q2;
        a.s2l = (float)(q2 - (double)a.s2h);
    }
    a.counts = nl->counts;
    a.nbrs = nl->nbrs;
    a.max_nn = nl->max_nn;
    a.table = nl->dpd_table;
    stream_key(AZP_RNG_DPD_GENERAL_WEIGHT, timestep, seed, a.k0, a.k1);
    a.force = out->force;
    a.virial = out->virial;
    a.pitch = out->virial_pitch ? out->virial_pitch : sys->N;
    const size_t smem = (size_t)nt2 * DPD_TBL * (sizeof(double) + sizeof(float)) +
                        (out->precision == AZP_FP32 ? (size_t)DPD_BLOCK * DPD_QUEUE * sizeof(uint32_t) : 0);
    if (out->precision == AZP_FP32) {
        launch_to_fixed(a.pos, nl->fixed, sys->N, sys->box, s);
        k_vel_f<<<(sys->N + 255) / 256, 256, 0, s>>>(a.vel, sys->N, nl->vel_f);
        return launch_dpd<float>(nl->tpp, a, smem, s);
    }
    return launch_dpd<double>(nl->tpp, a, smem, s);
}
