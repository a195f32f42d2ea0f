// velocity.cu -- binned mass-averaged velocity fields (src/VelocityFieldCompute.h with
// src/CartesianBinningOperation.h / src/CylindricalBinningOperation.h) and the
// centre-of-mass velocity (src/VelocityCompute.h) as one drop-in compute,
// azp_vfield_*.
//
// The reference's GPU path bins with FP64 atomicAdd on global memory
// (src/VelocityFieldComputeGPU.cuh:35-72): contended when bins are few and not
// reproducible from run to run. Here every contribution (mass, and the momentum
// m v turned into the bin's coordinate system) becomes a 64-bit fixed-point
// integer q = round(x 2^40), split into a high and a low 32-bit limb, and the
// limbs are summed as 64-bit integers. Integer sums do not depend on their order,
// so the result is the same bit for bit whatever the schedule:
//   * lanes of a warp that land in one bin first sum their limbs by shuffles
//     (a warp of particles in cell order usually shares a bin);
//   * blocks then add into a shared-memory histogram (few bins) or straight
//     into the global one (many bins), with integer atomics;
//   * a finishing pass joins the limbs, scales back, and divides.
// A contribution is resolved to 2^-41 absolute (half a unit of 2^-40) and must
// stay below 2^22 in magnitude; larger ones raise AZP_EBIT_RANGE.
#include <algorithm>
#include <cmath>
#include <new>

#include "common.cuh"
#include "integrate.cuh"

namespace azp
{
namespace
{
constexpr int kBlock = 256;
constexpr double kScale = 1099511627776.0;              // 2^40
constexpr double kInvScale = 9.094947017729282e-13;     // 2^-40
constexpr double kMaxFixed = 4611686018427387904.0;     // 2^62: |q| bound
constexpr uint32_t kSmemBins = 768;                      // 768 bins x 64 B = 48 KB
constexpr int kLimbs = 8;                                // (mass, p_x, p_y, p_z) x (high, low)

struct BinSpec {
    int kind;
    uint32_t nb[3];
    int use[3];
    double lo[3], hi[3];
    double scale[3];  // nb / (hi - lo)
    uint32_t total;
};

// src/BinningOperation.h:71-87: floor((x - lo) / (hi - lo) * n), inside [0, n).
// FP64 division is slow here (about 1/64 of the FP32 rate), so the bin comes
// from a multiplication by n / (hi - lo); a value within 1e-9 of a bin edge,
// where the two roundings could disagree, takes the reference's division.
AZP_HD bool bin1d(double x, double lo, double hi, double scale, uint32_t n, uint32_t& b)
{
    const double u = (x - lo) * scale;
    const double fu = floor(u);
    const double k = (u - fu < 1e-9 || fu + 1.0 - u < 1e-9) ? floor(((x - lo) / (hi - lo)) * n) : fu;
    if (k >= 0.0 && k < (double)n) {
        b = (uint32_t)k;
        return true;
    }
    return false;
}

// theta in [0, 2 pi) for the bin: atan2f, or the FP64 atan2 within 1e-5 of an
// edge (atan2f is good to a few 1e-7 here)
AZP_D bool bin_theta(const BinSpec& s, double x, double y, uint32_t& b)
{
    float tf = atan2f((float)y, (float)x);
    if (tf < 0.0f) tf += 6.283185307179586f;
    const double u = ((double)tf - s.lo[1]) * s.scale[1];
    const double fu = floor(u);
    const double guard = 1e-5 * s.scale[1];
    if (u - fu < guard || fu + 1.0 - u < guard) {
        double theta = atan2(y, x);
        if (theta < 0.0) theta += 2.0 * M_PI;
        return bin1d(theta, s.lo[1], s.hi[1], s.scale[1], s.nb[1], b);
    }
    if (fu >= 0.0 && fu < (double)s.nb[1]) {
        b = (uint32_t)fu;
        return true;
    }
    return false;
}

// src/CartesianBinningOperation.h:27-52, src/CylindricalBinningOperation.h:27-76.
// x: the position (binned axes already wrapped), p: the momentum m v
AZP_D bool bin_particle(const BinSpec& s, const double* x, const double* p, uint32_t& idx, double* t)
{
    uint32_t b[3] = {0u, 0u, 0u};
    if (s.kind == AZP_BINNING_CARTESIAN) {
        for (int d = 0; d < 3; ++d)
            if (s.use[d] && !bin1d(x[d], s.lo[d], s.hi[d], s.scale[d], s.nb[d], b[d])) return false;
        t[0] = p[0];
        t[1] = p[1];
        t[2] = p[2];
    } else {
        if (s.use[2] && !bin1d(x[2], s.lo[2], s.hi[2], s.scale[2], s.nb[2], b[2])) return false;
        if (s.use[1] && !bin_theta(s, x[0], x[1], b[1])) return false;
        // 1/r from rsqrtf and one Newton step in FP64 (relative error ~1e-14)
        const double r2 = x[0] * x[0] + x[1] * x[1];
        double c = 1.0, sn = 0.0, r = 0.0;
        if (r2 > 0.0) {
            const double g = (double)rsqrtf((float)r2);
            const double rinv = g * (1.5 - 0.5 * r2 * g * g);
            r = r2 * rinv;
            c = x[0] * rinv;
            sn = x[1] * rinv;
        }
        if (s.use[0] && !bin1d(r, s.lo[0], s.hi[0], s.scale[0], s.nb[0], b[0])) return false;
        t[0] = c * p[0] + sn * p[1];
        t[1] = -sn * p[0] + c * p[1];
        t[2] = p[2];
    }
    // src/BinningOperation.h:59-62 (z fastest)
    idx = b[2] + s.nb[2] * (b[1] + s.nb[1] * b[0]);
    return true;
}

// sum of v over the 32 lanes of the warp, result in every lane
AZP_D unsigned long long warp_sum(unsigned long long v)
{
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

__global__ void __launch_bounds__(kBlock) k_vfield(const double4_32a* __restrict__ pos,
                                                   const double4_32a* __restrict__ vel,
                                                   const uint32_t* __restrict__ group, uint32_t n, BoxD box,
                                                   const __grid_constant__ BinSpec spec, int use_smem,
                                                   unsigned long long* __restrict__ acc,
                                                   uint32_t* __restrict__ err)
{
    extern __shared__ unsigned long long s_acc[];
    if (use_smem) {
        for (uint32_t k = threadIdx.x; k < spec.total * kLimbs; k += kBlock) s_acc[k] = 0ull;
        __syncthreads();
    }
    unsigned long long* const hist = use_smem ? s_acc : acc;
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t stride = gridDim.x * kBlock;
    // every lane of a warp runs the same number of iterations (shuffles below)
    const uint32_t n_round = (n + stride - 1) / stride * stride;
    for (uint32_t m = blockIdx.x * kBlock + threadIdx.x; m < n_round; m += stride) {
        bool ok = false;
        uint32_t bin = 0xffffffffu;
        long long q[4] = {0, 0, 0, 0};
        if (m < n) {
            const uint32_t i = group ? group[m] : m;
            const double4_32a pp = pos[i];
            const double4_32a vv = vel[i];
            double x[3] = {pp.x, pp.y, pp.z};
            // src/VelocityFieldCompute.h:196-198: wrap into the box first (the axes
            // the bins read: the binned Cartesian ones; x, y and a binned z for
            // cylindrical bins)
            int img = 0;
            for (int d = 0; d < 3; ++d)
                if (spec.use[d] || (spec.kind == AZP_BINNING_CYLINDRICAL && d < 2))
                    wrap1(x[d], img, box.L[d], box.lo[d], box.hi[d]);
            const double mi = vv.w;
            // the mass folded into the fixed-point scale: m 2^40 is exact
            const double ms = mi * kScale;
            const double p[3] = {vv.x * ms, vv.y * ms, vv.z * ms};
            double t[3];
            ok = bin_particle(spec, x, p, bin, t);
            if (ok) {
                const double vals[4] = {ms, t[0], t[1], t[2]};
                for (int c = 0; c < 4; ++c) {
                    if (!(fabs(vals[c]) < kMaxFixed)) {
                        atomicOr(err, AZP_EBIT_RANGE);
                        ok = false;
                        break;
                    }
                    q[c] = __double2ll_rn(vals[c]);
                }
            }
        }
        if (!ok) bin = 0xffffffffu;
        // a warp whose lanes all fall in one bin sums by shuffles first
        const uint32_t peers = __match_any_sync(0xffffffffu, bin);
        const bool whole = peers == 0xffffffffu;
        if (whole && bin == 0xffffffffu) continue;
        for (int c = 0; c < 4; ++c) {
            unsigned long long hi = (unsigned long long)(q[c] >> 32);
            unsigned long long lo = (unsigned long long)(q[c] & 0xffffffffll);
            if (whole) {
                hi = warp_sum(hi);
                lo = warp_sum(lo);
            }
            if ((whole && lane == 0) || (!whole && bin != 0xffffffffu)) {
                if (hi) atomicAdd(&hist[(size_t)bin * kLimbs + 2 * c], hi);
                if (lo) atomicAdd(&hist[(size_t)bin * kLimbs + 2 * c + 1], lo);
            }
        }
    }
    if (use_smem) {
        __syncthreads();
        for (uint32_t k = threadIdx.x; k < spec.total * kLimbs; k += kBlock)
            if (s_acc[k]) atomicAdd(&acc[k], s_acc[k]);
    }
}

// limbs -> FP64 mass, momentum and mass-averaged velocity (src/VelocityFieldCompute.h:258-276)
__global__ void k_vfield_finish(const unsigned long long* __restrict__ acc, uint32_t total, double* __restrict__ mass,
                                double* __restrict__ momentum, double* __restrict__ velocity)
{
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= total) return;
    double v[4];
    for (int c = 0; c < 4; ++c) {
        const long long hi = (long long)acc[(size_t)k * kLimbs + 2 * c];
        const unsigned long long lo = acc[(size_t)k * kLimbs + 2 * c + 1];
        // sum = hi 2^32 + lo = th 2^32 + tl with 0 <= tl < 2^32; th is exact in a double
        const long long th = hi + (long long)(lo >> 32);
        const double tl = (double)(lo & 0xffffffffull);
        v[c] = ((double)th * 4294967296.0 + tl) * kInvScale;
    }
    if (mass) mass[k] = v[0];
    for (int d = 0; d < 3; ++d) {
        if (momentum) momentum[3 * k + d] = v[1 + d];
        if (velocity) velocity[3 * k + d] = v[0] > 0.0 ? v[1 + d] / v[0] : 0.0;
    }
}
}  // namespace
}  // namespace azp

struct azp_vfield {
    azp::BinSpec spec{};
    unsigned long long* acc = nullptr;  // [total][8] limbs
    uint32_t* err = nullptr;
};

extern "C" {

azp_vfield* azp_vfield_create(int kind, const uint32_t* num_bins, const double* lower, const double* upper, int* status)
{
    using namespace azp;
    auto fail = [&](int st) -> azp_vfield* {
        if (status) *status = st;
        return nullptr;
    };
    if (kind != AZP_BINNING_CARTESIAN && kind != AZP_BINNING_CYLINDRICAL) return fail(AZP_ERR_INVALID);
    if (!num_bins || !lower || !upper) return fail(AZP_ERR_INVALID);
    BinSpec s{};
    s.kind = kind;
    unsigned long long total = 1;
    for (int d = 0; d < 3; ++d) {
        s.use[d] = num_bins[d] > 0;
        s.nb[d] = s.use[d] ? num_bins[d] : 1u;
        s.lo[d] = lower[d];
        s.hi[d] = upper[d];
        if (s.use[d] && !(upper[d] > lower[d])) return fail(AZP_ERR_INVALID);
        s.scale[d] = s.use[d] ? (double)s.nb[d] / (upper[d] - lower[d]) : 0.0;
        total *= s.nb[d];
    }
    if (total > (1ull << 26)) return fail(record_error(AZP_ERR_TOO_LARGE, "azp_vfield_create: more than 2^26 bins"));
    s.total = (uint32_t)total;
    azp_vfield* v = new (std::nothrow) azp_vfield();
    if (!v) return fail(AZP_ERR_INVALID);
    v->spec = s;
    cudaError_t e = cudaMalloc(reinterpret_cast<void**>(&v->acc), sizeof(unsigned long long) * kLimbs * s.total);
    if (e == cudaSuccess) e = cudaMalloc(reinterpret_cast<void**>(&v->err), sizeof(uint32_t));
    if (e == cudaSuccess) e = cudaMemset(v->err, 0, sizeof(uint32_t));
    if (e != cudaSuccess) {
        cudaFree(v->acc);
        cudaFree(v->err);
        delete v;
        return fail(record_cuda_error(e, "azp_vfield_create"));
    }
    if (status) *status = AZP_OK;
    return v;
}

void azp_vfield_destroy(azp_vfield* v)
{
    if (!v) return;
    cudaFree(v->acc);
    cudaFree(v->err);
    delete v;
}

uint32_t azp_vfield_num_bins(const azp_vfield* v) { return v ? v->spec.total : 0u; }

int azp_vfield_compute(azp_vfield* v, const azp_system* sys, const uint32_t* group, uint32_t n_group, double* mass,
                       double* momentum, double* velocity, void* stream)
{
    using namespace azp;
    if (!v || !sys) return AZP_ERR_INVALID;
    for (int d = 0; d < 3; ++d)
        if (!(sys->box.L[d] > 0.0)) return AZP_ERR_INVALID;
    const uint32_t n = group ? n_group : sys->N;
    if (n > 0 && (!sys->pos || !sys->vel)) return AZP_ERR_INVALID;
    cudaStream_t s = as_stream(stream);
    const BinSpec& spec = v->spec;
    AZP_CUDA_TRY(cudaMemsetAsync(v->acc, 0, sizeof(unsigned long long) * kLimbs * spec.total, s));
    if (n > 0) {
        const int use_smem = spec.total <= kSmemBins;
        const size_t smem = use_smem ? sizeof(unsigned long long) * kLimbs * spec.total : 0;
        int dev = 0, sms = 152;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        const uint32_t grid = (uint32_t)std::min<unsigned long long>((n + kBlock - 1) / kBlock, 4ull * sms);
        k_vfield<<<grid, kBlock, smem, s>>>(reinterpret_cast<const double4_32a*>(sys->pos),
                                             reinterpret_cast<const double4_32a*>(sys->vel), group, n,
                                             make_box(sys->box), spec, use_smem, v->acc, v->err);
        AZP_CHECK_LAUNCH("k_vfield");
    }
    k_vfield_finish<<<(spec.total + 255) / 256, 256, 0, s>>>(v->acc, spec.total, mass, momentum, velocity);
    AZP_CHECK_LAUNCH("k_vfield_finish");
    return AZP_OK;
}

int azp_vfield_error(azp_vfield* v, uint32_t* err_word, void* stream)
{
    if (!v || !err_word) return AZP_ERR_INVALID;
    cudaStream_t s = azp::as_stream(stream);
    AZP_CUDA_TRY(cudaMemcpyAsync(err_word, v->err, sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
    AZP_CUDA_TRY(cudaStreamSynchronize(s));
    return AZP_OK;
}

}  // extern "C"
