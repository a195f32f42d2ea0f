// walls.cu -- azp_wall_forces: the azplugins wall potentials (LJ93, Colloid) over
// HOOMD's wall geometries, as the drop-in for
// gpu_compute_potential_external_forces<EvaluatorWalls<WallEvaluator*>>
// (src/PotentialExternalWallGPUKernel.cu.inc:26-30), and their param_type
// builders (src/WallEvaluatorLJ93.h:31-45, src/WallEvaluatorColloid.h:31-53).
//
// One thread per particle; the walls travel as a kernel argument (HOOMD passes
// its wall field by value too), declared __grid_constant__ so that every thread
// reads them from the constant bank (without it the device code's references
// into the 5.4 KB field make a per-thread copy in local memory). FP64 output: FP64 arithmetic throughout. FP32 output: FP32 arithmetic
// except the differences that cancel near a surface (walls.cuh), because FP64
// runs at about 1/64 of the FP32 rate and the FP64 form is bound by it.
#include <cmath>

#include "common.cuh"
#include "walls.cuh"

namespace azp
{
namespace
{
constexpr int kBlock = 128;

// one wall record of a caller's table (stride doubles each) zero-padded to 4
AZP_D void load_wall_record(const double* __restrict__ params, uint32_t t, int stride, double* p)
{
    for (int k = 0; k < 4; ++k) p[k] = k < stride ? __ldg(params + (size_t)t * stride + k) : 0.0;
}

// A block's chunk (reps x kBlock particles from base) in two passes: every
// thread screens its particles in FP32 (walls_near) and writes the outputs of
// the far ones at once (force, energy and virial of a particle no wall reaches:
// the same zeros, signs included, as the full evaluation gives), listing the near
// ones in shared memory; then the block's threads share out the list for the
// full evaluation. A warp's lanes so all work on particles some wall may reach,
// in whatever order the caller keeps its particles.
template<class Screen, class Eval>
AZP_D void screened_chunk(uint32_t N, uint32_t reps, uint32_t* s_list, Screen screen, Eval eval)
{
    __shared__ uint32_t s_n;
    if (threadIdx.x == 0) s_n = 0;
    __syncthreads();
    const uint32_t lane = threadIdx.x & 31u, chunk = reps * kBlock;
    const uint32_t base = blockIdx.x * chunk;
    for (uint32_t k = threadIdx.x; k < chunk; k += kBlock) {
        const uint32_t i = base + k;
        const bool nr = i < N && screen(i);
        const unsigned m = __ballot_sync(0xffffffffu, nr);
        uint32_t at = 0;
        if (lane == 0 && m) at = atomicAdd(&s_n, (uint32_t)__popc(m));
        at = __shfl_sync(0xffffffffu, at, 0);
        if (nr) s_list[at + __popc(m & ((1u << lane) - 1u))] = i;
    }
    __syncthreads();
    const uint32_t n = s_n;
    for (uint32_t k = threadIdx.x; k < n; k += kBlock) eval(s_list[k]);
}

// the screen's reach of a type: max(|r_cut|, r_extrap) (a NaN of either drops
// out, as it does from the evaluation)
AZP_D float type_reach(const double* r_cut, const double* r_extrap, uint32_t t)
{
    return (float)fmax(fabs(__ldg(r_cut + t)), __ldg(r_extrap + t));
}

template<class EV, typename T>
__global__ void __launch_bounds__(kBlock) k_walls(const double4_32a* __restrict__ pos,
                                                  const double* __restrict__ params, int stride,
                                                  const double* __restrict__ r_cut,
                                                  const double* __restrict__ r_extrap,
                                                  const __grid_constant__ WallField wf, float mag, uint32_t N,
                                                  uint32_t reps, T* __restrict__ force, T* __restrict__ virial,
                                                  uint32_t pitch)
{
    extern __shared__ uint32_t s_list[];
    auto write = [&](uint32_t i, const double* F, double U, const double* x) {
        if constexpr (sizeof(T) == 8)
            reinterpret_cast<double4_32a*>(force)[i] = make_double4_32a(F[0], F[1], F[2], U);
        else
            reinterpret_cast<float4*>(force)[i] = make_float4((float)F[0], (float)F[1], (float)F[2], (float)U);
        if (virial) {
            const double v[6] = {F[0] * x[0], F[0] * x[1], F[0] * x[2], F[1] * x[1], F[1] * x[2], F[2] * x[2]};
            for (int c = 0; c < 6; ++c) virial[(size_t)c * pitch + i] = (T)v[c];
        }
    };
    auto screen = [&](uint32_t i) {
        const double4_32a pp = pos[i];
        const uint32_t t = type_of(pp.w);
        const double x[3] = {pp.x, pp.y, pp.z};
        const float reach = type_reach(r_cut, r_extrap, t);
        const float tol = walls_screen_tol(x, mag + reach);
        if (walls_near(wf, reach + tol, __ldg(r_extrap + t) > 0.0, (float)x[0], (float)x[1], (float)x[2], tol))
            return true;
        const double F[3] = {0.0, 0.0, 0.0};
        write(i, F, 0.0, x);
        return false;
    };
    auto eval = [&](uint32_t i) {
        const double4_32a pp = pos[i];
        const uint32_t t = type_of(pp.w);
        double p[4];
        load_wall_record(params, t, stride, p);
        const double rc = __ldg(r_cut + t);
        const double x[3] = {pp.x, pp.y, pp.z};
        double F[3] = {0.0, 0.0, 0.0}, U = 0.0;
        walls_force<EV>(wf, p, rc * rc, __ldg(r_extrap + t), x, F, U);
        write(i, F, U, x);
    };
    screened_chunk(N, reps, s_list, screen, eval);
}

// FP32 output: FP32 arithmetic with the FP64 parts that cancellation needs
// (walls.cuh), per-type float records and reaches made once per block in shared
// memory
template<class EV, class EVF>
__global__ void __launch_bounds__(kBlock) k_walls_f(const double4_32a* __restrict__ pos,
                                                    const double* __restrict__ params, int stride,
                                                    const double* __restrict__ r_cut,
                                                    const double* __restrict__ r_extrap, uint32_t ntypes,
                                                    const __grid_constant__ WallField wf, float mag, uint32_t N,
                                                    uint32_t reps, float* __restrict__ force,
                                                    float* __restrict__ virial, uint32_t pitch)
{
    extern __shared__ float s_q[];
    float* s_reach = s_q + (size_t)ntypes * WALL_F;
    uint32_t* s_list = reinterpret_cast<uint32_t*>(s_reach + ntypes);
    for (uint32_t t = threadIdx.x; t < ntypes; t += kBlock) {
        double p[4];
        load_wall_record(params, t, stride, p);
        wall_record_f<EV>(p, r_cut[t], r_extrap[t], s_q + (size_t)t * WALL_F);
        s_reach[t] = type_reach(r_cut, r_extrap, t);
    }
    __syncthreads();
    auto write = [&](uint32_t i, const float* F, float U, const double* x) {
        reinterpret_cast<float4*>(force)[i] = make_float4(F[0], F[1], F[2], U);
        if (virial) {
            const float xf = (float)x[0], yf = (float)x[1], zf = (float)x[2];
            const float v[6] = {F[0] * xf, F[0] * yf, F[0] * zf, F[1] * yf, F[1] * zf, F[2] * zf};
            for (int c = 0; c < 6; ++c) virial[(size_t)c * pitch + i] = v[c];
        }
    };
    auto screen = [&](uint32_t i) {
        const double4_32a pp = pos[i];
        const uint32_t t = type_of(pp.w);
        const double x[3] = {pp.x, pp.y, pp.z};
        const float reach = s_reach[t];
        const float tol = walls_screen_tol(x, mag + reach);
        if (walls_near(wf, reach + tol, s_q[(size_t)t * WALL_F + 7] > 0.0f, (float)x[0], (float)x[1], (float)x[2],
                       tol))
            return true;
        const float F[3] = {0.0f, 0.0f, 0.0f};
        write(i, F, 0.0f, x);
        return false;
    };
    auto eval = [&](uint32_t i) {
        const double4_32a pp = pos[i];
        const double x[3] = {pp.x, pp.y, pp.z};
        float F[3] = {0.0f, 0.0f, 0.0f}, U = 0.0f;
        walls_force_f<EVF>(wf, s_q + (size_t)type_of(pp.w) * WALL_F, x, F, U);
        write(i, F, U, x);
    };
    screened_chunk(N, reps, s_list, screen, eval);
}

template<class EV, class EVF>
void launch_walls(const azp_system* sys, const double* params, int stride, const double* r_cut,
                  const double* r_extrap, const WallField& wf, const azp_forces* out, cudaStream_t s)
{
    // chunks of reps x kBlock particles: about eight blocks per SM, at least one
    // warp's worth of particles per thread-block pass
    int dev = 0, sms = 152;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const uint64_t per_block = (uint64_t)sys->N / ((uint64_t)8 * (uint64_t)sms * kBlock);
    const uint32_t reps = (uint32_t)std::min<uint64_t>(std::max<uint64_t>(per_block, 1), 16);
    const uint32_t chunk = reps * kBlock;
    const uint32_t grid = (uint32_t)(((uint64_t)sys->N + chunk - 1) / chunk);
    const uint32_t pitch = out->virial_pitch ? out->virial_pitch : sys->N;
    const auto* pos = reinterpret_cast<const double4_32a*>(sys->pos);
    const float mag = wall_field_extent(wf);
    const size_t smem_f = sizeof(float) * (WALL_F + 1) * sys->ntypes + sizeof(uint32_t) * chunk;
    if (out->precision == AZP_FP32 && smem_f > 48 * 1024)
        cudaFuncSetAttribute(k_walls_f<EV, EVF>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_f);
    if (out->precision == AZP_FP64)
        k_walls<EV, double><<<grid, kBlock, sizeof(uint32_t) * chunk, s>>>(
            pos, params, stride, r_cut, r_extrap, wf, mag, sys->N, reps, static_cast<double*>(out->force),
            static_cast<double*>(out->virial), pitch);
    else
        k_walls_f<EV, EVF><<<grid, kBlock, smem_f, s>>>(pos, params, stride, r_cut, r_extrap, sys->ntypes, wf, mag, sys->N, reps,
                                  static_cast<float*>(out->force), static_cast<float*>(out->virial), pitch);
}

bool unit(const double* v, double* u)
{
    const double n = std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    if (!(n > 0.0) || !std::isfinite(n)) return false;
    for (int d = 0; d < 3; ++d) u[d] = v[d] / n;
    return true;
}
}  // namespace

float wall_field_extent(const WallField& wf)
{
    double m = 0.0;
    auto l1 = [](const double* o) { return std::fabs(o[0]) + std::fabs(o[1]) + std::fabs(o[2]); };
    for (int k = 0; k < wf.ns; ++k) m = std::max(m, l1(wf.s[k].o) + std::fabs(wf.s[k].r));
    for (int k = 0; k < wf.nc; ++k) m = std::max(m, l1(wf.c[k].o) + std::fabs(wf.c[k].r));
    for (int k = 0; k < wf.np; ++k) m = std::max(m, l1(wf.p[k].o));
    // a field beyond float range screens nothing out (the tolerance goes infinite)
    return m < 1.0e37 ? (float)m : INFINITY;
}

int make_wall_field(const azp_walls* w, WallField* out)
{
    *out = WallField{};
    if (!w) return AZP_ERR_INVALID;
    if (w->n_spheres > (uint32_t)WALL_MAX_SPHERES || w->n_cylinders > (uint32_t)WALL_MAX_CYLINDERS ||
        w->n_planes > (uint32_t)WALL_MAX_PLANES)
        return record_error(AZP_ERR_INVALID, "azp_wall_forces: more walls than the wall field holds (20 spheres, "
                                             "20 cylinders, 60 planes)");
    if ((w->n_spheres && !w->spheres) || (w->n_cylinders && !w->cylinders) || (w->n_planes && !w->planes))
        return AZP_ERR_INVALID;
    out->ns = (int)w->n_spheres;
    out->nc = (int)w->n_cylinders;
    out->np = (int)w->n_planes;
    for (int k = 0; k < out->ns; ++k) {
        const azp_wall_sphere& s = w->spheres[k];
        if (!(s.r >= 0.0)) return AZP_ERR_INVALID;
        out->s[k].r = s.r;
        for (int d = 0; d < 3; ++d) out->s[k].o[d] = s.origin[d];
        out->s[k].inside = s.inside != 0;
        out->s[k].open = s.open != 0;
    }
    for (int k = 0; k < out->nc; ++k) {
        const azp_wall_cylinder& c = w->cylinders[k];
        if (!(c.r >= 0.0) || !unit(c.axis, out->c[k].ax)) return AZP_ERR_INVALID;
        out->c[k].r = c.r;
        for (int d = 0; d < 3; ++d) out->c[k].o[d] = c.origin[d];
        out->c[k].inside = c.inside != 0;
        out->c[k].open = c.open != 0;
    }
    for (int k = 0; k < out->np; ++k) {
        const azp_wall_plane& p = w->planes[k];
        if (!unit(p.normal, out->p[k].n)) return AZP_ERR_INVALID;
        for (int d = 0; d < 3; ++d) out->p[k].o[d] = p.origin[d];
        out->p[k].open = p.open != 0;
    }
    return AZP_OK;
}

}  // namespace azp

extern "C" {

int azp_wall_params_from_values(int kind, const double* v, double* out)
{
    if (!v || !out) return AZP_ERR_INVALID;
    if (kind != AZP_WALL_LJ93 && kind != AZP_WALL_COLLOID) return AZP_ERR_INVALID;
    for (int k = 0; k < azp::wall_record_doubles(kind); ++k) out[k] = 0.0;
    if (kind == AZP_WALL_LJ93) {
        // WallParametersLJ93(dict): sigma_3 = sigma^3, A
        const double A = v[0], sigma = v[1];
        out[0] = sigma * sigma * sigma;
        out[1] = A;
        return AZP_OK;
    }
    if (kind == AZP_WALL_COLLOID) {
        // WallParametersColloid(dict): c_1 = A sigma^6 / 7560, c_2 = A / 6, a
        const double A = v[0], a = v[1], sigma = v[2];
        const double sigma_3 = sigma * sigma * sigma;
        out[0] = A * sigma_3 * sigma_3 / 7560.0;
        out[1] = A / 6.0;
        out[2] = a;
        return AZP_OK;
    }
    return AZP_ERR_INVALID;
}

int azp_wall_params_to_values(int kind, const double* rec, double* v)
{
    if (!v || !rec) return AZP_ERR_INVALID;
    if (kind == AZP_WALL_LJ93) {
        // asDict(): sigma = cbrt(sigma_3)
        v[0] = rec[1];
        v[1] = std::cbrt(rec[0]);
        return AZP_OK;
    }
    if (kind == AZP_WALL_COLLOID) {
        // asDict(): A = 6 c_2, sigma = (7560 c_1 / A)^(1/6)
        const double A = 6.0 * rec[1];
        v[0] = A;
        v[1] = rec[2];
        v[2] = std::pow(7560.0 * rec[0] / A, 1.0 / 6.0);
        return AZP_OK;
    }
    return AZP_ERR_INVALID;
}

int azp_wall_forces(const azp_system* sys, int kind, const azp_walls* walls, const double* params, const double* r_cut,
                    const double* r_extrap, const azp_forces* out, void* stream)
{
    using namespace azp;
    if (!sys || !out || !out->force) return AZP_ERR_INVALID;
    if (kind != AZP_WALL_LJ93 && kind != AZP_WALL_COLLOID) return AZP_ERR_INVALID;
    if (out->precision != AZP_FP64 && out->precision != AZP_FP32) return AZP_ERR_INVALID;
    WallField wf;
    const int st = make_wall_field(walls, &wf);
    if (st) return st;
    if (sys->N == 0) return AZP_OK;
    if (!sys->pos || !params || !r_cut || !r_extrap) return AZP_ERR_INVALID;
    cudaStream_t s = as_stream(stream);
    if (sys->ntypes == 0 || sys->ntypes > 4096) return AZP_ERR_INVALID;
    if (kind == AZP_WALL_LJ93)
        launch_walls<WallLJ93, WallLJ93F>(sys, params, wall_record_doubles(kind), r_cut, r_extrap, wf, out, s);
    else
        launch_walls<WallColloid, WallColloidF>(sys, params, wall_record_doubles(kind), r_cut, r_extrap, wf, out,
                                                s);
    AZP_CHECK_LAUNCH("k_walls");
    return AZP_OK;
}

}  // extern "C"
