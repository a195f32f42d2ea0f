// integrate.cu -- standalone Langevin-flow step one / step two and Brownian-flow
// kernels (one thread per particle of the group), FP64 state.
#include "integrate.cuh"

namespace azp
{
constexpr int STEP_BLOCK = 256;

AZP_D double3 load_force(const void* f, int prec, uint32_t i)
{
    if (prec == AZP_FP32) {
        const float4 v = reinterpret_cast<const float4*>(f)[i];
        return make_double3(v.x, v.y, v.z);
    }
    const double4_32a v = reinterpret_cast<const double4_32a*>(f)[i];
    return make_double3(v.x, v.y, v.z);
}

__global__ void __launch_bounds__(STEP_BLOCK) k_step1(StepArgs a)
{
    const uint32_t g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= a.n) return;
    const uint32_t i = a.group ? a.group[g] : g;
    double4_32a p = a.pos[i];
    double4_32a v = a.vel[i];
    const double ax = a.accel[3 * i], ay = a.accel[3 * i + 1], az = a.accel[3 * i + 2];
    const double h = 0.5 * a.dt;
    p.x += (v.x + h * ax) * a.dt;
    p.y += (v.y + h * ay) * a.dt;
    p.z += (v.z + h * az) * a.dt;
    int ix = a.image[3 * i], iy = a.image[3 * i + 1], iz = a.image[3 * i + 2];
    wrap1(p.x, ix, a.L[0], a.lo[0], a.hi[0]);
    wrap1(p.y, iy, a.L[1], a.lo[1], a.hi[1]);
    wrap1(p.z, iz, a.L[2], a.lo[2], a.hi[2]);
    v.x += h * ax;
    v.y += h * ay;
    v.z += h * az;
    a.pos[i] = p;  // w (type bits) untouched
    a.vel[i] = v;
    a.image[3 * i] = ix;
    a.image[3 * i + 1] = iy;
    a.image[3 * i + 2] = iz;
}

__global__ void __launch_bounds__(STEP_BLOCK) k_step2(StepArgs a)
{
    __shared__ double s_gamma[MAX_GAMMA_TYPES];
    if (!a.use_lambda)
        for (uint32_t t = threadIdx.x; t < a.ntypes; t += blockDim.x) s_gamma[t] = a.gamma[t];
    __syncthreads();
    const uint32_t g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= a.n) return;
    const uint32_t i = a.group ? a.group[g] : g;
    const double4_32a p = a.pos[i];
    const double gam = a.use_lambda ? a.lambda * a.diameter[i] : s_gamma[type_of(p.w)];
    double ux, uy, uz;
    flow_at(a.flow, p.y, ux, uy, uz);
    const double c = a.noiseless ? 0.0 : sqrt(6.0 * gam * a.kT / a.dt);
    double r0, r1, r2;
    uniform3(AZP_RNG_LANGEVIN_FLOW, a.timestep, a.seed, a.tag[i], -c, c - (-c), r0, r1, r2);
    double4_32a v = a.vel[i];
    const double3 f = load_force(a.net_force, a.net_precision, i);
    const double minv = 1.0 / v.w;
    const double axx = (f.x + (r0 - gam * (v.x - ux))) * minv;
    const double ayy = (f.y + (r1 - gam * (v.y - uy))) * minv;
    const double azz = (f.z + (r2 - gam * (v.z - uz))) * minv;
    const double h = 0.5 * a.dt;
    v.x += h * axx;
    v.y += h * ayy;
    v.z += h * azz;
    a.vel[i] = v;
    a.accel[3 * i] = axx;
    a.accel[3 * i + 1] = ayy;
    a.accel[3 * i + 2] = azz;
}

__global__ void __launch_bounds__(STEP_BLOCK) k_brownian(StepArgs a)
{
    __shared__ double s_gamma[MAX_GAMMA_TYPES];
    if (!a.use_lambda)
        for (uint32_t t = threadIdx.x; t < a.ntypes; t += blockDim.x) s_gamma[t] = a.gamma[t];
    __syncthreads();
    const uint32_t g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= a.n) return;
    const uint32_t i = a.group ? a.group[g] : g;
    double4_32a p = a.pos[i];
    const double gam = a.use_lambda ? a.lambda * a.diameter[i] : s_gamma[type_of(p.w)];
    double ux, uy, uz;
    flow_at(a.flow, p.y, ux, uy, uz);
    const double c = a.noiseless ? 0.0 : sqrt(6.0 * gam * a.kT / a.dt);
    double r0, r1, r2;
    uniform3(AZP_RNG_BROWNIAN_FLOW, a.timestep, a.seed, a.tag[i], -c, c - (-c), r0, r1, r2);
    const double3 f = load_force(a.net_force, a.net_precision, i);
    double dx = (ux + (f.x + r0) / gam) * a.dt;
    double dy = (uy + (f.y + r1) / gam) * a.dt;
    double dz = (uz + (f.z + r2) / gam) * a.dt;
    if (a.max_disp > 0.0) {
        dx = fmin(fmax(dx, -a.max_disp), a.max_disp);
        dy = fmin(fmax(dy, -a.max_disp), a.max_disp);
        dz = fmin(fmax(dz, -a.max_disp), a.max_disp);
    }
    p.x += dx;
    p.y += dy;
    p.z += dz;
    int ix = a.image[3 * i], iy = a.image[3 * i + 1], iz = a.image[3 * i + 2];
    wrap1(p.x, ix, a.L[0], a.lo[0], a.hi[0]);
    wrap1(p.y, iy, a.L[1], a.lo[1], a.hi[1]);
    wrap1(p.z, iz, a.L[2], a.lo[2], a.hi[2]);
    a.pos[i] = p;  // type bits kept
    a.image[3 * i] = ix;
    a.image[3 * i + 1] = iy;
    a.image[3 * i + 2] = iz;
}

__global__ void k_uniform3(uint32_t id, uint64_t timestep, uint32_t seed, const uint32_t* __restrict__ tags,
                           uint32_t n, double lo, double width, double* __restrict__ out)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double r0, r1, r2;
    uniform3(id, timestep, seed, tags[i], lo, width, r0, r1, r2);
    out[3 * i] = r0;
    out[3 * i + 1] = r1;
    out[3 * i + 2] = r2;
}

int launch_step1(const StepArgs& a, cudaStream_t s)
{
    if (a.n == 0) return AZP_OK;
    k_step1<<<(a.n + STEP_BLOCK - 1) / STEP_BLOCK, STEP_BLOCK, 0, s>>>(a);
    AZP_CHECK_LAUNCH("k_step1");
    return AZP_OK;
}

int launch_step2(const StepArgs& a, cudaStream_t s)
{
    if (a.n == 0) return AZP_OK;
    if (!a.use_lambda && a.ntypes > MAX_GAMMA_TYPES) return AZP_ERR_INVALID;
    k_step2<<<(a.n + STEP_BLOCK - 1) / STEP_BLOCK, STEP_BLOCK, 0, s>>>(a);
    AZP_CHECK_LAUNCH("k_step2");
    return AZP_OK;
}

int launch_brownian(const StepArgs& a, cudaStream_t s)
{
    if (a.n == 0) return AZP_OK;
    if (!a.use_lambda && a.ntypes > MAX_GAMMA_TYPES) return AZP_ERR_INVALID;
    k_brownian<<<(a.n + STEP_BLOCK - 1) / STEP_BLOCK, STEP_BLOCK, 0, s>>>(a);
    AZP_CHECK_LAUNCH("k_brownian");
    return AZP_OK;
}

int launch_uniform3(uint32_t id, uint64_t timestep, uint32_t seed, const uint32_t* tags, uint32_t n, double lo,
                    double hi, double* out, cudaStream_t s)
{
    if (n == 0) return AZP_OK;
    k_uniform3<<<(n + 255) / 256, 256, 0, s>>>(id, timestep, seed, tags, n, lo, hi - lo, out);
    AZP_CHECK_LAUNCH("k_uniform3");
    return AZP_OK;
}

}  // namespace azp
