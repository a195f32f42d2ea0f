// engine.cu -- the resident MD engine (azp_md): state in cell order in HBM, one
// fused force-and-integrate launch per timestep, list rebuild + particle re-sort
// on the device when any particle moved more than r_buff / 2 since the last
// build (HOOMD's distance check), and CUDA-graph replay of the step sequence with
// the rebuild as a conditional node armed by the step kernel itself.
//
// Host-visible state is always in tag order; inside, index order is the cell
// order of the last rebuild and tag[] / rtag[] map between the two. The RNG is
// keyed by tag and timestep, so results do not depend on the order.
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "celllist.cuh"
#include "engine.cuh"
#include "engine_kernels.cuh"
#include "scan.cuh"

namespace azp
{
int launch_md_step(int pair_kind, int bond_kind, int precision, int integ, const MDArgs& a, cudaStream_t s)
{
    switch (pair_kind) {
    case -1: return launch_md_nopair(bond_kind, precision, integ, a, s);
    case AZP_PAIR_PERTURBED_LJ: return launch_md_plj(bond_kind, precision, integ, a, s);
    case AZP_PAIR_EXPANDED_YUKAWA: return launch_md_eyuk(bond_kind, precision, integ, a, s);
    case AZP_PAIR_HERTZ: return launch_md_hertz(bond_kind, precision, integ, a, s);
    case AZP_PAIR_COLLOID: return launch_md_colloid(bond_kind, precision, integ, a, s);
    case AZP_PAIR_DPD_GENERAL_WEIGHT: return launch_md_dpd(bond_kind, precision, integ, a, s);
    default: return AZP_ERR_INVALID;
    }
}

// ---------------------------------------------------------------- rebuild kernels
__global__ void k_zero_gated(uint32_t* __restrict__ p, uint32_t n, const uint32_t* __restrict__ gate)
{
    if (gated_off(gate)) return;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) p[i] = 0u;
}

struct PermArgs {
    const uint32_t* members;
    double4_32a *pos, *t_pos;   // pos NULL in FP32-force mode (the fixed words move instead)
    uint4 *fix, *t_fix;         // FP32-force mode: high and low fixed words, masses
    uint4 *lo, *t_lo;
    double *mass, *t_mass;
    uint4* fix_build;           // FP32-force mode: receives the new high words too
    double4_32a *vel, *t_vel;
    double *accel, *t_accel;
    int *image, *t_image;
    uint32_t *tag, *t_tag, *rtag;
    double *diam, *t_diam;
    uint32_t *cell_of, *t_cell;
    uint32_t N;
};

// temps[s] <- arrays[members[s]]
__global__ void k_perm_gather(PermArgs a, const uint32_t* __restrict__ gate)
{
    if (gated_off(gate)) return;
    const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= a.N) return;
    const uint32_t o = a.members[s];
    if (a.pos) a.t_pos[s] = a.pos[o];
    if (a.fix) {
        a.t_fix[s] = a.fix[o];
        a.t_lo[s] = a.lo[o];
        a.t_mass[s] = a.mass[o];
    }
    a.t_vel[s] = a.vel[o];
    a.t_accel[3 * s] = a.accel[3 * o];
    a.t_accel[3 * s + 1] = a.accel[3 * o + 1];
    a.t_accel[3 * s + 2] = a.accel[3 * o + 2];
    a.t_image[3 * s] = a.image[3 * o];
    a.t_image[3 * s + 1] = a.image[3 * o + 1];
    a.t_image[3 * s + 2] = a.image[3 * o + 2];
    a.t_tag[s] = a.tag[o];
    if (a.diam) a.t_diam[s] = a.diam[o];
    a.t_cell[s] = a.cell_of[o];
}

// arrays[s] <- temps[s]; rtag[tag[s]] = s
__global__ void k_perm_back(PermArgs a, const uint32_t* __restrict__ gate)
{
    if (gated_off(gate)) return;
    const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= a.N) return;
    if (a.pos) a.pos[s] = a.t_pos[s];
    if (a.fix) {
        const uint4 f = a.t_fix[s];
        a.fix[s] = f;
        a.fix_build[s] = f;
        a.lo[s] = a.t_lo[s];
        a.mass[s] = a.t_mass[s];
    }
    a.vel[s] = a.t_vel[s];
    a.accel[3 * s] = a.t_accel[3 * s];
    a.accel[3 * s + 1] = a.t_accel[3 * s + 1];
    a.accel[3 * s + 2] = a.t_accel[3 * s + 2];
    a.image[3 * s] = a.t_image[3 * s];
    a.image[3 * s + 1] = a.t_image[3 * s + 1];
    a.image[3 * s + 2] = a.t_image[3 * s + 2];
    const uint32_t t = a.t_tag[s];
    a.tag[s] = t;
    a.rtag[t] = s;
    if (a.diam) a.diam[s] = a.t_diam[s];
    a.cell_of[s] = a.t_cell[s];
}

// per-particle bond table and exclusions in the new index order, from the
// tag-order master table [k * N + tag]
__global__ void k_bond_table(const uint32_t* __restrict__ tag, const uint32_t* __restrict__ rtag,
                             const uint32_t* __restrict__ n_tag, const uint32_t* __restrict__ partner_tag,
                             const uint32_t* __restrict__ type_tag, uint32_t N, uint32_t* __restrict__ bt_n,
                             uint2* __restrict__ bt, uint32_t* __restrict__ ex_n, uint32_t* __restrict__ ex_idx,
                             int exclude, const uint32_t* __restrict__ gate)
{
    if (gated_off(gate)) return;
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= N) return;
    const uint32_t t = tag[i];
    const uint32_t n = n_tag[t];
    for (uint32_t k = 0; k < n; ++k) {
        const uint32_t p = rtag[partner_tag[(size_t)k * N + t]];
        bt[(size_t)k * N + i] = make_uint2(p, type_tag[(size_t)k * N + t]);
        if (exclude) ex_idx[(size_t)k * N + i] = p;
    }
    bt_n[i] = n;
    if (ex_n) ex_n[i] = exclude ? n : 0u;
}

// The kind of this list build, as two gates for the kernels that differ between
// them: out[0] the re-sorting build (forced, or after sort_every - 1
// order-keeping ones, counted in out[4]), out[2] the order-keeping one; both 0
// when the build is gated off. out[1] and out[3] stay 0 (the error word of a gate).
__global__ void k_sort_decide(const uint32_t* __restrict__ gate, uint32_t sort_every, int force,
                              uint32_t* __restrict__ out)
{
    const bool on = !gated_off(gate);
    const bool sort = force || out[4] + 1u >= sort_every;
    out[0] = on && sort ? 1u : 0u;
    out[1] = 0u;
    out[2] = on && !sort ? 1u : 0u;
    out[3] = 0u;
    if (on) out[4] = sort ? 0u : out[4] + 1u;
}

// an order-keeping build's new reference positions for the displacement test
__global__ void k_copy_fix_build(const uint4* __restrict__ fix, uint4* __restrict__ fix_build, uint32_t N,
                                 const uint32_t* __restrict__ gate)
{
    if (gated_off(gate)) return;
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < N) fix_build[i] = fix[i];
}

__global__ void k_finish_rebuild(uint32_t* __restrict__ flags, const uint32_t* __restrict__ gate)
{
    if (gated_off(gate)) return;
    flags[0] = 0u;
    flags[2] += 1u;
}

// first graph node of a replay: arm the first conditional from the request flag
__global__ void k_arm(const uint32_t* __restrict__ flags, cudaGraphConditionalHandle h)
{
    cudaGraphSetConditional(h, (flags[0] && !flags[1]) ? 1u : 0u);
}

// Langevin step one in place at the start of a run (src/TwoStepLangevinFlow.h:128-153)
__global__ void k_md_step1(double4_32a* __restrict__ pos, uint4* __restrict__ fix, const uint4* __restrict__ fix_build,
                           double4_32a* __restrict__ vel, const double* __restrict__ accel, int* __restrict__ image,
                           uint32_t N, double dt, double L0, double L1, double L2, double Li0, double Li1, double Li2,
                           float s0, float s1, float s2, float thresh2, uint32_t* __restrict__ flags,
                           uint32_t group_types)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    bool want = false;
    // a particle outside the method's group does not move
    const bool mover = i < N && (group_types == 0xffffffffu ||
                                 (type_of(pos[i].w) < 32u && ((group_types >> type_of(pos[i].w)) & 1u)));
    if (mover) {
        double4_32a p = pos[i];
        double4_32a v = vel[i];
        const double ax = accel[3 * i], ay = accel[3 * i + 1], az = accel[3 * i + 2];
        const double h = 0.5 * dt;
        p.x += (v.x + h * ax) * dt;
        p.y += (v.y + h * ay) * dt;
        p.z += (v.z + h * az) * dt;
        int wx = 0, wy = 0, wz = 0;
        wrap1(p.x, wx, L0, -0.5 * L0, 0.5 * L0);
        wrap1(p.y, wy, L1, -0.5 * L1, 0.5 * L1);
        wrap1(p.z, wz, L2, -0.5 * L2, 0.5 * L2);
        if (wx | wy | wz) {
            image[3 * i] += wx;
            image[3 * i + 1] += wy;
            image[3 * i + 2] += wz;
        }
        v.x += h * ax;
        v.y += h * ay;
        v.z += h * az;
        pos[i] = p;
        vel[i] = v;
        uint4 f;
        f.x = to_fixed(p.x, Li0);
        f.y = to_fixed(p.y, Li1);
        f.z = to_fixed(p.z, Li2);
        f.w = type_of(p.w);
        fix[i] = f;
        const uint4 fb = fix_build[i];
        const float dx = (float)(int32_t)(f.x - fb.x) * s0;
        const float dy = (float)(int32_t)(f.y - fb.y) * s1;
        const float dz = (float)(int32_t)(f.z - fb.z) * s2;
        want = dx * dx + dy * dy + dz * dz > thresh2;
    }
    if (__any_sync(0xffffffffu, want) && (threadIdx.x & 31) == 0) atomicOr(&flags[0], 1u);
}

// FP32-force mode: Langevin step one in place at the start of a run, on the
// 64-bit fixed positions and float-float velocities (fixed64.cuh)
__global__ void k_md_step1_fx(uint4* __restrict__ fix, uint4* __restrict__ lo, const uint4* __restrict__ fix_build,
                              VelFF* __restrict__ vel, const double* __restrict__ accel, int* __restrict__ image,
                              uint32_t N, float dt, float3 s64h, float3 s64l, float3 sfix, float thresh2,
                              uint32_t* __restrict__ flags, uint32_t group_types)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    bool want = false;
    // a particle outside the method's group does not move
    const bool mover = i < N && (group_types == 0xffffffffu ||
                                 (fix[i].w < 32u && ((group_types >> fix[i].w) & 1u)));
    if (mover) {
        uint4 f = fix[i];
        uint4 l = lo[i];
        VelFF v = vel[i];
        const float h = 0.5f * dt;
        const float kx = h * (float)accel[3 * i], ky = h * (float)accel[3 * i + 1], kz = h * (float)accel[3 * i + 2];
        bool bad = false;
        const int wx = fx_advance(f.x, l.x, (v.h.x + kx) * dt, s64h.x, s64l.x, bad);
        const int wy = fx_advance(f.y, l.y, (v.h.y + ky) * dt, s64h.y, s64l.y, bad);
        const int wz = fx_advance(f.z, l.z, (v.h.z + kz) * dt, s64h.z, s64l.z, bad);
        if (wx | wy | wz) {
            image[3 * i] += wx;
            image[3 * i + 1] += wy;
            image[3 * i + 2] += wz;
        }
        ff_add(v.h.x, v.l.x, kx);
        ff_add(v.h.y, v.l.y, ky);
        ff_add(v.h.z, v.l.z, kz);
        fix[i] = f;
        lo[i] = l;
        vel[i] = v;
        const uint4 fb = fix_build[i];
        const float dx = (float)(int32_t)(f.x - fb.x) * sfix.x;
        const float dy = (float)(int32_t)(f.y - fb.y) * sfix.y;
        const float dz = (float)(int32_t)(f.z - fb.z) * sfix.z;
        want = dx * dx + dy * dy + dz * dz > thresh2;
        if (bad) atomicOr(&flags[1], AZP_EBIT_NONFINITE);
    }
    if (__any_sync(0xffffffffu, want) && (threadIdx.x & 31) == 0) atomicOr(&flags[0], 1u);
}

// FP32-force mode: the walls' force and energy of each particle at the step's
// positions, for the step kernel to add: an FP32 screen on the high words, then
// the FP64 evaluation on the full 64-bit position for the particles some wall
// can reach (the others get zero)
__global__ void k_walls_fx(MDArgs a)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.N) return;
    const uint4 hw = __ldg(a.fix + i);
    double fw[4] = {0.0, 0.0, 0.0, 0.0};
    if (walls_near_f(a.walls, a.wall_tab, hw.w, (float)(int32_t)hw.x * a.sfix[0], (float)(int32_t)hw.y * a.sfix[1],
                     (float)(int32_t)hw.z * a.sfix[2], a.wall_tol)) {
        const uint4 lw = __ldg(a.flo + i);
        engine_walls(a.wall_kind, a.walls, a.wall_tab, fx_to_double(fx_join(hw.x, lw.x), a.l64[0]),
                     fx_to_double(fx_join(hw.y, lw.y), a.l64[1]), fx_to_double(fx_join(hw.z, lw.z), a.l64[2]), hw.w,
                     fw);
    }
    const_cast<float4*>(a.wall_f)[i] = make_float4((float)fw[0], (float)fw[1], (float)fw[2], (float)fw[3]);
}

// What a step reads of its neighbours while their owners update it in the same
// step, copied right before the step: DPD the velocities (FP64: (v, mass);
// FP32-force: the leading floats (v, 1/m)), ImageHarmonic bonds the image counts.
// Either output may be null.
__global__ void k_step_snapshot(const double4_32a* __restrict__ vel, const int* __restrict__ image, uint32_t N,
                                int fx, void* __restrict__ vel_out, int* __restrict__ img_out)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= N) return;
    if (vel_out) {
        if (fx)
            reinterpret_cast<float4*>(vel_out)[i] = reinterpret_cast<const VelFF*>(vel)[i].h;
        else
            reinterpret_cast<double4_32a*>(vel_out)[i] = vel[i];
    }
    if (img_out)
        for (int d = 0; d < 3; ++d) img_out[3 * (size_t)i + d] = image[3 * (size_t)i + d];
}

// FP32-force mode: FP64 state (k_load_state's layout) -> fixed words, float-float
// velocities (vel buffer, in place) and masses
__global__ void k_state_to_fx(const double4_32a* __restrict__ pos, double4_32a* __restrict__ vel,
                              uint4* __restrict__ fix, uint4* __restrict__ lo, double* __restrict__ mass, uint32_t N,
                              double Li0, double Li1, double Li2)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= N) return;
    const double4_32a p = pos[i];
    uint4 h, l;
    fx_split(fx_from_double(p.x, Li0), h.x, l.x);
    fx_split(fx_from_double(p.y, Li1), h.y, l.y);
    fx_split(fx_from_double(p.z, Li2), h.z, l.z);
    h.w = type_of(p.w);
    l.w = 0u;
    fix[i] = h;
    lo[i] = l;
    const double4_32a v = vel[i];
    VelFF f;
    f.h = make_float4((float)v.x, (float)v.y, (float)v.z, (float)(1.0 / v.w));
    f.l = make_float4((float)(v.x - (double)f.h.x), (float)(v.y - (double)f.h.y), (float)(v.z - (double)f.h.z), 0.0f);
    mass[i] = v.w;
    *reinterpret_cast<VelFF*>(vel + i) = f;
}

// Rows of three per particle (accelerations, image counts) of one full block of
// STATE_BLOCK tags move between the caller's buffer and shared memory as 16-byte
// vectors, so that over the host link they travel in whole lines; a partial last
// block, or a buffer off a 16-byte boundary, moves them one element at a time.
constexpr int STATE_BLOCK = 256;

template <int W, class T>
__device__ __forceinline__ void rows_copy(T* __restrict__ dst, const T* __restrict__ src)
{
    static_assert(W * STATE_BLOCK * sizeof(T) % 16 == 0, "whole vectors per block");
    constexpr int NV = W * STATE_BLOCK * (int)sizeof(T) / 16;
    for (int k = threadIdx.x; k < NV; k += STATE_BLOCK)
        reinterpret_cast<uint4*>(dst)[k] = reinterpret_cast<const uint4*>(src)[k];
}
template <class T>
__device__ __forceinline__ void rows3_copy(T* __restrict__ dst, const T* __restrict__ src)
{
    rows_copy<3>(dst, src);
}

// Rows of four doubles (positions, velocities) of tag t. A full block goes
// through shared memory (`full`, uniform over the block), so that it reads or
// writes the caller's buffer as one contiguous run of 16-byte vectors, a warp
// covering whole 128-byte lines per access: over the host link that moves a
// pinned buffer in place at the link's rate (two 16-byte accesses per lane at a
// 32-byte stride cover half of each line apiece, and wrote at about half of it).
__device__ __forceinline__ void put_row4(double* __restrict__ out, double* s, uint32_t t, bool full, double a,
                                         double b, double c, double d)
{
    if (full) {
        reinterpret_cast<double2*>(s)[2 * threadIdx.x] = make_double2(a, b);
        reinterpret_cast<double2*>(s)[2 * threadIdx.x + 1] = make_double2(c, d);
    } else {
        reinterpret_cast<double2*>(out)[2 * (size_t)t] = make_double2(a, b);
        reinterpret_cast<double2*>(out)[2 * (size_t)t + 1] = make_double2(c, d);
    }
}
__device__ __forceinline__ void get_row4(const double* __restrict__ in, const double* s, uint32_t t, bool full,
                                         double2& ab, double2& cd)
{
    const double2* src = full ? reinterpret_cast<const double2*>(s) + 2 * threadIdx.x
                              : reinterpret_cast<const double2*>(in) + 2 * (size_t)t;
    ab = src[0];
    cd = src[1];
}

// Writes particle i's rows of three (tag t, thread `lane` of the block) to the
// block's shared rows or straight to the outputs; the block then writes its shared
// rows out whole. `vec` is uniform over the block.
__device__ __forceinline__ void store_rows3(const double* __restrict__ accel, const int* __restrict__ image,
                                            uint32_t i, uint32_t t, bool live, bool vec, double* s_acc, int* s_img,
                                            double* __restrict__ accel_out, int* __restrict__ image_out,
                                            uint32_t t0)
{
    if (live)
        for (int d = 0; d < 3; ++d) {
            if (accel_out) {
                const double a = accel[3 * (size_t)i + d];
                if (vec) s_acc[3 * threadIdx.x + d] = a;
                else accel_out[3 * (size_t)t + d] = a;
            }
            if (image_out) {
                const int g = image[3 * (size_t)i + d];
                if (vec) s_img[3 * threadIdx.x + d] = g;
                else image_out[3 * (size_t)t + d] = g;
            }
        }
    if (vec) {
        __syncthreads();
        if (accel_out) rows3_copy(accel_out + 3 * (size_t)t0, s_acc);
        if (image_out) rows3_copy(image_out + 3 * (size_t)t0, s_img);
    }
}

// FP32-force mode: device state -> tag order output (the k_store_state layout)
__global__ void __launch_bounds__(STATE_BLOCK)
    k_store_state_fx(const uint4* __restrict__ fix, const uint4* __restrict__ lo, const VelFF* __restrict__ vel,
                     const double* __restrict__ mass, const double* __restrict__ accel, const int* __restrict__ image,
                     const uint32_t* __restrict__ rtag, uint32_t N, double l0, double l1, double l2,
                     double* __restrict__ pos_out, double* __restrict__ vel_out, double* __restrict__ accel_out,
                     int* __restrict__ image_out, int rows_aligned)
{
    __shared__ __align__(16) double s_acc[3 * STATE_BLOCK];
    __shared__ __align__(16) int s_img[3 * STATE_BLOCK];
    __shared__ __align__(16) double s_pos[4 * STATE_BLOCK], s_vel[4 * STATE_BLOCK];
    // one thread per tag: the outputs are written in order (they may be the
    // caller's pinned buffers, written over the host link)
    const uint32_t t0 = blockIdx.x * STATE_BLOCK;
    const uint32_t t = t0 + threadIdx.x;
    const bool live = t < N, full = t0 + STATE_BLOCK <= N, rows_vec = rows_aligned && full;
    const uint32_t i = live ? rtag[t] : 0u;
    if (live && pos_out) {
        const uint4 h = fix[i], l = lo[i];
        put_row4(pos_out, s_pos, t, full, fx_to_double(fx_join(h.x, l.x), l0), fx_to_double(fx_join(h.y, l.y), l1),
                 fx_to_double(fx_join(h.z, l.z), l2), (double)h.w);
    }
    if (live && vel_out) {
        const VelFF v = vel[i];
        put_row4(vel_out, s_vel, t, full, (double)v.h.x + (double)v.l.x, (double)v.h.y + (double)v.l.y,
                 (double)v.h.z + (double)v.l.z, mass[i]);
    }
    store_rows3(accel, image, i, t, live, rows_vec, s_acc, s_img, accel_out, image_out, t0);
    if (full) {
        if (!rows_vec) __syncthreads();
        if (pos_out) rows_copy<4>(pos_out + 4 * (size_t)t0, s_pos);
        if (vel_out) rows_copy<4>(vel_out + 4 * (size_t)t0, s_vel);
    }
}

// accelerations a = F / m (HOOMD sets them this way before the first step)
__global__ void k_accel_from_force(const double4_32a* __restrict__ f, const double4_32a* __restrict__ vel,
                                   const double* __restrict__ mass, double* __restrict__ accel, uint32_t N)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= N) return;
    const double4_32a F = f[i];
    const double minv = 1.0 / (mass ? mass[i] : vel[i].w);
    accel[3 * i] = F.x * minv;
    accel[3 * i + 1] = F.y * minv;
    accel[3 * i + 2] = F.z * minv;
}

// thermo partial sums per block (deterministic two-pass reduction)
constexpr int THERMO_BLOCK = 256;
__global__ void k_thermo_partials(const double4_32a* __restrict__ f, const double* __restrict__ vir,
                                  const double4_32a* __restrict__ vel, const double* __restrict__ mass, uint32_t N,
                                  double* __restrict__ part)
{
    __shared__ double s[THERMO_BLOCK][8];
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    double v[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    if (i < N) {
        v[0] = f[i].w;
        if (mass) {
            // FP32-force mode: float-float velocities
            const VelFF u = reinterpret_cast<const VelFF*>(vel)[i];
            const double x = (double)u.h.x + (double)u.l.x, y = (double)u.h.y + (double)u.l.y,
                         z = (double)u.h.z + (double)u.l.z;
            v[1] = 0.5 * mass[i] * (x * x + y * y + z * z);
        } else {
            const double4_32a u = vel[i];
            v[1] = 0.5 * u.w * (u.x * u.x + u.y * u.y + u.z * u.z);
        }
        for (int c = 0; c < 6; ++c) v[2 + c] = vir[(size_t)c * N + i];
    }
    for (int c = 0; c < 8; ++c) s[threadIdx.x][c] = v[c];
    __syncthreads();
    for (int st = THERMO_BLOCK / 2; st > 0; st >>= 1) {
        if ((int)threadIdx.x < st)
            for (int c = 0; c < 8; ++c) s[threadIdx.x][c] += s[threadIdx.x + st][c];
        __syncthreads();
    }
    if (threadIdx.x == 0)
        for (int c = 0; c < 8; ++c) part[(size_t)blockIdx.x * 8 + c] = s[0][c];
}

// one block of THERMO_BLOCK threads: thread t sums the partials of blocks t,
// t + THERMO_BLOCK, ... in order, then a fixed tree adds the threads' sums (the
// same order every call)
// out[0..7]: the sums; out[8..11]: the engine's eight flag words, so that one
// read returns both
__global__ void __launch_bounds__(THERMO_BLOCK) k_thermo_final(const double* __restrict__ part, uint32_t nb,
                                                              const uint32_t* __restrict__ flags,
                                                              double* __restrict__ out)
{
    __shared__ double s[THERMO_BLOCK][8];
    double acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    for (uint32_t b = threadIdx.x; b < nb; b += THERMO_BLOCK)
        for (int c = 0; c < 8; ++c) acc[c] += part[(size_t)b * 8 + c];
    for (int c = 0; c < 8; ++c) s[threadIdx.x][c] = acc[c];
    __syncthreads();
    for (int st = THERMO_BLOCK / 2; st > 0; st >>= 1) {
        if ((int)threadIdx.x < st)
            for (int c = 0; c < 8; ++c) s[threadIdx.x][c] += s[threadIdx.x + st][c];
        __syncthreads();
    }
    if (threadIdx.x < 8) out[threadIdx.x] = s[0][threadIdx.x];
    else if (threadIdx.x < 16) reinterpret_cast<uint32_t*>(out + 8)[threadIdx.x - 8] = flags[threadIdx.x - 8];
}

// index order -> tag order
__global__ void k_to_tag_order4(const double4_32a* __restrict__ src, const uint32_t* __restrict__ tag, uint32_t N,
                                double4_32a* __restrict__ dst)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < N) dst[tag[i]] = src[i];
}

__global__ void k_to_tag_order_n(const double* __restrict__ src, const uint32_t* __restrict__ tag, uint32_t N,
                                 int ncomp, int soa, double* __restrict__ dst)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= N) return;
    const uint32_t t = tag[i];
    for (int c = 0; c < ncomp; ++c) dst[(size_t)t * ncomp + c] = soa ? src[(size_t)c * N + i] : src[(size_t)i * ncomp + c];
}

__global__ void k_to_tag_order_i3(const int* __restrict__ src, const uint32_t* __restrict__ tag, uint32_t N,
                                  int* __restrict__ dst)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= N) return;
    const uint32_t t = tag[i];
    dst[3 * t] = src[3 * i];
    dst[3 * t + 1] = src[3 * i + 1];
    dst[3 * t + 2] = src[3 * i + 2];
}

// Reads the position and velocity rows of a full block into shared memory (see
// put_row4), followed by a barrier unless load_rows3 (rows_vec) gives one.
__device__ __forceinline__ void load_rows4(const double* __restrict__ pos_in, const double* __restrict__ vel_in,
                                           bool full, bool rows_vec, double* s_pos, double* s_vel, uint32_t t0)
{
    if (!full) return;
    rows_copy<4>(s_pos, pos_in + 4 * (size_t)t0);
    rows_copy<4>(s_vel, vel_in + 4 * (size_t)t0);
    if (!rows_vec) __syncthreads();
}

// Reads the rows of three of the block's tags (see store_rows3) into shared
// memory when `vec`; returns particle t's row values either way.
__device__ __forceinline__ void load_rows3(const double* __restrict__ accel_in, const int* __restrict__ image_in,
                                           uint32_t t, bool live, bool vec, double* s_acc, int* s_img, uint32_t t0,
                                           double a[3], int g[3])
{
    if (vec) {
        if (accel_in) rows3_copy(s_acc, accel_in + 3 * (size_t)t0);
        if (image_in) rows3_copy(s_img, image_in + 3 * (size_t)t0);
        __syncthreads();
    }
    if (!live) return;
    for (int d = 0; d < 3; ++d) {
        a[d] = !accel_in ? 0.0 : vec ? s_acc[3 * threadIdx.x + d] : accel_in[3 * (size_t)t + d];
        g[d] = !image_in ? 0 : vec ? s_img[3 * threadIdx.x + d] : image_in[3 * (size_t)t + d];
    }
}

// tag-order input (pos w = integer-valued type) -> device state, identity order
__global__ void __launch_bounds__(STATE_BLOCK)
    k_load_state(const double* __restrict__ pos_in, const double* __restrict__ vel_in,
                 const double* __restrict__ accel_in, const int* __restrict__ image_in,
                 const double* __restrict__ diam_in, uint32_t N, double4_32a* __restrict__ pos,
                 double4_32a* __restrict__ vel, double* __restrict__ accel, int* __restrict__ image,
                 double* __restrict__ diam, uint32_t* __restrict__ tag, uint32_t* __restrict__ rtag, int rows_aligned)
{
    __shared__ __align__(16) double s_acc[3 * STATE_BLOCK];
    __shared__ __align__(16) int s_img[3 * STATE_BLOCK];
    __shared__ __align__(16) double s_pos[4 * STATE_BLOCK], s_vel[4 * STATE_BLOCK];
    const uint32_t t0 = blockIdx.x * STATE_BLOCK;
    const uint32_t i = t0 + threadIdx.x;
    const bool live = i < N, full = t0 + STATE_BLOCK <= N;
    double a[3];
    int g[3];
    // the inputs may be the caller's pinned buffers, read over the host link
    load_rows4(pos_in, vel_in, full, rows_aligned && full, s_pos, s_vel, t0);
    load_rows3(accel_in, image_in, i, live, rows_aligned && full, s_acc, s_img, t0, a, g);
    if (!live) return;
    double2 p01, p23, v01, v23;
    get_row4(pos_in, s_pos, i, full, p01, p23);
    get_row4(vel_in, s_vel, i, full, v01, v23);
    pos[i] = make_double4_32a(p01.x, p01.y, p23.x, type_as_double((uint32_t)p23.y));
    vel[i] = make_double4_32a(v01.x, v01.y, v23.x, v23.y);
    for (int d = 0; d < 3; ++d) {
        accel[3 * (size_t)i + d] = a[d];
        image[3 * (size_t)i + d] = g[d];
    }
    if (diam) diam[i] = diam_in ? diam_in[i] : 1.0;
    tag[i] = i;
    rtag[i] = i;
}

// tag-order input -> device state in the engine's current index order (particle
// i takes the input row of its tag); tag / rtag are kept
__global__ void __launch_bounds__(STATE_BLOCK)
    k_load_state_ordered(const double* __restrict__ pos_in, const double* __restrict__ vel_in,
                         const double* __restrict__ accel_in, const int* __restrict__ image_in,
                         const double* __restrict__ diam_in, const uint32_t* __restrict__ rtag, uint32_t N,
                         double4_32a* __restrict__ pos, double4_32a* __restrict__ vel, double* __restrict__ accel,
                         int* __restrict__ image, double* __restrict__ diam, int rows_aligned)
{
    __shared__ __align__(16) double s_acc[3 * STATE_BLOCK];
    __shared__ __align__(16) int s_img[3 * STATE_BLOCK];
    // one thread per tag: the inputs are read in order
    __shared__ __align__(16) double s_pos[4 * STATE_BLOCK], s_vel[4 * STATE_BLOCK];
    const uint32_t t0 = blockIdx.x * STATE_BLOCK;
    const uint32_t t = t0 + threadIdx.x;
    const bool live = t < N, full = t0 + STATE_BLOCK <= N;
    double a[3];
    int g[3];
    // the inputs may be the caller's pinned buffers, read over the host link
    load_rows4(pos_in, vel_in, full, rows_aligned && full, s_pos, s_vel, t0);
    load_rows3(accel_in, image_in, t, live, rows_aligned && full, s_acc, s_img, t0, a, g);
    if (!live) return;
    const uint32_t i = rtag[t];
    double2 p01, p23, v01, v23;
    get_row4(pos_in, s_pos, t, full, p01, p23);
    get_row4(vel_in, s_vel, t, full, v01, v23);
    pos[i] = make_double4_32a(p01.x, p01.y, p23.x, type_as_double((uint32_t)p23.y));
    vel[i] = make_double4_32a(v01.x, v01.y, v23.x, v23.y);
    for (int d = 0; d < 3; ++d) {
        accel[3 * (size_t)i + d] = a[d];
        image[3 * (size_t)i + d] = g[d];
    }
    if (diam) diam[i] = diam_in ? diam_in[t] : 1.0;
}

// FP32-force mode, the three passes of an order-keeping load in one: tag-order
// input -> fixed words, float-float velocities and masses of particle i = rtag[t]
// (k_load_state_ordered + k_state_to_fx), and the rebuild request when i lies
// more than r_buff / 2 from its position at the last build (k_request_if_displaced)
__global__ void __launch_bounds__(STATE_BLOCK)
    k_load_state_ordered_fx(const double* __restrict__ pos_in, const double* __restrict__ vel_in,
                            const double* __restrict__ accel_in, const int* __restrict__ image_in,
                            const double* __restrict__ diam_in, const uint32_t* __restrict__ rtag, uint32_t N,
                            double Li0, double Li1, double Li2, uint4* __restrict__ fix, uint4* __restrict__ lo,
                            VelFF* __restrict__ velf, double* __restrict__ mass, double* __restrict__ accel,
                            int* __restrict__ image, double* __restrict__ diam, const uint4* __restrict__ fix_build,
                            float s0, float s1, float s2, float thresh2, uint32_t* __restrict__ flags, int rows_aligned)
{
    __shared__ __align__(16) double s_acc[3 * STATE_BLOCK];
    __shared__ __align__(16) int s_img[3 * STATE_BLOCK];
    __shared__ __align__(16) double s_pos[4 * STATE_BLOCK], s_vel[4 * STATE_BLOCK];
    const uint32_t t0 = blockIdx.x * STATE_BLOCK;
    const uint32_t t = t0 + threadIdx.x;
    const bool live = t < N, full = t0 + STATE_BLOCK <= N;
    double a3[3];
    int g3[3];
    // the inputs may be the caller's pinned buffers, read over the host link
    load_rows4(pos_in, vel_in, full, rows_aligned && full, s_pos, s_vel, t0);
    load_rows3(accel_in, image_in, t, live, rows_aligned && full, s_acc, s_img, t0, a3, g3);
    bool want = false;
    if (live) {
        const uint32_t i = rtag[t];
        double2 p01, p23, v01, v23;
        get_row4(pos_in, s_pos, t, full, p01, p23);
        get_row4(vel_in, s_vel, t, full, v01, v23);
        uint4 h, l;
        fx_split(fx_from_double(p01.x, Li0), h.x, l.x);
        fx_split(fx_from_double(p01.y, Li1), h.y, l.y);
        fx_split(fx_from_double(p23.x, Li2), h.z, l.z);
        h.w = type_of(type_as_double((uint32_t)p23.y));
        l.w = 0u;
        fix[i] = h;
        lo[i] = l;
        VelFF f;
        f.h = make_float4((float)v01.x, (float)v01.y, (float)v23.x, (float)(1.0 / v23.y));
        f.l = make_float4((float)(v01.x - (double)f.h.x), (float)(v01.y - (double)f.h.y),
                          (float)(v23.x - (double)f.h.z), 0.0f);
        velf[i] = f;
        mass[i] = v23.y;
        for (int d = 0; d < 3; ++d) {
            accel[3 * (size_t)i + d] = a3[d];
            image[3 * (size_t)i + d] = g3[d];
        }
        if (diam) diam[i] = diam_in ? diam_in[t] : 1.0;
        const uint4 fb = fix_build[i];
        const float dx = (float)(int32_t)(h.x - fb.x) * s0;
        const float dy = (float)(int32_t)(h.y - fb.y) * s1;
        const float dz = (float)(int32_t)(h.z - fb.z) * s2;
        want = dx * dx + dy * dy + dz * dz > thresh2;
    }
    if (__any_sync(0xffffffffu, want) && (threadIdx.x & 31) == 0) atomicOr(&flags[0], 1u);
}

// rebuild request when a particle of the loaded state lies more than r_buff / 2
// from its position at the last list build (the step kernels' criterion)
__global__ void k_request_if_displaced(const uint4* __restrict__ fix, const uint4* __restrict__ fix_build, uint32_t N,
                                       float s0, float s1, float s2, float thresh2, uint32_t* __restrict__ flags)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    bool want = false;
    if (i < N) {
        const uint4 f = fix[i], fb = fix_build[i];
        const float dx = (float)(int32_t)(f.x - fb.x) * s0;
        const float dy = (float)(int32_t)(f.y - fb.y) * s1;
        const float dz = (float)(int32_t)(f.z - fb.z) * s2;
        want = dx * dx + dy * dy + dz * dz > thresh2;
    }
    if (__any_sync(0xffffffffu, want) && (threadIdx.x & 31) == 0) atomicOr(&flags[0], 1u);
}

// device state -> tag order output (pos w = type as an integer-valued double)
__global__ void __launch_bounds__(STATE_BLOCK)
    k_store_state(const double4_32a* __restrict__ pos, const double4_32a* __restrict__ vel,
                  const double* __restrict__ accel, const int* __restrict__ image, const uint32_t* __restrict__ rtag,
                  uint32_t N, double* __restrict__ pos_out, double* __restrict__ vel_out,
                  double* __restrict__ accel_out, int* __restrict__ image_out, int rows_aligned)
{
    __shared__ __align__(16) double s_acc[3 * STATE_BLOCK];
    __shared__ __align__(16) int s_img[3 * STATE_BLOCK];
    __shared__ __align__(16) double s_pos[4 * STATE_BLOCK], s_vel[4 * STATE_BLOCK];
    // one thread per tag: the outputs are written in order, 16 bytes at a time
    const uint32_t t0 = blockIdx.x * STATE_BLOCK;
    const uint32_t t = t0 + threadIdx.x;
    const bool live = t < N, full = t0 + STATE_BLOCK <= N, rows_vec = rows_aligned && full;
    const uint32_t i = live ? rtag[t] : 0u;
    if (live && pos_out) {
        const double4_32a p = pos[i];
        put_row4(pos_out, s_pos, t, full, p.x, p.y, p.z, (double)type_of(p.w));
    }
    if (live && vel_out) {
        const double4_32a v = vel[i];
        put_row4(vel_out, s_vel, t, full, v.x, v.y, v.z, v.w);
    }
    store_rows3(accel, image, i, t, live, rows_vec, s_acc, s_img, accel_out, image_out, t0);
    if (full) {
        if (!rows_vec) __syncthreads();
        if (pos_out) rows_copy<4>(pos_out + 4 * (size_t)t0, s_pos);
        if (vel_out) rows_copy<4>(vel_out + 4 * (size_t)t0, s_vel);
    }
}

}  // namespace azp

using namespace azp;

struct azp_md {
    uint32_t N = 0, ntypes = 0, nbt = 0;
    int precision = AZP_FP64, pair_kind = -1, shift_mode = 0, bond_kind = -1, method = 0;
    int exclude_bonds = 1, use_lambda = 0, noiseless = 0, tpp = 1;
    // The particles are re-sorted into cell order at every sort_every-th list
    // build (and at every unconditional one); the builds between keep the order
    // and scan through the cell member table. 0 (the default): every 4th build
    // on a grid of at most 4 particles per cell and a 27-cell stencil, every
    // build otherwise. Measured on one GB300: the bead-spring melt (N =
    // 1,048,600, ~3 particles per cell, 2,000 steps) 6,063 timesteps/s
    // re-sorting at every build, 6,241 at every 4th, 6,107 at every 8th, 6,094 at
    // every 16th (the order drifts and the member-table scan slows); the others
    // lose instead, where drifted lanes scan more divergent rows than the re-sort
    // costs: the LJ fluid (~33 particles per cell) 12,591 -> 11,714 at every 4th,
    // the DPD fluid (~6.6) 0.612 -> 0.641 ms per step, the colloid mixture (~4
    // per cell of a subdivided grid with a 343-cell stencil) 1,114 -> 1,081.
    uint32_t sort_every = 0;
    // [sort, 0, keep, 0]: gates of the two kinds of build; [4]: order-keeping
    // builds since the last re-sort (kept across loaded states, unlike flags)
    uint32_t* sort_gate = nullptr;
    double r_buff = 0.4, dt = 0.005, kT = 1.0, lambda = 0.0, max_disp = 0.0, fcap = 0.0;
    uint32_t seed = 0;
    FlowD flow{};
    azp_box box{};
    std::vector<double> pair_params, r_cut, r_on, bond_params, gamma;
    std::vector<double> pair_table_host, noise_host;  // the device tables, kept for the step arguments
    // device state
    double4_32a* pos[2] = {nullptr, nullptr};
    uint4* fix[2] = {nullptr, nullptr};
    uint4* lo[2] = {nullptr, nullptr};  // FP32-force mode: low fixed words
    double* mass = nullptr;             // FP32-force mode: masses (vel holds VelFF records)
    double* t_mass = nullptr;
    int cur = 0;
    uint4* fix_build = nullptr;
    double4_32a* vel = nullptr;
    double* accel = nullptr;
    int* image = nullptr;
    uint32_t* tag = nullptr;
    uint32_t* rtag = nullptr;
    double* diam = nullptr;
    // permutation temps
    double4_32a* t_pos = nullptr;
    double4_32a* t_vel = nullptr;
    double* t_accel = nullptr;
    int* t_image = nullptr;
    uint32_t* t_tag = nullptr;
    double* t_diam = nullptr;
    uint32_t* t_cell = nullptr;
    // cells
    CellGrid grid{};
    uint32_t *cell_of = nullptr, *slot = nullptr, *cell_count = nullptr, *cell_start = nullptr, *members = nullptr,
             *scan_tmp = nullptr;
    // list
    uint32_t max_nn = 0;
    uint32_t* counts = nullptr;
    uint32_t* nbrs = nullptr;
    ListCut* cuts = nullptr;
    double rlist_max = 0.0, rlist_min = 0.0;
    // bonds
    uint32_t bt_width = 0;
    uint32_t *bt_n_tag = nullptr, *bt_partner_tag = nullptr, *bt_type_tag = nullptr;
    uint32_t* bt_n = nullptr;
    uint2* bt = nullptr;
    uint32_t* ex_n = nullptr;
    uint32_t* ex_idx = nullptr;
    double* d_bond_params = nullptr;
    double* d_pair_table = nullptr;
    double* h_thermo = nullptr;  // pinned readback of the thermo sums and flags
    long long* d_contact_q = nullptr;  // colloid gap forms in a cubic box
    double* d_gamma = nullptr;
    double* d_noise = nullptr;
    // harmonic barrier (bar_geom -1: none): per-type (k, offset), the device table
    // of per-(timestep, type) records and its header (first timestep, rows)
    int bar_geom = -1;
    std::vector<double> bar_params;
    double* d_bar_tab = nullptr;  // 16-byte records, as double pairs
    unsigned long long* d_bar_hdr = nullptr;
    bool bar_set = false;
    // wall potential (wall_kind -1: none): the walls and the per-type table
    int wall_kind = -1;
    WallField* d_walls = nullptr;
    double* d_wall_tab = nullptr;
    float4* d_wall_f = nullptr;  // FP32-force mode: per-particle wall force and energy
    float wall_tol = 0.0f;
    // integration group by type (0xffffffff: every particle)
    uint32_t group_types = 0xffffffffu;
    // shared-memory neighbour tiles of the single-type FP32-force step (null: off)
    uint32_t* tile_tab = nullptr;
    // temperature table of a varying kT (allocated on the first
    // azp_md_set_temperatures; null while kT is the constant of the config)
    unsigned long long* d_kT_hdr = nullptr;
    double* d_kT_tab = nullptr;
    double* d_noise_tab = nullptr;
    // DPD: kT of the thermostat and the step's velocity snapshot
    double dpd_kT = 0.0;
    double* d_dvel = nullptr;
    int* d_img0 = nullptr;
    // control
    uint32_t* flags = nullptr;  // [0] rebuild request [1] error bits [2] builds [3] max count [4] ticket
    unsigned long long* d_ts = nullptr;
    uint64_t timestep = 0;
    // outputs
    double4_32a* out_force = nullptr;
    double* out_virial = nullptr;
    double* partials = nullptr;
    double* thermo = nullptr;
    double4_32a* tmp4 = nullptr;  // tag-order staging [N]
    double* tmpd = nullptr;       // tag-order staging [N * 6]
    uint64_t launches = 0;
    bool have_state = false;
    // out_force / out_virial hold the forces of the current state (written by a
    // forces-only launch or by the closing step of a Langevin run)
    bool forces_valid = false;
    // host-transfer staging of azp_md_set_state / azp_md_get_state (tag order,
    // allocated on the first host transfer and kept: no allocation per call)
    double* st_pos = nullptr;
    double* st_vel = nullptr;
    double* st_acc = nullptr;
    int* st_img = nullptr;
    double* st_diam = nullptr;
    // entry snapshot of azp_md_run_checked (tag order, allocated on first use)
    double* snap_pos = nullptr;
    double* snap_vel = nullptr;
    double* snap_acc = nullptr;
    int* snap_img = nullptr;
    double* snap_diam = nullptr;
    // graphs
    bool use_graphs = true;
    cudaGraphExec_t gexec[2] = {nullptr, nullptr};  // pair of mid steps starting at cur = 0 / 1
    cudaGraphExec_t gexec_rb[2] = {nullptr, nullptr};  // conditional rebuild alone, at cur = 0 / 1
    uint32_t graph_steps = 0;
    cudaStream_t graph_stream = nullptr;
};

namespace
{
template<typename T> int dalloc(T** p, size_t n)
{
    *p = nullptr;
    if (n == 0) n = 1;
    const cudaError_t e = cudaMalloc(reinterpret_cast<void**>(p), sizeof(T) * n);
    return e == cudaSuccess ? AZP_OK : record_cuda_error(e, "cudaMalloc (engine)");
}

void free_graphs(azp_md* m)
{
    for (auto& g : m->gexec)
        if (g) {
            cudaGraphExecDestroy(g);
            g = nullptr;
        }
    for (auto& g : m->gexec_rb)
        if (g) {
            cudaGraphExecDestroy(g);
            g = nullptr;
        }
    m->graph_steps = 0;
}

void free_all(azp_md* m)
{
    free_graphs(m);
    void* ptrs[] = {m->pos[0], m->pos[1], m->fix[0], m->fix[1], m->lo[0], m->lo[1], m->mass, m->t_mass, m->fix_build, m->vel, m->accel, m->image, m->tag,
                    m->rtag, m->diam, m->sort_gate, m->t_pos, m->t_vel, m->t_accel, m->t_image, m->t_tag, m->t_diam, m->t_cell,
                    m->cell_of, m->slot, m->cell_count, m->cell_start, m->members, m->scan_tmp, m->counts, m->nbrs,
                    m->cuts, m->bt_n_tag, m->bt_partner_tag, m->bt_type_tag, m->bt_n, m->bt, m->ex_n, m->ex_idx,
                    m->d_bond_params, m->d_pair_table, m->d_gamma, m->d_noise, m->flags, m->d_ts, m->out_force, m->out_virial,
                    m->partials, m->thermo, m->tmp4, m->tmpd, m->snap_pos, m->snap_vel, m->snap_acc,
                    m->snap_img, m->snap_diam, m->st_pos, m->st_vel, m->st_acc, m->st_img, m->st_diam,
                    m->d_bar_tab, m->d_bar_hdr, m->d_walls, m->d_wall_tab, m->d_dvel, m->d_img0,
                    m->d_kT_hdr, m->d_kT_tab, m->d_noise_tab, m->tile_tab, m->d_wall_f, m->d_contact_q};
    for (void* p : ptrs) cudaFree(p);
    if (m->h_thermo) cudaFreeHost(m->h_thermo);
    m->h_thermo = nullptr;
}

uint32_t blocks_for(uint32_t n, uint32_t b) { return (n + b - 1) / b; }

MDArgs base_args(azp_md* m)
{
    MDArgs a{};
    a.pos = m->pos[m->cur];
    a.pos_next = m->pos[m->cur ^ 1];
    a.fix = m->fix[m->cur];
    a.fix_next = m->fix[m->cur ^ 1];
    a.fix_build = m->fix_build;
    a.vel = m->vel;
    a.accel = m->accel;
    a.image = m->image;
    a.tag = m->tag;
    a.diameter = m->diam;
    a.N = m->N;
    a.ntypes = m->ntypes;
    for (int d = 0; d < 3; ++d) {
        a.L[d] = m->box.L[d];
        a.Linv[d] = 1.0 / m->box.L[d];
        a.lo[d] = -0.5 * m->box.L[d];
        a.hi[d] = 0.5 * m->box.L[d];
        a.sfix[d] = (float)(m->box.L[d] * 2.3283064365386963e-10);
        a.fscale[d] = a.Linv[d] * 4294967296.0;
    }
    a.cubic = (m->box.L[0] == m->box.L[1] && m->box.L[1] == m->box.L[2]) ? 1 : 0;
    {
        const double q = m->box.L[0] * 2.3283064365386963e-10;
        const double q2 = q * q;
        a.s2h = (float)q2;
        a.s2l = (float)(q2 - (double)a.s2h);
    }
    a.counts = m->counts;
    a.nbrs = m->nbrs;
    a.max_nn = m->max_nn;
    a.pair_table = m->d_pair_table;
    a.contact_q = m->d_contact_q;
    a.bt_n = m->bt_n;
    a.bt = m->bt;
    a.bond_params = m->d_bond_params;
    a.nbondtypes = m->nbt;
    a.dt = m->dt;
    a.kT = m->kT;
    a.d_timestep = m->d_ts;
    a.d_timestep_rw = m->d_ts;
    a.seed = m->seed;
    a.noiseless = m->noiseless;
    a.gamma = m->d_gamma;
    a.noise = m->d_noise;
    a.use_lambda = m->use_lambda;
    a.lambda = m->lambda;
    a.flow = m->flow;
    a.max_disp = m->max_disp;
    a.fcap = m->fcap;
    const double half = 0.5 * m->r_buff;
    a.disp_thresh2 = (float)(half * half * (1.0 - 1e-5));
    a.flags = m->flags;
    a.out_force = m->out_force;
    a.out_virial = m->out_virial;
    a.set_cond = 0;
    a.next = 0;
    a.out = 0;
    a.tpp = m->tpp;
    a.tpp_shift = 0;
    while ((1 << a.tpp_shift) < m->tpp) ++a.tpp_shift;
    a.flo = m->lo[m->cur];
    a.flo_next = m->lo[m->cur ^ 1];
    a.velf = reinterpret_cast<VelFF*>(m->vel);
    for (int d = 0; d < 3; ++d) {
        const double s64 = 4294967296.0 / m->box.L[d];
        a.s64h[d] = (float)s64;
        a.s64l[d] = (float)(s64 - (double)a.s64h[d]);
        a.l64[d] = m->box.L[d] * 5.421010862427522e-20;
    }
    a.dtf = (float)m->dt;
    a.kTf = (float)m->kT;
    a.lambdaf = (float)m->lambda;
    a.fcapf = (float)m->fcap;
    a.max_dispf = (float)m->max_disp;
    // single-type systems: type pair 0, bond type 0 and type 0 as kernel arguments
    a.one_type = (m->ntypes == 1 && m->nbt <= 1 && !m->use_lambda) ? 1 : 0;
    for (int k = 0; k < MD_PAIR_TBL; ++k)
        a.rec0[k] = m->pair_table_host.empty() ? 0.0f : (float)m->pair_table_host[k];
    a.rc2_0 = m->pair_table_host.empty() ? 0.0 : m->pair_table_host[PAIR_REC];
    for (int k = 0; k < MD_BOND_F; ++k) a.bond0[k] = 0.0f;
    if (m->bond_kind == AZP_BOND_QUARTIC && !m->bond_params.empty()) QuarticBond::prepare_f(m->bond_params.data(), a.bond0);
    if (m->bond_kind == AZP_BOND_DOUBLE_WELL && !m->bond_params.empty())
        DoubleWellBond::prepare_f(m->bond_params.data(), a.bond0);
    if (m->bond_kind == AZP_BOND_IMAGE_HARMONIC && !m->bond_params.empty())
        HarmonicBond::prepare_f(m->bond_params.data(), a.bond0);
    a.gamma0 = m->gamma.empty() ? 0.0f : (float)m->gamma[0];
    a.noise0 = m->noise_host.empty() ? 0.0f : (float)m->noise_host[0];
    a.bar_geom = m->bar_geom;
    a.bar_tab = m->d_bar_tab;
    a.bar_hdr = m->d_bar_hdr;
    a.wall_kind = m->wall_kind;
    a.walls = m->d_walls;
    a.wall_tab = m->d_wall_tab;
    a.wall_f = m->d_wall_f;
    a.wall_tol = m->wall_tol;
    a.dvel = m->d_dvel;
    a.img0 = m->d_img0;
    a.group_types = m->group_types;
    a.kT_hdr = m->d_kT_hdr;
    a.kT_tab = m->d_kT_tab;
    a.noise_tab = m->d_noise_tab;
    a.tile = m->tile_tab;
    a.flowf.kind = m->flow.kind;
    if (m->flow.kind == AZP_FLOW_PARABOLIC) {
        a.flowf.a = (float)m->flow.a;
        a.flowf.b = (float)(1.0 / m->flow.b);
        a.flowf.c = 0.0f;
    } else {
        a.flowf.a = (float)m->flow.a;
        a.flowf.b = (float)m->flow.b;
        a.flowf.c = (float)m->flow.c;
    }
    return a;
}

// the list rebuild, gated by flags[0] (gate) or unconditional (gate NULL), with the
// re-sort of the particles into cell order when due (or forced)
int enqueue_rebuild(azp_md* m, cudaStream_t s, const uint32_t* gate, bool force_sort)
{
    const uint32_t N = m->N;
    if (N == 0) return AZP_OK;
    const uint32_t nb = blocks_for(N, 256);
    k_zero_gated<<<std::min<uint32_t>(blocks_for(m->grid.ncell, 256), 1024), 256, 0, s>>>(m->cell_count, m->grid.ncell,
                                                                                          gate);
    const bool fx = m->precision == AZP_FP32;
    if (fx) launch_cell_assign_fx(m->fix[m->cur], N, m->grid, m->cell_of, m->slot, m->cell_count, s, gate);
    else launch_cell_assign(m->pos[m->cur], N, m->grid, m->cell_of, m->slot, m->cell_count, s, gate);
    int st = exclusive_scan(m->cell_count, m->cell_start, m->grid.ncell, m->scan_tmp, s, gate);
    if (st) return st;
    launch_cell_scatter(m->cell_of, m->slot, m->cell_start, m->members, N, m->grid.ncell, s, gate);
    // shared-memory tiles need the cell order at every build
    const bool sparse = (uint64_t)N <= 4ull * m->grid.ncell && m->grid.reach[0] <= 1 && m->grid.reach[1] <= 1 &&
                        m->grid.reach[2] <= 1;
    const uint32_t every = m->sort_every ? m->sort_every : (sparse ? 4u : 1u);
    const int force = force_sort || every <= 1 || m->tile_tab != nullptr;
    k_sort_decide<<<1, 1, 0, s>>>(gate, every, force, m->sort_gate);
    const uint32_t* g_sort = m->sort_gate;
    const uint32_t* g_keep = m->sort_gate + 2;
    PermArgs p;
    p.members = m->members;
    p.pos = fx ? nullptr : m->pos[m->cur];
    p.t_pos = m->t_pos;
    // FP32-force mode: the next-step buffers serve as temporaries (the step after
    // the rebuild overwrites them)
    p.fix = fx ? m->fix[m->cur] : nullptr;
    p.t_fix = fx ? m->fix[m->cur ^ 1] : nullptr;
    p.lo = fx ? m->lo[m->cur] : nullptr;
    p.t_lo = fx ? m->lo[m->cur ^ 1] : nullptr;
    p.mass = m->mass;
    p.t_mass = m->t_mass;
    p.fix_build = m->fix_build;
    p.vel = m->vel;
    p.t_vel = m->t_vel;
    p.accel = m->accel;
    p.t_accel = m->t_accel;
    p.image = m->image;
    p.t_image = m->t_image;
    p.tag = m->tag;
    p.t_tag = m->t_tag;
    p.rtag = m->rtag;
    p.diam = m->diam;
    p.t_diam = m->t_diam;
    p.cell_of = m->cell_of;
    p.t_cell = m->t_cell;
    p.N = N;
    // the re-sorting build: the particles' arrays and the bond table in cell order
    k_perm_gather<<<nb, 256, 0, s>>>(p, g_sort);
    k_perm_back<<<nb, 256, 0, s>>>(p, g_sort);
    if (m->bond_kind >= 0)
        k_bond_table<<<nb, 256, 0, s>>>(m->tag, m->rtag, m->bt_n_tag, m->bt_partner_tag, m->bt_type_tag, N, m->bt_n,
                                        m->bt, m->ex_n, m->ex_idx, m->exclude_bonds, g_sort);
    if (!fx) launch_to_fixed2(m->pos[m->cur], m->fix[m->cur], m->fix_build, N, m->box, s, gate);
    // the order-keeping build: the new reference positions (the re-sort writes
    // them in FP32-force mode, launch_to_fixed2 in FP64 mode)
    if (fx) k_copy_fix_build<<<nb, 256, 0, s>>>(m->fix[m->cur], m->fix_build, N, g_keep);
    if (m->tile_tab) launch_tile_table(m->cell_of, m->cell_start, m->grid, N, m->tile_tab, g_sort, s);
    if (m->pair_kind >= 0) {
        // particles in cell order: the scan reads the cells' slot ranges directly;
        // otherwise through the cell member table
        launch_nlist_build(fx ? nullptr : m->pos[m->cur], m->fix[m->cur], N, m->box, m->grid, m->cell_start, nullptr,
                           m->cell_of, m->cuts, m->ntypes, m->ex_n, m->ex_idx, m->bt_width, nullptr, m->counts, m->nbrs,
                           m->max_nn, m->flags + 3, g_sort, s, fx ? m->lo[m->cur] : nullptr, m->rlist_min,
                           m->tile_tab);
        if (!force)
            launch_nlist_build(fx ? nullptr : m->pos[m->cur], m->fix[m->cur], N, m->box, m->grid, m->cell_start,
                               m->members, m->cell_of, m->cuts, m->ntypes, m->ex_n, m->ex_idx, m->bt_width, nullptr,
                               m->counts, m->nbrs, m->max_nn, m->flags + 3, g_keep, s, fx ? m->lo[m->cur] : nullptr,
                               m->rlist_min, nullptr);
    }
    k_finish_rebuild<<<1, 1, 0, s>>>(m->flags, gate);
    AZP_CHECK_LAUNCH("enqueue_rebuild");
    m->launches += 12 + (m->bond_kind >= 0) + (m->pair_kind >= 0) * (force ? 1 : 2);
    return AZP_OK;
}

// the step kernel, preceded for DPD and ImageHarmonic bonds by the snapshot it reads
int md_launch(azp_md* m, int integ, const MDArgs& a, cudaStream_t s)
{
    if (m->d_wall_f) {
        k_walls_fx<<<blocks_for(m->N, 256), 256, 0, s>>>(a);
        AZP_CHECK_LAUNCH("k_walls_fx");
        m->launches += 1;
    }
    if (m->d_dvel || m->d_img0) {
        k_step_snapshot<<<blocks_for(m->N, 256), 256, 0, s>>>(m->vel, m->image, m->N, m->precision == AZP_FP32 ? 1 : 0,
                                                              m->d_dvel, m->d_img0);
        AZP_CHECK_LAUNCH("k_step_snapshot");
        m->launches += 1;
    }
    return launch_md_step(m->pair_kind, m->bond_kind, m->precision, integ, a, s);
}

int enqueue_step(azp_md* m, int integ, int next, int out, cudaStream_t s, int set_cond,
                 cudaGraphConditionalHandle h)
{
    MDArgs a = base_args(m);
    a.next = next;
    a.out = out;
    a.set_cond = set_cond;
    a.next_cond = h;
    const int st = md_launch(m, integ, a, s);
    m->launches += 1;
    return st;
}

int enqueue_step1(azp_md* m, cudaStream_t s)
{
    const double half = 0.5 * m->r_buff;
    if (m->precision == AZP_FP32) {
        const MDArgs a = base_args(m);
        k_md_step1_fx<<<blocks_for(m->N, 256), 256, 0, s>>>(
            m->fix[m->cur], m->lo[m->cur], m->fix_build, a.velf, m->accel, m->image, m->N, a.dtf,
            make_float3(a.s64h[0], a.s64h[1], a.s64h[2]), make_float3(a.s64l[0], a.s64l[1], a.s64l[2]),
            make_float3(a.sfix[0], a.sfix[1], a.sfix[2]), a.disp_thresh2, m->flags, a.group_types);
        AZP_CHECK_LAUNCH("k_md_step1_fx");
        m->launches += 1;
        return AZP_OK;
    }
    k_md_step1<<<blocks_for(m->N, 256), 256, 0, s>>>(
        m->pos[m->cur], m->fix[m->cur], m->fix_build, m->vel, m->accel, m->image, m->N, m->dt, m->box.L[0],
        m->box.L[1], m->box.L[2], 1.0 / m->box.L[0], 1.0 / m->box.L[1], 1.0 / m->box.L[2],
        (float)(m->box.L[0] * 2.3283064365386963e-10), (float)(m->box.L[1] * 2.3283064365386963e-10),
        (float)(m->box.L[2] * 2.3283064365386963e-10), (float)(half * half * (1.0 - 1e-5)), m->flags,
        m->group_types);
    AZP_CHECK_LAUNCH("k_md_step1");
    m->launches += 1;
    return AZP_OK;
}

// Build the executable graph of two mid steps starting at buffer parity cur0:
//   arm -> IF(rebuild) -> step(next) -> IF(rebuild) -> step(next)
// Each step kernel arms the following conditional from its last block.
int build_pair_graph(azp_md* m, int cur0, int integ, cudaGraphExec_t* out)
{
    cudaGraph_t g = nullptr;
    AZP_CUDA_TRY(cudaGraphCreate(&g, 0));
    cudaGraphConditionalHandle h[2];
    for (int k = 0; k < 2; ++k) AZP_CUDA_TRY(cudaGraphConditionalHandleCreate(&h[k], g, 0, cudaGraphCondAssignDefault));
    const int saved_cur = m->cur;
    const uint64_t saved_launches = m->launches;
    m->cur = cur0;
    cudaStream_t s = m->graph_stream;
    cudaGraphNode_t prev = nullptr;
    int st = AZP_OK;
    // arm node
    {
        AZP_CUDA_TRY(cudaStreamBeginCaptureToGraph(s, g, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
        k_arm<<<1, 1, 0, s>>>(m->flags, h[0]);
        cudaGraph_t gg = nullptr;
        AZP_CUDA_TRY(cudaStreamEndCapture(s, &gg));
        size_t n = 0;
        AZP_CUDA_TRY(cudaGraphGetNodes(g, nullptr, &n));
        std::vector<cudaGraphNode_t> nodes(n);
        AZP_CUDA_TRY(cudaGraphGetNodes(g, nodes.data(), &n));
        prev = nodes.back();
    }
    for (int k = 0; k < 2 && st == AZP_OK; ++k) {
        cudaGraphNodeParams cp = {};
        cp.type = cudaGraphNodeTypeConditional;
        cp.conditional.handle = h[k];
        cp.conditional.type = cudaGraphCondTypeIf;
        cp.conditional.size = 1;
        cudaGraphNode_t cnode;
        AZP_CUDA_TRY(cudaGraphAddNode(&cnode, g, &prev, nullptr, 1, &cp));
        cudaGraph_t body = cp.conditional.phGraph_out[0];
        AZP_CUDA_TRY(cudaStreamBeginCaptureToGraph(s, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
        st = enqueue_rebuild(m, s, nullptr, false);
        cudaGraph_t bb = nullptr;
        const cudaError_t e1 = cudaStreamEndCapture(s, &bb);
        if (st) break;
        if (e1 != cudaSuccess) {
            st = record_cuda_error(e1, "capture rebuild body");
            break;
        }
        // the step node, depending on the conditional
        AZP_CUDA_TRY(cudaStreamBeginCaptureToGraph(s, g, &cnode, nullptr, 1, cudaStreamCaptureModeThreadLocal));
        st = enqueue_step(m, integ, 1, 0, s, k == 0 ? 1 : 0, k == 0 ? h[1] : 0);
        cudaGraph_t sg = nullptr;
        const cudaError_t e2 = cudaStreamEndCapture(s, &sg);
        if (st) break;
        if (e2 != cudaSuccess) {
            st = record_cuda_error(e2, "capture step");
            break;
        }
        // the captured nodes form one chain after cnode (DPD: snapshot -> step);
        // the next conditional depends on its last node
        cudaGraphNode_t tail = cnode;
        for (int hop = 0; hop < 8; ++hop) {
            size_t nd = 0;
            AZP_CUDA_TRY(cudaGraphNodeGetDependentNodes(tail, nullptr, nullptr, &nd));
            if (nd == 0) break;
            if (nd != 1) {
                st = AZP_ERR_CUDA;
                break;
            }
            AZP_CUDA_TRY(cudaGraphNodeGetDependentNodes(tail, &tail, nullptr, &nd));
        }
        if (st) break;
        if (tail == cnode) {
            st = AZP_ERR_CUDA;
            break;
        }
        prev = tail;
        m->cur ^= 1;
    }
    m->cur = saved_cur;
    m->launches = saved_launches;
    if (st == AZP_OK) {
        const cudaError_t e = cudaGraphInstantiate(out, g, 0);
        if (e != cudaSuccess) st = record_cuda_error(e, "cudaGraphInstantiate");
    }
    cudaGraphDestroy(g);
    return st;
}

// The rebuild alone as a graph: the arm node and the conditional rebuild body,
// with the buffers of parity cur0
int build_rebuild_graph(azp_md* m, int cur0, cudaGraphExec_t* out)
{
    cudaGraph_t g = nullptr;
    AZP_CUDA_TRY(cudaGraphCreate(&g, 0));
    cudaGraphConditionalHandle h;
    int st = AZP_OK;
    const int saved_cur = m->cur;
    m->cur = cur0;
    cudaStream_t s = m->graph_stream;
    cudaGraphNode_t arm = nullptr;
    cudaError_t e = cudaGraphConditionalHandleCreate(&h, g, 0, cudaGraphCondAssignDefault);
    if (e == cudaSuccess) e = cudaStreamBeginCaptureToGraph(s, g, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal);
    if (e == cudaSuccess) {
        k_arm<<<1, 1, 0, s>>>(m->flags, h);
        cudaGraph_t gg = nullptr;
        e = cudaStreamEndCapture(s, &gg);
    }
    if (e == cudaSuccess) {
        size_t n = 1;
        e = cudaGraphGetNodes(g, &arm, &n);
    }
    if (e == cudaSuccess) {
        cudaGraphNodeParams cp = {};
        cp.type = cudaGraphNodeTypeConditional;
        cp.conditional.handle = h;
        cp.conditional.type = cudaGraphCondTypeIf;
        cp.conditional.size = 1;
        cudaGraphNode_t cnode;
        e = cudaGraphAddNode(&cnode, g, &arm, nullptr, 1, &cp);
        if (e == cudaSuccess)
            e = cudaStreamBeginCaptureToGraph(s, cp.conditional.phGraph_out[0], nullptr, nullptr, 0,
                                              cudaStreamCaptureModeThreadLocal);
        if (e == cudaSuccess) {
            st = enqueue_rebuild(m, s, nullptr, false);
            cudaGraph_t bb = nullptr;
            e = cudaStreamEndCapture(s, &bb);
        }
    }
    if (e == cudaSuccess && st == AZP_OK) e = cudaGraphInstantiate(out, g, 0);
    if (e != cudaSuccess && st == AZP_OK) st = record_cuda_error(e, "rebuild graph");
    m->cur = saved_cur;
    cudaGraphDestroy(g);
    return st;
}

// The list rebuild if a step or a loaded state requested it: with graphs, one
// replay of the rebuild graph (its arm kernel decides; a rebuild that is not
// needed costs that one kernel); without, the rebuild kernels gated by the flag.
int rebuild_if_requested(azp_md* m, cudaStream_t s)
{
    if (!m->use_graphs) return enqueue_rebuild(m, s, m->flags, false);
    cudaGraphExec_t& ge = m->gexec_rb[m->cur];
    if (!ge) {
        const int st = build_rebuild_graph(m, m->cur, &ge);
        if (st) return st;
    }
    AZP_CUDA_TRY(cudaGraphLaunch(ge, s));
    m->launches += 1;
    return AZP_OK;
}

// the status the engine's eight flag words carry
int errors_from_flags(const azp_md* m, const uint32_t* f)
{
    if (f[3] > m->max_nn) return AZP_ERR_NLIST_OVERFLOW;
    if (f[1] & AZP_EBIT_BOND) return AZP_ERR_BOND;
    if (f[1] & AZP_EBIT_NONFINITE) return AZP_ERR_NONFINITE;
    return AZP_OK;
}

int check_errors(azp_md* m, cudaStream_t s)
{
    uint32_t f[8];
    AZP_CUDA_TRY(cudaMemcpyAsync(f, m->flags, sizeof(f), cudaMemcpyDeviceToHost, s));
    AZP_CUDA_TRY(cudaStreamSynchronize(s));
    return errors_from_flags(m, f);
}

// The device address of a host buffer the GPU can read and write in place:
// pinned memory mapped into the unified address space (cudaHostAlloc,
// cudaHostRegister, torch's pin_memory). On GB300 such a buffer is reached over
// NVLink-C2C, so the state kernels move it without a staging copy. Null for
// pageable memory (staged instead) or when AZP_ZERO_COPY=0.
void* mapped_view(const void* h)
{
    if (!h) return nullptr;
    static const bool off = [] {
        const char* e = std::getenv("AZP_ZERO_COPY");
        return e && e[0] == '0';
    }();
    if (off) return nullptr;
    cudaPointerAttributes at{};
    if (cudaPointerGetAttributes(&at, h) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    return (at.type == cudaMemoryTypeHost && at.devicePointer) ? at.devicePointer : nullptr;
}

// the state kernels move positions and velocities as 16-byte pairs
bool aligned16(const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15u) == 0u; }
// rows of three per particle (accelerations, image counts) move as 16-byte vectors
int rows_aligned(const void* accel, const void* image) { return aligned16(accel) && aligned16(image); }

// staging buffers of the host transfers (first use only)
int ensure_staging(azp_md* m)
{
    if (m->st_pos) return AZP_OK;
    const size_t N = m->N;
    int st = dalloc(&m->st_pos, 4 * N);
    if (!st) st = dalloc(&m->st_vel, 4 * N);
    if (!st) st = dalloc(&m->st_acc, 3 * N);
    if (!st) st = dalloc(&m->st_img, 3 * N);
    if (!st) st = dalloc(&m->st_diam, N);
    return st;
}

// device state -> tag-order FP64 arrays (either precision's state layout)
void enqueue_store_state(azp_md* m, double* pos, double* vel, double* accel, int* image, cudaStream_t s)
{
    const uint32_t N = m->N;
    if (m->precision == AZP_FP32)
        k_store_state_fx<<<blocks_for(N, STATE_BLOCK), STATE_BLOCK, 0, s>>>(
            m->fix[m->cur], m->lo[m->cur], reinterpret_cast<const VelFF*>(m->vel), m->mass, m->accel, m->image, m->rtag,
            N, m->box.L[0] * 5.421010862427522e-20, m->box.L[1] * 5.421010862427522e-20,
            m->box.L[2] * 5.421010862427522e-20, pos, vel, accel, image, rows_aligned(accel, image));
    else
        k_store_state<<<blocks_for(N, STATE_BLOCK), STATE_BLOCK, 0, s>>>(
            m->pos[m->cur], m->vel, m->accel, m->image, m->rtag, N, pos, vel, accel, image, rows_aligned(accel, image));
}


int size_list(azp_md* m, cudaStream_t s)
{
    // first build: measure the largest neighbour count and size the list
    if (m->pair_kind < 0) return AZP_OK;
    for (int attempt = 0; attempt < 4; ++attempt) {
        AZP_CUDA_TRY(cudaMemsetAsync(m->flags + 3, 0, sizeof(uint32_t), s));
        const uint32_t one = 1u;
        AZP_CUDA_TRY(cudaMemcpyAsync(m->flags, &one, sizeof(uint32_t), cudaMemcpyHostToDevice, s));
        int st = enqueue_rebuild(m, s, nullptr, true);
        if (st) return st;
        uint32_t need = 0;
        AZP_CUDA_TRY(cudaMemcpyAsync(&need, m->flags + 3, sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
        AZP_CUDA_TRY(cudaStreamSynchronize(s));
        if (need <= m->max_nn) return AZP_OK;
        // headroom for density fluctuations between builds
        cudaFree(m->nbrs);
        m->nbrs = nullptr;
        m->max_nn = (uint32_t)std::ceil(need * 1.5) + 16;
        st = dalloc(&m->nbrs, (size_t)m->N * m->max_nn);
        if (st) return st;
        free_graphs(m);
    }
    return AZP_ERR_NLIST_OVERFLOW;
}

}  // namespace

extern "C" {

azp_md* azp_md_create(const azp_md_config* c, int* status)
{
    auto fail = [&](int st, azp_md* m) -> azp_md* {
        if (status) *status = st;
        if (m) {
            free_all(m);
            delete m;
        }
        return nullptr;
    };
    // particle indices below 2^31: neighbour-list entries carry marks in bit 31
    if (!c || c->ntypes == 0 || c->ntypes > MAX_PAIR_TYPES || c->N >= 0x80000000u) return fail(AZP_ERR_INVALID, nullptr);
    for (int d = 0; d < 3; ++d)
        if (!(c->box.L[d] > 0.0)) return fail(AZP_ERR_INVALID, nullptr);
    if (c->precision != AZP_FP64 && c->precision != AZP_FP32) return fail(AZP_ERR_INVALID, nullptr);
    if (c->method != AZP_METHOD_LANGEVIN_FLOW && c->method != AZP_METHOD_BROWNIAN_FLOW)
        return fail(AZP_ERR_INVALID, nullptr);
    if ((c->pair_kind >= AZP_PAIR_NUM_KINDS && c->pair_kind != AZP_PAIR_DPD_GENERAL_WEIGHT) ||
        (c->bond_kind >= AZP_BOND_NUM_KINDS && c->bond_kind != AZP_BOND_IMAGE_HARMONIC))
        return fail(AZP_ERR_INVALID, nullptr);
    // the DPD thermostat acts on velocities: Langevin-type methods only (the
    // noiseless, drag-free Langevin step is HOOMD's ConstantVolume)
    if (c->pair_kind == AZP_PAIR_DPD_GENERAL_WEIGHT &&
        (c->method != AZP_METHOD_LANGEVIN_FLOW || !(c->dpd_kT >= 0.0) || c->shift_mode != AZP_MODE_NONE))
        return fail(record_error(AZP_ERR_UNSUPPORTED, "azp_md_create: DPD needs a Langevin-type method, kT >= 0 "
                                                      "and mode none"),
                    nullptr);
    if (!(c->dt > 0.0)) return fail(AZP_ERR_INVALID, nullptr);
    if (!c->use_lambda && !c->gamma) return fail(AZP_ERR_INVALID, nullptr);
    azp_md* m = new (std::nothrow) azp_md();
    if (!m) return fail(AZP_ERR_INVALID, nullptr);
    m->N = c->N;
    m->ntypes = c->ntypes;
    m->box = c->box;
    m->precision = c->precision;
    m->pair_kind = c->pair_kind < 0 ? -1 : c->pair_kind;
    m->shift_mode = c->shift_mode;
    m->bond_kind = (c->bond_kind < 0 || c->nbonds == 0) ? -1 : c->bond_kind;
    m->method = c->method;
    m->exclude_bonds = c->exclude_bonds;
    m->r_buff = c->r_buff;
    m->dt = c->dt;
    m->kT = c->kT;
    if (c->group_types != 0u) {
        if (c->ntypes > 32u) return fail(AZP_ERR_INVALID, m);
        m->group_types = c->group_types;
    }
    m->seed = c->seed;
    m->noiseless = c->noiseless;
    m->use_lambda = c->use_lambda;
    m->lambda = c->lambda;
    m->flow = make_flow(c->flow);
    m->max_disp = c->max_displacement;
    m->fcap = c->pair_force_cap > 0.0 ? c->pair_force_cap : 0.0;
    const uint32_t nt2 = c->ntypes * c->ntypes;
    if (m->pair_kind >= 0) {
        if (!c->pair_params || !c->r_cut) return fail(AZP_ERR_INVALID, m);
        // the caller's table, in the reference layout (pair_record_doubles per record)
        m->pair_params.assign(c->pair_params, c->pair_params + (size_t)nt2 * pair_record_doubles(m->pair_kind));
        m->r_cut.assign(c->r_cut, c->r_cut + nt2);
        if (c->r_on) m->r_on.assign(c->r_on, c->r_on + nt2);
        else m->r_on.assign(nt2, 0.0);
        // same per-type-pair r_cut in both directions
        for (uint32_t a = 0; a < c->ntypes; ++a)
            for (uint32_t b = 0; b < c->ntypes; ++b)
                if (m->r_cut[a * c->ntypes + b] != m->r_cut[b * c->ntypes + a]) return fail(AZP_ERR_INVALID, m);
    }
    if (!c->use_lambda) m->gamma.assign(c->gamma, c->gamma + c->ntypes);
    else m->gamma.assign(c->ntypes, 0.0);
    const char* env_tpp = std::getenv("AZP_TPP");
    m->tpp = env_tpp ? std::atoi(env_tpp) : 1;
    if (!(m->tpp == 1 || m->tpp == 2 || m->tpp == 4 || m->tpp == 8 || m->tpp == 16 || m->tpp == 32)) m->tpp = 1;
    const char* env_graph = std::getenv("AZP_GRAPHS");
    m->use_graphs = !(env_graph && env_graph[0] == '0');
    const char* env_sort = std::getenv("AZP_SORT_EVERY");
    if (env_sort) m->sort_every = (uint32_t)std::max(1, std::min(std::atoi(env_sort), 1 << 20));

    const uint32_t N = c->N;
    int st = AZP_OK;
#define CTRY(call)                                                  \
    do {                                                            \
        const cudaError_t e_ = (call);                              \
        if (e_ != cudaSuccess) return fail(record_cuda_error(e_, #call), m); \
    } while (0)
#define ALLOC(p, n) \
    do {            \
        st = dalloc(&(p), (n)); \
        if (st) return fail(st, m); \
    } while (0)
    ALLOC(m->pos[0], N);
    ALLOC(m->pos[1], N);
    ALLOC(m->fix[0], N);
    ALLOC(m->fix[1], N);
    ALLOC(m->fix_build, N);
    if (c->precision == AZP_FP32) {
        ALLOC(m->lo[0], N);
        ALLOC(m->lo[1], N);
        ALLOC(m->mass, N);
        ALLOC(m->t_mass, N);
    }
    ALLOC(m->vel, N);
    ALLOC(m->accel, (size_t)3 * N);
    ALLOC(m->image, (size_t)3 * N);
    ALLOC(m->tag, N);
    ALLOC(m->rtag, N);
    if (c->use_lambda) {
        ALLOC(m->diam, N);
        ALLOC(m->t_diam, N);
    }
    ALLOC(m->t_pos, N);
    ALLOC(m->t_vel, N);
    ALLOC(m->t_accel, (size_t)3 * N);
    ALLOC(m->t_image, (size_t)3 * N);
    ALLOC(m->t_tag, N);
    ALLOC(m->t_cell, N);
    ALLOC(m->cell_of, N);
    ALLOC(m->slot, N);
    ALLOC(m->members, N);
    ALLOC(m->counts, N);
    ALLOC(m->flags, 8);
    ALLOC(m->sort_gate, 8);
    CTRY(cudaMemset(m->sort_gate, 0, sizeof(uint32_t) * 8));
    ALLOC(m->d_ts, 1);
    ALLOC(m->out_force, N);
    ALLOC(m->out_virial, (size_t)6 * N);
    ALLOC(m->tmp4, N);
    ALLOC(m->tmpd, (size_t)6 * N);
    ALLOC(m->partials, (size_t)8 * (blocks_for(N, THERMO_BLOCK) + 1));
    ALLOC(m->thermo, 12);
    CTRY(cudaMallocHost(&m->h_thermo, sizeof(double) * 12));
    ALLOC(m->d_gamma, c->ntypes);
    ALLOC(m->d_noise, c->ntypes);
    if (c->pair_kind == AZP_PAIR_DPD_GENERAL_WEIGHT) ALLOC(m->d_dvel, (size_t)4 * N);
    if (m->bond_kind == AZP_BOND_IMAGE_HARMONIC) ALLOC(m->d_img0, (size_t)3 * N);
    CTRY(cudaMemset(m->flags, 0, sizeof(uint32_t) * 8));
    CTRY(cudaMemcpy(m->d_gamma, m->gamma.data(), sizeof(double) * c->ntypes, cudaMemcpyHostToDevice));
    {
        // noise amplitude per type, with the operations of the reference's
        // per-particle expression (src/TwoStepLangevinFlow.h:213-215)
        std::vector<double> noise(c->ntypes, 0.0);
        if (!c->noiseless)
            for (uint32_t t = 0; t < c->ntypes; ++t) noise[t] = std::sqrt(6.0 * m->gamma[t] * c->kT / c->dt);
        CTRY(cudaMemcpy(m->d_noise, noise.data(), sizeof(double) * c->ntypes, cudaMemcpyHostToDevice));
        m->noise_host = noise;
    }
    // pair table + list thresholds + cell grid
    if (m->pair_kind >= 0) {
        std::vector<double> table((size_t)nt2 * PAIR_TBL, 0.0);
        if (m->pair_kind == AZP_PAIR_DPD_GENERAL_WEIGHT) {
            // DpdEngine record: 1/r_cut, r_cut, A, gamma, s/2, sqrt(6 kT gamma / dt);
            // cut record: r_cut^2 (src/DPDPairEvaluatorGeneralWeight.h:165-255)
            m->dpd_kT = c->dpd_kT;
            for (uint32_t t = 0; t < nt2; ++t) {
                double* rec = &table[(size_t)t * PAIR_TBL];
                const double* p = &m->pair_params[(size_t)t * pair_record_doubles(AZP_PAIR_DPD_GENERAL_WEIGHT)];
                const double rc = m->r_cut[t];
                if (rc > 0.0) {
                    const double rcinv = 1.0 / std::sqrt(rc * rc);
                    rec[0] = rcinv;
                    rec[1] = 1.0 / rcinv;
                    rec[2] = p[0];
                    rec[3] = p[1];
                    rec[4] = 0.5 * p[2];
                    rec[5] = std::sqrt(6.0 * c->dpd_kT * p[1] / c->dt);
                    rec[PAIR_REC] = rc * rc;
                }
            }
        } else {
            st = build_pair_table(m->pair_kind, m->pair_params.data(), m->r_cut.data(), m->r_on.data(), m->shift_mode,
                                  c->ntypes, table.data());
            if (st) return fail(st, m);
        }
        ALLOC(m->d_pair_table, table.size());
        CTRY(cudaMemcpy(m->d_pair_table, table.data(), sizeof(double) * table.size(), cudaMemcpyHostToDevice));
        const bool dpd = c->pair_kind == AZP_PAIR_DPD_GENERAL_WEIGHT;
        if ((c->pair_kind == AZP_PAIR_COLLOID || dpd) && c->box.L[0] == c->box.L[1] && c->box.L[1] == c->box.L[2]) {
            // squared distances in the units of the integer r^2 of the FP32-force
            // step, (2^32 / L)^2: the colloid contact distances, the DPD cutoffs
            const double u = 4294967296.0 / c->box.L[0];
            std::vector<long long> cq(nt2, 0);
            bool fits = true;  // inside the half box: below 2^62 in these units
            for (size_t t = 0; t < nt2; ++t) {
                const double* rec = table.data() + t * PAIR_TBL;
                if (!dpd && !Colloid::gap_form(rec)) continue;
                const double c2 = dpd ? m->r_cut[t] * m->r_cut[t] : Colloid::contact2(rec);
                if (!(c2 < 0.25 * c->box.L[0] * c->box.L[0])) fits = false;
                else cq[t] = std::llround(c2 * u * u);
            }
            if (fits) {
                ALLOC(m->d_contact_q, nt2);
                CTRY(cudaMemcpy(m->d_contact_q, cq.data(), sizeof(long long) * nt2, cudaMemcpyHostToDevice));
            }
        }
        m->pair_table_host = table;
        std::vector<ListCut> cuts(nt2);
        make_list_cuts(m->r_cut.data(), c->ntypes, m->r_buff, m->box, cuts.data(), &m->rlist_max, &m->rlist_min);
        for (int d = 0; d < 3; ++d)
            if (m->rlist_max > 0.0 && m->box.L[d] < 2.0 * m->rlist_max) return fail(AZP_ERR_BOX_TOO_SMALL, m);
        ALLOC(m->cuts, nt2);
        CTRY(cudaMemcpy(m->cuts, cuts.data(), sizeof(ListCut) * nt2, cudaMemcpyHostToDevice));
        m->max_nn = 32;
        ALLOC(m->nbrs, (size_t)N * m->max_nn);
        // AZP_TILES=1: the single-type FP32-force step reads its neighbours from
        // shared-memory tiles instead of gathering them (bit-identical results;
        // measured slower on the bead-spring melt, so off by default)
        const char* env_tiles = std::getenv("AZP_TILES");
        const bool one = c->ntypes == 1 && (c->bond_kind < 0 || c->nbondtypes <= 1) && !c->use_lambda;
        if (c->precision == AZP_FP32 && one && m->tpp == 1 && m->pair_kind != AZP_PAIR_DPD_GENERAL_WEIGHT &&
            m->bond_kind != AZP_BOND_IMAGE_HARMONIC && env_tiles && env_tiles[0] == '1' &&
            grid_subdivision(m->rlist_max, m->rlist_min) == 1)
            ALLOC(m->tile_tab, (size_t)((N + TILE_P - 1) / TILE_P) * TILE_REC);
    }
    m->grid = make_grid(m->box, m->rlist_max > 0.0 ? m->rlist_max : std::max(m->box.L[0], 1.0),
                        grid_subdivision(m->rlist_max, m->rlist_min));
    ALLOC(m->cell_count, m->grid.ncell);
    ALLOC(m->cell_start, (size_t)m->grid.ncell + 1);
    ALLOC(m->scan_tmp, scan_tmp_words(m->grid.ncell));
    // bonds: tag-order master table
    if (m->bond_kind >= 0) {
        if (!c->bonds || !c->bond_types || !c->bond_params || c->nbondtypes == 0 ||
            c->nbondtypes > MD_MAX_BOND_TYPES)
            return fail(AZP_ERR_INVALID, m);
        m->nbt = c->nbondtypes;
        // the caller's records (bond_record_doubles each) zero-padded to 8 values
        m->bond_params.assign((size_t)c->nbondtypes * AZP_BOND_PARAM_DOUBLES, 0.0);
        for (uint32_t t = 0; t < c->nbondtypes; ++t)
            for (int k = 0; k < bond_record_doubles(m->bond_kind); ++k)
                m->bond_params[(size_t)t * AZP_BOND_PARAM_DOUBLES + k] =
                    c->bond_params[(size_t)t * bond_record_doubles(m->bond_kind) + k];
        std::vector<uint32_t> n(N, 0);
        for (uint32_t b = 0; b < c->nbonds; ++b) {
            const uint32_t x = c->bonds[2 * b], y = c->bonds[2 * b + 1];
            if (x >= N || y >= N || x == y || c->bond_types[b] >= c->nbondtypes) return fail(AZP_ERR_INVALID, m);
            n[x]++;
            n[y]++;
        }
        uint32_t w = 0;
        for (uint32_t i = 0; i < N; ++i) w = std::max(w, n[i]);
        m->bt_width = w;
        std::vector<uint32_t> partner((size_t)w * N, 0), btype((size_t)w * N, 0), fill(N, 0);
        for (uint32_t b = 0; b < c->nbonds; ++b) {
            const uint32_t x = c->bonds[2 * b], y = c->bonds[2 * b + 1], t = c->bond_types[b];
            partner[(size_t)fill[x] * N + x] = y;
            btype[(size_t)fill[x] * N + x] = t;
            fill[x]++;
            partner[(size_t)fill[y] * N + y] = x;
            btype[(size_t)fill[y] * N + y] = t;
            fill[y]++;
        }
        ALLOC(m->bt_n_tag, N);
        ALLOC(m->bt_partner_tag, (size_t)w * N);
        ALLOC(m->bt_type_tag, (size_t)w * N);
        ALLOC(m->bt_n, N);
        ALLOC(m->bt, (size_t)w * N);
        ALLOC(m->d_bond_params, m->bond_params.size());
        if (m->exclude_bonds) {
            ALLOC(m->ex_n, N);
            ALLOC(m->ex_idx, (size_t)w * N);
        }
        CTRY(cudaMemcpy(m->bt_n_tag, n.data(), sizeof(uint32_t) * N, cudaMemcpyHostToDevice));
        CTRY(cudaMemcpy(m->bt_partner_tag, partner.data(), sizeof(uint32_t) * partner.size(),
                                cudaMemcpyHostToDevice));
        CTRY(cudaMemcpy(m->bt_type_tag, btype.data(), sizeof(uint32_t) * btype.size(), cudaMemcpyHostToDevice));
        CTRY(cudaMemcpy(m->d_bond_params, m->bond_params.data(), sizeof(double) * m->bond_params.size(),
                                cudaMemcpyHostToDevice));
    }
    // harmonic barrier: the table of a run's locations is filled by
    // azp_md_set_barrier_locations before the first run
    if (c->barrier_params) {
        if (c->barrier_geometry != AZP_BARRIER_PLANAR && c->barrier_geometry != AZP_BARRIER_SPHERICAL)
            return fail(AZP_ERR_INVALID, m);
        m->bar_geom = c->barrier_geometry;
        m->bar_params.assign(c->barrier_params, c->barrier_params + 2 * (size_t)c->ntypes);
        ALLOC(m->d_bar_tab, (size_t)2 * AZP_MD_BARRIER_ROWS * c->ntypes);
        ALLOC(m->d_bar_hdr, 2);
    }
    // wall potential: the wall field and per-type rows (record, r_cut^2,
    // r_extrap, screening reach) in device memory
    if (c->walls) {
        if (c->wall_kind != AZP_WALL_LJ93 && c->wall_kind != AZP_WALL_COLLOID) return fail(AZP_ERR_INVALID, m);
        if (!c->wall_params || !c->wall_r_cut || !c->wall_r_extrap) return fail(AZP_ERR_INVALID, m);
        WallField wf;
        st = make_wall_field(c->walls, &wf);
        if (st) return fail(st, m);
        std::vector<double> tab((size_t)WALL_TAB * c->ntypes, 0.0);
        for (uint32_t t = 0; t < c->ntypes; ++t) {
            const int wd = wall_record_doubles(c->wall_kind);
            for (int k = 0; k < wd; ++k) tab[WALL_TAB * t + k] = c->wall_params[(size_t)wd * t + k];
            const double rc = c->wall_r_cut[t], rx = c->wall_r_extrap[t];
            if (!(rc >= 0.0) || !(rx >= 0.0)) return fail(AZP_ERR_INVALID, m);
            tab[WALL_TAB * t + 4] = rc * rc;
            tab[WALL_TAB * t + 5] = rx;
            tab[WALL_TAB * t + 6] = std::max(rc, rx);
        }
        ALLOC(m->d_walls, 1);
        ALLOC(m->d_wall_tab, tab.size());
        CTRY(cudaMemcpy(m->d_walls, &wf, sizeof(wf), cudaMemcpyHostToDevice));
        CTRY(cudaMemcpy(m->d_wall_tab, tab.data(), sizeof(double) * tab.size(), cudaMemcpyHostToDevice));
        m->wall_kind = c->wall_kind;
        if (m->precision == AZP_FP32) ALLOC(m->d_wall_f, N);
        // the FP32 screen's positions are good to a few L 2^-24 (hi word, float
        // scale); the float distances to the walls to 64 units of 2^-24 of
        // |x|_1 (at most |L|_1 / 2) + the walls' extent + the reach
        double reach_max = 0.0;
        for (uint32_t t = 0; t < c->ntypes; ++t) reach_max = std::max(reach_max, tab[WALL_TAB * t + 6]);
        const double Lmax = std::max(m->box.L[0], std::max(m->box.L[1], m->box.L[2]));
        const double L1 = m->box.L[0] + m->box.L[1] + m->box.L[2];
        m->wall_tol = (float)std::max(4e-6 * Lmax + 1e-5,
                                      0x1p-18 * (0.5 * L1 + (double)wall_field_extent(wf) + reach_max) + 1e-5);
    }
    CTRY(cudaStreamCreateWithFlags(&m->graph_stream, cudaStreamNonBlocking));
#undef ALLOC
#undef CTRY
    if (status) *status = AZP_OK;
    return m;
}

void azp_md_destroy(azp_md* m)
{
    if (!m) return;
    free_all(m);
    if (m->graph_stream) cudaStreamDestroy(m->graph_stream);
    delete m;
}

int azp_md_set_state(azp_md* m, const double* pos, const double* vel, const double* accel, const int32_t* image,
                     const double* diameter, uint64_t timestep, int on_device, void* stream)
{
    if (!m || !pos || !vel) return AZP_ERR_INVALID;
    cudaStream_t s = as_stream(stream);
    const uint32_t N = m->N;
    if (N == 0) return AZP_OK;
    const double *dp = pos, *dv = vel, *da = accel, *dd = diameter;
    const int* di = image;
    if (!on_device) {
        int st0 = ensure_staging(m);
        if (st0) return st0;
        // pinned buffers are read in place by the load kernels; pageable ones staged
        auto up = [&](const void* h, void* d, size_t bytes) -> const void* {
            if (!h) return nullptr;
            if (aligned16(h))
                if (void* v = mapped_view(h)) return v;
            cudaMemcpyAsync(d, h, bytes, cudaMemcpyHostToDevice, s);
            return d;
        };
        dp = (const double*)up(pos, m->st_pos, sizeof(double) * 4 * N);
        dv = (const double*)up(vel, m->st_vel, sizeof(double) * 4 * N);
        da = (const double*)up(accel, m->st_acc, sizeof(double) * 3 * N);
        di = (const int*)up(image, m->st_img, sizeof(int) * 3 * N);
        dd = (const double*)up(diameter, m->st_diam, sizeof(double) * N);
        AZP_CHECK_LAUNCH("azp_md_set_state (host to device)");
    } else if (!aligned16(pos) || !aligned16(vel)) {
        // device inputs not on a 16-byte boundary: aligned copies first
        int st0 = ensure_staging(m);
        if (st0) return st0;
        AZP_CUDA_TRY(cudaMemcpyAsync(m->st_pos, pos, sizeof(double) * 4 * N, cudaMemcpyDeviceToDevice, s));
        AZP_CUDA_TRY(cudaMemcpyAsync(m->st_vel, vel, sizeof(double) * 4 * N, cudaMemcpyDeviceToDevice, s));
        dp = m->st_pos;
        dv = m->st_vel;
    }
    m->cur = 0;
    m->forces_valid = false;
    m->timestep = timestep;
    const unsigned long long ts = timestep;
    AZP_CUDA_TRY(cudaMemcpyAsync(m->d_ts, &ts, sizeof(ts), cudaMemcpyHostToDevice, s));
    AZP_CUDA_TRY(cudaMemsetAsync(m->flags, 0, sizeof(uint32_t) * 8, s));
    int st = AZP_OK;
    bool placed = false;
    uint32_t flags_seen[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    if (m->have_state) {
        // Keep the current particle order and list: load the new state in index
        // order and rebuild only if some particle lies more than r_buff / 2 from
        // its position at the last build (a state read back from this engine and
        // set again moves nothing). A denser new state that overflows the list
        // takes the full path below.
        const MDArgs a = base_args(m);
        if (m->precision == AZP_FP32) {
            k_load_state_ordered_fx<<<blocks_for(N, STATE_BLOCK), STATE_BLOCK, 0, s>>>(
                dp, dv, da, di, dd, m->rtag, N, 1.0 / m->box.L[0], 1.0 / m->box.L[1], 1.0 / m->box.L[2], m->fix[0],
                m->lo[0], reinterpret_cast<VelFF*>(m->vel), m->mass, m->accel, m->image, m->diam, m->fix_build,
                a.sfix[0], a.sfix[1], a.sfix[2], a.disp_thresh2, m->flags, rows_aligned(da, di));
            AZP_CHECK_LAUNCH("k_load_state_ordered_fx");
        } else {
            k_load_state_ordered<<<blocks_for(N, STATE_BLOCK), STATE_BLOCK, 0, s>>>(
                dp, dv, da, di, dd, m->rtag, N, m->pos[0], m->vel, m->accel, m->image, m->diam, rows_aligned(da, di));
            AZP_CHECK_LAUNCH("k_load_state_ordered");
            launch_to_fixed(m->pos[0], m->fix[0], N, m->box, s);
            k_request_if_displaced<<<blocks_for(N, 256), 256, 0, s>>>(m->fix[0], m->fix_build, N, a.sfix[0],
                                                                       a.sfix[1], a.sfix[2], a.disp_thresh2, m->flags);
            AZP_CHECK_LAUNCH("k_request_if_displaced");
        }
        st = rebuild_if_requested(m, s);
        if (st) return st;
        AZP_CUDA_TRY(cudaMemcpyAsync(flags_seen, m->flags, sizeof(flags_seen), cudaMemcpyDeviceToHost, s));
        AZP_CUDA_TRY(cudaStreamSynchronize(s));
        placed = flags_seen[3] <= m->max_nn;
        if (!placed) AZP_CUDA_TRY(cudaMemsetAsync(m->flags, 0, sizeof(uint32_t) * 8, s));
    }
    if (!placed) {
        k_load_state<<<blocks_for(N, STATE_BLOCK), STATE_BLOCK, 0, s>>>(
            dp, dv, da, di, dd, N, m->pos[0], m->vel, m->accel, m->image, m->diam, m->tag, m->rtag, rows_aligned(da, di));
        AZP_CHECK_LAUNCH("k_load_state");
        if (m->precision == AZP_FP32) {
            k_state_to_fx<<<blocks_for(N, 256), 256, 0, s>>>(m->pos[0], m->vel, m->fix[0], m->lo[0], m->mass, N,
                                                              1.0 / m->box.L[0], 1.0 / m->box.L[1], 1.0 / m->box.L[2]);
            AZP_CHECK_LAUNCH("k_state_to_fx");
        }
        st = size_list(m, s);  // unconditional rebuild (sorts the particles)
        if (st == AZP_OK && m->pair_kind < 0) {
            const uint32_t one = 1u;
            AZP_CUDA_TRY(cudaMemcpyAsync(m->flags, &one, sizeof(uint32_t), cudaMemcpyHostToDevice, s));
            st = enqueue_rebuild(m, s, nullptr, true);
        }
        if (st) return st;
    }
    const bool forces = !accel && m->method == AZP_METHOD_LANGEVIN_FLOW;
    if (forces) {
        // HOOMD starts a run from a = F / m when no acceleration is known
        MDArgs a = base_args(m);
        a.out = 1;
        st = md_launch(m, MD_FORCES_ONLY, a, s);
        if (st) return st;
        k_accel_from_force<<<blocks_for(N, 256), 256, 0, s>>>(m->out_force, m->vel, m->mass, m->accel, N);
        AZP_CHECK_LAUNCH("k_accel_from_force");
        m->forces_valid = true;
    }
    m->have_state = true;
    // an order-keeping load that enqueued nothing after its flag read has its status
    if (placed && !forces) return errors_from_flags(m, flags_seen);
    return check_errors(m, s);
}

int azp_md_get_state(azp_md* m, double* pos, double* vel, double* accel, int32_t* image, uint64_t* timestep,
                     int on_device, void* stream)
{
    if (!m || !m->have_state) return AZP_ERR_INVALID;
    cudaStream_t s = as_stream(stream);
    const uint32_t N = m->N;
    // the timestep is read after the state is enqueued, so that one wait covers both
    auto read_timestep = [&]() -> int {
        if (!timestep) return AZP_OK;
        unsigned long long ts = 0;
        AZP_CUDA_TRY(cudaMemcpyAsync(&ts, m->d_ts, sizeof(ts), cudaMemcpyDeviceToHost, s));
        AZP_CUDA_TRY(cudaStreamSynchronize(s));
        *timestep = ts;
        return AZP_OK;
    };
    if (N == 0) return read_timestep();
    if (on_device && aligned16(pos) && aligned16(vel)) {
        enqueue_store_state(m, pos, vel, accel, image, s);
        AZP_CHECK_LAUNCH("k_store_state");
        return read_timestep();
    }
    if (!on_device) {
        // Pinned outputs mapped into the device's address space are written in
        // place by the store kernel, whole 128-byte lines per warp access; the
        // others are staged on the device and copied by the copy engines.
        auto view = [](void* h, bool vec) -> void* {
            void* v = h ? mapped_view(h) : nullptr;
            return v && (!vec || aligned16(v)) ? v : nullptr;
        };
        double* hp = (double*)view(pos, true);
        double* hv = (double*)view(vel, true);
        double* ha = (double*)view(accel, false);
        int* hi = (int*)view(image, false);
        if ((!pos || hp) && (!vel || hv) && (!accel || ha) && (!image || hi)) {
            enqueue_store_state(m, hp, hv, ha, hi, s);
            AZP_CHECK_LAUNCH("k_store_state");
            const int st = read_timestep();
            if (st) return st;
            AZP_CUDA_TRY(cudaStreamSynchronize(s));
            return AZP_OK;
        }
    }
    const cudaMemcpyKind back = on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
    int st0 = ensure_staging(m);
    if (st0) return st0;
    double* dp = pos ? m->st_pos : nullptr;
    double* dv = vel ? m->st_vel : nullptr;
    double* da = accel ? m->st_acc : nullptr;
    int* di = image ? m->st_img : nullptr;
    enqueue_store_state(m, dp, dv, da, di, s);
    AZP_CHECK_LAUNCH("k_store_state");
    if (pos) AZP_CUDA_TRY(cudaMemcpyAsync(pos, dp, sizeof(double) * 4 * N, back, s));
    if (vel) AZP_CUDA_TRY(cudaMemcpyAsync(vel, dv, sizeof(double) * 4 * N, back, s));
    if (accel) AZP_CUDA_TRY(cudaMemcpyAsync(accel, da, sizeof(double) * 3 * N, back, s));
    if (image) AZP_CUDA_TRY(cudaMemcpyAsync(image, di, sizeof(int) * 3 * N, back, s));
    const int st = read_timestep();
    if (st) return st;
    if (!on_device) AZP_CUDA_TRY(cudaStreamSynchronize(s));
    return AZP_OK;
}

int azp_md_set_barrier_locations(azp_md* m, uint64_t t_first, uint32_t n, const double* location, void* stream)
{
    if (!m || m->bar_geom < 0 || n == 0 || !location) return AZP_ERR_INVALID;
    if (n > AZP_MD_BARRIER_ROWS) {
        const std::string msg = "azp_md_set_barrier_locations: " + std::to_string(n) + " rows exceed the table of " +
                                std::to_string(AZP_MD_BARRIER_ROWS) + " (set the locations run by run)";
        return record_error(AZP_ERR_TOO_LARGE, msg.c_str());
    }
    for (uint32_t r = 0; r < n; ++r)
        if (!barrier_location_valid(m->bar_geom, location[r], m->box))
            return record_error(AZP_ERR_INVALID, "Barrier position is invalid");
    const uint32_t nt = m->ntypes;
    // records of c = location + offset (the driver's addition), FP64 (c, k) or FP32
    std::vector<double> tab((size_t)2 * n * nt);
    for (uint32_t r = 0; r < n; ++r)
        for (uint32_t t = 0; t < nt; ++t) {
            const double k = m->bar_params[2 * t], c = location[r] + m->bar_params[2 * t + 1];
            double* rec = &tab[2 * ((size_t)r * nt + t)];
            if (m->precision == AZP_FP32) {
                const BarrierRecF f = barrier_rec_f(m->bar_geom, c, k, m->box.L[1]);
                std::memcpy(rec, &f, sizeof(f));
            } else {
                rec[0] = c;
                rec[1] = k;
            }
        }
    const unsigned long long hdr[2] = {(unsigned long long)t_first, (unsigned long long)n};
    cudaStream_t s = as_stream(stream);
    // pageable sources: both copies are staged before the calls return
    AZP_CUDA_TRY(cudaMemcpyAsync(m->d_bar_tab, tab.data(), sizeof(double) * tab.size(), cudaMemcpyHostToDevice, s));
    AZP_CUDA_TRY(cudaMemcpyAsync(m->d_bar_hdr, hdr, sizeof(hdr), cudaMemcpyHostToDevice, s));
    AZP_CUDA_TRY(cudaStreamSynchronize(s));
    m->bar_set = true;
    m->forces_valid = false;
    return AZP_OK;
}

int azp_md_set_temperatures(azp_md* m, uint64_t t_first, uint32_t n, const double* kT, void* stream)
{
    if (!m || n == 0 || !kT) return AZP_ERR_INVALID;
    if (n > AZP_MD_KT_ROWS) {
        const std::string msg = "azp_md_set_temperatures: " + std::to_string(n) + " rows exceed the table of " +
                                std::to_string(AZP_MD_KT_ROWS) + " (set the temperatures run by run)";
        return record_error(AZP_ERR_TOO_LARGE, msg.c_str());
    }
    for (uint32_t r = 0; r < n; ++r)
        if (!(kT[r] >= 0.0) || !std::isfinite(kT[r])) return record_error(AZP_ERR_INVALID, "kT must be finite and >= 0");
    const uint32_t nt = m->ntypes;
    if (!m->d_kT_hdr) {
        // first table: allocate it, and drop the captured graphs, whose step
        // arguments were taken without one
        int st = dalloc(&m->d_kT_hdr, 2);
        if (!st) st = dalloc(&m->d_kT_tab, AZP_MD_KT_ROWS);
        if (!st) st = dalloc(&m->d_noise_tab, (size_t)AZP_MD_KT_ROWS * nt);
        if (st) return st;
        free_graphs(m);
    }
    // noise amplitude per (row, type) with the operations of the reference's
    // step two, sqrt(6 gamma kT / dt) (src/TwoStepLangevinFlow.h:213-215)
    std::vector<double> noise((size_t)n * nt, 0.0);
    if (!m->noiseless)
        for (uint32_t r = 0; r < n; ++r)
            for (uint32_t t = 0; t < nt; ++t) noise[(size_t)r * nt + t] = std::sqrt(6.0 * m->gamma[t] * kT[r] / m->dt);
    const unsigned long long hdr[2] = {(unsigned long long)t_first, (unsigned long long)n};
    cudaStream_t s = as_stream(stream);
    AZP_CUDA_TRY(cudaMemcpyAsync(m->d_kT_tab, kT, sizeof(double) * n, cudaMemcpyHostToDevice, s));
    AZP_CUDA_TRY(cudaMemcpyAsync(m->d_noise_tab, noise.data(), sizeof(double) * noise.size(), cudaMemcpyHostToDevice, s));
    AZP_CUDA_TRY(cudaMemcpyAsync(m->d_kT_hdr, hdr, sizeof(hdr), cudaMemcpyHostToDevice, s));
    AZP_CUDA_TRY(cudaStreamSynchronize(s));
    return AZP_OK;
}

int azp_md_run(azp_md* m, uint64_t steps, void* stream)
{
    if (!m || !m->have_state) return AZP_ERR_INVALID;
    if (m->bar_geom >= 0 && !m->bar_set)
        return record_error(AZP_ERR_INVALID, "azp_md_run: the barrier locations are not set");
    m->launches = 0;
    if (steps == 0 || m->N == 0) return AZP_OK;
    m->forces_valid = false;
    cudaStream_t s = as_stream(stream);
    const int integ = m->method == AZP_METHOD_BROWNIAN_FLOW ? MD_INTEG_BROWNIAN : MD_INTEG_LANGEVIN;
    int st = AZP_OK;
    // Langevin: step one opens the run, the last step closes it without one
    uint64_t mid = integ == MD_INTEG_LANGEVIN ? steps - 1 : steps;
    if (integ == MD_INTEG_LANGEVIN) {
        st = enqueue_step1(m, s);
        if (st) return st;
    }
    if (m->use_graphs && mid >= 2) {
        for (int p = 0; p < 2; ++p)
            if (!m->gexec[p]) {
                st = build_pair_graph(m, p, integ, &m->gexec[p]);
                if (st) return st;
            }
        while (mid >= 2) {
            AZP_CUDA_TRY(cudaGraphLaunch(m->gexec[m->cur], s));
            // arm + two step kernels (+ their snapshot kernels for DPD / ImageHarmonic);
            // the rebuild bodies run only when armed and are not counted
            m->launches += 3 + ((m->d_dvel || m->d_img0) ? 2 : 0) + (m->d_wall_f ? 2 : 0);
            mid -= 2;
        }
    }
    while (mid > 0) {
        st = rebuild_if_requested(m, s);
        if (st) return st;
        st = enqueue_step(m, integ, 1, 0, s, 0, 0);
        if (st) return st;
        m->cur ^= 1;
        --mid;
    }
    if (integ == MD_INTEG_LANGEVIN) {
        st = rebuild_if_requested(m, s);
        if (st) return st;
        st = enqueue_step(m, integ, 0, 1, s, 0, 0);
        if (st) return st;
        m->forces_valid = true;  // the closing step wrote the forces of the final state
    }
    m->timestep += steps;
    return AZP_OK;
}

int azp_md_forces(azp_md* m, double* force, double* virial, int on_device, void* stream)
{
    if (!m || !m->have_state) return AZP_ERR_INVALID;
    if (m->bar_geom >= 0 && !m->bar_set)
        return record_error(AZP_ERR_INVALID, "azp_md_forces: the barrier locations are not set");
    cudaStream_t s = as_stream(stream);
    const uint32_t N = m->N;
    if (N == 0) return AZP_OK;
    int st = rebuild_if_requested(m, s);
    if (st) return st;
    MDArgs a = base_args(m);
    a.out = 1;
    st = md_launch(m, MD_FORCES_ONLY, a, s);
    if (st) return st;
    m->forces_valid = true;
    k_to_tag_order4<<<blocks_for(N, 256), 256, 0, s>>>(m->out_force, m->tag, N, m->tmp4);
    k_to_tag_order_n<<<blocks_for(N, 256), 256, 0, s>>>(m->out_virial, m->tag, N, 6, 1, m->tmpd);
    AZP_CHECK_LAUNCH("azp_md_forces");
    const cudaMemcpyKind k = on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
    if (force) AZP_CUDA_TRY(cudaMemcpyAsync(force, m->tmp4, sizeof(double) * 4 * N, k, s));
    if (virial) AZP_CUDA_TRY(cudaMemcpyAsync(virial, m->tmpd, sizeof(double) * 6 * N, k, s));
    if (!on_device) AZP_CUDA_TRY(cudaStreamSynchronize(s));
    return check_errors(m, s);
}

int azp_md_thermo(azp_md* m, double* out, void* stream)
{
    if (!m || !m->have_state || !out) return AZP_ERR_INVALID;
    cudaStream_t s = as_stream(stream);
    const uint32_t N = m->N;
    for (int c = 0; c < 9; ++c) out[c] = 0.0;
    if (N == 0) return AZP_OK;
    if (!m->forces_valid) {
        if (m->bar_geom >= 0 && !m->bar_set)
            return record_error(AZP_ERR_INVALID, "azp_md_thermo: the barrier locations are not set");
        int st = rebuild_if_requested(m, s);
        if (st) return st;
        MDArgs a = base_args(m);
        a.out = 1;
        st = md_launch(m, MD_FORCES_ONLY, a, s);
        if (st) return st;
        m->forces_valid = true;
    }
    const uint32_t nb = blocks_for(N, THERMO_BLOCK);
    k_thermo_partials<<<nb, THERMO_BLOCK, 0, s>>>(m->out_force, m->out_virial, m->vel, m->mass, N, m->partials);
    k_thermo_final<<<1, THERMO_BLOCK, 0, s>>>(m->partials, nb, m->flags, m->thermo);
    AZP_CHECK_LAUNCH("azp_md_thermo");
    double* h = m->h_thermo;
    AZP_CUDA_TRY(cudaMemcpyAsync(h, m->thermo, sizeof(double) * 12, cudaMemcpyDeviceToHost, s));
    AZP_CUDA_TRY(cudaStreamSynchronize(s));
    uint32_t f[8];
    std::memcpy(f, h + 8, sizeof(f));
    for (int c = 0; c < 8; ++c) out[c] = h[c];
    out[8] = (double)f[2];
    // the error word came back with the sums (check_errors without a second read)
    if (f[3] > m->max_nn) return AZP_ERR_NLIST_OVERFLOW;
    if (f[1] & AZP_EBIT_BOND) return AZP_ERR_BOND;
    if (f[1] & AZP_EBIT_NONFINITE) return AZP_ERR_NONFINITE;
    return AZP_OK;
}

int azp_md_error(azp_md* m, uint32_t* err_word, void* stream)
{
    if (!m || !err_word) return AZP_ERR_INVALID;
    cudaStream_t s = as_stream(stream);
    uint32_t f[8];
    AZP_CUDA_TRY(cudaMemcpyAsync(f, m->flags, sizeof(f), cudaMemcpyDeviceToHost, s));
    AZP_CUDA_TRY(cudaStreamSynchronize(s));
    uint32_t e = f[1];
    if (f[3] > m->max_nn) e |= AZP_EBIT_NLIST_OVERFLOW;
    *err_word = e;
    return AZP_OK;
}

uint64_t azp_md_last_launches(const azp_md* m) { return m ? m->launches : 0; }

int azp_md_run_checked(azp_md* m, uint64_t steps, void* stream)
{
    if (!m || !m->have_state) return AZP_ERR_INVALID;
    cudaStream_t s = as_stream(stream);
    const uint32_t N = m->N;
    if (steps == 0 || N == 0) return azp_md_run(m, steps, stream);
    if (!m->snap_pos) {
        int st = dalloc(&m->snap_pos, (size_t)4 * N);
        if (!st) st = dalloc(&m->snap_vel, (size_t)4 * N);
        if (!st) st = dalloc(&m->snap_acc, (size_t)3 * N);
        if (!st) st = dalloc(&m->snap_img, (size_t)3 * N);
        if (!st && m->diam) st = dalloc(&m->snap_diam, N);
        if (st) return st;
    }
    unsigned long long ts0 = 0;
    AZP_CUDA_TRY(cudaMemcpyAsync(&ts0, m->d_ts, sizeof(ts0), cudaMemcpyDeviceToHost, s));
    enqueue_store_state(m, m->snap_pos, m->snap_vel, m->snap_acc, m->snap_img, s);
    if (m->diam) k_to_tag_order_n<<<blocks_for(N, 256), 256, 0, s>>>(m->diam, m->tag, N, 1, 0, m->snap_diam);
    AZP_CHECK_LAUNCH("k_store_state (snapshot)");
    AZP_CUDA_TRY(cudaStreamSynchronize(s));
    for (int attempt = 0; attempt < 4; ++attempt) {
        int st = azp_md_run(m, steps, stream);
        if (st) return st;
        uint32_t f[8];
        AZP_CUDA_TRY(cudaMemcpyAsync(f, m->flags, sizeof(f), cudaMemcpyDeviceToHost, s));
        AZP_CUDA_TRY(cudaStreamSynchronize(s));
        if (f[3] <= m->max_nn) return check_errors(m, s);
        // grow to the largest count seen and replay from the entry state
        cudaFree(m->nbrs);
        m->nbrs = nullptr;
        m->max_nn = (uint32_t)std::ceil(f[3] * 1.5) + 16;
        st = dalloc(&m->nbrs, (size_t)N * m->max_nn);
        if (st) return st;
        free_graphs(m);
        AZP_CUDA_TRY(cudaMemsetAsync(m->flags + 1, 0, sizeof(uint32_t) * 3, s));
        // the regrown list holds nothing yet: replay through the full set-up path
        // (sort and build), not the order-keeping one
        m->have_state = false;
        st = azp_md_set_state(m, m->snap_pos, m->snap_vel, m->snap_acc, m->snap_img, m->snap_diam, ts0, 1, stream);
        if (st) return st;
        m->launches = 0;
    }
    return AZP_ERR_NLIST_OVERFLOW;
}

int azp_md_time_step_kernel(azp_md* m, int reps, float* ms, void* stream)
{
    if (!m || !m->have_state || reps <= 0 || !ms) return AZP_ERR_INVALID;
    cudaStream_t s = as_stream(stream);
    const int integ = m->method == AZP_METHOD_BROWNIAN_FLOW ? MD_INTEG_BROWNIAN : MD_INTEG_LANGEVIN;
    m->forces_valid = false;
    cudaEvent_t e0, e1;
    AZP_CUDA_TRY(cudaEventCreate(&e0));
    AZP_CUDA_TRY(cudaEventCreate(&e1));
    int st = enqueue_step(m, integ, 1, 0, s, 0, 0);  // warm
    m->cur ^= 1;
    AZP_CUDA_TRY(cudaEventRecord(e0, s));
    for (int r = 0; r < reps && st == AZP_OK; ++r) {
        st = enqueue_step(m, integ, 1, 0, s, 0, 0);
        m->cur ^= 1;
    }
    AZP_CUDA_TRY(cudaEventRecord(e1, s));
    AZP_CUDA_TRY(cudaEventSynchronize(e1));
    float t = 0.0f;
    AZP_CUDA_TRY(cudaEventElapsedTime(&t, e0, e1));
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    *ms = t / (float)reps;
    return st;
}

}  // extern "C"
