// batch.cu -- many independent systems advanced together (azp_batch).
//
// S replicas of uneven size, each with its own periodic box, pair parameters and
// RNG seed, are packed into one particle array (replica r owns the index range
// [off_r, off_r + N_r) after every re-sort) and advanced by ONE fused force +
// Langevin launch per timestep for all replicas together, replayed from a CUDA
// graph; a list rebuild for all replicas runs as a graph conditional node when
// any particle of any replica moved more than r_buff / 2.
//
// Replicas never see each other: every replica has its own cell grid (global
// cell index = the replica's cell offset + its local cell), so candidate cells of
// a particle belong to its own replica only. Positions of replica r are stored as
// fixed-point fractions of ITS box, so the integer difference is its minimum
// image. Tags are per replica (0 .. N_r - 1) and the seed is the replica's: each
// replica draws exactly the noise it would draw run alone.
//
// One particle type per replica; pair potentials as in the single-system engine
// (the arithmetic of evaluators.cuh, FP32 forces with FP64 integration or FP64).
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <new>
#include <vector>

#include "celllist.cuh"
#include "evaluators.cuh"
#include "integrate.cuh"
#include "pair.cuh"
#include "scan.cuh"

namespace azp
{
struct SysInfo {
    double L[3], Linv[3], lo[3], hi[3], fscale[3];
    float sfix[3];
    float list_lo, list_hi;   // FP32 list prefilter thresholds
    double rlistsq;           // exact list decision
    double rcutsq;
    uint32_t cell_off;
    int dim[3];
    int reach[3];
    double cscale[3];         // dim / L
    uint32_t seed;
    uint32_t pad_;
    double rec[PAIR_TBL];     // pair kernel record + cut record (one type)
};

constexpr int BATCH_BLOCK = 256;      // default threads per block of the fused step
constexpr int BATCH_BLOCK_MAX = 512;  // largest block azp_batch_set_block accepts

AZP_D void comp_shfl_add(Comp& c, int m)
{
    const float s2 = __shfl_xor_sync(0xffffffffu, c.s, m);
    const float c2 = __shfl_xor_sync(0xffffffffu, c.c, m);
    c.add(s2);
    c.c += c2;
}

// ---------------------------------------------------------------- rebuild kernels
__global__ void k_b_zero(uint32_t* __restrict__ p, uint32_t n, const uint32_t* __restrict__ gate)
{
    if (gated_off(gate)) return;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) p[i] = 0u;
}

__device__ __forceinline__ int b_cell_coord(double x, double lo, double scale, int dim)
{
    int c = (int)floor((x - lo) * scale);
    if (c < 0) c += dim;
    if (c >= dim) c -= dim;
    return min(max(c, 0), dim - 1);
}

__global__ void k_b_assign(const double4_32a* __restrict__ pos, const uint16_t* __restrict__ sys, uint32_t N,
                           const SysInfo* __restrict__ info, uint32_t* __restrict__ cell_of,
                           uint32_t* __restrict__ slot, uint32_t* __restrict__ cell_count,
                           const uint32_t* __restrict__ gate)
{
    if (gated_off(gate)) return;
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= N) return;
    const SysInfo& si = info[sys[i]];
    const double4_32a p = pos[i];
    const int cx = b_cell_coord(p.x, si.lo[0], si.cscale[0], si.dim[0]);
    const int cy = b_cell_coord(p.y, si.lo[1], si.cscale[1], si.dim[1]);
    const int cz = b_cell_coord(p.z, si.lo[2], si.cscale[2], si.dim[2]);
    const uint32_t c = si.cell_off + ((uint32_t)cz * si.dim[1] + cy) * si.dim[0] + cx;
    cell_of[i] = c;
    slot[i] = atomicAdd(&cell_count[c], 1u);
}

__global__ void k_b_scatter(const uint32_t* __restrict__ cell_of, const uint32_t* __restrict__ slot,
                            const uint32_t* __restrict__ cell_start, uint32_t* __restrict__ members, uint32_t N,
                            const uint32_t* __restrict__ gate)
{
    if (gated_off(gate)) return;
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= N) return;
    members[cell_start[cell_of[i]] + slot[i]] = i;
}

// each cell's members sorted by index (deterministic order): one warp per 32
// consecutive cells, a lane per cell for small cells, the whole warp for crowded ones
__global__ void __launch_bounds__(kSortWarps * 32) k_b_cell_sort(const uint32_t* __restrict__ cell_start,
                                                                 uint32_t* __restrict__ members, uint32_t ncell,
                                                                 const uint32_t* __restrict__ gate)
{
    if (gated_off(gate)) return;
    __shared__ uint32_t s_rows[kSortWarps][kMaxSortedCell];
    sort_cells_warp(cell_start, members, ncell, s_rows[threadIdx.x >> 5]);
}

__global__ void __launch_bounds__(kSortWarps * 32) k_b_cell_sort_crowded(const uint32_t* __restrict__ cell_start,
                                                                         uint32_t* __restrict__ members,
                                                                         uint32_t ncell,
                                                                         const uint32_t* __restrict__ gate)
{
    if (gated_off(gate)) return;
    __shared__ uint32_t s_rows[kSortWarps][kMaxSortedCell];
    sort_cell_per_warp(cell_start, members, ncell, s_rows[threadIdx.x >> 5]);
}

struct BPerm {
    const uint32_t* members;
    double4_32a *pos, *t_pos, *vel, *t_vel;
    double *accel, *t_accel;
    int *image, *t_image;
    uint32_t *tag, *t_tag;
    uint16_t *sys, *t_sys;
    uint32_t *cell_of, *t_cell;
    uint32_t N;
};

__global__ void k_b_gather(BPerm a, const uint32_t* __restrict__ gate)
{
    if (gated_off(gate)) return;
    const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= a.N) return;
    const uint32_t o = a.members[s];
    a.t_pos[s] = a.pos[o];
    a.t_vel[s] = a.vel[o];
    for (int d = 0; d < 3; ++d) {
        a.t_accel[3 * s + d] = a.accel[3 * o + d];
        a.t_image[3 * s + d] = a.image[3 * o + d];
    }
    a.t_tag[s] = a.tag[o];
    a.t_sys[s] = a.sys[o];
    a.t_cell[s] = a.cell_of[o];
}

__global__ void k_b_back(BPerm a, const uint32_t* __restrict__ gate)
{
    if (gated_off(gate)) return;
    const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= a.N) return;
    a.pos[s] = a.t_pos[s];
    a.vel[s] = a.t_vel[s];
    for (int d = 0; d < 3; ++d) {
        a.accel[3 * s + d] = a.t_accel[3 * s + d];
        a.image[3 * s + d] = a.t_image[3 * s + d];
    }
    a.tag[s] = a.t_tag[s];
    a.sys[s] = a.t_sys[s];
    a.cell_of[s] = a.t_cell[s];
}

__global__ void k_b_fixed(const double4_32a* __restrict__ pos, const uint16_t* __restrict__ sys, uint32_t N,
                          const SysInfo* __restrict__ info, uint4* __restrict__ fa, uint4* __restrict__ fb,
                          const uint32_t* __restrict__ gate)
{
    if (gated_off(gate)) return;
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= N) return;
    const SysInfo& si = info[sys[i]];
    const double4_32a p = pos[i];
    uint4 f;
    f.x = to_fixed(p.x, si.Linv[0]);
    f.y = to_fixed(p.y, si.Linv[1]);
    f.z = to_fixed(p.z, si.Linv[2]);
    f.w = sys[i];
    fa[i] = f;
    fb[i] = f;
}

__global__ void __launch_bounds__(128)
    k_b_nlist(const double4_32a* __restrict__ pos, const uint4* __restrict__ fixed, const uint16_t* __restrict__ sys,
              uint32_t N, const SysInfo* __restrict__ info, const uint32_t* __restrict__ cell_start,
              const uint32_t* __restrict__ cell_of, uint32_t* __restrict__ counts, uint32_t* __restrict__ nbrs,
              uint32_t max_nn, uint32_t* __restrict__ maxcount, const uint32_t* __restrict__ gate)
{
    if (gated_off(gate)) return;
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= N) return;
    const SysInfo& si = info[sys[i]];
    const uint4 fi = fixed[i];
    const uint32_t c = cell_of[i] - si.cell_off;
    const int cx = (int)(c % si.dim[0]);
    const int cy = (int)((c / si.dim[0]) % si.dim[1]);
    const int cz = (int)(c / ((uint32_t)si.dim[0] * si.dim[1]));
    uint32_t n = 0;
    for (int oz = -si.reach[2]; oz <= si.reach[2]; ++oz) {
        int nz = cz + oz;
        nz += (nz < 0) ? si.dim[2] : 0;
        nz -= (nz >= si.dim[2]) ? si.dim[2] : 0;
        for (int oy = -si.reach[1]; oy <= si.reach[1]; ++oy) {
            int ny = cy + oy;
            ny += (ny < 0) ? si.dim[1] : 0;
            ny -= (ny >= si.dim[1]) ? si.dim[1] : 0;
            for (int ox = -si.reach[0]; ox <= si.reach[0]; ++ox) {
                int nx = cx + ox;
                nx += (nx < 0) ? si.dim[0] : 0;
                nx -= (nx >= si.dim[0]) ? si.dim[0] : 0;
                const uint32_t nc = si.cell_off + ((uint32_t)nz * si.dim[1] + ny) * si.dim[0] + nx;
                const uint32_t sb = cell_start[nc], se = cell_start[nc + 1];
                for (uint32_t j = sb; j < se; ++j) {
                    if (j == i) continue;
                    const uint4 fj = fixed[j];
                    const float dx = (float)(int32_t)(fi.x - fj.x) * si.sfix[0];
                    const float dy = (float)(int32_t)(fi.y - fj.y) * si.sfix[1];
                    const float dz = (float)(int32_t)(fi.z - fj.z) * si.sfix[2];
                    const float rs = dx * dx + dy * dy + dz * dz;
                    if (rs >= si.list_hi) continue;
                    if (!(rs < si.list_lo)) {
                        const double4_32a pi = pos[i];
                        const double4_32a pj = pos[j];
                        const double vx = min_image1(pi.x - pj.x, si.L[0], si.Linv[0]);
                        const double vy = min_image1(pi.y - pj.y, si.L[1], si.Linv[1]);
                        const double vz = min_image1(pi.z - pj.z, si.L[2], si.Linv[2]);
                        if (!(rsq_exact(vx, vy, vz) < si.rlistsq)) continue;
                    }
                    if (n < max_nn) nbrs[(size_t)n * N + i] = j;
                    ++n;
                }
            }
        }
    }
    counts[i] = n;
    if (n > max_nn) atomicMax(maxcount, n);
}

__global__ void k_b_finish(uint32_t* __restrict__ flags, const uint32_t* __restrict__ gate)
{
    if (gated_off(gate)) return;
    flags[0] = 0u;
    flags[2] += 1u;
}

__global__ void k_b_arm(const uint32_t* __restrict__ flags, cudaGraphConditionalHandle h)
{
    cudaGraphSetConditional(h, (flags[0] && !flags[1]) ? 1u : 0u);
}

// ---------------------------------------------------------------- fused step
struct BStep {
    const double4_32a* pos;
    double4_32a* pos_next;
    const uint4* fix;
    uint4* fix_next;
    const uint4* fix_build;
    double4_32a* vel;
    double* accel;
    int* image;
    const uint32_t* tag;
    const uint16_t* sys;
    const SysInfo* info;
    uint32_t N;
    const uint32_t* counts;
    const uint32_t* nbrs;
    uint32_t max_nn;
    double dt, kT, gamma, noise;
    int noiseless;
    FlowD flow;
    const unsigned long long* d_ts;
    unsigned long long* d_ts_rw;
    uint32_t* flags;
    float disp_thresh2;
    int next;
    int tpp;
    int block;  // threads per block of the launch
    cudaGraphConditionalHandle next_cond;
    int set_cond;
};

// neighbours gathered per batch in the FP32-force pair loop
#ifndef AZP_B_BATCH
#define AZP_B_BATCH 4
#endif
constexpr int B_BATCH = AZP_B_BATCH;

template<class PE, typename R>
__global__ void __launch_bounds__(BATCH_BLOCK_MAX) k_b_step(BStep a)
{
    const int tpp = a.tpp;
    const uint32_t gid = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t i = gid / tpp;
    const uint32_t sub = gid % tpp;
    const bool active = i < a.N;
    R fx = 0, fy = 0, fz = 0;
    Comp cx{0.f, 0.f}, cy{0.f, 0.f}, cz{0.f, 0.f};
    const SysInfo* si = active ? a.info + a.sys[i] : a.info;
    if (active) {
        R rec[PAIR_TBL];
#pragma unroll
        for (int k = 0; k < PAIR_TBL; ++k) rec[k] = (R)si->rec[k];
        const bool on = PE::enabled(rec);
        const uint32_t n = on ? min(a.counts[i], a.max_nn) : 0u;
        if constexpr (std::is_same<R, double>::value) {
            const double4_32a pi = a.pos[i];
            for (uint32_t k = sub; k < n; k += tpp) {
                const uint32_t j = a.nbrs[(size_t)k * a.N + i];
                const double4_32a pj = a.pos[j];
                const double dx = min_image1(pi.x - pj.x, si->L[0], si->Linv[0]);
                const double dy = min_image1(pi.y - pj.y, si->L[1], si->Linv[1]);
                const double dz = min_image1(pi.z - pj.z, si->L[2], si->Linv[2]);
                const double rsq = rsq_exact(dx, dy, dz);
                if (!(rsq < si->rcutsq)) continue;
                double fdr, e;
                PE::eval(rec, rsq, fdr, e);
                fx += dx * fdr;
                fy += dy * fdr;
                fz += dz * fdr;
            }
        } else {
            const uint4 fi = a.fix[i];
            const float rc2 = (float)si->rcutsq;
            // neighbours in batches of B_BATCH: the list entries of a batch first,
            // then their fixed-point words, so that B_BATCH gathers are in flight;
            // the pairs are then added in list order as one at a time would
            const uint32_t* col = a.nbrs + i;
            for (uint32_t kb = sub; kb < n; kb += B_BATCH * tpp) {
                uint32_t jj[B_BATCH];
                uint4 fj[B_BATCH];
#pragma unroll
                for (int u = 0; u < B_BATCH; ++u) {
                    const uint32_t k = kb + u * tpp;
                    jj[u] = k < n ? __ldg(col + (size_t)k * a.N) : i;
                }
#pragma unroll
                for (int u = 0; u < B_BATCH; ++u) fj[u] = __ldg(a.fix + jj[u]);
#pragma unroll
                for (int u = 0; u < B_BATCH; ++u) {
                    if (kb + u * tpp >= n) break;
                    const float dx = (float)(int32_t)(fi.x - fj[u].x) * si->sfix[0];
                    const float dy = (float)(int32_t)(fi.y - fj[u].y) * si->sfix[1];
                    const float dz = (float)(int32_t)(fi.z - fj[u].z) * si->sfix[2];
                    const float rsq = dx * dx + dy * dy + dz * dz;
                    if (rsq >= rc2 * 1.000004f) continue;
                    if (rsq >= rc2 * 0.999996f) {
                        const double4_32a pi = a.pos[i];
                        const double4_32a pj = a.pos[jj[u]];
                        const double vx = min_image1(pi.x - pj.x, si->L[0], si->Linv[0]);
                        const double vy = min_image1(pi.y - pj.y, si->L[1], si->Linv[1]);
                        const double vz = min_image1(pi.z - pj.z, si->L[2], si->Linv[2]);
                        if (!(rsq_exact(vx, vy, vz) < si->rcutsq)) continue;
                    }
                    float fdr, e;
                    PE::eval(rec, rsq, fdr, e);
                    cx.add(dx * fdr);
                    cy.add(dy * fdr);
                    cz.add(dz * fdr);
                }
            }
        }
    }
    for (int m = tpp >> 1; m > 0; m >>= 1) {
        if constexpr (std::is_same<R, double>::value) {
            fx += __shfl_xor_sync(0xffffffffu, fx, m);
            fy += __shfl_xor_sync(0xffffffffu, fy, m);
            fz += __shfl_xor_sync(0xffffffffu, fz, m);
        } else {
            comp_shfl_add(cx, m);
            comp_shfl_add(cy, m);
            comp_shfl_add(cz, m);
        }
    }
    bool want = false;
    if (active && sub == 0) {
        const unsigned long long ts = *a.d_ts;
        double4_32a p = a.pos[i];
        double4_32a v = a.vel[i];
        const uint32_t tg = a.tag[i];
        bool moved = false;
        if constexpr (std::is_same<R, double>::value) {
            double ux, uy, uz;
            flow_at(a.flow, p.y, ux, uy, uz);
            const double c = a.noiseless ? 0.0 : a.noise;
            double r0, r1, r2;
            uniform3(AZP_RNG_LANGEVIN_FLOW, ts, si->seed, tg, -c, c - (-c), r0, r1, r2);
            const double minv = 1.0 / v.w;
            const double ax = (fx + (r0 - a.gamma * (v.x - ux))) * minv;
            const double ay = (fy + (r1 - a.gamma * (v.y - uy))) * minv;
            const double az = (fz + (r2 - a.gamma * (v.z - uz))) * minv;
            const double h = 0.5 * a.dt;
            v.x += h * ax;
            v.y += h * ay;
            v.z += h * az;
            if (a.next) {
                p.x += (v.x + h * ax) * a.dt;
                p.y += (v.y + h * ay) * a.dt;
                p.z += (v.z + h * az) * a.dt;
                v.x += h * ax;
                v.y += h * ay;
                v.z += h * az;
                moved = true;
            } else {
                a.accel[3 * i] = ax;
                a.accel[3 * i + 1] = ay;
                a.accel[3 * i + 2] = az;
            }
        } else {
            float ux, uy, uz;
            flow_at_f(a.flow, (float)p.y, ux, uy, uz);
            const float c = a.noiseless ? 0.0f : (float)a.noise;
            const float g = (float)a.gamma, dt = (float)a.dt;
            float r0, r1, r2;
            uniform3f(AZP_RNG_LANGEVIN_FLOW, ts, si->seed, tg, -c, 2.0f * c, r0, r1, r2);
            const float minv = __frcp_rn((float)v.w);
            const float ax = (cx.value() + (r0 - g * ((float)v.x - ux))) * minv;
            const float ay = (cy.value() + (r1 - g * ((float)v.y - uy))) * minv;
            const float az = (cz.value() + (r2 - g * ((float)v.z - uz))) * minv;
            if (a.next) {
                const float kx = dt * ax, ky = dt * ay, kz = dt * az;
                p.x += (double)(((float)v.x + kx) * dt);
                p.y += (double)(((float)v.y + ky) * dt);
                p.z += (double)(((float)v.z + kz) * dt);
                v.x += (double)kx;
                v.y += (double)ky;
                v.z += (double)kz;
                moved = true;
            } else {
                const float h = 0.5f * dt;
                v.x += (double)(h * ax);
                v.y += (double)(h * ay);
                v.z += (double)(h * az);
                a.accel[3 * i] = ax;
                a.accel[3 * i + 1] = ay;
                a.accel[3 * i + 2] = az;
            }
        }
        a.vel[i] = v;
        if (moved) {
            int w[3] = {0, 0, 0};
            wrap1(p.x, w[0], si->L[0], si->lo[0], si->hi[0]);
            wrap1(p.y, w[1], si->L[1], si->lo[1], si->hi[1]);
            wrap1(p.z, w[2], si->L[2], si->lo[2], si->hi[2]);
            if (w[0] | w[1] | w[2])
                for (int d = 0; d < 3; ++d) a.image[3 * i + d] += w[d];
            a.pos_next[i] = p;
            uint4 f;
            f.x = to_fixed(p.x, si->Linv[0]);
            f.y = to_fixed(p.y, si->Linv[1]);
            f.z = to_fixed(p.z, si->Linv[2]);
            f.w = a.sys[i];
            a.fix_next[i] = f;
            const uint4 fb = a.fix_build[i];
            const float ddx = (float)(int32_t)(f.x - fb.x) * si->sfix[0];
            const float ddy = (float)(int32_t)(f.y - fb.y) * si->sfix[1];
            const float ddz = (float)(int32_t)(f.z - fb.z) * si->sfix[2];
            want = ddx * ddx + ddy * ddy + ddz * ddz > a.disp_thresh2;
            if (!(isfinite(p.x) && isfinite(p.y) && isfinite(p.z))) atomicOr(&a.flags[1], AZP_EBIT_NONFINITE);
        }
    }
    if (__any_sync(0xffffffffu, want) && (threadIdx.x & 31) == 0) atomicOr(&a.flags[0], 1u);
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        const uint32_t t = atomicAdd(&a.flags[4], 1u);
        if (t == gridDim.x - 1) {
            __threadfence();
            const uint32_t req = atomicAdd(&a.flags[0], 0u) && !atomicAdd(&a.flags[1], 0u);
            if (a.set_cond) cudaGraphSetConditional(a.next_cond, req ? 1u : 0u);
            a.flags[4] = 0u;
            *a.d_ts_rw = *a.d_ts_rw + 1ull;
        }
    }
}

// Langevin step one in place at the start of a run
__global__ void k_b_step1(double4_32a* __restrict__ pos, uint4* __restrict__ fix, const uint4* __restrict__ fix_build,
                          double4_32a* __restrict__ vel, const double* __restrict__ accel, int* __restrict__ image,
                          const uint16_t* __restrict__ sys, const SysInfo* __restrict__ info, uint32_t N, double dt,
                          float thresh2, uint32_t* __restrict__ flags)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    bool want = false;
    if (i < N) {
        const SysInfo& si = info[sys[i]];
        double4_32a p = pos[i];
        double4_32a v = vel[i];
        const double h = 0.5 * dt;
        const double ax = accel[3 * i], ay = accel[3 * i + 1], az = accel[3 * i + 2];
        p.x += (v.x + h * ax) * dt;
        p.y += (v.y + h * ay) * dt;
        p.z += (v.z + h * az) * dt;
        int w[3] = {0, 0, 0};
        wrap1(p.x, w[0], si.L[0], si.lo[0], si.hi[0]);
        wrap1(p.y, w[1], si.L[1], si.lo[1], si.hi[1]);
        wrap1(p.z, w[2], si.L[2], si.lo[2], si.hi[2]);
        if (w[0] | w[1] | w[2])
            for (int d = 0; d < 3; ++d) image[3 * i + d] += w[d];
        v.x += h * ax;
        v.y += h * ay;
        v.z += h * az;
        pos[i] = p;
        vel[i] = v;
        uint4 f;
        f.x = to_fixed(p.x, si.Linv[0]);
        f.y = to_fixed(p.y, si.Linv[1]);
        f.z = to_fixed(p.z, si.Linv[2]);
        f.w = sys[i];
        fix[i] = f;
        const uint4 fb = fix_build[i];
        const float dx = (float)(int32_t)(f.x - fb.x) * si.sfix[0];
        const float dy = (float)(int32_t)(f.y - fb.y) * si.sfix[1];
        const float dz = (float)(int32_t)(f.z - fb.z) * si.sfix[2];
        want = dx * dx + dy * dy + dz * dz > thresh2;
    }
    if (__any_sync(0xffffffffu, want) && (threadIdx.x & 31) == 0) atomicOr(&flags[0], 1u);
}

__global__ void k_b_load(const double* __restrict__ pos_in, const double* __restrict__ vel_in,
                         const double* __restrict__ acc_in, const int* __restrict__ img_in,
                         const uint32_t* __restrict__ sys_of, const uint32_t* __restrict__ tag_of, uint32_t N,
                         double4_32a* __restrict__ pos, double4_32a* __restrict__ vel, double* __restrict__ acc,
                         int* __restrict__ img, uint32_t* __restrict__ tag, uint16_t* __restrict__ sys,
                         uint32_t* __restrict__ rindex)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= N) return;
    pos[i] = make_double4_32a(pos_in[4 * i], pos_in[4 * i + 1], pos_in[4 * i + 2], type_as_double(0u));
    vel[i] = make_double4_32a(vel_in[4 * i], vel_in[4 * i + 1], vel_in[4 * i + 2], vel_in[4 * i + 3]);
    for (int d = 0; d < 3; ++d) {
        acc[3 * i + d] = acc_in ? acc_in[3 * i + d] : 0.0;
        img[3 * i + d] = img_in ? img_in[3 * i + d] : 0;
    }
    tag[i] = tag_of[i];
    sys[i] = (uint16_t)sys_of[i];
    rindex[i] = i;
}

// device state -> packed order (replica offsets + tag)
__global__ void k_b_store(const double4_32a* __restrict__ pos, const double4_32a* __restrict__ vel,
                          const double* __restrict__ acc, const int* __restrict__ img, const uint32_t* __restrict__ tag,
                          const uint16_t* __restrict__ sys, const uint32_t* __restrict__ sys_off, uint32_t N,
                          double* __restrict__ pos_out, double* __restrict__ vel_out, double* __restrict__ acc_out,
                          int* __restrict__ img_out)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= N) return;
    const uint32_t o = sys_off[sys[i]] + tag[i];
    const double4_32a p = pos[i];
    const double4_32a v = vel[i];
    pos_out[4 * o] = p.x;
    pos_out[4 * o + 1] = p.y;
    pos_out[4 * o + 2] = p.z;
    pos_out[4 * o + 3] = 0.0;
    vel_out[4 * o] = v.x;
    vel_out[4 * o + 1] = v.y;
    vel_out[4 * o + 2] = v.z;
    vel_out[4 * o + 3] = v.w;
    for (int d = 0; d < 3; ++d) {
        acc_out[3 * o + d] = acc[3 * i + d];
        img_out[3 * o + d] = img[3 * i + d];
    }
}

template<class PE>
int launch_b_step(int precision, const BStep& a, cudaStream_t s)
{
    const uint32_t blocks = (uint32_t)(((size_t)a.N * a.tpp + a.block - 1) / a.block);
    if (blocks == 0) return AZP_OK;
    if (precision == AZP_FP32)
        k_b_step<PE, float><<<blocks, a.block, 0, s>>>(a);
    else
        k_b_step<PE, double><<<blocks, a.block, 0, s>>>(a);
    AZP_CHECK_LAUNCH("k_b_step");
    return AZP_OK;
}

int launch_b_step_kind(int kind, int precision, const BStep& a, cudaStream_t s)
{
    switch (kind) {
    case AZP_PAIR_PERTURBED_LJ: return launch_b_step<PerturbedLJ>(precision, a, s);
    case AZP_PAIR_EXPANDED_YUKAWA: return launch_b_step<ExpandedYukawa>(precision, a, s);
    case AZP_PAIR_HERTZ: return launch_b_step<Hertz>(precision, a, s);
    case AZP_PAIR_COLLOID: return launch_b_step<Colloid>(precision, a, s);
    default: return AZP_ERR_INVALID;
    }
}

}  // namespace azp

using namespace azp;

struct azp_batch {
    uint32_t S = 0, N = 0;
    std::vector<uint32_t> n_of, off;
    int precision = AZP_FP64, kind = 0, tpp = 1, block = BATCH_BLOCK;
    double dt = 0.005, kT = 1.0, gamma = 1.0, r_buff = 0.4;
    int noiseless = 0;
    FlowD flow{};
    SysInfo* info = nullptr;
    uint32_t* sys_off = nullptr;
    // state
    double4_32a* pos[2] = {nullptr, nullptr};
    uint4* fix[2] = {nullptr, nullptr};
    uint4* fix_build = nullptr;
    int cur = 0;
    double4_32a* vel = nullptr;
    double* accel = nullptr;
    int* image = nullptr;
    uint32_t* tag = nullptr;
    uint16_t* sys = nullptr;
    // temps
    double4_32a *t_pos = nullptr, *t_vel = nullptr;
    double* t_accel = nullptr;
    int* t_image = nullptr;
    uint32_t* t_tag = nullptr;
    uint16_t* t_sys = nullptr;
    uint32_t* t_cell = nullptr;
    // cells / list
    uint32_t ncell = 0;
    uint32_t *cell_of = nullptr, *slot = nullptr, *cell_count = nullptr, *cell_start = nullptr, *members = nullptr,
             *scan_tmp = nullptr, *rindex = nullptr;
    uint32_t max_nn = 32;
    uint32_t *counts = nullptr, *nbrs = nullptr;
    uint32_t* flags = nullptr;
    unsigned long long* d_ts = nullptr;
    uint64_t launches = 0;
    bool have_state = false, use_graphs = true;
    cudaGraphExec_t gexec[2] = {nullptr, nullptr};
    cudaStream_t gstream = nullptr;
};

namespace
{
template<typename T> int balloc(T** p, size_t n)
{
    *p = nullptr;
    const cudaError_t e = cudaMalloc(reinterpret_cast<void**>(p), sizeof(T) * (n ? n : 1));
    return e == cudaSuccess ? AZP_OK : record_cuda_error(e, "cudaMalloc (batch)");
}

void b_free_graphs(azp_batch* b)
{
    for (auto& g : b->gexec)
        if (g) {
            cudaGraphExecDestroy(g);
            g = nullptr;
        }
}

void b_free(azp_batch* b)
{
    b_free_graphs(b);
    void* ptrs[] = {b->info, b->sys_off, b->pos[0], b->pos[1], b->fix[0], b->fix[1], b->fix_build, b->vel, b->accel,
                    b->image, b->tag, b->sys, b->t_pos, b->t_vel, b->t_accel, b->t_image, b->t_tag, b->t_sys,
                    b->t_cell, b->cell_of, b->slot, b->cell_count, b->cell_start, b->members, b->scan_tmp,
                    b->rindex, b->counts, b->nbrs, b->flags, b->d_ts};
    for (void* p : ptrs) cudaFree(p);
    if (b->gstream) cudaStreamDestroy(b->gstream);
}

uint32_t nblk(uint32_t n) { return (n + 255) / 256; }

int b_rebuild(azp_batch* b, cudaStream_t s, const uint32_t* gate)
{
    const uint32_t N = b->N;
    k_b_zero<<<std::min<uint32_t>(nblk(b->ncell), 1024), 256, 0, s>>>(b->cell_count, b->ncell, gate);
    k_b_assign<<<nblk(N), 256, 0, s>>>(b->pos[b->cur], b->sys, N, b->info, b->cell_of, b->slot, b->cell_count, gate);
    int st = exclusive_scan(b->cell_count, b->cell_start, b->ncell, b->scan_tmp, s, gate);
    if (st) return st;
    k_b_scatter<<<nblk(N), 256, 0, s>>>(b->cell_of, b->slot, b->cell_start, b->members, N, gate);
    if (crowded_grid(N, b->ncell))
        k_b_cell_sort_crowded<<<(b->ncell + kSortWarps - 1) / kSortWarps, kSortWarps * 32, 0, s>>>(
            b->cell_start, b->members, b->ncell, gate);
    else
        k_b_cell_sort<<<(b->ncell + 32 * kSortWarps - 1) / (32 * kSortWarps), kSortWarps * 32, 0, s>>>(
            b->cell_start, b->members, b->ncell, gate);
    BPerm p;
    p.members = b->members;
    p.pos = b->pos[b->cur];
    p.t_pos = b->t_pos;
    p.vel = b->vel;
    p.t_vel = b->t_vel;
    p.accel = b->accel;
    p.t_accel = b->t_accel;
    p.image = b->image;
    p.t_image = b->t_image;
    p.tag = b->tag;
    p.t_tag = b->t_tag;
    p.sys = b->sys;
    p.t_sys = b->t_sys;
    p.cell_of = b->cell_of;
    p.t_cell = b->t_cell;
    p.N = N;
    k_b_gather<<<nblk(N), 256, 0, s>>>(p, gate);
    k_b_back<<<nblk(N), 256, 0, s>>>(p, gate);
    k_b_fixed<<<nblk(N), 256, 0, s>>>(b->pos[b->cur], b->sys, N, b->info, b->fix[b->cur], b->fix_build, gate);
    k_b_nlist<<<(N + 127) / 128, 128, 0, s>>>(b->pos[b->cur], b->fix[b->cur], b->sys, N, b->info, b->cell_start,
                                              b->cell_of, b->counts, b->nbrs, b->max_nn, b->flags + 3, gate);
    k_b_finish<<<1, 1, 0, s>>>(b->flags, gate);
    AZP_CHECK_LAUNCH("b_rebuild");
    b->launches += 12;
    return AZP_OK;
}

BStep b_args(azp_batch* b)
{
    BStep a{};
    a.pos = b->pos[b->cur];
    a.pos_next = b->pos[b->cur ^ 1];
    a.fix = b->fix[b->cur];
    a.fix_next = b->fix[b->cur ^ 1];
    a.fix_build = b->fix_build;
    a.vel = b->vel;
    a.accel = b->accel;
    a.image = b->image;
    a.tag = b->tag;
    a.sys = b->sys;
    a.info = b->info;
    a.N = b->N;
    a.counts = b->counts;
    a.nbrs = b->nbrs;
    a.max_nn = b->max_nn;
    a.dt = b->dt;
    a.kT = b->kT;
    a.gamma = b->gamma;
    a.noise = std::sqrt(6.0 * b->gamma * b->kT / b->dt);
    a.noiseless = b->noiseless;
    a.flow = b->flow;
    a.d_ts = b->d_ts;
    a.d_ts_rw = b->d_ts;
    a.flags = b->flags;
    const double half = 0.5 * b->r_buff;
    a.disp_thresh2 = (float)(half * half * (1.0 - 1e-5));
    a.tpp = b->tpp;
    a.block = b->block;
    return a;
}

int b_step(azp_batch* b, int next, cudaStream_t s, int set_cond, cudaGraphConditionalHandle h)
{
    BStep a = b_args(b);
    a.next = next;
    a.set_cond = set_cond;
    a.next_cond = h;
    b->launches += 1;
    return launch_b_step_kind(b->kind, b->precision, a, s);
}

int b_build_graph(azp_batch* b, int cur0, cudaGraphExec_t* out)
{
    cudaGraph_t g = nullptr;
    AZP_CUDA_TRY(cudaGraphCreate(&g, 0));
    cudaGraphConditionalHandle h[2];
    for (int k = 0; k < 2; ++k) AZP_CUDA_TRY(cudaGraphConditionalHandleCreate(&h[k], g, 0, cudaGraphCondAssignDefault));
    const int saved = b->cur;
    const uint64_t saved_l = b->launches;
    b->cur = cur0;
    cudaStream_t s = b->gstream;
    int st = AZP_OK;
    cudaGraphNode_t prev = nullptr;
    AZP_CUDA_TRY(cudaStreamBeginCaptureToGraph(s, g, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
    k_b_arm<<<1, 1, 0, s>>>(b->flags, h[0]);
    cudaGraph_t tmp = nullptr;
    AZP_CUDA_TRY(cudaStreamEndCapture(s, &tmp));
    {
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
        AZP_CUDA_TRY(cudaStreamBeginCaptureToGraph(s, cp.conditional.phGraph_out[0], nullptr, nullptr, 0,
                                                   cudaStreamCaptureModeThreadLocal));
        st = b_rebuild(b, s, nullptr);
        AZP_CUDA_TRY(cudaStreamEndCapture(s, &tmp));
        if (st) break;
        AZP_CUDA_TRY(cudaStreamBeginCaptureToGraph(s, g, &cnode, nullptr, 1, cudaStreamCaptureModeThreadLocal));
        st = b_step(b, 1, s, k == 0 ? 1 : 0, k == 0 ? h[1] : 0);
        AZP_CUDA_TRY(cudaStreamEndCapture(s, &tmp));
        if (st) break;
        size_t nd = 0;
        AZP_CUDA_TRY(cudaGraphNodeGetDependentNodes(cnode, nullptr, nullptr, &nd));
        std::vector<cudaGraphNode_t> deps(nd);
        AZP_CUDA_TRY(cudaGraphNodeGetDependentNodes(cnode, deps.data(), nullptr, &nd));
        if (nd != 1) {
            st = AZP_ERR_CUDA;
            break;
        }
        prev = deps[0];
        b->cur ^= 1;
    }
    b->cur = saved;
    b->launches = saved_l;
    if (st == AZP_OK) {
        const cudaError_t e = cudaGraphInstantiate(out, g, 0);
        if (e != cudaSuccess) st = record_cuda_error(e, "cudaGraphInstantiate (batch)");
    }
    cudaGraphDestroy(g);
    return st;
}

}  // namespace

extern "C" {

azp_batch* azp_batch_create(const azp_batch_config* c, int* status)
{
    auto fail = [&](int st, azp_batch* b) -> azp_batch* {
        if (status) *status = st;
        if (b) {
            b_free(b);
            delete b;
        }
        return nullptr;
    };
    if (!c || c->nsys == 0 || c->nsys > 65535 || !c->N || !c->L || !c->pair_params || !c->r_cut || !c->seeds)
        return fail(AZP_ERR_INVALID, nullptr);
    if (c->precision != AZP_FP64 && c->precision != AZP_FP32) return fail(AZP_ERR_INVALID, nullptr);
    if (c->pair_kind < 0 || c->pair_kind >= AZP_PAIR_NUM_KINDS || !(c->dt > 0.0)) return fail(AZP_ERR_INVALID, nullptr);
    azp_batch* b = new (std::nothrow) azp_batch();
    if (!b) return fail(AZP_ERR_INVALID, nullptr);
    b->S = c->nsys;
    b->precision = c->precision;
    b->kind = c->pair_kind;
    b->dt = c->dt;
    b->kT = c->kT;
    b->gamma = c->gamma;
    b->r_buff = c->r_buff;
    b->noiseless = c->noiseless;
    b->flow = make_flow(c->flow);
    const char* env_tpp = std::getenv("AZP_TPP");
    b->tpp = env_tpp ? std::atoi(env_tpp) : 1;
    if (!(b->tpp == 1 || b->tpp == 2 || b->tpp == 4 || b->tpp == 8 || b->tpp == 16 || b->tpp == 32)) b->tpp = 1;
    const char* env_graph = std::getenv("AZP_GRAPHS");
    b->use_graphs = !(env_graph && env_graph[0] == '0');
    b->n_of.assign(c->N, c->N + c->nsys);
    b->off.assign(c->nsys + 1, 0);
    for (uint32_t r = 0; r < c->nsys; ++r) b->off[r + 1] = b->off[r] + c->N[r];
    b->N = b->off[c->nsys];
    std::vector<SysInfo> info(c->nsys);
    uint32_t cell_off = 0;
    for (uint32_t r = 0; r < c->nsys; ++r) {
        SysInfo& si = info[r];
        azp_box box;
        for (int d = 0; d < 3; ++d) box.L[d] = c->L[3 * r + d];
        const double rc = c->r_cut[r];
        ListCut cut;
        double rmax = 0.0;
        make_list_cuts(&rc, 1, c->r_buff, box, &cut, &rmax);
        for (int d = 0; d < 3; ++d) {
            if (!(box.L[d] > 0.0)) return fail(AZP_ERR_INVALID, b);
            if (box.L[d] < 2.0 * rmax) return fail(AZP_ERR_BOX_TOO_SMALL, b);
            si.L[d] = box.L[d];
            si.Linv[d] = 1.0 / box.L[d];
            si.lo[d] = -0.5 * box.L[d];
            si.hi[d] = 0.5 * box.L[d];
            si.fscale[d] = si.Linv[d] * 4294967296.0;
            si.sfix[d] = (float)(box.L[d] * 2.3283064365386963e-10);
        }
        si.list_lo = cut.lo;
        si.list_hi = cut.hi;
        si.rlistsq = cut.rlistsq;
        const CellGrid g = make_grid(box, rmax);
        si.cell_off = cell_off;
        for (int d = 0; d < 3; ++d) {
            si.dim[d] = g.dim[d];
            si.reach[d] = g.reach[d];
            si.cscale[d] = g.scale[d];
        }
        cell_off += g.ncell;
        si.seed = c->seeds[r];
        const double zero = 0.0;
        int st = AZP_OK;
        double rec[PAIR_TBL];
        st = build_pair_table(c->pair_kind, c->pair_params + (size_t)pair_record_doubles(c->pair_kind) * r, &rc, &zero,
                              c->shift_mode, 1, rec);
        if (st) return fail(st, b);
        for (int k = 0; k < PAIR_TBL; ++k) si.rec[k] = rec[k];
        // the evaluator subtracts the shift itself in the single-system kernel; here fold it
        si.rcutsq = rec[PAIR_REC];
    }
    b->ncell = cell_off;
    const uint32_t N = b->N;
    int st = AZP_OK;
#define BALLOC(p, n)             \
    do {                         \
        st = balloc(&(p), (n));  \
        if (st) return fail(st, b); \
    } while (0)
    BALLOC(b->info, c->nsys);
    BALLOC(b->sys_off, c->nsys + 1);
    BALLOC(b->pos[0], N);
    BALLOC(b->pos[1], N);
    BALLOC(b->fix[0], N);
    BALLOC(b->fix[1], N);
    BALLOC(b->fix_build, N);
    BALLOC(b->vel, N);
    BALLOC(b->accel, (size_t)3 * N);
    BALLOC(b->image, (size_t)3 * N);
    BALLOC(b->tag, N);
    BALLOC(b->sys, N);
    BALLOC(b->t_pos, N);
    BALLOC(b->t_vel, N);
    BALLOC(b->t_accel, (size_t)3 * N);
    BALLOC(b->t_image, (size_t)3 * N);
    BALLOC(b->t_tag, N);
    BALLOC(b->t_sys, N);
    BALLOC(b->t_cell, N);
    BALLOC(b->cell_of, N);
    BALLOC(b->slot, N);
    BALLOC(b->members, N);
    BALLOC(b->rindex, N);
    BALLOC(b->cell_count, b->ncell);
    BALLOC(b->cell_start, (size_t)b->ncell + 1);
    BALLOC(b->scan_tmp, scan_tmp_words(b->ncell));
    BALLOC(b->counts, N);
    BALLOC(b->nbrs, (size_t)N * b->max_nn);
    BALLOC(b->flags, 8);
    BALLOC(b->d_ts, 1);
#undef BALLOC
    if (cudaMemcpy(b->info, info.data(), sizeof(SysInfo) * c->nsys, cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(b->sys_off, b->off.data(), sizeof(uint32_t) * (c->nsys + 1), cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemset(b->flags, 0, sizeof(uint32_t) * 8) != cudaSuccess ||
        cudaStreamCreateWithFlags(&b->gstream, cudaStreamNonBlocking) != cudaSuccess)
        return fail(record_cuda_error(cudaGetLastError(), "batch set-up"), b);
    if (status) *status = AZP_OK;
    return b;
}

void azp_batch_destroy(azp_batch* b)
{
    if (!b) return;
    b_free(b);
    delete b;
}

int azp_batch_set_state(azp_batch* b, const double* pos, const double* vel, const double* accel, const int32_t* image,
                        uint64_t timestep, void* stream)
{
    if (!b || !pos || !vel) return AZP_ERR_INVALID;
    cudaStream_t s = as_stream(stream);
    const uint32_t N = b->N;
    std::vector<uint32_t> sys_of(N), tag_of(N);
    for (uint32_t r = 0; r < b->S; ++r)
        for (uint32_t k = 0; k < b->n_of[r]; ++k) {
            sys_of[b->off[r] + k] = r;
            tag_of[b->off[r] + k] = k;
        }
    double *dp, *dv, *da = nullptr;
    int* di = nullptr;
    uint32_t *ds, *dt;
    AZP_CUDA_TRY(cudaMalloc(&dp, sizeof(double) * 4 * N));
    AZP_CUDA_TRY(cudaMalloc(&dv, sizeof(double) * 4 * N));
    AZP_CUDA_TRY(cudaMalloc(&ds, sizeof(uint32_t) * N));
    AZP_CUDA_TRY(cudaMalloc(&dt, sizeof(uint32_t) * N));
    AZP_CUDA_TRY(cudaMemcpyAsync(dp, pos, sizeof(double) * 4 * N, cudaMemcpyHostToDevice, s));
    AZP_CUDA_TRY(cudaMemcpyAsync(dv, vel, sizeof(double) * 4 * N, cudaMemcpyHostToDevice, s));
    AZP_CUDA_TRY(cudaMemcpyAsync(ds, sys_of.data(), sizeof(uint32_t) * N, cudaMemcpyHostToDevice, s));
    AZP_CUDA_TRY(cudaMemcpyAsync(dt, tag_of.data(), sizeof(uint32_t) * N, cudaMemcpyHostToDevice, s));
    if (accel) {
        AZP_CUDA_TRY(cudaMalloc(&da, sizeof(double) * 3 * N));
        AZP_CUDA_TRY(cudaMemcpyAsync(da, accel, sizeof(double) * 3 * N, cudaMemcpyHostToDevice, s));
    }
    if (image) {
        AZP_CUDA_TRY(cudaMalloc(&di, sizeof(int) * 3 * N));
        AZP_CUDA_TRY(cudaMemcpyAsync(di, image, sizeof(int) * 3 * N, cudaMemcpyHostToDevice, s));
    }
    b->cur = 0;
    k_b_load<<<nblk(N), 256, 0, s>>>(dp, dv, da, di, ds, dt, N, b->pos[0], b->vel, b->accel, b->image, b->tag, b->sys,
                                     b->rindex);
    const unsigned long long ts = timestep;
    AZP_CUDA_TRY(cudaMemcpyAsync(b->d_ts, &ts, sizeof(ts), cudaMemcpyHostToDevice, s));
    AZP_CUDA_TRY(cudaMemsetAsync(b->flags, 0, sizeof(uint32_t) * 8, s));
    int st = AZP_OK;
    for (int attempt = 0; attempt < 4; ++attempt) {
        AZP_CUDA_TRY(cudaMemsetAsync(b->flags + 3, 0, sizeof(uint32_t), s));
        st = b_rebuild(b, s, nullptr);
        if (st) break;
        uint32_t need = 0;
        AZP_CUDA_TRY(cudaMemcpyAsync(&need, b->flags + 3, sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
        AZP_CUDA_TRY(cudaStreamSynchronize(s));
        if (need <= b->max_nn) break;
        cudaFree(b->nbrs);
        b->max_nn = (uint32_t)std::ceil(need * 1.3) + 8;
        st = balloc(&b->nbrs, (size_t)N * b->max_nn);
        if (st) break;
        b_free_graphs(b);
    }
    AZP_CUDA_TRY(cudaStreamSynchronize(s));
    cudaFree(dp);
    cudaFree(dv);
    cudaFree(ds);
    cudaFree(dt);
    cudaFree(da);
    cudaFree(di);
    b->have_state = (st == AZP_OK);
    return st;
}

int azp_batch_get_state(azp_batch* b, double* pos, double* vel, double* accel, int32_t* image, void* stream)
{
    if (!b || !b->have_state || !pos || !vel || !accel || !image) return AZP_ERR_INVALID;
    cudaStream_t s = as_stream(stream);
    const uint32_t N = b->N;
    double *dp, *dv, *da;
    int* di;
    AZP_CUDA_TRY(cudaMalloc(&dp, sizeof(double) * 4 * N));
    AZP_CUDA_TRY(cudaMalloc(&dv, sizeof(double) * 4 * N));
    AZP_CUDA_TRY(cudaMalloc(&da, sizeof(double) * 3 * N));
    AZP_CUDA_TRY(cudaMalloc(&di, sizeof(int) * 3 * N));
    k_b_store<<<nblk(N), 256, 0, s>>>(b->pos[b->cur], b->vel, b->accel, b->image, b->tag, b->sys, b->sys_off, N, dp, dv,
                                      da, di);
    AZP_CUDA_TRY(cudaMemcpyAsync(pos, dp, sizeof(double) * 4 * N, cudaMemcpyDeviceToHost, s));
    AZP_CUDA_TRY(cudaMemcpyAsync(vel, dv, sizeof(double) * 4 * N, cudaMemcpyDeviceToHost, s));
    AZP_CUDA_TRY(cudaMemcpyAsync(accel, da, sizeof(double) * 3 * N, cudaMemcpyDeviceToHost, s));
    AZP_CUDA_TRY(cudaMemcpyAsync(image, di, sizeof(int) * 3 * N, cudaMemcpyDeviceToHost, s));
    AZP_CUDA_TRY(cudaStreamSynchronize(s));
    cudaFree(dp);
    cudaFree(dv);
    cudaFree(da);
    cudaFree(di);
    return AZP_OK;
}

int azp_batch_run(azp_batch* b, uint64_t steps, void* stream)
{
    if (!b || !b->have_state) return AZP_ERR_INVALID;
    b->launches = 0;
    if (steps == 0) return AZP_OK;
    cudaStream_t s = as_stream(stream);
    const uint32_t N = b->N;
    const double half = 0.5 * b->r_buff;
    k_b_step1<<<nblk(N), 256, 0, s>>>(b->pos[b->cur], b->fix[b->cur], b->fix_build, b->vel, b->accel, b->image, b->sys,
                                      b->info, N, b->dt, (float)(half * half * (1.0 - 1e-5)), b->flags);
    AZP_CHECK_LAUNCH("k_b_step1");
    b->launches += 1;
    uint64_t mid = steps - 1;
    int st = AZP_OK;
    if (b->use_graphs && mid >= 2) {
        for (int p = 0; p < 2; ++p)
            if (!b->gexec[p]) {
                st = b_build_graph(b, p, &b->gexec[p]);
                if (st) return st;
            }
        while (mid >= 2) {
            AZP_CUDA_TRY(cudaGraphLaunch(b->gexec[b->cur], s));
            b->launches += 3;
            mid -= 2;
        }
    }
    while (mid > 0) {
        st = b_rebuild(b, s, b->flags);
        if (st) return st;
        st = b_step(b, 1, s, 0, 0);
        if (st) return st;
        b->cur ^= 1;
        --mid;
    }
    st = b_rebuild(b, s, b->flags);
    if (st) return st;
    return b_step(b, 0, s, 0, 0);
}

int azp_batch_error(azp_batch* b, uint32_t* err_word, uint32_t* n_builds, void* stream)
{
    if (!b || !err_word) return AZP_ERR_INVALID;
    cudaStream_t s = as_stream(stream);
    uint32_t f[8];
    AZP_CUDA_TRY(cudaMemcpyAsync(f, b->flags, sizeof(f), cudaMemcpyDeviceToHost, s));
    AZP_CUDA_TRY(cudaStreamSynchronize(s));
    uint32_t e = f[1];
    if (f[3] > b->max_nn) e |= AZP_EBIT_NLIST_OVERFLOW;
    *err_word = e;
    if (n_builds) *n_builds = f[2];
    return AZP_OK;
}

int azp_batch_set_block(azp_batch* b, int block)
{
    if (!b || !(block == 64 || block == 128 || block == 256 || block == 512)) return AZP_ERR_INVALID;
    if (b->block != block) b_free_graphs(b);
    b->block = block;
    return AZP_OK;
}

int azp_batch_set_tpp(azp_batch* b, int tpp)
{
    if (!b || !(tpp == 1 || tpp == 2 || tpp == 4 || tpp == 8 || tpp == 16 || tpp == 32)) return AZP_ERR_INVALID;
    if (b->tpp != tpp) b_free_graphs(b);
    b->tpp = tpp;
    return AZP_OK;
}

uint64_t azp_batch_last_launches(const azp_batch* b) { return b ? b->launches : 0; }

}  // extern "C"
