// nlist.cu -- cell list and full neighbour list on the device, and the
// standalone azp_nlist object of the C ABI (replaces HOOMD's
// NeighborListGPUBinned + CellListGPU behind hoomd.md.nlist.Cell).
//
// Membership contract (oracle/azp_oracle.cpp, orc_nlist_*): j != i is listed for
// i when r_cut(ti, tj) > 0, |min_image(x_i - x_j)|^2 < (r_cut + r_buff)^2 in FP64
// with every product and sum rounded separately, and j is not excluded.
// The FP64 test runs only for candidates whose FP32 fixed-point distance falls in
// a narrow band around r_list; everything else is decided in FP32 with a margin
// larger than its worst-case error, so the sets are bit-exact.
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <new>
#include <vector>

#include "celllist.cuh"
#include "fixed64.cuh"
#include "nlist_impl.cuh"
#include "scan.cuh"

namespace azp
{
// ---------------------------------------------------------------- host helpers
CellGrid make_grid(const azp_box& box, double rlist_max, int sub)
{
    CellGrid g;
    g.ncell = 1;
    // cell width >= r_list / sub, the stencil reaching sub cells each way;
    // widened if the grid would exceed 2^24 cells
    if (sub < 1) sub = 1;
    double w = rlist_max / sub;
    if (w > 0.0) {
        while ((box.L[0] / w) * (box.L[1] / w) * (box.L[2] / w) > 16777216.0) w *= 1.25;
    }
    for (int d = 0; d < 3; ++d) {
        int n = w > 0.0 ? (int)std::floor(box.L[d] / w) : 1;
        int reach = sub;
        if (n < 2 * reach + 1) {
            // too few cells for distinct images along this axis: one cell
            n = 1;
            reach = 0;
        }
        g.dim[d] = n;
        g.reach[d] = reach;
        g.lo[d] = -0.5 * box.L[d];
        g.scale[d] = (double)n / box.L[d];
        g.ncell *= (uint32_t)n;
    }
    return g;
}

int grid_subdivision(double rlist_max, double rlist_min)
{
    static const int forced = [] {
        const char* e = std::getenv("AZP_NL_SUB");
        const int v = e ? std::atoi(e) : 0;
        return v >= 1 && v <= 4 ? v : 0;
    }();
    if (forced) return forced;
    // cutoffs far apart (the colloid mixture: 10.4 against 3.4): cells of the
    // smallest list radius, so that the short-ranged pairs scan fewer candidates
    // (measured there: 985 -> 1,165 timesteps/s at 3); one radius: r_list cells
    if (!(rlist_min > 0.0) || !(rlist_max > rlist_min)) return 1;
    return std::max(1, std::min(3, (int)(rlist_max / rlist_min)));
}

void make_list_cuts(const double* r_cut, uint32_t ntypes, double r_buff, const azp_box& box, ListCut* out,
                    double* rlist_max, double* rlist_min)
{
    double rmax = 0.0, rmin = 1e300;
    for (uint32_t t = 0; t < ntypes * ntypes; ++t) {
        if (r_cut[t] > 0.0) {
            const double rl = r_cut[t] + r_buff;
            rmax = std::max(rmax, rl);
            rmin = std::min(rmin, rl);
        }
    }
    const double Lmax = std::max(box.L[0], std::max(box.L[1], box.L[2]));
    // worst-case relative error of the FP32 fixed-point rsq: float rounding of
    // three components and their squares (< 1e-6) plus the fixed-point rounding
    // of both positions (L 2^-33 each) against the smallest list radius.
    double delta = 4e-6;
    if (rmax > 0.0) delta = std::max(delta, 16.0 * Lmax * 2.3283064365386963e-10 / rmin);
    for (uint32_t t = 0; t < ntypes * ntypes; ++t) {
        ListCut c;
        if (r_cut[t] > 0.0) {
            const double rl = r_cut[t] + r_buff;
            c.rlistsq = rl * rl;
            c.lo = std::nextafter((float)(c.rlistsq * (1.0 - delta)), 0.0f);
            c.hi = std::nextafter((float)(c.rlistsq * (1.0 + delta)), 1e30f);
        } else {
            c.rlistsq = 0.0;
            c.lo = -1.0f;
            c.hi = -1.0f;  // rsq_f >= hi always: never listed
        }
        c.pad = 0.0f;
        out[t] = c;
    }
    *rlist_max = rmax;
    if (rlist_min) *rlist_min = rmax > 0.0 ? rmin : 0.0;
}

// ---------------------------------------------------------------- kernels
__global__ void k_to_fixed(const double4_32a* __restrict__ pos, uint4* __restrict__ fixed, uint32_t N, double lx,
                           double ly, double lz)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= N) return;
    const double4_32a p = pos[i];
    uint4 f;
    f.x = to_fixed(p.x, lx);
    f.y = to_fixed(p.y, ly);
    f.z = to_fixed(p.z, lz);
    f.w = type_of(p.w);
    fixed[i] = f;
}

__device__ __forceinline__ int cell_coord(double x, double lo, double scale, int dim)
{
    int c = (int)floor((x - lo) * scale);
    if (c < 0) c += dim;
    if (c >= dim) c -= dim;
    return min(max(c, 0), dim - 1);
}

__global__ void k_cell_assign(const double4_32a* __restrict__ pos, uint32_t N, CellGrid g, uint32_t* __restrict__ cell_of,
                              uint32_t* __restrict__ slot, uint32_t* __restrict__ cell_count,
                              const uint32_t* __restrict__ gate)
{
    if (gated_off(gate)) return;
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= N) return;
    const double4_32a p = pos[i];
    const int cx = cell_coord(p.x, g.lo[0], g.scale[0], g.dim[0]);
    const int cy = cell_coord(p.y, g.lo[1], g.scale[1], g.dim[1]);
    const int cz = cell_coord(p.z, g.lo[2], g.scale[2], g.dim[2]);
    const uint32_t c = ((uint32_t)cz * g.dim[1] + cy) * g.dim[0] + cx;
    cell_of[i] = c;
    slot[i] = atomicAdd(&cell_count[c], 1u);
}

__global__ void k_cell_scatter(const uint32_t* __restrict__ cell_of, const uint32_t* __restrict__ slot,
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
__global__ void __launch_bounds__(kSortWarps * 32) k_cell_sort(const uint32_t* __restrict__ cell_start,
                                                               uint32_t* __restrict__ members, uint32_t ncell,
                                                               const uint32_t* __restrict__ gate)
{
    if (gated_off(gate)) return;
    __shared__ uint32_t s_rows[kSortWarps][kMaxSortedCell];
    sort_cells_warp(cell_start, members, ncell, s_rows[threadIdx.x >> 5]);
}

// crowded grids: a warp per cell
__global__ void __launch_bounds__(kSortWarps * 32) k_cell_sort_crowded(const uint32_t* __restrict__ cell_start,
                                                                       uint32_t* __restrict__ members, uint32_t ncell,
                                                                       const uint32_t* __restrict__ gate)
{
    if (gated_off(gate)) return;
    __shared__ uint32_t s_rows[kSortWarps][kMaxSortedCell];
    sort_cell_per_warp(cell_start, members, ncell, s_rows[threadIdx.x >> 5]);
}

struct BoxArgs {
    double L[3], Linv[3];
    double l64[3];  // L * 2^-64 (64-bit fixed-point unit)
    float sfix[3];  // L * 2^-32 (fixed-point unit)
};

inline BoxArgs box_args(const azp_box& b)
{
    BoxArgs a;
    for (int d = 0; d < 3; ++d) {
        a.L[d] = b.L[d];
        a.Linv[d] = 1.0 / b.L[d];
        a.l64[d] = b.L[d] * 5.421010862427522e-20;
        a.sfix[d] = (float)(b.L[d] * 2.3283064365386963e-10);
    }
    return a;
}

// FP64 position of particle i from its 64-bit fixed-point words (fixed64.cuh)
__device__ __forceinline__ double4_32a fx_position(const uint4* __restrict__ hi, const uint4* __restrict__ lo,
                                                   uint32_t i, const BoxArgs& bx)
{
    const uint4 h = hi[i], l = lo[i];
    return make_double4_32a(fx_to_double(fx_join(h.x, l.x), bx.l64[0]), fx_to_double(fx_join(h.y, l.y), bx.l64[1]),
                            fx_to_double(fx_join(h.z, l.z), bx.l64[2]), 0.0);
}

// cell of each particle from the high words of its 64-bit fixed position:
// [-2^31, 2^31) maps linearly onto [0, dim) in integer arithmetic
__global__ void k_cell_assign_fx(const uint4* __restrict__ fixed, uint32_t N, CellGrid g,
                                 uint32_t* __restrict__ cell_of, uint32_t* __restrict__ slot,
                                 uint32_t* __restrict__ cell_count, const uint32_t* __restrict__ gate)
{
    if (gated_off(gate)) return;
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= N) return;
    const uint4 f = fixed[i];
    const uint32_t cx = (uint32_t)(((uint64_t)(f.x ^ 0x80000000u) * (uint32_t)g.dim[0]) >> 32);
    const uint32_t cy = (uint32_t)(((uint64_t)(f.y ^ 0x80000000u) * (uint32_t)g.dim[1]) >> 32);
    const uint32_t cz = (uint32_t)(((uint64_t)(f.z ^ 0x80000000u) * (uint32_t)g.dim[2]) >> 32);
    const uint32_t c = (cz * (uint32_t)g.dim[1] + cy) * (uint32_t)g.dim[0] + cx;
    cell_of[i] = c;
    slot[i] = atomicAdd(&cell_count[c], 1u);
}

constexpr uint32_t MAX_LIST_TYPES = 16;  // ntypes^2 <= 256 thresholds in shared memory
constexpr int NLIST_BLOCK = 128;
static_assert(TILE_P % NLIST_BLOCK == 0, "a list-build block lies inside one tile block");
constexpr uint32_t NL_EX_REG = 4;  // exclusion keys of a particle held in registers
// Candidates in the FP32 band around r_list are appended with this mark and
// decided exactly in the compaction pass: the scan loop then holds no call and
// no FP64 state (measured at N = 1M: 40 registers instead of 64, the build 20 %
// faster, the same sets).
constexpr uint32_t NL_BAND = 0x80000000u;
constexpr uint32_t NL_MAX_N = NL_BAND - 1;  // particle indices stay below the mark

// The oracle's exact FP64 decision for a candidate inside the ambiguous band
// of the FP32 prefilter. Out of line: a candidate lands in the band about once
// per million.
__device__ __noinline__ bool nl_exact_within(uint32_t i, uint32_t j, double rlistsq, const BoxArgs& bx,
                                             const double4_32a* __restrict__ pos, const uint4* __restrict__ fixed,
                                             const uint4* __restrict__ lo)
{
    const double4_32a a = lo ? fx_position(fixed, lo, i, bx) : pos[i];
    const double4_32a b = lo ? fx_position(fixed, lo, j, bx) : pos[j];
    const double vx = min_image1(a.x - b.x, bx.L[0], bx.Linv[0]);
    const double vy = min_image1(a.y - b.y, bx.L[1], bx.Linv[1]);
    const double vz = min_image1(a.z - b.z, bx.L[2], bx.Linv[2]);
    return rsq_exact(vx, vy, vz) < rlistsq;
}

// exclusion keys of a particle beyond the NL_EX_REG held in registers
__device__ __noinline__ bool nl_excluded_tail(uint32_t i, uint32_t kj, uint32_t nex, uint32_t N,
                                              const uint32_t* __restrict__ ex_keys)
{
    for (uint32_t e = NL_EX_REG; e < nex; ++e)
        if (ex_keys[(size_t)e * N + i] == kj) return true;
    return false;
}

// Full list, one thread per particle. For every (y, z) offset row of the 3x3x3
// cell stencil, the x-neighbour cells cx-1, cx, cx+1 are consecutive cell
// indices, so their particles are one contiguous slot range (members[s], or s
// itself when the particles are stored in cell order); at the x faces the
// wrapped cell is a second range. The scan per candidate is one 16-byte gather,
// the integer minimum image and the FP32 prefilter; ONE_TYPE keeps the
// thresholds of a single-type system in registers.
template<bool ONE_TYPE, bool SORTED>
__global__ void __launch_bounds__(NLIST_BLOCK)
    k_nlist_build_threads(const double4_32a* __restrict__ pos, const uint4* __restrict__ fixed, uint32_t N, BoxArgs bx,
                          CellGrid g, const uint32_t* __restrict__ cell_start, const uint32_t* __restrict__ members,
                          const uint32_t* __restrict__ cell_of, const ListCut* __restrict__ cuts, uint32_t ntypes,
                          const uint32_t* __restrict__ ex_n, const uint32_t* __restrict__ ex_keys,
                          const uint32_t* __restrict__ keys, uint32_t* __restrict__ counts,
                          uint32_t* __restrict__ nbrs, uint32_t max_nn, uint32_t* __restrict__ flags,
                          const uint32_t* __restrict__ gate, const uint4* __restrict__ lo,
                          const uint32_t* __restrict__ tile)
{
    if (gated_off(gate)) return;
    __shared__ ListCut s_cut[MAX_LIST_TYPES * MAX_LIST_TYPES];
    // the tile record of this block's particles (NLIST_BLOCK divides TILE_P)
    __shared__ uint32_t s_trec[TILE_REC];
    const uint32_t nt2 = ntypes * ntypes;
    for (uint32_t t = threadIdx.x; t < nt2; t += blockDim.x) s_cut[t] = cuts[t];
    if (tile && threadIdx.x < TILE_REC)
        s_trec[threadIdx.x] = tile[(size_t)(blockIdx.x * blockDim.x / TILE_P) * TILE_REC + threadIdx.x];
    __syncthreads();

    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= N) return;
    const uint4 fi = __ldg(fixed + i);
    const uint32_t row = fi.w * ntypes;
    const ListCut cut0 = s_cut[0];
    const uint32_t nex = ex_n ? __ldg(ex_n + i) : 0u;
    const uint32_t cc = __ldg(cell_of + i);
    const int dx = g.dim[0], dy = g.dim[1], dz = g.dim[2];
    const int cx = (int)(cc % (uint32_t)dx);
    const int cy = (int)((cc / (uint32_t)dx) % (uint32_t)dy);
    const int cz = (int)(cc / ((uint32_t)dx * (uint32_t)dy));
    // the x-cells cx - reach .. cx + reach: one contiguous range inside the row,
    // and the wrapped part at an x face, contiguous too ([wb, we]; empty: wb > we)
    int x0 = cx - g.reach[0], x1 = cx + g.reach[0], wb = 1, we = 0;
    if (x0 < 0) {
        wb = dx + x0;
        we = dx - 1;
        x0 = 0;
    }
    if (x1 >= dx) {
        wb = 0;
        we = x1 - dx;
        x1 = dx - 1;
    }
    uint32_t ex[NL_EX_REG];
#pragma unroll
    for (uint32_t e = 0; e < NL_EX_REG; ++e) ex[e] = e < nex ? __ldg(ex_keys + (size_t)e * N + i) : 0xffffffffu;
    uint32_t n = 0;
    // one candidate: the integer minimum image, the FP32 prefilter, the append
    const auto test = [&](uint32_t j, const uint4& fj) {
        const float ddx = (float)(int32_t)(fi.x - fj.x) * bx.sfix[0];
        const float ddy = (float)(int32_t)(fi.y - fj.y) * bx.sfix[1];
        const float ddz = (float)(int32_t)(fi.z - fj.z) * bx.sfix[2];
        const float rs = ddx * ddx + ddy * ddy + ddz * ddz;
        const ListCut cut = ONE_TYPE ? cut0 : s_cut[row + fj.w];
        // within r_list or in the band around it: appended (i itself, its
        // excluded partners and the band candidates, marked, too; the pass
        // below takes out what does not belong)
        if (rs < cut.hi) {
            if (n < max_nn) nbrs[(size_t)n * N + i] = rs < cut.lo ? j : (j | NL_BAND);
            ++n;
        }
    };
    for (int oz = -g.reach[2]; oz <= g.reach[2]; ++oz) {
        int nz = cz + oz;
        nz += (nz < 0) ? dz : 0;
        nz -= (nz >= dz) ? dz : 0;
        for (int oy = -g.reach[1]; oy <= g.reach[1]; ++oy) {
            int ny = cy + oy;
            ny += (ny < 0) ? dy : 0;
            ny -= (ny >= dy) ? dy : 0;
            const uint32_t rb = ((uint32_t)nz * dy + ny) * dx;
            for (int part = 0; part < 2; ++part) {
                uint32_t sb, se;
                if (part == 0) {
                    sb = __ldg(cell_start + rb + x0);
                    se = __ldg(cell_start + rb + x1 + 1);
                } else {
                    if (wb > we) break;
                    sb = __ldg(cell_start + rb + wb);
                    se = __ldg(cell_start + rb + we + 1);
                }
#pragma unroll 4
                for (uint32_t sl = sb; sl < se; ++sl) {
                    const uint32_t j = SORTED ? sl : __ldg(members + sl);
                    test(j, __ldg(fixed + j));
                }
            }
        }
    }
    // Compact the row in place: drop i itself and the excluded partners, keeping
    // the order. The warp-wide scan above stays a load, a test and an append; the
    // exclusion compares run once per listed entry here instead of on every
    // candidate iteration. Overflow is judged on the raw count, which bounds the
    // true one, so a row that lost entries to the capacity is always reported.
    const uint32_t stored = min(n, max_nn);
    uint32_t m = 0;
    for (uint32_t k = 0; k < stored; ++k) {
        uint32_t j = nbrs[(size_t)k * N + i];
        const bool marked = (j & NL_BAND) != 0u;
        bool drop = false;
        if (marked) {
            // a candidate in the band around r_list: the oracle's exact FP64 decision
            j &= ~NL_BAND;
            const ListCut cut = ONE_TYPE ? cut0 : s_cut[row + __ldg(fixed + j).w];
            drop = !nl_exact_within(i, j, cut.rlistsq, bx, pos, fixed, lo);
        }
        drop |= j == i;
        if (nex && !drop) {
            const uint32_t kj = keys ? __ldg(keys + j) : j;
#pragma unroll
            for (uint32_t e = 0; e < NL_EX_REG; ++e) drop |= ex[e] == kj;
            if (nex > NL_EX_REG) drop |= nl_excluded_tail(i, kj, nex, N, ex_keys);
        }
        if (!drop) {
            if (tile) nbrs[(size_t)m * N + i] = tile_encode(s_trec, j);
            else if (m != k || marked) nbrs[(size_t)m * N + i] = j;  // a kept band entry loses its mark
            ++m;
        }
    }
    counts[i] = n > max_nn ? n : m;
    if (n > max_nn) atomicMax(&flags[0], n);
}

// Block records of the shared-memory tiles: for every stencil row of the block's
// TILE_P particles, the range of particle indices that row's x-ranges cover
// (cx - 1 .. cx + 1 clipped to the row; the wrapped cell at an x face stays
// outside and is addressed globally), merged into disjoint ranges in increasing
// order with their offsets in the tile. A block whose ranges exceed TILE_CAP
// records (a row wrapping through a y or z face makes its range span most of the
// box) gets 0 ranges: its entries are all global.
__global__ void __launch_bounds__(TILE_P) k_tile_table(const uint32_t* __restrict__ cell_of,
                                                       const uint32_t* __restrict__ cell_start, CellGrid g, uint32_t N,
                                                       uint32_t* __restrict__ tab, const uint32_t* __restrict__ gate)
{
    if (gated_off(gate)) return;
    __shared__ uint32_t s_lo[TILE_MAX_RANGES], s_hi[TILE_MAX_RANGES];
    if (threadIdx.x < TILE_MAX_RANGES) {
        s_lo[threadIdx.x] = 0xffffffffu;
        s_hi[threadIdx.x] = 0u;
    }
    __syncthreads();
    const uint32_t i = blockIdx.x * TILE_P + threadIdx.x;
    if (i < N) {
        const uint32_t cc = __ldg(cell_of + i);
        const int dx = g.dim[0], dy = g.dim[1], dz = g.dim[2];
        const int cx = (int)(cc % (uint32_t)dx);
        const int cy = (int)((cc / (uint32_t)dx) % (uint32_t)dy);
        const int cz = (int)(cc / ((uint32_t)dx * (uint32_t)dy));
        const int x0 = max(cx - g.reach[0], 0), x1 = min(cx + g.reach[0], dx - 1);
        uint32_t r = 0;
        for (int oz = -g.reach[2]; oz <= g.reach[2]; ++oz) {
            int nz = cz + oz;
            nz += (nz < 0) ? dz : 0;
            nz -= (nz >= dz) ? dz : 0;
            for (int oy = -g.reach[1]; oy <= g.reach[1]; ++oy, ++r) {
                int ny = cy + oy;
                ny += (ny < 0) ? dy : 0;
                ny -= (ny >= dy) ? dy : 0;
                const uint32_t rb = ((uint32_t)nz * dy + ny) * dx;
                const uint32_t sb = __ldg(cell_start + rb + x0), se = __ldg(cell_start + rb + x1 + 1);
                if (se > sb) {
                    atomicMin(&s_lo[r], sb);
                    atomicMax(&s_hi[r], se);
                }
            }
        }
    }
    __syncthreads();
    if (threadIdx.x != 0) return;
    uint32_t lo[TILE_MAX_RANGES], hi[TILE_MAX_RANGES], n = 0;
    for (uint32_t r = 0; r < TILE_MAX_RANGES; ++r)
        if (s_hi[r] > s_lo[r]) {
            // insertion by begin
            uint32_t k = n++;
            while (k > 0 && lo[k - 1] > s_lo[r]) {
                lo[k] = lo[k - 1];
                hi[k] = hi[k - 1];
                --k;
            }
            lo[k] = s_lo[r];
            hi[k] = s_hi[r];
        }
    // merge overlapping or touching ranges
    uint32_t m = 0;
    for (uint32_t k = 0; k < n; ++k) {
        if (m > 0 && lo[k] <= hi[m - 1]) {
            hi[m - 1] = max(hi[m - 1], hi[k]);
        } else {
            lo[m] = lo[k];
            hi[m] = hi[k];
            ++m;
        }
    }
    uint32_t* t = tab + (size_t)blockIdx.x * TILE_REC;
    uint32_t total = 0;
    for (uint32_t k = 0; k < m; ++k) {
        t[2 + 3 * k] = lo[k];
        t[3 + 3 * k] = hi[k];
        t[4 + 3 * k] = total;
        total += hi[k] - lo[k];
    }
    t[0] = total <= TILE_CAP ? m : 0u;
    t[1] = total;
}

void launch_tile_table(const uint32_t* cell_of, const uint32_t* cell_start, const CellGrid& g, uint32_t N,
                       uint32_t* tab, const uint32_t* gate, cudaStream_t s)
{
    if (N == 0) return;
    k_tile_table<<<(N + TILE_P - 1) / TILE_P, TILE_P, 0, s>>>(cell_of, cell_start, g, N, tab, gate);
}

// ---------------------------------------------------------------- launch helpers
void launch_to_fixed(const double4_32a* pos, uint4* fixed, uint32_t N, const azp_box& box, cudaStream_t s)
{
    if (N == 0) return;
    k_to_fixed<<<(N + 255) / 256, 256, 0, s>>>(pos, fixed, N, 1.0 / box.L[0], 1.0 / box.L[1], 1.0 / box.L[2]);
}

void launch_cell_assign(const double4_32a* pos, uint32_t N, const CellGrid& g, uint32_t* cell_of, uint32_t* slot,
                        uint32_t* cell_count, cudaStream_t s, const uint32_t* gate)
{
    if (N == 0) return;
    k_cell_assign<<<(N + 255) / 256, 256, 0, s>>>(pos, N, g, cell_of, slot, cell_count, gate);
}

void launch_cell_scatter(const uint32_t* cell_of, const uint32_t* slot, const uint32_t* cell_start,
                         uint32_t* members, uint32_t N, uint32_t ncell, cudaStream_t s, const uint32_t* gate)
{
    if (N == 0) return;
    k_cell_scatter<<<(N + 255) / 256, 256, 0, s>>>(cell_of, slot, cell_start, members, N, gate);
    if (crowded_grid(N, ncell))
        k_cell_sort_crowded<<<(ncell + kSortWarps - 1) / kSortWarps, kSortWarps * 32, 0, s>>>(cell_start, members,
                                                                                            ncell, gate);
    else
        k_cell_sort<<<(ncell + 32 * kSortWarps - 1) / (32 * kSortWarps), kSortWarps * 32, 0, s>>>(cell_start, members,
                                                                                                  ncell, gate);
}

__global__ void k_to_fixed2(const double4_32a* __restrict__ pos, uint4* __restrict__ fa, uint4* __restrict__ fb,
                            uint32_t N, double lx, double ly, double lz, const uint32_t* __restrict__ gate)
{
    if (gated_off(gate)) return;
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= N) return;
    const double4_32a p = pos[i];
    uint4 f;
    f.x = to_fixed(p.x, lx);
    f.y = to_fixed(p.y, ly);
    f.z = to_fixed(p.z, lz);
    f.w = type_of(p.w);
    fa[i] = f;
    if (fb) fb[i] = f;
}

void launch_to_fixed2(const double4_32a* pos, uint4* a, uint4* b, uint32_t N, const azp_box& box, cudaStream_t s,
                      const uint32_t* gate)
{
    if (N == 0) return;
    k_to_fixed2<<<(N + 255) / 256, 256, 0, s>>>(pos, a, b, N, 1.0 / box.L[0], 1.0 / box.L[1], 1.0 / box.L[2], gate);
}

void launch_nlist_build(const double4_32a* pos, const uint4* fixed, uint32_t N, const azp_box& box, const CellGrid& g,
                        const uint32_t* cell_start, const uint32_t* members, const uint32_t* cell_of,
                        const ListCut* cuts, uint32_t ntypes, const uint32_t* ex_n, const uint32_t* ex_keys,
                        uint32_t ex_width, const uint32_t* keys, uint32_t* counts, uint32_t* nbrs,
                        uint32_t max_nn, uint32_t* flags, const uint32_t* gate, cudaStream_t s, const uint4* lo,
                        double rlist_min, const uint32_t* tile)
{
    (void)ex_width;
    (void)rlist_min;
    if (N == 0) return;
    const BoxArgs bx = box_args(box);
    const uint32_t blocks = (N + NLIST_BLOCK - 1) / NLIST_BLOCK;
#define AZP_NL_ARGS                                                                                              \
    pos, fixed, N, bx, g, cell_start, members, cell_of, cuts, ntypes, ex_n, ex_keys, keys, counts, nbrs, max_nn, \
        flags, gate, lo, members ? nullptr : tile
    if (ntypes == 1) {
        if (members) k_nlist_build_threads<true, false><<<blocks, NLIST_BLOCK, 0, s>>>(AZP_NL_ARGS);
        else k_nlist_build_threads<true, true><<<blocks, NLIST_BLOCK, 0, s>>>(AZP_NL_ARGS);
    } else {
        if (members) k_nlist_build_threads<false, false><<<blocks, NLIST_BLOCK, 0, s>>>(AZP_NL_ARGS);
        else k_nlist_build_threads<false, true><<<blocks, NLIST_BLOCK, 0, s>>>(AZP_NL_ARGS);
    }
#undef AZP_NL_ARGS
}

void launch_cell_assign_fx(const uint4* fixed, uint32_t N, const CellGrid& g, uint32_t* cell_of, uint32_t* slot,
                           uint32_t* cell_count, cudaStream_t s, const uint32_t* gate)
{
    if (N == 0) return;
    k_cell_assign_fx<<<(N + 255) / 256, 256, 0, s>>>(fixed, N, g, cell_of, slot, cell_count, gate);
}

}  // namespace azp

// ==================================================================== C ABI object
namespace
{
void free_nl(azp_nlist* nl)
{
    cudaFree(nl->counts);
    cudaFree(nl->nbrs);
    cudaFree(nl->cuts);
    cudaFree(nl->fixed);
    cudaFree(nl->cell_of);
    cudaFree(nl->slot);
    cudaFree(nl->members);
    cudaFree(nl->cell_count);
    cudaFree(nl->cell_start);
    cudaFree(nl->scan_tmp);
    cudaFree(nl->flags);
    cudaFree(nl->ex_n);
    cudaFree(nl->ex_keys);
    cudaFree(nl->table);
    cudaFree(nl->cutbuf);
    cudaFree(nl->adj_table);
    cudaFree(nl->vel_f);
    cudaFree(nl->dpd_table);
}

int ensure_cells(azp_nlist* nl, uint32_t ncell)
{
    if (ncell <= nl->ncell_cap) return AZP_OK;
    cudaFree(nl->cell_count);
    cudaFree(nl->cell_start);
    cudaFree(nl->scan_tmp);
    nl->cell_count = nl->cell_start = nl->scan_tmp = nullptr;
    AZP_CUDA_TRY(cudaMalloc(&nl->cell_count, sizeof(uint32_t) * ncell));
    AZP_CUDA_TRY(cudaMalloc(&nl->cell_start, sizeof(uint32_t) * (ncell + 1)));
    AZP_CUDA_TRY(cudaMalloc(&nl->scan_tmp, sizeof(uint32_t) * azp::scan_tmp_words(ncell)));
    nl->ncell_cap = ncell;
    return AZP_OK;
}
}  // namespace

extern "C" {

azp_nlist* azp_nlist_create(uint32_t N, uint32_t ntypes, uint32_t max_neighbors, int* status)
{
    int st = AZP_OK;
    azp_nlist* nl = new (std::nothrow) azp_nlist();
    // list entries carry a mark in bit 31 between the scan and the compaction
    if (!nl || ntypes == 0 || ntypes > azp::MAX_LIST_TYPES || N > azp::NL_MAX_N) {
        if (status) *status = AZP_ERR_INVALID;
        delete nl;
        return nullptr;
    }
    nl->N = N;
    nl->ntypes = ntypes;
    nl->max_nn = max_neighbors ? max_neighbors : 64;
    const size_t n1 = N ? N : 1;
    auto fail = [&](cudaError_t e, const char* w) {
        st = azp::record_cuda_error(e, w);
    };
    cudaError_t e;
    if ((e = cudaMalloc(&nl->counts, sizeof(uint32_t) * n1)) != cudaSuccess) fail(e, "nlist counts");
    if (!st && (e = cudaMalloc(&nl->nbrs, sizeof(uint32_t) * n1 * nl->max_nn)) != cudaSuccess) fail(e, "nlist nbrs");
    if (!st && (e = cudaMalloc(&nl->cuts, sizeof(azp::ListCut) * ntypes * ntypes)) != cudaSuccess) fail(e, "cuts");
    if (!st && (e = cudaMalloc(&nl->fixed, sizeof(uint4) * n1)) != cudaSuccess) fail(e, "fixed");
    if (!st && (e = cudaMalloc(&nl->cell_of, sizeof(uint32_t) * n1)) != cudaSuccess) fail(e, "cell_of");
    if (!st && (e = cudaMalloc(&nl->slot, sizeof(uint32_t) * n1)) != cudaSuccess) fail(e, "slot");
    if (!st && (e = cudaMalloc(&nl->members, sizeof(uint32_t) * n1)) != cudaSuccess) fail(e, "members");
    if (!st && (e = cudaMalloc(&nl->flags, sizeof(uint32_t) * 4)) != cudaSuccess) fail(e, "flags");
    if (!st && (e = cudaMalloc(&nl->table, sizeof(double) * ntypes * ntypes * 12)) != cudaSuccess) fail(e, "table");
    if (!st && (e = cudaMalloc(&nl->cutbuf, sizeof(double) * ntypes * ntypes * 2)) != cudaSuccess) fail(e, "cutbuf");
    if (!st && (e = cudaMalloc(&nl->adj_table, sizeof(double) * 6 * 12 * ntypes * ntypes)) != cudaSuccess)
        fail(e, "adj_table");
    if (!st && (e = cudaMalloc(&nl->vel_f, sizeof(float4) * n1)) != cudaSuccess) fail(e, "vel_f");
    if (!st && (e = cudaMalloc(&nl->dpd_table, sizeof(double) * 8 * ntypes * ntypes)) != cudaSuccess)
        fail(e, "dpd_table");
    if (st) {
        free_nl(nl);
        delete nl;
        if (status) *status = st;
        return nullptr;
    }
    if (status) *status = AZP_OK;
    return nl;
}

void azp_nlist_destroy(azp_nlist* nl)
{
    if (!nl) return;
    free_nl(nl);
    delete nl;
}

int azp_nlist_set_cutoffs(azp_nlist* nl, const double* r_cut, double r_buff)
{
    if (!nl || !r_cut || r_buff < 0.0) return AZP_ERR_INVALID;
    const uint32_t nt2 = nl->ntypes * nl->ntypes;
    for (uint32_t a = 0; a < nl->ntypes; ++a)
        for (uint32_t b = 0; b < nl->ntypes; ++b)
            if (r_cut[a * nl->ntypes + b] != r_cut[b * nl->ntypes + a]) return AZP_ERR_INVALID;
    nl->r_cut.assign(r_cut, r_cut + nt2);
    nl->r_buff = r_buff;
    nl->have_cuts = true;
    return AZP_OK;
}

int azp_nlist_set_exclusions(azp_nlist* nl, const uint32_t* start, const uint32_t* partners)
{
    if (!nl) return AZP_ERR_INVALID;
    cudaFree(nl->ex_n);
    cudaFree(nl->ex_keys);
    nl->ex_n = nl->ex_keys = nullptr;
    nl->ex_width = 0;
    if (!start) return AZP_OK;
    const uint32_t N = nl->N;
    uint32_t w = 0;
    for (uint32_t i = 0; i < N; ++i) w = std::max(w, start[i + 1] - start[i]);
    if (w == 0) return AZP_OK;
    std::vector<uint32_t> n(N), keys((size_t)w * N, 0xffffffffu);
    for (uint32_t i = 0; i < N; ++i) {
        n[i] = start[i + 1] - start[i];
        for (uint32_t k = 0; k < n[i]; ++k) keys[(size_t)k * N + i] = partners[start[i] + k];
    }
    AZP_CUDA_TRY(cudaMalloc(&nl->ex_n, sizeof(uint32_t) * N));
    AZP_CUDA_TRY(cudaMalloc(&nl->ex_keys, sizeof(uint32_t) * keys.size()));
    AZP_CUDA_TRY(cudaMemcpy(nl->ex_n, n.data(), sizeof(uint32_t) * N, cudaMemcpyHostToDevice));
    AZP_CUDA_TRY(cudaMemcpy(nl->ex_keys, keys.data(), sizeof(uint32_t) * keys.size(), cudaMemcpyHostToDevice));
    nl->ex_width = w;
    return AZP_OK;
}

int azp_nlist_build(azp_nlist* nl, const azp_system* sys, void* stream)
{
    if (!nl || !sys || !nl->have_cuts || sys->N != nl->N || sys->ntypes != nl->ntypes) return AZP_ERR_INVALID;
    cudaStream_t s = azp::as_stream(stream);
    const uint32_t N = nl->N;
    std::vector<azp::ListCut> cuts(nl->ntypes * nl->ntypes);
    double rmax = 0.0;
    double rmin = 0.0;
    azp::make_list_cuts(nl->r_cut.data(), nl->ntypes, nl->r_buff, sys->box, cuts.data(), &rmax, &rmin);
    for (int d = 0; d < 3; ++d)
        if (rmax > 0.0 && sys->box.L[d] < 2.0 * rmax) return AZP_ERR_BOX_TOO_SMALL;
    const azp::CellGrid g = azp::make_grid(sys->box, rmax, azp::grid_subdivision(rmax, rmin));
    int st = ensure_cells(nl, g.ncell);
    if (st) return st;
    AZP_CUDA_TRY(cudaMemcpyAsync(nl->cuts, cuts.data(), sizeof(azp::ListCut) * cuts.size(), cudaMemcpyHostToDevice, s));
    if (N == 0) {
        nl->n_builds++;
        return AZP_OK;
    }
    const double4_32a* pos = reinterpret_cast<const double4_32a*>(sys->pos);
    for (int attempt = 0; attempt < 3; ++attempt) {
        AZP_CUDA_TRY(cudaMemsetAsync(nl->cell_count, 0, sizeof(uint32_t) * g.ncell, s));
        AZP_CUDA_TRY(cudaMemsetAsync(nl->flags, 0, sizeof(uint32_t) * 4, s));
        azp::launch_to_fixed(pos, nl->fixed, N, sys->box, s);
        azp::launch_cell_assign(pos, N, g, nl->cell_of, nl->slot, nl->cell_count, s);
        st = azp::exclusive_scan(nl->cell_count, nl->cell_start, g.ncell, nl->scan_tmp, s);
        if (st) return st;
        azp::launch_cell_scatter(nl->cell_of, nl->slot, nl->cell_start, nl->members, N, g.ncell, s);
        azp::launch_nlist_build(pos, nl->fixed, N, sys->box, g, nl->cell_start, nl->members, nl->cell_of, nl->cuts,
                                nl->ntypes, nl->ex_n, nl->ex_keys, nl->ex_width, nullptr, nl->counts, nl->nbrs,
                                nl->max_nn, nl->flags, nullptr, s, nullptr, rmin);
        AZP_CHECK_LAUNCH("azp_nlist_build");
        uint32_t need = 0;
        AZP_CUDA_TRY(cudaMemcpyAsync(&need, nl->flags, sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
        AZP_CUDA_TRY(cudaStreamSynchronize(s));
        if (need <= nl->max_nn) {
            nl->n_builds++;
            return AZP_OK;
        }
        // grow (HOOMD re-allocates and rebuilds on overflow as well)
        cudaFree(nl->nbrs);
        nl->nbrs = nullptr;
        nl->max_nn = need + 8;
        AZP_CUDA_TRY(cudaMalloc(&nl->nbrs, sizeof(uint32_t) * (size_t)N * nl->max_nn));
    }
    return AZP_ERR_NLIST_OVERFLOW;
}

int azp_nlist_view(const azp_nlist* nl, const uint32_t** counts, const uint32_t** neighbors, uint32_t* max_neighbors,
                   uint32_t* n_builds)
{
    if (!nl) return AZP_ERR_INVALID;
    if (counts) *counts = nl->counts;
    if (neighbors) *neighbors = nl->nbrs;
    if (max_neighbors) *max_neighbors = nl->max_nn;
    if (n_builds) *n_builds = nl->n_builds;
    return AZP_OK;
}

}  // extern "C"

extern "C" int azp_nlist_set_tpp(azp_nlist* nl, int tpp)
{
    if (!nl || !(tpp == 1 || tpp == 2 || tpp == 4 || tpp == 8 || tpp == 16 || tpp == 32)) return AZP_ERR_INVALID;
    nl->tpp = tpp;
    return AZP_OK;
}

extern "C" int azp_nlist_download(const azp_nlist* nl, uint32_t* counts, uint32_t* neighbors, void* stream)
{
    if (!nl || !counts || !neighbors) return AZP_ERR_INVALID;
    cudaStream_t s = azp::as_stream(stream);
    if (nl->N == 0) return AZP_OK;
    AZP_CUDA_TRY(cudaMemcpyAsync(counts, nl->counts, sizeof(uint32_t) * nl->N, cudaMemcpyDeviceToHost, s));
    AZP_CUDA_TRY(cudaMemcpyAsync(neighbors, nl->nbrs, sizeof(uint32_t) * (size_t)nl->N * nl->max_nn,
                                 cudaMemcpyDeviceToHost, s));
    AZP_CUDA_TRY(cudaStreamSynchronize(s));
    return AZP_OK;
}
