// celllist.cuh -- cell binning and neighbour-list construction shared by the
// standalone azp_nlist object and the resident engine.
#pragma once

#include "common.cuh"

namespace azp
{
// cells holding more particles than this are not sorted by index
constexpr uint32_t kMaxSortedCell = 512;
// warps per block of the cell-sort kernels (each warp: 32 consecutive cells)
constexpr int kSortWarps = 8;
// cells up to this size are sorted by one lane, larger ones by the whole warp
constexpr uint32_t kSerialCell = 12;

// Insertion sort of a small cell's members by one thread (a handful of entries:
// the dense-melt case of about three particles per cell)
__device__ __forceinline__ void thread_sort_cell(uint32_t* __restrict__ members, uint32_t b, uint32_t e)
{
    for (uint32_t a = b + 1; a < e; ++a) {
        const uint32_t v = members[a];
        uint32_t k = a;
        while (k > b && members[k - 1] > v) {
            members[k] = members[k - 1];
            --k;
        }
        members[k] = v;
    }
}

// Sort the members of one cell, members[b, e), by particle index: the order in
// which atomics placed them is not deterministic, the sorted order is. One warp
// per cell: the members are staged in the warp's shared-memory row s_row
// (kMaxSortedCell entries), and the rank of each member is the number of members
// with a smaller index (indices are distinct), counted by a broadcast read of the
// row per compare; each lane ranks up to four members per pass over the row, so
// a cell of n members costs n * ceil(n / 128) shared-memory reads per lane. A
// cell above kMaxSortedCell keeps its arrival order (only a broken configuration
// crowds a cell that much). Warp-uniform control flow; no block barrier.
__device__ __forceinline__ void warp_sort_cell(uint32_t* __restrict__ members, uint32_t b, uint32_t e,
                                               uint32_t* __restrict__ s_row)
{
    const uint32_t n = e - b;
    if (n < 2 || n > kMaxSortedCell) return;
    const uint32_t lane = threadIdx.x & 31u;
    for (uint32_t k = lane; k < n; k += 32u) s_row[k] = members[b + k];
    __syncwarp();
    for (uint32_t base = 0; base < n; base += 128u) {
        uint32_t v[4], r[4] = {0u, 0u, 0u, 0u};
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const uint32_t k = base + (uint32_t)u * 32u + lane;
            v[u] = k < n ? s_row[k] : 0xffffffffu;
        }
        for (uint32_t q = 0; q < n; ++q) {
            const uint32_t x = s_row[q];
#pragma unroll
            for (int u = 0; u < 4; ++u) r[u] += x < v[u] ? 1u : 0u;
        }
#pragma unroll
        for (int u = 0; u < 4; ++u)
            if (base + (uint32_t)u * 32u + lane < n) members[b + r[u]] = v[u];
    }
}

// Cells of width >= r_list_max along each axis; an axis with fewer than 3 cells
// is scanned as a single cell (no duplicate images).
struct CellGrid {
    int dim[3];
    int reach[3];    // stencil cells each way (the subdivision), 0 for an axis too short for it
    double lo[3];    // -L/2
    double scale[3]; // dim / L
    uint32_t ncell;
};

// sub: cells of width >= r_list_max / sub and a stencil of sub cells each way
CellGrid make_grid(const azp_box& box, double rlist_max, int sub = 1);
// the subdivision the engine and the list object use: AZP_NL_SUB when set, else
// the ratio of the largest to the smallest list radius, 1 to 3
int grid_subdivision(double rlist_max, double rlist_min);

// Per type pair thresholds of the list decision (host-built, ntypes^2 entries).
struct ListCut {
    double rlistsq;  // exact FP64 test: rsq < rlistsq
    float lo, hi;    // FP32 prefilter: rsq_f < lo -> listed, rsq_f >= hi -> not listed
    float pad;
};

// Shared-memory neighbour tiles of the single-type FP32-force step. Particles
// are stored in cell order, so the list candidates of a block of TILE_P
// consecutive particles lie, stencil row by stencil row, in a few contiguous
// particle-index ranges; the step stages those ranges of 16-byte position
// records in shared memory and the list addresses them there. Per block one
// record of TILE_REC words: [0] number of ranges (0: the block is not tiled),
// [1] total records, then per range k: begin [2 + 3k], end [3 + 3k], tile offset
// [4 + 3k]. A list entry below 2^31 is a tile offset; TILE_GLOBAL | j is the
// particle index j (candidates outside the ranges: the wrapped cell at an x
// face, or a block whose ranges exceed TILE_CAP records).
constexpr uint32_t TILE_P = 256;
constexpr uint32_t TILE_REC = 32;
constexpr uint32_t TILE_MAX_RANGES = 9;
constexpr uint32_t TILE_CAP = 3072;  // 48 KB of 16-byte records
constexpr uint32_t TILE_GLOBAL = 0x80000000u;

// list entry of particle j for the block record t
__device__ __forceinline__ uint32_t tile_encode(const uint32_t* t, uint32_t j)
{
    const uint32_t nr = t[0];
    for (uint32_t k = 0; k < nr; ++k) {
        const uint32_t b = t[2 + 3 * k], e = t[3 + 3 * k];
        if (j >= b && j < e) return t[4 + 3 * k] + (j - b);
    }
    return TILE_GLOBAL | j;
}

// particle index of a list entry for the block record t
__device__ __forceinline__ uint32_t tile_decode(const uint32_t* __restrict__ t, uint32_t e)
{
    if (e & TILE_GLOBAL) return e & ~TILE_GLOBAL;
    const uint32_t nr = __ldg(t);
    for (uint32_t k = 0; k < nr; ++k) {
        const uint32_t off = __ldg(t + 4 + 3 * k), b = __ldg(t + 2 + 3 * k), e2 = __ldg(t + 3 + 3 * k);
        if (e >= off && e < off + (e2 - b)) return b + (e - off);
    }
    return 0u;  // not reached for entries the list build wrote
}

// Launch helpers (all stream-ordered, no allocation, no synchronisation).
// fixed[N] <- 16-byte fixed-point shadow of pos (x, y, z fractions of L, type)
void launch_to_fixed(const double4_32a* pos, uint4* fixed, uint32_t N, const azp_box& box, cudaStream_t s);

// cell_of[i], slot[i] (arrival order inside the cell) and cell_count[c] += 1.
// cell_count must be zeroed by the caller.
void launch_cell_assign(const double4_32a* pos, uint32_t N, const CellGrid& g, uint32_t* cell_of, uint32_t* slot,
                        uint32_t* cell_count, cudaStream_t s, const uint32_t* gate = nullptr);

// members[cell_start[c] + rank] = i with the rank of i among the particles of
// its cell in increasing index order (deterministic: a stable counting sort).
void launch_cell_scatter(const uint32_t* cell_of, const uint32_t* slot, const uint32_t* cell_start,
                         uint32_t* members, uint32_t N, uint32_t ncell, cudaStream_t s,
                         const uint32_t* gate = nullptr);

// Full neighbour list. members == NULL means the particles are already stored in
// cell order (members[s] = s). keys: exclusion keys of particles (NULL: index);
// ex_n[i] / ex_keys[k * N + i]: excluded keys of particle i. Rows are written
// column-major nbrs[k * N + i]; counts[i] = the true count even past max_nn;
// flags[0] = max count over particles (atomicMax), used to detect overflow.
void launch_nlist_build(const double4_32a* pos, const uint4* fixed, uint32_t N, const azp_box& box, const CellGrid& g,
                        const uint32_t* cell_start, const uint32_t* members, const uint32_t* cell_of,
                        const ListCut* cuts, uint32_t ntypes, const uint32_t* ex_n, const uint32_t* ex_keys,
                        uint32_t ex_width, const uint32_t* keys, uint32_t* counts, uint32_t* nbrs,
                        uint32_t max_nn, uint32_t* flags, const uint32_t* gate, cudaStream_t s,
                        const uint4* lo, double rlist_min, const uint32_t* tile = nullptr);
// tile != NULL: particles in cell order (members NULL), entries encoded for the
// block records of launch_tile_table.

// block records of the shared-memory tiles (particles in cell order, cell_of of
// the last binning): tab[(N + TILE_P - 1) / TILE_P][TILE_REC]
void launch_tile_table(const uint32_t* cell_of, const uint32_t* cell_start, const CellGrid& g, uint32_t N,
                       uint32_t* tab, const uint32_t* gate, cudaStream_t s);
// lo != NULL: positions are the 64-bit fixed words (fixed = high, lo = low) of the
// FP32-force engine, and the exact FP64 test runs on their FP64 conversion.
// rlist_min: the smallest listed r_cut + r_buff (sets the FP32 band of the
// shared-memory staged build).

// cell_of / slot / cell_count from the high words of 64-bit fixed positions
void launch_cell_assign_fx(const uint4* fixed, uint32_t N, const CellGrid& g, uint32_t* cell_of, uint32_t* slot,
                           uint32_t* cell_count, cudaStream_t s, const uint32_t* gate);

// fixed-point shadow of pos into one or two arrays (gated)
void launch_to_fixed2(const double4_32a* pos, uint4* a, uint4* b, uint32_t N, const azp_box& box, cudaStream_t s,
                      const uint32_t* gate);

// host: thresholds for r_cut[ntypes^2], r_buff and the box
void make_list_cuts(const double* r_cut, uint32_t ntypes, double r_buff, const azp_box& box, ListCut* out,
                    double* rlist_max, double* rlist_min = nullptr);

// The cells of one warp, 32 consecutive cells from (global warp index) * 32: a
// lane sorts its own cell when it holds at most kSerialCell members, then the
// warp sorts the larger ones together, one after another (warp_sort_cell).
__device__ __forceinline__ void sort_cells_warp(const uint32_t* __restrict__ cell_start,
                                                uint32_t* __restrict__ members, uint32_t ncell,
                                                uint32_t* __restrict__ s_row)
{
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t c = (blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5)) * 32u + lane;
    uint32_t b = 0u, e = 0u;
    if (c < ncell) {
        b = cell_start[c];
        e = cell_start[c + 1];
    }
    const uint32_t n = e - b;
    if (n >= 2u && n <= kSerialCell) thread_sort_cell(members, b, e);
    uint32_t big = __ballot_sync(0xffffffffu, n > kSerialCell && n <= kMaxSortedCell);
    while (big) {
        const int l = __ffs(big) - 1;
        big &= big - 1u;
        const uint32_t bb = __shfl_sync(0xffffffffu, b, l), ee = __shfl_sync(0xffffffffu, e, l);
        warp_sort_cell(members, bb, ee, s_row);
        __syncwarp();
    }
}

// Crowded grids (more than kSerialCell particles per cell on average): one warp
// per cell, so that the cells are sorted side by side instead of 32 after one
// another in each warp.
__device__ __forceinline__ void sort_cell_per_warp(const uint32_t* __restrict__ cell_start,
                                                   uint32_t* __restrict__ members, uint32_t ncell,
                                                   uint32_t* __restrict__ s_row)
{
    const uint32_t c = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (c >= ncell) return;  // warp-uniform
    const uint32_t b = cell_start[c], e = cell_start[c + 1];
    if (e - b <= kSerialCell) {
        if ((threadIdx.x & 31u) == 0u && e - b >= 2u) thread_sort_cell(members, b, e);
        return;
    }
    warp_sort_cell(members, b, e, s_row);
}

// whether a grid of ncell cells holding N particles is sorted a warp per cell
inline bool crowded_grid(uint32_t N, uint32_t ncell) { return ncell > 0 && N > kSerialCell * ncell; }

}  // namespace azp
