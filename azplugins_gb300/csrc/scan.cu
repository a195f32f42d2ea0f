// scan.cu -- device exclusive prefix sum (warp-shuffle block scans, three launches).
#include "scan.cuh"

namespace azp
{
__device__ __forceinline__ uint32_t block_inclusive_scan(uint32_t v, uint32_t* s_warp)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t t = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v += t;
    }
    if (lane == 31) s_warp[warp] = v;
    __syncthreads();
    if (warp == 0) {
        const int nw = blockDim.x >> 5;
        uint32_t w = lane < nw ? s_warp[lane] : 0u;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t t = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += t;
        }
        if (lane < nw) s_warp[lane] = w;
    }
    __syncthreads();
    if (warp > 0) v += s_warp[warp - 1];
    return v;
}

__global__ void k_scan_blocks(const uint32_t* __restrict__ in, uint32_t* __restrict__ out,
                              uint32_t* __restrict__ sums, uint32_t n, const uint32_t* __restrict__ gate)
{
    if (gated_off(gate)) return;
    __shared__ uint32_t s_warp[32];
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t v = i < n ? in[i] : 0u;
    const uint32_t inc = block_inclusive_scan(v, s_warp);
    if (i < n) out[i] = inc;
    if (threadIdx.x == blockDim.x - 1) sums[blockIdx.x] = inc;
}

__global__ void k_scan_sums(uint32_t* __restrict__ sums, uint32_t nb, const uint32_t* __restrict__ gate)
{
    if (gated_off(gate)) return;
    __shared__ uint32_t s_warp[32];
    __shared__ uint32_t s_carry;
    if (threadIdx.x == 0) s_carry = 0u;
    __syncthreads();
    for (uint32_t base = 0; base < nb; base += blockDim.x) {
        const uint32_t i = base + threadIdx.x;
        const uint32_t v = i < nb ? sums[i] : 0u;
        const uint32_t inc = block_inclusive_scan(v, s_warp);
        const uint32_t carry = s_carry;
        if (i < nb) sums[i] = carry + inc - v;
        __syncthreads();
        if (threadIdx.x == blockDim.x - 1) s_carry = carry + inc;
        __syncthreads();
    }
}

__global__ void k_scan_finish(const uint32_t* __restrict__ in, uint32_t* __restrict__ out,
                              const uint32_t* __restrict__ sums, uint32_t n, const uint32_t* __restrict__ gate)
{
    if (gated_off(gate)) return;
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) {
        const uint32_t v = in[i];
        const uint32_t inc = out[i] + sums[blockIdx.x];
        out[i] = inc - v;
        if (i == n - 1) out[n] = inc;
    }
}

int exclusive_scan(const uint32_t* in, uint32_t* out, uint32_t n, uint32_t* tmp, cudaStream_t s,
                   const uint32_t* gate)
{
    if (n == 0) return AZP_ERR_INVALID;
    const uint32_t nb = (n + SCAN_BLOCK - 1) / SCAN_BLOCK;
    k_scan_blocks<<<nb, SCAN_BLOCK, 0, s>>>(in, out, tmp, n, gate);
    k_scan_sums<<<1, SCAN_BLOCK, 0, s>>>(tmp, nb, gate);
    k_scan_finish<<<nb, SCAN_BLOCK, 0, s>>>(in, out, tmp, n, gate);
    AZP_CHECK_LAUNCH("exclusive_scan");
    return AZP_OK;
}

}  // namespace azp
