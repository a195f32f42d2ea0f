// scan.cuh -- device exclusive prefix sum over uint32 (three launches, any n).
#pragma once

#include "common.cuh"

namespace azp
{
constexpr int SCAN_BLOCK = 1024;

// block-local inclusive scan of in[] into out[] and the block total into sums[]
__global__ void k_scan_blocks(const uint32_t* __restrict__ in, uint32_t* __restrict__ out,
                              uint32_t* __restrict__ sums, uint32_t n, const uint32_t* __restrict__ gate);
// exclusive scan of sums[nb] in place, by one block
__global__ void k_scan_sums(uint32_t* __restrict__ sums, uint32_t nb, const uint32_t* __restrict__ gate);
// out[i] = inclusive[i] + sums[block] - in[i]  (exclusive); out[n] = total
__global__ void k_scan_finish(const uint32_t* __restrict__ in, uint32_t* __restrict__ out,
                              const uint32_t* __restrict__ sums, uint32_t n, const uint32_t* __restrict__ gate);

// Exclusive scan of in[n] into out[n+1] (out[n] = total). tmp needs
// scan_tmp_words(n) uint32. in may equal out only if the caller does not need in.
inline uint32_t scan_tmp_words(uint32_t n) { return (n + SCAN_BLOCK - 1) / SCAN_BLOCK + 1; }
// gate: device flag, the kernels do nothing while *gate == 0 (NULL: always run)
int exclusive_scan(const uint32_t* in, uint32_t* out, uint32_t n, uint32_t* tmp, cudaStream_t s,
                   const uint32_t* gate = nullptr);

}  // namespace azp
