// CTA-wide exclusive prefix sum shared by the radix sort (sort.cu) and the cell ordering
// of the track sampler (sample.cu).
#pragma once

#include <stdint.h>

namespace mlc {

// Exclusive prefix sum of v over the CTA's threads in thread order, and the CTA's total in
// *agg: an inclusive scan within each warp (shuffles), the warps' totals scanned by warp 0
// in shared memory, each thread's warp offset added.  blockDim.x a multiple of 32, <= 1024;
// every thread of the CTA calls it (two barriers inside).
__device__ __forceinline__ uint32_t block_exclusive_sum(uint32_t v, uint32_t* agg, uint32_t* wsum) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  uint32_t x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) wsum[warp] = x;
  __syncthreads();
  if (warp == 0) {
    uint32_t w = lane < nwarps ? wsum[lane] : 0u;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= o) w += y;
    }
    wsum[lane] = w;  // inclusive totals of warps 0..lane
  }
  __syncthreads();
  *agg = wsum[nwarps - 1];
  return (warp ? wsum[warp - 1] : 0u) + x - v;
}

}  // namespace mlc
