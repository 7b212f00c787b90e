// scan_util.cuh — block-wide prefix sums used by the ordered compactions.
#pragma once
#include "common.cuh"

namespace sg {

// Exclusive prefix sum of `v` over the block (blockDim.x a multiple of 32,
// <= 1024).  Returns the exclusive prefix; *total receives the block sum.
// `sm` must hold 33 ints.
SLOAM_D int block_excl_scan(int v, int* sm, int* total) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  int x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    int y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) sm[wid] = x;
  __syncthreads();
  if (wid == 0) {
    int w = lane < nw ? sm[lane] : 0;
    int s = w;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      int y = __shfl_up_sync(0xffffffffu, s, o);
      if (lane >= o) s += y;
    }
    if (lane < nw) sm[lane] = s - w;
    if (lane == 31) sm[32] = s;
  }
  __syncthreads();
  int r = sm[wid] + x - v;
  *total = sm[32];
  __syncthreads();
  return r;
}

// Sum of the first `nb` entries of a global array, by the whole block.
SLOAM_D int block_sum_prefix(const int32_t* a, int nb, int* sm) {
  int s = 0;
  for (int k = threadIdx.x; k < nb; k += blockDim.x) s += a[k];
  s = warp_sumi(s);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  if (lane == 0) sm[wid] = s;
  __syncthreads();
  int t = 0;
  if (threadIdx.x < 32) {
    t = lane < nw ? sm[lane] : 0;
    t = warp_sumi(t);
    if (lane == 0) sm[32] = t;
  }
  __syncthreads();
  int r = sm[32];
  __syncthreads();
  return r;
}

}  // namespace sg
