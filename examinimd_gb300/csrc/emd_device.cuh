// Device-side helpers shared by the kernel files.
#pragma once
#include <cuda_runtime.h>

namespace emd {

constexpr unsigned FULL_MASK = 0xffffffffu;

__device__ __forceinline__ void latch_status(unsigned* status, unsigned bits) {
  if (status) atomicOr(status, bits);
}

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(FULL_MASK, v, o);
  return v;
}

__device__ __forceinline__ int warp_sum_int(int v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(FULL_MASK, v, o);
  return v;
}

// Block-wide sum in a fixed order (lane tree, then warp tree); result valid
// in thread 0.  `sh` needs blockDim.x/32 doubles.
__device__ __forceinline__ double block_sum(double v, double* sh) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  v = warp_sum(v);
  if (lane == 0) sh[w] = v;
  __syncthreads();
  const int nw = (blockDim.x + 31) >> 5;
  double t = 0.0;
  if (w == 0) {
    t = lane < nw ? sh[lane] : 0.0;
    t = warp_sum(t);
  }
  __syncthreads();
  return t;
}

}  // namespace emd
