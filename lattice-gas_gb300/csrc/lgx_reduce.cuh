// lgx_reduce.cuh -- block-wide sums of 64-bit counters, added to device memory
// with one atomic per block and counter (a warp-level atomic per counter,
// thousands of them on one address, serialises in L2).
#pragma once

#include <cuda_runtime.h>

namespace lgx {

// Adds the block's sums of v[0..N) to out[0..N) (two's-complement 64-bit).
// Every thread of the block must call it.
template <int N>
__device__ __forceinline__ void block_add(long long (&v)[N], unsigned long long* out) {
  __shared__ long long part[32][N];
  const unsigned lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
#pragma unroll
  for (int off = 16; off > 0; off >>= 1)
#pragma unroll
    for (int k = 0; k < N; ++k) v[k] += __shfl_down_sync(0xffffffffu, v[k], off);
  if (lane == 0)
#pragma unroll
    for (int k = 0; k < N; ++k) part[warp][k] = v[k];
  __syncthreads();
  if (warp == 0) {
    const unsigned nw = (blockDim.x + 31u) >> 5;
#pragma unroll
    for (int k = 0; k < N; ++k) {
      long long s = lane < nw ? part[lane][k] : 0;
#pragma unroll
      for (int off = 16; off > 0; off >>= 1) s += __shfl_down_sync(0xffffffffu, s, off);
      if (lane == 0 && s) atomicAdd(out + k, (unsigned long long)s);
    }
  }
}

}  // namespace lgx
