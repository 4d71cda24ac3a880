// lgx_reduce.cuh -- block-wide sums of 64-bit counters, added to device memory
// with one atomic per block and counter (a warp-level atomic per counter,
// thousands of them on one address, serialises in L2).
#pragma once

#include <cuda_runtime.h>

#include "lgx_internal.hpp"

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

// One-launch totals for a call that waits for them: every block writes its sums
// of v[0..N) to its own slot (slots = ticket + 2, N words per block, at most
// kReduceMaxBlocks blocks), and the last block to finish (a ticket it sets back
// to zero) adds the slots and writes the totals to `out`, page-locked host memory
// mapped into the device's address space.  No zeroing before the launch and no
// copy after it: one operation on the stream instead of three.  Integer sums, so
// the order of the blocks does not matter.  With `flag` set, the totals are followed
// (after a system-scope fence) by `seq` in *flag, which the host can wait for
// instead of synchronising the stream.  Every thread of the block must call it.
template <int N>
__device__ __forceinline__ void block_total_to_host(long long (&v)[N], unsigned long long* ticket,
                                                    unsigned long long* out,
                                                    unsigned long long* flag = nullptr,
                                                    unsigned long long seq = 0) {
  __shared__ long long part[32][N];
  __shared__ bool last;
  const unsigned lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
#pragma unroll
  for (int off = 16; off > 0; off >>= 1)
#pragma unroll
    for (int k = 0; k < N; ++k) v[k] += __shfl_down_sync(0xffffffffu, v[k], off);
  if (lane == 0)
#pragma unroll
    for (int k = 0; k < N; ++k) part[warp][k] = v[k];
  __syncthreads();
  unsigned long long* slots = ticket + 2;
  if (warp == 0) {
    const unsigned nw = (blockDim.x + 31u) >> 5;
#pragma unroll
    for (int k = 0; k < N; ++k) {
      long long s = lane < nw ? part[lane][k] : 0;
#pragma unroll
      for (int off = 16; off > 0; off >>= 1) s += __shfl_down_sync(0xffffffffu, s, off);
      if (lane == 0) slots[blockIdx.x * N + k] = (unsigned long long)s;
    }
    if (lane == 0) {
      __threadfence();
      last = atomicAdd(ticket, 1ull) == gridDim.x - 1u;
    }
  }
  __syncthreads();
  if (!last || warp != 0) return;
  __threadfence();
#pragma unroll
  for (int k = 0; k < N; ++k) {
    unsigned long long s = 0;
    for (unsigned b = lane; b < gridDim.x; b += 32u) s += __ldcg(slots + b * N + k);
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) s += __shfl_down_sync(0xffffffffu, s, off);
    if (lane == 0) out[k] = s;
  }
  if (lane == 0) {
    *ticket = 0ull;
    if (flag) {
      __threadfence_system();
      *reinterpret_cast<volatile unsigned long long*>(flag) = seq;
    }
  }
}

}  // namespace lgx
