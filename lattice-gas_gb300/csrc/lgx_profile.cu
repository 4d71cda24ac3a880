// lgx_profile.cu -- row and column profiles of the lattice on the device.
//
// transport.rs watches one Fourier mode through two profiles of the state:
// row_ux, the mean x-velocity of each row, and column_uy, the mean y-velocity
// of each column (src/transport.rs:51-91), both from the exact integer moments
// of moments.rs with the wall particles counted (WITH_WALLS).  The reference
// gathers the whole lattice to the host to form them; here they are reduced
// on the device and only h + w floats leave it.
//
// One launch covers many lattices (blockIdx.y) and a band of kRows rows each
// (blockIdx.x).  A warp sums a row's words by popcount; for the columns a
// thread owns 8 columns (one byte of a word) and adds the bits of each plane
// into eight byte-wide counters at once, flushing them into the column sums
// with atomics at the end of its band.  The last block of a lattice to finish
// turns the sums into f32 velocities exactly as the reference does, clears
// the column sums for the next use, and resets the block counter.
//
// A lattice in a batch is profiled only at its own sample points: local steps
// first + i * every, i < count, with sample i written to slot i of its
// trajectory buffers.
#include <cuda_runtime.h>

#include "lgx_profile.hpp"

namespace lgx {
namespace {

constexpr int kThreads = 256;
constexpr uint32_t kRows = 16;  // rows per block; byte counters stay below 256
constexpr float kSqrt3_2 = 0.8660254f;

// The 8 bits of x spread to the low bit of 8 bytes (bit i -> byte i).
__device__ __forceinline__ uint64_t spread8(uint32_t x) {
  const uint64_t t = ((uint64_t)x * 0x0101010101010101ull) & 0x8040201008040201ull;
  return ((t + 0x7F7F7F7F7F7F7F7Full) & 0x8080808080808080ull) >> 7;
}

__device__ __forceinline__ int32_t byte_of(uint64_t v, int i) { return (int32_t)((v >> (8 * i)) & 0xFFu); }

__global__ void __launch_bounds__(kThreads) lgx_profile_kernel(const ProfArgs p) {
  const ProfDesc& d = p.descs[blockIdx.y];
  const uint64_t local = (p.base ? *p.base : 0ull) + p.k_after;
  const uint64_t t = d.offset + local;
  if (t < d.first) return;
  const uint64_t rel = t - d.first;
  if (d.every == 0 ? rel != 0 : rel % d.every != 0) return;
  const uint64_t slot = d.every ? rel / d.every : 0;
  if (slot >= d.count) return;
  const Dims dm = d.dm;  // in registers, not read through d at every use
  const uint32_t nchunks = (dm.h + kRows - 1) / kRows;
  if (blockIdx.x >= nchunks) return;
  const uint32_t par = (d.cur0 + (uint32_t)local) & 1u;
  const uint32_t* a = par ? d.planes[1] : d.planes[0];
  const size_t S = dm.total;
  const uint32_t y0 = blockIdx.x * kRows, y1 = min(y0 + kRows, dm.h);
  const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;

  // rows: a warp per row (the bits past the row's end are zero)
  for (uint32_t y = y0 + warp; y < y1; y += kThreads / 32) {
    int32_t mass = 0, px2 = 0, py2 = 0;
    for (uint32_t j = lane; j < dm.wpr; j += 32) {
      const size_t o = (size_t)y * dm.wpr + j;
      int32_t c[7];
#pragma unroll
      for (int q = 0; q < 7; ++q) c[q] = __popc(__ldg(a + q * S + o));
      mass += c[0] + c[1] + c[2] + c[3] + c[4] + c[5] + c[6];
      px2 += 2 * c[0] + c[1] - c[2] - 2 * c[3] - c[4] + c[5];  // CX2
      py2 += c[1] + c[2] - c[4] - c[5];                         // CY2
    }
#pragma unroll
    for (int o = 16; o; o >>= 1) {
      mass += __shfl_down_sync(0xffffffffu, mass, o);
      px2 += __shfl_down_sync(0xffffffffu, px2, o);
      py2 += __shfl_down_sync(0xffffffffu, py2, o);
    }
    if (lane == 0) {
      d.rows[y] = mass;
      d.rows[dm.h + y] = px2;
      d.rows[2 * dm.h + y] = py2;
    }
  }

  // columns: thread = (word j, byte q), eight columns, byte-wide counters
  for (uint32_t pr = threadIdx.x; pr < dm.wpr * 4u; pr += kThreads) {
    const uint32_t j = pr >> 2, q = pr & 3u;
    uint64_t m = 0, pxp = 0, pxn = 0, pyp = 0, pyn = 0;
    for (uint32_t y = y0; y < y1; ++y) {
      const size_t o = (size_t)y * dm.wpr + j;
      uint64_t s[7];
#pragma unroll
      for (int k = 0; k < 7; ++k) s[k] = spread8((__ldg(a + k * S + o) >> (8 * q)) & 0xFFu);
      m += s[0] + s[1] + s[2] + s[3] + s[4] + s[5] + s[6];
      pxp += 2 * s[0] + s[1] + s[5];
      pxn += s[2] + 2 * s[3] + s[4];
      pyp += s[1] + s[2];
      pyn += s[4] + s[5];
    }
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      const uint32_t x = j * 32u + q * 8u + i;
      if (x >= dm.w) break;
      const int32_t mi = byte_of(m, i);
      if (mi == 0) continue;  // no particles: nothing to add
      atomicAdd(d.cols + x, mi);
      atomicAdd(d.cols + dm.w + x, byte_of(pxp, i) - byte_of(pxn, i));
      atomicAdd(d.cols + 2 * dm.w + x, byte_of(pyp, i) - byte_of(pyn, i));
    }
  }

  // the last block of this lattice forms the velocities
  __shared__ bool last;
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) last = atomicAdd(d.done, 1u) == nchunks - 1u;
  __syncthreads();
  if (!last) return;
  __threadfence();
  if (d.row_u) {
    float* out = d.row_u + slot * dm.h;
    for (uint32_t y = threadIdx.x; y < dm.h; y += kThreads) {
      const int32_t mass = __ldcg(d.rows + y), px2 = __ldcg(d.rows + dm.h + y);
      // Moments::velocity (src/moments.rs:91-97): px2 as f32 * 0.5 / m
      out[y] = mass ? __fdiv_rn(__fmul_rn(__int2float_rn(px2), 0.5f), __int2float_rn(mass)) : 0.0f;
    }
  }
  for (uint32_t x = threadIdx.x; x < dm.w; x += kThreads) {
    const int32_t mass = __ldcg(d.cols + x), px2 = __ldcg(d.cols + dm.w + x),
                  py2 = __ldcg(d.cols + 2 * dm.w + x);
    if (d.col_u) {
      // column_uy (src/transport.rs:76-83): py2 as f32 * SQRT3_2 / mass as f32
      d.col_u[slot * dm.w + x] =
          mass > 0 ? __fdiv_rn(__fmul_rn(__int2float_rn(py2), kSqrt3_2), __int2float_rn(mass)) : 0.0f;
    }
    if (d.col_sums) {
      d.col_sums[x] = mass;
      d.col_sums[dm.w + x] = px2;
      d.col_sums[2 * dm.w + x] = py2;
    }
    d.cols[x] = 0;
    d.cols[dm.w + x] = 0;
    d.cols[2 * dm.w + x] = 0;
  }
  if (threadIdx.x == 0) *d.done = 0u;
}

}  // namespace

uint32_t profile_chunks(uint32_t h) { return (h + kRows - 1) / kRows; }

cudaError_t launch_profile(const ProfArgs& p, uint32_t max_h, cudaStream_t st) {
  if (p.nlat == 0) return cudaSuccess;
  if (p.nlat > 65535u) return cudaErrorInvalidValue;
  const dim3 grid(profile_chunks(max_h), p.nlat);
  lgx_profile_kernel<<<grid, kThreads, 0, st>>>(p);
  return cudaGetLastError();
}

}  // namespace lgx
