// lgx_init.cu -- the equilibrium fill on the device.
//
// Lattice::init_equilibrium (src/lattice.rs:197-208) walks the cells in
// row-major order with one generator, Rng::new(seed ^ 0xA5A51234): a solid
// cell becomes SOLID_BIT and takes no draw, a fluid cell takes three draws (four
// with rest particles) and becomes an equilibrium sample.  The draw index of a
// fluid cell is therefore (fluid cells before it) x draws per cell, so a thread
// that owns a run of cells can start from that index with a jump-ahead instead
// of walking the generator from the first cell.
//
// Cells are handled in words of 32 (a bitplane word, or 32 consecutive bytes),
// one word per thread, or 8 on fills large enough to give every SM several
// blocks that way.  Two launches: the first counts the fluid cells of each
// block's contiguous range of words; the second has each block add up the
// counts of the blocks before it, then walk its range 256 segments at a time,
// with a block-wide scan giving each thread the fluid cells before its segment.
#include <cuda_runtime.h>

#include <algorithm>
#include <mutex>
#include <vector>

#include "lgx_internal.hpp"
#include "lgx_rng.cuh"

namespace lgx {
namespace {

constexpr int kThreads = 256;
constexpr uint32_t kSegWordsLarge = 8;  // 32-cell words per thread on large fills
// Fills of fewer words than this take one word per thread: with eight, a
// small lattice's few blocks run on a few SMs, each thread walking 256 cells.
constexpr uint64_t kLargeFillWords = 152ull * 8 * 256 * kSegWordsLarge;
constexpr int kFillJumps = 48;     // draw indices below 2^48

struct FillArgs {
  EqFill f;
  uint64_t nwords;      // 32-cell words in cell order
  uint64_t nseg;        // segments of seg_words words
  uint32_t seg_words;   // 32-cell words per thread
  uint64_t per_block;   // segments per block (a multiple of kThreads)
  uint64_t s0;          // generator state before the first draw
  unsigned long long* blk;  // fluid cells per block
  const uint64_t* jump;     // [kFillJumps][64] columns of M^(2^i)
};

// Fluid cells of word `wd` as a bit mask (bit b = cell 32 wd + b), and for the
// planes the valid cells.
__device__ __forceinline__ uint32_t fluid_mask(const FillArgs& p, uint64_t wd) {
  if (p.f.planes) {
    const uint32_t j = (uint32_t)(wd % p.f.dm.wpr);
    const uint32_t valid = (j == p.f.dm.lastword) ? p.f.dm.tail : 0xffffffffu;
    return ~__ldg(p.f.solid + wd) & valid;
  }
  const uint64_t c0 = wd * 32u;
  uint32_t m = 0;
  if (c0 + 32u <= p.f.n) {
    const uint4* v = reinterpret_cast<const uint4*>(p.f.cells + c0);
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const uint4 q = v[h];
      const uint32_t u[4] = {q.x, q.y, q.z, q.w};
#pragma unroll
      for (int k = 0; k < 4; ++k)
#pragma unroll
        for (int b = 0; b < 4; ++b)
          m |= (((u[k] >> (8 * b + 7)) & 1u) ^ 1u) << (16 * h + 4 * k + b);
    }
  } else {
    for (uint32_t b = 0; c0 + b < p.f.n; ++b) m |= (uint32_t)(!(p.f.cells[c0 + b] & 0x80u)) << b;
  }
  return m;
}

__device__ __forceinline__ uint32_t segment_count(const FillArgs& p, uint64_t seg) {
  uint32_t c = 0;
  const uint64_t w0 = seg * p.seg_words;
  const uint64_t w1 = min(w0 + p.seg_words, p.nwords);
  for (uint64_t wd = w0; wd < w1; ++wd) c += __popc(fluid_mask(p, wd));
  return c;
}

// Block-wide exclusive scan of one value per thread; returns the block total.
__device__ __forceinline__ uint32_t block_scan(uint32_t v, uint32_t* excl, uint32_t* smem) {
  const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
  uint32_t x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= (uint32_t)o) x += y;
  }
  if (lane == 31u) smem[warp] = x;
  __syncthreads();
  if (warp == 0) {
    uint32_t t = lane < kThreads / 32 ? smem[lane] : 0u;
#pragma unroll
    for (int o = 1; o < kThreads / 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, t, o);
      if (lane >= (uint32_t)o) t += y;
    }
    if (lane < kThreads / 32) smem[lane] = t;  // inclusive warp totals
  }
  __syncthreads();
  *excl = x - v + (warp ? smem[warp - 1] : 0u);
  const uint32_t total = smem[kThreads / 32 - 1];
  __syncthreads();  // smem is reused by the next call
  return total;
}

__global__ void __launch_bounds__(kThreads) lgx_fill_count_kernel(const FillArgs p) {
  __shared__ unsigned long long part[kThreads / 32];
  const uint64_t s0 = blockIdx.x * p.per_block;
  const uint64_t s1 = min(s0 + p.per_block, p.nseg);
  unsigned long long c = 0;
  for (uint64_t s = s0 + threadIdx.x; s < s1; s += kThreads) c += segment_count(p, s);
#pragma unroll
  for (int o = 16; o; o >>= 1) c += __shfl_down_sync(0xffffffffu, c, o);
  if ((threadIdx.x & 31u) == 0) part[threadIdx.x >> 5] = c;
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned long long t = 0;
    for (int w = 0; w < kThreads / 32; ++w) t += part[w];
    p.blk[blockIdx.x] = t;
  }
}

__global__ void __launch_bounds__(kThreads) lgx_fill_sample_kernel(const FillArgs p) {
  __shared__ uint64_t jump[kFillJumps * 64];
  __shared__ uint32_t scan[kThreads / 32];
  __shared__ unsigned long long part[kThreads / 32];
  for (int i = threadIdx.x; i < kFillJumps * 64; i += kThreads) jump[i] = p.jump[i];
  // fluid cells in the blocks before this one
  unsigned long long base = 0;
  for (uint32_t b = threadIdx.x; b < blockIdx.x; b += kThreads) base += p.blk[b];
#pragma unroll
  for (int o = 16; o; o >>= 1) base += __shfl_down_sync(0xffffffffu, base, o);
  if ((threadIdx.x & 31u) == 0) part[threadIdx.x >> 5] = base;
  __syncthreads();
  base = 0;
  for (int w = 0; w < kThreads / 32; ++w) base += part[w];

  const uint32_t per = p.f.rest ? 4u : 3u;
  const uint64_t s0 = blockIdx.x * p.per_block;
  const uint64_t s1 = min(s0 + p.per_block, p.nseg);
  for (uint64_t t0 = s0; t0 < s1; t0 += kThreads) {
    const uint64_t seg = t0 + threadIdx.x;
    const uint32_t mine = seg < s1 ? segment_count(p, seg) : 0u;
    uint32_t before = 0;
    const uint32_t tile = block_scan(mine, &before, scan);
    if (seg < s1) {
      uint64_t st = jump_ahead(p.s0, (base + before) * per, jump);
      const uint64_t w0 = seg * p.seg_words;
      const uint64_t w1 = min(w0 + p.seg_words, p.nwords);
      for (uint64_t wd = w0; wd < w1; ++wd) {
        uint32_t m = fluid_mask(p, wd);
        if (p.f.planes) {
          uint32_t o[7] = {0, 0, 0, 0, 0, 0, 0};
          if (p.f.thresh_rows || p.f.thresh_cols) {
            // thresholds by row, or by column (32 j + b)
            const uint32_t y = (uint32_t)(wd / p.f.dm.wpr), j = (uint32_t)(wd % p.f.dm.wpr);
            uint32_t t[7];
            if (p.f.thresh_rows) {
#pragma unroll
              for (int d = 0; d < 7; ++d) t[d] = __ldg(p.f.thresh_rows + (size_t)y * 7 + d);
            }
            while (m) {
              const uint32_t b = __ffs(m) - 1;
              m &= m - 1;
              if (p.f.thresh_cols) {
#pragma unroll
                for (int d = 0; d < 7; ++d)
                  t[d] = __ldg(p.f.thresh_cols + (size_t)(j * 32u + b) * 7 + d);
              }
              const uint32_t s = equilibrium_sample(t, p.f.rest, st);
#pragma unroll
              for (int d = 0; d < 7; ++d) o[d] |= ((s >> d) & 1u) << b;
            }
          } else {
            while (m) {
              const uint32_t b = __ffs(m) - 1;
              m &= m - 1;
              const uint32_t s = equilibrium_sample(p.f.thresh, p.f.rest, st);
#pragma unroll
              for (int d = 0; d < 7; ++d) o[d] |= ((s >> d) & 1u) << b;
            }
          }
#pragma unroll
          for (int d = 0; d < 7; ++d) p.f.planes[(size_t)d * p.f.dm.total + wd] = o[d];
        } else {
          const uint64_t c0 = wd * 32u;
          if (c0 + 32u <= p.f.n) {
            uint32_t o[8];
#pragma unroll
            for (int k = 0; k < 8; ++k) {
              uint32_t v = 0;
#pragma unroll
              for (int b = 0; b < 4; ++b) {
                const uint32_t bit = 4 * k + b;
                const uint32_t s = ((m >> bit) & 1u)
                                       ? equilibrium_sample(p.f.thresh, p.f.rest, st)
                                       : 0x80u;
                v |= s << (8 * b);
              }
              o[k] = v;
            }
            uint4* dst = reinterpret_cast<uint4*>(p.f.cells + c0);
            dst[0] = make_uint4(o[0], o[1], o[2], o[3]);
            dst[1] = make_uint4(o[4], o[5], o[6], o[7]);
          } else {
            for (uint32_t b = 0; c0 + b < p.f.n; ++b)
              p.f.cells[c0 + b] =
                  ((m >> b) & 1u) ? equilibrium_sample(p.f.thresh, p.f.rest, st) : 0x80u;
          }
        }
      }
    }
    base += tile;
  }
}

// The jump matrices M^(2^i), i < kFillJumps, on the current device: built and
// copied once per device for the process (24 KB).
cudaError_t device_jumps(const uint64_t** out) {
  static std::mutex mu;
  static const uint64_t* table[64] = {};
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> g(mu);
  if (!table[dev]) {
    std::vector<uint64_t> jumps = build_jumps();
    jumps.resize((size_t)kFillJumps * 64);
    void* p = nullptr;
    e = cudaMalloc(&p, jumps.size() * sizeof(uint64_t));
    if (e != cudaSuccess) return e;
    e = cudaMemcpy(p, jumps.data(), jumps.size() * sizeof(uint64_t), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
      cudaFree(p);
      return e;
    }
    table[dev] = (const uint64_t*)p;
  }
  *out = table[dev];
  return cudaSuccess;
}

}  // namespace

cudaError_t launch_equilibrium_fill(const EqFill& f, cudaStream_t st) {
  FillArgs p{};
  p.f = f;
  p.nwords = f.planes ? (uint64_t)f.dm.total : (f.n + 31) / 32;
  if (p.nwords == 0) return cudaSuccess;
  const uint64_t cells = p.nwords * 32u;
  if ((cells * 4u) >> kFillJumps) return cudaErrorInvalidValue;  // draw index range
  if (!f.planes && (reinterpret_cast<uintptr_t>(f.cells) & 15u)) return cudaErrorInvalidValue;
  if ((f.thresh_rows || f.thresh_cols) && (!f.planes || (f.thresh_rows && f.thresh_cols)))
    return cudaErrorInvalidValue;
  p.seg_words = p.nwords >= kLargeFillWords ? kSegWordsLarge : 1u;
  p.nseg = (p.nwords + p.seg_words - 1) / p.seg_words;
  // a few blocks per SM, each over a contiguous range of whole tiles
  const uint64_t tiles = (p.nseg + kThreads - 1) / kThreads;
  const uint64_t nblk = std::min<uint64_t>(tiles, 152u * 8u);
  p.per_block = ((tiles + nblk - 1) / nblk) * kThreads;
  const uint32_t grid = (uint32_t)((p.nseg + p.per_block - 1) / p.per_block);
  p.s0 = rng_seed(f.seed);

  cudaError_t e = device_jumps(&p.jump);
  if (e != cudaSuccess) return e;
  void* scratch = nullptr;
  if (f.scratch) {
    p.blk = f.scratch;
  } else {
    e = cudaMallocAsync(&scratch, (size_t)grid * 8u, st);
    if (e != cudaSuccess) return e;
    p.blk = (unsigned long long*)scratch;
  }
  lgx_fill_count_kernel<<<grid, kThreads, 0, st>>>(p);
  lgx_fill_sample_kernel<<<grid, kThreads, 0, st>>>(p);
  e = cudaGetLastError();
  const cudaError_t e2 = scratch ? cudaFreeAsync(scratch, st) : cudaSuccess;
  return e != cudaSuccess ? e : e2;
}

}  // namespace lgx
