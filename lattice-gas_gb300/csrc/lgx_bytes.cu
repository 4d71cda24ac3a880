// lgx_bytes.cu -- the reference's byte-per-cell update, on the GPU.
//
// The reference's CPU lattice (src/lattice.rs) draws its collisions from a
// different random stream than its GPU bitplanes do: one xorshift64*
// generator per band of rows (bands of ceil(h / threads) rows), one draw per
// non-obstacle cell in row-major order, and a padded lookup table
// (src/collision.rs:72-119); the inflow re-seed after each step draws from one
// serial generator (src/lattice.rs:270-285).  Its golden tests pin that stream
// bit for bit.  This file runs the same stream on the device.
//
// The draws are sequential within a band, so a thread takes a 64-cell segment
// of one row and first jumps the band's generator to the segment's draw index.
// That index counts the band's non-obstacle cells before the segment, and
// obstacles never move, so it is fixed when cells are loaded; the host stores
// it as the jump polynomial z^k mod P (lgx_rng.cuh), and each block folds the
// first 64 states of its bands' generators into tables over 4-bit chunks of
// the polynomial, so a jump is 16 shared-memory lookups.
//
// A block stages a tile of rows (rows y0-1 .. y0+R) in shared memory with
// asynchronous copies, all in flight at once; each segment sits in its own
// 80-byte slot (15 pad bytes, the left halo byte, 64 cells; the right halo is
// the byte after the cells).  Five 16-byte chunks per slot is an odd count, so
// the lanes of a warp, one segment each, read their 16-byte chunks from
// distinct banks.  A thread walks its segment 16 cells at a time: one chunk per
// row, the neighbours by funnel shifts, the six arrival bits gathered for four
// cells at once.  Results go to a padded output tile and out with coalesced
// stores.
//
// The inflow re-seed after the step (src/lattice.rs:270-285) draws from one
// serial stream, 3 or 4 draws per non-obstacle cell of the leftmost columns,
// and depends only on that stream and the obstacles, so it is fused: every
// inflow cell (or, for inflows wider than 64 columns, every group of 8 cells
// of a row, to bound the table) has its own jump polynomial, the host passes
// the stream's first 64 states with the launch, and the block's threads draw
// the tile's inflow cells while its rows are in flight, into the output tile,
// where the collision results leave them be.  Many short draws finish sooner
// than a few long ones: this phase runs beside the tile's loads.
#include <cuda_runtime.h>
#include <string.h>

#include <algorithm>
#include <map>
#include <new>
#include <string>
#include <tuple>
#include <vector>

#include "../../include/lgx.h"
#include "lgx_internal.hpp"
#include "lgx_reduce.cuh"
#include "lgx_rng.cuh"

namespace {

using lgx::jump_entry;
using lgx::jump_poly;
using lgx::rng_seed;
using lgx::xorshift;

constexpr uint32_t kSeg = 64;             // cells per thread segment
constexpr uint32_t kThreads = 256;        // largest block
constexpr uint32_t kMaxRows = 8;          // rows per tile
constexpr uint32_t kSlot = kSeg + 16;     // input slot: 15 pad bytes, left halo, cells
constexpr uint32_t kOutPitch = kSeg + 4;  // output slot: 17 words
constexpr uint32_t kMaxStride = 30;       // outcomes per state in the padded table
constexpr uint32_t kInGroupWide = 8;      // inflow cells per jump polynomial, wide inflows
constexpr uint32_t kInNarrow = 64;        // inflows up to this wide: one polynomial a cell
constexpr uint32_t kLutBytes = 128 * kMaxStride;
static_assert((kSlot / 16) % 2 == 1 && (kOutPitch / 4) % 2 == 1, "odd pitches");
static_assert(kLutBytes % 16 == 0, "tile alignment");
constexpr uint8_t kSolid = 0x80, kRest = 0x40;
constexpr uint64_t kMul = lgx::kRngMul;
constexpr int kChunk = 4;                            // bits per jump-table chunk
constexpr uint32_t kTab = (64 / kChunk) << kChunk;  // entries per generator's table

struct ByteStepArgs {
  const uint8_t* old;
  uint8_t* out;
  const uint8_t* table;  // 128 * stride outcomes
  uint32_t stride;
  uint32_t w, h, band;   // band: rows per generator
  uint32_t segs;         // segments per row
  uint32_t cols, rows;   // tile: segments and rows
  uint32_t tiles_c;      // tiles across a row
  uint32_t nbands;       // band tables per block
  const uint64_t* poly;  // per segment: z^k mod P, k its first draw within the band
  uint64_t base_seed;    // seed ^ steps * 0x9E3779B97F4A7C15
  // the inflow re-seed
  uint32_t inlet_cols, inlet_group, inlet_groups;  // cells per group, groups per row
  const uint64_t* inlet_poly;  // per row and inflow group: z^k mod P, k the draws before it
  uint32_t t[7];
  int rest;
  uint64_t inlet_states[64];  // the stream's first 64 states (seed ^ steps after the step
                              // * 0xD1B54A32D192ED03)
};

__host__ __device__ __forceinline__ uint32_t in_row_bytes(uint32_t cols) {
  return cols * kSlot + 16;
}

// Band tables, the band generators' states, the collision table, the input
// tile, the output tile.
size_t step_smem_bytes(uint32_t cols, uint32_t rows, uint32_t nbands) {
  return (size_t)nbands * (kTab + 64) * 8 + kLutBytes + (size_t)(rows + 2) * in_row_bytes(cols) +
         ((size_t)rows * cols * kOutPitch + 15) / 16 * 16;
}

// Row y - 1 of the lattice, periodic, for y in 0 .. h + 1.
__device__ __forceinline__ uint32_t wrap_row(uint32_t y, uint32_t h) {
  return y == 0 ? h - 1 : (y - 1 >= h ? y - 1 - h : y - 1);
}

__device__ __forceinline__ uint32_t lds32(const uint8_t* p) {
  return *reinterpret_cast<const uint32_t*>(p);
}

__device__ __forceinline__ uint4 lds128(const uint8_t* p) {
  return *reinterpret_cast<const uint4*>(p);
}

__device__ __forceinline__ void cp_async16(void* dst, const void* src) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(
                   (uint32_t)__cvta_generic_to_shared(dst)),
               "l"(__cvta_generic_to_global(src))
               : "memory");
}

__device__ __forceinline__ void cp_async4(void* dst, const void* src) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(
                   (uint32_t)__cvta_generic_to_shared(dst)),
               "l"(__cvta_generic_to_global(src))
               : "memory");
}

__device__ __forceinline__ void cp_async_wait_all() {
  asm volatile("cp.async.wait_all;\n" ::: "memory");
}

// Four cells of row y from the words of rows y-1 (u), y (m) and y+1 (d) at
// their columns, with the words on either side (p, n).  Direction d arrives
// from the neighbour in the opposite direction (src/hex.rs:36-41): bit 0 from
// (x-1, y), bit 3 from (x+1, y); from row y-1 bits 1 and 2, from row y+1 bits
// 5 and 4, at columns (x-1, x) on even rows and (x, x+1) on odd rows.  Then
// bounce-back on obstacles, and on other cells the padded table's outcome for
// one draw of the band's generator (src/lattice.rs:324-364).
template <bool ODD>
__device__ __forceinline__ uint32_t gather4(uint32_t pu, uint32_t wu, uint32_t nu, uint32_t pm,
                                            uint32_t wm, uint32_t nm, uint32_t pd, uint32_t wd,
                                            uint32_t nd) {
  uint32_t a = (__funnelshift_l(pm, wm, 8) & 0x01010101u) |
               (__funnelshift_r(wm, nm, 8) & 0x08080808u) | (wm & 0x40404040u);
  if (ODD)
    a |= (wu & 0x02020202u) | (__funnelshift_r(wu, nu, 8) & 0x04040404u) |
         (__funnelshift_r(wd, nd, 8) & 0x10101010u) | (wd & 0x20202020u);
  else
    a |= (__funnelshift_l(pu, wu, 8) & 0x02020202u) | (wu & 0x04040404u) |
         (wd & 0x10101010u) | (__funnelshift_l(pd, wd, 8) & 0x20202020u);
  return a;
}

// The state of cell B of four (bit 7 of each byte of `a` is clear).
template <int B>
__device__ __forceinline__ uint32_t state_byte(uint32_t a) {
  return a >> (8 * B) & 0xFFu;
}

__device__ __forceinline__ uint32_t draw_k(uint64_t& st, uint32_t stride) {
  st = xorshift(st);
  return __umulhi((uint32_t)((st * kMul) >> 32), stride);
}

template <int B>
__device__ __forceinline__ uint32_t cell_out(uint32_t a, uint32_t wm, uint32_t bounce, uint64_t& st,
                                             const uint8_t* lut, uint32_t stride) {
  if (wm >> (8 * B + 7) & 1u) return bounce >> (8 * B) & 0xFFu;
  const uint32_t k = draw_k(st, stride);
  return lut[state_byte<B>(a) * stride + k];
}

__device__ __forceinline__ uint32_t bounce4(uint32_t a) {
  // the six moving bits turned by half a circle
  const uint32_t m = a & 0x3F3F3F3Fu;
  return 0x80808080u | (a & 0x40404040u) | ((m << 3) & 0x38383838u) | ((m >> 3) & 0x07070707u);
}

template <bool ODD>
__device__ __forceinline__ uint32_t step4(uint32_t pu, uint32_t wu, uint32_t nu, uint32_t pm,
                                          uint32_t wm, uint32_t nm, uint32_t pd, uint32_t wd,
                                          uint32_t nd, uint64_t& st, const uint8_t* lut,
                                          uint32_t stride) {
  const uint32_t a = gather4<ODD>(pu, wu, nu, pm, wm, nm, pd, wd, nd);
  if (!(wm & 0x80808080u)) {
    uint32_t res = 0;
    uint32_t k;
    k = draw_k(st, stride);
    res = lut[state_byte<0>(a) * stride + k];
    k = draw_k(st, stride);
    res |= (uint32_t)lut[state_byte<1>(a) * stride + k] << 8;
    k = draw_k(st, stride);
    res |= (uint32_t)lut[state_byte<2>(a) * stride + k] << 16;
    k = draw_k(st, stride);
    res |= (uint32_t)lut[state_byte<3>(a) * stride + k] << 24;
    return res;
  }
  const uint32_t bo = bounce4(a);
  return cell_out<0>(a, wm, bo, st, lut, stride) | cell_out<1>(a, wm, bo, st, lut, stride) << 8 |
         cell_out<2>(a, wm, bo, st, lut, stride) << 16 | cell_out<3>(a, wm, bo, st, lut, stride) << 24;
}

// The staged word for cells x .. x+3 of a segment: the collision results,
// except on non-obstacle inflow cells, whose sample is already staged.
__device__ __forceinline__ void put4(uint32_t* dst, uint32_t res, uint32_t x, uint32_t wm,
                                     uint32_t inlet_cols) {
  if (x < inlet_cols) {
    const uint32_t n = inlet_cols - x;
    uint32_t keep = ((~wm & 0x80808080u) >> 7) * 0xFFu;
    if (n < 4) keep &= (1u << (8 * n)) - 1;
    res = (res & ~keep) | (*dst & keep);
  }
  *dst = res;
}

// One thread's segment: `len` cells of row y, 16 at a time, from the input
// slots of rows y-1, y, y+1 into its output slot.
template <bool ODD>
__device__ __forceinline__ void walk(const uint8_t* up, const uint8_t* mid, const uint8_t* dn,
                                     uint8_t* o, uint32_t first, uint32_t len, uint64_t st,
                                     const uint8_t* lut, uint32_t stride, uint32_t inlet_cols) {
  uint32_t pu = lds32(up + 12), pm = lds32(mid + 12), pd = lds32(dn + 12);
  uint4 cu = lds128(up + 16), cm = lds128(mid + 16), cd = lds128(dn + 16);
  for (uint32_t g = 0; g < len; g += 16) {
    const uint4 xu = lds128(up + 32 + g), xm = lds128(mid + 32 + g), xd = lds128(dn + 32 + g);
    uint32_t* og = reinterpret_cast<uint32_t*>(o + g);
    const uint32_t r0 = step4<ODD>(pu, cu.x, cu.y, pm, cm.x, cm.y, pd, cd.x, cd.y, st, lut, stride);
    const uint32_t r1 = step4<ODD>(cu.x, cu.y, cu.z, cm.x, cm.y, cm.z, cd.x, cd.y, cd.z, st, lut, stride);
    const uint32_t r2 = step4<ODD>(cu.y, cu.z, cu.w, cm.y, cm.z, cm.w, cd.y, cd.z, cd.w, st, lut, stride);
    const uint32_t r3 = step4<ODD>(cu.z, cu.w, xu.x, cm.z, cm.w, xm.x, cd.z, cd.w, xd.x, st, lut, stride);
    if (first + g < inlet_cols) {
      put4(og, r0, first + g, cm.x, inlet_cols);
      put4(og + 1, r1, first + g + 4, cm.y, inlet_cols);
      put4(og + 2, r2, first + g + 8, cm.z, inlet_cols);
      put4(og + 3, r3, first + g + 12, cm.w, inlet_cols);
    } else {
      og[0] = r0;
      og[1] = r1;
      og[2] = r2;
      og[3] = r3;
    }
    pu = cu.w;
    pm = cm.w;
    pd = cd.w;
    cu = xu;
    cm = xm;
    cd = xd;
  }
}

// The inflow samples of a tile's rows y0 .. y0+R-1 and columns c0 .. (up to the
// inflow's edge), G cells of a row per task, into the output tile.
template <uint32_t G>
__device__ __forceinline__ void inflow_tile(const ByteStepArgs& p, uint8_t* out, uint32_t y0,
                                            uint32_t R, uint32_t C, uint32_t c0, uint32_t ncols,
                                            uint32_t tid, uint32_t nt) {
  const uint32_t n_in = min(p.inlet_cols, c0 + ncols) - c0;
  const uint32_t n_g = (n_in + G - 1) / G;
  for (uint32_t i = tid; i < R * n_g; i += nt) {
    const uint32_t r = i / n_g, x0 = (i - r * n_g) * G;
    const uint32_t n = min(G, n_in - x0);
    const uint8_t* cell = p.old + (size_t)(y0 + r) * p.w + c0 + x0;
    if (G == 1 && (__ldg(cell) & kSolid)) continue;
    const uint64_t pk = __ldg(p.inlet_poly + (size_t)(y0 + r) * p.inlet_groups + (c0 + x0) / G);
    uint64_t st = 0;
#pragma unroll
    for (int j = 0; j < 64; ++j)
      if (pk >> j & 1u) st ^= p.inlet_states[j];
    for (uint32_t x = 0; x < n; ++x) {
      if (G > 1 && (__ldg(cell + x) & kSolid)) continue;
      const uint32_t xt = x0 + x;
      out[(r * C + xt / kSeg) * kOutPitch + xt % kSeg] =
          lgx::equilibrium_sample(p.t, p.rest != 0, st);
    }
  }
}

__global__ void __launch_bounds__(kThreads) lgx_byte_step_kernel(const __grid_constant__ ByteStepArgs p) {
  extern __shared__ __align__(16) uint8_t smem[];
  const uint32_t tid = threadIdx.x, nt = blockDim.x;
  const uint32_t tc = blockIdx.x % p.tiles_c, tr = blockIdx.x / p.tiles_c;
  const uint32_t y0 = tr * p.rows;
  const uint32_t R = min(p.rows, p.h - y0);
  const uint32_t s0 = tc * p.cols;
  const uint32_t C = min(p.cols, p.segs - s0);
  const uint32_t c0 = s0 * kSeg;
  const uint32_t ncols = min(C * kSeg, p.w - c0);
  const uint32_t b0 = y0 / p.band, nb = (y0 + R - 1) / p.band - b0 + 1;
  const uint32_t RB = C * kSlot + 16;  // input row bytes

  uint64_t* tab = reinterpret_cast<uint64_t*>(smem);
  uint64_t* states = tab + p.nbands * kTab;
  uint8_t* lut = reinterpret_cast<uint8_t*>(states + p.nbands * 64);
  uint8_t* in = lut + kLutBytes;
  uint8_t* out = in + (p.rows + 2) * in_row_bytes(p.cols);

  // Launched with programmatic dependent launch: the collision table and the
  // band generators' states depend on nothing the previous step writes, so
  // they are under way while that step drains; its cells are read only after
  // griddepcontrol.wait (the previous grid complete and its writes visible).
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
  for (uint32_t i = tid; i < 32u * p.stride; i += nt) cp_async4(lut + i * 4, p.table + i * 4);
  // the first 64 states of each band's generator
  if (tid < nb) {
    uint64_t x = rng_seed(p.base_seed ^ ((uint64_t)(b0 + tid + 1) << 32));
    for (int j = 0; j < 64; ++j) {
      states[tid * 64 + j] = x;
      x = xorshift(x);
    }
  }
  asm volatile("griddepcontrol.wait;" ::: "memory");
  // rows y0-1 .. y0+R of the tile's columns, in flight together
  const uint32_t in_rows = R + 2;
  for (uint32_t r = 0; r < in_rows; ++r) {
    const uint32_t gy = wrap_row(y0 + r, p.h);
    const uint8_t* row = p.old + (size_t)gy * p.w + c0;
    uint8_t* dst = in + r * RB + 16;
    if ((p.w & 15u) == 0) {
      for (uint32_t k = tid; k < (ncols >> 4); k += nt)
        cp_async16(dst + (k >> 2) * kSlot + (k & 3u) * 16, row + k * 16);
    } else if ((p.w & 3u) == 0) {
      for (uint32_t k = tid; k < (ncols >> 2); k += nt)
        cp_async4(dst + (k >> 4) * kSlot + (k & 15u) * 4, row + k * 4);
    } else {
      for (uint32_t x = tid; x < ncols; x += nt) dst[(x / kSeg) * kSlot + x % kSeg] = __ldg(row + x);
    }
  }
  // halo bytes at the tile's two edges when it is narrower than a row (the
  // others are copied from neighbouring slots once the tile has landed)
  const uint32_t len_last = ncols - (C - 1) * kSeg;
  if (p.tiles_c > 1) {
    for (uint32_t i = tid; i < in_rows * 2; i += nt) {
      const uint32_t r = i >> 1, gy = wrap_row(y0 + r, p.h);
      const uint8_t* row = p.old + (size_t)gy * p.w;
      if (i & 1u)
        in[r * RB + (C - 1) * kSlot + 16 + len_last] = __ldg(row + (c0 + ncols == p.w ? 0 : c0 + ncols));
      else
        in[r * RB + 15] = __ldg(row + (c0 ? c0 - 1 : p.w - 1));
    }
  }
  // the inflow cells of the tile, into the output tile
  if (c0 < p.inlet_cols) {
    if (p.inlet_group == 1)
      inflow_tile<1>(p, out, y0, R, C, c0, ncols, tid, nt);
    else
      inflow_tile<kInGroupWide>(p, out, y0, R, C, c0, ncols, tid, nt);
  }
  cp_async_wait_all();
  __syncthreads();
  for (uint32_t i = tid; i < nb * kTab; i += nt)
    tab[i] = jump_entry<kChunk>(states + (i / kTab) * 64, i % kTab);
  // halo bytes between slots; across the row's ends when the tile spans it
  for (uint32_t r = 0; r < in_rows; ++r) {
    uint8_t* row = in + r * RB;
    for (uint32_t s = tid; s < C; s += nt) {
      uint8_t* slot = row + s * kSlot;
      if (s > 0)
        slot[15] = slot[16 + kSeg - 1 - kSlot];
      else if (p.tiles_c == 1)
        slot[15] = row[(C - 1) * kSlot + 16 + len_last - 1];
      if (s + 1 < C)
        slot[16 + kSeg] = slot[kSlot + 16];
      else if (p.tiles_c == 1)
        slot[16 + len_last] = row[16];
    }
  }
  __syncthreads();

  const uint32_t r = tid / C, s = tid - r * C;
  if (r < R) {
    const uint32_t y = y0 + r;
    const uint32_t first = c0 + s * kSeg, len = min(kSeg, p.w - first);
    uint64_t st = jump_poly<kChunk>(__ldg(p.poly + (size_t)y * p.segs + s0 + s),
                                    tab + (y / p.band - b0) * kTab);
    const uint8_t* up = in + r * RB + s * kSlot;
    uint8_t* o = out + (r * C + s) * kOutPitch;
    if (y & 1u)
      walk<true>(up, up + RB, up + 2 * RB, o, first, len, st, lut, p.stride, p.inlet_cols);
    else
      walk<false>(up, up + RB, up + 2 * RB, o, first, len, st, lut, p.stride, p.inlet_cols);
  }
  __syncthreads();
  for (uint32_t rr = 0; rr < R; ++rr) {
    const uint8_t* src = out + rr * C * kOutPitch;
    uint8_t* row = p.out + (size_t)(y0 + rr) * p.w + c0;
    if ((p.w & 3u) == 0) {
      for (uint32_t j = tid; j < (ncols >> 2); j += nt)
        reinterpret_cast<uint32_t*>(row)[j] = lds32(src + (j >> 4) * kOutPitch + (j & 15u) * 4);
    } else {
      for (uint32_t x = tid; x < ncols; x += nt) row[x] = src[(x / kSeg) * kOutPitch + x % kSeg];
    }
  }
}

// The WITH_WALLS moments of byte cells, read 8 cells per 64-bit word: bit d of
// every byte is counted by one popcount, and mass = sum, px2 and py2 weight the
// six moving bits by CX2 and CY2 (src/hex.rs, src/moments.rs:37-74); bit 7,
// the obstacle flag, is not a particle (src/lattice.rs:299-312).  out[0..2]:
// mass, px2, py2 as 64-bit two's-complement sums.
__global__ void __launch_bounds__(256) lgx_byte_moments_kernel(const uint8_t* __restrict__ cells,
                                                               size_t n,
                                                               unsigned long long* out,
                                                               unsigned long long* ticket,
                                                               unsigned long long* flag,
                                                               unsigned long long seq) {
  constexpr unsigned long long kBit0 = 0x0101010101010101ull;
  long long mass = 0, px2 = 0, py2 = 0;
  const uint64_t* w = reinterpret_cast<const uint64_t*>(cells);
  const size_t nw = n / 8;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < nw;
       i += (size_t)gridDim.x * blockDim.x) {
    const uint64_t x = __ldg(w + i);
    int c[7];
#pragma unroll
    for (int d = 0; d < 7; ++d) c[d] = __popcll(x & (kBit0 << d));
    mass += c[0] + c[1] + c[2] + c[3] + c[4] + c[5] + c[6];
    px2 += 2 * c[0] + c[1] - c[2] - 2 * c[3] - c[4] + c[5];
    py2 += c[1] + c[2] - c[4] - c[5];
  }
  if (blockIdx.x == 0 && threadIdx.x < n - nw * 8) {  // the last n % 8 cells
    const uint32_t x = cells[nw * 8 + threadIdx.x];
    int c[7];
#pragma unroll
    for (int d = 0; d < 7; ++d) c[d] = (x >> d) & 1u;
    mass += c[0] + c[1] + c[2] + c[3] + c[4] + c[5] + c[6];
    px2 += 2 * c[0] + c[1] - c[2] - 2 * c[3] - c[4] + c[5];
    py2 += c[1] + c[2] - c[4] - c[5];
  }
  long long v[3] = {mass, px2, py2};
  if (ticket)
    lgx::block_total_to_host<3>(v, ticket, out, flag, seq);
  else
    lgx::block_add<3>(v, out);
}

// ticket null: out is device memory, zeroed first; else out is mapped host memory
// the last block writes and ticket the counter buffer's word 4 (one operation).
cudaError_t launch_byte_moments(const uint8_t* cells, size_t n, unsigned long long* out,
                                cudaStream_t st, unsigned long long* ticket = nullptr,
                                unsigned long long* flag = nullptr, unsigned long long seq = 0) {
  if (!ticket) {
    cudaError_t e = cudaMemsetAsync(out, 0, 3 * sizeof(unsigned long long), st);
    if (e != cudaSuccess) return e;
  }
  size_t blocks = (n / 8 + 255) / 256;
  blocks = std::max<size_t>(1, std::min<size_t>(blocks, lgx::kReduceMaxBlocks));
  lgx_byte_moments_kernel<<<(unsigned)blocks, 256, 0, st>>>(cells, n, out, ticket, flag, seq);
  return cudaGetLastError();
}

// Host: the padded collision table (src/collision.rs:72-98).
void build_table(bool rest, std::vector<uint8_t>* data, uint32_t* stride) {
  static const int CX2[6] = {2, 1, -1, -2, -1, 1}, CY2[6] = {0, 1, 1, 0, -1, -1};
  const int n = rest ? 128 : 64;
  std::map<std::tuple<int, int, int>, std::vector<uint8_t>> groups;
  auto key = [&](int s) {
    int m = 0, x = 0, y = 0;
    for (int d = 0; d < 6; ++d)
      if (s >> d & 1) {
        ++m;
        x += CX2[d];
        y += CY2[d];
      }
    if (s & kRest) ++m;
    return std::make_tuple(m, x, y);
  };
  for (int s = 0; s < n; ++s) groups[key(s)].push_back((uint8_t)s);
  uint32_t st = 1;
  for (auto& kv : groups) {
    uint32_t a = st, b = (uint32_t)kv.second.size();
    while (b) {
      const uint32_t t = a % b;
      a = b;
      b = t;
    }
    st = st / a * (uint32_t)kv.second.size();
  }
  // Always 128 states: without rest particles a state with bit 6 set never
  // arises from the reference's own updates, and its rows here keep the state,
  // so no cell value can index past the table.
  data->assign((size_t)128 * st, 0);
  for (int s = 0; s < 128; ++s) {
    if (s >= n) {
      for (uint32_t k = 0; k < st; ++k) (*data)[(size_t)s * st + k] = (uint8_t)s;
      continue;
    }
    const auto& g = groups[key(s)];
    for (uint32_t k = 0; k < st; ++k) (*data)[(size_t)s * st + k] = g[k % g.size()];
  }
  *stride = st;
}

// The step kernel's dynamic shared memory limit, raised once per device to
// the largest tile plan_tiles can make.
cudaError_t ensure_step_attributes(int device) {
  static bool done[64] = {};
  if (device >= 0 && device < 64 && done[device]) return cudaSuccess;
  size_t most = 0;
  for (uint32_t r = 1; r <= kMaxRows; ++r)
    most = std::max(most, step_smem_bytes(kThreads / r, r, r));
  cudaError_t e = cudaFuncSetAttribute(
      lgx_byte_step_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)most);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(lgx_byte_step_kernel, cudaFuncAttributePreferredSharedMemoryCarveout,
                             (int)cudaSharedmemCarveoutMaxShared);
  if (e == cudaSuccess && device >= 0 && device < 64) done[device] = true;
  return e;
}

int cuda_fail(cudaError_t e, const char* what) {
  lgx::set_error(std::string(what) + ": " + cudaGetErrorString(e));
  return LGX_ERR_CUDA;
}

#define LGX_CUDA(call)                                  \
  do {                                                  \
    cudaError_t e_ = (call);                            \
    if (e_ != cudaSuccess) return cuda_fail(e_, #call); \
  } while (0)

}  // namespace

struct lgx_byte_lattice {
  int device = 0;
  cudaStream_t stream = nullptr;
  uint32_t w = 0, h = 0, threads = 1, band = 0, inlet_cols = 0, segs_per_row = 0;
  // step tiles: segments and rows per block, tiles across a row, band tables
  uint32_t tile_cols = 0, tile_rows = 0, tiles_c = 0, tiles = 0, nbands = 0, block = 0;
  size_t smem = 0;
  bool rest = true;
  float density = 0, ux = 0, uy = 0;
  uint64_t seed = 0, steps = 0;
  uint32_t thresh[7] = {};
  uint8_t* cells[2] = {nullptr, nullptr};
  int cur = 0;
  uint8_t* table = nullptr;
  uint32_t stride = 0;
  uint64_t* seg_poly = nullptr;
  uint64_t* inlet_poly = nullptr;
  // coarse-graining and counting go through the bitplane kernels
  lgx::Dims dm{};
  uint32_t* planes = nullptr;
  uint32_t* solid = nullptr;
  uint32_t* anysolid = nullptr;
  unsigned long long* counter = nullptr;
  unsigned long long* fill_scratch = nullptr;  // the equilibrium fill's block counts
  bool has_field = false;
  uint32_t bx = 0, by = 0, bw = 0, bh = 0;
  float* field = nullptr;
  int32_t* sums = nullptr;
};

namespace {

// Inflow cells per jump polynomial, and groups per row (at least one, for the
// allocation).
uint32_t inlet_group(const lgx_byte_lattice* L) {
  return L->inlet_cols <= kInNarrow ? 1u : kInGroupWide;
}

uint32_t inlet_groups(const lgx_byte_lattice* L) {
  const uint32_t g = inlet_group(L);
  return std::max((L->inlet_cols + g - 1) / g, 1u);
}

void free_bytes(lgx_byte_lattice* L) {
  cudaSetDevice(L->device);
  if (L->stream) cudaStreamSynchronize(L->stream);
  void* ptrs[] = {L->cells[0], L->cells[1], L->table,    L->seg_poly, L->inlet_poly, L->planes,
                  L->solid,    L->anysolid, L->counter, L->field,    L->sums, L->fill_scratch};
  for (void* p : ptrs) cudaFree(p);
  if (L->stream) cudaStreamDestroy(L->stream);
  delete L;
}

// The jump polynomial of every segment's first draw within its band, and of
// every inflow group's first draw in the inflow stream (row-major over the
// leftmost columns, 3 or 4 draws per non-obstacle cell), from the obstacles in
// `cells` (host copy).
int build_offsets(lgx_byte_lattice* L, const uint8_t* cells) {
  static const uint64_t q = lgx::rng_charpoly();
  if (!q) {
    lgx::set_error("the generator's characteristic polynomial failed its check");
    return LGX_ERR_STATE;
  }
  const uint32_t w = L->w, h = L->h;
  const uint32_t groups = inlet_groups(L), gs = inlet_group(L);
  std::vector<uint64_t> seg((size_t)h * L->segs_per_row), inl((size_t)h * groups, 1);
  uint64_t pk = 1;
  for (uint32_t y = 0; y < h; ++y) {
    if (y % L->band == 0) pk = 1;
    for (uint32_t s = 0; s < L->segs_per_row; ++s) {
      seg[(size_t)y * L->segs_per_row + s] = pk;
      const uint32_t x1 = std::min(w, (s + 1) * kSeg);
      for (uint32_t x = s * kSeg; x < x1; ++x)
        if (!(cells[(size_t)y * w + x] & kSolid)) pk = lgx::poly_mulz(pk, q);
    }
  }
  const uint32_t per = L->rest ? 4u : 3u;
  pk = 1;
  for (uint32_t y = 0; y < h; ++y)
    for (uint32_t x = 0; x < L->inlet_cols; ++x) {
      if (x % gs == 0) inl[(size_t)y * groups + x / gs] = pk;
      if (!(cells[(size_t)y * w + x] & kSolid))
        for (uint32_t i = 0; i < per; ++i) pk = lgx::poly_mulz(pk, q);
    }
  LGX_CUDA(cudaMemcpyAsync(L->seg_poly, seg.data(), seg.size() * 8, cudaMemcpyHostToDevice,
                           L->stream));
  LGX_CUDA(cudaMemcpyAsync(L->inlet_poly, inl.data(), inl.size() * 8, cudaMemcpyHostToDevice,
                           L->stream));
  LGX_CUDA(cudaStreamSynchronize(L->stream));
  return LGX_OK;
}

// Step tiles: a block takes up to 256 segments, as whole rows (up to 8) when a
// row has fewer, and as many band tables as its rows meet.
void plan_tiles(lgx_byte_lattice* L) {
  const uint32_t segs = L->segs_per_row;
  L->tile_cols = std::min(segs, kThreads);
  L->tile_rows = std::min(std::min(kMaxRows, kThreads / L->tile_cols), L->h);
  L->tiles_c = (segs + L->tile_cols - 1) / L->tile_cols;
  const uint32_t tiles_r = (L->h + L->tile_rows - 1) / L->tile_rows;
  L->tiles = L->tiles_c * tiles_r;
  L->nbands = 1;
  for (uint32_t t = 0; t < tiles_r; ++t) {
    const uint32_t y0 = t * L->tile_rows, y1 = std::min(L->h, y0 + L->tile_rows) - 1;
    L->nbands = std::max(L->nbands, y1 / L->band - y0 / L->band + 1);
  }
  L->block = std::min(kThreads, (L->tile_cols * L->tile_rows + 31) / 32 * 32);
  L->smem = step_smem_bytes(L->tile_cols, L->tile_rows, L->nbands);
}

}  // namespace

extern "C" {

int lgx_byte_create(size_t w, size_t h, float density, float ux, float uy, size_t inlet_cols,
                    int rest, size_t threads, uint64_t seed, lgx_byte_lattice** out) {
  if (!out) {
    lgx::set_error("null output");
    return LGX_ERR_ARG;
  }
  *out = nullptr;
  if (h % 2 != 0 || w <= 4 || h <= 4) {  // src/lattice.rs:137-138
    lgx::set_error("row count must be even, and the lattice larger than 4 x 4");
    return LGX_ERR_ARG;
  }
  if (w * h >= (1ull << 31)) {
    lgx::set_error("lattice too large for the byte path");
    return LGX_ERR_ARG;
  }
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    lgx::set_error("no CUDA device on this machine");
    return LGX_ERR_NO_DEVICE;
  }
  lgx_byte_lattice* L = new (std::nothrow) lgx_byte_lattice();
  if (!L) {
    lgx::set_error("out of host memory");
    return LGX_ERR_ALLOC;
  }
  cudaGetDevice(&L->device);
  L->w = (uint32_t)w;
  L->h = (uint32_t)h;
  L->rest = rest != 0;
  L->density = density;
  L->ux = ux;
  L->uy = uy;
  L->inlet_cols = (uint32_t)std::min(inlet_cols, w);
  L->threads = (uint32_t)std::max<size_t>(threads, 1);
  const uint32_t nthreads = std::min(L->threads, L->h);
  L->band = (L->h + nthreads - 1) / nthreads;  // src/lattice.rs:232-236
  L->segs_per_row = (L->w + kSeg - 1) / kSeg;
  L->seed = seed;
  lgx::equilibrium_thresholds(density, ux, uy, L->rest, L->thresh);
  L->dm = lgx::make_dims(L->w, L->h, 0);
  std::vector<uint8_t> table;
  build_table(L->rest, &table, &L->stride);
  if (L->stride > kMaxStride) {
    lgx::set_error("collision table wider than the kernel's");
    delete L;
    return LGX_ERR_STATE;
  }
  plan_tiles(L);
  const size_t cells = w * h, total = L->dm.total;
  cudaError_t e = cudaStreamCreateWithFlags(&L->stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaMalloc(&L->cells[0], cells);
  if (e == cudaSuccess) e = cudaMalloc(&L->cells[1], cells);
  if (e == cudaSuccess) e = cudaMalloc(&L->table, table.size());
  if (e == cudaSuccess) e = cudaMalloc(&L->seg_poly, (size_t)L->h * L->segs_per_row * 8);
  if (e == cudaSuccess)
    e = cudaMalloc(&L->inlet_poly, (size_t)L->h * inlet_groups(L) * 8);
  if (e == cudaSuccess) e = cudaMalloc(&L->planes, total * 7 * 4);
  if (e == cudaSuccess) e = cudaMalloc(&L->solid, total * 4);
  if (e == cudaSuccess) e = cudaMalloc(&L->anysolid, ((total + 31) / 32) * 4);
  // count, the three moments, one-launch totals' slots (zeroed)
  if (e == cudaSuccess) e = cudaMalloc(&L->counter, lgx::kCounterWords * 8);
  if (e == cudaSuccess) e = cudaMemset(L->counter, 0, lgx::kCounterWords * 8);
  if (e == cudaSuccess) e = cudaMemset(L->cells[0], 0, cells);
  if (e == cudaSuccess) e = cudaMemcpy(L->table, table.data(), table.size(), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = ensure_step_attributes(L->device);
  if (e != cudaSuccess) {
    const int rc = e == cudaErrorMemoryAllocation ? LGX_ERR_ALLOC : LGX_ERR_CUDA;
    lgx::set_error(std::string("lgx_byte_create: ") + cudaGetErrorString(e));
    free_bytes(L);
    return rc;
  }
  std::vector<uint8_t> zero(cells, 0);
  const int rc = build_offsets(L, zero.data());
  if (rc) {
    free_bytes(L);
    return rc;
  }
  *out = L;
  return LGX_OK;
}

int lgx_byte_destroy(lgx_byte_lattice* L) {
  if (L) free_bytes(L);
  return LGX_OK;
}

int lgx_byte_load(lgx_byte_lattice* L, const uint8_t* cells, size_t n) {
  if (!L || !cells || n != (size_t)L->w * L->h) {
    lgx::set_error("wrong number of cells");
    return LGX_ERR_ARG;
  }
  LGX_CUDA(cudaSetDevice(L->device));
  const int rc = build_offsets(L, cells);
  if (rc) return rc;
  LGX_CUDA(cudaMemcpyAsync(L->cells[L->cur], cells, n, cudaMemcpyHostToDevice, L->stream));
  LGX_CUDA(cudaStreamSynchronize(L->stream));
  return LGX_OK;
}

// Lattice::restart (src/lattice.rs:188-193).
int lgx_byte_restart(lgx_byte_lattice* L, const uint8_t* cells, size_t n, uint64_t seed) {
  const int rc = lgx_byte_load(L, cells, n);
  if (rc) return rc;
  L->seed = seed;
  L->steps = 0;
  return LGX_OK;
}

// Lattice::init_equilibrium (src/lattice.rs:197-208), on the device.  The
// obstacles stay where they are, so the draw offsets need no update.
int lgx_byte_init_equilibrium(lgx_byte_lattice* L) {
  if (!L) {
    lgx::set_error("null lattice");
    return LGX_ERR_ARG;
  }
  LGX_CUDA(cudaSetDevice(L->device));
  lgx::EqFill f{};
  f.cells = L->cells[L->cur];
  f.n = (size_t)L->w * L->h;
  f.seed = L->seed ^ 0xA5A51234ull;
  f.rest = L->rest;
  memcpy(f.thresh, L->thresh, sizeof(f.thresh));
  if (!L->fill_scratch) LGX_CUDA(cudaMalloc(&L->fill_scratch, lgx::kFillScratchBytes));
  f.scratch = L->fill_scratch;
  LGX_CUDA(lgx::launch_equilibrium_fill(f, L->stream));
  LGX_CUDA(cudaStreamSynchronize(L->stream));
  return LGX_OK;
}

int lgx_byte_store(lgx_byte_lattice* L, uint8_t* cells, size_t n) {
  if (!L || !cells || n != (size_t)L->w * L->h) {
    lgx::set_error("wrong number of cells");
    return LGX_ERR_ARG;
  }
  LGX_CUDA(cudaSetDevice(L->device));
  LGX_CUDA(cudaMemcpyAsync(cells, L->cells[L->cur], n, cudaMemcpyDeviceToHost, L->stream));
  LGX_CUDA(cudaStreamSynchronize(L->stream));
  return LGX_OK;
}

// Lattice::advance (src/lattice.rs:222-264).
int lgx_byte_advance(lgx_byte_lattice* L, uint64_t n) {
  if (!L) {
    lgx::set_error("null lattice");
    return LGX_ERR_ARG;
  }
  LGX_CUDA(cudaSetDevice(L->device));
  for (uint64_t i = 0; i < n; ++i) {
    ByteStepArgs a;
    a.old = L->cells[L->cur];
    a.out = L->cells[L->cur ^ 1];
    a.table = L->table;
    a.stride = L->stride;
    a.w = L->w;
    a.h = L->h;
    a.band = L->band;
    a.segs = L->segs_per_row;
    a.cols = L->tile_cols;
    a.rows = L->tile_rows;
    a.tiles_c = L->tiles_c;
    a.nbands = L->nbands;
    a.poly = L->seg_poly;
    a.base_seed = L->seed ^ (L->steps * 0x9E3779B97F4A7C15ull);
    a.inlet_cols = L->inlet_cols;
    a.inlet_group = inlet_group(L);
    a.inlet_groups = inlet_groups(L);
    a.inlet_poly = L->inlet_poly;
    uint64_t x = rng_seed(L->seed ^ ((L->steps + 1) * 0xD1B54A32D192ED03ull));
    for (int j = 0; j < 64; ++j, x = xorshift(x)) a.inlet_states[j] = x;
    memcpy(a.t, L->thresh, sizeof(a.t));
    a.rest = L->rest ? 1 : 0;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(L->tiles);
    cfg.blockDim = dim3(L->block);
    cfg.dynamicSmemBytes = L->smem;
    cfg.stream = L->stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    LGX_CUDA(cudaLaunchKernelEx(&cfg, lgx_byte_step_kernel, a));
    L->cur ^= 1;
    L->steps += 1;
  }
  LGX_CUDA(cudaStreamSynchronize(L->stream));
  return LGX_OK;
}

int lgx_byte_attach_field(lgx_byte_lattice* L, size_t bx, size_t by) {
  if (!L || bx == 0 || by == 0) {
    lgx::set_error("bad argument");
    return LGX_ERR_ARG;
  }
  LGX_CUDA(cudaSetDevice(L->device));
  cudaFree(L->field);
  cudaFree(L->sums);
  L->field = nullptr;
  L->sums = nullptr;
  L->bx = (uint32_t)bx;
  L->by = (uint32_t)by;
  L->bw = L->w / L->bx;
  L->bh = L->h / L->by;
  const size_t nb = std::max<size_t>((size_t)L->bw * L->bh, 1);
  LGX_CUDA(cudaMalloc(&L->field, nb * 16));
  LGX_CUDA(cudaMalloc(&L->sums, nb * 16));
  LGX_CUDA(cudaMemset(L->field, 0, nb * 16));
  LGX_CUDA(cudaMemset(L->sums, 0, nb * 16));
  L->has_field = true;
  return LGX_OK;
}

// Field::sample (src/render.rs:61-120) of the current cells.
int lgx_byte_sample_field(lgx_byte_lattice* L, float alpha) {
  if (!L || !L->has_field) {
    lgx::set_error("no field attached");
    return LGX_ERR_STATE;
  }
  LGX_CUDA(cudaSetDevice(L->device));
  LGX_CUDA(lgx::launch_pack(L->cells[L->cur], L->dm, L->planes, L->solid, L->anysolid, L->stream));
  lgx::SampleArgs sa;
  sa.a = L->planes;
  sa.solid = L->solid;
  sa.dm = L->dm;
  sa.bx = L->bx;
  sa.by = L->by;
  sa.bw = L->bw;
  sa.bh = L->bh;
  sa.alpha = alpha;
  const size_t nb = (size_t)L->bw * L->bh;
  sa.ux = L->field;
  sa.uy = L->field + nb;
  sa.rho = L->field + 2 * nb;
  sa.sol = L->field + 3 * nb;
  sa.sums = L->sums;
  LGX_CUDA(lgx::launch_sample(sa, L->stream));
  LGX_CUDA(cudaStreamSynchronize(L->stream));
  return LGX_OK;
}

int lgx_byte_read_field(lgx_byte_lattice* L, float* ux, float* uy, float* rho, float* sol,
                        size_t n_blocks) {
  if (!L || !L->has_field || n_blocks != (size_t)L->bw * L->bh) {
    lgx::set_error("no field attached, or block grid mismatch");
    return LGX_ERR_ARG;
  }
  LGX_CUDA(cudaSetDevice(L->device));
  float* dst[4] = {ux, uy, rho, sol};
  for (int i = 0; i < 4; ++i)
    if (dst[i] && n_blocks)
      LGX_CUDA(cudaMemcpyAsync(dst[i], L->field + i * n_blocks, n_blocks * 4,
                               cudaMemcpyDeviceToHost, L->stream));
  LGX_CUDA(cudaStreamSynchronize(L->stream));
  return LGX_OK;
}

// Lattice::total_particles (src/lattice.rs:299-312).
int lgx_byte_total_particles(lgx_byte_lattice* L, uint64_t* out) {
  if (!L || !out) {
    lgx::set_error("null argument");
    return LGX_ERR_ARG;
  }
  LGX_CUDA(cudaSetDevice(L->device));
  unsigned long long local = 0;
  unsigned long long* v = lgx::host_result_words();
  unsigned long long* dv = lgx::host_result_device();
  if (v && dv) {  // one launch that writes the moments into the mapped result words
    const unsigned long long seq = lgx::host_result_seq();
    LGX_CUDA(launch_byte_moments(L->cells[L->cur], (size_t)L->w * L->h, dv, L->stream,
                                 L->counter + 4, dv + 7, seq));
    LGX_CUDA(lgx::host_result_wait(seq, L->stream));
  } else {
    if (!v) v = &local;
    LGX_CUDA(launch_byte_moments(L->cells[L->cur], (size_t)L->w * L->h, L->counter + 1,
                                 L->stream));
    LGX_CUDA(cudaMemcpyAsync(v, L->counter + 1, 8, cudaMemcpyDeviceToHost, L->stream));
    LGX_CUDA(cudaStreamSynchronize(L->stream));
  }
  *out = *v;
  return LGX_OK;
}

// Lattice::mean_velocity (src/lattice.rs:286-294): the WITH_WALLS moments of
// every cell, then Moments::velocity.
int lgx_byte_mean_velocity(lgx_byte_lattice* L, float* ux, float* uy) {
  if (!L || !ux || !uy) {
    lgx::set_error("null argument");
    return LGX_ERR_ARG;
  }
  LGX_CUDA(cudaSetDevice(L->device));
  unsigned long long local[3];
  unsigned long long* v = lgx::host_result_words();
  unsigned long long* dv = lgx::host_result_device();
  if (v && dv) {
    const unsigned long long seq = lgx::host_result_seq();
    LGX_CUDA(launch_byte_moments(L->cells[L->cur], (size_t)L->w * L->h, dv, L->stream,
                                 L->counter + 4, dv + 7, seq));
    LGX_CUDA(lgx::host_result_wait(seq, L->stream));
  } else {
    if (!v) v = local;
    LGX_CUDA(launch_byte_moments(L->cells[L->cur], (size_t)L->w * L->h, L->counter + 1,
                                 L->stream));
    LGX_CUDA(cudaMemcpyAsync(v, L->counter + 1, 3 * sizeof(*v), cudaMemcpyDeviceToHost,
                             L->stream));
    LGX_CUDA(cudaStreamSynchronize(L->stream));
  }
  lgx::moments_velocity((int64_t)v[0], (int64_t)v[1], (int64_t)v[2], ux, uy);
  return LGX_OK;
}

int lgx_byte_steps(lgx_byte_lattice* L, uint64_t* out) {
  if (!L || !out) {
    lgx::set_error("null argument");
    return LGX_ERR_ARG;
  }
  *out = L->steps;
  return LGX_OK;
}

}  // extern "C"
