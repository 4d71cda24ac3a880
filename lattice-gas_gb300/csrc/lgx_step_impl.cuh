// lgx_step_impl.cuh -- the per-word bitplane update and the per-block
// coarse-graining, shared by the single-lattice and the batched kernels.
#pragma once

#include "lgx_device.cuh"
#include "lgx_internal.hpp"

namespace lgx {

// Plane loads.  LD_NC: the read-only path (the single-step and batched
// kernels, whose planes do not change during the launch).  LD_CG: through L2
// (ld.global.cg), for planes written by other SMs during the launch (the
// persistent kernels).  LD_GENERIC: a plain load through a generic address,
// for planes held in this CTA's or another cluster CTA's shared memory.
enum { LD_NC = 0, LD_CG = 1, LD_GENERIC = 2 };

template <int LD>
__device__ __forceinline__ uint32_t ldp(const uint32_t* p) {
  if (LD == LD_NC) return __ldg(p);
  if (LD == LD_CG) return __ldcg(p);
  return *p;
}

// Word to the left of `j` in the same row, with the row's periodic wrap: for
// j == 0 the bit that enters is bit `lastbit` of the last word, placed at 31.
template <int LD>
__device__ __forceinline__ uint32_t left_word(const uint32_t* row, uint32_t j, bool in_warp,
                                              uint32_t shuffled, const Dims& dm) {
  if (in_warp) return shuffled;
  if (j > 0) return ldp<LD>(row + j - 1);
  return ldp<LD>(row + dm.lastword) << (31u - dm.lastbit);
}

// Bits x+1 into x: (w >> 1) | (next << 31), and on the last word of the row
// the bit at `lastbit` comes from bit 0 of word 0 (src/gpu.rs:248-254).
template <int LD>
__device__ __forceinline__ uint32_t shift_from_right(uint32_t w, const uint32_t* row, uint32_t j,
                                                     bool in_warp, uint32_t shuffled,
                                                     const Dims& dm) {
  uint32_t hi = in_warp ? shuffled : ((j + 1u < dm.wpr) ? ldp<LD>(row + j + 1u) : 0u);
  uint32_t v = __funnelshift_r(w, hi, 1);
  if (j == dm.lastword)
    v = (v & ~(1u << dm.lastbit)) | ((ldp<LD>(row) & 1u) << dm.lastbit);
  return v;
}

// The update of one lattice word: word j of row y, global word index g (for
// the draws' key, the obstacle planes and the inflow).  rows[d] points at
// word 0 of the row plane d is gathered from (planes 1, 2: row y-1; 0, 3, 6:
// row y; 4, 5: row y+1), out at word j of row y of plane 0 of the
// destination, whose planes are `ostride` words apart.  All 32 lanes of the
// warp call this together with consecutive words (lanes past the end repeat
// the last word and do not store: `live`).
template <bool REST, int LD>
__device__ __forceinline__ void step_core(const uint32_t* const rows[7], uint32_t* out,
                                          size_t ostride, const uint32_t* __restrict__ solid,
                                          const uint32_t* __restrict__ anysolid,
                                          const uint32_t* __restrict__ inlet, const Dims& dm,
                                          const Draws& s, uint32_t g, uint32_t y, uint32_t j,
                                          bool live) {
  const uint32_t lane = threadIdx.x & 31u;
  const bool odd = y & 1u;
  const uint32_t *r0 = rows[0], *r1 = rows[1], *r2 = rows[2], *r3 = rows[3], *r4 = rows[4],
                 *r5 = rows[5];
  const uint32_t w0 = ldp<LD>(r0 + j), w1 = ldp<LD>(r1 + j);
  const uint32_t w2 = ldp<LD>(r2 + j), w3 = ldp<LD>(r3 + j);
  const uint32_t w4 = ldp<LD>(r4 + j), w5 = ldp<LD>(r5 + j);
  const uint32_t w6 = ldp<LD>(rows[6] + j);
  // With the planes in shared memory (the resident kernels) the inflow's words
  // for this word are loaded with the planes, so that their latency passes
  // during the collision (eight 64 x 64 lattices with inflows: 1.71 -> 1.47 us
  // per step); the register-limited global-memory kernels load them after it
  // (early, their large lattices lost up to 15%).
  constexpr bool kEarlyInflow = LD == LD_GENERIC;
  const bool inflow = j < dm.iw;
  uint32_t bern[7] = {0u, 0u, 0u, 0u, 0u, 0u, 0u};
  if (kEarlyInflow && inflow) {
    const uint32_t* bp = inlet + ((size_t)y * dm.iw + j) * 7u;
#pragma unroll
    for (int d = 0; d < 7; ++d) bern[d] = __ldg(bp + d);
  }

  // Partner lanes hold the neighbouring word of the same plane and row
  // exactly when they sit in the same row.
  const unsigned FULL = 0xffffffffu;
  const uint32_t l0 = __shfl_up_sync(FULL, w0, 1), l1 = __shfl_up_sync(FULL, w1, 1);
  const uint32_t l5 = __shfl_up_sync(FULL, w5, 1);
  const uint32_t q2 = __shfl_down_sync(FULL, w2, 1), q3 = __shfl_down_sync(FULL, w3, 1);
  const uint32_t q4 = __shfl_down_sync(FULL, w4, 1);
  const bool lok = lane > 0u && j > 0u;
  const bool rok = lane < 31u && j + 1u < dm.wpr;

  // Gather (src/gpu.rs:237-265).  Direction d takes from the neighbour in the
  // opposite direction; the column offset depends on the row's parity:
  //   d0: x-1        d3: x+1
  //   d1: even x-1, odd x      d2: even x, odd x+1     (row y-1)
  //   d4: even x, odd x+1      d5: even x-1, odd x     (row y+1)
  uint32_t n[7];
  n[0] = __funnelshift_l(left_word<LD>(r0, j, lok, l0, dm), w0, 1);
  n[3] = shift_from_right<LD>(w3, r3, j, rok, q3, dm);
  if (odd) {
    n[1] = w1;
    n[2] = shift_from_right<LD>(w2, r2, j, rok, q2, dm);
    n[4] = shift_from_right<LD>(w4, r4, j, rok, q4, dm);
    n[5] = w5;
  } else {
    n[1] = __funnelshift_l(left_word<LD>(r1, j, lok, l1, dm), w1, 1);
    n[2] = w2;
    n[4] = w4;
    n[5] = __funnelshift_l(left_word<LD>(r5, j, lok, l5, dm), w5, 1);
  }
  n[6] = w6;

  uint32_t o[7];
  collide<REST>(n, s, o);

  // Obstacle words are rare.  A warp covers the 32 words g & ~31 .. g | 31, whose
  // summary bits are one anysolid word, so the whole warp skips the solid
  // load and the bounce-back select together when that word is zero.
  const uint32_t any = __ldg(anysolid + (g >> 5));
  uint32_t sm = 0u;
  uint32_t res[7];
  if (any != 0u) {
    if ((any >> (g & 31u)) & 1u) sm = __ldg(solid + g);
    walls(n, o, sm, res);
  } else {
#pragma unroll
    for (int d = 0; d < 7; ++d) res[d] = o[d];
  }

  if (inflow) {  // inflow re-seed of the leftmost columns (src/gpu.rs:296-306)
    const uint32_t span = min(dm.inlet_cols - j * 32u, 32u);
    const uint32_t imask = (span >= 32u) ? 0xffffffffu : ((1u << span) - 1u);
    const uint32_t apply = imask & ~sm;
    const uint32_t* bp = inlet + ((size_t)y * dm.iw + j) * 7u;
#pragma unroll
    for (int d = 0; d < 7; ++d) {
      const uint32_t b = kEarlyInflow ? bern[d] : __ldg(bp + d);
      res[d] = (res[d] & ~apply) | (b & apply);
    }
  }

  if (dm.tail != 0xffffffffu && j == dm.lastword) {  // clear the bits past the row's end
#pragma unroll
    for (int d = 0; d < 7; ++d) res[d] &= dm.tail;
  }
  if (live) {
#pragma unroll
    for (int d = 0; d < 7; ++d) out[d * ostride] = res[d];
  }
}

// One step of lattice word g of planes a -> b (g clamped into range for idle
// lanes, which still take part in the shuffles; `live` lanes store).
template <bool REST, bool COHERENT>
__device__ __forceinline__ void step_word(const uint32_t* a, uint32_t* b,
                                          const uint32_t* __restrict__ solid,
                                          const uint32_t* __restrict__ anysolid,
                                          const uint32_t* __restrict__ inlet, const Dims& dm,
                                          const Draws& s, uint32_t g, bool live) {
  const uint32_t t = __umulhi(g, dm.div_m);
  const uint32_t y = (t + ((g - t) >> dm.div_s1)) >> dm.div_s2;  // g / wpr
  const uint32_t j = g - y * dm.wpr;
  const uint32_t ym = (y == 0u) ? dm.h - 1u : y - 1u;
  const uint32_t yp = (y + 1u == dm.h) ? 0u : y + 1u;
  const size_t S = dm.total;
  const uint32_t* rows[7] = {a + 0 * S + (size_t)y * dm.wpr,  a + 1 * S + (size_t)ym * dm.wpr,
                             a + 2 * S + (size_t)ym * dm.wpr, a + 3 * S + (size_t)y * dm.wpr,
                             a + 4 * S + (size_t)yp * dm.wpr, a + 5 * S + (size_t)yp * dm.wpr,
                             a + 6 * S + (size_t)y * dm.wpr};
  step_core<REST, COHERENT ? LD_CG : LD_NC>(rows, b + g, S, solid, anysolid, inlet, dm, s, g, y,
                                            j, live);
}

// V consecutive words of one row held by one lane (V = 2 or 4), loaded and
// stored as one 64- or 128-bit access per plane.
template <int V> struct LaneWords;
template <> struct LaneWords<2> {
  typedef uint2 T;
  static __device__ __forceinline__ void get(const T& t, uint32_t* v) { v[0] = t.x; v[1] = t.y; }
  static __device__ __forceinline__ T make(const uint32_t* v) { return make_uint2(v[0], v[1]); }
};
template <> struct LaneWords<4> {
  typedef uint4 T;
  static __device__ __forceinline__ void get(const T& t, uint32_t* v) {
    v[0] = t.x; v[1] = t.y; v[2] = t.z; v[3] = t.w;
  }
  static __device__ __forceinline__ T make(const uint32_t* v) {
    return make_uint4(v[0], v[1], v[2], v[3]);
  }
};

// One step of words gq .. gq+V-1 of planes a -> b, V consecutive words of one
// row per lane, for lattices whose rows are a whole number of such groups
// (wpr % V == 0; then every plane row starts on a 16-byte boundary).  The
// same update as step_word, word for word; what V words share is computed
// once: the row, its neighbours and their pointers, the wrap and edge
// predicates, one shuffle per plane and side (the neighbour word inside the
// lane's group is already in a register), the obstacle summary and the
// inflow and tail tests.  All 32 lanes call this together with consecutive
// groups; lanes past the end repeat the last group and do not store.  INFLOW
// false compiles the update without the inflow (for lattices with none: the
// registers its early loads hold are then free).
template <bool REST, int V, int E, bool INFLOW = true>
__device__ __forceinline__ void step_lane_words(const uint32_t* __restrict__ a,
                                                uint32_t* __restrict__ b,
                                                const uint32_t* __restrict__ solid,
                                                const uint32_t* __restrict__ anysolid,
                                                const uint32_t* __restrict__ inlet,
                                                const Dims& dm, const Draws* s, uint32_t seed32,
                                                uint32_t gq, bool live) {
  typedef LaneWords<V> LW;
  typedef typename LW::T VT;
  const uint32_t lane = threadIdx.x & 31u;
  const uint32_t t = __umulhi(gq, dm.div_m);
  const uint32_t y = (t + ((gq - t) >> dm.div_s1)) >> dm.div_s2;  // gq / wpr
  const uint32_t j0 = gq - y * dm.wpr;
  const uint32_t ym = (y == 0u) ? dm.h - 1u : y - 1u;
  const uint32_t yp = (y + 1u == dm.h) ? 0u : y + 1u;
  const size_t S = dm.total;
  const uint32_t* rc = a + (size_t)y * dm.wpr;   // row y, plane 0
  const uint32_t* rm = a + (size_t)ym * dm.wpr;  // row y-1
  const uint32_t* rp = a + (size_t)yp * dm.wpr;  // row y+1
  // plane d's row: 1, 2 from y-1; 0, 3, 6 from y; 4, 5 from y+1
  const uint32_t* r[7] = {rc, rm + S, rm + 2 * S, rc + 3 * S, rp + 4 * S, rp + 5 * S, rc + 6 * S};
  uint32_t w[7][V];
#pragma unroll
  for (int d = 0; d < 7; ++d) LW::get(__ldg(reinterpret_cast<const VT*>(r[d] + j0)), w[d]);
  // The inflow's Bernoulli words for the group's first word, loaded with the
  // planes so that their latency passes during the collision (with V words per
  // lane every warp of a lattice up to 32 V words wide holds a row start).
  const bool inflow0 = INFLOW && j0 < dm.iw;
  uint32_t bern0[7] = {0u, 0u, 0u, 0u, 0u, 0u, 0u};
  if (inflow0) {
    const uint32_t* bp = inlet + ((size_t)y * dm.iw + j0) * 7u;
#pragma unroll
    for (int d = 0; d < 7; ++d) bern0[d] = __ldg(bp + d);
  }

  const unsigned FULL = 0xffffffffu;
  const bool lok = lane > 0u && j0 > 0u;        // lane - 1 holds words j0-V .. j0-1 of this row
  const bool rok = lane < 31u && j0 + V < dm.wpr;  // lane + 1 holds j0+V .. j0+2V-1
  const bool last = j0 + V == dm.wpr;           // word V-1 is the row's last word
  // the word left of j0 for planes 0, 1, 5 and right of j0+V-1 for 2, 3, 4
  uint32_t lw[3], rw[3];
  {
    const int lp[3] = {0, 1, 5}, rpn[3] = {2, 3, 4};
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      const uint32_t l = __shfl_up_sync(FULL, w[lp[i]][V - 1], 1);
      const uint32_t q = __shfl_down_sync(FULL, w[rpn[i]][0], 1);
      lw[i] = lok ? l : (j0 > 0u ? __ldg(r[lp[i]] + j0 - 1u)
                                 : __ldg(r[lp[i]] + dm.lastword) << (31u - dm.lastbit));
      rw[i] = rok ? q : (last ? 0u : __ldg(r[rpn[i]] + j0 + V));
    }
  }
  // bit 0 of word 0 of the rows planes 2, 3, 4 read, the wrap into the last word
  uint32_t wrap[3] = {0u, 0u, 0u};
  if (last) {
    wrap[0] = __ldg(r[2]) & 1u;
    wrap[1] = __ldg(r[3]) & 1u;
    wrap[2] = __ldg(r[4]) & 1u;
  }

  // obstacle summary bits of the V words (V divides 32, groups are aligned)
  const uint32_t abits = (__ldg(anysolid + (gq >> 5)) >> (gq & 31u)) & ((1u << V) - 1u);
  const bool warp_solid = __any_sync(FULL, abits != 0u);
  uint32_t sw[V];
#pragma unroll
  for (int q = 0; q < V; ++q) sw[q] = 0u;
  if (abits != 0u) LW::get(__ldg(reinterpret_cast<const VT*>(solid + gq)), sw);

  const bool odd = y & 1u;
  uint32_t res[7][V];
#pragma unroll
  for (int q = 0; q < V; ++q) {
    auto left = [&](int i, int d) { return q > 0 ? w[d][q - 1] : lw[i]; };
    auto right = [&](int i, int d) -> uint32_t {
      uint32_t v = __funnelshift_r(w[d][q], q < V - 1 ? w[d][q + 1] : rw[i], 1);
      if (q == V - 1 && last) v = (v & ~(1u << dm.lastbit)) | (wrap[i] << dm.lastbit);
      return v;
    };
    uint32_t n[7];
    n[0] = __funnelshift_l(left(0, 0), w[0][q], 1);
    n[3] = right(1, 3);
    if (odd) {
      n[1] = w[1][q];
      n[2] = right(0, 2);
      n[4] = right(2, 4);
      n[5] = w[5][q];
    } else {
      n[1] = __funnelshift_l(left(1, 1), w[1][q], 1);
      n[2] = w[2][q];
      n[4] = w[4][q];
      n[5] = __funnelshift_l(left(2, 5), w[5][q], 1);
    }
    n[6] = w[6][q];
    uint32_t o[7];
    if (q < E) {
      collide<REST>(n, s[q], o);
    } else {
      const Draws sq = draws((gq + q) ^ seed32);
      collide<REST>(n, sq, o);
    }
    if (warp_solid) {
      uint32_t rr[7];
      walls(n, o, sw[q], rr);
#pragma unroll
      for (int d = 0; d < 7; ++d) res[d][q] = rr[d];
    } else {
#pragma unroll
      for (int d = 0; d < 7; ++d) res[d][q] = o[d];
    }
  }

  if (inflow0) {  // inflow re-seed of the leftmost columns (src/gpu.rs:296-306)
#pragma unroll
    for (int q = 0; q < V; ++q) {
      const uint32_t j = j0 + q;
      if (j < dm.iw) {
        const uint32_t span = min(dm.inlet_cols - j * 32u, 32u);
        const uint32_t imask = (span >= 32u) ? 0xffffffffu : ((1u << span) - 1u);
        const uint32_t apply = imask & ~sw[q];
        const uint32_t* bern = inlet + ((size_t)y * dm.iw + j) * 7u;
#pragma unroll
        for (int d = 0; d < 7; ++d) {
          const uint32_t b = q == 0 ? bern0[d] : __ldg(bern + d);
          res[d][q] = (res[d][q] & ~apply) | (b & apply);
        }
      }
    }
  }
  if (last) {  // clear the bits past the row's end
#pragma unroll
    for (int d = 0; d < 7; ++d) res[d][V - 1] &= dm.tail;
  }
  if (live) {
#pragma unroll
    for (int d = 0; d < 7; ++d) *reinterpret_cast<VT*>(b + d * S + gq) = LW::make(res[d]);
  }
}

// The end of one field block's coarse-graining, from its exact sums and its
// running averages before the blend (u0, v0, r0): the sums out, the block's
// f32 velocity (Moments::velocity, src/moments.rs:91-97) and its blend into the
// averages with round-to-nearest intrinsics, so no fused multiply-add can
// change the last bit (lgca_sample, src/gpu.rs:324-377).
__device__ __forceinline__ void sample_finish(const SampleArgs& p, uint32_t blk, int mass, int px,
                                              int py, int nsolid, float u0, float v0, float r0) {
  constexpr float kSqrt3_2 = 0.8660254f;  // src/hex.rs:25
  const uint32_t nb = p.bw * p.bh;
  if (p.sums) {
    p.sums[blk] = mass;
    p.sums[nb + blk] = px;
    p.sums[2 * nb + blk] = py;
    p.sums[3 * nb + blk] = nsolid;
  }
  const float n = __uint2float_rn(p.bx * p.by);
  const float m = __int2float_rn(mass);
  float vx = 0.0f, vy = 0.0f;
  if (mass > 0) {
    vx = __fdiv_rn(__fmul_rn(__int2float_rn(px), 0.5f), m);
    vy = __fdiv_rn(__fmul_rn(__int2float_rn(py), kSqrt3_2), m);
  }
  const float a = p.alpha;
  p.ux[blk] = __fadd_rn(u0, __fmul_rn(a, __fsub_rn(vx, u0)));
  p.uy[blk] = __fadd_rn(v0, __fmul_rn(a, __fsub_rn(vy, v0)));
  p.rho[blk] = __fadd_rn(r0, __fmul_rn(a, __fsub_rn(__fdiv_rn(m, n), r0)));
  p.sol[blk] = __fdiv_rn(__int2float_rn(nsolid), n);
}

// Coarse-graining by tiles (SampleTiles): CTA `tile` takes `per` consecutive
// blocks of one block row; its lanes take the words those blocks' columns cover
// (one word per lane, so a warp's loads are coalesced) and its warps the block
// row's rows (every blockDim.x / 32-th row).  A word meets at most three blocks
// of kTileMinWidth or more columns; a thread sums, over its rows, its word's
// masked popcounts for each block it meets and adds them into the CTA's
// per-block totals in shared memory (acc), which a thread per block then
// finishes.  The totals are the same exact integers as sample_block's, so the
// field is the same; the warp per block there reads each word's 32-byte sector
// once per block that meets it, with lanes a row apart.  BATCH rows' words are
// loaded before any is counted, so their loads are in flight together.  The
// caller has let its dependents launch; this waits for the previous grid
// (griddepcontrol.wait) before it reads the state or the running averages
// (WAIT false: the caller has waited already).
__device__ __forceinline__ uint32_t bit_range(uint32_t lo, uint32_t hi) {  // bits [lo, hi)
  return hi - lo >= 32u ? 0xffffffffu : (((1u << (hi - lo)) - 1u) << lo);
}

template <int BATCH, bool WAIT = true>
__device__ __forceinline__ void sample_tile(const SampleArgs& p, uint32_t tile, uint32_t per,
                                            uint32_t ncx, int (*acc)[kTileMaxBlocks]) {
  const uint32_t t = threadIdx.x, rows = blockDim.x >> 5;
  for (uint32_t i = t; i < 4u * kTileMaxBlocks; i += blockDim.x) (&acc[0][0])[i] = 0;
  const uint32_t jb = tile / ncx, ib0 = (tile - jb * ncx) * per;
  const uint32_t nb = min(per, p.bw - ib0);
  const uint32_t fb = jb * p.bw + ib0;  // field index of the tile's first block
  __syncthreads();
  if (WAIT) asm volatile("griddepcontrol.wait;" ::: "memory");
  float u0 = 0.0f, v0 = 0.0f, r0 = 0.0f;
  if (t < nb) {
    u0 = p.ux[fb + t];
    v0 = p.uy[fb + t];
    r0 = p.rho[fb + t];
  }
  const uint32_t x0 = ib0 * p.bx, x1 = x0 + nb * p.bx;  // the tile's columns
  const uint32_t w0 = x0 >> 5, nw = ((x1 - 1u) >> 5) - w0 + 1u;
  const size_t S = p.dm.total;
  const size_t row0 = (size_t)jb * p.by;
  for (uint32_t wo = t & 31u; wo < nw; wo += 32u) {
    const uint32_t wi = w0 + wo;
    const uint32_t lo = max(x0, wi << 5), hi = min(x1, (wi << 5) + 32u);
    const uint32_t b0 = lo / p.bx;  // the first block the word meets
    uint32_t m[3];
#pragma unroll
    for (int s = 0; s < 3; ++s) {
      const uint32_t c0 = max(lo, (b0 + s) * p.bx), c1 = min(hi, (b0 + s + 1u) * p.bx);
      m[s] = c1 > c0 ? bit_range(c0 - (wi << 5), c1 - (wi << 5)) : 0u;
    }
    int mass[3] = {0, 0, 0}, px[3] = {0, 0, 0}, py[3] = {0, 0, 0}, ns[3] = {0, 0, 0};
    for (uint32_t rb = t >> 5; rb < p.by; rb += rows * BATCH) {
      uint32_t sw[BATCH], pl[BATCH][7];
#pragma unroll
      for (int q = 0; q < BATCH; ++q) {  // a row past the block row loads nothing, counts 0
        const uint32_t r = rb + q * rows;
        const size_t at = (row0 + r) * p.dm.wpr + wi;
        const bool in = r < p.by;
        sw[q] = in ? __ldg(p.solid + at) : 0u;
#pragma unroll
        for (int d = 0; d < 7; ++d) pl[q][d] = in ? __ldg(p.a + d * S + at) : 0u;
      }
#pragma unroll
      for (int q = 0; q < BATCH; ++q) {
#pragma unroll
        for (int s = 0; s < 3; ++s) {
          if (!m[s]) continue;  // most words meet one or two blocks
          const uint32_t sm = sw[q] & m[s];
          const uint32_t fm = m[s] & ~sm;
          ns[s] += __popc(sm);
          const int c0 = __popc(pl[q][0] & fm), c1 = __popc(pl[q][1] & fm);
          const int c2 = __popc(pl[q][2] & fm), c3 = __popc(pl[q][3] & fm);
          const int c4 = __popc(pl[q][4] & fm), c5 = __popc(pl[q][5] & fm);
          const int c6 = __popc(pl[q][6] & fm);
          mass[s] += c0 + c1 + c2 + c3 + c4 + c5 + c6;
          // CX2 = {2, 1, -1, -2, -1, 1}, CY2 = {0, 1, 1, 0, -1, -1}
          px[s] += 2 * (c0 - c3) + c1 - c2 - c4 + c5;
          py[s] += c1 + c2 - c4 - c5;
        }
      }
    }
#pragma unroll
    for (int s = 0; s < 3; ++s) {
      if (!m[s]) continue;
      const uint32_t k = b0 + s - ib0;
      atomicAdd(&acc[0][k], mass[s]);
      atomicAdd(&acc[1][k], px[s]);
      atomicAdd(&acc[2][k], py[s]);
      atomicAdd(&acc[3][k], ns[s]);
    }
  }
  __syncthreads();
  if (t < nb) sample_finish(p, fb + t, acc[0][t], acc[1][t], acc[2][t], acc[3][t], u0, v0, r0);
}

// Coarse-graining of field block `blk` of one lattice by one whole warp
// (lgca_sample, src/gpu.rs:324-377).  Lanes take rows of the block; each row
// contributes the masked popcounts of the one to several words the block's
// columns straddle.  The sums are exact 32-bit integers (mass, px2 = sum
// CX2 * count, py2, nsolid), reduced across the warp, and only then turned
// into f32 velocity and blended into the running average with
// round-to-nearest intrinsics, so no fused multiply-add can change the last
// bit (Moments::velocity, src/moments.rs:91).  EARLY: lane 0 reads the block's
// running averages before the planes, so the two reads' latencies overlap (the
// stand-alone sampling kernel; the resident kernels, short of registers, read
// them after the sums).
template <bool EARLY = false>
__device__ __forceinline__ void sample_block(const SampleArgs& p, uint32_t blk) {
  const uint32_t lane = threadIdx.x & 31u;
  float u0 = 0.0f, v0 = 0.0f, r0 = 0.0f;
  if (EARLY && lane == 0) {
    u0 = p.ux[blk];
    v0 = p.uy[blk];
    r0 = p.rho[blk];
  }
  const uint32_t jb = blk / p.bw, ib = blk - jb * p.bw;
  const uint32_t x0 = ib * p.bx, x1 = x0 + p.bx;
  const uint32_t w0 = x0 >> 5, w1 = (x1 - 1u) >> 5;
  const size_t S = p.dm.total;
  int mass = 0, px = 0, py = 0, nsolid = 0;
  for (uint32_t r = lane; r < p.by; r += 32u) {
    const size_t base = (size_t)(jb * p.by + r) * p.dm.wpr;
    for (uint32_t wi = w0; wi <= w1; ++wi) {
      const uint32_t lo = max(x0, wi << 5) - (wi << 5);
      const uint32_t hi = min(x1, (wi + 1u) << 5) - (wi << 5);
      const uint32_t m = (hi - lo >= 32u) ? 0xffffffffu : (((1u << (hi - lo)) - 1u) << lo);
      const uint32_t sm = __ldg(p.solid + base + wi) & m;
      nsolid += __popc(sm);
      const uint32_t fm = m & ~sm;
      const int c0 = __popc(__ldcg(p.a + 0 * S + base + wi) & fm);
      const int c1 = __popc(__ldcg(p.a + 1 * S + base + wi) & fm);
      const int c2 = __popc(__ldcg(p.a + 2 * S + base + wi) & fm);
      const int c3 = __popc(__ldcg(p.a + 3 * S + base + wi) & fm);
      const int c4 = __popc(__ldcg(p.a + 4 * S + base + wi) & fm);
      const int c5 = __popc(__ldcg(p.a + 5 * S + base + wi) & fm);
      const int c6 = __popc(__ldcg(p.a + 6 * S + base + wi) & fm);
      mass += c0 + c1 + c2 + c3 + c4 + c5 + c6;
      // CX2 = {2, 1, -1, -2, -1, 1}, CY2 = {0, 1, 1, 0, -1, -1}
      px += 2 * (c0 - c3) + c1 - c2 - c4 + c5;
      py += c1 + c2 - c4 - c5;
    }
  }
  const unsigned FULL = 0xffffffffu;
  mass = __reduce_add_sync(FULL, mass);
  px = __reduce_add_sync(FULL, px);
  py = __reduce_add_sync(FULL, py);
  nsolid = __reduce_add_sync(FULL, nsolid);
  if (lane != 0) return;
  if (!EARLY) {
    u0 = p.ux[blk];
    v0 = p.uy[blk];
    r0 = p.rho[blk];
  }
  sample_finish(p, blk, mass, px, py, nsolid, u0, v0, r0);
}

}  // namespace lgx
