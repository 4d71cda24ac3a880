// lgx_temporal.cu -- K steps per pass over HBM (temporal blocking).
//
// A warp owns a tile: a strip of 29 consecutive words of a row range
// [y0, y0 + R).  Its 32 lanes hold words a-2 .. a+29 (mod wpr): lanes 2..30
// are the strip, lanes 0, 1 and 31 are halo.  The warp walks down the rows
// y0-K .. y0+R+K-1, loading each input row once, and pushes it through K
// pipeline stages kept in registers: stage s turns rows r-1, r, r+1 of stage
// s-1 into row r of stage s, the horizontal neighbour bits coming from the
// adjacent lanes by shuffle.  Only stage K's rows inside the strip and the
// band are stored.  The result is bit-identical to K single steps.
//
// Why the halo suffices: a halo lane's outer neighbour is not computed, so
// its wrong bit enters at the lane's outer edge and moves inward one bit per
// stage; for K <= 30 it never reaches a strip lane.  Two halo lanes on the
// left keep the periodic wrap exact for any width: word 0's left neighbour is
// bit `lastbit` of the last word, which may hold a single valid bit, and that
// word's own left neighbour then has to be a full word held in registers.
// The bits of the last word past the row's end are never read into a valid
// bit (the shift from the right overwrites bit `lastbit` from word 0), so they
// are only masked off at the final store, as the single-step kernel does.
#include <algorithm>

#include "lgx_device.cuh"
#include "lgx_internal.hpp"

namespace lgx {
namespace {

constexpr int kTBThreads = 128;
constexpr uint32_t kStrip = 29;

// Window slots of one stage boundary: the newest row (all 7 planes), the row
// before it (planes 0, 1, 2, 3, 6 still needed) and the one before that
// (planes 1, 2).
struct Win {
  uint32_t c[7];           // row t
  uint32_t p0, p1, p2, p3, p6;  // row t-1
  uint32_t q1, q2;         // row t-2
};

__device__ __forceinline__ void push(Win& w, const uint32_t in[7]) {
  w.q1 = w.p1;
  w.q2 = w.p2;
  w.p0 = w.c[0];
  w.p1 = w.c[1];
  w.p2 = w.c[2];
  w.p3 = w.c[3];
  w.p6 = w.c[6];
#pragma unroll
  for (int d = 0; d < 7; ++d) w.c[d] = in[d];
}

// Row r = t-1 of the next stage from window w (rows t-2, t-1, t of this
// stage).  j is the lane's word, `valid` whether it is a real strip word.
template <bool REST>
__device__ __forceinline__ void stage_row(const Win& w, uint32_t r, uint32_t j, uint32_t seed32,
                                          const TemporalArgs& p, const uint32_t* inlet,
                                          uint32_t out[7]) {
  const Dims& dm = p.dm;
  const unsigned FULL = 0xffffffffu;
  const bool odd = r & 1u;
  // row r (= t-1): planes 0, 3, 6; row r-1 (= t-2): planes 1, 2; row r+1 (= t): 4, 5
  const uint32_t a0 = w.p0, a3 = w.p3, a6 = w.p6;
  const uint32_t b1 = w.q1, b2 = w.q2;
  const uint32_t c4 = w.c[4], c5 = w.c[5];
  const uint32_t l0 = __shfl_up_sync(FULL, a0, 1), l1 = __shfl_up_sync(FULL, b1, 1);
  const uint32_t l5 = __shfl_up_sync(FULL, c5, 1);
  const uint32_t q2 = __shfl_down_sync(FULL, b2, 1), q3 = __shfl_down_sync(FULL, a3, 1);
  const uint32_t q4 = __shfl_down_sync(FULL, c4, 1);
  // The lane to the left holds word j-1, or the last word when j == 0, whose
  // bit `lastbit` is the one that wraps (src/gpu.rs:256-261).
  const uint32_t lsh = (j == 0u) ? 31u - dm.lastbit : 0u;
  auto from_left = [&](uint32_t v, uint32_t left) { return __funnelshift_l(left << lsh, v, 1); };
  // The lane to the right holds word j+1, or word 0 when j is the last word,
  // whose bit 0 enters at bit `lastbit` (src/gpu.rs:248-254).
  auto from_right = [&](uint32_t v, uint32_t right) {
    uint32_t x = __funnelshift_r(v, right, 1);
    if (j == dm.lastword) x = (x & ~(1u << dm.lastbit)) | ((right & 1u) << dm.lastbit);
    return x;
  };
  uint32_t n[7];
  n[0] = from_left(a0, l0);
  n[3] = from_right(a3, q3);
  if (odd) {
    n[1] = b1;
    n[2] = from_right(b2, q2);
    n[4] = from_right(c4, q4);
    n[5] = c5;
  } else {
    n[1] = from_left(b1, l1);
    n[2] = b2;
    n[4] = c4;
    n[5] = from_left(c5, l5);
  }
  n[6] = a6;
  const uint32_t word = r * dm.wpr + j;
  const Draws s = draws(word ^ seed32);
  uint32_t o[7];
  collide<REST>(n, s, o);
  const uint32_t any = __ldg(p.anysolid + (word >> 5));
  uint32_t sm = 0u;
  if ((any >> (word & 31u)) & 1u) sm = __ldg(p.solid + word);
  walls(n, o, sm, out);
  if (j < dm.iw) {
    const uint32_t span = min(dm.inlet_cols - j * 32u, 32u);
    const uint32_t imask = (span >= 32u) ? 0xffffffffu : ((1u << span) - 1u);
    const uint32_t apply = imask & ~sm;
    const uint32_t* bern = inlet + ((size_t)r * dm.iw + j) * 7u;
#pragma unroll
    for (int d = 0; d < 7; ++d) out[d] = (out[d] & ~apply) | (__ldg(bern + d) & apply);
  }
}

template <int K, bool REST>
__global__ void __launch_bounds__(kTBThreads) lgx_temporal_kernel(const TemporalArgs p) {
  const Dims& dm = p.dm;
  const uint32_t lane = threadIdx.x & 31u;
  const uint32_t tile = blockIdx.x * (kTBThreads / 32) + (threadIdx.x >> 5);
  if (tile >= p.nstrips * p.nbands) return;  // whole warp
  const uint32_t strip = tile % p.nstrips, band = tile / p.nstrips;
  const uint32_t a = strip * kStrip;
  const uint32_t j = (a + lane + 2u * dm.wpr - 2u) % dm.wpr;
  const bool mine = lane >= 2u && lane <= 30u && a + lane - 2u < dm.wpr;
  const uint32_t y0 = band * p.band_rows, y1 = min(y0 + p.band_rows, dm.h);
  const size_t S = dm.total;

  Win win[K];
#pragma unroll
  for (int b = 0; b < K; ++b) {
#pragma unroll
    for (int d = 0; d < 7; ++d) win[b].c[d] = 0u;
    win[b].p0 = win[b].p1 = win[b].p2 = win[b].p3 = win[b].p6 = win[b].q1 = win[b].q2 = 0u;
  }
  const uint32_t nit = (y1 - y0) + 2u * K;
  for (uint32_t i = 0; i < nit; ++i) {
    // input row t = y0 - K + i (mod h)
    const uint32_t t = (y0 + dm.h * 2u - K + i) % dm.h;
    uint32_t row[7];
#pragma unroll
    for (int d = 0; d < 7; ++d) row[d] = __ldg(p.a + d * S + (size_t)t * dm.wpr + j);
    push(win[0], row);
    // stage s (1..K) computes row t - s once it has three rows of stage s-1
#pragma unroll
    for (int s = 1; s <= K; ++s) {
      if (i < 2u * s) break;
      const uint32_t r = (t + dm.h * 2u - s) % dm.h;
      const uint32_t* inlet = dm.iw ? p.inlet + (size_t)(s - 1) * dm.h * dm.iw * 7u : nullptr;
      uint32_t res[7];
      stage_row<REST>(win[s - 1], r, j, step_seed32(p.seed, p.steps + s - 1), p, inlet, res);
      if (s < K) {
        push(win[s], res);
      } else if (mine) {
        // the final stage's row r = y0 + i - 2K lies in [y0, y1) for i >= 2K
        if (j == dm.lastword && dm.tail != 0xffffffffu) {
#pragma unroll
          for (int d = 0; d < 7; ++d) res[d] &= dm.tail;
        }
#pragma unroll
        for (int d = 0; d < 7; ++d) p.b[d * S + (size_t)r * dm.wpr + j] = res[d];
      }
    }
  }
}

}  // namespace

bool temporal_supported(const Dims& dm, uint32_t k) {
  return dm.wpr >= 64u && (k == 4u || k == 8u);
}

cudaError_t launch_temporal(const TemporalArgs& t, bool rest, uint32_t k, cudaStream_t st) {
  const uint32_t tiles = t.nstrips * t.nbands;
  const uint32_t blocks = (tiles + kTBThreads / 32 - 1) / (kTBThreads / 32);
  if (k == 4) {
    if (rest)
      lgx_temporal_kernel<4, true><<<blocks, kTBThreads, 0, st>>>(t);
    else
      lgx_temporal_kernel<4, false><<<blocks, kTBThreads, 0, st>>>(t);
  } else if (k == 8) {
    if (rest)
      lgx_temporal_kernel<8, true><<<blocks, kTBThreads, 0, st>>>(t);
    else
      lgx_temporal_kernel<8, false><<<blocks, kTBThreads, 0, st>>>(t);
  } else {
    return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

// Bands of up to 128 rows, shorter when the lattice would give fewer than
// about 16 warps per SM (152 SMs), but at least 4k rows: each band also
// computes k rows of halo above and below.
void temporal_tiling(const Dims& dm, uint32_t k, TemporalArgs* t) {
  t->nstrips = (dm.wpr + kStrip - 1) / kStrip;
  const uint32_t fill = (uint32_t)(((uint64_t)dm.h * t->nstrips) / (152u * 16u));
  t->band_rows = std::max<uint32_t>(4u * k, std::min<uint32_t>(128u, fill));
  t->nbands = (dm.h + t->band_rows - 1) / t->band_rows;
}

}  // namespace lgx
