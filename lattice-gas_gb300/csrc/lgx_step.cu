// lgx_step.cu -- the bitplane step kernel and the inlet draw kernel.
//
// One thread per 32-cell lattice word, threads laid over the words in the
// order they sit in memory (y * wpr + j), so a warp covers 32 consecutive
// words of one or two rows.  Each thread loads its own word of the seven
// planes from the three rows the hexagonal gather reads (row y-1: planes 1, 2;
// row y: planes 0, 3, 6; row y+1: planes 4, 5), and the one bit it needs from
// each horizontal neighbour comes from the neighbouring lane by a warp
// shuffle; only lanes at a warp edge or a row end load it from memory.  The
// word then goes through the selector draws, the generated LOP3 collision,
// bounce-back, the inlet blend and the tail mask, and is stored.
//
// Semantics follow lgca_step (src/gpu.rs:203-310) bit for bit; the inlet's
// Bernoulli words, which depend only on (word, step) and not on the state, are
// drawn ahead by lgx_inlet_kernel so that no warp of the step runs a
// 168-hash chain for one lane while 31 wait.
#include "lgx_device.cuh"
#include "lgx_internal.hpp"

namespace lgx {

namespace {

#ifndef LGX_STEP_THREADS
#define LGX_STEP_THREADS 256
#endif
constexpr int kStepThreads = LGX_STEP_THREADS;

// Word to the left of `j` in the same row, with the row's periodic wrap: for
// j == 0 the bit that enters is bit `lastbit` of the last word, placed at 31.
__device__ __forceinline__ uint32_t left_word(const uint32_t* __restrict__ row, uint32_t j,
                                              bool in_warp, uint32_t shuffled,
                                              const Dims& dm) {
  if (in_warp) return shuffled;
  if (j > 0) return __ldg(row + j - 1);
  return __ldg(row + dm.lastword) << (31u - dm.lastbit);
}

// Bits x+1 into x: (w >> 1) | (next << 31), and on the last word of the row
// the bit at `lastbit` comes from bit 0 of word 0 (src/gpu.rs:248-254).
__device__ __forceinline__ uint32_t shift_from_right(uint32_t w, const uint32_t* __restrict__ row,
                                                     uint32_t j, bool in_warp, uint32_t shuffled,
                                                     const Dims& dm) {
  uint32_t hi = in_warp ? shuffled : ((j + 1u < dm.wpr) ? __ldg(row + j + 1u) : 0u);
  uint32_t v = __funnelshift_r(w, hi, 1);
  if (j == dm.lastword) v = (v & ~(1u << dm.lastbit)) | ((__ldg(row) & 1u) << dm.lastbit);
  return v;
}

template <bool REST>
__global__ void __launch_bounds__(kStepThreads) lgx_step_kernel(const StepArgs p) {
  const Dims& dm = p.dm;
  const uint32_t lane = threadIdx.x & 31u;
  uint32_t g = blockIdx.x * kStepThreads + threadIdx.x;
  const bool live = g < dm.total;
  if (!live) g = dm.total - 1u;  // idle lanes still take part in the shuffles

  const uint32_t y = g / dm.wpr;
  const uint32_t j = g - y * dm.wpr;
  const bool odd = y & 1u;
  const uint32_t ym = (y == 0u) ? dm.h - 1u : y - 1u;
  const uint32_t yp = (y + 1u == dm.h) ? 0u : y + 1u;
  const uint32_t* __restrict__ a = p.a;
  const size_t S = dm.total;

  const uint32_t* r0 = a + 0 * S + (size_t)y * dm.wpr;
  const uint32_t* r1 = a + 1 * S + (size_t)ym * dm.wpr;
  const uint32_t* r2 = a + 2 * S + (size_t)ym * dm.wpr;
  const uint32_t* r3 = a + 3 * S + (size_t)y * dm.wpr;
  const uint32_t* r4 = a + 4 * S + (size_t)yp * dm.wpr;
  const uint32_t* r5 = a + 5 * S + (size_t)yp * dm.wpr;

  const uint32_t w0 = __ldg(r0 + j), w1 = __ldg(r1 + j), w2 = __ldg(r2 + j);
  const uint32_t w3 = __ldg(r3 + j), w4 = __ldg(r4 + j), w5 = __ldg(r5 + j);
  const uint32_t w6 = __ldg(a + 6 * S + g);

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
  n[0] = __funnelshift_l(left_word(r0, j, lok, l0, dm), w0, 1);
  n[3] = shift_from_right(w3, r3, j, rok, q3, dm);
  if (odd) {
    n[1] = w1;
    n[2] = shift_from_right(w2, r2, j, rok, q2, dm);
    n[4] = shift_from_right(w4, r4, j, rok, q4, dm);
    n[5] = w5;
  } else {
    n[1] = __funnelshift_l(left_word(r1, j, lok, l1, dm), w1, 1);
    n[2] = w2;
    n[4] = w4;
    n[5] = __funnelshift_l(left_word(r5, j, lok, l5, dm), w5, 1);
  }
  n[6] = w6;

  // Draws keyed on the lattice word, not the thread (src/gpu.rs:267-273).
  const Draws s = draws(g ^ step_seed32(p.seed, p.steps));
  uint32_t o[7];
  collide<REST>(n, s, o);

  uint32_t sm = 0u;
  if ((__ldg(p.anysolid + (g >> 5)) >> (g & 31u)) & 1u) sm = __ldg(p.solid + g);
  uint32_t res[7];
  walls(n, o, sm, res);

  if (j < dm.iw) {  // inflow re-seed of the leftmost columns (src/gpu.rs:296-306)
    const uint32_t span = min(dm.inlet_cols - j * 32u, 32u);
    const uint32_t imask = (span >= 32u) ? 0xffffffffu : ((1u << span) - 1u);
    const uint32_t apply = imask & ~sm;
    const uint32_t* bern = p.inlet + ((size_t)y * dm.iw + j) * 7u;
#pragma unroll
    for (int d = 0; d < 7; ++d) res[d] = (res[d] & ~apply) | (__ldg(bern + d) & apply);
  }

  const uint32_t mask = (j == dm.lastword) ? dm.tail : 0xffffffffu;
  if (live) {
#pragma unroll
    for (int d = 0; d < 7; ++d) p.b[d * S + g] = res[d] & mask;
  }
}

// One thread per (step, row, inlet word): the inflow's Bernoulli words for
// that step, the hash chain seeded by word ^ seed32 ^ 0x9e3779b9 and carried
// across the seven planes (src/gpu.rs:300-305).
__global__ void __launch_bounds__(128) lgx_inlet_kernel(const InletArgs p) {
  const uint32_t per_step = p.dm.h * p.dm.iw;
  const uint32_t idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= per_step * p.nsteps) return;
  const uint32_t s = idx / per_step;
  const uint32_t rem = idx - s * per_step;
  const uint32_t y = rem / p.dm.iw;
  const uint32_t jw = rem - y * p.dm.iw;
  const uint32_t word = y * p.dm.wpr + jw;
  uint32_t r = mix(word ^ step_seed32(p.seed, p.steps + s) ^ kGolden32);
  uint32_t* out = p.out + (size_t)idx * 7u;
#pragma unroll 1
  for (int d = 0; d < 7; ++d) out[d] = bernoulli(p.thresh[d], r);
}

}  // namespace

cudaError_t launch_step(const StepArgs& s, bool rest, cudaStream_t st) {
  const uint32_t blocks = (s.dm.total + kStepThreads - 1) / kStepThreads;
  if (rest)
    lgx_step_kernel<true><<<blocks, kStepThreads, 0, st>>>(s);
  else
    lgx_step_kernel<false><<<blocks, kStepThreads, 0, st>>>(s);
  return cudaGetLastError();
}

cudaError_t launch_inlet(const InletArgs& s, cudaStream_t st) {
  const uint32_t n = s.dm.h * s.dm.iw * s.nsteps;
  if (n == 0) return cudaSuccess;
  lgx_inlet_kernel<<<(n + 127) / 128, 128, 0, st>>>(s);
  return cudaGetLastError();
}

}  // namespace lgx
