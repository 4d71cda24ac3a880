// lgx_step.cu -- the bitplane step: a single-step kernel, a persistent
// multi-step kernel, and the inlet draw kernel.
//
// Both step kernels give a warp 32 consecutive lattice words (y * wpr + j),
// one or two rows' worth, lane = word.  Each lane loads its own word of the
// seven planes from the three rows the hexagonal gather reads (row y-1:
// planes 1, 2; row y: planes 0, 3, 6; row y+1: planes 4, 5), and the one bit
// it needs from each horizontal neighbour comes from the neighbouring lane by
// a warp shuffle; only lanes at a chunk edge or a row end load it.  The word
// then goes through the selector draws, the generated LOP3 collision,
// bounce-back, the inlet blend and the tail mask, and is stored.
//
// lgx_step_kernel runs one step per launch.  lgx_wave_kernel runs K steps per
// cooperative launch: every CTA owns an equal, contiguous range of 32-word
// chunks for all K steps, and before step s it waits (bounded) only for the
// CTAs owning the rows next to its own to publish step s-1.  No CTA ever
// recomputes another's rows, and there is no grid-wide barrier: the wave of
// steps moves through the lattice with local dependencies only.
//
// Semantics follow lgca_step (src/gpu.rs:203-310) bit for bit; the inlet's
// Bernoulli words, which depend only on (word, step) and not on the state, are
// drawn ahead by lgx_inlet_kernel so that no warp of the step runs a
// 168-hash chain for one lane while 31 wait.
#include <algorithm>

#include "lgx_device.cuh"
#include "lgx_internal.hpp"

namespace lgx {

namespace {

#ifndef LGX_STEP_THREADS
#define LGX_STEP_THREADS 256
#endif
constexpr int kStepThreads = LGX_STEP_THREADS;

#ifndef LGX_WAVE_SLEEP
#define LGX_WAVE_SLEEP 1
#endif

// Plane loads.  Within the persistent kernel the planes change between steps
// and are written by other SMs, so they are read through L2 (ld.global.cg);
// the single-step kernel may use the read-only path.
template <bool COHERENT>
__device__ __forceinline__ uint32_t ldp(const uint32_t* p) {
  if (COHERENT) return __ldcg(p);
  return __ldg(p);
}

// Word to the left of `j` in the same row, with the row's periodic wrap: for
// j == 0 the bit that enters is bit `lastbit` of the last word, placed at 31.
template <bool COHERENT>
__device__ __forceinline__ uint32_t left_word(const uint32_t* row, uint32_t j, bool in_warp,
                                              uint32_t shuffled, const Dims& dm) {
  if (in_warp) return shuffled;
  if (j > 0) return ldp<COHERENT>(row + j - 1);
  return ldp<COHERENT>(row + dm.lastword) << (31u - dm.lastbit);
}

// Bits x+1 into x: (w >> 1) | (next << 31), and on the last word of the row
// the bit at `lastbit` comes from bit 0 of word 0 (src/gpu.rs:248-254).
template <bool COHERENT>
__device__ __forceinline__ uint32_t shift_from_right(uint32_t w, const uint32_t* row, uint32_t j,
                                                     bool in_warp, uint32_t shuffled,
                                                     const Dims& dm) {
  uint32_t hi = in_warp ? shuffled : ((j + 1u < dm.wpr) ? ldp<COHERENT>(row + j + 1u) : 0u);
  uint32_t v = __funnelshift_r(w, hi, 1);
  if (j == dm.lastword)
    v = (v & ~(1u << dm.lastbit)) | ((ldp<COHERENT>(row) & 1u) << dm.lastbit);
  return v;
}

// One step of lattice word g (g clamped into range for idle lanes, which
// still take part in the shuffles; `live` lanes store).  All 32 lanes of the
// warp call this together with consecutive g.
template <bool REST, bool COHERENT>
__device__ __forceinline__ void step_word(const uint32_t* a, uint32_t* b,
                                          const uint32_t* __restrict__ solid,
                                          const uint32_t* __restrict__ anysolid,
                                          const uint32_t* __restrict__ inlet, const Dims& dm,
                                          const Draws& s, uint32_t g, bool live) {
  const uint32_t lane = threadIdx.x & 31u;
  const uint32_t y = g / dm.wpr;
  const uint32_t j = g - y * dm.wpr;
  const bool odd = y & 1u;
  const uint32_t ym = (y == 0u) ? dm.h - 1u : y - 1u;
  const uint32_t yp = (y + 1u == dm.h) ? 0u : y + 1u;
  const size_t S = dm.total;

  const uint32_t* r0 = a + 0 * S + (size_t)y * dm.wpr;
  const uint32_t* r1 = a + 1 * S + (size_t)ym * dm.wpr;
  const uint32_t* r2 = a + 2 * S + (size_t)ym * dm.wpr;
  const uint32_t* r3 = a + 3 * S + (size_t)y * dm.wpr;
  const uint32_t* r4 = a + 4 * S + (size_t)yp * dm.wpr;
  const uint32_t* r5 = a + 5 * S + (size_t)yp * dm.wpr;

  const uint32_t w0 = ldp<COHERENT>(r0 + j), w1 = ldp<COHERENT>(r1 + j);
  const uint32_t w2 = ldp<COHERENT>(r2 + j), w3 = ldp<COHERENT>(r3 + j);
  const uint32_t w4 = ldp<COHERENT>(r4 + j), w5 = ldp<COHERENT>(r5 + j);
  const uint32_t w6 = ldp<COHERENT>(a + 6 * S + g);

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
  n[0] = __funnelshift_l(left_word<COHERENT>(r0, j, lok, l0, dm), w0, 1);
  n[3] = shift_from_right<COHERENT>(w3, r3, j, rok, q3, dm);
  if (odd) {
    n[1] = w1;
    n[2] = shift_from_right<COHERENT>(w2, r2, j, rok, q2, dm);
    n[4] = shift_from_right<COHERENT>(w4, r4, j, rok, q4, dm);
    n[5] = w5;
  } else {
    n[1] = __funnelshift_l(left_word<COHERENT>(r1, j, lok, l1, dm), w1, 1);
    n[2] = w2;
    n[4] = w4;
    n[5] = __funnelshift_l(left_word<COHERENT>(r5, j, lok, l5, dm), w5, 1);
  }
  n[6] = w6;

  uint32_t o[7];
  collide<REST>(n, s, o);

  uint32_t sm = 0u;
  if ((__ldg(anysolid + (g >> 5)) >> (g & 31u)) & 1u) sm = __ldg(solid + g);
  uint32_t res[7];
  walls(n, o, sm, res);

  if (j < dm.iw) {  // inflow re-seed of the leftmost columns (src/gpu.rs:296-306)
    const uint32_t span = min(dm.inlet_cols - j * 32u, 32u);
    const uint32_t imask = (span >= 32u) ? 0xffffffffu : ((1u << span) - 1u);
    const uint32_t apply = imask & ~sm;
    const uint32_t* bern = inlet + ((size_t)y * dm.iw + j) * 7u;
#pragma unroll
    for (int d = 0; d < 7; ++d) res[d] = (res[d] & ~apply) | (__ldg(bern + d) & apply);
  }

  const uint32_t mask = (j == dm.lastword) ? dm.tail : 0xffffffffu;
  if (live) {
#pragma unroll
    for (int d = 0; d < 7; ++d) b[d * S + g] = res[d] & mask;
  }
}

// One step per launch, launched with programmatic stream serialisation.  The
// collision draws depend only on (word, seed, step), never on the lattice, so
// a block computes them first, lets the next step's grid start launching, and
// only then waits for the previous step's grid to finish and its writes to be
// visible (griddepcontrol.wait).  Step N+1's draws thereby fill the SMs that
// step N's last blocks leave idle.  Without a programmatic predecessor the
// wait returns at once, so the kernel is also correct launched plainly.
template <bool REST>
__global__ void __launch_bounds__(kStepThreads) lgx_step_kernel(const StepArgs p) {
  uint32_t g = blockIdx.x * kStepThreads + threadIdx.x;
  const bool live = g < p.dm.total;
  if (!live) g = p.dm.total - 1u;
  // Draws keyed on the lattice word, not the thread (src/gpu.rs:267-273).
  const Draws s = draws(g ^ step_seed32(p.seed, p.steps));
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
  asm volatile("griddepcontrol.wait;" ::: "memory");
  step_word<REST, false>(p.a, p.b, p.solid, p.anysolid, p.inlet, p.dm, s, g, live);
}

// ---- the persistent multi-step kernel ---------------------------------------

__device__ __forceinline__ uint32_t ld_acquire(const uint32_t* p) {
  uint32_t v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ void st_release(uint32_t* p, uint32_t v) {
  asm volatile("st.release.gpu.global.u32 [%0], %1;" : : "l"(p), "r"(v) : "memory");
}

// First chunk of CTA b when nchunks are split over nb CTAs as evenly as possible.
__device__ __forceinline__ uint32_t chunk_begin(uint32_t b, uint32_t nchunks, uint32_t nb) {
  return (uint32_t)(((uint64_t)b * nchunks) / nb);
}

// The CTA that owns chunk c (inverse of chunk_begin).
__device__ __forceinline__ uint32_t chunk_owner(uint32_t c, uint32_t nchunks, uint32_t nb) {
  return (uint32_t)((((uint64_t)c + 1u) * nb - 1u) / nchunks);
}

// The interval of CTAs owning row y (its first and last word).
__device__ __forceinline__ void row_owners(uint32_t y, const Dims& dm, uint32_t nchunks,
                                           uint32_t nb, uint32_t* lo, uint32_t* hi) {
  *lo = chunk_owner((y * dm.wpr) >> 5, nchunks, nb);
  *hi = chunk_owner((y * dm.wpr + dm.wpr - 1u) >> 5, nchunks, nb);
}

// Polls before a wait gives up: the first 256 are back to back, the rest
// sleep ~64 ns each, so the limit is a few hundred milliseconds -- far beyond
// any honest wait for a neighbour's step.
constexpr uint32_t kSpinLimit = 1u << 22;

template <bool REST>
__global__ void __launch_bounds__(kStepThreads) lgx_wave_kernel(const WaveArgs p) {
  const Dims& dm = p.dm;
  const uint32_t nb = gridDim.x, b = blockIdx.x;
  const uint32_t nchunks = (dm.total + 31u) >> 5;
  const uint32_t c0 = chunk_begin(b, nchunks, nb), c1 = chunk_begin(b + 1u, nchunks, nb);
  const uint32_t warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;

  // The CTAs whose rows this one reads: owners of the rows from one above its
  // first row to one below its last (with the periodic wrap in y).  Ownership
  // is monotonic in the word index, so each row range maps to an interval.
  __shared__ uint32_t dep_lo[3], dep_hi[3];
  __shared__ int bail;
  if (threadIdx.x == 0) {
    bail = 0;
    const uint32_t ya = (c0 * 32u) / dm.wpr;
    const uint32_t yb = (min(c1 * 32u, dm.total) - 1u) / dm.wpr;
    uint32_t lo, hi, t;
    row_owners(ya == 0u ? dm.h - 1u : ya - 1u, dm, nchunks, nb, &lo, &hi);
    dep_lo[0] = lo;
    dep_hi[0] = hi;
    row_owners(ya, dm, nchunks, nb, &lo, &t);
    row_owners(yb, dm, nchunks, nb, &t, &hi);
    dep_lo[1] = lo;
    dep_hi[1] = hi;
    row_owners(yb + 1u == dm.h ? 0u : yb + 1u, dm, nchunks, nb, &lo, &hi);
    dep_lo[2] = lo;
    dep_hi[2] = hi;
  }
  __syncthreads();

  for (uint32_t s = 1; s <= p.nsteps; ++s) {
    if (s > 1) {
      // Wait until every CTA whose rows we read has published step s-1
      // (which also means it no longer reads the rows we are about to
      // overwrite).  Bounded: on timeout or a peer's error, record and leave.
      for (int r = 0; r < 3; ++r) {
        const uint32_t lo = dep_lo[r], hi = dep_hi[r];
        for (uint32_t c = lo + threadIdx.x; c <= hi; c += blockDim.x) {
          if (c == b) continue;
          uint32_t spins = 0;
          while (ld_acquire(p.done + c) < s - 1u) {
            if (++spins > kSpinLimit || ld_acquire(p.error) != 0u) {
              atomicCAS(p.error, 0u, 1u);
              bail = 1;
              break;
            }
#if LGX_WAVE_SLEEP
            if (spins > 256u) __nanosleep(64);
#endif
          }
        }
      }
      __syncthreads();
      if (bail) return;
    }
    const bool odd_step = s & 1u;  // selects, not indexes: keeps p out of local memory
    const uint32_t* src = odd_step ? p.planes[0] : p.planes[1];
    uint32_t* dst = odd_step ? p.planes[1] : p.planes[0];
    const uint32_t* inlet = dm.iw ? p.inlet + (size_t)(s - 1u) * dm.h * dm.iw * 7u : nullptr;
    const uint32_t seed32 = step_seed32(p.seed, p.steps + s - 1u);
    for (uint32_t c = c0 + warp; c < c1; c += nwarps) {
      uint32_t g = c * 32u + (threadIdx.x & 31u);
      const bool live = g < dm.total;
      if (!live) g = dm.total - 1u;
      const Draws dr = draws(g ^ seed32);
      step_word<REST, true>(src, dst, p.solid, p.anysolid, inlet, dm, dr, g, live);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      __threadfence();
      st_release(p.done + b, s);
    }
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
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((s.dm.total + kStepThreads - 1) / kStepThreads);
  cfg.blockDim = dim3(kStepThreads);
  cfg.dynamicSmemBytes = 0;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  if (rest) return cudaLaunchKernelEx(&cfg, lgx_step_kernel<true>, s);
  return cudaLaunchKernelEx(&cfg, lgx_step_kernel<false>, s);
}

cudaError_t wave_grid(bool rest, uint32_t total, uint32_t* grid) {
  int dev = 0, sms = 0, per_sm = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (e == cudaSuccess)
    e = rest ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, lgx_wave_kernel<true>,
                                                             kStepThreads, 0)
             : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, lgx_wave_kernel<false>,
                                                             kStepThreads, 0);
  if (e != cudaSuccess) return e;
  const uint32_t nchunks = (total + 31u) / 32u;
  *grid = std::max<uint32_t>(1u, std::min<uint32_t>((uint32_t)(sms * per_sm), nchunks));
  return cudaSuccess;
}

cudaError_t launch_wave(const WaveArgs& w, bool rest, uint32_t grid, cudaStream_t st) {
  void* args[] = {(void*)&w};
  if (rest)
    return cudaLaunchCooperativeKernel((const void*)lgx_wave_kernel<true>, dim3(grid),
                                       dim3(kStepThreads), args, 0, st);
  return cudaLaunchCooperativeKernel((const void*)lgx_wave_kernel<false>, dim3(grid),
                                     dim3(kStepThreads), args, 0, st);
}

cudaError_t launch_inlet(const InletArgs& s, cudaStream_t st) {
  const uint32_t n = s.dm.h * s.dm.iw * s.nsteps;
  if (n == 0) return cudaSuccess;
  lgx_inlet_kernel<<<(n + 127) / 128, 128, 0, st>>>(s);
  return cudaGetLastError();
}

}  // namespace lgx
