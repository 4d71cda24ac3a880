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
#include "lgx_step_impl.cuh"

namespace lgx {

namespace {

// The single-step kernel's word-per-lane shapes, both compiled for six resident
// blocks per SM: 128-thread blocks with two consecutive 32-word chunks per warp
// (two independent word updates per thread for the scheduler to interleave:
// 7.69 -> 7.22 us per wake-run step, 95.6 -> 91.4 us at 16384 x 8192), and
// 256-thread blocks with one chunk per warp (twice the threads in flight, for
// lattices too small to fill the GPU).  The lane shapes (several consecutive
// words per lane, lgx_step_lanes_kernel) come after them.
constexpr uint32_t kTwoChunkMinWords = 152u * 6u * 256u;  // one wave of two-chunk blocks
constexpr int kWaveThreads = 256;  // the persistent kernel's blocks
// Resident blocks per SM the register allocation must allow: six 128-thread
// blocks of two chunks per warp (85 registers); four 256-thread blocks of one
// chunk per warp (64 registers: at six, 40 registers, the update spilled 72 bytes
// and a 2048 x 1280 step took 5.03 us against 3.57).
#ifndef LGX_STEP_MINB
#define LGX_STEP_MINB 6
#endif
#ifndef LGX_STEP_MINB1
#define LGX_STEP_MINB1 4
#endif

#ifndef LGX_WAVE_SLEEP
#define LGX_WAVE_SLEEP 1
#endif

// One step per launch, launched with programmatic stream serialisation.  The
// collision draws depend only on (word, seed, step), never on the lattice, so
// a block computes them first, lets the next step's grid start launching, and
// only then waits for the previous step's grid to finish and its writes to be
// visible (griddepcontrol.wait).  Step N+1's draws thereby fill the SMs that
// step N's last blocks leave idle.  Without a programmatic predecessor the
// wait returns at once, so the kernel is also correct launched plainly.
//
// SAMPLE: the grid ends with p.tiles.nblocks coarse-graining tiles of the
// state the step reads (sample_tile), which run beside the step's blocks; the
// step writes the other plane set, and the next grid waits for both.  Last, so
// that a step that fills the GPU in one wave starts whole and the tiles take
// the slots its blocks leave (wake run: 3.8-3.9 us per sample against 4.3-4.7
// with the tiles first).
template <bool REST, int WORDS, bool SAMPLE = false>
__global__ void __launch_bounds__(256 / WORDS, WORDS == 1 ? LGX_STEP_MINB1 : LGX_STEP_MINB)
    lgx_step_kernel(const StepArgs p) {
  const uint32_t bid = blockIdx.x;
  if (SAMPLE) {
    const uint32_t nstep = gridDim.x - p.tiles.nblocks;
    if (bid >= nstep) {
      asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
      __shared__ int acc[4][kTileMaxBlocks];
      sample_tile<WORDS == 1 ? 2 : 4>(p.tiles.s, bid - nstep, p.tiles.per, p.tiles.ncx, acc);
      return;
    }
  }
  // a warp takes WORDS consecutive 32-word chunks; a block covers 256 words
  constexpr int kStepWords = WORDS;
  const uint32_t g0 = bid * 256u + (threadIdx.x & ~31u) * kStepWords + (threadIdx.x & 31u);
  const uint32_t seed32 = step_seed32(p.seed, p.steps);
  uint32_t g[kStepWords];
  bool live[kStepWords];
  Draws s[kStepWords];
#pragma unroll
  for (int q = 0; q < kStepWords; ++q) {
    g[q] = g0 + 32u * q;
    live[q] = g[q] < p.dm.total;
    if (!live[q]) g[q] = p.dm.total - 1u;
    // Draws keyed on the lattice word, not the thread (src/gpu.rs:267-273).
    s[q] = draws(g[q] ^ seed32);
  }
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
  asm volatile("griddepcontrol.wait;" ::: "memory");
#pragma unroll
  for (int q = 0; q < kStepWords; ++q)
    step_word<REST, false>(p.a, p.b, p.solid, p.anysolid, p.inlet, p.dm, s[q], g[q], live[q]);
}

// One step per launch with V consecutive words per lane (V = 2 or 4; rows a
// whole number of V-word groups): a warp takes 32 V consecutive words, four
// warps a block.  All V draws of the lane come first, as above, then the
// planes arrive in 64- or 128-bit loads.  Four words per lane are compiled for
// four resident blocks (128 registers), two for six (80).  Measured against
// other choices on GB300 (us per step, wake run / 32768 x 16384): making the
// draws after the wait, 7.64 / 290.8 against 6.20 / 290.1 (the draws no longer
// fill the previous step's drain); half of them before it, 6.93 / 315;
// three resident blocks of 155 registers, 7.35 / 339; five of 96, draws
// after the wait, 9.11 / 290.1.  The hash outputs' shifts as multiplies on the
// FMA pipe: 6.03 / 297.0.  Two words per lane are allowed six blocks per SM (80
// registers), five with the inflow compiled in: at six it spilled 24 bytes, and a
// 2048 x 1280 step with an 8-column inflow took 4.55 us against 3.89.
// SAMPLE: coarse-graining tiles end the grid, as in lgx_step_kernel.
template <bool REST, int V, bool INFLOW, bool SAMPLE = false>
__global__ void __launch_bounds__(128, V == 4 ? 4 : (INFLOW ? 5 : 6))
    lgx_step_lanes_kernel(const StepArgs p) {
  const uint32_t bid = blockIdx.x;
  if (SAMPLE) {
    const uint32_t nstep = gridDim.x - p.tiles.nblocks;
    if (bid >= nstep) {
      asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
      __shared__ int acc[4][kTileMaxBlocks];
      sample_tile<4>(p.tiles.s, bid - nstep, p.tiles.per, p.tiles.ncx, acc);
      return;
    }
  }
  constexpr int E = V;  // draws made before the wait
  const uint32_t warp = bid * 4u + (threadIdx.x >> 5);
  uint32_t gq = warp * (32u * V) + (threadIdx.x & 31u) * V;
  const bool live = gq < p.dm.total;
  if (!live) gq = p.dm.total - V;
  const uint32_t seed32 = step_seed32(p.seed, p.steps);
  Draws s[E > 0 ? E : 1];
#pragma unroll
  for (int q = 0; q < E; ++q) s[q] = draws((gq + q) ^ seed32);
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
  asm volatile("griddepcontrol.wait;" ::: "memory");
  step_lane_words<REST, V, E, INFLOW>(p.a, p.b, p.solid, p.anysolid, p.inlet, p.dm, s, seed32,
                                      gq, live);
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
__global__ void __launch_bounds__(kWaveThreads) lgx_wave_kernel(const WaveArgs p) {
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
// across the seven planes (src/gpu.rs:300-305).  Launched with programmatic
// stream serialisation: the words depend only on (word, step), so a thread
// makes all seven while the step before it drains, and waits for that step's
// grid (griddepcontrol.wait) only to write them into the buffer the steps of
// the previous chunk read.  The next step waits for this grid in turn.
__global__ void __launch_bounds__(128) lgx_inlet_kernel(const InletArgs p) {
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
  const uint32_t per_step = p.dm.h * p.dm.iw;
  const uint32_t idx = blockIdx.x * blockDim.x + threadIdx.x;
  const bool live = idx < per_step * p.nsteps;
  const uint32_t i = live ? idx : 0u;
  const uint32_t s = i / per_step;
  const uint32_t rem = i - s * per_step;
  const uint32_t y = rem / p.dm.iw;
  const uint32_t jw = rem - y * p.dm.iw;
  const uint32_t word = y * p.dm.wpr + jw;
  uint32_t r = mix(word ^ step_seed32(p.seed, p.steps + s) ^ kGolden32);
  uint32_t v[7];
#pragma unroll
  for (int d = 0; d < 7; ++d) v[d] = bernoulli(p.thresh[d], r);
  asm volatile("griddepcontrol.wait;" ::: "memory");
  if (!live) return;
  uint32_t* out = p.out + (size_t)idx * 7u;
#pragma unroll
  for (int d = 0; d < 7; ++d) out[d] = v[d];
}

}  // namespace

// The shape by size: from one full wave of two-chunk blocks up, four words per
// lane where the rows allow it (wake run 7.07 -> 6.20 us per step, 32768 x
// 16384 347 -> 290 us), else two, else two chunks per warp; below that two
// words per lane where they fit (2048 x 1280: 5.04 -> 4.30 us), else one chunk.
uint32_t step_shape(const Dims& dm, uint32_t shape) {
  if (shape == kShapeLanes4 && dm.wpr % 4u == 0u) return shape;
  if (shape == kShapeLanes2 && dm.wpr % 2u == 0u) return shape;
  if (shape == kShapeChunk1 || shape == kShapeChunk2) return shape;
  if (dm.total >= kTwoChunkMinWords) {
    if (dm.wpr % 4u == 0u) return kShapeLanes4;
    return dm.wpr % 2u == 0u ? kShapeLanes2 : kShapeChunk2;
  }
  return dm.wpr % 2u == 0u ? kShapeLanes2 : kShapeChunk1;
}

template <bool S>
cudaError_t launch_shape(const cudaLaunchConfig_t& cfg, const StepArgs& s, uint32_t shape,
                         bool rest, bool in) {
  switch (shape) {
    case kShapeLanes4:
      if (in)
        return rest ? cudaLaunchKernelEx(&cfg, lgx_step_lanes_kernel<true, 4, true, S>, s)
                    : cudaLaunchKernelEx(&cfg, lgx_step_lanes_kernel<false, 4, true, S>, s);
      return rest ? cudaLaunchKernelEx(&cfg, lgx_step_lanes_kernel<true, 4, false, S>, s)
                  : cudaLaunchKernelEx(&cfg, lgx_step_lanes_kernel<false, 4, false, S>, s);
    case kShapeLanes2:
      if (in)
        return rest ? cudaLaunchKernelEx(&cfg, lgx_step_lanes_kernel<true, 2, true, S>, s)
                    : cudaLaunchKernelEx(&cfg, lgx_step_lanes_kernel<false, 2, true, S>, s);
      return rest ? cudaLaunchKernelEx(&cfg, lgx_step_lanes_kernel<true, 2, false, S>, s)
                  : cudaLaunchKernelEx(&cfg, lgx_step_lanes_kernel<false, 2, false, S>, s);
    case kShapeChunk2:
      return rest ? cudaLaunchKernelEx(&cfg, lgx_step_kernel<true, 2, S>, s)
                  : cudaLaunchKernelEx(&cfg, lgx_step_kernel<false, 2, S>, s);
    default:
      return rest ? cudaLaunchKernelEx(&cfg, lgx_step_kernel<true, 1, S>, s)
                  : cudaLaunchKernelEx(&cfg, lgx_step_kernel<false, 1, S>, s);
  }
}

cudaError_t launch_step(const StepArgs& s, bool rest, cudaStream_t st) {
  cudaLaunchConfig_t cfg = {};
  uint32_t shape = step_shape(s.dm, s.words);
  // The lane shapes move planes and obstacles in 64- or 128-bit accesses, so
  // they need those buffers 8- or 16-byte aligned.  The engine's own are; a
  // caller's (lgx_step_planes_noalloc) may be word-aligned only, and then the
  // word-per-lane shape of the same size runs.
  const uintptr_t al = (uintptr_t)s.a | (uintptr_t)s.b | (uintptr_t)s.solid;
  if ((shape == kShapeLanes4 && (al & 15u)) || (shape == kShapeLanes2 && (al & 7u)))
    shape = s.dm.total >= kTwoChunkMinWords ? kShapeChunk2 : kShapeChunk1;
  cfg.gridDim = dim3((s.dm.total + 255u) / 256u);
  cfg.blockDim = dim3(shape == kShapeChunk1 ? 256 : 128);
  if (shape == kShapeLanes2) cfg.gridDim = dim3((s.dm.total + 255u) / 256u);
  if (shape == kShapeLanes4) cfg.gridDim = dim3((s.dm.total + 511u) / 512u);
  cfg.dynamicSmemBytes = 0;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  // the lane shapes come with and without the inflow (its early loads cost
  // registers: 0.8% on 32768 x 16384 without one, against 2.9% gained on the
  // wake run and 5.7% at 1024 x 512 with one)
  const bool in = s.dm.iw != 0u;
  if (s.tiles.nblocks == 0u) return launch_shape<false>(cfg, s, shape, rest, in);
  cfg.gridDim.x += s.tiles.nblocks;
  return launch_shape<true>(cfg, s, shape, rest, in);
}

cudaError_t wave_grid(bool rest, uint32_t total, uint32_t* grid) {
  int dev = 0, sms = 0, per_sm = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (e == cudaSuccess)
    e = rest ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, lgx_wave_kernel<true>,
                                                             kWaveThreads, 0)
             : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, lgx_wave_kernel<false>,
                                                             kWaveThreads, 0);
  if (e != cudaSuccess) return e;
  const uint32_t nchunks = (total + 31u) / 32u;
  *grid = std::max<uint32_t>(1u, std::min<uint32_t>((uint32_t)(sms * per_sm), nchunks));
  return cudaSuccess;
}

cudaError_t launch_wave(const WaveArgs& w, bool rest, uint32_t grid, cudaStream_t st) {
  void* args[] = {(void*)&w};
  if (rest)
    return cudaLaunchCooperativeKernel((const void*)lgx_wave_kernel<true>, dim3(grid),
                                       dim3(kWaveThreads), args, 0, st);
  return cudaLaunchCooperativeKernel((const void*)lgx_wave_kernel<false>, dim3(grid),
                                     dim3(kWaveThreads), args, 0, st);
}

cudaError_t launch_inlet(const InletArgs& s, cudaStream_t st) {
  const uint32_t n = s.dm.h * s.dm.iw * s.nsteps;
  if (n == 0) return cudaSuccess;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((n + 127) / 128);
  cfg.blockDim = dim3(128);
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, lgx_inlet_kernel, s);
}

}  // namespace lgx
