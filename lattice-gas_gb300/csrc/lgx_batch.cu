// lgx_batch.cu -- many lattices of uneven sizes advanced together.
//
// The reference advances one lattice per command buffer and, when it wants
// several (transport::measure's two measurements), one per host thread and
// Metal queue (src/transport.rs:299-313).  Small lattices cannot fill a GPU,
// so here one launch steps every lattice of a batch: blocks of 256 threads
// are laid over the concatenated word ranges (each lattice padded to whole
// blocks), a block finds its lattice by binary search over the per-lattice
// block prefix, and runs the same per-word update as the single-lattice
// kernel.  The step kernels are
// chained with programmatic dependent launch, a batched coarse-graining
// kernel samples every lattice's field, and a sampling interval's launches
// are captured once into a CUDA graph that is replayed for every interval:
// a device-side counter of batch steps (advanced by the graph's last node)
// gives each replay its step numbers, ping-pong parity and seeds.
#include <algorithm>

#include "lgx_batch.hpp"
#include "lgx_device.cuh"
#include "lgx_step_impl.cuh"

namespace lgx {
namespace {

// A block of the batched step covers 256 lattice words (the unit of the block
// tables): WORDS consecutive 32-word chunks per warp, 256 / WORDS threads,
// compiled for 4 * WORDS resident blocks per SM (64 registers).

template <bool REST>
// dm: the lattice's Dims copied into registers (read through d at every use, as
// the update reads them, they are loads from global memory on the step's path:
// one 2048 x 1280 lattice replayed from graphs ran 4.0 against 3.2 us per step).
__device__ __forceinline__ void batch_word(const LatDesc& d, const Dims& dm, uint64_t local,
                                           uint32_t k, uint32_t g, bool live, const Draws& s) {
  const uint32_t par = (d.cur0 + (uint32_t)local) & 1u;
  const uint32_t* src = par ? d.planes[1] : d.planes[0];
  uint32_t* dst = par ? d.planes[0] : d.planes[1];
  const uint32_t* inlet = dm.iw ? d.inlet + (size_t)k * dm.h * dm.iw * 7u : nullptr;
  step_word<REST, false>(src, dst, d.solid, d.anysolid, inlet, dm, s, g, live);
}

// One step of every lattice of one rule in the batch (blocks first_block ..
// first_block + gridDim.x - 1 of the block table).  `k` is the step's index
// within the captured interval; the batch step is *base + k.
// Largest i < n with prefix[i] <= x (prefix[0] == 0, non-decreasing): the
// entry that owns item x when entry i owns prefix[i] .. prefix[i+1] - 1.
__device__ __forceinline__ uint32_t owner_of(const uint32_t* prefix, uint32_t n, uint32_t x) {
  uint32_t lo = 0, hi = n;
  while (hi - lo > 1u) {
    const uint32_t mid = (lo + hi) >> 1;
    if (__ldg(prefix + mid) <= x) lo = mid; else hi = mid;
  }
  return lo;
}

// One step of the lattice words a block covers; RULE: 0 six-direction, 1 rest
// particles, 2 the lattice's own (a block belongs to one lattice, so the rule
// is uniform across it: one launch serves a batch mixing both).
template <int RULE, int WORDS>
__device__ __forceinline__ void batch_block(const BatchStepArgs& p) {
  const uint32_t blk = p.first_block + blockIdx.x;
  const uint32_t li = p.owner ? __ldg(p.owner + blk) : owner_of(p.block0, p.nlat, blk);
  const LatDesc& d = p.descs[li];
  const Dims dm = d.dm;
  const uint32_t g0 = (blk - __ldg(p.block0 + li)) * 256u + (threadIdx.x & ~31u) * WORDS +
                      (threadIdx.x & 31u);
  const uint64_t local = *p.base + p.k;
  const uint32_t seed32 = step_seed32(d.seed, d.steps0 + local);
  uint32_t g[WORDS];
  bool live[WORDS];
  Draws s[WORDS];
#pragma unroll
  for (int q = 0; q < WORDS; ++q) {
    g[q] = g0 + 32u * q;
    live[q] = g[q] < dm.total;
    if (!live[q]) g[q] = dm.total - 1u;
    s[q] = draws(g[q] ^ seed32);
  }
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
  asm volatile("griddepcontrol.wait;" ::: "memory");
#pragma unroll
  for (int q = 0; q < WORDS; ++q) {
    if (RULE == 2 ? d.rest != 0 : RULE == 1)
      batch_word<true>(d, dm, local, p.k, g[q], live[q], s[q]);
    else
      batch_word<false>(d, dm, local, p.k, g[q], live[q], s[q]);
  }
}

template <int RULE, int WORDS>
__global__ void __launch_bounds__(256 / WORDS, 4 * WORDS) lgx_batch_step_kernel(BatchStepArgs p) {
  batch_block<RULE, WORDS>(p);
}

// The same step with two consecutive words per lane (128 threads, 64-bit plane
// accesses; a block still covers 256 words, so the block tables are the
// same).  A block of a lattice whose words per row are odd runs the two-chunk
// mapping instead (the branch is uniform across the block).
// V consecutive words per lane from word gq of lattice d (all 32 lanes of the
// warp together), the draws made before the wait on the previous step.
template <int RULE, int V, bool INFLOW>
__device__ __forceinline__ void batch_lane_words(const BatchStepArgs& p, const LatDesc& d,
                                                 uint32_t gq) {
  const Dims dm = d.dm;  // in registers (batch_word)
  const bool live = gq < dm.total;
  if (!live) gq = dm.total - V;
  const uint64_t local = *p.base + p.k;
  const uint32_t seed32 = step_seed32(d.seed, d.steps0 + local);
  Draws s[V];
#pragma unroll
  for (int q = 0; q < V; ++q) s[q] = draws((gq + q) ^ seed32);
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
  asm volatile("griddepcontrol.wait;" ::: "memory");
  const uint32_t par = (d.cur0 + (uint32_t)local) & 1u;
  const uint32_t* src = par ? d.planes[1] : d.planes[0];
  uint32_t* dst = par ? d.planes[0] : d.planes[1];
  const uint32_t* inlet = dm.iw ? d.inlet + (size_t)p.k * dm.h * dm.iw * 7u : nullptr;
  if (RULE == 2 ? d.rest != 0 : RULE == 1)
    step_lane_words<true, V, V, INFLOW>(src, dst, d.solid, d.anysolid, inlet, dm, s, seed32, gq,
                                        live);
  else
    step_lane_words<false, V, V, INFLOW>(src, dst, d.solid, d.anysolid, inlet, dm, s, seed32,
                                         gq, live);
}

// Four consecutive words per lane in 64-thread blocks (256 words a block).  A
// block of a lattice whose words per row are not a multiple of four takes four
// 32-word chunks per warp instead.
template <int RULE, bool INFLOW>
__global__ void __launch_bounds__(64, 8) lgx_batch_lanes4_kernel(BatchStepArgs p) {
  const uint32_t blk = p.first_block + blockIdx.x;
  const uint32_t li = p.owner ? __ldg(p.owner + blk) : owner_of(p.block0, p.nlat, blk);
  const LatDesc& d = p.descs[li];
  if (d.dm.wpr & 3u) {
    batch_block<RULE, 4>(p);
    return;
  }
  batch_lane_words<RULE, 4, INFLOW>(p, d, (blk - __ldg(p.block0 + li)) * 256u + threadIdx.x * 4u);
}

// Six blocks per SM for launches of a wave or more (five cost the transport sweep
// 1272 -> 1209 Gsite/s); launches of less than one wave of such blocks, which are
// latency-bound, take a five-block build with room for more registers (with the
// inflow compiled in, the six-block build spilled: one 2048 x 1280 lattice with an
// inflow replayed from graphs, 4.95 -> 4.01 us per step; without one, 3.70 -> 3.41).
template <int RULE, bool INFLOW, int MINB = 6>
__global__ void __launch_bounds__(128, MINB) lgx_batch_lanes_kernel(BatchStepArgs p) {
  const uint32_t blk = p.first_block + blockIdx.x;
  const uint32_t li = p.owner ? __ldg(p.owner + blk) : owner_of(p.block0, p.nlat, blk);
  const LatDesc& d = p.descs[li];
  const Dims dm = d.dm;  // in registers (batch_word)
  if (dm.wpr & 1u) {
    batch_block<RULE, 2>(p);
    return;
  }
  uint32_t gq = (blk - __ldg(p.block0 + li)) * 256u + threadIdx.x * 2u;
  const bool live = gq < dm.total;
  if (!live) gq = dm.total - 2u;
  const uint64_t local = *p.base + p.k;
  const uint32_t seed32 = step_seed32(d.seed, d.steps0 + local);
  Draws s[2];
  s[0] = draws(gq ^ seed32);
  s[1] = draws((gq + 1u) ^ seed32);
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
  asm volatile("griddepcontrol.wait;" ::: "memory");
  const uint32_t par = (d.cur0 + (uint32_t)local) & 1u;
  const uint32_t* src = par ? d.planes[1] : d.planes[0];
  uint32_t* dst = par ? d.planes[0] : d.planes[1];
  const uint32_t* inlet = dm.iw ? d.inlet + (size_t)p.k * dm.h * dm.iw * 7u : nullptr;
  if (RULE == 2 ? d.rest != 0 : RULE == 1)
    step_lane_words<true, 2, 2, INFLOW>(src, dst, d.solid, d.anysolid, inlet, dm, s, seed32, gq,
                                        live);
  else
    step_lane_words<false, 2, 2, INFLOW>(src, dst, d.solid, d.anysolid, inlet, dm, s, seed32,
                                         gq, live);
}

// Inlet draws for steps base .. base + nsteps - 1 of every lattice with an
// inlet: one thread per (lattice, step, row, inlet word).
__global__ void __launch_bounds__(128) lgx_batch_inlet_kernel(BatchInletArgs p) {
  const uint32_t idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= p.total_items) return;
  const uint32_t lo = owner_of(p.item0, p.nlat, idx);
  const LatDesc& d = p.descs[lo];
  const uint32_t per_step = d.dm.h * d.dm.iw;
  const uint32_t rel = idx - p.item0[lo];
  const uint32_t s = rel / per_step;
  const uint32_t rem = rel - s * per_step;
  const uint32_t y = rem / d.dm.iw;
  const uint32_t jw = rem - y * d.dm.iw;
  const uint32_t word = y * d.dm.wpr + jw;
  const uint64_t local = *p.base + s;
  uint32_t r = mix(word ^ step_seed32(d.seed, d.steps0 + local) ^ kGolden32);
  uint32_t* out = d.inlet + (size_t)rel * 7u;
#pragma unroll 1
  for (int k = 0; k < 7; ++k) out[k] = bernoulli(d.thresh[k], r);
}

// Coarse-graining of every lattice with a field: one warp per field block,
// the lattice found by binary search over the block prefix.  The state read
// is the one after batch step *base + k_after.  Launched with programmatic
// stream serialisation, as the one-lattice sampling kernel is: the next step's
// grid may start its draws at once; this one waits for the step before it.
__global__ void __launch_bounds__(256) lgx_batch_sample_kernel(BatchSampleArgs p) {
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
  asm volatile("griddepcontrol.wait;" ::: "memory");
  const uint32_t task = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (task >= p.total_blocks) return;
  const uint32_t lo = owner_of(p.blk0, p.nlat, task);
  const LatDesc& d = p.descs[lo];
  const uint64_t local = *p.base + p.k_after;
  const uint32_t par = (d.cur0 + (uint32_t)local) & 1u;
  SampleArgs sa;
  sa.a = par ? d.planes[1] : d.planes[0];
  sa.solid = d.solid;
  sa.dm = d.dm;
  sa.bx = d.bx;
  sa.by = d.by;
  sa.bw = d.bw;
  sa.bh = d.bh;
  sa.alpha = d.alpha;
  const uint32_t nb = d.bw * d.bh;
  sa.ux = d.field;
  sa.uy = d.field + nb;
  sa.rho = d.field + 2 * nb;
  sa.sol = d.field + 3 * nb;
  sa.sums = d.sums;
  sample_block<true>(sa, task - p.blk0[lo]);
}

// The same for the lattices whose fields are coarse-grained by tiles: a CTA
// per tile (sample_tile), its lattice found by binary search over the tile
// prefix.
__global__ void __launch_bounds__(256) lgx_batch_sample_tiles_kernel(BatchSampleArgs p) {
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
  asm volatile("griddepcontrol.wait;" ::: "memory");
  __shared__ int acc[4][kTileMaxBlocks];
  const uint32_t lo = owner_of(p.tile0, p.nlat, blockIdx.x);
  const LatDesc& d = p.descs[lo];
  const uint64_t local = *p.base + p.k_after;
  const uint32_t par = (d.cur0 + (uint32_t)local) & 1u;
  SampleArgs sa;
  sa.a = par ? d.planes[1] : d.planes[0];
  sa.solid = d.solid;
  sa.dm = d.dm;
  sa.bx = d.bx;
  sa.by = d.by;
  sa.bw = d.bw;
  sa.bh = d.bh;
  sa.alpha = d.alpha;
  const uint32_t nb = d.bw * d.bh;
  sa.ux = d.field;
  sa.uy = d.field + nb;
  sa.rho = d.field + 2 * nb;
  sa.sol = d.field + 3 * nb;
  sa.sums = d.sums;
  uint32_t per, ncx;
  tile_shape(d.bx, d.bw, &per, &ncx);
  sample_tile<4, false>(sa, blockIdx.x - p.tile0[lo], per, ncx, acc);
}

__global__ void lgx_batch_base_kernel(uint64_t* base, uint32_t n) { *base += n; }

__global__ void lgx_batch_owner_kernel(const uint32_t* block0, uint32_t nlat, uint32_t nblocks,
                                       uint32_t* owner) {
  const uint32_t b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b < nblocks) owner[b] = owner_of(block0, nlat, b);
}

}  // namespace

cudaError_t launch_batch_step(const BatchStepArgs& a, uint32_t nblocks, int rule, int words,
                              cudaStream_t st) {
  const bool inflow = (words & kBatchNoInflow) == 0;
  words &= ~kBatchNoInflow;
  if (words == 0) words = kBatchLanes2;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(nblocks);
  cfg.blockDim = dim3(words == 1 ? 256 : words == kBatchLanes4 ? 64 : 128);
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  if (words == kBatchLanes4) {
    if (inflow) {
      if (rule == kRuleMixed) return cudaLaunchKernelEx(&cfg, lgx_batch_lanes4_kernel<2, true>, a);
      if (rule == kRuleRest) return cudaLaunchKernelEx(&cfg, lgx_batch_lanes4_kernel<1, true>, a);
      return cudaLaunchKernelEx(&cfg, lgx_batch_lanes4_kernel<0, true>, a);
    }
    if (rule == kRuleMixed) return cudaLaunchKernelEx(&cfg, lgx_batch_lanes4_kernel<2, false>, a);
    if (rule == kRuleRest) return cudaLaunchKernelEx(&cfg, lgx_batch_lanes4_kernel<1, false>, a);
    return cudaLaunchKernelEx(&cfg, lgx_batch_lanes4_kernel<0, false>, a);
  }
  if (words == kBatchLanes2) {
    if (inflow && nblocks < 152u * 6u) {
      if (rule == kRuleMixed)
        return cudaLaunchKernelEx(&cfg, lgx_batch_lanes_kernel<2, true, 5>, a);
      if (rule == kRuleRest) return cudaLaunchKernelEx(&cfg, lgx_batch_lanes_kernel<1, true, 5>, a);
      return cudaLaunchKernelEx(&cfg, lgx_batch_lanes_kernel<0, true, 5>, a);
    }
    if (inflow) {
      if (rule == kRuleMixed) return cudaLaunchKernelEx(&cfg, lgx_batch_lanes_kernel<2, true>, a);
      if (rule == kRuleRest) return cudaLaunchKernelEx(&cfg, lgx_batch_lanes_kernel<1, true>, a);
      return cudaLaunchKernelEx(&cfg, lgx_batch_lanes_kernel<0, true>, a);
    }
    if (nblocks < 152u * 6u) {
      if (rule == kRuleMixed)
        return cudaLaunchKernelEx(&cfg, lgx_batch_lanes_kernel<2, false, 5>, a);
      if (rule == kRuleRest) return cudaLaunchKernelEx(&cfg, lgx_batch_lanes_kernel<1, false, 5>, a);
      return cudaLaunchKernelEx(&cfg, lgx_batch_lanes_kernel<0, false, 5>, a);
    }
    if (rule == kRuleMixed) return cudaLaunchKernelEx(&cfg, lgx_batch_lanes_kernel<2, false>, a);
    if (rule == kRuleRest) return cudaLaunchKernelEx(&cfg, lgx_batch_lanes_kernel<1, false>, a);
    return cudaLaunchKernelEx(&cfg, lgx_batch_lanes_kernel<0, false>, a);
  }
  if (words == 2) {
    if (rule == kRuleMixed) return cudaLaunchKernelEx(&cfg, lgx_batch_step_kernel<2, 2>, a);
    if (rule == kRuleRest) return cudaLaunchKernelEx(&cfg, lgx_batch_step_kernel<1, 2>, a);
    return cudaLaunchKernelEx(&cfg, lgx_batch_step_kernel<0, 2>, a);
  }
  if (rule == kRuleMixed) return cudaLaunchKernelEx(&cfg, lgx_batch_step_kernel<2, 1>, a);
  if (rule == kRuleRest) return cudaLaunchKernelEx(&cfg, lgx_batch_step_kernel<1, 1>, a);
  return cudaLaunchKernelEx(&cfg, lgx_batch_step_kernel<0, 1>, a);
}

cudaError_t launch_batch_inlet(const BatchInletArgs& a, cudaStream_t st) {
  if (a.total_items == 0) return cudaSuccess;
  lgx_batch_inlet_kernel<<<(a.total_items + 127) / 128, 128, 0, st>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_batch_sample(const BatchSampleArgs& a, cudaStream_t st) {
  cudaLaunchConfig_t cfg = {};
  cfg.blockDim = dim3(256);
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  cudaError_t e = cudaSuccess;
  if (a.total_blocks) {
    cfg.gridDim = dim3((a.total_blocks + 7) / 8);
    e = cudaLaunchKernelEx(&cfg, lgx_batch_sample_kernel, a);
  }
  if (e == cudaSuccess && a.total_tiles) {
    cfg.gridDim = dim3(a.total_tiles);
    e = cudaLaunchKernelEx(&cfg, lgx_batch_sample_tiles_kernel, a);
  }
  return e;
}

cudaError_t launch_batch_owner(const uint32_t* block0, uint32_t nlat, uint32_t nblocks,
                               uint32_t* owner, cudaStream_t st) {
  if (nblocks == 0) return cudaSuccess;
  lgx_batch_owner_kernel<<<(nblocks + 255) / 256, 256, 0, st>>>(block0, nlat, nblocks, owner);
  return cudaGetLastError();
}

cudaError_t launch_batch_base(uint64_t* base, uint32_t n, cudaStream_t st) {
  lgx_batch_base_kernel<<<1, 1, 0, st>>>(base, n);
  return cudaGetLastError();
}

}  // namespace lgx
