// lgx_batch.hpp -- device-side descriptors of a batch of lattices.
#pragma once

#include "../../include/lgx.h"
#include "lgx_internal.hpp"

namespace lgx {

// One lattice as the batched kernels see it.  After batch step `local` its
// state lives in planes[(cur0 + local) & 1].
struct LatDesc {
  uint32_t* planes[2];
  const uint32_t* solid;
  const uint32_t* anysolid;
  uint32_t* inlet;  // draws for the steps of the current interval, [k][h][iw][7]
  Dims dm;
  uint64_t seed;
  uint64_t steps0;  // the lattice's step count when the batch was set up
  uint32_t cur0;
  uint32_t rest;
  uint32_t thresh[7];
  float* field;     // ux | uy | rho | sol, bw*bh each; null without a field
  int32_t* sums;
  uint32_t bx, by, bw, bh;
  float alpha;
};

struct BatchStepArgs {
  const LatDesc* descs;
  const uint32_t* block0;  // prefix of per-lattice 256-word blocks, nlat + 1 entries
  const uint32_t* owner;   // lattice of each block (null: binary search of block0)
  uint32_t nlat;
  const uint64_t* base;    // batch steps completed before this interval
  uint32_t k;              // step index within the interval
  uint32_t first_block;    // this launch's first block (rest lattices come first)
};

struct BatchInletArgs {
  const LatDesc* descs;
  const uint32_t* item0;  // prefix of per-lattice draw items, nlat + 1 entries
  uint32_t nlat;
  uint32_t total_items;
  const uint64_t* base;
};

struct BatchSampleArgs {
  const LatDesc* descs;
  const uint32_t* blk0;  // prefix of per-lattice field blocks, nlat + 1 entries
  uint32_t nlat;
  uint32_t total_blocks;
  const uint64_t* base;
  uint32_t k_after;      // sample the state after batch step *base + k_after
  // lattices coarse-grained by tiles (blocks >= kTileMinWidth columns): the
  // prefix of their tile counts (tile_shape), nlat + 1 entries; their blocks
  // are not in blk0.  Null / 0: none.
  const uint32_t* tile0 = nullptr;
  uint32_t total_tiles = 0;
};

// Sampling schedule of a lattice within one resident launch: it is
// coarse-grained after step t (1-based) when since + t is a multiple of
// every, or t == left (its last step); every == 0: never.
struct ResSched {
  uint32_t every, since, left;
};

// `len` steps of lattices first_lat .. first_lat + nlat - 1 (of descs and
// sched), one thread-block cluster each, in one launch.  The batch step
// before the first of them is *base (null: 0); after local step t the state of
// a lattice is in planes[(cur0 + t) & 1].  Inlet draws as for the batched step.
// ksteps > 1 (with clusters of more than one CTA): up to ksteps steps between
// cluster barriers, each CTA keeping ksteps halo rows on either side of its
// band and recomputing them; 0 or 1: one cluster barrier per step.
struct ResidentArgs {
  const LatDesc* descs;
  const ResSched* sched;
  uint32_t first_lat;
  const uint64_t* base;
  uint32_t len;
  uint32_t ksteps;
};
bool resident_config_valid(uint32_t csize, uint32_t threads);
// Shared memory one CTA of a csize-CTA cluster holds for a lattice (both
// buffers of its band, with ksteps halo rows either side when ksteps > 1), and
// whether the lattice can run resident that way (every band at least ksteps rows).
constexpr size_t kResidentMaxSmem = 200u * 1024u;
size_t resident_smem_bytes(const Dims& dm, uint32_t csize, uint32_t ksteps = 1);
bool resident_fits(const Dims& dm, uint32_t csize, uint32_t ksteps = 1);
// The threads a CTA of the fixed-word resident kernels needs for a lattice
// (one word each: the whole lattice in one CTA, or a band with its recomputed
// halo rows under ksteps >= 2 steps per cluster barrier), or 0 where those
// kernels cannot hold it (a plane of a band over 1024 words; clusters of more
// than one CTA at one step per barrier).  A launch can take them when every
// lattice's count is nonzero and the largest fits its threads (at most 512).
constexpr uint32_t kResidentFixedMaxThreads = 512;
uint32_t resident_fixed_threads(const Dims& dm, uint32_t csize, uint32_t ksteps = 1);
bool resident_fixed_usable(uint32_t fixed_threads, uint32_t threads);
// Whether launch_resident takes the fixed-word kernels for a launch of this shape.
bool resident_runs_fixed(uint32_t fixed_threads, uint32_t csize, uint32_t threads,
                         uint32_t ksteps);
// LGX_RESIDENT_FIXED: 0 never the fixed-word kernels, 2 the tuner times only
// shapes that take them (where a class has any), 1 (unset) the tuner's choice.
int resident_fixed_mode();
cudaError_t launch_resident_fixed(const ResidentArgs& a, uint32_t nlat, uint32_t csize,
                                  uint32_t threads, cudaStream_t st);
// smem: dynamic shared memory per CTA, at least resident_smem_bytes of every
// lattice of the launch; fixed_threads: the largest resident_fixed_threads of
// them (0 if any is 0): the fixed-word kernels run where it fits the threads.
cudaError_t launch_resident(const ResidentArgs& a, uint32_t nlat, uint32_t csize,
                            uint32_t threads, size_t smem, uint32_t fixed_threads,
                            cudaStream_t st);

// The rule of the blocks a batched step launch covers.
constexpr int kRuleNoRest = 0, kRuleRest = 1, kRuleMixed = 2;
// words: 32-word chunks per warp (1: 256-thread blocks, 2: 128-thread blocks),
// or kBatchLanes2 (and 0): two consecutive words per lane in 128-thread blocks,
// lattices with an odd number of words per row taking two chunks per warp.  A
// block covers 256 words every way.  Two words per lane share one row's index
// and pointer work and load each plane in one 64-bit access: faster than either
// chunk shape at every size measured (transport sweep 1224 -> 1275
// Gsite-updates/s; eight 2048 x 1280 lattices 14.7 -> 12.8 us per step; eight
// 256 x 256 3.37 -> 3.05 us).
// kBatchLanes4: four words per lane in 64-thread blocks, for launches whose
// every lattice has a multiple of 4 words per row (a block of another lattice
// would take four chunks per warp, slow: the mixed-width transport sweep ran at
// 971 against 1276 Gsite-updates/s); it pays from one full wave of such blocks
// up (eight 2048 x 1280 lattices 12.76 -> 11.44 us per step, one 4096 x 2304
// 6.78 -> 5.97) and loses below it (one 2048 x 1280, 3.05 -> 5.26).
// kBatchNoInflow, or-ed in: no lattice of the launch has an inflow, so the
// lane kernels compiled without one run (the inflow's early loads cost
// registers: the transport sweep, which has none, ran at 1215 with them
// against 1275 Gsite-updates/s without).
constexpr int kBatchLanes2 = 3, kBatchLanes4 = 4, kBatchNoInflow = 0x10;
// The shape a batched step launch of `nblocks` 256-word blocks takes, given
// whether every lattice it covers has a multiple of 4 words per row and
// whether any has an inflow.
inline int batch_step_words(uint32_t nblocks, bool all_wpr4, bool any_inflow) {
  return (all_wpr4 && nblocks >= 152u * 8u ? kBatchLanes4 : kBatchLanes2) |
         (any_inflow ? 0 : kBatchNoInflow);
}
cudaError_t launch_batch_step(const BatchStepArgs& a, uint32_t nblocks, int rule, int words,
                              cudaStream_t st);
cudaError_t launch_batch_inlet(const BatchInletArgs& a, cudaStream_t st);
// owner[b] = the lattice whose blocks include block b, for b < nblocks.
cudaError_t launch_batch_owner(const uint32_t* block0, uint32_t nlat, uint32_t nblocks,
                               uint32_t* owner, cudaStream_t st);
cudaError_t launch_batch_sample(const BatchSampleArgs& a, cudaStream_t st);
cudaError_t launch_batch_base(uint64_t* base, uint32_t n, cudaStream_t st);

// Work enqueued inside the captured graphs, after every batch step
// (per_step) or once at the end of every interval that samples: called with
// the batch's stream, its device step counter for the interval and the step's
// index within the interval plus one (the state after batch step
// *base + k_after).  A per-step hook needs every lattice in one chain of
// per-step launches; an end-of-interval hook works with any policy.  Setting
// a hook drops the graphs captured without it.
typedef cudaError_t (*BatchStepHook)(void* ctx, cudaStream_t st, const uint64_t* base,
                                     uint32_t k_after);
int batch_set_step_hook(lgx_batch* b, BatchStepHook fn, void* ctx, bool per_step);

// lgx_batch_create_ex, with the batch's work on `stream` when it is not null
// (a member lattice's own stream, borrowed: the batch neither creates nor
// destroys it, so events recorded on that stream bracket the batch's work).
int batch_create(lgx_lattice* const* lats, size_t n, int policy, cudaStream_t stream,
                 lgx_batch** out);

}  // namespace lgx
