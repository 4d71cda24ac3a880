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
};

cudaError_t launch_batch_step(const BatchStepArgs& a, uint32_t nblocks, bool rest,
                              cudaStream_t st);
cudaError_t launch_batch_inlet(const BatchInletArgs& a, cudaStream_t st);
cudaError_t launch_batch_sample(const BatchSampleArgs& a, cudaStream_t st);
cudaError_t launch_batch_base(uint64_t* base, uint32_t n, cudaStream_t st);

// Work enqueued after every batch step, inside the captured graphs: called
// with the batch's stream, its device step counter for the interval and the
// step's index within the interval plus one (the state after batch step
// *base + k_after).  Setting a hook drops the graphs captured without it.
typedef cudaError_t (*BatchStepHook)(void* ctx, cudaStream_t st, const uint64_t* base,
                                     uint32_t k_after);
int batch_set_step_hook(lgx_batch* b, BatchStepHook fn, void* ctx);

}  // namespace lgx
