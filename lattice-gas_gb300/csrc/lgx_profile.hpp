// lgx_profile.hpp -- row and column profiles (internal).
#pragma once

#include "lgx_internal.hpp"

namespace lgx {

// One lattice to profile.  The state after local step t lives in
// planes[(cur0 + t) & 1].  It is profiled when offset + t = first + i * every
// for i < count (every == 0: only offset + t == first), sample i going to
// slot i of row_u ([count][h]) and col_u ([count][w]).
struct ProfDesc {
  const uint32_t* planes[2];
  uint32_t cur0;
  Dims dm;
  int32_t* rows;       // [3][h] mass, px2, py2 of each row (scratch)
  int32_t* cols;       // [3][w] of each column; zero between launches
  uint32_t* done;      // blocks finished; zero between launches
  float* row_u;        // row_ux trajectory, or null
  float* col_u;        // column_uy trajectory, or null
  int32_t* col_sums;   // copy of the column sums [3][w], or null
  uint64_t offset, first, every;
  uint32_t count;
};

struct ProfArgs {
  const ProfDesc* descs;
  uint32_t nlat;
  const uint64_t* base;  // steps completed before this interval (null: 0)
  uint32_t k_after;      // profile the state after step *base + k_after
};

// Scratch words one lattice of height h and width w needs: rows + cols + done.
inline size_t profile_scratch_words(uint32_t w, uint32_t h) { return 3ull * h + 3ull * w + 1; }
uint32_t profile_chunks(uint32_t h);
cudaError_t launch_profile(const ProfArgs& p, uint32_t max_h, cudaStream_t st);

}  // namespace lgx
