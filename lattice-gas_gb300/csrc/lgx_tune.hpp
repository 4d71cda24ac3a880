// lgx_tune.hpp -- the size-class tuner (internal).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace lgx {

// Lattices up to this many words per plane may be stepped by the resident kernel.
constexpr uint32_t kResidentMaxWords = 32768;

// How a size class is stepped, and what the choice was based on (microseconds
// per step of the class's synthetic lattices, each way).
struct ClassPlan {
  bool resident;
  uint32_t csize, threads;  // cluster shape of the resident kernel
  uint32_t ksteps;          // and its steps per cluster barrier (1, 2, 4 or 8)
  float step_us, resident_us;
  uint32_t words, count;    // the class: words per lattice and lattice count, rounded up
  uint32_t tuned_count;     // synthetic lattices actually timed
};

// Words per lattice rounded up to the class's power of two (at least 64).
uint32_t class_bucket(uint32_t words);

// The plan for `count` lattices of up to `words` words on `device` (the
// current device), timed on first use and cached for the process.
cudaError_t plan_class(int device, uint32_t words, uint32_t count, bool rest, ClassPlan* out);

// How LGX_STEP_AUTO steps one lattice: the fastest of one launch per step (in
// each kernel shape that applies, kShape*), the persistent wave kernel, temporal
// blocking of 4 or 8 steps and, for lattices below one full wave of step
// blocks, the one-lattice batch (LGX_STEP_GRAPH), timed on a
// scratch lattice of the same shape on first use of its size class (words
// rounded up to a power of two, whether it is wide enough for temporal
// blocking, the rule, whether the words per row are a multiple of 4 or 2) and
// cached for the process.  Times are microseconds per step; 0 where a mode does
// not apply.
struct StepPlan {
  int mode;        // LGX_STEP_SINGLE, LGX_STEP_WAVE, LGX_STEP_TEMPORAL or LGX_STEP_GRAPH
  uint32_t depth;  // temporal depth when TEMPORAL
  uint32_t words;  // the single-step kernel's shape (kShape*)
  float single_us, single1_us, single2_us, wave_us, temporal4_us, temporal8_us, graph_us;
  float lanes2_us, lanes4_us;
};
int plan_step_mode(int device, uint32_t w, uint32_t h, bool rest, StepPlan* out);

}  // namespace lgx
