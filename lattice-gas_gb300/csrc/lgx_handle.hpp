// lgx_handle.hpp -- the lattice handle behind the C ABI (internal).
#pragma once

#include <cuda_runtime.h>

#include "../../include/lgx.h"
#include "lgx_internal.hpp"

namespace lgx {
// Steps whose inlet draws are made in one launch, and the most steps one
// persistent launch runs.
constexpr uint32_t kInletChunk = 128;
}  // namespace lgx

// Mirrors GpuLattice (src/gpu.rs:453-476): the ping-pong planes, the solid
// plane and its one-bit-per-word summary, the coarse-grained field, and the
// stream everything of this lattice runs on.
struct lgx_lattice {
  int device = 0;
  cudaStream_t stream = nullptr;
  lgx::Dims dm{};
  bool rest = true;
  uint64_t seed = 0;
  uint64_t steps = 0;
  uint32_t thresh[7] = {0, 0, 0, 0, 0, 0, 0};
  uint32_t* planes[2] = {nullptr, nullptr};
  int cur = 0;
  uint32_t* solid = nullptr;
  uint32_t* anysolid = nullptr;
  uint8_t* cells = nullptr;  // staging for load/store, w*h bytes
  unsigned long long* counter = nullptr;
  // inlet draws for the current chunk of steps
  uint32_t* inlet = nullptr;
  uint32_t inlet_cap = 0;      // steps the buffer holds
  size_t inlet_words = 0;      // its size in words
  uint64_t inlet_first = 0;    // step index of slot 0
  uint32_t inlet_valid = 0;    // slots filled
  // field
  bool has_field = false;
  uint32_t bx = 0, by = 0, bw = 0, bh = 0;
  float* field = nullptr;      // ux | uy | rho | sol, bw*bh each
  int32_t* sums = nullptr;     // mass | px2 | py2 | nsolid
  cudaEvent_t ev[8] = {};
  uint64_t launches = 0;     // kernels this handle has launched
  // persistent multi-step kernel
  int step_mode = LGX_STEP_AUTO;
  uint32_t temporal_depth = 4;  // steps per pass in LGX_STEP_TEMPORAL
  bool auto_resolved = false;   // LGX_STEP_AUTO: the tuner's choice below is set
  int auto_mode = LGX_STEP_SINGLE;
  uint32_t auto_depth = 0;
  uint32_t auto_words = 0;        // the single-step kernel's shape (lgx::kShape*)
  float auto_us[9] = {};  // single (best, 1 and 2 chunks), wave, temporal 4, 8, graph,
                          // single (2 and 4 words per lane)
  uint32_t step_words = 0;        // a pinned kernel shape, lgx::kShape* (0: the tuner's or
                                  // by size)
  // LGX_STEP_GRAPH: a batch of this lattice alone, whose work runs on the
  // lattice's stream; made at first use, dropped when the inlet or the field
  // (which a batch lays out when it is made) changes
  lgx_batch* solo = nullptr;
  unsigned long long* fill_scratch = nullptr;  // the equilibrium fill's block counts
  uint32_t wave_grid = 0;    // co-resident CTAs; 0 until first used
  uint32_t* done = nullptr;  // [wave_grid] published step per CTA
  uint32_t* error = nullptr; // timeout flag
  // row and column profiles: scratch, row_ux[h], column_uy[w], column sums
  // [3][w] and the device copy of the profile descriptor, one allocation
  void* prof = nullptr;
  float* vort = nullptr;  // device address of vort_host: the field's vorticity (bw*bh),
                          // then its mean velocity (2)
  float* vort_host = nullptr;  // page-locked copy of the same, for the read-back
  void* mean_scratch = nullptr;  // the mean velocity's segment tables (device)
};

// The equilibrium fill's scratch for this lattice, made at its first fill.
inline cudaError_t ensure_fill_scratch(lgx_lattice* l) {
  return l->fill_scratch ? cudaSuccess : cudaMalloc(&l->fill_scratch, lgx::kFillScratchBytes);
}
