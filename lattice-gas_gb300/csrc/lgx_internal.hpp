// lgx_internal.hpp -- declarations shared by the library's translation units.
// Not part of the public C ABI (that is include/lgx.h).
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

#include <string>

namespace lgx {

// Geometry of one lattice in the bitplane layout.
struct Dims {
  uint32_t w, h;
  uint32_t wpr;       // words per row, ceil(w / 32)
  uint32_t total;     // wpr * h, words per plane
  uint32_t lastword;  // (w - 1) / 32
  uint32_t lastbit;   // (w - 1) % 32
  uint32_t tail;      // valid-bit mask of the last word of a row
  uint32_t iw;        // words of a row the inlet touches, ceil(inlet_cols / 32)
  uint32_t inlet_cols;
  // g / wpr == (t + ((g - t) >> div_s1)) >> div_s2 with t = mulhi(g, div_m), for
  // every 32-bit g (the round-up multiply-shift method for unsigned division)
  uint32_t div_m, div_s1, div_s2;
};

Dims make_dims(uint32_t w, uint32_t h, uint32_t inlet_cols);

// One step of one lattice: a -> b.
// Coarse-graining of one lattice into bw x bh blocks of bx x by cells.
struct SampleArgs {
  const uint32_t* a;
  const uint32_t* solid;
  Dims dm;
  uint32_t bx, by, bw, bh;
  float alpha;
  float* ux;
  float* uy;
  float* rho;
  float* sol;
  int32_t* sums;  // [4][bw*bh]: mass, px2, py2, nsolid
};

// Coarse-graining by tiles (blocks at least kTileMinWidth columns wide): CTAs
// over `per` consecutive blocks of one block row each, `ncx` of them per block
// row, `nblocks` in all (0: none).  A single step can carry one: its grid then
// leads with these CTAs, which coarse-grain the step's input state.
constexpr uint32_t kTileMinWidth = 16;
constexpr uint32_t kTileMaxBlocks = 64;
struct SampleTiles {
  SampleArgs s;
  uint32_t per, ncx, nblocks;
};
// The tiling of a field, or false when its blocks are too narrow for tiles.
bool sample_tiling(const SampleArgs& s, SampleTiles* t);
// A block row of bw blocks of bx columns in tiles: as many blocks per tile as
// keep their words within one warp's lanes (a block-aligned start can sit 31
// columns into its first word), spread evenly; bx >= kTileMinWidth.
__host__ __device__ inline void tile_shape(uint32_t bx, uint32_t bw, uint32_t* per,
                                           uint32_t* ncx) {
  uint32_t most = (1024u - 31u) / bx;
  most = most < 1u ? 1u : (most > kTileMaxBlocks ? kTileMaxBlocks : most);
  *ncx = (bw + most - 1u) / most;
  *per = (bw + *ncx - 1u) / *ncx;
}

struct StepArgs {
  const uint32_t* a;
  uint32_t* b;
  const uint32_t* solid;
  const uint32_t* anysolid;
  const uint32_t* inlet;  // Bernoulli words for this step, [h][iw][7]; null when iw == 0
  Dims dm;
  uint64_t seed;
  uint64_t steps;  // steps taken before this one
  uint32_t words;  // the kernel's shape, a kShape* value (0: chosen by the lattice's size)
  SampleTiles tiles = {};  // the state this step reads, coarse-grained alongside (nblocks > 0)
};

// Shapes of the single-step kernel.  Chunk1, Chunk2: one word per lane, a warp
// takes one or two 32-word chunks (256- and 128-thread blocks).  Lanes2,
// Lanes4: two or four consecutive words per lane in 64- or 128-bit accesses,
// for lattices whose words per row are a multiple of that count.
constexpr uint32_t kShapeChunk1 = 1, kShapeChunk2 = 2, kShapeLanes2 = 3, kShapeLanes4 = 4;
// The shape a launch with `shape` requested runs: the request when it applies
// to the lattice, else the size-based default.
uint32_t step_shape(const Dims& dm, uint32_t shape);

// `nsteps` steps of one lattice in one cooperative launch.  The state after
// local step s lives in planes[s & 1]; done[b] is the last step CTA b has
// published (zeroed before the launch); error is set if a wait times out.
struct WaveArgs {
  uint32_t* planes[2];
  const uint32_t* solid;
  const uint32_t* anysolid;
  const uint32_t* inlet;  // [nsteps][h][iw][7]; null when iw == 0
  Dims dm;
  uint64_t seed;
  uint64_t steps;  // steps taken before the first of these
  uint32_t nsteps;
  uint32_t* done;
  uint32_t* error;
};

// K steps in one pass over HBM (temporal blocking): a -> b after K steps.
struct TemporalArgs {
  const uint32_t* a;
  uint32_t* b;
  const uint32_t* solid;
  const uint32_t* anysolid;
  const uint32_t* inlet;  // [K][h][iw][7] draws of the K steps; null when iw == 0
  Dims dm;
  uint64_t seed;
  uint64_t steps;  // steps taken before the first of the K
  uint32_t nstrips, nbands, band_rows;
};

// Inlet Bernoulli words for `nsteps` consecutive steps starting at `steps`,
// written to out[s][y][jw][d].
struct InletArgs {
  uint32_t* out;
  Dims dm;
  uint64_t seed;
  uint64_t steps;
  uint32_t nsteps;
  uint32_t thresh[7];
};

cudaError_t launch_step(const StepArgs& s, bool rest, cudaStream_t st);
cudaError_t launch_inlet(const InletArgs& s, cudaStream_t st);
// Co-resident CTAs for the persistent kernel on the current device (at most
// one per 32-word chunk).
cudaError_t wave_grid(bool rest, uint32_t total, uint32_t* grid);
cudaError_t launch_wave(const WaveArgs& w, bool rest, uint32_t grid, cudaStream_t st);
// Temporal blocking: supported depths and widths, the tiling, the launch.
bool temporal_supported(const Dims& dm, uint32_t k);
void temporal_tiling(const Dims& dm, uint32_t k, TemporalArgs* t);  // k steps per pass
cudaError_t launch_temporal(const TemporalArgs& t, bool rest, uint32_t k, cudaStream_t st);
// flag set: the last block to finish (done: a zeroed counter it sets back) writes
// seq to *flag, mapped host memory, after the field (host_result_wait).
cudaError_t launch_sample(const SampleArgs& s, cudaStream_t st, unsigned int* done = nullptr,
                          unsigned long long* flag = nullptr, unsigned long long seq = 0);
// Field::vorticity and Field::mean_velocity of a field laid out ux | uy | rho |
// sol (bw * bh each), in one launch: vort gets bw * bh floats and mean (mean ux,
// mean uy); either may be null.  mean_scratch: mean_scratch_bytes() of device
// memory zeroed before its first use, kept for the field's later calls (null: the
// mean velocity takes its single-chain kernel).
size_t mean_scratch_bytes();
// With flag set (and mean_scratch, which holds the launch's done counter), the
// last block to finish writes seq to *flag after every result (host_result_wait).
cudaError_t launch_field_analyses(const float* field, uint32_t bw, uint32_t bh, uint32_t bx,
                                  uint32_t by, float* vort, float* mean, void* mean_scratch,
                                  cudaStream_t st, unsigned long long* flag = nullptr,
                                  unsigned long long seq = 0);
// A lattice's counter buffer: the particle count (word 0), the three moments
// (1..3), the ticket of one-launch totals (4), the done counter of a waited-for
// coarse-graining launch (5), and the totals' per-block slots (6..) for grids of
// up to kReduceMaxBlocks blocks; zeroed when made.
constexpr unsigned kReduceMaxBlocks = 304;
constexpr size_t kCounterWords = 6 + (size_t)kReduceMaxBlocks * 3;
// Particles on the lattice into out[0]; the WITH_WALLS moments of every cell
// (src/moments.rs:37-74, 126-138) into out[0..2] = mass, px2, py2 as 64-bit
// two's-complement sums.  ticket null: out is device memory, zeroed first (two
// operations); else ticket is a lattice counter buffer's word 4 (zero between
// launches) and out mapped host memory the kernel writes (one operation).
// With flag set (mapped host memory too), the last block writes seq there after
// the totals (host_result_wait).
cudaError_t launch_count(const uint32_t* a, const Dims& dm, unsigned long long* out,
                         cudaStream_t st, unsigned long long* ticket = nullptr,
                         unsigned long long* flag = nullptr, unsigned long long seq = 0);
cudaError_t launch_moments(const uint32_t* a, const Dims& dm, unsigned long long* out,
                           cudaStream_t st, unsigned long long* ticket = nullptr,
                           unsigned long long* flag = nullptr, unsigned long long seq = 0);
// Moments::velocity (src/moments.rs:91-97): momentum per particle in f32, (0, 0)
// for no particles.
void moments_velocity(int64_t mass, int64_t px2, int64_t py2, float* ux, float* uy);
// Eight page-locked 64-bit words for this host thread, for results of a few
// bytes read back by a call that synchronises before it returns (a copy to
// pageable memory goes through a staging copy); null if none could be had.  The
// words are mapped into the devices' address space: host_result_device gives
// their device address (null if it cannot), for kernels that write them.
unsigned long long* host_result_words();
unsigned long long* host_result_device();
// Word 7 of those words is a completion flag: host_result_seq() gives the next
// sequence number for a launch to write there after its results, and
// host_result_wait(seq, st) returns once it has (a spin on the mapped word: about
// 1.5 us sooner than cudaStreamSynchronize on GB300), falling back to synchronising
// the stream (which also reports a failed launch) when it has not within 20 ms.
unsigned long long host_result_seq();
cudaError_t host_result_wait(unsigned long long seq, cudaStream_t st);
// Byte cells (w*h, row-major) <-> planes + solid + anysolid.
cudaError_t launch_pack(const uint8_t* cells, const Dims& dm, uint32_t* planes, uint32_t* solid,
                        uint32_t* anysolid, cudaStream_t st);
cudaError_t launch_unpack(const uint32_t* planes, const uint32_t* solid, const Dims& dm,
                          uint8_t* cells, cudaStream_t st);
// Exhaustive circuit check: out[i] for i < n_states * 48 (src/gpu.rs:399-417).
cudaError_t launch_verify(uint32_t* out, uint32_t n, bool rest, cudaStream_t st);

// Host-side equilibrium thresholds (src/lattice.rs:59-92), f32 without fusion.
void equilibrium_thresholds(float density, float ux, float uy, bool rest, uint32_t out[7]);
// The equilibrium fill of Lattice::init_equilibrium (src/lattice.rs:197-208)
// on the device: every fluid cell (not solid) gets an equilibrium sample from
// Rng::new(seed), cell order row-major; solid cells get no particles (bytes:
// exactly the solid bit).  Target: the seven planes of a bitplane lattice, or
// n byte cells (16-byte aligned) when `planes` is null.
struct EqFill {
  uint32_t* planes;
  const uint32_t* solid;
  Dims dm;
  uint8_t* cells;
  size_t n;
  uint64_t seed;
  uint32_t thresh[7];
  bool rest;
  // Planes target only: thresholds per row ([h][7], the shear-wave start of
  // src/transport.rs:188-200) or per column ([w][7], transport.rs:240-252)
  // in device memory, in place of `thresh`; at most one is set.
  const uint32_t* thresh_rows;
  const uint32_t* thresh_cols;
  // Device scratch of kFillScratchBytes for the fill's per-block counts, kept by
  // the caller across fills; null: allocated and freed around this fill.
  unsigned long long* scratch;
};
constexpr size_t kFillScratchBytes = 152 * 8 * 8;  // one count per block, at most 1216 blocks
cudaError_t launch_equilibrium_fill(const EqFill& f, cudaStream_t st);


void set_error(const std::string& msg);

}  // namespace lgx
