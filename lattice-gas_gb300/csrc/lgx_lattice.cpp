// lgx_lattice.cpp -- the lattice handle behind the C ABI (include/lgx.h).
//
// Mirrors GpuLattice (src/gpu.rs:453-755): it owns the ping-pong planes, the
// solid plane and its one-bit-per-word summary, the coarse-grained field, and
// a CUDA stream.  Steps are enqueued back to back on that stream and the call
// waits once at the end, as the reference's advance_sampling commits its
// command buffers and waits (src/gpu.rs:668-706).
#include <cuda_runtime.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <new>
#include <string>

#include "../../include/lgx.h"
#include "lgx_batch.hpp"
#include "lgx_handle.hpp"
#include "lgx_profile.hpp"
#include "lgx_tune.hpp"
#include "lgx_internal.hpp"

namespace lgx {

namespace {
thread_local std::string g_last_error;
}

void set_error(const std::string& msg) { g_last_error = msg; }

Dims make_dims(uint32_t w, uint32_t h, uint32_t inlet_cols) {
  Dims d;
  d.w = w;
  d.h = h;
  d.wpr = (w + 31u) / 32u;
  d.total = d.wpr * h;
  d.lastword = (w - 1u) / 32u;
  d.lastbit = (w - 1u) % 32u;
  d.tail = (d.lastbit == 31u) ? 0xffffffffu : ((1u << (d.lastbit + 1u)) - 1u);
  d.inlet_cols = std::min(inlet_cols, w);
  d.iw = (d.inlet_cols + 31u) / 32u;
  uint32_t l = 0;  // ceil(log2(wpr))
  while ((1ull << l) < d.wpr) ++l;
  d.div_m = (uint32_t)(((1ull << 32) * ((1ull << l) - d.wpr)) / d.wpr + 1u);
  d.div_s1 = l < 1u ? l : 1u;
  d.div_s2 = l > 1u ? l - 1u : 0u;
  return d;
}


}  // namespace lgx


  bool rest = true;
  uint64_t seed = 0;
  uint64_t steps = 0;
  uint32_t thresh[7] = {0, 0, 0, 0, 0, 0, 0};

namespace {

int cuda_fail(cudaError_t e, const char* what) {
  lgx::set_error(std::string(what) + ": " + cudaGetErrorString(e));
  return LGX_ERR_CUDA;
}

#define LGX_CUDA(call)                                        \
  do {                                                        \
    cudaError_t e_ = (call);                                  \
    if (e_ != cudaSuccess) return cuda_fail(e_, #call);       \
  } while (0)

int check_lat(lgx_lattice* lat) {
  if (!lat) {
    lgx::set_error("null lattice handle");
    return LGX_ERR_ARG;
  }
  cudaError_t e = cudaSetDevice(lat->device);
  if (e != cudaSuccess) return cuda_fail(e, "cudaSetDevice");
  return LGX_OK;
}

// The one-lattice batch of LGX_STEP_GRAPH, if made.
void drop_solo(lgx_lattice* lat) {
  if (lat->solo) lgx_batch_destroy(lat->solo);
  lat->solo = nullptr;
}

void free_lattice(lgx_lattice* lat) {
  cudaSetDevice(lat->device);
  drop_solo(lat);  // before the stream it borrows
  if (lat->stream) cudaStreamSynchronize(lat->stream);
  cudaFree(lat->planes[0]);
  cudaFree(lat->planes[1]);
  cudaFree(lat->solid);
  cudaFree(lat->anysolid);
  cudaFree(lat->cells);
  cudaFree(lat->counter);
  cudaFree(lat->inlet);
  cudaFree(lat->field);
  cudaFree(lat->sums);
  cudaFree(lat->prof);
  cudaFree(lat->fill_scratch);
  if (lat->vort_host) cudaFreeHost(lat->vort_host);  // lat->vort maps into it
  cudaFree(lat->mean_scratch);
  cudaFree(lat->done);
  cudaFree(lat->error);
  for (auto& e : lat->ev)
    if (e) cudaEventDestroy(e);
  if (lat->stream) cudaStreamDestroy(lat->stream);
  delete lat;
}

// Draw the inlet words for the next `want` steps if the chunk in hand does
// not cover step `lat->steps`.
int ensure_inlet(lgx_lattice* lat, uint64_t want) {
  if (lat->dm.iw == 0) return LGX_OK;
  if (lat->steps >= lat->inlet_first && lat->steps < lat->inlet_first + lat->inlet_valid)
    return LGX_OK;
  const uint32_t n = (uint32_t)std::min<uint64_t>(want, lgx::kInletChunk);
  // words one step of draws occupies; the inlet width can change between calls
  const size_t per_step = (size_t)lat->dm.h * lat->dm.iw * 7;
  if (n > lat->inlet_cap || per_step * lgx::kInletChunk > lat->inlet_words) {
    // the buffer may still be read by enqueued steps
    LGX_CUDA(cudaStreamSynchronize(lat->stream));
    cudaFree(lat->inlet);
    lat->inlet = nullptr;
    lat->inlet_cap = 0;
    lat->inlet_words = 0;
    LGX_CUDA(cudaMalloc(&lat->inlet, per_step * lgx::kInletChunk * sizeof(uint32_t)));
    lat->inlet_cap = lgx::kInletChunk;
    lat->inlet_words = per_step * lgx::kInletChunk;
  }
  lgx::InletArgs ia;
  ia.out = lat->inlet;
  ia.dm = lat->dm;
  ia.seed = lat->seed;
  ia.steps = lat->steps;
  ia.nsteps = n;
  memcpy(ia.thresh, lat->thresh, sizeof(ia.thresh));
  LGX_CUDA(lgx::launch_inlet(ia, lat->stream));
  lat->launches += 1;
  lat->inlet_first = lat->steps;
  lat->inlet_valid = n;
  return LGX_OK;
}

lgx::SampleArgs sample_args(const lgx_lattice* lat, float alpha) {
  const size_t nb = (size_t)lat->bw * lat->bh;
  lgx::SampleArgs sa;
  sa.a = lat->planes[lat->cur];
  sa.solid = lat->solid;
  sa.dm = lat->dm;
  sa.bx = lat->bx;
  sa.by = lat->by;
  sa.bw = lat->bw;
  sa.bh = lat->bh;
  sa.alpha = alpha;
  sa.ux = lat->field;
  sa.uy = lat->field + nb;
  sa.rho = lat->field + 2 * nb;
  sa.sol = lat->field + 3 * nb;
  sa.sums = lat->sums;
  return sa;
}

int launch_sample(lgx_lattice* lat, float alpha, unsigned long long* flag = nullptr,
                  unsigned long long seq = 0) {
  if (!lat->has_field) return LGX_OK;
  const lgx::SampleArgs sa = sample_args(lat, alpha);
  LGX_CUDA(lgx::launch_sample(sa, lat->stream, reinterpret_cast<unsigned int*>(lat->counter + 5),
                              flag, seq));
  lat->launches += 1;
  return LGX_OK;
}

int enqueue_wave(lgx_lattice* lat, uint32_t k) {
  if (lat->wave_grid == 0) {
    uint32_t grid = 0;
    LGX_CUDA(lgx::wave_grid(lat->rest, lat->dm.total, &grid));
    LGX_CUDA(cudaMalloc(&lat->done, grid * sizeof(uint32_t)));
    LGX_CUDA(cudaMalloc(&lat->error, sizeof(uint32_t)));
    LGX_CUDA(cudaMemsetAsync(lat->error, 0, sizeof(uint32_t), lat->stream));
    lat->wave_grid = grid;
  }
  lgx::WaveArgs wa;
  wa.planes[0] = lat->planes[lat->cur];
  wa.planes[1] = lat->planes[lat->cur ^ 1];
  wa.solid = lat->solid;
  wa.anysolid = lat->anysolid;
  wa.inlet = lat->dm.iw ? lat->inlet + (size_t)(lat->steps - lat->inlet_first) * lat->dm.h *
                                           lat->dm.iw * 7
                        : nullptr;
  wa.dm = lat->dm;
  wa.seed = lat->seed;
  wa.steps = lat->steps;
  wa.nsteps = k;
  wa.done = lat->done;
  wa.error = lat->error;
  LGX_CUDA(cudaMemsetAsync(lat->done, 0, lat->wave_grid * sizeof(uint32_t), lat->stream));
  LGX_CUDA(lgx::launch_wave(wa, lat->rest, lat->wave_grid, lat->stream));
  lat->launches += 1;
  lat->cur ^= (int)(k & 1u);
  lat->steps += k;
  return LGX_OK;
}

// K steps in one pass (temporal blocking); the caller checked the inlet
// chunk covers them.
int enqueue_temporal(lgx_lattice* lat, uint32_t k) {
  lgx::TemporalArgs ta;
  ta.a = lat->planes[lat->cur];
  ta.b = lat->planes[lat->cur ^ 1];
  ta.solid = lat->solid;
  ta.anysolid = lat->anysolid;
  ta.inlet = lat->dm.iw ? lat->inlet + (size_t)(lat->steps - lat->inlet_first) * lat->dm.h *
                                           lat->dm.iw * 7
                        : nullptr;
  ta.dm = lat->dm;
  ta.seed = lat->seed;
  ta.steps = lat->steps;
  lgx::temporal_tiling(lat->dm, k, &ta);
  LGX_CUDA(lgx::launch_temporal(ta, lat->rest, k, lat->stream));
  lat->launches += 1;
  lat->cur ^= 1;
  lat->steps += k;
  return LGX_OK;
}

// tiles: coarse-graining of the state this step reads, run in the step's grid
// (null: none).
int enqueue_single(lgx_lattice* lat, const lgx::SampleTiles* tiles = nullptr) {
  lgx::StepArgs sa;
  sa.a = lat->planes[lat->cur];
  sa.b = lat->planes[lat->cur ^ 1];
  sa.solid = lat->solid;
  sa.anysolid = lat->anysolid;
  sa.inlet = lat->dm.iw ? lat->inlet + (size_t)(lat->steps - lat->inlet_first) * lat->dm.h *
                                           lat->dm.iw * 7
                        : nullptr;
  sa.dm = lat->dm;
  sa.seed = lat->seed;
  sa.steps = lat->steps;
  sa.words = lat->step_words ? lat->step_words
             : (lat->step_mode == LGX_STEP_AUTO && lat->auto_resolved) ? lat->auto_words
                                                                        : 0u;
  if (tiles) sa.tiles = *tiles;
  LGX_CUDA(lgx::launch_step(sa, lat->rest, lat->stream));
  lat->launches += 1;
  lat->cur ^= 1;
  lat->steps += 1;
  return LGX_OK;
}

// Enqueue n steps, sampling every `every` steps and after the last
// (src/gpu.rs:668-706).  In the persistent mode one launch runs up to the
// next sampling point, the end of the inlet chunk in hand, or kInletChunk.
// LGX_STEP_AUTO: the step-mode tuner's choice for this lattice's size class.
int resolve_auto(lgx_lattice* lat) {
  if (lat->auto_resolved) return LGX_OK;
  lgx::StepPlan p;
  if (lgx::plan_step_mode(lat->device, lat->dm.w, lat->dm.h, lat->rest, &p) != LGX_OK) {
    // the tuner could not run here (e.g. no room for its scratch lattice): the
    // reference's own launch pattern, one kernel per step
    cudaGetLastError();
    p = lgx::StepPlan{};
    p.mode = LGX_STEP_SINGLE;
  }
  lat->auto_mode = p.mode;
  lat->auto_depth = p.depth;
  lat->auto_words = p.words;
  lat->auto_us[0] = p.single_us;
  lat->auto_us[1] = p.single1_us;
  lat->auto_us[2] = p.single2_us;
  lat->auto_us[3] = p.wave_us;
  lat->auto_us[4] = p.temporal4_us;
  lat->auto_us[5] = p.temporal8_us;
  lat->auto_us[6] = p.graph_us;
  lat->auto_us[7] = p.lanes2_us;
  lat->auto_us[8] = p.lanes4_us;
  lat->auto_resolved = true;
  return LGX_OK;
}

// LGX_STEP_GRAPH: runs of at least this many steps, sampling no more often
// than every kGraphMinEvery steps, go through the lattice's one-lattice batch
// (captured CUDA graphs, or the resident kernel for a small lattice); other
// runs take one launch per step.  A batch launches one graph per sampling
// interval, which costs about as much as 10-15 single-step launches save.
constexpr uint64_t kGraphMinSteps = 8;
constexpr uint64_t kGraphMinEvery = 16;

int advance_graph(lgx_lattice* lat, uint64_t n, uint64_t every, float alpha) {
  if (!lat->solo) {
    lgx_lattice* one[1] = {lat};
    const int rc = lgx::batch_create(one, 1, LGX_BATCH_AUTO, lat->stream, &lat->solo);
    if (rc) {
      lat->solo = nullptr;
      return rc;
    }
  }
  uint64_t k0 = 0, k1 = 0, g = 0;
  lgx_batch_launch_count(lat->solo, &k0, &g);
  const int rc = lgx_batch_advance_sampling(lat->solo, n, every, alpha);
  lgx_batch_launch_count(lat->solo, &k1, &g);
  lat->launches += k1 - k0;
  return rc;
}

int enqueue_steps(lgx_lattice* lat, uint64_t n, uint64_t every, float alpha) {
  uint64_t left = n, since = 0;
  int mode = lat->step_mode;
  uint32_t tk = lat->temporal_depth;
  if (mode == LGX_STEP_AUTO && n > 0) {
    const int rc = resolve_auto(lat);
    if (rc) return rc;
    mode = lat->auto_mode;
    if (mode == LGX_STEP_TEMPORAL) tk = lat->auto_depth;
  }
  const bool wave = mode == LGX_STEP_WAVE;
  const bool temporal = mode == LGX_STEP_TEMPORAL && lgx::temporal_supported(lat->dm, tk);
  // One launch per step: a sampling point followed by another step of the run
  // is coarse-grained inside that step's grid (its tiles read the state the
  // step reads), which saves the sampling kernel's launch and the drain of the
  // steps around it; the run's last sampling point takes the sampling kernel.
  lgx::SampleTiles tiles;
  bool pending = false;
  while (left > 0) {
    int rc = ensure_inlet(lat, left);
    if (rc) return rc;
    uint64_t k = 1;
    const bool fits = left >= tk && (every == 0 || every - since >= tk) &&
                      (lat->dm.iw == 0 || lat->inlet_first + lat->inlet_valid - lat->steps >= tk);
    if (temporal && fits) {
      k = tk;
      rc = enqueue_temporal(lat, tk);
    } else if (wave) {
      k = std::min<uint64_t>(left, lgx::kInletChunk);
      if (every > 0) k = std::min<uint64_t>(k, every - since);
      if (lat->dm.iw) k = std::min<uint64_t>(k, lat->inlet_first + lat->inlet_valid - lat->steps);
      rc = enqueue_wave(lat, (uint32_t)k);
    } else {
      rc = enqueue_single(lat, pending ? &tiles : nullptr);
      pending = false;
    }
    if (rc) return rc;
    left -= k;
    since += k;
    if (every > 0 && (since >= every || left == 0)) {
      since = 0;
      if (left > 0 && !wave && !temporal && lat->has_field &&
          lgx::sample_tiling(sample_args(lat, alpha), &tiles))
        pending = true;
      else
        rc = launch_sample(lat, alpha);
      if (rc) return rc;
    }
  }
  return LGX_OK;
}

// After a sync: did a persistent launch time out waiting on a peer?
int check_wave_error(lgx_lattice* lat) {
  if (!lat->error) return LGX_OK;
  uint32_t v = 0;
  LGX_CUDA(cudaMemcpy(&v, lat->error, sizeof(v), cudaMemcpyDeviceToHost));
  if (v) {
    cudaMemset(lat->error, 0, sizeof(uint32_t));
    lgx::set_error("persistent step kernel timed out waiting for a neighbouring block; "
                   "the lattice state is undefined");
    return LGX_ERR_CUDA;
  }
  return LGX_OK;
}

}  // namespace

namespace {

// Profiles of the current state into the lattice's profile buffers; returns
// the device addresses of row_ux, column_uy and the column sums.
int run_profile(lgx_lattice* lat, float** row_u, float** col_u, int32_t** col_sums) {
  const lgx::Dims& dm = lat->dm;
  const size_t scratch = lgx::profile_scratch_words(dm.w, dm.h) * 4;
  const size_t off_row = (scratch + 255) & ~(size_t)255;
  const size_t off_col = off_row + (((size_t)dm.h * 4 + 255) & ~(size_t)255);
  const size_t off_sum = off_col + (((size_t)dm.w * 4 + 255) & ~(size_t)255);
  const size_t off_desc = off_sum + (((size_t)dm.w * 12 + 255) & ~(size_t)255);
  char* base = (char*)lat->prof;
  if (!base) {
    LGX_CUDA(cudaMalloc(&lat->prof, off_desc + sizeof(lgx::ProfDesc)));
    base = (char*)lat->prof;
    LGX_CUDA(cudaMemsetAsync(base, 0, scratch, lat->stream));  // column sums, counter
  }
  lgx::ProfDesc d{};
  d.planes[0] = d.planes[1] = lat->planes[lat->cur];
  d.dm = dm;
  d.rows = (int32_t*)base;
  d.cols = d.rows + 3 * (size_t)dm.h;
  d.done = (uint32_t*)(d.cols + 3 * (size_t)dm.w);
  d.row_u = (float*)(base + off_row);
  d.col_u = (float*)(base + off_col);
  d.col_sums = (int32_t*)(base + off_sum);
  d.first = 0;
  d.every = 0;
  d.count = 1;
  lgx::ProfDesc* dd = (lgx::ProfDesc*)(base + off_desc);
  LGX_CUDA(cudaMemcpyAsync(dd, &d, sizeof(d), cudaMemcpyHostToDevice, lat->stream));
  lgx::ProfArgs pa{dd, 1, nullptr, 0};
  LGX_CUDA(lgx::launch_profile(pa, dm.h, lat->stream));
  lat->launches += 1;
  *row_u = d.row_u;
  *col_u = d.col_u;
  *col_sums = d.col_sums;
  return LGX_OK;
}

}  // namespace

extern "C" {

const char* lgx_last_error(void) { return lgx::g_last_error.c_str(); }

int lgx_create(size_t w, size_t h, int rest, uint64_t seed, lgx_lattice** out) {
  if (!out) {
    lgx::set_error("lgx_create: null output");
    return LGX_ERR_ARG;
  }
  *out = nullptr;
  if (h % 2 != 0) {
    lgx::set_error("row count must be even for the lattice to wrap cleanly in y");
    return LGX_ERR_ARG;
  }
  if (w <= 4 || h <= 4) {
    lgx::set_error("lattice is too small");
    return LGX_ERR_ARG;
  }
  const size_t wpr = (w + 31) / 32;
  if (wpr * h * 7 >= (1ull << 32) || w >= (1ull << 31)) {
    lgx::set_error("lattice is too large for 32-bit word indices");
    return LGX_ERR_ARG;
  }
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    lgx::set_error("no CUDA device on this machine");
    return LGX_ERR_NO_DEVICE;
  }
  lgx_lattice* lat = new (std::nothrow) lgx_lattice();
  if (!lat) {
    lgx::set_error("out of host memory");
    return LGX_ERR_ALLOC;
  }
  cudaGetDevice(&lat->device);
  lat->dm = lgx::make_dims((uint32_t)w, (uint32_t)h, 0);
  lat->rest = rest != 0;
  lat->seed = seed;
  const size_t total = lat->dm.total;
  cudaError_t e = cudaStreamCreateWithFlags(&lat->stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaMalloc(&lat->planes[0], total * 7 * sizeof(uint32_t));
  if (e == cudaSuccess) e = cudaMalloc(&lat->planes[1], total * 7 * sizeof(uint32_t));
  if (e == cudaSuccess) e = cudaMalloc(&lat->solid, total * sizeof(uint32_t));
  if (e == cudaSuccess) e = cudaMalloc(&lat->anysolid, ((total + 31) / 32) * sizeof(uint32_t));
  if (e == cudaSuccess) e = cudaMalloc(&lat->cells, w * h);
  // the particle count, the three WITH_WALLS moments, one-launch totals' slots
  if (e == cudaSuccess) e = cudaMalloc(&lat->counter, lgx::kCounterWords * 8);
  if (e == cudaSuccess) e = cudaMemsetAsync(lat->counter, 0, lgx::kCounterWords * 8, lat->stream);
  for (int i = 0; i < 8 && e == cudaSuccess; ++i) e = cudaEventCreate(&lat->ev[i]);
  if (e == cudaSuccess) e = cudaMemsetAsync(lat->planes[0], 0, total * 7 * 4, lat->stream);
  if (e == cudaSuccess) e = cudaMemsetAsync(lat->planes[1], 0, total * 7 * 4, lat->stream);
  if (e == cudaSuccess) e = cudaMemsetAsync(lat->solid, 0, total * 4, lat->stream);
  if (e == cudaSuccess)
    e = cudaMemsetAsync(lat->anysolid, 0, ((total + 31) / 32) * 4, lat->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(lat->stream);
  if (e != cudaSuccess) {
    const int rc = (e == cudaErrorMemoryAllocation) ? LGX_ERR_ALLOC : LGX_ERR_CUDA;
    lgx::set_error(std::string("lgx_create: ") + cudaGetErrorString(e));
    free_lattice(lat);
    return rc;
  }
  *out = lat;
  return LGX_OK;
}

int lgx_destroy(lgx_lattice* lat) {
  if (!lat) return LGX_OK;
  free_lattice(lat);
  return LGX_OK;
}

int lgx_device_name(lgx_lattice* lat, char* buf, size_t len) {
  int rc = check_lat(lat);
  if (rc) return rc;
  cudaDeviceProp prop;
  LGX_CUDA(cudaGetDeviceProperties(&prop, lat->device));
  if (buf && len) snprintf(buf, len, "%s", prop.name);
  return LGX_OK;
}

int lgx_set_inlet(lgx_lattice* lat, size_t cols, float density, float ux, float uy, int rest) {
  int rc = check_lat(lat);
  if (rc) return rc;
  lat->dm = lgx::make_dims(lat->dm.w, lat->dm.h, (uint32_t)std::min<size_t>(cols, lat->dm.w));
  lgx::equilibrium_thresholds(density, ux, uy, rest != 0, lat->thresh);
  drop_solo(lat);  // its inlet buffers were sized for the old inlet
  lat->inlet_valid = 0;  // draws depend on the thresholds
  return LGX_OK;
}

int lgx_attach_field(lgx_lattice* lat, size_t bx, size_t by) {
  int rc = check_lat(lat);
  if (rc) return rc;
  if (bx == 0 || by == 0) {
    lgx::set_error("block size must be positive");
    return LGX_ERR_ARG;
  }
  LGX_CUDA(cudaStreamSynchronize(lat->stream));
  drop_solo(lat);  // its block tables were laid out for the old field
  cudaFree(lat->field);
  cudaFree(lat->sums);
  if (lat->vort_host) cudaFreeHost(lat->vort_host);  // sized for the old block grid
  lat->field = nullptr;
  lat->sums = nullptr;
  lat->vort = nullptr;
  lat->vort_host = nullptr;
  lat->has_field = false;
  lat->bx = (uint32_t)bx;
  lat->by = (uint32_t)by;
  lat->bw = lat->dm.w / (uint32_t)bx;
  lat->bh = lat->dm.h / (uint32_t)by;
  const size_t nb = std::max<size_t>((size_t)lat->bw * lat->bh, 1);
  LGX_CUDA(cudaMalloc(&lat->field, 4 * nb * sizeof(float)));
  LGX_CUDA(cudaMalloc(&lat->sums, 4 * nb * sizeof(int32_t)));
  LGX_CUDA(cudaMemsetAsync(lat->field, 0, 4 * nb * sizeof(float), lat->stream));
  LGX_CUDA(cudaMemsetAsync(lat->sums, 0, 4 * nb * sizeof(int32_t), lat->stream));
  LGX_CUDA(cudaStreamSynchronize(lat->stream));
  lat->has_field = true;
  return LGX_OK;
}

int lgx_load(lgx_lattice* lat, const uint8_t* cells, size_t n) {
  int rc = check_lat(lat);
  if (rc) return rc;
  if (n != (size_t)lat->dm.w * lat->dm.h || !cells) {
    lgx::set_error("wrong number of cells");
    return LGX_ERR_ARG;
  }
  LGX_CUDA(cudaMemcpyAsync(lat->cells, cells, n, cudaMemcpyHostToDevice, lat->stream));
  LGX_CUDA(lgx::launch_pack(lat->cells, lat->dm, lat->planes[lat->cur], lat->solid,
                            lat->anysolid, lat->stream));
  lat->launches += 1;
  LGX_CUDA(cudaStreamSynchronize(lat->stream));
  return LGX_OK;
}

int lgx_restart(lgx_lattice* lat, const uint8_t* cells, size_t n, uint64_t seed) {
  int rc = lgx_load(lat, cells, n);
  if (rc) return rc;
  lat->seed = seed;
  lat->steps = 0;
  lat->inlet_valid = 0;
  return LGX_OK;
}

int lgx_init_equilibrium(lgx_lattice* lat, float density, float ux, float uy, uint64_t seed) {
  int rc = check_lat(lat);
  if (rc) return rc;
  lgx::EqFill f{};
  f.planes = lat->planes[lat->cur];
  f.solid = lat->solid;
  f.dm = lat->dm;
  f.seed = seed ^ 0xA5A51234ull;  // src/lattice.rs:198
  f.rest = lat->rest;
  lgx::equilibrium_thresholds(density, ux, uy, lat->rest, f.thresh);
  LGX_CUDA(ensure_fill_scratch(lat));
  f.scratch = lat->fill_scratch;
  LGX_CUDA(lgx::launch_equilibrium_fill(f, lat->stream));
  lat->launches += 2;
  LGX_CUDA(cudaStreamSynchronize(lat->stream));
  return LGX_OK;
}

int lgx_store(lgx_lattice* lat, uint8_t* cells, size_t n) {
  int rc = check_lat(lat);
  if (rc) return rc;
  if (n != (size_t)lat->dm.w * lat->dm.h || !cells) {
    lgx::set_error("wrong number of cells");
    return LGX_ERR_ARG;
  }
  LGX_CUDA(lgx::launch_unpack(lat->planes[lat->cur], lat->solid, lat->dm, lat->cells,
                              lat->stream));
  lat->launches += 1;
  LGX_CUDA(cudaMemcpyAsync(cells, lat->cells, n, cudaMemcpyDeviceToHost, lat->stream));
  LGX_CUDA(cudaStreamSynchronize(lat->stream));
  return LGX_OK;
}

int lgx_advance(lgx_lattice* lat, uint64_t n) { return lgx_advance_sampling(lat, n, 0, 0.0f); }

int lgx_advance_sampling(lgx_lattice* lat, uint64_t n, uint64_t every, float alpha) {
  int rc = check_lat(lat);
  if (rc) return rc;
  int mode = lat->step_mode;
  if (mode == LGX_STEP_AUTO && n > 0) {
    rc = resolve_auto(lat);
    if (rc) return rc;
    mode = lat->auto_mode;
  }
  if (mode == LGX_STEP_GRAPH && n >= kGraphMinSteps && (every == 0 || every >= kGraphMinEvery)) {
    rc = advance_graph(lat, n, every, alpha);
    if (rc == LGX_OK || lat->step_mode == LGX_STEP_GRAPH) return rc;
    // AUTO: no one-lattice batch here (e.g. no memory for it); one launch per step
    cudaGetLastError();
  }
  rc = enqueue_steps(lat, n, every, alpha);
  if (rc) return rc;
  LGX_CUDA(cudaStreamSynchronize(lat->stream));
  return check_wave_error(lat);
}

int lgx_set_step_mode(lgx_lattice* lat, int mode) {
  if (!lat || (mode != LGX_STEP_AUTO && mode != LGX_STEP_SINGLE && mode != LGX_STEP_WAVE &&
               mode != LGX_STEP_TEMPORAL && mode != LGX_STEP_GRAPH)) {
    lgx::set_error("lgx_set_step_mode: bad handle or mode");
    return LGX_ERR_ARG;
  }
  lat->step_mode = mode;
  return LGX_OK;
}

int lgx_get_step_plan(lgx_lattice* lat, lgx_step_plan* out) {
  int rc = check_lat(lat);
  if (rc) return rc;
  if (!out) {
    lgx::set_error("lgx_get_step_plan: null output");
    return LGX_ERR_ARG;
  }
  rc = resolve_auto(lat);
  if (rc) return rc;
  out->mode = lat->auto_mode;
  out->depth = lat->auto_depth;
  out->words = lat->auto_words;
  out->single_us = lat->auto_us[0];
  out->single1_us = lat->auto_us[1];
  out->single2_us = lat->auto_us[2];
  out->wave_us = lat->auto_us[3];
  out->temporal4_us = lat->auto_us[4];
  out->temporal8_us = lat->auto_us[5];
  out->graph_us = lat->auto_us[6];
  out->lanes2_us = lat->auto_us[7];
  out->lanes4_us = lat->auto_us[8];
  return LGX_OK;
}

int lgx_set_step_shape(lgx_lattice* lat, int shape) {
  if (!lat || shape < LGX_SHAPE_AUTO || shape > LGX_SHAPE_LANES4) {
    lgx::set_error("lgx_set_step_shape: bad handle or shape (0 to 4)");
    return LGX_ERR_ARG;
  }
  lat->step_words = (uint32_t)shape;
  return LGX_OK;
}

int lgx_set_temporal_depth(lgx_lattice* lat, int k) {
  if (!lat || (k != 4 && k != 8)) {
    lgx::set_error("lgx_set_temporal_depth: depth must be 4 or 8");
    return LGX_ERR_ARG;
  }
  lat->temporal_depth = (uint32_t)k;
  return LGX_OK;
}

int lgx_sample_field(lgx_lattice* lat, float alpha) {
  int rc = check_lat(lat);
  if (rc) return rc;
  unsigned long long* flag = lgx::host_result_device();
  if (flag && lat->has_field && lat->bw * lat->bh > 0) {  // the kernel says when it is done
    const unsigned long long seq = lgx::host_result_seq();
    rc = launch_sample(lat, alpha, flag + 7, seq);
    if (rc) return rc;
    LGX_CUDA(lgx::host_result_wait(seq, lat->stream));
    return LGX_OK;
  }
  rc = launch_sample(lat, alpha);
  if (rc) return rc;
  LGX_CUDA(cudaStreamSynchronize(lat->stream));
  return LGX_OK;
}

int lgx_read_field(lgx_lattice* lat, float* ux, float* uy, float* rho, float* sol,
                   size_t n_blocks) {
  int rc = check_lat(lat);
  if (rc) return rc;
  if (!lat->has_field) {
    lgx::set_error("no field attached to this lattice");
    return LGX_ERR_STATE;
  }
  const size_t nb = (size_t)lat->bw * lat->bh;
  if (n_blocks != nb) {
    lgx::set_error("the field on the device has a different block grid from the one being filled");
    return LGX_ERR_ARG;
  }
  float* dst[4] = {ux, uy, rho, sol};
  for (int i = 0; i < 4; ++i)
    if (dst[i] && nb)
      LGX_CUDA(cudaMemcpyAsync(dst[i], lat->field + i * nb, nb * sizeof(float),
                               cudaMemcpyDeviceToHost, lat->stream));
  LGX_CUDA(cudaStreamSynchronize(lat->stream));
  return LGX_OK;
}

// The field analyses' results: one page-locked host buffer, mapped into the
// device's address space, that the analysis kernel writes directly (vorticity,
// bw * bh floats, then the mean velocity's two), so a call is one launch and one
// synchronisation with no copy between them.
static int field_scratch(lgx_lattice* lat, float** out) {
  if (!lat->has_field) {
    lgx::set_error("no field attached to this lattice");
    return LGX_ERR_STATE;
  }
  const size_t bytes = ((size_t)lat->bw * lat->bh + 2) * 4;
  if (!lat->vort_host) {
    LGX_CUDA(cudaHostAlloc((void**)&lat->vort_host, bytes, cudaHostAllocMapped));
    const cudaError_t e = cudaHostGetDevicePointer((void**)&lat->vort, lat->vort_host, 0);
    if (e != cudaSuccess) {
      cudaFreeHost(lat->vort_host);
      lat->vort_host = nullptr;
      lat->vort = nullptr;
      LGX_CUDA(e);
    }
  }
  if (!lat->mean_scratch) {  // the mean velocity's segment tables (and their counter at 0)
    LGX_CUDA(cudaMalloc(&lat->mean_scratch, lgx::mean_scratch_bytes()));
    const cudaError_t e = cudaMemset(lat->mean_scratch, 0, lgx::mean_scratch_bytes());
    if (e != cudaSuccess) {
      cudaFree(lat->mean_scratch);
      lat->mean_scratch = nullptr;
      LGX_CUDA(e);
    }
  }
  *out = lat->vort;
  return LGX_OK;
}

// Field::vorticity and/or Field::mean_velocity of the attached field: one launch
// that writes what was asked for into the mapped result buffer, one wait.
static int field_analyses(lgx_lattice* lat, float* w, float* mx, float* my) {
  float* d = nullptr;
  int rc = field_scratch(lat, &d);
  if (rc) return rc;
  const size_t nb = (size_t)lat->bw * lat->bh;
  const bool mean = mx != nullptr;
  unsigned long long* flag = lgx::host_result_device();
  const unsigned long long seq = flag ? lgx::host_result_seq() : 0;
  LGX_CUDA(lgx::launch_field_analyses(lat->field, lat->bw, lat->bh, lat->bx, lat->by,
                                      w ? d : nullptr, mean ? d + nb : nullptr,
                                      lat->mean_scratch, lat->stream, flag ? flag + 7 : nullptr,
                                      seq));
  lat->launches += 1;
  if (flag)
    LGX_CUDA(lgx::host_result_wait(seq, lat->stream));
  else
    LGX_CUDA(cudaStreamSynchronize(lat->stream));
  if (w) memcpy(w, lat->vort_host, nb * 4);
  if (mean) {
    *mx = lat->vort_host[nb];
    *my = lat->vort_host[nb + 1];
  }
  return LGX_OK;
}

int lgx_field_vorticity(lgx_lattice* lat, float* w, size_t n_blocks) {
  int rc = check_lat(lat);
  if (rc) return rc;
  if (!lat->has_field) {
    lgx::set_error("no field attached to this lattice");
    return LGX_ERR_STATE;
  }
  if (!w || n_blocks != (size_t)lat->bw * lat->bh) {
    lgx::set_error("lgx_field_vorticity: need one value per field block");
    return LGX_ERR_ARG;
  }
  return field_analyses(lat, w, nullptr, nullptr);
}

int lgx_field_mean_velocity(lgx_lattice* lat, float* ux, float* uy) {
  int rc = check_lat(lat);
  if (rc) return rc;
  if (!ux || !uy) {
    lgx::set_error("lgx_field_mean_velocity: null output");
    return LGX_ERR_ARG;
  }
  return field_analyses(lat, nullptr, ux, uy);
}

int lgx_field_analyses(lgx_lattice* lat, float* w, size_t n_blocks, float* ux, float* uy) {
  int rc = check_lat(lat);
  if (rc) return rc;
  if (!lat->has_field) {
    lgx::set_error("no field attached to this lattice");
    return LGX_ERR_STATE;
  }
  if (w && n_blocks != (size_t)lat->bw * lat->bh) {
    lgx::set_error("lgx_field_analyses: need one vorticity value per field block");
    return LGX_ERR_ARG;
  }
  if ((ux == nullptr) != (uy == nullptr) || (!w && !ux)) {
    lgx::set_error("lgx_field_analyses: ask for the vorticity, the mean velocity (both "
                   "components) or both");
    return LGX_ERR_ARG;
  }
  return field_analyses(lat, w, ux, uy);
}

int lgx_read_block_sums(lgx_lattice* lat, int32_t* mass, int32_t* px2, int32_t* py2,
                        int32_t* nsolid, size_t n_blocks) {
  int rc = check_lat(lat);
  if (rc) return rc;
  if (!lat->has_field) {
    lgx::set_error("no field attached to this lattice");
    return LGX_ERR_STATE;
  }
  const size_t nb = (size_t)lat->bw * lat->bh;
  if (n_blocks != nb) {
    lgx::set_error("block grid mismatch");
    return LGX_ERR_ARG;
  }
  int32_t* dst[4] = {mass, px2, py2, nsolid};
  for (int i = 0; i < 4; ++i)
    if (dst[i] && nb)
      LGX_CUDA(cudaMemcpyAsync(dst[i], lat->sums + i * nb, nb * sizeof(int32_t),
                               cudaMemcpyDeviceToHost, lat->stream));
  LGX_CUDA(cudaStreamSynchronize(lat->stream));
  return LGX_OK;
}

int lgx_row_ux(lgx_lattice* lat, float* ux, size_t n) {
  int rc = check_lat(lat);
  if (rc) return rc;
  if (!ux || n != lat->dm.h) {
    lgx::set_error("lgx_row_ux: need one value per row");
    return LGX_ERR_ARG;
  }
  float *ru, *cu;
  int32_t* cs;
  rc = run_profile(lat, &ru, &cu, &cs);
  if (rc) return rc;
  LGX_CUDA(cudaMemcpyAsync(ux, ru, n * 4, cudaMemcpyDeviceToHost, lat->stream));
  LGX_CUDA(cudaStreamSynchronize(lat->stream));
  return LGX_OK;
}

int lgx_column_uy(lgx_lattice* lat, float* uy, size_t n) {
  int rc = check_lat(lat);
  if (rc) return rc;
  if (!uy || n != lat->dm.w) {
    lgx::set_error("lgx_column_uy: need one value per column");
    return LGX_ERR_ARG;
  }
  float *ru, *cu;
  int32_t* cs;
  rc = run_profile(lat, &ru, &cu, &cs);
  if (rc) return rc;
  LGX_CUDA(cudaMemcpyAsync(uy, cu, n * 4, cudaMemcpyDeviceToHost, lat->stream));
  LGX_CUDA(cudaStreamSynchronize(lat->stream));
  return LGX_OK;
}

int lgx_line_sums(lgx_lattice* lat, int32_t* rows, size_t n_rows, int32_t* cols, size_t n_cols) {
  int rc = check_lat(lat);
  if (rc) return rc;
  if ((rows && n_rows != 3ull * lat->dm.h) || (cols && n_cols != 3ull * lat->dm.w)) {
    lgx::set_error("lgx_line_sums: rows holds 3 x h values, cols 3 x w");
    return LGX_ERR_ARG;
  }
  float *ru, *cu;
  int32_t* cs;
  rc = run_profile(lat, &ru, &cu, &cs);
  if (rc) return rc;
  if (rows)
    LGX_CUDA(cudaMemcpyAsync(rows, lat->prof, n_rows * 4, cudaMemcpyDeviceToHost, lat->stream));
  if (cols) LGX_CUDA(cudaMemcpyAsync(cols, cs, n_cols * 4, cudaMemcpyDeviceToHost, lat->stream));
  LGX_CUDA(cudaStreamSynchronize(lat->stream));
  return LGX_OK;
}

int lgx_total_particles(lgx_lattice* lat, uint64_t* out) {
  int rc = check_lat(lat);
  if (rc) return rc;
  if (!out) {
    lgx::set_error("null output");
    return LGX_ERR_ARG;
  }
  unsigned long long local = 0;
  unsigned long long* v = lgx::host_result_words();
  unsigned long long* dv = lgx::host_result_device();
  if (v && dv) {  // one launch that writes the total into the mapped result word
    const unsigned long long seq = lgx::host_result_seq();
    LGX_CUDA(lgx::launch_count(lat->planes[lat->cur], lat->dm, dv, lat->stream,
                               lat->counter + 4, dv + 7, seq));
    lat->launches += 1;
    LGX_CUDA(lgx::host_result_wait(seq, lat->stream));
    *out = v[0];
    return LGX_OK;
  }
  if (!v) v = &local;
  LGX_CUDA(lgx::launch_count(lat->planes[lat->cur], lat->dm, lat->counter, lat->stream));
  lat->launches += 1;
  LGX_CUDA(cudaMemcpyAsync(v, lat->counter, sizeof(*v), cudaMemcpyDeviceToHost, lat->stream));
  LGX_CUDA(cudaStreamSynchronize(lat->stream));
  *out = *v;
  return LGX_OK;
}

int lgx_mean_velocity(lgx_lattice* lat, float* ux, float* uy) {
  int rc = check_lat(lat);
  if (rc) return rc;
  if (!ux || !uy) {
    lgx::set_error("lgx_mean_velocity: null output");
    return LGX_ERR_ARG;
  }
  unsigned long long local[3];
  unsigned long long* v = lgx::host_result_words();
  unsigned long long* dv = lgx::host_result_device();
  if (v && dv) {  // one launch that writes the moments into the mapped result words
    const unsigned long long seq = lgx::host_result_seq();
    LGX_CUDA(lgx::launch_moments(lat->planes[lat->cur], lat->dm, dv, lat->stream,
                                 lat->counter + 4, dv + 7, seq));
    LGX_CUDA(lgx::host_result_wait(seq, lat->stream));
  } else {
    if (!v) v = local;
    LGX_CUDA(lgx::launch_moments(lat->planes[lat->cur], lat->dm, lat->counter + 1, lat->stream));
    LGX_CUDA(cudaMemcpyAsync(v, lat->counter + 1, 3 * sizeof(*v), cudaMemcpyDeviceToHost,
                             lat->stream));
    LGX_CUDA(cudaStreamSynchronize(lat->stream));
  }
  lat->launches += 1;
  lgx::moments_velocity((int64_t)v[0], (int64_t)v[1], (int64_t)v[2], ux, uy);
  return LGX_OK;
}

int lgx_steps(lgx_lattice* lat, uint64_t* out) {
  if (!lat || !out) {
    lgx::set_error("null argument");
    return LGX_ERR_ARG;
  }
  *out = lat->steps;
  return LGX_OK;
}

int lgx_launch_count(lgx_lattice* lat, uint64_t* out) {
  if (!lat || !out) {
    lgx::set_error("null argument");
    return LGX_ERR_ARG;
  }
  *out = lat->launches;
  return LGX_OK;
}

int lgx_stream(lgx_lattice* lat, void** stream) {
  if (!lat || !stream) {
    lgx::set_error("null argument");
    return LGX_ERR_ARG;
  }
  *stream = (void*)lat->stream;
  return LGX_OK;
}

int lgx_timing_mark(lgx_lattice* lat, int slot) {
  int rc = check_lat(lat);
  if (rc) return rc;
  if (slot < 0 || slot >= 8) {
    lgx::set_error("timing slot out of range");
    return LGX_ERR_ARG;
  }
  LGX_CUDA(cudaEventRecord(lat->ev[slot], lat->stream));
  return LGX_OK;
}

int lgx_timing_elapsed(lgx_lattice* lat, int a, int b, float* ms) {
  int rc = check_lat(lat);
  if (rc) return rc;
  if (a < 0 || a >= 8 || b < 0 || b >= 8 || !ms) {
    lgx::set_error("timing slot out of range");
    return LGX_ERR_ARG;
  }
  LGX_CUDA(cudaEventSynchronize(lat->ev[b]));
  LGX_CUDA(cudaEventElapsedTime(ms, lat->ev[a], lat->ev[b]));
  return LGX_OK;
}

int lgx_select_device(int ordinal) {
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    lgx::set_error("no CUDA device on this machine");
    return LGX_ERR_NO_DEVICE;
  }
  if (ordinal < 0 || ordinal >= ndev) {
    lgx::set_error("device ordinal out of range");
    return LGX_ERR_ARG;
  }
  LGX_CUDA(cudaSetDevice(ordinal));
  return LGX_OK;
}

int lgx_host_alloc(size_t bytes, void** out) {
  if (!out) {
    lgx::set_error("null output");
    return LGX_ERR_ARG;
  }
  *out = nullptr;
  cudaError_t e = cudaHostAlloc(out, bytes ? bytes : 1, cudaHostAllocDefault);
  if (e != cudaSuccess) {
    cudaGetLastError();
    lgx::set_error(std::string("cudaHostAlloc: ") + cudaGetErrorString(e));
    return e == cudaErrorMemoryAllocation ? LGX_ERR_ALLOC : LGX_ERR_CUDA;
  }
  return LGX_OK;
}

int lgx_host_free(void* p) {
  if (p) LGX_CUDA(cudaFreeHost(p));
  return LGX_OK;
}

int lgx_verify_circuit(int rest, uint32_t* out, size_t n) {
  const size_t want = (size_t)48 * (rest ? 128 : 64);
  if (!out || n != want) {
    lgx::set_error("lgx_verify_circuit: n must be 48 * n_states");
    return LGX_ERR_ARG;
  }
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    lgx::set_error("no CUDA device on this machine");
    return LGX_ERR_NO_DEVICE;
  }
  uint32_t* d = nullptr;
  LGX_CUDA(cudaMalloc(&d, n * sizeof(uint32_t)));
  cudaError_t e = lgx::launch_verify(d, (uint32_t)n, rest != 0, 0);
  if (e == cudaSuccess) e = cudaMemcpy(out, d, n * sizeof(uint32_t), cudaMemcpyDeviceToHost);
  cudaFree(d);
  if (e != cudaSuccess) return cuda_fail(e, "lgx_verify_circuit");
  return LGX_OK;
}

}  // extern "C"
