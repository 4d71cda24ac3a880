// lgx_tune.cpp -- how to step a size class of lattices, chosen by measurement.
//
// A batch groups its small lattices into size classes (words per lattice
// rounded up to a power of two).  For each class the tuner times, on
// synthetic lattices of the class's size and count, the two ways the batch can
// step it: one batched launch per step, or the resident kernel (a cluster of
// csize CTAs of `threads` threads per lattice holding it in shared memory, all
// steps of an interval in one launch) for every cluster shape whose shared
// memory holds the lattice and that gives each warp between one and sixteen
// 32-word chunks.  The fastest wins.  Results are kept per device and
// class for the life of the process, so a class is timed once.
//
// The synthetic lattices are zero-filled: the step's work does not depend on
// the state (the collision is a fixed circuit, the draws a fixed chain), only
// on the word count and the obstacle summary, which is clear.
#include <cuda_runtime.h>

#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <chrono>
#include <map>
#include <mutex>
#include <tuple>
#include <vector>

#include "../../include/lgx.h"
#include "lgx_batch.hpp"
#include "lgx_handle.hpp"
#include "lgx_tune.hpp"

namespace lgx {
namespace {

constexpr uint32_t kTuneSteps = 48;
constexpr uint32_t kResidentTuneSteps = 128;  // the longest interval a batch launches
constexpr size_t kTuneMaxWords = 4u << 20;  // per-plane words of all synthetic lattices

std::mutex g_mu;
std::map<std::tuple<int, uint32_t, uint32_t, bool>, ClassPlan> g_plans;
std::map<std::tuple<int, uint32_t, bool, bool, uint32_t>, StepPlan> g_step_plans;

struct Scratch {
  std::vector<void*> ptrs;
  cudaStream_t st = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  ~Scratch() {
    if (st) cudaStreamSynchronize(st);
    for (void* p : ptrs) cudaFree(p);
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    if (st) cudaStreamDestroy(st);
  }
  cudaError_t alloc(void** p, size_t bytes) {
    cudaError_t e = cudaMalloc(p, bytes);
    if (e == cudaSuccess) {
      ptrs.push_back(*p);
      e = cudaMemsetAsync(*p, 0, bytes, st);
    }
    return e;
  }
};

cudaError_t measure(uint32_t words, uint32_t count, bool rest, ClassPlan* out) {
  Scratch s;
  cudaError_t e = cudaStreamCreateWithFlags(&s.st, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreate(&s.e0);
  if (e == cudaSuccess) e = cudaEventCreate(&s.e1);
  if (e != cudaSuccess) return e;
  // a square lattice of `words` words (a power of two): rows of
  // 2^floor((log2 words - 5) / 2) words, as many rows as cells per row or twice
  // as many, an even row count.  The cluster shapes whose bands fit one word per
  // thread, and the halo rows that several steps per barrier recompute, depend
  // on the row width; square lattices are the common case (the transport
  // measurements, the reference's 256 x 256 benchmark).
  uint32_t lg = 0;
  while ((2u << lg) <= words) ++lg;
  const uint32_t wpr = lg >= 5 ? 1u << ((lg - 5) / 2) : 1u;
  uint32_t h = std::max<uint32_t>(6, (words + wpr - 1) / wpr);
  h += h & 1u;
  const Dims dm = make_dims(wpr * 32u, h, 0);
  const uint32_t n = (uint32_t)std::max<size_t>(
      1, std::min<size_t>(count, kTuneMaxWords / dm.total));
  void *planes, *zero, *descs, *sched, *block0, *owner, *base;
  e = s.alloc(&planes, (size_t)n * 2 * 7 * dm.total * 4);
  if (e == cudaSuccess) e = s.alloc(&zero, (size_t)dm.total * 4 + ((dm.total + 31) / 32) * 4);
  if (e == cudaSuccess) e = s.alloc(&descs, (size_t)n * sizeof(LatDesc));
  if (e == cudaSuccess) e = s.alloc(&sched, (size_t)n * sizeof(ResSched));
  if (e == cudaSuccess) e = s.alloc(&block0, (size_t)(n + 1) * 4);
  if (e == cudaSuccess) e = s.alloc(&owner, (size_t)n * ((dm.total + 255) / 256) * 4);
  if (e == cudaSuccess) e = s.alloc(&base, 8);
  if (e != cudaSuccess) return e;
  std::vector<LatDesc> d(n);
  std::vector<uint32_t> b0(n + 1, 0);
  for (uint32_t i = 0; i < n; ++i) {
    LatDesc& x = d[i];
    memset(&x, 0, sizeof(x));
    x.planes[0] = (uint32_t*)planes + (size_t)i * 14 * dm.total;
    x.planes[1] = x.planes[0] + 7 * (size_t)dm.total;
    x.solid = (const uint32_t*)zero;
    x.anysolid = (const uint32_t*)zero + dm.total;
    x.dm = dm;
    x.seed = i;
    x.rest = rest ? 1u : 0u;
    b0[i + 1] = b0[i] + (dm.total + 255) / 256;
  }
  e = cudaMemcpyAsync(descs, d.data(), n * sizeof(LatDesc), cudaMemcpyHostToDevice, s.st);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(block0, b0.data(), (n + 1) * 4, cudaMemcpyHostToDevice, s.st);
  if (e == cudaSuccess)
    e = launch_batch_owner((const uint32_t*)block0, n, b0[n], (uint32_t*)owner, s.st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s.st);
  if (e != cudaSuccess) return e;

  auto time_it = [&](auto&& run, float* us) -> cudaError_t {
    cudaError_t r = run();  // warm-up (and first-launch costs)
    if (r == cudaSuccess) r = cudaEventRecord(s.e0, s.st);
    if (r == cudaSuccess) r = run();
    if (r == cudaSuccess) r = cudaEventRecord(s.e1, s.st);
    if (r == cudaSuccess) r = cudaEventSynchronize(s.e1);
    float ms = 0;
    if (r == cudaSuccess) r = cudaEventElapsedTime(&ms, s.e0, s.e1);
    *us = ms * 1e3f / kTuneSteps;
    return r;
  };
  // one launch per step, replayed from a graph as the batch replays it
  const int rule = rest ? kRuleRest : kRuleNoRest;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  e = cudaStreamBeginCapture(s.st, cudaStreamCaptureModeThreadLocal);
  for (uint32_t k = 0; k < kTuneSteps && e == cudaSuccess; ++k) {
    BatchStepArgs sa{(const LatDesc*)descs, (const uint32_t*)block0, (const uint32_t*)owner, n,
                     (const uint64_t*)base, k, 0};
    e = launch_batch_step(sa, b0[n], rule, kBatchLanes2 | kBatchNoInflow, s.st);
  }
  cudaError_t e2 = cudaStreamEndCapture(s.st, &graph);
  if (e == cudaSuccess) e = e2;
  if (e == cudaSuccess) e = cudaGraphInstantiate(&exec, graph, 0);
  if (graph) cudaGraphDestroy(graph);
  if (e == cudaSuccess) e = time_it([&]() { return cudaGraphLaunch(exec, s.st); }, &out->step_us);
  if (exec) {
    cudaStreamSynchronize(s.st);
    cudaGraphExecDestroy(exec);
  }
  if (e != cudaSuccess) return e;
  out->resident = false;
  out->csize = out->threads = out->ksteps = 0;
  out->resident_us = 0;
  out->tuned_count = n;
  // LGX_RESIDENT_STEPS (1, 2, 4 or 8) pins the steps per cluster barrier of
  // multi-CTA shapes (and, above 1, leaves out single-CTA ones), for tests and
  // measurements; otherwise 1 and 4 are timed, and 8 on the fixed-word kernels
  // (on the others 4 was the best of 2, 4 and 8 on 256 x 256 lattices, and every
  // shape timed costs the first call of a class: timing all four made the
  // 22-density transport scan's one call 0.22 -> 0.27 s; the fixed-word kernels
  // gain from 4 to 8, one 256 x 256 lattice 1.11 -> 1.02 us per step)
  uint32_t pinned_k = 0;
  if (const char* v = getenv("LGX_RESIDENT_STEPS")) {
    const int k = atoi(v);
    if (k == 1 || k == 2 || k == 4 || k == 8) pinned_k = (uint32_t)k;
  }
  // LGX_RESIDENT_FIXED=2 (tests): only the shapes that run on the fixed-word
  // kernels, where the class has any
  const bool only_fixed = resident_fixed_mode() == 2;
  for (int pass = only_fixed ? 0 : 1; pass < 2 && out->resident_us == 0; ++pass)
  for (uint32_t cs : {1u, 2u, 4u, 8u, 16u})
    for (uint32_t th : {128u, 256u, 512u, 1024u})
      for (uint32_t kk : {1u, 2u, 4u, 8u}) {
        if (kk > 1 && cs == 1) continue;  // one CTA: block barriers only
        if (pinned_k && (cs > 1 ? kk != pinned_k : pinned_k > 1)) continue;
        const uint32_t ft = resident_fixed_threads(dm, cs, kk);
        const bool fx = resident_runs_fixed(ft, cs, th, kk);
        if (!pinned_k && kk != 1 && kk != 4 && !(kk == 8 && fx)) continue;
        // chunks of one step, the halo rows recomputed included
        const uint32_t nchunks = (dm.total + cs * 2 * (kk - 1) * dm.wpr + 31) / 32;
        const uint32_t warps = cs * th / 32;
        // the fixed-word kernels take one word per thread: only the smallest
        // block that holds a CTA's words is worth timing
        if (fx) {
          if (th > 128 && ft <= th / 2) continue;
        } else if (pass == 0 || warps > nchunks || warps * 16 < nchunks) {
          continue;
        }
        if (!resident_fits(dm, cs, kk)) continue;
        float us = 0;
        // one launch of a full interval, as the batch runs it
        ResidentArgs ra{(const LatDesc*)descs, (const ResSched*)sched, 0, (const uint64_t*)base,
                        kResidentTuneSteps, kk};
        const size_t smem = resident_smem_bytes(dm, cs, kk);
        cudaError_t r =
            time_it([&]() {
              return launch_resident(ra, n, cs, th, smem, ft, s.st);
            }, &us);
        us *= (float)kTuneSteps / (float)kResidentTuneSteps;
        if (r != cudaSuccess) {
          cudaGetLastError();  // a cluster shape this device cannot place: skip it
          continue;
        }
        if (out->resident_us == 0 || us < out->resident_us) {
          out->resident_us = us;
          out->csize = cs;
          out->threads = th;
          out->ksteps = kk;
        }
      }
  // The resident kernel wins ties within 5%: it launches once per interval, not
  // once per step, and where the two time alike it was the faster in use (eight
  // 256 x 256 lattices timed 2.32-2.37 resident against 2.26-2.39 us per step, a
  // choice that flipped from process to process; transport::measure at 256 x 256
  // took 43 ms with the resident kernel and 50 ms without).
  out->resident = out->resident_us > 0 && out->resident_us < 1.05f * out->step_us;
  return cudaSuccess;
}

// Microseconds per step of `mode` on the scratch lattice: the median of three
// runs of about 1.5 ms of steps each (a multiple of 8, at least 8).  <0: the
// mode failed to run here.
float time_mode_once(lgx_lattice* t, int mode, uint32_t depth, float est_us);

float time_mode(lgx_lattice* t, int mode, uint32_t depth, float est_us) {
  float r[3];
  for (int i = 0; i < 3; ++i) {
    r[i] = time_mode_once(t, mode, depth, est_us > 0 ? est_us : (i ? r[0] : 0.0f));
    if (r[i] < 0) return r[i];
  }
  std::sort(r, r + 3);
  return r[1];
}

// One run of about 1.5 ms of steps, as calls of lgx_advance of up to 64 steps
// each (the public call, which waits for its steps) timed by the host clock:
// what a caller sees, the host's launch rate included.  A first call of the
// same length is not timed (GRAPH captures its graph there).
float time_mode_once(lgx_lattice* t, int mode, uint32_t depth, float est_us) {
  if (lgx_set_step_mode(t, mode) || (depth && lgx_set_temporal_depth(t, (int)depth))) return -1;
  uint64_t k = est_us > 0 ? (uint64_t)(1500.0f / est_us) : 64;
  k = std::min<uint64_t>(std::max<uint64_t>(k, 8), 2048);
  const uint64_t per = std::min<uint64_t>((k + 7) / 8 * 8, 64);
  const uint64_t calls = std::max<uint64_t>(1, k / per);
  if (lgx_advance(t, per)) {
    cudaGetLastError();
    return -1;
  }
  const auto t0 = std::chrono::steady_clock::now();
  for (uint64_t c = 0; c < calls; ++c)
    if (lgx_advance(t, per)) {
      cudaGetLastError();
      return -1;
    }
  const double us =
      std::chrono::duration<double, std::micro>(std::chrono::steady_clock::now() - t0).count();
  return (float)(us / (double)(calls * per));
}

// Lattices up to one full wave of the single-step kernel's blocks (six
// resident 256-word blocks per SM) are offered the one-lattice batch: below
// that the GPU is not full, and one launch per step runs at the host's launch
// rate rather than the kernel's.
uint32_t graph_max_words(int device) {
  int sms = 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return (uint32_t)sms * 6u * 256u;
}

}  // namespace

int plan_step_mode(int device, uint32_t w, uint32_t h, bool rest, StepPlan* out) {
  const Dims dm = make_dims(w, h, 0);
  const bool wide = temporal_supported(dm, 4);
  // the words per row decide which shapes apply: a multiple of 4, of 2, or neither
  const uint32_t lanes = dm.wpr % 4u == 0u ? 4u : dm.wpr % 2u == 0u ? 2u : 1u;
  const auto key = std::make_tuple(device, class_bucket(dm.total), wide, rest, lanes);
  {
    std::lock_guard<std::mutex> g(g_mu);
    auto it = g_step_plans.find(key);
    if (it != g_step_plans.end()) {
      *out = it->second;
      return LGX_OK;
    }
  }
  lgx_lattice* t = nullptr;
  int rc = lgx_create(w, h, rest ? 1 : 0, 0x7E57ull, &t);
  if (rc) return rc;
  StepPlan p{};
  p.mode = LGX_STEP_SINGLE;
  p.words = kShapeChunk1;
  const float est = time_mode(t, LGX_STEP_SINGLE, 0, 0);
  // The candidates: the single-step kernel's shapes (a word per lane in one or
  // two chunks per warp, two or four consecutive words per lane where the rows
  // allow), the wave kernel, temporal blocking, the one-lattice batch.  They
  // are timed in interleaved rounds (every candidate once per round) and each
  // keeps the median of its rounds, so that a fast or slow spell of the host,
  // which paces one launch per step on lattices that do not fill the GPU,
  // falls on all of them alike rather than on whichever ran then.
  struct Cand {
    int mode;
    uint32_t depth, shape;
    float* us;
  };
  std::vector<Cand> cands;
  float* shape_us[4] = {&p.single1_us, &p.single2_us, &p.lanes2_us, &p.lanes4_us};
  for (uint32_t shape = kShapeChunk1; shape <= kShapeLanes4; ++shape)
    if (step_shape(dm, shape) == shape)
      cands.push_back({LGX_STEP_SINGLE, 0, shape, shape_us[shape - 1]});
  cands.push_back({LGX_STEP_WAVE, 0, 0, &p.wave_us});
  if (wide) {
    cands.push_back({LGX_STEP_TEMPORAL, 4, 0, &p.temporal4_us});
    cands.push_back({LGX_STEP_TEMPORAL, 8, 0, &p.temporal8_us});
  }
  if (dm.total <= graph_max_words(device)) cands.push_back({LGX_STEP_GRAPH, 0, 0, &p.graph_us});
  constexpr int kRounds = 5;
  std::vector<std::vector<float>> runs(cands.size());
  for (int r = 0; r < kRounds; ++r)
    for (size_t c = 0; c < cands.size(); ++c) {
      if (!runs[c].empty() && runs[c].back() < 0) continue;  // failed here: out
      t->step_words = cands[c].shape;
      runs[c].push_back(time_mode_once(t, cands[c].mode, cands[c].depth, est));
    }
  t->step_words = 0;
  for (size_t c = 0; c < cands.size(); ++c) {
    std::vector<float>& v = runs[c];
    if (v.empty() || v.back() < 0) continue;  // stays 0: not available
    std::sort(v.begin(), v.end());
    *cands[c].us = v[v.size() / 2];
  }
  for (uint32_t shape = kShapeChunk1; shape <= kShapeLanes4; ++shape) {
    const float us = *shape_us[shape - 1];
    if (us > 0 && (p.single_us <= 0 || us < p.single_us)) {
      p.single_us = us;
      p.words = shape;
    }
  }
  lgx_destroy(t);
  if (p.single_us <= 0) {
    set_error("step-mode tuner: the one-launch-per-step run failed");
    return LGX_ERR_CUDA;
  }
  float best = p.single_us;
  if (p.wave_us > 0 && p.wave_us < best) {
    best = p.wave_us;
    p.mode = LGX_STEP_WAVE;
  }
  if (p.temporal4_us > 0 && p.temporal4_us < best) {
    best = p.temporal4_us;
    p.mode = LGX_STEP_TEMPORAL;
    p.depth = 4;
  }
  if (p.temporal8_us > 0 && p.temporal8_us < best) {
    best = p.temporal8_us;
    p.mode = LGX_STEP_TEMPORAL;
    p.depth = 8;
  }
  // Graph replays do not depend on the host keeping ahead of the GPU, as one
  // launch per step does on these lattices (its rate moves with the host's
  // load: 3.3 to 5.0 us per step at 2048 x 1280 across runs, and within one
  // process the tuner once timed one launch per step at 3.73 against 4.13 us for
  // graphs, then ran it at 4.9 us per step where graphs run at 4.0), so they win
  // ties within 15%.
  if (p.graph_us > 0 && p.graph_us < 1.15f * best) {
    best = p.graph_us;
    p.mode = LGX_STEP_GRAPH;
    p.depth = 0;
  }
  std::lock_guard<std::mutex> g(g_mu);
  g_step_plans[key] = p;
  *out = p;
  return LGX_OK;
}

uint32_t class_bucket(uint32_t words) {
  uint32_t b = 64;
  while (b < words) b <<= 1;
  return b;
}

cudaError_t plan_class(int device, uint32_t words, uint32_t count, bool rest, ClassPlan* out) {
  const uint32_t wb = class_bucket(words);
  uint32_t cb = 1;
  while (cb < count) cb <<= 1;
  const auto key = std::make_tuple(device, wb, cb, rest);
  {
    std::lock_guard<std::mutex> g(g_mu);
    auto it = g_plans.find(key);
    if (it != g_plans.end()) {
      *out = it->second;
      return cudaSuccess;
    }
  }
  ClassPlan p{};
  cudaError_t e = measure(wb, cb, rest, &p);
  if (e != cudaSuccess) return e;
  p.words = wb;
  p.count = cb;
  std::lock_guard<std::mutex> g(g_mu);
  g_plans[key] = p;
  *out = p;
  return cudaSuccess;
}

}  // namespace lgx
