// lgx_batch_host.cpp -- the batch handle: many lattices advanced together.
//
// A batch borrows lattices created with lgx_create (their planes, fields and
// inlet settings) and advances all of them together.  Lattices are grouped
// into size classes; the tuner (lgx_tune.cpp) decides for each class of small
// lattices whether it runs on the resident kernel (a cluster per lattice, all
// steps of an interval in one launch) or with the rest, one batched launch
// per step.  For each sampling interval the batch replays a CUDA graph
// captured on first use:
//   [batched inlet draws] -+-> chain 1: L x batched step (programmatic dependent launch) -+
//                          +-> chain 2: L x batched step                                 -+
//                          +-> one resident launch per class (own sampling)              -+
//                                      -> [batched coarse-graining] -> counter += L
// The graph holds only device pointers to the descriptor table and the step
// counter, so one capture serves every interval of the same length.
#include <cuda_runtime.h>

#include <stdlib.h>

#include <algorithm>
#include <new>
#include <string>
#include <vector>

#include "../../include/lgx.h"
#include "lgx_batch.hpp"
#include "lgx_handle.hpp"
#include "lgx_tune.hpp"

namespace {

struct GraphEntry {
  uint32_t len;
  bool sample;
  cudaGraphExec_t exec;
  lgx::ResSched* sched;  // resident lattices' schedule for this interval shape
};

// A chain of per-step launches over lattices [first, first + count), with its
// own block table; several chains run as parallel branches of the graph so
// that one chain's launch gaps are filled by the others' blocks.
struct StepGroup {
  uint32_t first = 0, count = 0, nblocks = 0, rest_blocks = 0;
  bool wpr4 = true;     // every lattice of the chain has a multiple of 4 words per row
  bool inflow = false;  // some lattice of the chain has an inflow
  uint32_t* d_block0 = nullptr;
  uint32_t* d_owner = nullptr;
  cudaStream_t st = nullptr;  // null for the batch's own stream
  cudaEvent_t done = nullptr;
};

// A size class on the resident kernel: lattices [first, first + count).
struct ResClass {
  uint32_t first, count;
  lgx::ClassPlan plan;
  size_t smem;  // shared memory per CTA: the largest member's band
  uint32_t fixed_threads;  // the largest member's resident_fixed_threads (0: one has none)
};

int cuda_fail(cudaError_t e, const char* what) {
  lgx::set_error(std::string(what) + ": " + cudaGetErrorString(e));
  return LGX_ERR_CUDA;
}

#define LGX_CUDA(call)                                  \
  do {                                                  \
    cudaError_t e_ = (call);                            \
    if (e_ != cudaSuccess) return cuda_fail(e_, #call); \
  } while (0)

}  // namespace

struct lgx_batch {
  int device = 0;
  cudaStream_t stream = nullptr;
  bool own_stream = true;  // false: a member lattice's stream, borrowed
  std::vector<lgx_lattice*> lats;
  std::vector<lgx::LatDesc> descs;
  lgx::LatDesc* d_descs = nullptr;
  uint32_t* d_item0 = nullptr;
  uint32_t* d_blk0 = nullptr;
  uint32_t* d_tile0 = nullptr;
  uint64_t* d_base = nullptr;
  uint32_t nblocks = 0;
  uint32_t rest_blocks = 0;     // leading per-step blocks, those of rest-particle lattices
  uint32_t items_per_step = 0;  // inlet draw items of one step, all lattices
  uint64_t item0_len = 1;       // the interval length d_item0 holds the prefix for
  uint32_t field_blocks = 0;  // blocks coarse-grained a warp each
  uint32_t field_tiles = 0;   // tiles of the lattices coarse-grained by tiles
  std::vector<uint32_t*> inlet_bufs;
  std::vector<GraphEntry> graphs;
  uint64_t launches = 0;
  uint64_t graph_launches = 0;
  cudaEvent_t ev[8] = {};
  lgx::BatchStepHook hook = nullptr;
  void* hook_ctx = nullptr;
  bool hook_per_step = true;
  int policy = LGX_BATCH_AUTO;
  uint32_t nstep = 0;                 // leading lattices stepped one launch per step
  std::vector<ResClass> classes;      // then the resident classes
  std::vector<lgx_batch_class> plan;  // every class, as reported
  cudaStream_t side = nullptr;        // resident launches' branch of the graph
  cudaEvent_t fork = nullptr, join = nullptr;
  std::vector<StepGroup> groups;      // chains of per-step launches
};

namespace {

// The per-step chains: contiguous runs of the per-step lattices, balanced by
// blocks.  Two chains fill each other's launch gaps (+6% on the 64-lattice
// transport sweep; three or four gain nothing more); LGX_BATCH_CHAINS
// overrides the count at creation.
void free_chains(lgx_batch* b) {
  for (auto& g : b->groups) {
    cudaFree(g.d_block0);
    cudaFree(g.d_owner);
    if (g.done) cudaEventDestroy(g.done);
    if (g.st) cudaStreamDestroy(g.st);
  }
  b->groups.clear();
}

cudaError_t build_chains(lgx_batch* b, uint32_t ngroups) {
  free_chains(b);
  ngroups = std::min<uint32_t>(ngroups, b->nstep);
  std::vector<uint32_t> block0(b->nstep + 1, 0);
  for (uint32_t i = 0; i < b->nstep; ++i)
    block0[i + 1] = block0[i] + (b->lats[i]->dm.total + 255) / 256;
  cudaError_t e = cudaSuccess;
  for (uint32_t g = 0, i = 0; g < ngroups && e == cudaSuccess; ++g) {
    StepGroup sg;
    sg.first = i;
    const uint64_t target = (uint64_t)block0[b->nstep] * (g + 1) / ngroups;
    std::vector<uint32_t> gb0(1, 0);
    while (i < b->nstep && (g + 1 == ngroups || block0[i] < target || sg.count == 0)) {
      gb0.push_back(gb0.back() + block0[i + 1] - block0[i]);
      if (b->lats[i]->rest) sg.rest_blocks = gb0.back();
      sg.wpr4 = sg.wpr4 && b->lats[i]->dm.wpr % 4u == 0u;
      sg.inflow = sg.inflow || b->lats[i]->dm.iw != 0u;
      ++sg.count;
      ++i;
    }
    if (sg.count == 0) continue;
    sg.nblocks = gb0.back();
    b->groups.push_back(sg);
    StepGroup& G = b->groups.back();
    e = cudaMalloc(&G.d_block0, gb0.size() * 4);
    if (e == cudaSuccess)
      e = cudaMemcpy(G.d_block0, gb0.data(), gb0.size() * 4, cudaMemcpyHostToDevice);
    if (e == cudaSuccess && G.nblocks) e = cudaMalloc(&G.d_owner, (size_t)G.nblocks * 4);
    if (e == cudaSuccess)
      e = lgx::launch_batch_owner(G.d_block0, G.count, G.nblocks, G.d_owner, b->stream);
    if (e == cudaSuccess && g > 0) e = cudaStreamCreateWithFlags(&G.st, cudaStreamNonBlocking);
    if (e == cudaSuccess && g > 0) e = cudaEventCreateWithFlags(&G.done, cudaEventDisableTiming);
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(b->stream);
  return e;
}

void free_batch(lgx_batch* b) {
  cudaSetDevice(b->device);
  if (b->stream) cudaStreamSynchronize(b->stream);
  for (auto& g : b->graphs) {
    cudaGraphExecDestroy(g.exec);
    cudaFree(g.sched);
  }
  for (auto* p : b->inlet_bufs) cudaFree(p);
  free_chains(b);
  if (b->fork) cudaEventDestroy(b->fork);
  if (b->join) cudaEventDestroy(b->join);
  if (b->side) cudaStreamDestroy(b->side);
  cudaFree(b->d_descs);
  cudaFree(b->d_item0);
  cudaFree(b->d_blk0);
  cudaFree(b->d_tile0);
  cudaFree(b->d_base);
  for (auto& ev : b->ev)
    if (ev) cudaEventDestroy(ev);
  if (b->stream && b->own_stream) cudaStreamDestroy(b->stream);
  delete b;
}

// Snapshot the member lattices into descriptors (steps, parity, field).
int setup_descs(lgx_batch* b, float alpha) {
  const size_t n = b->lats.size();
  b->descs.resize(n);
  for (size_t i = 0; i < n; ++i) {
    lgx_lattice* l = b->lats[i];
    lgx::LatDesc& d = b->descs[i];
    d.planes[0] = l->planes[l->cur];
    d.planes[1] = l->planes[l->cur ^ 1];
    d.solid = l->solid;
    d.anysolid = l->anysolid;
    d.inlet = b->inlet_bufs[i];
    d.dm = l->dm;
    d.seed = l->seed;
    d.steps0 = l->steps;
    d.cur0 = 0;
    d.rest = l->rest ? 1u : 0u;
    for (int k = 0; k < 7; ++k) d.thresh[k] = l->thresh[k];
    d.field = l->has_field ? l->field : nullptr;
    d.sums = l->has_field ? l->sums : nullptr;
    d.bx = l->bx;
    d.by = l->by;
    d.bw = l->has_field ? l->bw : 0;
    d.bh = l->has_field ? l->bh : 0;
    d.alpha = alpha;
  }
  LGX_CUDA(cudaMemcpyAsync(b->d_descs, b->descs.data(), n * sizeof(lgx::LatDesc),
                           cudaMemcpyHostToDevice, b->stream));
  LGX_CUDA(cudaMemsetAsync(b->d_base, 0, sizeof(uint64_t), b->stream));
  return LGX_OK;
}

// One launch per step: the specialised kernel when every lattice has the same
// rule, the mixed one otherwise (rest-particle lattices' blocks come first).
int step_rule(uint32_t rest_blocks, uint32_t nblocks) {
  if (rest_blocks == nblocks) return lgx::kRuleRest;
  if (rest_blocks == 0) return lgx::kRuleNoRest;
  return lgx::kRuleMixed;
}

int capture(lgx_batch* b, uint32_t len, bool sample, cudaGraphExec_t* out,
            lgx::ResSched** sched_out) {
  // the resident lattices sample at the end of the interval, when it samples
  const size_t n = b->lats.size();
  lgx::ResSched* sched = nullptr;
  if (!b->classes.empty()) {
    std::vector<lgx::ResSched> h(n, lgx::ResSched{sample ? len : 0u, 0u, len});
    LGX_CUDA(cudaMalloc(&sched, n * sizeof(lgx::ResSched)));
    *sched_out = sched;
    LGX_CUDA(cudaMemcpy(sched, h.data(), n * sizeof(lgx::ResSched), cudaMemcpyHostToDevice));
  }
  cudaGraph_t graph = nullptr;
  LGX_CUDA(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
  cudaError_t e = cudaSuccess;
  if (b->items_per_step) {
    lgx::BatchInletArgs ia{b->d_descs, b->d_item0, (uint32_t)b->lats.size(),
                           b->items_per_step * len, b->d_base};
    // the draws of one lattice are laid out step-major in its own buffer, so
    // the item prefix scales with the interval length
    e = lgx::launch_batch_inlet(ia, b->stream);
  }
  // branches: the resident classes (when there is also a per-step chain) and
  // every per-step chain after the first
  const bool res_branch = !b->classes.empty() && b->nstep;
  const bool fork = res_branch || b->groups.size() > 1;
  if (e == cudaSuccess && fork) e = cudaEventRecord(b->fork, b->stream);
  if (e == cudaSuccess && res_branch) e = cudaStreamWaitEvent(b->side, b->fork, 0);
  for (size_t g = 1; g < b->groups.size() && e == cudaSuccess; ++g)
    e = cudaStreamWaitEvent(b->groups[g].st, b->fork, 0);
  cudaStream_t rs = res_branch ? b->side : b->stream;
  for (const ResClass& c : b->classes) {
    if (e != cudaSuccess) break;
    lgx::ResidentArgs ra{b->d_descs, sched, c.first, b->d_base, len, c.plan.ksteps};
    e = lgx::launch_resident(ra, c.count, c.plan.csize, c.plan.threads, c.smem,
                             c.fixed_threads, rs);
  }
  for (size_t g = 0; g < b->groups.size() && e == cudaSuccess; ++g) {
    const StepGroup& sg = b->groups[g];
    cudaStream_t st = sg.st ? sg.st : b->stream;
    for (uint32_t k = 0; k < len && e == cudaSuccess; ++k) {
      // rest-particle lattices' blocks first, then the six-direction ones
      lgx::BatchStepArgs sa{b->d_descs + sg.first, sg.d_block0, sg.d_owner, sg.count,
                            b->d_base, k, 0};
      e = lgx::launch_batch_step(sa, sg.nblocks, step_rule(sg.rest_blocks, sg.nblocks),
                                 lgx::batch_step_words(sg.nblocks, sg.wpr4, sg.inflow), st);
      if (e == cudaSuccess && b->hook && b->hook_per_step)
        e = b->hook(b->hook_ctx, st, b->d_base, k + 1);
    }
    if (e == cudaSuccess && sg.st) {
      e = cudaEventRecord(sg.done, sg.st);
      if (e == cudaSuccess) e = cudaStreamWaitEvent(b->stream, sg.done, 0);
    }
  }
  if (e == cudaSuccess && sample && (b->field_blocks || b->field_tiles)) {
    lgx::BatchSampleArgs sp{b->d_descs, b->d_blk0, b->nstep,  b->field_blocks,
                            b->d_base,  len,       b->d_tile0, b->field_tiles};
    e = lgx::launch_batch_sample(sp, b->stream);
  }
  if (e == cudaSuccess && res_branch) {
    e = cudaEventRecord(b->join, b->side);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(b->stream, b->join, 0);
  }
  if (e == cudaSuccess && sample && b->hook && !b->hook_per_step)
    e = b->hook(b->hook_ctx, b->stream, b->d_base, len);
  if (e == cudaSuccess) e = lgx::launch_batch_base(b->d_base, len, b->stream);
  cudaError_t e2 = cudaStreamEndCapture(b->stream, &graph);
  if (e != cudaSuccess) {
    if (graph) cudaGraphDestroy(graph);
    return cuda_fail(e, "batch graph capture");
  }
  if (e2 != cudaSuccess) return cuda_fail(e2, "cudaStreamEndCapture");
  e = cudaGraphInstantiate(out, graph, 0);
  cudaGraphDestroy(graph);
  if (e != cudaSuccess) return cuda_fail(e, "cudaGraphInstantiate");
  return LGX_OK;
}

// Captured interval shapes a batch keeps; lengths beyond them run as
// power-of-two pieces, so a caller that advances by many different lengths
// does not pay a capture for each.
constexpr size_t kMaxGraphs = 24;

bool has_graph(const lgx_batch* b, uint32_t len, bool sample) {
  for (const auto& g : b->graphs)
    if (g.len == len && g.sample == sample) return true;
  return false;
}

int graph_for(lgx_batch* b, uint32_t len, bool sample, cudaGraphExec_t* out) {
  for (auto& g : b->graphs)
    if (g.len == len && g.sample == sample) {
      *out = g.exec;
      return LGX_OK;
    }
  cudaGraphExec_t ex = nullptr;
  lgx::ResSched* sched = nullptr;
  int rc = capture(b, len, sample, &ex, &sched);
  if (rc) {
    cudaFree(sched);
    return rc;
  }
  b->graphs.push_back({len, sample, ex, sched});
  *out = ex;
  return LGX_OK;
}

}  // namespace

namespace lgx {

int batch_set_step_hook(lgx_batch* b, BatchStepHook fn, void* ctx, bool per_step) {
  if (!b) {
    lgx::set_error("null batch handle");
    return LGX_ERR_ARG;
  }
  if (fn && per_step && !b->classes.empty()) {
    lgx::set_error("a per-step hook needs every lattice stepped one launch per step");
    return LGX_ERR_STATE;
  }
  LGX_CUDA(cudaSetDevice(b->device));
  LGX_CUDA(cudaStreamSynchronize(b->stream));
  if (fn && per_step && b->groups.size() > 1)
    LGX_CUDA(build_chains(b, 1));  // the hook follows every step of every lattice
  for (auto& g : b->graphs) {
    cudaGraphExecDestroy(g.exec);
    cudaFree(g.sched);
  }
  b->graphs.clear();
  b->hook = fn;
  b->hook_ctx = ctx;
  b->hook_per_step = per_step;
  return LGX_OK;
}

}  // namespace lgx

extern "C" {

int lgx_batch_create(lgx_lattice* const* lats, size_t n, lgx_batch** out) {
  return lgx::batch_create(lats, n, LGX_BATCH_AUTO, nullptr, out);
}

int lgx_batch_create_ex(lgx_lattice* const* lats, size_t n, int policy, lgx_batch** out) {
  return lgx::batch_create(lats, n, policy, nullptr, out);
}

}  // extern "C"

// A batch whose work runs on `stream` (a member lattice's own stream, which it
// neither creates nor destroys), or on a stream of its own when that is null.
int lgx::batch_create(lgx_lattice* const* lats, size_t n, int policy, cudaStream_t stream,
                      lgx_batch** out) {
  if (policy != LGX_BATCH_AUTO && policy != LGX_BATCH_PER_STEP && policy != LGX_BATCH_RESIDENT) {
    lgx::set_error("lgx_batch_create_ex: unknown policy");
    return LGX_ERR_ARG;
  }
  if (!out || !lats || n == 0) {
    lgx::set_error("lgx_batch_create: need at least one lattice");
    return LGX_ERR_ARG;
  }
  *out = nullptr;
  for (size_t i = 0; i < n; ++i)
    if (!lats[i] || lats[i]->device != lats[0]->device) {
      lgx::set_error("lgx_batch_create: null lattice, or lattices on different devices");
      return LGX_ERR_ARG;
    }
  for (size_t i = 0; i < n; ++i)
    for (size_t j = 0; j < i; ++j)
      if (lats[i] == lats[j]) {
        lgx::set_error("lgx_batch_create: a lattice appears twice");
        return LGX_ERR_ARG;
      }
  lgx_batch* b = new (std::nothrow) lgx_batch();
  if (!b) {
    lgx::set_error("out of host memory");
    return LGX_ERR_ALLOC;
  }
  b->device = lats[0]->device;
  b->policy = policy;
  cudaError_t e = cudaSetDevice(b->device);
  // size classes of the small lattices (words rounded up to a power of two,
  // and the rule), each planned by the tuner
  std::vector<int> cls(n, -1);
  struct Key {
    uint32_t words;
    bool rest;
    uint32_t count;
    lgx::ClassPlan plan;
  };
  std::vector<Key> keys;
  for (size_t i = 0; i < n && policy != LGX_BATCH_PER_STEP; ++i) {
    if (lats[i]->dm.total > lgx::kResidentMaxWords) continue;
    const uint32_t wb = lgx::class_bucket(lats[i]->dm.total);
    size_t k = 0;
    while (k < keys.size() && !(keys[k].words == wb && keys[k].rest == lats[i]->rest)) ++k;
    if (k == keys.size()) keys.push_back({wb, lats[i]->rest, 0, {}});
    keys[k].count += 1;
    cls[i] = (int)k;
  }
  std::sort(keys.begin(), keys.end(), [](const Key& a, const Key& c) {
    return a.words != c.words ? a.words < c.words : a.rest > c.rest;
  });
  for (size_t i = 0; i < n; ++i) {  // class index after the sort
    if (cls[i] < 0) continue;
    const uint32_t wb = lgx::class_bucket(lats[i]->dm.total);
    size_t k = 0;
    while (!(keys[k].words == wb && keys[k].rest == lats[i]->rest)) ++k;
    cls[i] = (int)k;
  }
  std::vector<bool> res_class(keys.size(), false);
  for (size_t k = 0; k < keys.size() && e == cudaSuccess; ++k) {
    if (lgx::plan_class(b->device, keys[k].words, keys[k].count, keys[k].rest, &keys[k].plan) !=
        cudaSuccess) {
      // the tuner could not run here (e.g. no room for its synthetic lattices):
      // the class takes one launch per step
      cudaGetLastError();
      keys[k].plan = lgx::ClassPlan{};
    }
    lgx::ClassPlan& p = keys[k].plan;
    res_class[k] = policy == LGX_BATCH_RESIDENT ? p.csize != 0 : p.resident;
    // every member's band must fit, and hold the halo rows of the class's steps
    // per cluster barrier (fewer steps per barrier where a member's bands are short)
    auto all_fit = [&](uint32_t kk) {
      for (size_t i = 0; i < n; ++i)
        if (cls[i] == (int)k && !lgx::resident_fits(lats[i]->dm, p.csize, kk)) return false;
      return true;
    };
    if (p.ksteps == 0) p.ksteps = 1;
    while (res_class[k] && p.ksteps > 1 && !all_fit(p.ksteps)) p.ksteps /= 2;
    if (res_class[k] && !all_fit(p.ksteps)) res_class[k] = false;
    lgx_batch_class c{};
    c.words = keys[k].words;
    c.lattices = keys[k].count;
    c.rest = keys[k].rest ? 1 : 0;
    c.resident = res_class[k] ? 1 : 0;
    c.cluster = p.csize;
    c.threads = p.threads;
    c.steps_per_barrier = p.ksteps;
    c.step_us = p.step_us;
    c.resident_us = p.resident_us;
    b->plan.push_back(c);
  }
  // order: per-step lattices (rest-particle ones first, so each rule's blocks
  // are one contiguous run), then each resident class
  for (int pass = 0; pass < 2; ++pass)
    for (size_t i = 0; i < n; ++i)
      if ((cls[i] < 0 || !res_class[cls[i]]) && lats[i]->rest == (pass == 0))
        b->lats.push_back(lats[i]);
  b->nstep = (uint32_t)b->lats.size();
  for (size_t k = 0; k < keys.size(); ++k) {
    if (!res_class[k]) continue;
    ResClass rc{(uint32_t)b->lats.size(), 0, keys[k].plan, 0, 0};
    bool fixed = true;
    for (size_t i = 0; i < n; ++i)
      if (cls[i] == (int)k) {
        b->lats.push_back(lats[i]);
        rc.smem = std::max(rc.smem, lgx::resident_smem_bytes(lats[i]->dm, rc.plan.csize,
                                                             rc.plan.ksteps));
        const uint32_t ft =
            lgx::resident_fixed_threads(lats[i]->dm, rc.plan.csize, rc.plan.ksteps);
        fixed = fixed && ft != 0;
        rc.fixed_threads = std::max(rc.fixed_threads, ft);
      }
    if (!fixed) rc.fixed_threads = 0;
    b->plan[k].word_per_thread = lgx::resident_runs_fixed(rc.fixed_threads, rc.plan.csize,
                                                          rc.plan.threads, rc.plan.ksteps);
    rc.count = (uint32_t)b->lats.size() - rc.first;
    b->classes.push_back(rc);
  }
  lats = b->lats.data();
  if (stream) {
    b->stream = stream;
    b->own_stream = false;
  } else if (e == cudaSuccess) {
    e = cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking);
  }
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&b->side, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->join, cudaEventDisableTiming);
  for (int i = 0; i < 8 && e == cudaSuccess; ++i) e = cudaEventCreate(&b->ev[i]);
  // block table of the per-step lattices: each padded to whole 256-word blocks
  // and the coarse-graining tables: a warp per block for fields of narrow
  // blocks, tiles (tile_shape) for the others
  std::vector<uint32_t> block0(n + 1, 0), item0(n + 1, 0), blk0(n + 1, 0), tile0(n + 1, 0);
  for (size_t i = 0; i < n && e == cudaSuccess; ++i) {
    const lgx_lattice* l = lats[i];
    const lgx::Dims& dm = l->dm;
    const bool step = i < b->nstep;
    block0[i + 1] = block0[i] + (step ? (dm.total + 255) / 256 : 0);
    if (step && l->rest) b->rest_blocks = block0[i + 1];
    item0[i + 1] = item0[i] + dm.h * dm.iw;
    const bool field = step && l->has_field && l->bw * l->bh > 0;
    const bool tiled = field && l->bx >= lgx::kTileMinWidth;
    uint32_t per = 0, ncx = 0;
    if (tiled) lgx::tile_shape(l->bx, l->bw, &per, &ncx);
    blk0[i + 1] = blk0[i] + (field && !tiled ? l->bw * l->bh : 0);
    tile0[i + 1] = tile0[i] + (tiled ? ncx * l->bh : 0);
  }
  b->nblocks = block0[n];
  b->items_per_step = item0[n];
  b->field_blocks = blk0[n];
  b->field_tiles = tile0[n];
  if (e == cudaSuccess) e = cudaMalloc(&b->d_descs, n * sizeof(lgx::LatDesc));
  if (e == cudaSuccess) e = cudaMalloc(&b->d_item0, (n + 1) * sizeof(uint32_t));
  if (e == cudaSuccess) e = cudaMalloc(&b->d_blk0, (n + 1) * sizeof(uint32_t));
  if (e == cudaSuccess) e = cudaMalloc(&b->d_tile0, (n + 1) * sizeof(uint32_t));
  if (e == cudaSuccess) e = cudaMalloc(&b->d_base, sizeof(uint64_t));
  uint32_t chains = 2;
  if (const char* v = getenv("LGX_BATCH_CHAINS")) chains = (uint32_t)std::max(1, atoi(v));
  if (e == cudaSuccess) e = build_chains(b, chains);
  if (e == cudaSuccess) e = cudaStreamSynchronize(b->stream);
  // The batched inlet kernel writes lattice i's draws for step s of the
  // interval at item (item0[i] * len + s * h * iw ...); lay the prefix out
  // for the longest interval and let each buffer hold kInletChunk steps.
  b->inlet_bufs.assign(n, nullptr);
  for (size_t i = 0; i < n && e == cudaSuccess; ++i) {
    const lgx::Dims& dm = lats[i]->dm;
    if (dm.iw)
      e = cudaMalloc(&b->inlet_bufs[i], (size_t)lgx::kInletChunk * dm.h * dm.iw * 7 * 4);
  }
  if (e == cudaSuccess) e = cudaMemcpy(b->d_item0, item0.data(), (n + 1) * 4, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(b->d_blk0, blk0.data(), (n + 1) * 4, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(b->d_tile0, tile0.data(), (n + 1) * 4, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    const int rc = (e == cudaErrorMemoryAllocation) ? LGX_ERR_ALLOC : LGX_ERR_CUDA;
    lgx::set_error(std::string("lgx_batch_create: ") + cudaGetErrorString(e));
    free_batch(b);
    return rc;
  }
  *out = b;
  return LGX_OK;
}

extern "C" {

int lgx_batch_destroy(lgx_batch* b) {
  if (b) free_batch(b);
  return LGX_OK;
}

int lgx_batch_advance_sampling(lgx_batch* b, uint64_t n, uint64_t every, float alpha) {
  if (!b) {
    lgx::set_error("null batch handle");
    return LGX_ERR_ARG;
  }
  LGX_CUDA(cudaSetDevice(b->device));
  // Field and block tables were laid out at creation; pending work on a
  // member's own stream finishes first.
  for (lgx_lattice* l : b->lats)
    if (l->stream != b->stream) LGX_CUDA(cudaStreamSynchronize(l->stream));
  int rc = setup_descs(b, alpha);
  if (rc) return rc;
  // The inlet draws of an interval are laid out per lattice as [k][h][iw][7];
  // the batched inlet kernel's item index runs lattice-major with each
  // lattice's items for the whole interval contiguous, so the prefix is
  // scaled by the interval length when the interval differs from one step.
  uint64_t left = n, since = 0;
  while (left > 0) {
    uint64_t len = std::min<uint64_t>(left, lgx::kInletChunk);
    if (every > 0) len = std::min<uint64_t>(len, every - since);
    bool sample = every > 0 && (since + len >= every || len == left);
    if (b->graphs.size() >= kMaxGraphs && !has_graph(b, (uint32_t)len, sample)) {
      // enough shapes captured: run a new length as power-of-two pieces
      uint64_t p2 = 1;
      while (p2 * 2 <= len) p2 *= 2;
      len = p2;
      sample = every > 0 && (since + len >= every || len == left);
    }
    if (b->items_per_step && b->item0_len != len) {
      // prefix for this interval length (kept on the device while it repeats)
      std::vector<uint32_t> item0(b->lats.size() + 1, 0);
      for (size_t i = 0; i < b->lats.size(); ++i)
        item0[i + 1] = item0[i] + (uint32_t)len * b->lats[i]->dm.h * b->lats[i]->dm.iw;
      LGX_CUDA(cudaMemcpyAsync(b->d_item0, item0.data(), item0.size() * 4,
                               cudaMemcpyHostToDevice, b->stream));
      b->item0_len = len;
    }
    cudaGraphExec_t ex = nullptr;
    rc = graph_for(b, (uint32_t)len, sample, &ex);
    if (rc) return rc;
    LGX_CUDA(cudaGraphLaunch(ex, b->stream));
    b->graph_launches += 1;
    const uint64_t per_step = b->groups.size();
    b->launches += len * (per_step + (b->hook && b->hook_per_step ? 1 : 0)) + 1 +
                   (b->hook && !b->hook_per_step && sample ? 1 : 0) +
                   (sample && b->field_blocks ? 1 : 0) + (sample && b->field_tiles ? 1 : 0) +
                   (b->items_per_step ? 1 : 0) +
                   b->classes.size();
    left -= len;
    since += len;
    if (sample) since = 0;
  }
  LGX_CUDA(cudaStreamSynchronize(b->stream));
  for (lgx_lattice* l : b->lats) {
    l->steps += n;
    l->cur ^= (int)(n & 1u);
    l->inlet_valid = 0;  // the lattice's own inlet draws are for earlier steps
  }
  return LGX_OK;
}

int lgx_batch_advance(lgx_batch* b, uint64_t n) { return lgx_batch_advance_sampling(b, n, 0, 0.f); }

int lgx_batch_plan(lgx_batch* b, lgx_batch_class* out, size_t cap, size_t* n) {
  if (!b || !n || (cap && !out)) {
    lgx::set_error("lgx_batch_plan: bad argument");
    return LGX_ERR_ARG;
  }
  *n = b->plan.size();
  for (size_t i = 0; i < b->plan.size() && i < cap; ++i) out[i] = b->plan[i];
  return LGX_OK;
}

int lgx_batch_launch_count(lgx_batch* b, uint64_t* kernels, uint64_t* graphs) {
  if (!b) {
    lgx::set_error("null batch handle");
    return LGX_ERR_ARG;
  }
  if (kernels) *kernels = b->launches;
  if (graphs) *graphs = b->graph_launches;
  return LGX_OK;
}

int lgx_batch_timing_mark(lgx_batch* b, int slot) {
  if (!b || slot < 0 || slot >= 8) {
    lgx::set_error("lgx_batch_timing_mark: bad argument");
    return LGX_ERR_ARG;
  }
  LGX_CUDA(cudaEventRecord(b->ev[slot], b->stream));
  return LGX_OK;
}

int lgx_batch_timing_elapsed(lgx_batch* b, int a, int c, float* ms) {
  if (!b || a < 0 || a >= 8 || c < 0 || c >= 8 || !ms) {
    lgx::set_error("lgx_batch_timing_elapsed: bad argument");
    return LGX_ERR_ARG;
  }
  LGX_CUDA(cudaEventSynchronize(b->ev[c]));
  LGX_CUDA(cudaEventElapsedTime(ms, b->ev[a], b->ev[c]));
  return LGX_OK;
}

}  // extern "C"
