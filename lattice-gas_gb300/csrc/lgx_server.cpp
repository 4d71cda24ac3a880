// lgx_server.cpp -- a serving loop with continuous batching.
//
// Requests (a lattice, its run length, sampling period, block size and
// inflow) are submitted from any thread.  One server thread admits them
// against a fixed device-memory budget, keeps every admitted lattice's planes
// resident on the device, and advances all of them together in ticks: a tick
// is as many steps (up to 128) as every resident lattice can take before one
// of them reaches its end, run as one batched launch per step (programmatic
// dependent launch, both collision rules in one launch), with one batched
// coarse-graining of exactly the lattices that reach a sampling point after
// the steps where any do.  A finished lattice's field, exact block sums and
// particle count are copied back (only the moments ever leave the device),
// its memory returns to the pool, and waiting requests take its place the
// next tick -- so requests arriving while others run join them on the GPU.
//
// Every step count is known on the host, so the loop never reads the device
// to decide anything: it runs up to kRing ticks ahead of the GPU, reusing a
// ring of descriptor buffers as their events complete.
//
// The physics of each lattice is exactly lgx_advance_sampling on a fresh
// lattice with the same cells and seed (src/gpu.rs:668-706): samples every
// sample_every steps and after the last, the field starting from zero.
#include <cuda_runtime.h>
#include <string.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <new>
#include <string>
#include <thread>
#include <vector>

#include "../../include/lgx.h"
#include "lgx_batch.hpp"
#include "lgx_handle.hpp"

namespace {

constexpr int kRing = 4;
constexpr size_t kMaxSamplePoints = 16;  // batched coarse-grainings per tick
constexpr size_t kChains = 2;            // parallel launch chains per tick

double now_s() {
  using namespace std::chrono;
  return duration<double>(steady_clock::now().time_since_epoch()).count();
}

struct Req {
  uint64_t id = 0;
  lgx_request spec{};
  std::vector<uint8_t> cells;
  int state = LGX_REQ_QUEUED;
  std::string error;
  double t_submit = 0, t_admit = 0, t_done = 0;
  bool cancel = false;
  // device
  lgx::Dims dm{};
  uint32_t thresh[7] = {};
  uint32_t bw = 0, bh = 0;
  size_t bytes = 0;
  uint32_t* planes[2] = {nullptr, nullptr};
  uint32_t* solid = nullptr;
  uint32_t* anysolid = nullptr;
  uint8_t* dcells = nullptr;
  uint32_t* inlet = nullptr;
  float* field = nullptr;
  int32_t* sums = nullptr;
  unsigned long long* count = nullptr;
  uint64_t steps_done = 0, since = 0;
  int cur = 0;
  // results, page-locked
  float* res_field = nullptr;
  int32_t* res_sums = nullptr;
  unsigned long long* res_count = nullptr;
  cudaEvent_t done_ev = nullptr;
};

size_t device_bytes(const lgx::Dims& dm, uint32_t nb) {
  const size_t total = dm.total;
  size_t b = 2 * total * 7 * 4 + total * 4 + ((total + 31) / 32) * 4 + (size_t)dm.w * dm.h;
  b += (size_t)lgx::kInletChunk * dm.h * dm.iw * 7 * 4;
  b += (size_t)nb * 32 + 8;
  return b;
}

}  // namespace

struct lgx_server {
  int device = 0;
  cudaStream_t stream = nullptr;
  cudaStream_t stream2 = nullptr;           // the second launch chain of a tick
  cudaEvent_t fork = nullptr, join = nullptr;
  cudaMemPool_t pool = nullptr;
  size_t budget = 0, in_use = 0;
  size_t max_active = 0;
  std::mutex mu;
  std::condition_variable cv;
  std::thread thr;
  bool stop = false;
  uint64_t next_id = 1;
  std::map<uint64_t, std::unique_ptr<Req>> reqs;
  std::deque<Req*> pending;
  std::vector<Req*> active;
  std::vector<Req*> retiring;
  // tick ring
  struct Slot {
    void* host = nullptr;   // pinned: descs | block0 | item0 | blk tables
    void* dev = nullptr;
    cudaEvent_t ev = nullptr;   // the tick's end
    cudaEvent_t ev0 = nullptr;  // and its start, for the device time of ticks
    uint32_t* owner = nullptr;  // lattice of each step block (stream-ordered allocation)
    size_t owner_cap = 0;
    bool used = false;
  } ring[kRing];
  size_t slot_bytes = 0;
  int next_slot = 0;
  uint64_t* d_zero = nullptr;
  // statistics (written by the server thread without the lock)
  std::atomic<uint64_t> ticks{0}, launches{0}, site_updates{0};
  std::atomic<size_t> in_use_now{0};
  std::atomic<size_t> peak_bytes{0}, peak_active{0};
  std::atomic<uint64_t> gpu_busy_ns{0};  // device time of finished ticks
  std::atomic<uint64_t> host_tick_ns{0};  // host time spent in ticks
  std::atomic<uint64_t> host_wait_ns{0};  // of which waiting for a ring slot (the device)
  int fault_alloc = 0;  // test hook: fail the next N admissions' allocation
  std::string fatal;
};

namespace {

void release_device(lgx_server* s, Req* r) {
  void* ptrs[] = {r->planes[0], r->planes[1], r->solid, r->anysolid, r->dcells,
                  r->inlet,     r->field,     r->sums,  r->count};
  for (void* p : ptrs)
    if (p) cudaFreeAsync(p, s->stream);
  r->planes[0] = r->planes[1] = nullptr;
  r->solid = r->anysolid = nullptr;
  r->dcells = nullptr;
  r->inlet = nullptr;
  r->field = nullptr;
  r->sums = nullptr;
  r->count = nullptr;
  s->in_use -= r->bytes;
  s->in_use_now = s->in_use;
  r->bytes = 0;
}

// Allocate and load one request; false (with r->error) on failure.  Runs on
// the server thread without the lock; `inject` is the test hook's decision.
bool admit(lgx_server* s, Req* r, bool inject) {
  const lgx_request& q = r->spec;
  r->dm = lgx::make_dims((uint32_t)q.w, (uint32_t)q.h, (uint32_t)q.inlet_cols);
  r->bw = (uint32_t)(q.w / q.bx);
  r->bh = (uint32_t)(q.h / q.by);
  const uint32_t nb = r->bw * r->bh;
  r->bytes = device_bytes(r->dm, nb);
  lgx::equilibrium_thresholds(q.density, q.ux, q.uy, q.rest_particles != 0, r->thresh);
  if (inject) {
    r->error = "allocation failed (injected)";
    r->bytes = 0;
    return false;
  }
  const size_t total = r->dm.total;
  cudaError_t e = cudaSuccess;
  auto A = [&](void** p, size_t n) {
    if (e == cudaSuccess && n) e = cudaMallocFromPoolAsync(p, n, s->pool, s->stream);
  };
  A((void**)&r->planes[0], total * 7 * 4);
  A((void**)&r->planes[1], total * 7 * 4);
  A((void**)&r->solid, total * 4);
  A((void**)&r->anysolid, ((total + 31) / 32) * 4);
  A((void**)&r->dcells, (size_t)q.w * q.h);
  if (r->dm.iw) A((void**)&r->inlet, (size_t)lgx::kInletChunk * r->dm.h * r->dm.iw * 7 * 4);
  if (nb) A((void**)&r->field, (size_t)nb * 4 * 4);
  if (nb) A((void**)&r->sums, (size_t)nb * 4 * 4);
  A((void**)&r->count, sizeof(unsigned long long));
  s->in_use += r->bytes;
  s->in_use_now = s->in_use;
  if (s->in_use > s->peak_bytes) s->peak_bytes = s->in_use;
  if (e == cudaSuccess && nb) {
    e = cudaMemsetAsync(r->field, 0, (size_t)nb * 16, s->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(r->sums, 0, (size_t)nb * 16, s->stream);
  }
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(r->dcells, r->cells.data(), r->cells.size(), cudaMemcpyHostToDevice,
                        s->stream);
  if (e == cudaSuccess)
    e = lgx::launch_pack(r->dcells, r->dm, r->planes[0], r->solid, r->anysolid, s->stream);
  if (e == cudaSuccess && !r->res_field) {
    e = cudaHostAlloc((void**)&r->res_field, std::max<size_t>(nb, 1) * 16, cudaHostAllocDefault);
    if (e == cudaSuccess)
      e = cudaHostAlloc((void**)&r->res_sums, std::max<size_t>(nb, 1) * 16, cudaHostAllocDefault);
    if (e == cudaSuccess)
      e = cudaHostAlloc((void**)&r->res_count, sizeof(unsigned long long), cudaHostAllocDefault);
  }
  if (e == cudaSuccess && !r->done_ev) e = cudaEventCreateWithFlags(&r->done_ev, cudaEventDisableTiming);
  if (e != cudaSuccess) {
    cudaGetLastError();
    r->error = std::string("admission: ") + cudaGetErrorString(e);
    release_device(s, r);
    return false;
  }
  std::vector<uint8_t>().swap(r->cells);  // the cells now live on the device
  s->launches += 1;
  r->steps_done = 0;
  r->since = 0;
  r->cur = 0;
  r->t_admit = now_s();
  return true;
}

// Enqueue the copies of a finished lattice's moments and free its memory.
void retire(lgx_server* s, Req* r) {
  const uint32_t nb = r->bw * r->bh;
  cudaError_t e = cudaSuccess;
  if (nb) {
    e = cudaMemcpyAsync(r->res_field, r->field, (size_t)nb * 16, cudaMemcpyDeviceToHost,
                        s->stream);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(r->res_sums, r->sums, (size_t)nb * 16, cudaMemcpyDeviceToHost,
                          s->stream);
  }
  if (e == cudaSuccess)
    e = lgx::launch_count(r->planes[r->cur], r->dm, r->count, s->stream);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(r->res_count, r->count, sizeof(unsigned long long),
                        cudaMemcpyDeviceToHost, s->stream);
  if (e == cudaSuccess) e = cudaEventRecord(r->done_ev, s->stream);
  s->launches += 1;
  release_device(s, r);
  if (e != cudaSuccess) {
    r->error = std::string("retire: ") + cudaGetErrorString(e);
    r->state = LGX_REQ_FAILED;
    r->t_done = now_s();
    return;
  }
  s->retiring.push_back(r);
}

// Wait for a ring slot's tick and add its device time to the statistics.
cudaError_t settle(lgx_server* s, lgx_server::Slot& slot) {
  cudaError_t e = cudaEventSynchronize(slot.ev);
  float ms = 0;
  if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, slot.ev0, slot.ev);
  if (e == cudaSuccess) s->gpu_busy_ns += (uint64_t)(ms * 1e6);
  slot.used = false;
  return e;
}

// Sampling points a lattice reaches during a tick of `len` steps: k in
// 1..len with since + k a multiple of its period, and its last step.
template <typename F>
void due_points(const Req* r, uint64_t len, F&& mark) {
  const uint64_t every = r->spec.sample_every;
  if (every == 0) return;
  for (uint64_t k = every - r->since; k <= len; k += every) mark(k);
  const uint64_t left = r->spec.steps - r->steps_done;
  if (left <= len && (r->since + left) % every != 0) mark(left);  // once, if not a multiple
}

// One tick: every active lattice advances `len` steps (fewer if the tick would
// hold more than kMaxSamplePoints sampling points); after each step at which
// some lattices reach a sampling point, one batched coarse-graining of exactly
// those lattices.
cudaError_t tick(lgx_server* s, uint64_t len) {
  auto& slot = s->ring[s->next_slot];
  s->next_slot = (s->next_slot + 1) % kRing;
  if (slot.used) {
    const double t_wait = now_s();
    cudaError_t e = settle(s, slot);
    s->host_wait_ns += (uint64_t)((now_s() - t_wait) * 1e9);
    if (e != cudaSuccess) return e;
  }
  slot.used = true;
  const size_t n = s->active.size();
  // the steps after which someone samples, at most kMaxSamplePoints of them
  std::vector<char> mark(len + 1, 0);
  for (Req* r : s->active) due_points(r, len, [&](uint64_t k) { mark[k] = 1; });
  std::vector<uint32_t> pts;
  for (uint64_t k = 1; k <= len; ++k) {
    if (!mark[k]) continue;
    if (pts.size() == kMaxSamplePoints) {
      len = pts.back();
      break;
    }
    pts.push_back((uint32_t)k);
  }
  // chains: contiguous runs of the active lattices balanced by blocks, run as
  // parallel launch chains on the server's two streams
  const size_t m = pts.size();
  std::vector<uint32_t> words_blocks(n);
  uint64_t total_blocks = 0;
  for (size_t i = 0; i < n; ++i) {
    words_blocks[i] = (s->active[i]->dm.total + 255) / 256;
    total_blocks += words_blocks[i];
  }
  const size_t nch = std::min<size_t>(kChains, n);
  std::vector<size_t> cfirst(nch + 1, n);
  {
    size_t i = 0;
    uint64_t acc = 0;
    for (size_t c = 0; c < nch; ++c) {
      cfirst[c] = i;
      const uint64_t target = total_blocks * (c + 1) / nch;
      // at least one lattice per chain: leave one for each chain after this one
      const size_t stop = n - (nch - 1 - c);
      while (i < stop && (c + 1 == nch || acc < target || i == cfirst[c])) acc += words_blocks[i++];
    }
    cfirst[nch] = n;
  }
  // slot layout: descs[n] | item0[n+1] | per chain c: block0[nc+1] | blk[m][nc+1] |
  // tl[m][nc+1] (per sampling point, the prefixes of field blocks coarse-grained a
  // warp each and of tiles, for the lattices that sample there)
  lgx::LatDesc* descs = (lgx::LatDesc*)slot.host;
  uint32_t* item0 = (uint32_t*)(descs + n);
  std::vector<size_t> off(nch);  // each chain's block0, in words from item0
  size_t words = n + 1;
  for (size_t c = 0; c < nch; ++c) {
    off[c] = words;
    words += (1 + 2 * m) * (cfirst[c + 1] - cfirst[c] + 1);
  }
  const size_t bytes = n * sizeof(lgx::LatDesc) + words * sizeof(uint32_t);
  item0[0] = 0;
  std::vector<uint32_t> nblocks(nch, 0), rest_blocks(nch, 0);
  std::vector<char> wpr4(nch, 1);    // every lattice of the chain: a multiple of 4 words per row
  std::vector<char> inflow(nch, 0);  // some lattice of the chain has an inflow
  for (size_t c = 0; c < nch; ++c) {
    const size_t nc = cfirst[c + 1] - cfirst[c];
    uint32_t* block0 = item0 + off[c];
    uint32_t* blk = block0 + nc + 1;
    uint32_t* tl = blk + m * (nc + 1);
    block0[0] = 0;
    for (size_t j = 0; j < m; ++j) blk[j * (nc + 1)] = tl[j * (nc + 1)] = 0;
    for (size_t q = 0; q < nc; ++q) {
      const size_t i = cfirst[c] + q;
      Req* r = s->active[i];
      lgx::LatDesc& d = descs[i];
      d.planes[0] = r->planes[r->cur];
      d.planes[1] = r->planes[r->cur ^ 1];
      d.solid = r->solid;
      d.anysolid = r->anysolid;
      d.inlet = r->inlet;
      d.dm = r->dm;
      d.seed = r->spec.seed;
      d.steps0 = r->steps_done;
      d.cur0 = 0;
      d.rest = r->spec.rest_particles ? 1u : 0u;
      memcpy(d.thresh, r->thresh, sizeof(d.thresh));
      d.field = r->field;
      d.sums = r->sums;
      d.bx = (uint32_t)r->spec.bx;
      d.by = (uint32_t)r->spec.by;
      d.bw = r->bw;
      d.bh = r->bh;
      d.alpha = r->spec.alpha;
      block0[q + 1] = block0[q] + words_blocks[i];
      if (r->spec.rest_particles) rest_blocks[c] = block0[q + 1];
      if (r->dm.wpr % 4u) wpr4[c] = 0;
      if (r->dm.iw) inflow[c] = 1;
      item0[i + 1] = item0[i] + (uint32_t)len * r->dm.h * r->dm.iw;
      for (size_t j = 0; j < m; ++j) {
        blk[j * (nc + 1) + q + 1] = blk[j * (nc + 1) + q];
        tl[j * (nc + 1) + q + 1] = tl[j * (nc + 1) + q];
      }
      const bool tiled = d.bx >= lgx::kTileMinWidth && r->bw * r->bh > 0;
      uint32_t per = 0, ncx = 0;
      if (tiled) lgx::tile_shape(d.bx, d.bw, &per, &ncx);
      due_points(r, len, [&](uint64_t k) {
        const size_t j = std::lower_bound(pts.begin(), pts.end(), (uint32_t)k) - pts.begin();
        if (tiled)
          tl[j * (nc + 1) + q + 1] = tl[j * (nc + 1) + q] + ncx * r->bh;
        else
          blk[j * (nc + 1) + q + 1] = blk[j * (nc + 1) + q] + r->bw * r->bh;
      });
    }
    nblocks[c] = block0[nc];
  }
  uint8_t* dev = (uint8_t*)slot.dev;
  lgx::LatDesc* d_descs = (lgx::LatDesc*)dev;
  uint32_t* d_item0 = (uint32_t*)(d_descs + n);
  cudaError_t e = cudaEventRecord(slot.ev0, s->stream);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(slot.dev, slot.host, bytes, cudaMemcpyHostToDevice, s->stream);
  if (e == cudaSuccess && total_blocks > slot.owner_cap) {  // grow the block-owner table
    if (slot.owner) e = cudaFreeAsync(slot.owner, s->stream);
    slot.owner = nullptr;
    slot.owner_cap = 0;
    const size_t cap = 2 * (size_t)total_blocks;
    if (e == cudaSuccess)
      e = cudaMallocFromPoolAsync((void**)&slot.owner, cap * 4, s->pool, s->stream);
    if (e == cudaSuccess) slot.owner_cap = cap;
  }
  std::vector<uint32_t*> owner(nch);
  for (size_t c = 0, o = 0; c < nch && e == cudaSuccess; o += nblocks[c], ++c) {
    owner[c] = slot.owner + o;
    e = lgx::launch_batch_owner(d_item0 + off[c], (uint32_t)(cfirst[c + 1] - cfirst[c]),
                                nblocks[c], owner[c], s->stream);
    s->launches += 1;
  }
  if (e == cudaSuccess && item0[n]) {
    lgx::BatchInletArgs ia{d_descs, d_item0, (uint32_t)n, item0[n], s->d_zero};
    e = lgx::launch_batch_inlet(ia, s->stream);
    s->launches += 1;
  }
  if (e == cudaSuccess && nch > 1) {
    e = cudaEventRecord(s->fork, s->stream);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(s->stream2, s->fork, 0);
  }
  for (size_t c = 0; c < nch && e == cudaSuccess; ++c) {
    cudaStream_t st = c == 0 ? s->stream : s->stream2;
    const size_t nc = cfirst[c + 1] - cfirst[c];
    const lgx::LatDesc* dd = d_descs + cfirst[c];
    const uint32_t* d_block0 = d_item0 + off[c];
    const uint32_t* blk = item0 + off[c] + nc + 1;
    const int rule = rest_blocks[c] == nblocks[c] ? lgx::kRuleRest
                     : rest_blocks[c] == 0       ? lgx::kRuleNoRest
                                                 : lgx::kRuleMixed;
    size_t j = 0;
    for (uint32_t k = 0; k < len && e == cudaSuccess; ++k) {
      lgx::BatchStepArgs sa{dd, d_block0, owner[c], (uint32_t)nc, s->d_zero, k, 0};
      e = lgx::launch_batch_step(sa, nblocks[c], rule,
                                 lgx::batch_step_words(nblocks[c], wpr4[c], inflow[c]), st);
      s->launches += 1;
      if (e == cudaSuccess && j < m && pts[j] == k + 1) {
        const uint32_t* tb = blk + j * (nc + 1);
        const uint32_t* tt = tb + m * (nc + 1);
        if (tb[nc] || tt[nc]) {
          const uint32_t* d_tb = d_block0 + nc + 1 + j * (nc + 1);
          lgx::BatchSampleArgs sp{dd, d_tb, (uint32_t)nc, tb[nc], s->d_zero,
                                  k + 1, d_tb + m * (nc + 1), tt[nc]};
          e = lgx::launch_batch_sample(sp, st);
          s->launches += (tb[nc] ? 1 : 0) + (tt[nc] ? 1 : 0);
        }
        ++j;
      }
    }
  }
  if (e == cudaSuccess && nch > 1) {
    e = cudaEventRecord(s->join, s->stream2);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(s->stream, s->join, 0);
  }
  if (e == cudaSuccess) e = cudaEventRecord(slot.ev, s->stream);
  if (e != cudaSuccess) return e;
  s->ticks += 1;
  for (Req* r : s->active) {
    const uint64_t every = r->spec.sample_every;
    r->steps_done += len;
    r->since = every ? (r->since + len) % every : 0;
    r->cur ^= (int)(len & 1u);
    s->site_updates += (uint64_t)r->spec.w * r->spec.h * len;
  }
  return cudaSuccess;
}

void serve(lgx_server* s) {
  cudaSetDevice(s->device);
  std::unique_lock<std::mutex> lk(s->mu);
  while (true) {
    // completions
    for (size_t i = 0; i < s->retiring.size();) {
      Req* r = s->retiring[i];
      if (cudaEventQuery(r->done_ev) == cudaSuccess) {
        r->state = r->cancel ? LGX_REQ_CANCELLED : LGX_REQ_DONE;
        r->t_done = now_s();
        s->retiring.erase(s->retiring.begin() + i);
        s->cv.notify_all();
      } else {
        ++i;
      }
    }
    if (s->stop && s->pending.empty() && s->active.empty() && s->retiring.empty()) break;
    if (s->stop) {
      for (Req* r : s->pending) {
        r->state = LGX_REQ_CANCELLED;
        r->t_done = now_s();
      }
      s->pending.clear();
      for (Req* r : s->active) r->cancel = true;
    }
    // cancellations of running lattices
    for (size_t i = 0; i < s->active.size();) {
      Req* r = s->active[i];
      if (r->cancel) {
        s->active.erase(s->active.begin() + i);
        retire(s, r);
      } else {
        ++i;
      }
    }
    // admission, first fit in arrival order; allocations and copies run
    // outside the lock so submitters are never held up by them
    for (auto it = s->pending.begin(); it != s->pending.end() && s->active.size() < s->max_active;) {
      Req* r = *it;
      const lgx::Dims dm = lgx::make_dims((uint32_t)r->spec.w, (uint32_t)r->spec.h,
                                          (uint32_t)r->spec.inlet_cols);
      const size_t need = device_bytes(dm, (uint32_t)((r->spec.w / r->spec.bx) *
                                                      (r->spec.h / r->spec.by)));
      if (s->in_use + need > s->budget) {
        ++it;
        continue;
      }
      it = s->pending.erase(it);
      const size_t pos = it - s->pending.begin();
      const bool inject = s->fault_alloc > 0;
      if (inject) s->fault_alloc -= 1;
      lk.unlock();
      const bool ok = admit(s, r, inject);
      lk.lock();
      it = s->pending.begin() + std::min(pos, s->pending.size());
      if (ok) {
        r->state = LGX_REQ_RUNNING;
        // rest-particle lattices first: each rule's blocks form one run
        if (r->spec.rest_particles)
          s->active.insert(std::find_if(s->active.begin(), s->active.end(),
                                        [](Req* a) { return !a->spec.rest_particles; }),
                           r);
        else
          s->active.push_back(r);
        if (s->active.size() > s->peak_active) s->peak_active = s->active.size();
      } else {
        r->state = LGX_REQ_FAILED;
        r->t_done = now_s();
        s->cv.notify_all();
      }
    }
    if (s->active.empty()) {
      for (auto& sl : s->ring)  // idle: account the ticks still in the ring
        if (sl.used) settle(s, sl);
      if (s->retiring.empty())
        s->cv.wait_for(lk, std::chrono::milliseconds(2));
      else {
        lk.unlock();
        std::this_thread::sleep_for(std::chrono::microseconds(50));
        lk.lock();
      }
      continue;
    }
    // the tick: up to the nearest end among the residents (sampling points
    // fall inside it)
    uint64_t len = lgx::kInletChunk;
    for (Req* r : s->active) len = std::min<uint64_t>(len, r->spec.steps - r->steps_done);
    lk.unlock();
    const double t_tick = now_s();
    cudaError_t e = tick(s, len);
    s->host_tick_ns += (uint64_t)((now_s() - t_tick) * 1e9);
    lk.lock();
    if (e != cudaSuccess) {
      s->fatal = std::string("serving tick: ") + cudaGetErrorString(e);
      for (Req* r : s->active) {
        release_device(s, r);
        r->state = LGX_REQ_FAILED;
        r->error = s->fatal;
        r->t_done = now_s();
      }
      s->active.clear();
      s->cv.notify_all();
      continue;
    }
    for (size_t i = 0; i < s->active.size();) {
      Req* r = s->active[i];
      if (r->steps_done >= r->spec.steps) {
        s->active.erase(s->active.begin() + i);
        retire(s, r);
      } else {
        ++i;
      }
    }
  }
}

Req* find(lgx_server* s, uint64_t id) {
  auto it = s->reqs.find(id);
  return it == s->reqs.end() ? nullptr : it->second.get();
}

void free_req(Req* r) {
  if (r->res_field) cudaFreeHost(r->res_field);
  if (r->res_sums) cudaFreeHost(r->res_sums);
  if (r->res_count) cudaFreeHost(r->res_count);
  if (r->done_ev) cudaEventDestroy(r->done_ev);
  r->res_field = nullptr;
  r->res_sums = nullptr;
  r->res_count = nullptr;
  r->done_ev = nullptr;
}

}  // namespace

extern "C" {

int lgx_server_create(size_t budget_bytes, size_t max_active, lgx_server** out) {
  if (!out || budget_bytes == 0 || max_active == 0 || max_active > 4096) {
    lgx::set_error("lgx_server_create: need a budget and 1..4096 resident lattices");
    return LGX_ERR_ARG;
  }
  *out = nullptr;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    lgx::set_error("no CUDA device on this machine");
    return LGX_ERR_NO_DEVICE;
  }
  lgx_server* s = new (std::nothrow) lgx_server();
  if (!s) {
    lgx::set_error("out of host memory");
    return LGX_ERR_ALLOC;
  }
  cudaGetDevice(&s->device);
  s->budget = budget_bytes;
  s->max_active = max_active;
  cudaError_t e = cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&s->stream2, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&s->fork, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&s->join, cudaEventDisableTiming);
  if (e == cudaSuccess) {
    cudaMemPoolProps props = {};
    props.allocType = cudaMemAllocationTypePinned;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = s->device;
    e = cudaMemPoolCreate(&s->pool, &props);
  }
  if (e == cudaSuccess) {
    uint64_t keep = UINT64_MAX;  // keep freed memory in the pool between ticks
    e = cudaMemPoolSetAttribute(s->pool, cudaMemPoolAttrReleaseThreshold, &keep);
  }
  s->slot_bytes = max_active * sizeof(lgx::LatDesc) +
                  ((max_active + 1) + (1 + 2 * kMaxSamplePoints) * (max_active + kChains)) *
                      sizeof(uint32_t);
  for (int i = 0; i < kRing && e == cudaSuccess; ++i) {
    e = cudaHostAlloc(&s->ring[i].host, s->slot_bytes, cudaHostAllocDefault);
    if (e == cudaSuccess) e = cudaMalloc(&s->ring[i].dev, s->slot_bytes);
    if (e == cudaSuccess) e = cudaEventCreate(&s->ring[i].ev);
    if (e == cudaSuccess) e = cudaEventCreate(&s->ring[i].ev0);
  }
  if (e == cudaSuccess) e = cudaMalloc(&s->d_zero, sizeof(uint64_t));
  if (e == cudaSuccess) e = cudaMemset(s->d_zero, 0, sizeof(uint64_t));
  if (e != cudaSuccess) {
    lgx::set_error(std::string("lgx_server_create: ") + cudaGetErrorString(e));
    lgx_server_destroy(s);
    return LGX_ERR_CUDA;
  }
  s->thr = std::thread(serve, s);
  *out = s;
  return LGX_OK;
}

int lgx_server_destroy(lgx_server* s) {
  if (!s) return LGX_OK;
  if (s->thr.joinable()) {
    {
      std::lock_guard<std::mutex> g(s->mu);
      s->stop = true;
    }
    s->cv.notify_all();
    s->thr.join();
  }
  cudaSetDevice(s->device);
  if (s->stream) cudaStreamSynchronize(s->stream);
  for (auto& kv : s->reqs) free_req(kv.second.get());
  for (auto& sl : s->ring) {
    if (sl.host) cudaFreeHost(sl.host);
    if (sl.dev) cudaFree(sl.dev);
    if (sl.ev) cudaEventDestroy(sl.ev);
    if (sl.ev0) cudaEventDestroy(sl.ev0);
    if (sl.owner) cudaFree(sl.owner);
  }
  cudaFree(s->d_zero);
  if (s->pool) cudaMemPoolDestroy(s->pool);
  if (s->fork) cudaEventDestroy(s->fork);
  if (s->join) cudaEventDestroy(s->join);
  if (s->stream2) cudaStreamDestroy(s->stream2);
  if (s->stream) cudaStreamDestroy(s->stream);
  delete s;
  return LGX_OK;
}

int lgx_server_submit(lgx_server* s, const lgx_request* q, uint64_t* id) {
  if (!s || !q || !id) {
    lgx::set_error("lgx_server_submit: null argument");
    return LGX_ERR_ARG;
  }
  if (q->h % 2 != 0 || q->w <= 4 || q->h <= 4 || !q->cells || q->bx == 0 || q->by == 0 ||
      q->steps == 0) {
    lgx::set_error("lgx_server_submit: bad lattice (h even, w > 4, h > 4), cells, block or steps");
    return LGX_ERR_ARG;
  }
  const lgx::Dims dm = lgx::make_dims((uint32_t)q->w, (uint32_t)q->h, (uint32_t)q->inlet_cols);
  const size_t need = device_bytes(dm, (uint32_t)((q->w / q->bx) * (q->h / q->by)));
  if (need > s->budget) {
    lgx::set_error("lgx_server_submit: the lattice alone exceeds the device-memory budget");
    return LGX_ERR_BUSY;
  }
  auto r = std::make_unique<Req>();
  r->spec = *q;
  r->spec.cells = nullptr;
  r->cells.assign(q->cells, q->cells + q->w * q->h);
  r->t_submit = now_s();
  std::lock_guard<std::mutex> g(s->mu);
  if (s->stop) {
    lgx::set_error("lgx_server_submit: server is shutting down");
    return LGX_ERR_STATE;
  }
  r->id = s->next_id++;
  *id = r->id;
  s->pending.push_back(r.get());
  s->reqs[r->id] = std::move(r);
  s->cv.notify_all();
  return LGX_OK;
}

int lgx_server_poll(lgx_server* s, uint64_t id, int* state) {
  if (!s || !state) {
    lgx::set_error("null argument");
    return LGX_ERR_ARG;
  }
  std::lock_guard<std::mutex> g(s->mu);
  Req* r = find(s, id);
  if (!r) {
    lgx::set_error("unknown request");
    return LGX_ERR_ARG;
  }
  *state = r->state;
  return LGX_OK;
}

int lgx_server_wait(lgx_server* s, uint64_t id, double timeout_s, int* state) {
  if (!s) {
    lgx::set_error("null server");
    return LGX_ERR_ARG;
  }
  std::unique_lock<std::mutex> lk(s->mu);
  Req* r = find(s, id);
  if (!r) {
    lgx::set_error("unknown request");
    return LGX_ERR_ARG;
  }
  const auto deadline = std::chrono::steady_clock::now() +
                        std::chrono::duration<double>(timeout_s < 0 ? 1e9 : timeout_s);
  while (r->state == LGX_REQ_QUEUED || r->state == LGX_REQ_RUNNING) {
    if (s->cv.wait_until(lk, deadline) == std::cv_status::timeout) break;
  }
  if (state) *state = r->state;
  if (r->state == LGX_REQ_QUEUED || r->state == LGX_REQ_RUNNING) {
    lgx::set_error("lgx_server_wait: timed out");
    return LGX_ERR_BUSY;
  }
  return LGX_OK;
}

int lgx_server_result(lgx_server* s, uint64_t id, float* ux, float* uy, float* rho, float* sol,
                      int32_t* mass, int32_t* px2, int32_t* py2, int32_t* nsolid, size_t n_blocks,
                      uint64_t* particles, double* latency_s) {
  if (!s) {
    lgx::set_error("null server");
    return LGX_ERR_ARG;
  }
  std::lock_guard<std::mutex> g(s->mu);
  Req* r = find(s, id);
  if (!r) {
    lgx::set_error("unknown request");
    return LGX_ERR_ARG;
  }
  if (r->state != LGX_REQ_DONE) {
    lgx::set_error(r->state == LGX_REQ_FAILED ? "request failed: " + r->error
                                              : std::string("request has no result"));
    return LGX_ERR_STATE;
  }
  const size_t nb = (size_t)r->bw * r->bh;
  if (n_blocks != nb) {
    lgx::set_error("block grid mismatch");
    return LGX_ERR_ARG;
  }
  float* f[4] = {ux, uy, rho, sol};
  for (int i = 0; i < 4; ++i)
    if (f[i] && nb) memcpy(f[i], r->res_field + i * nb, nb * 4);
  int32_t* m[4] = {mass, px2, py2, nsolid};
  for (int i = 0; i < 4; ++i)
    if (m[i] && nb) memcpy(m[i], r->res_sums + i * nb, nb * 4);
  if (particles) *particles = *r->res_count;
  if (latency_s) *latency_s = r->t_done - r->t_submit;
  return LGX_OK;
}

int lgx_server_cancel(lgx_server* s, uint64_t id) {
  if (!s) {
    lgx::set_error("null server");
    return LGX_ERR_ARG;
  }
  std::lock_guard<std::mutex> g(s->mu);
  Req* r = find(s, id);
  if (!r) {
    lgx::set_error("unknown request");
    return LGX_ERR_ARG;
  }
  if (r->state == LGX_REQ_QUEUED) {
    s->pending.erase(std::remove(s->pending.begin(), s->pending.end(), r), s->pending.end());
    r->state = LGX_REQ_CANCELLED;
    r->t_done = now_s();
    s->cv.notify_all();
  } else if (r->state == LGX_REQ_RUNNING) {
    r->cancel = true;
  }
  return LGX_OK;
}

int lgx_server_release(lgx_server* s, uint64_t id) {
  if (!s) {
    lgx::set_error("null server");
    return LGX_ERR_ARG;
  }
  std::unique_ptr<Req> keep;
  {
    std::lock_guard<std::mutex> g(s->mu);
    auto it = s->reqs.find(id);
    if (it == s->reqs.end()) {
      lgx::set_error("unknown request");
      return LGX_ERR_ARG;
    }
    Req* r = it->second.get();
    if (r->state == LGX_REQ_QUEUED || r->state == LGX_REQ_RUNNING ||
        std::find(s->retiring.begin(), s->retiring.end(), r) != s->retiring.end()) {
      lgx::set_error("lgx_server_release: request still in flight");
      return LGX_ERR_STATE;
    }
    keep = std::move(it->second);
    s->reqs.erase(it);
  }
  free_req(keep.get());
  return LGX_OK;
}

int lgx_server_get_stats(lgx_server* s, lgx_server_stats* out) {
  if (!s || !out) {
    lgx::set_error("null argument");
    return LGX_ERR_ARG;
  }
  std::lock_guard<std::mutex> g(s->mu);
  memset(out, 0, sizeof(*out));
  out->ticks = s->ticks;
  out->kernel_launches = s->launches;
  out->site_updates = s->site_updates;
  out->bytes_in_use = s->in_use_now;
  out->peak_bytes = s->peak_bytes;
  out->peak_active = s->peak_active;
  out->gpu_busy_ns = s->gpu_busy_ns;
  out->host_tick_ns = s->host_tick_ns;
  out->host_wait_ns = s->host_wait_ns;
  out->active = s->active.size();
  out->queued = s->pending.size();
  for (auto& kv : s->reqs) {
    const Req* r = kv.second.get();
    if (r->state == LGX_REQ_DONE) out->completed += 1;
    if (r->state == LGX_REQ_FAILED) out->failed += 1;
    if (r->state == LGX_REQ_CANCELLED) out->cancelled += 1;
  }
  return LGX_OK;
}

int lgx_request_device_bytes(const lgx_request* q, size_t* out) {
  if (!q || !out || q->bx == 0 || q->by == 0 || q->w == 0 || q->h == 0) {
    lgx::set_error("lgx_request_device_bytes: bad request");
    return LGX_ERR_ARG;
  }
  const lgx::Dims dm = lgx::make_dims((uint32_t)q->w, (uint32_t)q->h, (uint32_t)q->inlet_cols);
  *out = device_bytes(dm, (uint32_t)((q->w / q->bx) * (q->h / q->by)));
  return LGX_OK;
}

int lgx_server_inject_alloc_failure(lgx_server* s, int count) {
  if (!s || count < 0) {
    lgx::set_error("bad argument");
    return LGX_ERR_ARG;
  }
  std::lock_guard<std::mutex> g(s->mu);
  s->fault_alloc = count;
  return LGX_OK;
}

}  // extern "C"
