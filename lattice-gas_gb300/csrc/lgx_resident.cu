// lgx_resident.cu -- many steps of small lattices in one launch, the state in
// the shared memory of a thread-block cluster.
//
// A lattice of a few thousand words is too small to fill the GPU for one step,
// so stepping it one launch per step costs a launch's latency per step however
// little work the step is.  Here one cluster of C CTAs owns one lattice for a
// whole interval.  CTA r holds rows [r h / C, (r + 1) h / C) of both ping-pong
// buffers in its shared memory ([2][7][ceil(h / C)][wpr] words); a step reads
// its own rows there and the one row above and below its band from the
// neighbouring CTAs' shared memory (distributed shared memory, through
// addresses from map_shared_rank), writes its rows of the other buffer, and
// meets the others at a cluster barrier (arrive.release / wait.acquire; the
// next step's draws are made between arrive and wait).  The planes are read
// from global memory once at the start and written back once at the end, and
// at each sampling point, where the cluster coarse-grains from global memory
// after writing its rows there.
//
// Clusters never wait on one another, so any number of lattices can share the
// launch; clusters the GPU cannot hold at once run when others finish.
#include <cooperative_groups.h>

#include <stdlib.h>

#include <mutex>

#include "lgx_batch.hpp"
#include "lgx_step_impl.cuh"

namespace cg = cooperative_groups;

namespace lgx {
namespace {

__device__ __forceinline__ uint32_t band_start(uint32_t r, uint32_t h, uint32_t c) {
  return (uint32_t)(((uint64_t)r * h) / c);
}

template <int THREADS>
__global__ void __launch_bounds__(THREADS) lgx_resident_kernel(const ResidentArgs p) {
  extern __shared__ uint32_t shm[];
  const cg::cluster_group cluster = cg::this_cluster();
  const uint32_t C = cluster.num_blocks(), rank = cluster.block_rank();
  const uint32_t li = p.first_lat + blockIdx.x / C;
  const LatDesc& d = p.descs[li];
  const ResSched sch = p.sched[li];
  const Dims dm = d.dm;  // in registers, not read through d at every use
  const size_t S = dm.total;
  const uint32_t y0 = band_start(rank, dm.h, C), y1 = band_start(rank + 1u, dm.h, C);
  const uint32_t cap = (dm.h + C - 1u) / C;      // rows of the largest band
  const size_t lps = (size_t)cap * dm.wpr;       // local plane stride
  const size_t lbs = 7 * lps;                    // local buffer stride
  const uint32_t nw = (y1 - y0) * dm.wpr;        // words of this band
  const uint64_t base = p.base ? *p.base : 0ull;
  const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5, nwarps = THREADS / 32;
  const uint32_t nb = d.bw * d.bh;

  // this band of the state the interval starts from, into buffer 0
  {
    const uint32_t* g = ((d.cur0 + (uint32_t)base) & 1u) ? d.planes[1] : d.planes[0];
    for (uint32_t i = threadIdx.x; i < nw; i += THREADS)
#pragma unroll
      for (int q = 0; q < 7; ++q) shm[q * lps + i] = __ldcg(g + q * S + (size_t)y0 * dm.wpr + i);
  }
  // Write band buffer `buf` to the global planes of parity `par`.
  auto store_band = [&](uint32_t buf, uint32_t par) {
    uint32_t* g = par ? d.planes[1] : d.planes[0];
    for (uint32_t i = threadIdx.x; i < nw; i += THREADS)
#pragma unroll
      for (int q = 0; q < 7; ++q) g[q * S + (size_t)y0 * dm.wpr + i] = shm[buf * lbs + q * lps + i];
  };
  cluster.sync();  // every band is loaded before a neighbour reads it

  // Word c * 32 + lane of the band; lanes past its end repeat its last word.
  const uint32_t nch = (nw + 31u) >> 5;
  auto word_of = [&](uint32_t c, uint32_t* lw, bool* live) {
    *lw = c * 32u + lane;
    *live = *lw < nw;
    if (!*live) *lw = nw - 1u;
  };
  auto div_wpr = [&](uint32_t x) {  // x / wpr by the lattice's multiply-shift
    const uint32_t t = __umulhi(x, dm.div_m);
    return (t + ((x - t) >> dm.div_s1)) >> dm.div_s2;
  };
  auto global_word = [&](uint32_t lw) {
    const uint32_t yr = div_wpr(lw);
    return (y0 + yr) * dm.wpr + (lw - yr * dm.wpr);
  };
  // The rows next to the band belong to the neighbouring CTAs (every band has
  // at least two rows): the row above the band is the last row of rank - 1's,
  // the row below is the first of rank + 1's.
  const uint32_t up = (rank + C - 1u) % C, down = (rank + 1u) % C;
  const uint32_t ya = (y0 == 0u) ? dm.h - 1u : y0 - 1u;  // the row above the band
  const uint32_t up_last = ya - band_start(up, dm.h, C);
  uint32_t* up_base = cluster.map_shared_rank(shm, up) + (size_t)up_last * dm.wpr;
  uint32_t* down_base = cluster.map_shared_rank(shm, down);
  // The draws of a warp's first chunk for step k are made while the cluster
  // barrier of step k - 1 is pending: they depend on (word, step) only.
  uint32_t lw0;
  bool live0;
  word_of(min(warp, nch - 1u), &lw0, &live0);
  const uint32_t g0 = global_word(lw0);
  Draws first = draws(g0 ^ step_seed32(d.seed, d.steps0 + base));

  for (uint32_t k = 0; k < p.len; ++k) {
    const uint64_t local = base + k;
    const uint32_t sb = k & 1u, db = sb ^ 1u;
    const uint32_t seed32 = step_seed32(d.seed, d.steps0 + local);
    const uint32_t* inlet = dm.iw ? d.inlet + (size_t)k * dm.h * dm.iw * 7u : nullptr;
    // plane q of row yy (in the band or next to it) of the source buffer
    auto row = [&](uint32_t q, uint32_t yy) -> const uint32_t* {
      const size_t off = sb * lbs + q * lps;
      if (yy - y0 < y1 - y0) return shm + off + (size_t)(yy - y0) * dm.wpr;
      return (yy == ya ? up_base : down_base) + off;
    };
    // one CTA holds the whole lattice: every row is in this CTA's shared
    // memory, addressed from `shm` so that the loads compile to shared loads
    auto own = [&](uint32_t q, uint32_t yy) -> const uint32_t* {
      return shm + sb * lbs + q * lps + (size_t)yy * dm.wpr;
    };
    auto step_chunks = [&](auto&& rowf) {
      for (uint32_t c = warp; c < nch; c += nwarps) {
        uint32_t lw;
        bool live;
        word_of(c, &lw, &live);
        const uint32_t yr = div_wpr(lw), j = lw - yr * dm.wpr, y = y0 + yr;
        const uint32_t g = y * dm.wpr + j;
        const uint32_t ym = (y == 0u) ? dm.h - 1u : y - 1u;
        const uint32_t yp = (y + 1u == dm.h) ? 0u : y + 1u;
        const uint32_t* rows[7] = {rowf(0, y),  rowf(1, ym), rowf(2, ym), rowf(3, y),
                                   rowf(4, yp), rowf(5, yp), rowf(6, y)};
        uint32_t* out = shm + db * lbs + (size_t)yr * dm.wpr + j;
        const Draws s = c == warp ? first : draws(g ^ seed32);
        if (d.rest)
          step_core<true, LD_GENERIC>(rows, out, lps, d.solid, d.anysolid, inlet, dm, s, g, y,
                                      j, live);
        else
          step_core<false, LD_GENERIC>(rows, out, lps, d.solid, d.anysolid, inlet, dm, s, g, y,
                                       j, live);
      }
    };
    if (C == 1u)
      step_chunks(own);
    else
      step_chunks(row);
    if (C == 1u) {
      // the whole lattice in this CTA: a block barrier orders its shared memory
      __syncthreads();
      if (k + 1u < p.len) first = draws(g0 ^ step_seed32(d.seed, d.steps0 + local + 1u));
    } else {
      // arrive (shared-memory stores released at cluster scope), draw ahead, wait
      asm volatile("barrier.cluster.arrive.release.aligned;" ::: "memory");
      if (k + 1u < p.len) first = draws(g0 ^ step_seed32(d.seed, d.steps0 + local + 1u));
      asm volatile("barrier.cluster.wait.acquire.aligned;" ::: "memory");
    }
    // sampling point after step k + 1 of this launch: from global memory
    const uint32_t t = k + 1u;
    const bool due = nb && sch.every && ((sch.since + t) % sch.every == 0u || t == sch.left);
    if (due) {
      const uint32_t par = (d.cur0 + (uint32_t)(local + 1u)) & 1u;
      store_band(db, par);
      if (C == 1u)
        __syncthreads();
      else
        cluster.sync();
      SampleArgs sa;
      sa.a = par ? d.planes[1] : d.planes[0];
      sa.solid = d.solid;
      sa.dm = dm;
      sa.bx = d.bx;
      sa.by = d.by;
      sa.bw = d.bw;
      sa.bh = d.bh;
      sa.alpha = d.alpha;
      sa.ux = d.field;
      sa.uy = d.field + nb;
      sa.rho = d.field + 2 * nb;
      sa.sol = d.field + 3 * nb;
      sa.sums = d.sums;
      for (uint32_t b = rank * nwarps + warp; b < nb; b += C * nwarps) sample_block(sa, b);
    }
  }
  // the state after the interval, to the planes the next launch reads
  store_band(p.len & 1u, (d.cur0 + (uint32_t)(base + p.len)) & 1u);
}

// Up to K = p.ksteps steps between cluster barriers (clusters of C > 1 CTAs).
// CTA r keeps, for each of the two buffers, local rows 0 .. nb + 2K - 1 of its
// band [y0, y1) widened by K rows either side (local row i is lattice row
// y0 - K + i, periodic in y).  A super-step of k <= K steps (cut at sampling
// points and at the end of the launch) begins with a cluster barrier (every
// band of the current buffer is complete), copies the k rows above and below
// the band from the neighbouring CTAs' bands (distributed shared memory), and
// arrives at a second barrier phase: the neighbours may overwrite their
// current buffer from their second step on, so the CTA waits on that phase
// after its first step.  Step s of the super-step computes local rows
// K - k + s .. K + nb + k - s - 1 (one row fewer on each side per step) from
// the other buffer, with block barriers between steps, so after k steps the
// band is exact.  Every word's update is the same step_core as everywhere,
// keyed on the lattice word, so results are bit-identical to single steps.
template <int THREADS>
__global__ void __launch_bounds__(THREADS) lgx_resident_multi_kernel(const ResidentArgs p) {
  extern __shared__ uint32_t shm[];
  const cg::cluster_group cluster = cg::this_cluster();
  const uint32_t C = cluster.num_blocks(), rank = cluster.block_rank();
  const uint32_t li = p.first_lat + blockIdx.x / C;
  const LatDesc& d = p.descs[li];
  const ResSched sch = p.sched[li];
  const Dims dm = d.dm;  // in registers, not read through d at every use
  const size_t S = dm.total;
  const uint32_t K = p.ksteps;
  const uint32_t y0 = band_start(rank, dm.h, C), y1 = band_start(rank + 1u, dm.h, C);
  const uint32_t nb = y1 - y0;                    // rows of this band (>= K)
  const uint32_t cap = (dm.h + C - 1u) / C;       // rows of the largest band
  const size_t lps = (size_t)(cap + 2u * K) * dm.wpr;  // local plane stride
  const size_t lbs = 7 * lps;                     // local buffer stride
  const uint64_t base = p.base ? *p.base : 0ull;
  const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5, nwarps = THREADS / 32;
  const uint32_t nbf = d.bw * d.bh;
  const uint32_t bandw = nb * dm.wpr;             // words of the band

  // the band of the state the interval starts from, into local rows K.. of buffer 0
  {
    const uint32_t* g = ((d.cur0 + (uint32_t)base) & 1u) ? d.planes[1] : d.planes[0];
    for (uint32_t i = threadIdx.x; i < bandw; i += THREADS)
#pragma unroll
      for (int q = 0; q < 7; ++q)
        shm[q * lps + (size_t)K * dm.wpr + i] = __ldcg(g + q * S + (size_t)y0 * dm.wpr + i);
  }
  auto store_band = [&](uint32_t buf, uint32_t par) {
    uint32_t* g = par ? d.planes[1] : d.planes[0];
    for (uint32_t i = threadIdx.x; i < bandw; i += THREADS)
#pragma unroll
      for (int q = 0; q < 7; ++q)
        g[q * S + (size_t)y0 * dm.wpr + i] = shm[buf * lbs + q * lps + (size_t)K * dm.wpr + i];
  };
  // The K rows above the band are the last K of rank - 1's band (local rows
  // nb_up .. nb_up + K - 1 there), the K below the first K of rank + 1's (local
  // rows K .. 2K - 1); every band has at least K rows.
  const uint32_t up = (rank + C - 1u) % C, down = (rank + 1u) % C;
  const uint32_t nb_up = band_start(up + 1u, dm.h, C) - band_start(up, dm.h, C);
  const uint32_t* up_shm = cluster.map_shared_rank(shm, up);
  const uint32_t* down_shm = cluster.map_shared_rank(shm, down);
  auto div_wpr = [&](uint32_t x) {  // x / wpr by the lattice's multiply-shift
    const uint32_t t = __umulhi(x, dm.div_m);
    return (t + ((x - t) >> dm.div_s1)) >> dm.div_s2;
  };

  uint32_t cur = 0;  // the buffer holding the state after step t
  for (uint32_t t = 0; t < p.len;) {
    // this super-step: up to K steps, ending at the next sampling point
    uint32_t k = min(K, p.len - t);
    if (nbf && sch.every)
      for (uint32_t s = 1; s < k; ++s)
        if ((sch.since + t + s) % sch.every == 0u || t + s == sch.left) {
          k = s;
          break;
        }
    // (1) every band of buffer `cur` is complete (and loaded, before the first)
    asm volatile("barrier.cluster.arrive.release.aligned;" ::: "memory");
    asm volatile("barrier.cluster.wait.acquire.aligned;" ::: "memory");
    // the k rows on either side of the band, from the neighbours' bands
    {
      const uint32_t hw = k * dm.wpr;  // words per plane and side
      for (uint32_t i = threadIdx.x; i < 7u * hw; i += THREADS) {
        const uint32_t q = i / hw, w = i - q * hw;
        const size_t off = cur * lbs + q * lps;
        shm[off + (size_t)(K - k) * dm.wpr + w] = up_shm[off + (size_t)(K + nb_up - k) * dm.wpr + w];
        shm[off + (size_t)(K + nb) * dm.wpr + w] = down_shm[off + (size_t)K * dm.wpr + w];
      }
    }
    // (2) done reading the neighbours' buffer `cur`: they may overwrite it
    // from their second step on, after waiting for this phase
    asm volatile("barrier.cluster.arrive.release.aligned;" ::: "memory");
    __syncthreads();  // the halo rows are in place for every warp
    for (uint32_t s = 1; s <= k; ++s) {
      const uint64_t local = base + t + s - 1u;
      const uint32_t seed32 = step_seed32(d.seed, d.steps0 + local);
      const uint32_t* inlet = dm.iw ? d.inlet + (size_t)(t + s - 1u) * dm.h * dm.iw * 7u : nullptr;
      const uint32_t r0 = K - k + s;                          // first local row
      const uint32_t nw = (nb + 2u * (k - s)) * dm.wpr;       // words this step
      const uint32_t nch = (nw + 31u) >> 5;
      const uint32_t sb = cur, db = cur ^ 1u;
      for (uint32_t c = warp; c < nch; c += nwarps) {
        uint32_t lw = c * 32u + lane;
        const bool live = lw < nw;
        if (!live) lw = nw - 1u;
        const uint32_t rr = div_wpr(lw), j = lw - rr * dm.wpr;
        const uint32_t r = r0 + rr;                           // local row
        uint32_t y = y0 + dm.h - K + r;                       // lattice row
        if (y >= dm.h) y -= dm.h;
        if (y >= dm.h) y -= dm.h;
        const uint32_t g = y * dm.wpr + j;
        const uint32_t* src = shm + sb * lbs;
        const uint32_t* rows[7] = {src + 0 * lps + (size_t)r * dm.wpr,
                                   src + 1 * lps + (size_t)(r - 1u) * dm.wpr,
                                   src + 2 * lps + (size_t)(r - 1u) * dm.wpr,
                                   src + 3 * lps + (size_t)r * dm.wpr,
                                   src + 4 * lps + (size_t)(r + 1u) * dm.wpr,
                                   src + 5 * lps + (size_t)(r + 1u) * dm.wpr,
                                   src + 6 * lps + (size_t)r * dm.wpr};
        uint32_t* out = shm + db * lbs + (size_t)r * dm.wpr + j;
        const Draws dr = draws(g ^ seed32);
        if (d.rest)
          step_core<true, LD_GENERIC>(rows, out, lps, d.solid, d.anysolid, inlet, dm, dr, g, y,
                                      j, live);
        else
          step_core<false, LD_GENERIC>(rows, out, lps, d.solid, d.anysolid, inlet, dm, dr, g, y,
                                       j, live);
      }
      cur ^= 1u;
      __syncthreads();
      if (s == 1u) asm volatile("barrier.cluster.wait.acquire.aligned;" ::: "memory");
    }
    t += k;
    // sampling point after step t of this launch: from global memory
    const bool due = nbf && sch.every && ((sch.since + t) % sch.every == 0u || t == sch.left);
    if (due) {
      const uint32_t par = (d.cur0 + (uint32_t)(base + t)) & 1u;
      store_band(cur, par);
      cluster.sync();
      SampleArgs sa;
      sa.a = par ? d.planes[1] : d.planes[0];
      sa.solid = d.solid;
      sa.dm = dm;
      sa.bx = d.bx;
      sa.by = d.by;
      sa.bw = d.bw;
      sa.bh = d.bh;
      sa.alpha = d.alpha;
      sa.ux = d.field;
      sa.uy = d.field + nbf;
      sa.rho = d.field + 2 * nbf;
      sa.sol = d.field + 3 * nbf;
      sa.sums = d.sums;
      for (uint32_t b = rank * nwarps + warp; b < nbf; b += C * nwarps) sample_block(sa, b);
    }
  }
  // the state after the interval, to the planes the next launch reads
  store_band(cur, (d.cur0 + (uint32_t)(base + p.len)) & 1u);
}

// The kernel attributes a launch needs (16-CTA clusters are an opt-in; dynamic
// shared memory above 48 KB too), set once per device and kernel: setting them
// costs host time on every launch otherwise.
template <int THREADS, bool MULTI>
cudaError_t ensure_attributes(size_t smem) {
  constexpr int kMaxDev = 64;
  static std::mutex mu;
  static size_t smem_set[kMaxDev] = {};
  static bool wide_set[kMaxDev] = {};
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess || dev < 0 || dev >= kMaxDev) return e != cudaSuccess ? e : cudaErrorInvalidDevice;
  const void* fn = MULTI ? (const void*)lgx_resident_multi_kernel<THREADS>
                         : (const void*)lgx_resident_kernel<THREADS>;
  std::lock_guard<std::mutex> g(mu);
  if (!wide_set[dev]) {
    e = cudaFuncSetAttribute(fn, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
    if (e != cudaSuccess) return e;
    wide_set[dev] = true;
  }
  if (smem > smem_set[dev]) {
    e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)kResidentMaxSmem);
    if (e != cudaSuccess) return e;
    smem_set[dev] = kResidentMaxSmem;
  }
  return cudaSuccess;
}

template <int THREADS>
cudaError_t launch_resident_t(const ResidentArgs& a, uint32_t nlat, uint32_t csize,
                              size_t smem, cudaStream_t st) {
  const bool multi = a.ksteps > 1u && csize > 1u;
  cudaError_t e = multi ? ensure_attributes<THREADS, true>(smem)
                        : ensure_attributes<THREADS, false>(smem);
  if (e != cudaSuccess) return e;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(nlat * csize);
  cfg.blockDim = dim3(THREADS);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = csize;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  if (multi) return cudaLaunchKernelEx(&cfg, lgx_resident_multi_kernel<THREADS>, a);
  return cudaLaunchKernelEx(&cfg, lgx_resident_kernel<THREADS>, a);
}

}  // namespace

bool resident_config_valid(uint32_t csize, uint32_t threads) {
  return (csize == 1 || csize == 2 || csize == 4 || csize == 8 || csize == 16) &&
         (threads == 128 || threads == 256 || threads == 512 || threads == 1024);
}

size_t resident_smem_bytes(const Dims& dm, uint32_t csize, uint32_t ksteps) {
  const size_t cap = (dm.h + csize - 1) / csize;
  const size_t halo = (ksteps > 1 && csize > 1) ? 2 * (size_t)ksteps : 0;
  return 2 * 7 * (cap + halo) * dm.wpr * sizeof(uint32_t);
}

bool resident_fits(const Dims& dm, uint32_t csize, uint32_t ksteps) {
  if (dm.h < 2 * csize || resident_smem_bytes(dm, csize, ksteps) > kResidentMaxSmem) return false;
  return ksteps <= 1 || csize == 1 || dm.h / csize >= ksteps;  // the smallest band
}

// LGX_RESIDENT_FIXED=0 keeps every launch on the kernels of this file, so that
// tests and measurements can compare them with the fixed-word kernels.
int resident_fixed_mode() {
  static const int mode = [] {
    const char* v = getenv("LGX_RESIDENT_FIXED");
    return v && v[0] == '0' ? 0 : v && v[0] == '2' ? 2 : 1;
  }();
  return mode;
}
static bool fixed_kernels_enabled() { return resident_fixed_mode() != 0; }

bool resident_runs_fixed(uint32_t fixed_threads, uint32_t csize, uint32_t threads,
                         uint32_t ksteps) {
  return fixed_kernels_enabled() && resident_fixed_usable(fixed_threads, threads) &&
         (csize == 1u || ksteps > 1u);
}

cudaError_t launch_resident(const ResidentArgs& a, uint32_t nlat, uint32_t csize,
                            uint32_t threads, size_t smem, uint32_t fixed_threads,
                            cudaStream_t st) {
  if (nlat == 0 || a.len == 0) return cudaSuccess;
  if (resident_runs_fixed(fixed_threads, csize, threads, a.ksteps))
    return launch_resident_fixed(a, nlat, csize, threads, st);
  if (!resident_config_valid(csize, threads) || smem > kResidentMaxSmem)
    return cudaErrorInvalidValue;
  switch (threads) {
    case 128: return launch_resident_t<128>(a, nlat, csize, smem, st);
    case 256: return launch_resident_t<256>(a, nlat, csize, smem, st);
    case 512: return launch_resident_t<512>(a, nlat, csize, smem, st);
    default: return launch_resident_t<1024>(a, nlat, csize, smem, st);
  }
}

}  // namespace lgx
