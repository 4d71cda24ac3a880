// lgx_resident_fixed.cu -- the resident kernels for lattices whose band gives
// every thread of a CTA at most one word.
//
// Small lattices are latency-bound: a step is one warp's chain of dependent
// instructions through one word's update, and the cluster barrier between steps.
// Here each thread owns the same word of its CTA's band for the whole launch,
// so the update's step-invariant part is computed once per launch: the shared
// memory addresses of the thirteen words it gathers (the seven planes of its
// word and the six neighbouring words the shifts bring bits in from), the
// edge-of-row shifts and masks, the obstacle word and the inflow mask.  A step
// is then thirteen shared loads, a gather without branches (a word's row parity
// only selects shift amounts), the collision, and seven shared stores; and the
// draws of the next step are made inside the step, where the scheduler can
// interleave their hash chain with the collision.
//
// The state lives in a fixed layout: buffer b, plane q, local row r, column c
// at word b * 7 * kFxPlaneWords + q * kFxPlaneWords + r * wpr + c, so every
// plane and buffer offset is an immediate of the load and store instructions.
// Two kernels:
//  * one CTA per lattice (clusters of one): the whole lattice in the CTA, a
//    block barrier per step;
//  * clusters of 2-16 CTAs with K >= 2 steps per cluster barrier: CTA r keeps
//    its band with K halo rows either side (local row i is lattice row
//    y0 - K + i), copies the k <= K rows next to its band from the neighbouring
//    CTAs at the start of a super-step of k steps and recomputes the halo rows,
//    one fewer on each side per step (the same schedule and barriers as
//    lgx_resident_multi_kernel).
// Every word's update keys its draws on the lattice word and step and reads the
// same neighbours as the single-step kernel, so results are bit-identical.
#include <cooperative_groups.h>

#include <mutex>

#include "lgx_batch.hpp"
#include "lgx_step_impl.cuh"

namespace cg = cooperative_groups;

namespace lgx {
namespace {

constexpr uint32_t kFxPlaneWords = 1024;
constexpr uint32_t kFxPlaneBytes = kFxPlaneWords * 4u;
constexpr uint32_t kFxBufWords = 7u * kFxPlaneWords;
constexpr uint32_t kFxBufBytes = kFxBufWords * 4u;
constexpr uint32_t kFxSmemBytes = 2u * kFxBufBytes;  // 56 KB

__device__ __forceinline__ uint32_t fx_band_start(uint32_t r, uint32_t h, uint32_t c) {
  return (uint32_t)(((uint64_t)r * h) / c);
}

template <uint32_t OFF>
__device__ __forceinline__ uint32_t lds(uint32_t a) {
  uint32_t v;
  asm volatile("ld.shared.u32 %0, [%1+%2];" : "=r"(v) : "r"(a), "n"(OFF) : "memory");
  return v;
}
template <uint32_t OFF>
__device__ __forceinline__ void sts(uint32_t a, uint32_t v) {
  asm volatile("st.shared.u32 [%0+%1], %2;" ::"r"(a), "n"(OFF), "r"(v) : "memory");
}

// The step-invariant part of one thread's word update.
struct FixedWord {
  uint32_t c_y, c_ym, c_yp;  // shared addresses (buffer 0, plane 0) of column j of
  uint32_t l_y, l_ym, l_yp;  // the word's row and the rows above and below; of the
  uint32_t r_y, r_ym, r_yp;  // column to its left (jl) and to its right (jr)
  uint32_t g;                // lattice word: the draws' key, the obstacle and inflow words
  uint32_t shl;              // the left word's shift: 31 - lastbit at j == 0, else 0
  uint32_t fix;              // bit lastbit on a row's last word when lastbit < 31, else 0
  uint32_t sh_even, sh_odd, fix_odd;  // shifts of planes 1, 5 (even rows) and 2, 4 (odd)
  uint32_t sm;               // obstacle word
  uint32_t apply;            // inflow re-seed mask (0 off the inflow)
  uint32_t tail;             // valid bits (all ones off a row's last word)
  uint32_t boff;             // the word's draws within one step's [h][iw][7] inflow block
};

// Word j of local row r (lattice row y), its gather rows local rm (above) and
// rp (below), in a band whose buffer 0 begins at shared address `sbase`.
__device__ __forceinline__ FixedWord fixed_word(uint32_t sbase, const Dims& dm, uint32_t r,
                                                uint32_t rm, uint32_t rp, uint32_t y,
                                                uint32_t j, bool live,
                                                const uint32_t* __restrict__ solid) {
  FixedWord f;
  const uint32_t jl = j ? j - 1u : dm.lastword;
  const uint32_t jr = j + 1u < dm.wpr ? j + 1u : 0u;
  auto at = [&](uint32_t row, uint32_t col) { return sbase + (row * dm.wpr + col) * 4u; };
  f.c_y = at(r, j), f.c_ym = at(rm, j), f.c_yp = at(rp, j);
  f.l_y = at(r, jl), f.l_ym = at(rm, jl), f.l_yp = at(rp, jl);
  f.r_y = at(r, jr), f.r_ym = at(rm, jr), f.r_yp = at(rp, jr);
  f.g = y * dm.wpr + j;
  f.shl = j ? 0u : 31u - dm.lastbit;
  f.fix = (j == dm.lastword && dm.lastbit != 31u) ? 1u << dm.lastbit : 0u;
  const bool odd = y & 1u;
  f.sh_even = odd ? 0u : 1u;
  f.sh_odd = odd ? 1u : 0u;
  f.fix_odd = odd ? f.fix : 0u;
  f.sm = live ? __ldg(solid + f.g) : 0u;
  f.apply = 0u;
  f.boff = 0u;
  if (j < dm.iw) {
    const uint32_t span = min(dm.inlet_cols - j * 32u, 32u);
    const uint32_t imask = (span >= 32u) ? 0xffffffffu : ((1u << span) - 1u);
    f.apply = imask & ~f.sm;
    f.boff = (y * dm.iw + j) * 7u;
  }
  f.tail = j == dm.lastword ? dm.tail : 0xffffffffu;
  return f;
}

// v with bit `fix` (one bit or none) replaced by bit 0 of hi.
__device__ __forceinline__ uint32_t put_bit(uint32_t v, uint32_t hi, uint32_t fix) {
  return (v & ~fix) | (fix & (0u - (hi & 1u)));
}

// One step of one word from buffer SB into buffer SB ^ 1 (stored when `store`),
// the next step's draws made on the way.  The neighbours (src/gpu.rs:237-265):
// d0 x-1, d3 x+1 of row y; d1 (x-1 on even rows) and d2 (x+1 on odd rows) of
// row y-1; d4 (x+1 on odd rows) and d5 (x-1 on even rows) of row y+1.
template <int SB, bool REST>
__device__ __forceinline__ void fixed_step(const FixedWord& f, const Draws& cur, Draws& nxt,
                                           uint32_t next_key, bool any_solid, bool inflow,
                                           const uint32_t bern[7], bool ragged, bool store) {
  constexpr uint32_t o = SB * kFxBufBytes, P = kFxPlaneBytes;
  const uint32_t w0 = lds<o + 0 * P>(f.c_y), w1 = lds<o + 1 * P>(f.c_ym);
  const uint32_t w2 = lds<o + 2 * P>(f.c_ym), w3 = lds<o + 3 * P>(f.c_y);
  const uint32_t w4 = lds<o + 4 * P>(f.c_yp), w5 = lds<o + 5 * P>(f.c_yp);
  const uint32_t w6 = lds<o + 6 * P>(f.c_y);
  const uint32_t l0 = lds<o + 0 * P>(f.l_y), r3 = lds<o + 3 * P>(f.r_y);
  const uint32_t l1 = lds<o + 1 * P>(f.l_ym), r2 = lds<o + 2 * P>(f.r_ym);
  const uint32_t r4 = lds<o + 4 * P>(f.r_yp), l5 = lds<o + 5 * P>(f.l_yp);
  nxt = draws(next_key);
  uint32_t n[7];
  n[0] = __funnelshift_l(l0 << f.shl, w0, 1);
  n[1] = __funnelshift_l(l1 << f.shl, w1, f.sh_even);
  n[2] = put_bit(__funnelshift_r(w2, r2, f.sh_odd), r2, f.fix_odd);
  n[3] = put_bit(__funnelshift_r(w3, r3, 1), r3, f.fix);
  n[4] = put_bit(__funnelshift_r(w4, r4, f.sh_odd), r4, f.fix_odd);
  n[5] = __funnelshift_l(l5 << f.shl, w5, f.sh_even);
  n[6] = w6;
  uint32_t res[7];
  collide<REST>(n, cur, res);
  if (any_solid) {
    uint32_t o2[7];
#pragma unroll
    for (int d = 0; d < 7; ++d) o2[d] = res[d];
    walls(n, o2, f.sm, res);
  }
  if (inflow) {  // inflow re-seed of the leftmost columns (src/gpu.rs:296-306)
#pragma unroll
    for (int d = 0; d < 7; ++d) res[d] = (res[d] & ~f.apply) | (bern[d] & f.apply);
  }
  if (ragged) {  // clear the bits past the row's end
#pragma unroll
    for (int d = 0; d < 7; ++d) res[d] &= f.tail;
  }
  if (store) {
    constexpr uint32_t t = (SB ^ 1) * kFxBufBytes;
    sts<t + 0 * P>(f.c_y, res[0]);
    sts<t + 1 * P>(f.c_y, res[1]);
    sts<t + 2 * P>(f.c_y, res[2]);
    sts<t + 3 * P>(f.c_y, res[3]);
    sts<t + 4 * P>(f.c_y, res[4]);
    sts<t + 5 * P>(f.c_y, res[5]);
    sts<t + 6 * P>(f.c_y, res[6]);
  }
}

// The inflow draws of step k of the launch for this thread's word (zeros off
// the inflow or past the launch's last step); inlet and its per-step stride held
// in registers.
__device__ __forceinline__ void load_bern(const uint32_t* inlet, size_t stride,
                                          const FixedWord& f, bool lane_inflow, uint32_t k,
                                          uint32_t len, uint32_t bern[7]) {
  const bool on = lane_inflow && k < len;
  const uint32_t* bp = inlet + (size_t)k * stride + f.boff;
#pragma unroll
  for (int q = 0; q < 7; ++q) bern[q] = on ? __ldg(bp + q) : 0u;
}

// The sampling points of a lattice within the launch: after step t (1-based)
// when since + t is a multiple of every, or t == left (sampling only when the
// lattice has a field and every > 0).  `next` is the next multiple's t.
struct SampleClock {
  bool on;
  uint32_t every, left, next;
  __device__ __forceinline__ SampleClock(const ResSched& s, bool field) {
    on = field && s.every;
    every = s.every;
    left = s.left;
    next = on ? s.every - s.since % s.every : 0u;
  }
  // whether t is a sampling point; call with t increasing
  __device__ __forceinline__ bool due(uint32_t t) {
    if (!on) return false;
    bool d = t == left;
    if (t == next) {
      d = true;
      next += every;
    }
    return d;
  }
  // steps from t to the next sampling point after it (UINT32_MAX: none)
  __device__ __forceinline__ uint32_t until(uint32_t t) const {
    if (!on) return 0xffffffffu;
    uint32_t u = next - t;
    if (left > t) u = min(u, left - t);
    return u;
  }
};

// Coarse-grain lattice li's state held in global planes `par` (all of its
// CTAs' bands stored): field blocks rank * nwarps + warp, step C * nwarps.
__device__ __forceinline__ void sample_from_global(const LatDesc& d, uint32_t par, uint32_t first,
                                                   uint32_t stride) {
  const uint32_t nbf = d.bw * d.bh;
  SampleArgs sa;
  sa.a = par ? d.planes[1] : d.planes[0];
  sa.solid = d.solid;
  sa.dm = d.dm;
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
  for (uint32_t b = first; b < nbf; b += stride) sample_block(sa, b);
}

// One CTA per lattice: the whole lattice in this CTA, one word per thread.
template <int THREADS, bool REST>
__device__ __forceinline__ void fixed_single(const ResidentArgs& p, uint32_t* shm) {
  const uint32_t li = p.first_lat + blockIdx.x;
  const LatDesc& d = p.descs[li];
  const Dims dm = d.dm;
  const size_t S = dm.total;
  const uint32_t nw = dm.total;
  const uint64_t base = p.base ? *p.base : 0ull;
  const uint32_t warp = threadIdx.x >> 5;
  const uint32_t sbase = (uint32_t)__cvta_generic_to_shared(shm);
  {
    const uint32_t* g = ((d.cur0 + (uint32_t)base) & 1u) ? d.planes[1] : d.planes[0];
    for (uint32_t i = threadIdx.x; i < nw; i += THREADS)
#pragma unroll
      for (int q = 0; q < 7; ++q) shm[q * kFxPlaneWords + i] = __ldcg(g + q * S + i);
  }
  auto store_band = [&](uint32_t buf, uint32_t par) {
    uint32_t* g = par ? d.planes[1] : d.planes[0];
    for (uint32_t i = threadIdx.x; i < nw; i += THREADS)
#pragma unroll
      for (int q = 0; q < 7; ++q) g[q * S + i] = shm[buf * kFxBufWords + q * kFxPlaneWords + i];
  };
  const bool live = threadIdx.x < nw;
  const uint32_t lw = live ? threadIdx.x : nw - 1u;
  const uint32_t t0 = __umulhi(lw, dm.div_m);
  const uint32_t y = (t0 + ((lw - t0) >> dm.div_s1)) >> dm.div_s2;  // lw / wpr
  const uint32_t j = lw - y * dm.wpr;
  const uint32_t ym = y ? y - 1u : dm.h - 1u, yp = y + 1u == dm.h ? 0u : y + 1u;
  const FixedWord f = fixed_word(sbase, dm, y, ym, yp, y, j, live, d.solid);
  const bool any_solid = __any_sync(0xffffffffu, f.sm != 0u);
  const bool inflow = dm.iw != 0u, lane_inflow = inflow && j < dm.iw;
  const bool ragged = dm.tail != 0xffffffffu;
  SampleClock clock(p.sched[li], d.bw * d.bh != 0u);
  const uint64_t s0 = d.steps0 + base, seed = d.seed;
  const uint32_t* inl = d.inlet;
  const size_t istride = (size_t)dm.h * dm.iw * 7u;
  Draws cur = draws(f.g ^ step_seed32(seed, s0)), nxt;
  uint32_t bern[7], bnext[7];
  if (inflow) load_bern(inl, istride, f, lane_inflow, 0, p.len, bern);
  __syncthreads();  // the lattice is in buffer 0
  for (uint32_t k = 0; k < p.len; ++k) {
    const uint32_t key = f.g ^ step_seed32(seed, s0 + k + 1u);
    if (inflow) load_bern(inl, istride, f, lane_inflow, k + 1u, p.len, bnext);
    if (k & 1u)
      fixed_step<1, REST>(f, cur, nxt, key, any_solid, inflow, bern, ragged, live);
    else
      fixed_step<0, REST>(f, cur, nxt, key, any_solid, inflow, bern, ragged, live);
    cur = nxt;
    if (inflow)
#pragma unroll
      for (int q = 0; q < 7; ++q) bern[q] = bnext[q];
    __syncthreads();
    if (clock.due(k + 1u)) {
      const uint32_t par = (d.cur0 + (uint32_t)(base + k + 1u)) & 1u;
      store_band((k + 1u) & 1u, par);
      __syncthreads();
      sample_from_global(d, par, warp, THREADS / 32);
    }
  }
  store_band(p.len & 1u, (d.cur0 + (uint32_t)(base + p.len)) & 1u);
}

template <int THREADS>
__global__ void __launch_bounds__(THREADS) lgx_resident_fixed_kernel(const ResidentArgs p) {
  extern __shared__ __align__(16) uint32_t shm[];
  if (p.descs[p.first_lat + blockIdx.x].rest)
    fixed_single<THREADS, true>(p, shm);
  else
    fixed_single<THREADS, false>(p, shm);
}

// Clusters of C > 1 CTAs, K = p.ksteps >= 2 steps per cluster barrier.  Thread
// t owns word t % wpr of local row 1 + t / wpr (local rows 1 .. nb + 2K - 2:
// rows 0 and nb + 2K - 1 are only ever read); at step s of a super-step of k
// steps it updates its word if its row is within K - k + s .. K + nb + k - s - 1.
template <int THREADS, bool REST>
__device__ __forceinline__ void fixed_multi(const ResidentArgs& p, uint32_t* shm) {
  const cg::cluster_group cluster = cg::this_cluster();
  const uint32_t C = cluster.num_blocks(), rank = cluster.block_rank();
  const uint32_t li = p.first_lat + blockIdx.x / C;
  const LatDesc& d = p.descs[li];
  const Dims dm = d.dm;
  const size_t S = dm.total;
  const uint32_t K = p.ksteps;
  const uint32_t y0 = fx_band_start(rank, dm.h, C), y1 = fx_band_start(rank + 1u, dm.h, C);
  const uint32_t nb = y1 - y0;
  const uint32_t bandw = nb * dm.wpr;
  const uint64_t base = p.base ? *p.base : 0ull;
  const uint32_t warp = threadIdx.x >> 5;
  const uint32_t sbase = (uint32_t)__cvta_generic_to_shared(shm);
  {
    const uint32_t* g = ((d.cur0 + (uint32_t)base) & 1u) ? d.planes[1] : d.planes[0];
    for (uint32_t i = threadIdx.x; i < bandw; i += THREADS)
#pragma unroll
      for (int q = 0; q < 7; ++q)
        shm[q * kFxPlaneWords + K * dm.wpr + i] = __ldcg(g + q * S + (size_t)y0 * dm.wpr + i);
  }
  auto store_band = [&](uint32_t buf, uint32_t par) {
    uint32_t* g = par ? d.planes[1] : d.planes[0];
    for (uint32_t i = threadIdx.x; i < bandw; i += THREADS)
#pragma unroll
      for (int q = 0; q < 7; ++q)
        g[q * S + (size_t)y0 * dm.wpr + i] =
            shm[buf * kFxBufWords + q * kFxPlaneWords + K * dm.wpr + i];
  };
  // the K rows above the band are the last K of rank - 1's band, the K below
  // the first K of rank + 1's; every band has at least K rows
  const uint32_t up = (rank + C - 1u) % C, down = (rank + 1u) % C;
  const uint32_t nb_up = fx_band_start(up + 1u, dm.h, C) - fx_band_start(up, dm.h, C);
  const uint32_t* up_shm = cluster.map_shared_rank(shm, up);
  const uint32_t* down_shm = cluster.map_shared_rank(shm, down);

  const uint32_t words = (nb + 2u * K - 2u) * dm.wpr;
  const bool live = threadIdx.x < words;
  const uint32_t lw = live ? threadIdx.x : words - 1u;
  const uint32_t t0 = __umulhi(lw, dm.div_m);
  const uint32_t rr = (t0 + ((lw - t0) >> dm.div_s1)) >> dm.div_s2;  // lw / wpr
  const uint32_t j = lw - rr * dm.wpr;
  const uint32_t r = rr + 1u;  // local row
  uint32_t y = y0 + dm.h - K + r;
  if (y >= dm.h) y -= dm.h;
  if (y >= dm.h) y -= dm.h;
  const FixedWord f = fixed_word(sbase, dm, r, r - 1u, r + 1u, y, j, live, d.solid);
  const bool any_solid = __any_sync(0xffffffffu, f.sm != 0u);
  const bool inflow = dm.iw != 0u, lane_inflow = inflow && j < dm.iw;
  const bool ragged = dm.tail != 0xffffffffu;
  SampleClock clock(p.sched[li], d.bw * d.bh != 0u);
  const uint64_t s0 = d.steps0 + base, seed = d.seed;
  const uint32_t* inl = d.inlet;
  const size_t istride = (size_t)dm.h * dm.iw * 7u;
  Draws cur = draws(f.g ^ step_seed32(seed, s0)), nxt;
  uint32_t bern[7], bnext[7];
  if (inflow) load_bern(inl, istride, f, lane_inflow, 0, p.len, bern);

  uint32_t buf = 0;  // the buffer holding the state after step t
  for (uint32_t t = 0; t < p.len;) {
    const uint32_t k = min(min(K, p.len - t), clock.until(t));
    // (1) every band of buffer `buf` is complete (and loaded, before the first)
    asm volatile("barrier.cluster.arrive.release.aligned;" ::: "memory");
    asm volatile("barrier.cluster.wait.acquire.aligned;" ::: "memory");
    {
      const uint32_t hw = k * dm.wpr;  // words per plane and side
      const uint32_t off = buf * kFxBufWords;
      for (uint32_t i = threadIdx.x; i < 7u * hw; i += THREADS) {
        const uint32_t q = i / hw, w = i - q * hw;
        const uint32_t po = off + q * kFxPlaneWords;
        shm[po + (K - k) * dm.wpr + w] = up_shm[po + (K + nb_up - k) * dm.wpr + w];
        shm[po + (K + nb) * dm.wpr + w] = down_shm[po + K * dm.wpr + w];
      }
    }
    // (2) done reading the neighbours' buffer: they may overwrite it from their
    // second step on, after waiting for this phase
    asm volatile("barrier.cluster.arrive.release.aligned;" ::: "memory");
    __syncthreads();
    for (uint32_t s = 1; s <= k; ++s) {
      const uint32_t ks = t + s - 1u;  // step of the launch
      const uint32_t key = f.g ^ step_seed32(seed, s0 + ks + 1u);
      const bool act = live && r - (K - k + s) < nb + 2u * (k - s);
      if (inflow) load_bern(inl, istride, f, lane_inflow, ks + 1u, p.len, bnext);
      if (__any_sync(0xffffffffu, act)) {
        if (buf)
          fixed_step<1, REST>(f, cur, nxt, key, any_solid, inflow, bern, ragged, act);
        else
          fixed_step<0, REST>(f, cur, nxt, key, any_solid, inflow, bern, ragged, act);
      } else {
        nxt = draws(key);
      }
      cur = nxt;
      if (inflow)
#pragma unroll
        for (int q = 0; q < 7; ++q) bern[q] = bnext[q];
      buf ^= 1u;
      __syncthreads();
      if (s == 1u) asm volatile("barrier.cluster.wait.acquire.aligned;" ::: "memory");
    }
    t += k;
    if (clock.due(t)) {
      const uint32_t par = (d.cur0 + (uint32_t)(base + t)) & 1u;
      store_band(buf, par);
      cluster.sync();
      sample_from_global(d, par, rank * (THREADS / 32) + warp, C * (THREADS / 32));
    }
  }
  store_band(buf, (d.cur0 + (uint32_t)(base + p.len)) & 1u);
}

template <int THREADS>
__global__ void __launch_bounds__(THREADS) lgx_resident_fixed_multi_kernel(const ResidentArgs p) {
  extern __shared__ __align__(16) uint32_t shm[];
  const uint32_t C = cg::this_cluster().num_blocks();
  if (p.descs[p.first_lat + blockIdx.x / C].rest)
    fixed_multi<THREADS, true>(p, shm);
  else
    fixed_multi<THREADS, false>(p, shm);
}

template <int THREADS, bool MULTI>
cudaError_t fixed_attributes() {
  constexpr int kMaxDev = 64;
  static std::mutex mu;
  static bool set[kMaxDev] = {};
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess || dev < 0 || dev >= kMaxDev)
    return e != cudaSuccess ? e : cudaErrorInvalidDevice;
  const void* fn = MULTI ? (const void*)lgx_resident_fixed_multi_kernel<THREADS>
                         : (const void*)lgx_resident_fixed_kernel<THREADS>;
  std::lock_guard<std::mutex> g(mu);
  if (!set[dev]) {
    e = cudaFuncSetAttribute(fn, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kFxSmemBytes);
    if (e != cudaSuccess) return e;
    set[dev] = true;
  }
  return cudaSuccess;
}

template <int THREADS>
cudaError_t launch_fixed_t(const ResidentArgs& a, uint32_t nlat, uint32_t csize,
                           cudaStream_t st) {
  const bool multi = csize > 1u;
  cudaError_t e = multi ? fixed_attributes<THREADS, true>() : fixed_attributes<THREADS, false>();
  if (e != cudaSuccess) return e;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(nlat * csize);
  cfg.blockDim = dim3(THREADS);
  cfg.dynamicSmemBytes = kFxSmemBytes;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = csize;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  if (multi) return cudaLaunchKernelEx(&cfg, lgx_resident_fixed_multi_kernel<THREADS>, a);
  return cudaLaunchKernelEx(&cfg, lgx_resident_fixed_kernel<THREADS>, a);
}

}  // namespace

uint32_t resident_fixed_threads(const Dims& dm, uint32_t csize, uint32_t ksteps) {
  if (csize == 1u) return dm.total <= kFxPlaneWords ? dm.total : 0u;
  if (ksteps < 2u) return 0u;
  const uint32_t cap = (dm.h + csize - 1u) / csize;
  const uint32_t rows = cap + 2u * ksteps;
  if ((uint64_t)rows * dm.wpr > kFxPlaneWords) return 0u;
  return (rows - 2u) * dm.wpr;
}

bool resident_fixed_usable(uint32_t fixed_threads, uint32_t threads) {
  return fixed_threads != 0u && fixed_threads <= threads && threads <= kResidentFixedMaxThreads;
}

cudaError_t launch_resident_fixed(const ResidentArgs& a, uint32_t nlat, uint32_t csize,
                                  uint32_t threads, cudaStream_t st) {
  if (nlat == 0 || a.len == 0) return cudaSuccess;
  if (csize > 1u && a.ksteps < 2u) return cudaErrorInvalidValue;
  switch (threads) {
    case 128: return launch_fixed_t<128>(a, nlat, csize, st);
    case 256: return launch_fixed_t<256>(a, nlat, csize, st);
    case 512: return launch_fixed_t<512>(a, nlat, csize, st);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace lgx
