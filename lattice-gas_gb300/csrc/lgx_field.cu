// lgx_field.cu -- coarse-graining, particle count, byte<->plane transposes and
// the exhaustive circuit check.
//
// Coarse-graining (lgca_sample, src/gpu.rs:324-377): CTAs over tiles of a block
// row for blocks 16 or more columns wide, else one warp per block of the field
// (sample_block in lgx_step_impl.cuh).
#include <limits.h>
#include <stddef.h>
#include <stdlib.h>

#include "lgx_device.cuh"
#include "lgx_internal.hpp"
#include "lgx_reduce.cuh"
#include "lgx_step_impl.cuh"

namespace lgx {

// A single f32 product on the host (one rounding, as the reference's `by as f32 * SQRT3_2`).
static inline float __fmul_rn_host(float a, float b) { return a * b; }

namespace {

// Launched with programmatic stream serialisation: the next step's grid may
// start launching (and make its draws) at once, and the coarse-graining waits
// for the step before it to complete (griddepcontrol.wait) before it reads the
// planes.  The next step, in turn, waits for this grid to complete before it
// writes.  Launched plainly, the wait returns at once.
__global__ void __launch_bounds__(256) lgx_sample_kernel(const SampleArgs p, unsigned int* done,
                                                         unsigned long long* flag,
                                                         unsigned long long seq) {
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
  asm volatile("griddepcontrol.wait;" ::: "memory");
  const uint32_t blk = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (blk < p.bw * p.bh) sample_block<true>(p, blk);  // whole warps
  if (!flag) return;
  // a call that waits for the field: the last block to finish says so
  __threadfence_system();
  __syncthreads();
  if (threadIdx.x == 0 && atomicAdd(done, 1u) == gridDim.x - 1u) {
    *done = 0u;
    __threadfence_system();
    *reinterpret_cast<volatile unsigned long long*>(flag) = seq;
  }
}

// The tiles of sample_tile as a grid of their own (256 threads: eight rows
// apart), launched with programmatic serialisation as lgx_sample_kernel is.
__global__ void __launch_bounds__(256) lgx_sample_tiles_kernel(const SampleArgs p, uint32_t per,
                                                               uint32_t ncx, unsigned int* done,
                                                               unsigned long long* flag,
                                                               unsigned long long seq) {
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
  __shared__ int acc[4][kTileMaxBlocks];
  sample_tile<4>(p, blockIdx.x, per, ncx, acc);
  if (!flag) return;
  __threadfence_system();
  __syncthreads();
  if (threadIdx.x == 0 && atomicAdd(done, 1u) == gridDim.x - 1u) {
    *done = 0u;
    __threadfence_system();
    *reinterpret_cast<volatile unsigned long long*>(flag) = seq;
  }
}

// Particles on the lattice, obstacle sites included, tail-masked
// (lgca_count, src/gpu.rs:381-395), into a 64-bit counter.
// out: device counter (zeroed before the launch), or, with ticket set, mapped host
// memory that the last block writes (block_total_to_host).
__global__ void __launch_bounds__(256) lgx_count_kernel(const uint32_t* __restrict__ a, Dims dm,
                                                        unsigned long long* out,
                                                        unsigned long long* ticket,
                                                        unsigned long long* flag,
                                                        unsigned long long seq) {
  unsigned long long acc = 0;
  const size_t S = dm.total;
  for (uint32_t g = blockIdx.x * blockDim.x + threadIdx.x; g < dm.total;
       g += gridDim.x * blockDim.x) {
    const uint32_t j = g % dm.wpr;
    const uint32_t m = (j == dm.lastword) ? dm.tail : 0xffffffffu;
    uint32_t c = 0;
#pragma unroll
    for (int d = 0; d < 7; ++d) c += __popc(__ldg(a + d * S + g) & m);
    acc += c;
  }
  long long v[1] = {(long long)acc};
  if (ticket)
    block_total_to_host<1>(v, ticket, out, flag, seq);
  else
    block_add<1>(v, out);
}

// Lattice mass and momentum, obstacle sites included: per word the popcounts
// of the seven planes weighted by CX2 and CY2 (src/hex.rs), summed exactly.
__global__ void __launch_bounds__(256) lgx_moments_kernel(const uint32_t* __restrict__ a, Dims dm,
                                                          unsigned long long* out,
                                                          unsigned long long* ticket,
                                                          unsigned long long* flag,
                                                          unsigned long long seq) {
  long long mass = 0, px2 = 0, py2 = 0;
  const size_t S = dm.total;
  for (uint32_t g = blockIdx.x * blockDim.x + threadIdx.x; g < dm.total;
       g += gridDim.x * blockDim.x) {
    const uint32_t j = g % dm.wpr;
    const uint32_t m = (j == dm.lastword) ? dm.tail : 0xffffffffu;
    int c[7];
#pragma unroll
    for (int d = 0; d < 7; ++d) c[d] = __popc(__ldg(a + d * S + g) & m);
    mass += c[0] + c[1] + c[2] + c[3] + c[4] + c[5] + c[6];
    px2 += 2 * c[0] + c[1] - c[2] - 2 * c[3] - c[4] + c[5];
    py2 += c[1] + c[2] - c[4] - c[5];
  }
  long long v[3] = {mass, px2, py2};
  if (ticket)
    block_total_to_host<3>(v, ticket, out, flag, seq);
  else
    block_add<3>(v, out);
}

// Bytes -> planes: one warp per lattice word; lane k reads column 32 j + k and
// eight ballots give the seven planes and the solid word (src/gpu.rs:572-610).
__global__ void __launch_bounds__(256) lgx_pack_kernel(const uint8_t* __restrict__ cells, Dims dm,
                                                       uint32_t* planes, uint32_t* solid,
                                                       uint32_t* anysolid) {
  const uint32_t lane = threadIdx.x & 31u;
  const uint32_t g = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (g >= dm.total) return;
  const uint32_t y = g / dm.wpr, j = g - y * dm.wpr;
  const uint32_t x = j * 32u + lane;
  const uint32_t c = (x < dm.w) ? cells[(size_t)y * dm.w + x] : 0u;
  uint32_t mine = 0;
#pragma unroll
  for (int d = 0; d < 8; ++d) {
    const uint32_t v = __ballot_sync(0xffffffffu, (c >> d) & 1u);
    if (lane == (uint32_t)d) mine = v;
  }
  if (lane < 7u) planes[(size_t)lane * dm.total + g] = mine;
  if (lane == 7u) {
    solid[g] = mine;
    if (mine) atomicOr(anysolid + (g >> 5), 1u << (g & 31u));
  }
}

// Planes -> bytes (src/gpu.rs:630-652): bit k of the eight words of lattice
// word j is the byte of column 32 j + k.
__global__ void __launch_bounds__(256) lgx_unpack_kernel(const uint32_t* __restrict__ planes,
                                                         const uint32_t* __restrict__ solid,
                                                         Dims dm, uint8_t* cells) {
  const uint32_t lane = threadIdx.x & 31u;
  const uint32_t g = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (g >= dm.total) return;
  const uint32_t y = g / dm.wpr, j = g - y * dm.wpr;
  const uint32_t x = j * 32u + lane;
  uint32_t word = (lane < 7u) ? __ldg(planes + (size_t)lane * dm.total + g)
                              : (lane == 7u ? __ldg(solid + g) : 0u);
  uint32_t c = 0;
#pragma unroll
  for (int d = 0; d < 8; ++d) c |= ((__shfl_sync(0xffffffffu, word, d) >> lane) & 1u) << d;
  if (x < dm.w) cells[(size_t)y * dm.w + x] = (uint8_t)c;
}

// The exhaustive check of the circuit the step runs (lgca_verify,
// src/gpu.rs:399-417): thread i evaluates collide on all-lanes-equal inputs
// for state i / 48 and draw (i / 24 % 2, i / 6 % 4, i % 6).
template <bool REST>
__global__ void lgx_verify_kernel(uint32_t* out, uint32_t n) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uint32_t five = i % 6u, three = (i / 6u) % 4u, two = (i / 24u) % 2u, state = i / 48u;
  uint32_t nn[7];
  for (int d = 0; d < 7; ++d) nn[d] = ((state >> d) & 1u) ? 0xffffffffu : 0u;
  Draws s;
  s.s2 = two ? 0xffffffffu : 0u;
  for (int k = 0; k < 3; ++k) s.s3[k] = (three == (uint32_t)k) ? 0xffffffffu : 0u;
  for (int k = 0; k < 5; ++k) s.s5[k] = (five == (uint32_t)k) ? 0xffffffffu : 0u;
  uint32_t o[7];
  collide<REST>(nn, s, o);
  uint32_t r = 0u, bad = 0u;
  for (int d = 0; d < 7; ++d) {
    if (o[d] == 0xffffffffu)
      r |= 1u << d;
    else if (o[d] != 0u)
      bad = 1u;
  }
  out[i] = r | (bad << 16);
}

}  // namespace

// Field::vorticity (src/render.rs:127-143) of block k: on the block grid, dv/dx by a
// one-sided difference at the first and last column and a central one between,
// du/dy central with the rows periodic; f32 operations one by one, rounded to
// nearest, as the reference's Rust (which never fuses).
__device__ __forceinline__ float vorticity_at(const float* __restrict__ ux,
                                              const float* __restrict__ uy, uint32_t k,
                                              uint32_t bw, uint32_t bh, float dx, float dy) {
  const uint32_t j = k / bw, i = k - j * bw;
  const uint32_t ip = min(i + 1u, bw - 1u), im = i ? i - 1u : 0u;
  const uint32_t jp = j + 1u < bh ? j + 1u : 0u, jm = j ? j - 1u : bh - 1u;
  const float dvdx = __fdiv_rn(__fsub_rn(uy[j * bw + ip], uy[j * bw + im]),
                               __fmul_rn(__uint2float_rn(ip - im), dx));
  const float dudy = __fdiv_rn(__fsub_rn(ux[jp * bw + i], ux[jm * bw + i]), __fmul_rn(2.0f, dy));
  return __fsub_rn(dvdx, dudy);
}

// Field::mean_velocity (src/render.rs:146-161) by one block: the f32 sums run in
// block order, as the reference adds them, so each is one dependent chain of
// adds on one thread: lane 0 of warp 0 adds the x components, lane 0 of warp 1
// the y components, on different schedulers.  The other six warps stage the
// field in chunks of kMeanChunk blocks into two shared buffers: while the
// adding threads work through chunk c, they load chunk c + 1, every load of a
// thread issued before any of its stores, so a chunk costs one memory latency
// rather than one per row of threads.  Each non-solid block's velocity is
// staged as it is and each solid block's (and the padding's) as -0.0: adding
// -0.0 leaves every f32 unchanged in round-to-nearest (x + -0 = x,
// +0 + -0 = +0, -0 + -0 = -0), so the sums are the reference's with no test in
// the adding loop.  An adding thread reads 32 values ahead of the adds that use
// them (two register sets), so the chain of f32 adds, not the shared-memory
// latency, sets its pace.  The reference's count n adds 1.0f per non-solid
// block: the exact count up to 2^24, where it stops growing; the block counts
// with a reduction and rounds the same way.
constexpr uint32_t kMeanChunk = 2048;  // blocks per staged chunk (8 KB per sum)
constexpr uint32_t kAnalysisThreads = 256;
constexpr uint32_t kStagers = kAnalysisThreads - 64;  // warps 2.. stage, warps 0, 1 add
constexpr uint32_t kStagePer = (kMeanChunk + kStagers - 1) / kStagers;

__device__ __forceinline__ uint32_t stage_chunk(const float* __restrict__ ux,
                                                const float* __restrict__ uy,
                                                const float* __restrict__ sol, uint32_t nb,
                                                uint32_t c0, float* fx, float* fy) {
  const uint32_t t = threadIdx.x - 64u;
  float vx[kStagePer], vy[kStagePer], vs[kStagePer];
  uint32_t fluid = 0;
  // all three loads of every block first, none waiting on another's value: one
  // memory latency per chunk (the velocity loads once waited on the solid
  // fraction's, two latencies per row of threads)
#pragma unroll
  for (uint32_t i = 0; i < kStagePer; ++i) {
    const uint32_t k = t + i * kStagers;
    const bool in = k < kMeanChunk && c0 + k < nb;
    const uint32_t at = in ? c0 + k : 0u;
    vs[i] = in ? __ldg(sol + at) : 1.0f;
    vx[i] = __ldg(ux + at);
    vy[i] = __ldg(uy + at);
  }
#pragma unroll
  for (uint32_t i = 0; i < kStagePer; ++i) {
    const bool f = vs[i] < 0.5f;
    vx[i] = f ? vx[i] : -0.0f;
    vy[i] = f ? vy[i] : -0.0f;
    fluid += f ? 1u : 0u;
  }
#pragma unroll
  for (uint32_t i = 0; i < kStagePer; ++i) {
    const uint32_t k = t + i * kStagers;
    if (k < kMeanChunk) {
      fx[k] = vx[i];
      fy[k] = vy[i];
    }
  }
  return fluid;
}

// One chain: s + q[0] + q[1] + ... over `nq` float4s (a multiple of kAhead), in
// order, the next kAhead float4s loaded while the current ones are added (32
// adds, about 140 cycles, cover a shared-memory load's latency).
constexpr uint32_t kAhead = 8;
__device__ __forceinline__ float add_in_order(float s, const float4* q, uint32_t nq) {
  float4 a[kAhead];
#pragma unroll
  for (int i = 0; i < (int)kAhead; ++i) a[i] = q[i];
  for (uint32_t k = 0; k < nq; k += kAhead) {
    const uint32_t kn = k + kAhead < nq ? k + kAhead : k;  // the last round rereads its own
    float4 n[kAhead];
#pragma unroll
    for (int i = 0; i < (int)kAhead; ++i) n[i] = q[kn + i];
#pragma unroll
    for (int i = 0; i < (int)kAhead; ++i) {
      s = __fadd_rn(s, a[i].x);
      s = __fadd_rn(s, a[i].y);
      s = __fadd_rn(s, a[i].z);
      s = __fadd_rn(s, a[i].w);
    }
#pragma unroll
    for (int i = 0; i < (int)kAhead; ++i) a[i] = n[i];
  }
  return s;
}

// The sum over a block of kAnalysisThreads threads' counts, on thread 0: each
// warp adds its own (one reduction instruction), thread 0 adds the warps'.  (A
// 64-bit shared-memory atomicAdd from every thread serialises: it cost about 25k
// cycles per block.)
__device__ __forceinline__ unsigned long long block_count(uint32_t v, uint32_t* s_warp) {
  const uint32_t w = __reduce_add_sync(0xffffffffu, v);
  if ((threadIdx.x & 31u) == 0u) s_warp[threadIdx.x >> 5] = w;
  __syncthreads();
  unsigned long long c = 0;
  if (threadIdx.x == 0)
#pragma unroll
    for (uint32_t i = 0; i < kAnalysisThreads / 32; ++i) c += s_warp[i];
  return c;
}

__device__ __forceinline__ void mean_velocity_block(const float* __restrict__ ux,
                                                    const float* __restrict__ uy,
                                                    const float* __restrict__ sol, uint32_t nb,
                                                    float* __restrict__ out) {
  __shared__ float4 s_ux[2][kMeanChunk / 4], s_uy[2][kMeanChunk / 4];
  __shared__ uint32_t s_warp[kAnalysisThreads / 32];
  __shared__ float s_sy;
  float sum = 0.0f;  // x on thread 0, y on thread 32
  uint32_t mine = 0;
  const bool stager = threadIdx.x >= 64u;
  const uint32_t nchunks = (nb + kMeanChunk - 1u) / kMeanChunk;
  if (stager && nchunks)
    mine += stage_chunk(ux, uy, sol, nb, 0, reinterpret_cast<float*>(s_ux[0]),
                        reinterpret_cast<float*>(s_uy[0]));
  __syncthreads();
  for (uint32_t c = 0; c < nchunks; ++c) {
    const uint32_t cur = c & 1u;
    if (stager) {
      if (c + 1u < nchunks)
        mine += stage_chunk(ux, uy, sol, nb, (c + 1u) * kMeanChunk,
                            reinterpret_cast<float*>(s_ux[cur ^ 1u]),
                            reinterpret_cast<float*>(s_uy[cur ^ 1u]));
    } else if ((threadIdx.x & 31u) == 0u) {
      const uint32_t len = min(kMeanChunk, nb - c * kMeanChunk);
      const uint32_t nq = ((len + 31u) & ~31u) / 4u;  // float4s, a multiple of kAhead
      // each thread names its own shared array, so that its loads stay
      // shared-memory loads (a pointer picked at run time would be generic)
      if (threadIdx.x == 0)
        sum = add_in_order(sum, s_ux[cur], nq);
      else
        sum = add_in_order(sum, s_uy[cur], nq);
    }
    __syncthreads();
  }
  if (threadIdx.x == 32) s_sy = sum;
  const unsigned long long c = block_count(mine, s_warp);  // its barrier orders s_sy too
  if (threadIdx.x == 0) {
    const float n = c <= (1ull << 24) ? (float)c : 16777216.0f;
    out[0] = n == 0.0f ? 0.0f : __fdiv_rn(sum, n);
    out[1] = n == 0.0f ? 0.0f : __fdiv_rn(s_sy, n);
  }
}

// The field analyses of one field in one launch: block 0 forms the mean velocity
// when `mean` is set, the other blocks the vorticity (one thread per field block)
// when `vort` is set.
// The end of every block of an analyses launch whose results the host waits for
// on a flag: each thread's results are made visible to the host, and the last
// block to finish (a counter it sets back to zero) writes seq to *flag.  Every
// thread of the block must call it.
__device__ __forceinline__ void analyses_done(unsigned int* done, unsigned long long* flag,
                                              unsigned long long seq) {
  if (!flag) return;
  __threadfence_system();
  __syncthreads();
  if (threadIdx.x == 0 && atomicAdd(done, 1u) == gridDim.x - 1u) {
    *done = 0u;
    __threadfence_system();
    *reinterpret_cast<volatile unsigned long long*>(flag) = seq;
  }
}

__global__ void __launch_bounds__(kAnalysisThreads) lgx_field_analyses_kernel(
    const float* __restrict__ ux, const float* __restrict__ uy, const float* __restrict__ sol,
    uint32_t bw, uint32_t bh, float dx, float dy, float* __restrict__ vort,
    float* __restrict__ mean, unsigned int* done, unsigned long long* flag,
    unsigned long long seq) {
  uint32_t b = blockIdx.x;
  if (mean && b == 0) {
    mean_velocity_block(ux, uy, sol, bw * bh, mean);
  } else {
    if (mean) b -= 1u;
    const uint32_t k = b * kAnalysisThreads + threadIdx.x;
    if (vort && k < bw * bh) vort[k] = vorticity_at(ux, uy, k, bw, bh, dx, dy);
  }
  analyses_done(done, flag, seq);
}

// ---- the mean velocity's sums in segments, speculatively ----
//
// The sums must come out as the reference's in-order f32 additions, which is one
// chain of dependent adds (4.1 cycles each on GB300: 13 us for 6,528 blocks).  The
// field's nb values are cut into k <= 16 segments of L values.  Segment 0 is summed
// from +0 as the reference sums it.  For every later segment j and each of the two
// sums, kSpecParts blocks sum the segment in order from kSpecGuesses consecutive f32
// start values (one per thread) centred on the exact sum of the values before it; the in-order f32 partial sum differs from that exact sum by its
// accumulated rounding, usually a few to a few hundred units in the last place.
// The last of these blocks to finish walks the segments: with the exact partial
// sum s at the start of segment j, the thread whose start value is s (found by the
// distance in representable floats from the centre) has summed segment j exactly
// as the reference would have, so its end value is the exact partial sum at the
// next segment; where s is not among the guesses (or is not finite) the segment is
// summed from s in order instead.  Every path adds the same values in the same
// order with the same roundings, so the result is bit-equal to the chain.  Solid
// blocks enter as -0.0, as in the chained kernel above.
// start values per segment and sum (256, 512 and 1,024 timed alike on the
// 2048 x 1280 field, 20.6-21.1 us per call; 2,048 and shorter segments, more
// blocks for the last one to wait for, 22-23 us)
constexpr uint32_t kSpecGuesses = 512;
constexpr uint32_t kSpecParts = kSpecGuesses / kAnalysisThreads;  // blocks per segment and sum
constexpr uint32_t kSpecMaxSegments = 16;
constexpr uint32_t kSpecMinSegment = 512;    // values per segment, at least
constexpr uint32_t kSpecMaxSegment = 4096;
constexpr uint32_t kSpecMaxBlocks = kSpecMaxSegments * kSpecMaxSegment;  // 65,536

// Device scratch of one field's segmented sums, zeroed once before its first use
// (the block counter returns to zero at the end of every launch).
struct MeanScratch {
  unsigned int counter;
  unsigned int done;  // blocks of the launch finished (analyses_done)
  unsigned long long fluid;
  float first[2];
  float pad2[2];
  int center[2][kSpecMaxSegments];  // the centre's order index (INT_MIN: none usable)
  float table[2][kSpecMaxSegments][kSpecGuesses];  // 16-byte aligned: offset 160
};
static_assert(offsetof(MeanScratch, table) % 16 == 0, "the tables are read as float4s");

// A float's index in the order of representable floats (-0.0 and +0.0 both 0).
__device__ __forceinline__ int f_order(float f) {
  const int b = __float_as_int(f);
  return b >= 0 ? b : -(b & 0x7fffffff);
}
__device__ __forceinline__ float f_from_order(int o) {
  if (o > 0x7f7fffff || o < -0x7f7fffff) return __int_as_float(0x7fc00000);  // past the finite
  return o >= 0 ? __int_as_float(o) : __int_as_float((-o) | (int)0x80000000);
}

// A field block's value in the sum: its velocity component, -0.0 where solid
// (both loads issued before either is looked at, so a loop keeps them in flight).
__device__ __forceinline__ float mean_term(const float* __restrict__ u,
                                           const float* __restrict__ sol, uint32_t i) {
  const float s = __ldg(sol + i), v = __ldg(u + i);
  return s < 0.5f ? v : -0.0f;
}

// values [i0, i0 + len) of the masked component into dst[0 .. round up to 32),
// padded with -0.0; returns the float4 count (a multiple of kAhead)
__device__ __forceinline__ uint32_t stage_terms(const float* __restrict__ u,
                                                const float* __restrict__ sol, uint32_t i0,
                                                uint32_t len, float* dst) {
  const uint32_t padded = (len + 31u) & ~31u;
  for (uint32_t i = threadIdx.x; i < padded; i += kAnalysisThreads)
    dst[i] = i < len ? mean_term(u, sol, i0 + i) : -0.0f;
  return padded / 4u;
}

// The combining block copies, for every segment, the kSpecWindow table entries
// around the centre into shared memory in one round of loads (almost every walk
// lands there); an entry outside that window is read from L2.
constexpr uint32_t kSpecWindow = 256;
constexpr uint32_t kSpecWindowWords = 2u * (kSpecMaxSegments - 1u) * kSpecWindow;
constexpr uint32_t kSpecShared = kSpecWindowWords + kSpecMaxSegment;

__device__ __forceinline__ void mean_spec_block(const float* __restrict__ ux,
                                                const float* __restrict__ uy,
                                                const float* __restrict__ sol, uint32_t nb,
                                                uint32_t L, uint32_t k, uint32_t b,
                                                MeanScratch* ms, float* out, int mode) {
  // a segment's values (block 0: both sums' segment 0, x at 0 and y at 4096); in
  // the combining block the table windows, then at kSpecWindowWords a segment to sum
  __shared__ __align__(16) float s_mem[kSpecShared];
  __shared__ int s_center[2][kSpecMaxSegments];
  __shared__ long long s_red[kAnalysisThreads / 32];
  __shared__ uint32_t s_warp[kAnalysisThreads / 32];
  __shared__ float s_res[2];
  __shared__ int s_hit[2];
  __shared__ bool s_last;
  const uint32_t tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5;
  const uint32_t G = kSpecGuesses;
  if (b == 0) {
    const uint32_t len = min(L, nb);
    const uint32_t nq = stage_terms(ux, sol, 0, len, s_mem);
    stage_terms(uy, sol, 0, len, s_mem + kSpecMaxSegment);
    uint32_t fluid = 0;
#pragma unroll 8
    for (uint32_t i = tid; i < nb; i += kAnalysisThreads) fluid += __ldg(sol + i) < 0.5f ? 1u : 0u;
    const unsigned long long count = block_count(fluid, s_warp);  // and the staging is done
    if (tid == 0 || tid == 32) {
      const float s = tid ? add_in_order(0.0f, reinterpret_cast<const float4*>(s_mem + kSpecMaxSegment), nq)
                          : add_in_order(0.0f, reinterpret_cast<const float4*>(s_mem), nq);
      ms->first[tid ? 1 : 0] = s;
    }
    if (tid == 0) ms->fluid = count;
  } else {
    const uint32_t q = (b - 1u) / kSpecParts, part = (b - 1u) - q * kSpecParts;
    const uint32_t z = q / (k - 1u);                // 0: x, 1: y
    const uint32_t j = q - z * (k - 1u) + 1u;        // segment 1 .. k-1
    const uint32_t gi = part * kAnalysisThreads + tid;  // this thread's guess
    const float* u = z ? uy : ux;
    const uint32_t i0 = j * L, len = min(L, nb - i0);
    // the sum of the values before the segment in 64-bit fixed point (units of
    // 2^-40: within n * 2^-41 of the exact sum, no overflow for |values| < 64 and
    // n <= 2^16; FP64 is slow here), in a fixed order; a value out of that range
    // leaves no centre
    long long acc = 0;
    bool bad = false;
    for (uint32_t i = tid; i < i0; i += 24u * kAnalysisThreads) {  // 48 loads in flight
      float v[24], sv[24];
#pragma unroll
      for (uint32_t q = 0; q < 24; ++q) {
        const uint32_t ii = i + q * kAnalysisThreads;
        const bool in = ii < i0;
        sv[q] = in ? __ldg(sol + ii) : 1.0f;
        v[q] = in ? __ldg(u + ii) : 0.0f;
      }
#pragma unroll
      for (uint32_t q = 0; q < 24; ++q) {
        const float t = sv[q] < 0.5f ? v[q] : 0.0f;
        bad |= !(fabsf(t) < 64.0f);
        acc += __float2ll_rn(__fmul_rn(t, 1099511627776.0f));
      }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
    if (lane == 0) s_red[warp] = acc;
    const uint32_t nq = stage_terms(u, sol, i0, len, s_mem);
    const bool anybad = __syncthreads_or(bad);  // and the segment is staged
    long long pre = 0;
#pragma unroll
    for (uint32_t w = 0; w < kAnalysisThreads / 32; ++w) pre += s_red[w];
    const float c = anybad ? __int_as_float(0x7fc00000)
                           : __fmul_rn(__ll2float_rn(pre), 9.094947017729282e-13f);  // 2^-40
    const int co = f_order(c);
    const float start = f_from_order(co + (int)gi - (int)(G / 2u));
    ms->table[z][j][gi] = add_in_order(start, reinterpret_cast<const float4*>(s_mem), nq);
    if (tid == 0 && part == 0) ms->center[z][j] = isfinite(c) ? co : INT_MIN;
  }
  // the last of the 1 + 2 (k - 1) kSpecParts blocks to finish combines
  __threadfence();
  __syncthreads();
  if (tid == 0) s_last = atomicAdd(&ms->counter, 1u) == 2u * (k - 1u) * kSpecParts;
  __syncthreads();
  if (!s_last) return;
  __threadfence();
  // what the walk reads, in one round of loads: the table windows around the
  // centres, the centres, segment 0's sums
  constexpr uint32_t W4 = kSpecWindow / 4u, w0 = (kSpecGuesses - kSpecWindow) / 2u;
  for (uint32_t i = tid; i < 2u * (k - 1u) * W4; i += kAnalysisThreads) {
    const uint32_t r = i / W4, z = r / (k - 1u), j = r - z * (k - 1u) + 1u;
    reinterpret_cast<float4*>(s_mem)[i] =
        __ldcg(reinterpret_cast<const float4*>(&ms->table[z][j][w0]) + (i - r * W4));
  }
  if (tid < 2u * kSpecMaxSegments)
    s_center[tid / kSpecMaxSegments][tid % kSpecMaxSegments] =
        __ldcg(&ms->center[tid / kSpecMaxSegments][tid % kSpecMaxSegments]);
  if (tid < 2) s_res[tid] = __ldcg(&ms->first[tid]);
  __syncthreads();
  // the walk: threads 0 and 1 follow the x and the y sum through the tables,
  // segment after segment, until a segment whose start is not among its guesses;
  // the whole block then stages that segment and thread 0 sums it in order
  float* seg = s_mem + kSpecWindowWords;
  if (tid < 2) s_hit[tid] = 1;  // s_hit[z]: the next segment of sum z to walk
  __syncthreads();
  for (;;) {
    if (tid < 2) {
      uint32_t j = (uint32_t)s_hit[tid];
      float s = s_res[tid];
      for (; j < k; ++j) {
        const int c = s_center[tid][j];
        const long long o = (long long)f_order(s) - (long long)c + (long long)(G / 2u);
        const bool take = mode == 1 || (mode == 2 && (j & 1u) == 0u);
        if (!(take && c != INT_MIN && isfinite(s) && o >= 0 && o < (long long)G)) break;
        const uint32_t w = (uint32_t)o - w0;  // wraps when o < w0
        s = w < kSpecWindow ? s_mem[(tid * (k - 1u) + j - 1u) * kSpecWindow + w]
                            : __ldcg(&ms->table[tid][j][(uint32_t)o]);
      }
      s_res[tid] = s;
      s_hit[tid] = (int)j;
    }
    __syncthreads();
    const uint32_t z = (uint32_t)s_hit[0] < k ? 0u : 1u;
    const uint32_t j = (uint32_t)s_hit[z];
    if (j >= k) break;  // both walks are through (the same for every thread)
    const uint32_t i0 = j * L;
    const uint32_t nq = stage_terms(z ? uy : ux, sol, i0, min(L, nb - i0), seg);
    __syncthreads();
    if (tid == 0) {
      s_res[z] = add_in_order(s_res[z], reinterpret_cast<const float4*>(seg), nq);
      s_hit[z] = (int)j + 1;
    }
    __syncthreads();
  }
  if (tid == 0) {
    const unsigned long long cnt = __ldcg(&ms->fluid);
    const float n = cnt <= (1ull << 24) ? (float)cnt : 16777216.0f;
    out[0] = n == 0.0f ? 0.0f : __fdiv_rn(s_res[0], n);
    out[1] = n == 0.0f ? 0.0f : __fdiv_rn(s_res[1], n);
    ms->counter = 0u;  // for the next launch
  }
}

// The field analyses with the segmented mean: the first 1 + 2 (k - 1) kSpecParts
// blocks the mean velocity's segments, the rest the vorticity when `vort` is set.
__global__ void __launch_bounds__(kAnalysisThreads) lgx_field_mean_spec_kernel(
    const float* __restrict__ ux, const float* __restrict__ uy, const float* __restrict__ sol,
    uint32_t bw, uint32_t bh, float dx, float dy, float* __restrict__ vort,
    float* __restrict__ mean, MeanScratch* ms, uint32_t L, uint32_t k, int mode,
    unsigned long long* flag, unsigned long long seq) {
  const uint32_t nmean = 1u + 2u * (k - 1u) * kSpecParts;
  if (blockIdx.x < nmean) {
    mean_spec_block(ux, uy, sol, bw * bh, L, k, blockIdx.x, ms, mean, mode);
  } else {
    const uint32_t kk = (blockIdx.x - nmean) * kAnalysisThreads + threadIdx.x;
    if (vort && kk < bw * bh) vort[kk] = vorticity_at(ux, uy, kk, bw, bh, dx, dy);
  }
  analyses_done(&ms->done, flag, seq);
}

// LGX_MEAN_SPECULATE (tests): 0 sums every segment in order in the combining block,
// 2 takes the guess tables of even segments only; 1 (unset) takes every table.
int mean_spec_mode() {
  static const int mode = [] {
    const char* v = getenv("LGX_MEAN_SPECULATE");
    return v && v[0] == '0' ? 0 : v && v[0] == '2' ? 2 : 1;
  }();
  return mode;
}

size_t mean_scratch_bytes() { return sizeof(MeanScratch); }

cudaError_t launch_field_analyses(const float* field, uint32_t bw, uint32_t bh, uint32_t bx,
                                  uint32_t by, float* vort, float* mean, void* mean_scratch,
                                  cudaStream_t st, unsigned long long* flag,
                                  unsigned long long seq) {
  if (!mean_scratch) flag = nullptr;  // the done counter lives there
  const uint32_t nb = bw * bh;
  const uint32_t vblocks = vort ? (nb + kAnalysisThreads - 1u) / kAnalysisThreads : 0u;
  const float dx = (float)bx;
  const float dy = __fmul_rn_host((float)by, 0.8660254f);
  if (mean && mean_scratch && nb <= kSpecMaxBlocks) {
    uint32_t L = (nb + kSpecMaxSegments - 1u) / kSpecMaxSegments;
    L = (L + 31u) & ~31u;
    if (L < kSpecMinSegment) L = kSpecMinSegment;
    const uint32_t k = nb ? (nb + L - 1u) / L : 1u;
    lgx_field_mean_spec_kernel<<<1u + 2u * (k - 1u) * kSpecParts + vblocks, kAnalysisThreads,
                                 0, st>>>(
        field, field + nb, field + 3 * nb, bw, bh, dx, dy, vort, mean,
        (MeanScratch*)mean_scratch, L, k, mean_spec_mode(), flag, seq);
    return cudaGetLastError();
  }
  const uint32_t blocks = (mean ? 1u : 0u) + vblocks;
  if (blocks == 0) return cudaSuccess;
  unsigned int* done = mean_scratch ? &((MeanScratch*)mean_scratch)->done : nullptr;
  lgx_field_analyses_kernel<<<blocks, kAnalysisThreads, 0, st>>>(
      field, field + nb, field + 3 * nb, bw, bh, dx, dy, vort, mean, done, flag, seq);
  return cudaGetLastError();
}

cudaError_t launch_moments(const uint32_t* a, const Dims& dm, unsigned long long* out,
                           cudaStream_t st, unsigned long long* ticket, unsigned long long* flag,
                           unsigned long long seq) {
  if (!ticket) {
    cudaError_t e = cudaMemsetAsync(out, 0, 3 * sizeof(unsigned long long), st);
    if (e != cudaSuccess) return e;
  }
  uint32_t blocks = (dm.total + 255) / 256;
  if (blocks > kReduceMaxBlocks) blocks = kReduceMaxBlocks;  // two per SM, grid-stride beyond
  lgx_moments_kernel<<<blocks, 256, 0, st>>>(a, dm, out, ticket, flag, seq);
  return cudaGetLastError();
}

bool sample_tiling(const SampleArgs& s, SampleTiles* t) {
  if (s.bx < kTileMinWidth || s.bw * s.bh == 0) return false;
  t->s = s;
  tile_shape(s.bx, s.bw, &t->per, &t->ncx);
  t->nblocks = t->ncx * s.bh;
  return true;
}

cudaError_t launch_sample(const SampleArgs& s, cudaStream_t st, unsigned int* done,
                          unsigned long long* flag, unsigned long long seq) {
  const uint32_t nb = s.bw * s.bh;
  if (nb == 0) return cudaSuccess;
  cudaLaunchConfig_t cfg{};
  cfg.blockDim = dim3(256);
  cfg.dynamicSmemBytes = 0;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  SampleTiles t;
  if (sample_tiling(s, &t)) {
    cfg.gridDim = dim3(t.nblocks);
    return cudaLaunchKernelEx(&cfg, lgx_sample_tiles_kernel, s, t.per, t.ncx, done, flag, seq);
  }
  cfg.gridDim = dim3((nb + 7) / 8);
  return cudaLaunchKernelEx(&cfg, lgx_sample_kernel, s, done, flag, seq);
}

cudaError_t launch_count(const uint32_t* a, const Dims& dm, unsigned long long* out,
                         cudaStream_t st, unsigned long long* ticket, unsigned long long* flag,
                         unsigned long long seq) {
  if (!ticket) {
    cudaError_t e = cudaMemsetAsync(out, 0, sizeof(unsigned long long), st);
    if (e != cudaSuccess) return e;
  }
  uint32_t blocks = (dm.total + 255) / 256;
  if (blocks > kReduceMaxBlocks) blocks = kReduceMaxBlocks;  // two per SM, grid-stride beyond
  lgx_count_kernel<<<blocks, 256, 0, st>>>(a, dm, out, ticket, flag, seq);
  return cudaGetLastError();
}

cudaError_t launch_pack(const uint8_t* cells, const Dims& dm, uint32_t* planes, uint32_t* solid,
                        uint32_t* anysolid, cudaStream_t st) {
  cudaError_t e = cudaMemsetAsync(anysolid, 0, ((dm.total + 31) / 32) * sizeof(uint32_t), st);
  if (e != cudaSuccess) return e;
  lgx_pack_kernel<<<(dm.total + 7) / 8, 256, 0, st>>>(cells, dm, planes, solid, anysolid);
  return cudaGetLastError();
}

cudaError_t launch_unpack(const uint32_t* planes, const uint32_t* solid, const Dims& dm,
                          uint8_t* cells, cudaStream_t st) {
  lgx_unpack_kernel<<<(dm.total + 7) / 8, 256, 0, st>>>(planes, solid, dm, cells);
  return cudaGetLastError();
}

cudaError_t launch_verify(uint32_t* out, uint32_t n, bool rest, cudaStream_t st) {
  if (rest)
    lgx_verify_kernel<true><<<(n + 127) / 128, 128, 0, st>>>(out, n);
  else
    lgx_verify_kernel<false><<<(n + 127) / 128, 128, 0, st>>>(out, n);
  return cudaGetLastError();
}

}  // namespace lgx
