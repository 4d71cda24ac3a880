// lgx_bytes.cu -- the reference's byte-per-cell update, on the GPU.
//
// The reference's CPU lattice (src/lattice.rs) draws its collisions from a
// different random stream than its GPU bitplanes do: one xorshift64*
// generator per band of rows (bands of ceil(h / threads) rows), one draw per
// non-obstacle cell in row-major order, and a padded lookup table
// (src/collision.rs:161-210); the inflow re-seed after each step draws from one
// serial generator (src/lattice.rs:270-285).  Its golden tests pin that stream
// bit for bit.  This file runs the same stream on the device.
//
// The draws are sequential within a band, so a thread takes a segment of one
// row and first jumps the band's generator to the segment's draw index.  The
// generator's state update is linear over GF(2), x -> M x, so k steps are M^k x;
// with the 32 matrices M^(2^i) (columns precomputed on the host) a jump is at
// most 32 matrix-vector products.  The draw index of every segment is fixed:
// it counts the non-obstacle cells of the band before the segment, and
// obstacles never move, so those offsets are computed once when cells are
// loaded.  The inflow is the same with one stream and 3 or 4 draws per cell.
#include <cuda_runtime.h>
#include <string.h>

#include <algorithm>
#include <map>
#include <new>
#include <string>
#include <tuple>
#include <vector>

#include "../../include/lgx.h"
#include "lgx_internal.hpp"
#include "lgx_rng.cuh"

namespace {

using lgx::jump_ahead;
using lgx::rng_seed;
using lgx::xorshift;

constexpr uint32_t kSeg = 128;     // cells per thread segment
constexpr int kJumps = 32;         // the first 32 jump matrices: offsets below 2^32
constexpr uint8_t kSolid = 0x80, kRest = 0x40;
constexpr uint64_t kMul = lgx::kRngMul;

struct ByteStepArgs {
  const uint8_t* old;
  uint8_t* out;
  const uint8_t* table;  // n_states * stride outcomes
  uint32_t stride;
  uint32_t w, h, band;  // band: rows per generator
  uint32_t segs_per_row;
  const uint32_t* seg_off;  // draw index of each segment within its band
  const uint64_t* jump;
  uint64_t base_seed;       // seed ^ steps * 0x9E3779B97F4A7C15
};

struct ByteInletArgs {
  uint8_t* cells;
  uint32_t w, h, cols;
  const uint32_t* row_off;  // draws before row y
  const uint64_t* jump;
  uint64_t seed;            // seed ^ steps * 0xD1B54A32D192ED03 (steps after the step)
  uint32_t t[7];
  int rest;
};

// One row segment of the fused propagate-then-collide gather
// (src/lattice.rs:324-364).
__global__ void __launch_bounds__(128) lgx_byte_step_kernel(const ByteStepArgs p) {
  __shared__ uint64_t jump[kJumps * 64];
  __shared__ uint8_t table[128 * 30];
  for (uint32_t i = threadIdx.x; i < kJumps * 64; i += blockDim.x) jump[i] = p.jump[i];
  const uint32_t tsize = 128u * p.stride;
  for (uint32_t i = threadIdx.x; i < tsize; i += blockDim.x) table[i] = p.table[i];
  __syncthreads();
  const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= p.h * p.segs_per_row) return;
  const uint32_t y = s / p.segs_per_row;
  const uint32_t x0 = (s - y * p.segs_per_row) * kSeg;
  const uint32_t x1 = min(x0 + kSeg, p.w);
  const uint32_t b = y / p.band;
  uint64_t st = jump_ahead(rng_seed(p.base_seed ^ ((uint64_t)(b + 1) << 32)), p.seg_off[s], jump);

  // Column offsets to the neighbour a particle arrives from: direction d takes
  // from the neighbour in the opposite direction (src/hex.rs:36-41).
  const bool odd = y & 1u;
  const int DXE[6] = {1, 0, -1, -1, -1, 0};
  const int DXO[6] = {1, 1, 0, -1, 0, 1};
  const int DY[6] = {0, 1, 1, 0, -1, -1};
  const int OPP[6] = {3, 4, 5, 0, 1, 2};
  int sdx[6];
  const uint8_t* srow[6];
  for (int d = 0; d < 6; ++d) {
    const int bk = OPP[d];
    sdx[d] = odd ? DXO[bk] : DXE[bk];
    int sy = (int)y + DY[bk];
    if (sy < 0) sy += (int)p.h;
    if (sy >= (int)p.h) sy -= (int)p.h;
    srow[d] = p.old + (size_t)sy * p.w;
  }
  const uint8_t* row = p.old + (size_t)y * p.w;
  uint8_t* orow = p.out + (size_t)y * p.w;
  for (uint32_t x = x0; x < x1; ++x) {
    const uint8_t here = __ldg(row + x);
    uint8_t state = here & kRest;
    for (int d = 0; d < 6; ++d) {
      int sx = (int)x + sdx[d];
      if (sx < 0) sx += (int)p.w;
      if (sx >= (int)p.w) sx -= (int)p.w;
      state |= __ldg(srow[d] + sx) & (uint8_t)(1u << d);
    }
    uint8_t o;
    if (here & kSolid) {
      const uint8_t m = state & 0x3F;
      o = kSolid | (state & kRest) | (uint8_t)(((m << 3) | (m >> 3)) & 0x3F);
    } else {
      st = xorshift(st);
      const uint32_t r = (uint32_t)((st * kMul) >> 32);
      const uint32_t k = (uint32_t)(((uint64_t)r * p.stride) >> 32);
      o = table[state * p.stride + k];
    }
    orow[x] = o;
  }
}

// The inflow re-seed of the leftmost columns, one thread per row, each
// jumping the step's single generator to the row's first draw
// (src/lattice.rs:270-285, Equilibrium::sample at src/lattice.rs:102-115).
__global__ void __launch_bounds__(128) lgx_byte_inlet_kernel(const ByteInletArgs p) {
  __shared__ uint64_t jump[kJumps * 64];
  for (uint32_t i = threadIdx.x; i < kJumps * 64; i += blockDim.x) jump[i] = p.jump[i];
  __syncthreads();
  const uint32_t y = blockIdx.x * blockDim.x + threadIdx.x;
  if (y >= p.h) return;
  uint64_t st = jump_ahead(rng_seed(p.seed), p.row_off[y], jump);
  uint8_t* row = p.cells + (size_t)y * p.w;
  for (uint32_t x = 0; x < p.cols; ++x) {
    if (row[x] & kSolid) continue;
    row[x] = lgx::equilibrium_sample(p.t, p.rest != 0, st);
  }
}

// Host: the padded collision table (src/collision.rs:161-188).
void build_table(bool rest, std::vector<uint8_t>* data, uint32_t* stride) {
  static const int CX2[6] = {2, 1, -1, -2, -1, 1}, CY2[6] = {0, 1, 1, 0, -1, -1};
  const int n = rest ? 128 : 64;
  std::map<std::tuple<int, int, int>, std::vector<uint8_t>> groups;
  auto key = [&](int s) {
    int m = 0, x = 0, y = 0;
    for (int d = 0; d < 6; ++d)
      if (s >> d & 1) {
        ++m;
        x += CX2[d];
        y += CY2[d];
      }
    if (s & kRest) ++m;
    return std::make_tuple(m, x, y);
  };
  for (int s = 0; s < n; ++s) groups[key(s)].push_back((uint8_t)s);
  uint32_t st = 1;
  for (auto& kv : groups) {
    uint32_t a = st, b = (uint32_t)kv.second.size();
    while (b) {
      const uint32_t t = a % b;
      a = b;
      b = t;
    }
    st = st / a * (uint32_t)kv.second.size();
  }
  // Always 128 states: without rest particles a state with bit 6 set never
  // arises from the reference's own updates, and its rows here keep the state,
  // so no cell value can index past the table.
  data->assign((size_t)128 * st, 0);
  for (int s = 0; s < 128; ++s) {
    if (s >= n) {
      for (uint32_t k = 0; k < st; ++k) (*data)[(size_t)s * st + k] = (uint8_t)s;
      continue;
    }
    const auto& g = groups[key(s)];
    for (uint32_t k = 0; k < st; ++k) (*data)[(size_t)s * st + k] = g[k % g.size()];
  }
  *stride = st;
}

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

struct lgx_byte_lattice {
  int device = 0;
  cudaStream_t stream = nullptr;
  uint32_t w = 0, h = 0, threads = 1, band = 0, inlet_cols = 0, segs_per_row = 0;
  bool rest = true;
  float density = 0, ux = 0, uy = 0;
  uint64_t seed = 0, steps = 0;
  uint32_t thresh[7] = {};
  uint8_t* cells[2] = {nullptr, nullptr};
  int cur = 0;
  uint8_t* table = nullptr;
  uint32_t stride = 0;
  uint64_t* jump = nullptr;
  uint32_t* seg_off = nullptr;
  uint32_t* row_off = nullptr;
  // coarse-graining and counting go through the bitplane kernels
  lgx::Dims dm{};
  uint32_t* planes = nullptr;
  uint32_t* solid = nullptr;
  uint32_t* anysolid = nullptr;
  unsigned long long* counter = nullptr;
  bool has_field = false;
  uint32_t bx = 0, by = 0, bw = 0, bh = 0;
  float* field = nullptr;
  int32_t* sums = nullptr;
};

namespace {

void free_bytes(lgx_byte_lattice* L) {
  cudaSetDevice(L->device);
  if (L->stream) cudaStreamSynchronize(L->stream);
  void* ptrs[] = {L->cells[0], L->cells[1], L->table, L->jump, L->seg_off, L->row_off,
                  L->planes,   L->solid,    L->anysolid, L->counter, L->field, L->sums};
  for (void* p : ptrs) cudaFree(p);
  if (L->stream) cudaStreamDestroy(L->stream);
  delete L;
}

// Draw offsets of every segment and of every inflow row, from the obstacles
// in `cells` (host copy).
int build_offsets(lgx_byte_lattice* L, const uint8_t* cells) {
  const uint32_t w = L->w, h = L->h;
  std::vector<uint32_t> seg((size_t)h * L->segs_per_row), row(h, 0);
  uint64_t count = 0;
  for (uint32_t y = 0; y < h; ++y) {
    if (y % L->band == 0) count = 0;
    for (uint32_t s = 0; s < L->segs_per_row; ++s) {
      seg[(size_t)y * L->segs_per_row + s] = (uint32_t)count;
      const uint32_t x1 = std::min(w, (s + 1) * kSeg);
      for (uint32_t x = s * kSeg; x < x1; ++x) count += !(cells[(size_t)y * w + x] & kSolid);
    }
    if (count >= (1ull << 32)) {
      lgx::set_error("a band has more than 2^32 fluid cells");
      return LGX_ERR_ARG;
    }
  }
  const uint32_t per = L->rest ? 4u : 3u;
  uint64_t draws = 0;
  for (uint32_t y = 0; y < h; ++y) {
    row[y] = (uint32_t)draws;
    for (uint32_t x = 0; x < L->inlet_cols; ++x) draws += per * !(cells[(size_t)y * w + x] & kSolid);
  }
  LGX_CUDA(cudaMemcpyAsync(L->seg_off, seg.data(), seg.size() * 4, cudaMemcpyHostToDevice,
                           L->stream));
  LGX_CUDA(cudaMemcpyAsync(L->row_off, row.data(), row.size() * 4, cudaMemcpyHostToDevice,
                           L->stream));
  LGX_CUDA(cudaStreamSynchronize(L->stream));
  return LGX_OK;
}

}  // namespace

extern "C" {

int lgx_byte_create(size_t w, size_t h, float density, float ux, float uy, size_t inlet_cols,
                    int rest, size_t threads, uint64_t seed, lgx_byte_lattice** out) {
  if (!out) {
    lgx::set_error("null output");
    return LGX_ERR_ARG;
  }
  *out = nullptr;
  if (h % 2 != 0 || w <= 4 || h <= 4) {  // src/lattice.rs:137-138
    lgx::set_error("row count must be even, and the lattice larger than 4 x 4");
    return LGX_ERR_ARG;
  }
  if (w * h >= (1ull << 31)) {
    lgx::set_error("lattice too large for the byte path");
    return LGX_ERR_ARG;
  }
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    lgx::set_error("no CUDA device on this machine");
    return LGX_ERR_NO_DEVICE;
  }
  lgx_byte_lattice* L = new (std::nothrow) lgx_byte_lattice();
  if (!L) {
    lgx::set_error("out of host memory");
    return LGX_ERR_ALLOC;
  }
  cudaGetDevice(&L->device);
  L->w = (uint32_t)w;
  L->h = (uint32_t)h;
  L->rest = rest != 0;
  L->density = density;
  L->ux = ux;
  L->uy = uy;
  L->inlet_cols = (uint32_t)std::min(inlet_cols, w);
  L->threads = (uint32_t)std::max<size_t>(threads, 1);
  const uint32_t nthreads = std::min(L->threads, L->h);
  L->band = (L->h + nthreads - 1) / nthreads;  // src/lattice.rs:232-236
  L->segs_per_row = (L->w + kSeg - 1) / kSeg;
  L->seed = seed;
  lgx::equilibrium_thresholds(density, ux, uy, L->rest, L->thresh);
  L->dm = lgx::make_dims(L->w, L->h, 0);
  std::vector<uint8_t> table;
  build_table(L->rest, &table, &L->stride);
  std::vector<uint64_t> jumps = lgx::build_jumps();
  jumps.resize((size_t)kJumps * 64);
  const size_t cells = w * h, total = L->dm.total;
  cudaError_t e = cudaStreamCreateWithFlags(&L->stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaMalloc(&L->cells[0], cells);
  if (e == cudaSuccess) e = cudaMalloc(&L->cells[1], cells);
  if (e == cudaSuccess) e = cudaMalloc(&L->table, table.size());
  if (e == cudaSuccess) e = cudaMalloc(&L->jump, jumps.size() * 8);
  if (e == cudaSuccess) e = cudaMalloc(&L->seg_off, (size_t)L->h * L->segs_per_row * 4);
  if (e == cudaSuccess) e = cudaMalloc(&L->row_off, (size_t)L->h * 4);
  if (e == cudaSuccess) e = cudaMalloc(&L->planes, total * 7 * 4);
  if (e == cudaSuccess) e = cudaMalloc(&L->solid, total * 4);
  if (e == cudaSuccess) e = cudaMalloc(&L->anysolid, ((total + 31) / 32) * 4);
  if (e == cudaSuccess) e = cudaMalloc(&L->counter, 8);
  if (e == cudaSuccess) e = cudaMemset(L->cells[0], 0, cells);
  if (e == cudaSuccess) e = cudaMemcpy(L->table, table.data(), table.size(), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(L->jump, jumps.data(), jumps.size() * 8, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    const int rc = e == cudaErrorMemoryAllocation ? LGX_ERR_ALLOC : LGX_ERR_CUDA;
    lgx::set_error(std::string("lgx_byte_create: ") + cudaGetErrorString(e));
    free_bytes(L);
    return rc;
  }
  std::vector<uint8_t> zero(cells, 0);
  const int rc = build_offsets(L, zero.data());
  if (rc) {
    free_bytes(L);
    return rc;
  }
  *out = L;
  return LGX_OK;
}

int lgx_byte_destroy(lgx_byte_lattice* L) {
  if (L) free_bytes(L);
  return LGX_OK;
}

int lgx_byte_load(lgx_byte_lattice* L, const uint8_t* cells, size_t n) {
  if (!L || !cells || n != (size_t)L->w * L->h) {
    lgx::set_error("wrong number of cells");
    return LGX_ERR_ARG;
  }
  LGX_CUDA(cudaSetDevice(L->device));
  const int rc = build_offsets(L, cells);
  if (rc) return rc;
  LGX_CUDA(cudaMemcpyAsync(L->cells[L->cur], cells, n, cudaMemcpyHostToDevice, L->stream));
  LGX_CUDA(cudaStreamSynchronize(L->stream));
  return LGX_OK;
}

// Lattice::restart (src/lattice.rs:188-193).
int lgx_byte_restart(lgx_byte_lattice* L, const uint8_t* cells, size_t n, uint64_t seed) {
  const int rc = lgx_byte_load(L, cells, n);
  if (rc) return rc;
  L->seed = seed;
  L->steps = 0;
  return LGX_OK;
}

// Lattice::init_equilibrium (src/lattice.rs:197-208), on the device.  The
// obstacles stay where they are, so the draw offsets need no update.
int lgx_byte_init_equilibrium(lgx_byte_lattice* L) {
  if (!L) {
    lgx::set_error("null lattice");
    return LGX_ERR_ARG;
  }
  LGX_CUDA(cudaSetDevice(L->device));
  lgx::EqFill f{};
  f.cells = L->cells[L->cur];
  f.n = (size_t)L->w * L->h;
  f.seed = L->seed ^ 0xA5A51234ull;
  f.rest = L->rest;
  memcpy(f.thresh, L->thresh, sizeof(f.thresh));
  LGX_CUDA(lgx::launch_equilibrium_fill(f, L->stream));
  LGX_CUDA(cudaStreamSynchronize(L->stream));
  return LGX_OK;
}

int lgx_byte_store(lgx_byte_lattice* L, uint8_t* cells, size_t n) {
  if (!L || !cells || n != (size_t)L->w * L->h) {
    lgx::set_error("wrong number of cells");
    return LGX_ERR_ARG;
  }
  LGX_CUDA(cudaSetDevice(L->device));
  LGX_CUDA(cudaMemcpyAsync(cells, L->cells[L->cur], n, cudaMemcpyDeviceToHost, L->stream));
  LGX_CUDA(cudaStreamSynchronize(L->stream));
  return LGX_OK;
}

// Lattice::advance (src/lattice.rs:222-264).
int lgx_byte_advance(lgx_byte_lattice* L, uint64_t n) {
  if (!L) {
    lgx::set_error("null lattice");
    return LGX_ERR_ARG;
  }
  LGX_CUDA(cudaSetDevice(L->device));
  const uint32_t nseg = L->h * L->segs_per_row;
  for (uint64_t i = 0; i < n; ++i) {
    ByteStepArgs a;
    a.old = L->cells[L->cur];
    a.out = L->cells[L->cur ^ 1];
    a.table = L->table;
    a.stride = L->stride;
    a.w = L->w;
    a.h = L->h;
    a.band = L->band;
    a.segs_per_row = L->segs_per_row;
    a.seg_off = L->seg_off;
    a.jump = L->jump;
    a.base_seed = L->seed ^ (L->steps * 0x9E3779B97F4A7C15ull);
    lgx_byte_step_kernel<<<(nseg + 127) / 128, 128, 0, L->stream>>>(a);
    LGX_CUDA(cudaGetLastError());
    L->cur ^= 1;
    L->steps += 1;
    if (L->inlet_cols) {
      ByteInletArgs b;
      b.cells = L->cells[L->cur];
      b.w = L->w;
      b.h = L->h;
      b.cols = L->inlet_cols;
      b.row_off = L->row_off;
      b.jump = L->jump;
      b.seed = L->seed ^ (L->steps * 0xD1B54A32D192ED03ull);
      memcpy(b.t, L->thresh, sizeof(b.t));
      b.rest = L->rest ? 1 : 0;
      lgx_byte_inlet_kernel<<<(L->h + 127) / 128, 128, 0, L->stream>>>(b);
      LGX_CUDA(cudaGetLastError());
    }
  }
  LGX_CUDA(cudaStreamSynchronize(L->stream));
  return LGX_OK;
}

int lgx_byte_attach_field(lgx_byte_lattice* L, size_t bx, size_t by) {
  if (!L || bx == 0 || by == 0) {
    lgx::set_error("bad argument");
    return LGX_ERR_ARG;
  }
  LGX_CUDA(cudaSetDevice(L->device));
  cudaFree(L->field);
  cudaFree(L->sums);
  L->field = nullptr;
  L->sums = nullptr;
  L->bx = (uint32_t)bx;
  L->by = (uint32_t)by;
  L->bw = L->w / L->bx;
  L->bh = L->h / L->by;
  const size_t nb = std::max<size_t>((size_t)L->bw * L->bh, 1);
  LGX_CUDA(cudaMalloc(&L->field, nb * 16));
  LGX_CUDA(cudaMalloc(&L->sums, nb * 16));
  LGX_CUDA(cudaMemset(L->field, 0, nb * 16));
  LGX_CUDA(cudaMemset(L->sums, 0, nb * 16));
  L->has_field = true;
  return LGX_OK;
}

// Field::sample (src/render.rs:61-120) of the current cells.
int lgx_byte_sample_field(lgx_byte_lattice* L, float alpha) {
  if (!L || !L->has_field) {
    lgx::set_error("no field attached");
    return LGX_ERR_STATE;
  }
  LGX_CUDA(cudaSetDevice(L->device));
  LGX_CUDA(lgx::launch_pack(L->cells[L->cur], L->dm, L->planes, L->solid, L->anysolid, L->stream));
  lgx::SampleArgs sa;
  sa.a = L->planes;
  sa.solid = L->solid;
  sa.dm = L->dm;
  sa.bx = L->bx;
  sa.by = L->by;
  sa.bw = L->bw;
  sa.bh = L->bh;
  sa.alpha = alpha;
  const size_t nb = (size_t)L->bw * L->bh;
  sa.ux = L->field;
  sa.uy = L->field + nb;
  sa.rho = L->field + 2 * nb;
  sa.sol = L->field + 3 * nb;
  sa.sums = L->sums;
  LGX_CUDA(lgx::launch_sample(sa, L->stream));
  LGX_CUDA(cudaStreamSynchronize(L->stream));
  return LGX_OK;
}

int lgx_byte_read_field(lgx_byte_lattice* L, float* ux, float* uy, float* rho, float* sol,
                        size_t n_blocks) {
  if (!L || !L->has_field || n_blocks != (size_t)L->bw * L->bh) {
    lgx::set_error("no field attached, or block grid mismatch");
    return LGX_ERR_ARG;
  }
  LGX_CUDA(cudaSetDevice(L->device));
  float* dst[4] = {ux, uy, rho, sol};
  for (int i = 0; i < 4; ++i)
    if (dst[i] && n_blocks)
      LGX_CUDA(cudaMemcpyAsync(dst[i], L->field + i * n_blocks, n_blocks * 4,
                               cudaMemcpyDeviceToHost, L->stream));
  LGX_CUDA(cudaStreamSynchronize(L->stream));
  return LGX_OK;
}

// Lattice::total_particles (src/lattice.rs:299-312).
int lgx_byte_total_particles(lgx_byte_lattice* L, uint64_t* out) {
  if (!L || !out) {
    lgx::set_error("null argument");
    return LGX_ERR_ARG;
  }
  LGX_CUDA(cudaSetDevice(L->device));
  LGX_CUDA(lgx::launch_pack(L->cells[L->cur], L->dm, L->planes, L->solid, L->anysolid, L->stream));
  LGX_CUDA(lgx::launch_count(L->planes, L->dm, L->counter, L->stream));
  unsigned long long v = 0;
  LGX_CUDA(cudaMemcpyAsync(&v, L->counter, 8, cudaMemcpyDeviceToHost, L->stream));
  LGX_CUDA(cudaStreamSynchronize(L->stream));
  *out = v;
  return LGX_OK;
}

int lgx_byte_steps(lgx_byte_lattice* L, uint64_t* out) {
  if (!L || !out) {
    lgx::set_error("null argument");
    return LGX_ERR_ARG;
  }
  *out = L->steps;
  return LGX_OK;
}

}  // extern "C"
