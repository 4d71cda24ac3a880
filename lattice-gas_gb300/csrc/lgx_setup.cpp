// lgx_setup.cpp -- host-side lattice setup: the reference's generator,
// equilibrium thresholds and sampler, obstacles and the shear-wave start.
//
// These produce the byte cells a caller loads into a lattice; they mirror
// src/rng.rs, src/lattice.rs:41-116 and 188-220, src/hex.rs:52-55 and
// src/transport.rs:188-200.  All f32 arithmetic is written one operation per
// statement and the file is compiled with -ffp-contract=off, so nothing is
// fused: the reference's Rust never contracts a multiply-add.
#include <math.h>
#include <string.h>

#include <atomic>
#include <chrono>

#include <cuda_runtime.h>

#include "../../include/lgx.h"
#include "lgx_internal.hpp"

namespace lgx {
namespace {

constexpr float kSqrt3_2 = 0.8660254f;

}  // namespace

// Moments::velocity (src/moments.rs:91-97), in the reference's f32 order:
// (px2 as f32 * 0.5) / m and (py2 as f32 * SQRT3_2) / m with m = mass as f32.
void moments_velocity(int64_t mass, int64_t px2, int64_t py2, float* ux, float* uy) {
  if (mass == 0) {
    *ux = 0.0f;
    *uy = 0.0f;
    return;
  }
  const float m = (float)mass;
  *ux = (float)px2 * 0.5f / m;
  *uy = (float)py2 * kSqrt3_2 / m;
}

unsigned long long* host_result_words() {
  thread_local unsigned long long* words = nullptr;
  thread_local bool tried = false;
  if (!tried) {
    tried = true;
    void* p = nullptr;
    if (cudaHostAlloc(&p, 8 * sizeof(unsigned long long),
                      cudaHostAllocPortable | cudaHostAllocMapped) == cudaSuccess)
      words = (unsigned long long*)p;
    else
      cudaGetLastError();
  }
  return words;
}

unsigned long long host_result_seq() {
  thread_local unsigned long long seq = 0;
  return ++seq;
}

cudaError_t host_result_wait(unsigned long long seq, cudaStream_t st) {
  volatile unsigned long long* flag = host_result_words() + 7;
  const auto t0 = std::chrono::steady_clock::now();
  for (unsigned n = 0;; ++n) {
    if (*flag == seq) {
      std::atomic_thread_fence(std::memory_order_acquire);  // the results were written first
      return cudaSuccess;
    }
    if ((n & 1023u) == 1023u &&
        std::chrono::steady_clock::now() - t0 > std::chrono::milliseconds(20))
      break;
  }
  return cudaStreamSynchronize(st);
}

unsigned long long* host_result_device() {
  thread_local unsigned long long* dev = nullptr;
  thread_local bool tried = false;
  if (!tried) {
    tried = true;
    unsigned long long* h = host_result_words();
    void* d = nullptr;
    if (h && cudaHostGetDevicePointer(&d, h, 0) == cudaSuccess)
      dev = (unsigned long long*)d;
    else
      cudaGetLastError();
  }
  return dev;
}

namespace {
constexpr float kCXF[6] = {1.0f, 0.5f, -0.5f, -1.0f, -0.5f, 0.5f};
constexpr float kCYF[6] = {0.0f, kSqrt3_2, kSqrt3_2, 0.0f, -kSqrt3_2, -kSqrt3_2};
constexpr uint8_t kSolid = 0x80;
constexpr uint8_t kRest = 0x40;

// xorshift64* with a splitmix-style scramble of the seed (src/rng.rs:8-34).
struct Rng {
  uint64_t s;
  explicit Rng(uint64_t seed) {
    uint64_t x = seed ^ 0x9E3779B97F4A7C15ull;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    s = (x ^ (x >> 31)) | 1ull;
  }
  uint64_t next() {
    uint64_t x = s;
    x ^= x << 13;
    x ^= x >> 7;
    x ^= x << 17;
    s = x;
    return x * 0x2545F4914F6CDD1Dull;
  }
};

// ceil(p * 2^24) clamped to [0, 2^24]; NaN -> 0 (src/lattice.rs:59-69).
uint32_t threshold(float p) {
  const float one = 16777216.0f;
  const float t = ceilf(p * one);
  if (t >= one) return 1u << 24;
  if (t > 0.0f) return (uint32_t)t;
  return 0u;
}

struct Equilibrium {
  uint32_t t[7];
  bool rest;
  Equilibrium(float density, float ux, float uy, bool rest_) : rest(rest_) {
    equilibrium_thresholds(density, ux, uy, rest_, t);
  }
  // Three generator steps give two 24-bit samples each (bits 40..64 and
  // 16..40), one more gives the rest particle (src/lattice.rs:102-115).
  uint8_t sample(Rng& r) const {
    uint8_t s = 0;
    for (int d = 0; d < 6; d += 2) {
      const uint64_t v = r.next();
      s |= (uint8_t)(((uint32_t)(v >> 40) < t[d]) << d);
      s |= (uint8_t)(((((uint32_t)(v >> 16)) & 0xFFFFFFu) < t[d + 1]) << (d + 1));
    }
    if (rest && (uint32_t)(r.next() >> 40) < t[6]) s |= kRest;
    return s;
  }
};

void site_position(size_t x, size_t y, float* px, float* py) {
  *px = (float)x + ((y & 1) ? 0.5f : 0.0f);
  *py = (float)y * kSqrt3_2;
}

// Half-open index ranges that contain every site whose position can fall in
// [lo, hi] (rows: y * sqrt(3)/2; columns: x or x + 1/2), widened by two sites.
// Non-finite bounds fall back to the whole axis.
void row_range(float lo, float hi, size_t h, size_t* a, size_t* b) {
  if (!(isfinite(lo) && isfinite(hi))) { *a = 0; *b = h; return; }
  const double l = floor((double)lo / 0.8660254) - 2.0, u = ceil((double)hi / 0.8660254) + 3.0;
  *a = l <= 0.0 ? 0 : (l >= (double)h ? h : (size_t)l);
  *b = u <= 0.0 ? 0 : (u >= (double)h ? h : (size_t)u);
}
void col_range(float lo, float hi, size_t w, size_t* a, size_t* b) {
  if (!(isfinite(lo) && isfinite(hi))) { *a = 0; *b = w; return; }
  const double l = floor((double)lo) - 2.0, u = ceil((double)hi) + 3.0;
  *a = l <= 0.0 ? 0 : (l >= (double)w ? w : (size_t)l);
  *b = u <= 0.0 ? 0 : (u >= (double)w ? w : (size_t)u);
}

}  // namespace

void equilibrium_thresholds(float density, float ux, float uy, bool rest, uint32_t out[7]) {
  const float bias = rest ? 2.0f * 7.0f / 6.0f : 2.0f;
  for (int d = 0; d < 6; ++d) {
    const float a = kCXF[d] * ux;
    const float b = kCYF[d] * uy;
    const float s = a + b;
    const float q = bias * s;
    const float r = 1.0f + q;
    out[d] = threshold(density * r);
  }
  out[6] = rest ? threshold(density) : 0u;
}

}  // namespace lgx

extern "C" {

int lgx_equilibrium_thresholds(float density, float ux, float uy, int rest, uint32_t out[7]) {
  if (!out) {
    lgx::set_error("lgx_equilibrium_thresholds: null output");
    return LGX_ERR_ARG;
  }
  lgx::equilibrium_thresholds(density, ux, uy, rest != 0, out);
  return LGX_OK;
}

int lgx_cells_init_equilibrium(uint8_t* cells, size_t n, float density, float ux, float uy,
                               int rest, uint64_t seed) {
  if (!cells && n) {
    lgx::set_error("lgx_cells_init_equilibrium: null cells");
    return LGX_ERR_ARG;
  }
  lgx::Rng rng(seed ^ 0xA5A51234ull);
  const lgx::Equilibrium eq(density, ux, uy, rest != 0);
  for (size_t i = 0; i < n; ++i)
    cells[i] = (cells[i] & lgx::kSolid) ? lgx::kSolid : eq.sample(rng);
  return LGX_OK;
}

int lgx_cells_add_box(uint8_t* cells, size_t w, size_t h, float x0, float x1, float y0, float y1,
                      int strict) {
  if (!cells && w * h) {
    lgx::set_error("lgx_cells_add_box: null cells");
    return LGX_ERR_ARG;
  }
  // The predicate is evaluated on every site the reference's add_solid would
  // test that can possibly satisfy it: a bounding range with two sites of
  // margin, so the f32 comparisons decide exactly the same sites.
  size_t ya, yb, xa, xb;
  lgx::row_range(y0, y1, h, &ya, &yb);
  lgx::col_range(x0, x1, w, &xa, &xb);
  for (size_t y = ya; y < yb; ++y)
    for (size_t x = xa; x < xb; ++x) {
      float px, py;
      lgx::site_position(x, y, &px, &py);
      const bool in = strict ? (px > x0 && px < x1 && py > y0 && py < y1)
                             : (px >= x0 && px <= x1 && py >= y0 && py <= y1);
      if (in) cells[y * w + x] = lgx::kSolid;
    }
  return LGX_OK;
}

int lgx_cells_add_circle(uint8_t* cells, size_t w, size_t h, float cx, float cy, float r) {
  if (!cells && w * h) {
    lgx::set_error("lgx_cells_add_circle: null cells");
    return LGX_ERR_ARG;
  }
  const float rr = r * r;
  size_t ya, yb, xa, xb;
  lgx::row_range(cy - fabsf(r), cy + fabsf(r), h, &ya, &yb);
  lgx::col_range(cx - fabsf(r), cx + fabsf(r), w, &xa, &xb);
  for (size_t y = ya; y < yb; ++y)
    for (size_t x = xa; x < xb; ++x) {
      float px, py;
      lgx::site_position(x, y, &px, &py);
      const float dx = px - cx;
      const float dy = py - cy;
      const float a = dx * dx;
      const float b = dy * dy;
      if (a + b <= rr) cells[y * w + x] = lgx::kSolid;
    }
  return LGX_OK;
}

int lgx_cells_shear_wave(uint8_t* cells, size_t w, size_t h, float density, const float* ux_row,
                         int rest, uint64_t rng_seed) {
  if ((!cells || !ux_row) && w * h) {
    lgx::set_error("lgx_cells_shear_wave: null argument");
    return LGX_ERR_ARG;
  }
  lgx::Rng rng(rng_seed);
  for (size_t y = 0; y < h; ++y) {
    const lgx::Equilibrium eq(density, ux_row[y], 0.0f, rest != 0);
    for (size_t x = 0; x < w; ++x) cells[y * w + x] = eq.sample(rng);
  }
  return LGX_OK;
}

}  // extern "C"
