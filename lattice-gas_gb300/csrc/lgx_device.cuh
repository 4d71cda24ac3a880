// lgx_device.cuh -- device-side building blocks of the bitplane step.
//
// Layout in HBM (one lattice): seven planes of 32-cell words, plane-major,
// plane d at d * total + y * wpr + j, wpr = ceil(w / 32), bit k of word j is
// column 32 j + k (the reference's layout, src/gpu.rs:453-476 and 586-603).
// The solid plane lives on its own (never ping-pongs) with a one-bit-per-word
// summary `anysolid` so the step skips the solid load on almost every word.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "generated/collide.cuh"

namespace lgx {

constexpr uint32_t kGolden32 = 0x9e3779b9u;
constexpr uint64_t kGolden64 = 0x9E3779B97F4A7C15ull;

// Per-step seed of the counter-based draws: the low 32 bits of
// seed ^ steps * 0x9E3779B97F4A7C15 with `steps` counted before the step
// (src/gpu.rs:555).
__host__ __device__ __forceinline__ uint32_t step_seed32(uint64_t seed, uint64_t steps) {
  return (uint32_t)(seed ^ (steps * kGolden64));
}

// The stateless avalanche hash (src/gpu.rs:147-151).
__host__ __device__ __forceinline__ uint32_t mix(uint32_t x) {
  x ^= x >> 16;
  x *= 0x7feb352du;
  x ^= x >> 15;
  x *= 0x846ca68bu;
  x ^= x >> 16;
  return x;
}

// Selectors for the collision of one word: a fair bit, a one-hot choice of
// three and a one-hot choice of five by rejection sampling, 19 hashes in one
// chain (src/gpu.rs:157-180).  A lane left unresolved keeps its state.  The
// one-hot words come from the generated lgx_selectors (nested form, mapped to
// lop3).
struct Draws {
  uint32_t s2;
  uint32_t s3[3];
  uint32_t s5[5];
};

// The chain r_{k+1} = mix(r_k) for k = 0..18, r_{-1} = key.  The hash both
// begins and ends with x ^= x >> 16, and that map is an involution (the high
// half is unchanged and the low half is xored with it twice), so in the
// conjugated variable u_k = r_k ^ (r_k >> 16) the chain is
//     u_{k+1} = M2(S15(M1(u_k))),   M1 = *0x7feb352d, S15 = ^(>>15), M2 = *0x846ca68b
// and each output is recovered as r_k = u_k ^ (u_k >> 16).  Same values, two
// fewer logic instructions per hash.
__host__ __device__ __forceinline__ Draws draws(uint32_t key) {
  Draws d;
  uint32_t r[18];
  uint32_t u = key ^ (key >> 16);
  u *= 0x7feb352du;
  u ^= u >> 15;
  u *= 0x846ca68bu;
  d.s2 = u ^ (u >> 16);
#pragma unroll
  for (int i = 0; i < 18; ++i) {
    u *= 0x7feb352du;
    u ^= u >> 15;
    u *= 0x846ca68bu;
    r[i] = u ^ (u >> 16);
  }
  lgx_selectors(r, d.s3, d.s5);
  return d;
}

// A word of independent Bernoulli(t / 2^24) bits, reading the threshold from
// its least significant bit up; `r` chains across calls.  t == 0 and
// t >= 2^24 return without advancing the chain (src/gpu.rs:189-198).
__host__ __device__ __forceinline__ uint32_t bernoulli(uint32_t t, uint32_t& r) {
  if (t == 0u) return 0u;
  if (t >= (1u << 24)) return 0xffffffffu;
  uint32_t x = 0u;
  for (uint32_t j = 0; j < 24u; ++j) {
    r = mix(r);
    x = ((t >> j) & 1u) ? (r | x) : (r & x);
  }
  return x;
}

template <bool REST>
__device__ __forceinline__ void collide(const uint32_t n[7], const Draws& s, uint32_t o[7]) {
  if (REST)
    lgx_collide_rest(n, s.s2, s.s3, s.s5, o);
  else
    lgx_collide_norest(n, s.s2, s.s3, s.s5, o);
}

// Bounce-back on obstacle sites: every particle leaves the way it came and
// nothing collides (src/gpu.rs:284-291).
__device__ __forceinline__ void walls(const uint32_t n[7], const uint32_t o[7], uint32_t sm,
                                      uint32_t res[7]) {
#pragma unroll
  for (int d = 0; d < 6; ++d) res[d] = (sm & n[(d + 3) % 6]) | (~sm & o[d]);
  res[6] = (sm & n[6]) | (~sm & o[6]);
}

}  // namespace lgx
