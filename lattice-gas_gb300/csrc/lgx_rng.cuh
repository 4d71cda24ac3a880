// lgx_rng.cuh -- the reference's xorshift64* generator on the device, with
// jump-ahead.
//
// Rng::new scrambles the seed splitmix-style and steps x ^= x << 13,
// x ^= x >> 7, x ^= x << 17, returning x * 0x2545F4914F6CDD1D (src/rng.rs:8-34).
// The state update is linear over GF(2): x -> M x, so k steps are M^k x.  With
// the columns of M^(2^i) precomputed on the host, a jump of k steps is one
// matrix-vector product per set bit of k, each the xor of the columns picked
// by the state's set bits.
#pragma once

#include <stdint.h>

#include <vector>

namespace lgx {

constexpr int kJumpBits = 64;  // M^(2^i) for i < 64: any 64-bit jump

__host__ __device__ __forceinline__ uint64_t rng_seed(uint64_t seed) {
  uint64_t s = seed ^ 0x9E3779B97F4A7C15ull;
  s = (s ^ (s >> 30)) * 0xBF58476D1CE4E5B9ull;
  s = (s ^ (s >> 27)) * 0x94D049BB133111EBull;
  return (s ^ (s >> 31)) | 1ull;
}

__host__ __device__ __forceinline__ uint64_t xorshift(uint64_t x) {
  x ^= x << 13;
  x ^= x >> 7;
  x ^= x << 17;
  return x;
}

constexpr uint64_t kRngMul = 0x2545F4914F6CDD1Dull;

// x <- M^k x, with jump[i * 64 + j] the j-th column of M^(2^i).
__device__ __forceinline__ uint64_t jump_ahead(uint64_t x, uint64_t k, const uint64_t* jump) {
  for (int i = 0; k; ++i, k >>= 1) {
    if (!(k & 1u)) continue;
    const uint64_t* col = jump + i * 64;
    uint64_t r = 0, v = x;
    while (v) {
      const int j = __ffsll((long long)v) - 1;
      r ^= col[j];
      v &= v - 1;
    }
    x = r;
  }
  return x;
}

// Host: columns of M^(2^i), i < kJumpBits.
inline std::vector<uint64_t> build_jumps() {
  auto apply = [](const uint64_t* cols, uint64_t v) {
    uint64_t r = 0;
    for (int j = 0; j < 64; ++j)
      if (v >> j & 1) r ^= cols[j];
    return r;
  };
  std::vector<uint64_t> J((size_t)kJumpBits * 64);
  for (int j = 0; j < 64; ++j) J[j] = xorshift(1ull << j);
  for (int i = 1; i < kJumpBits; ++i)
    for (int j = 0; j < 64; ++j)
      J[(size_t)i * 64 + j] = apply(&J[(size_t)(i - 1) * 64], J[(size_t)(i - 1) * 64 + j]);
  return J;
}

// One cell from the equilibrium thresholds t[0..6]: three generator steps give
// two 24-bit samples each (bits 40..64 and 16..40), a fourth the rest particle
// (src/lattice.rs:102-115).  Returns the cell byte.
__device__ __forceinline__ uint8_t equilibrium_sample(const uint32_t t[7], bool rest,
                                                      uint64_t& st) {
  uint8_t s = 0;
#pragma unroll
  for (int d = 0; d < 6; d += 2) {
    st = xorshift(st);
    const uint64_t v = st * kRngMul;
    s |= (uint8_t)(((uint32_t)(v >> 40) < t[d]) << d);
    s |= (uint8_t)(((((uint32_t)(v >> 16)) & 0xFFFFFFu) < t[d + 1]) << (d + 1));
  }
  if (rest) {
    st = xorshift(st);
    if ((uint32_t)((st * kRngMul) >> 40) < t[6]) s |= 0x40;
  }
  return s;
}

}  // namespace lgx
