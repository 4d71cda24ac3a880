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

// Jump polynomials (Haramoto, Matsumoto, L'Ecuyer, Panneton and Nishimura,
// "Efficient jump ahead for F2-linear random number generators", 2008).  With
// P(z) = z^64 + q(z) the characteristic polynomial of M, P(M) = 0, so
// M^k = p_k(M) with p_k = z^k mod P, and M^k x = xor of M^j x over the set
// coefficients j of p_k.  When many jumps start from the same x (every segment
// of one band), the 64 states M^j x are shared and folded into tables over
// B-bit chunks of p_k, T[c][n] = xor over the set bits b of n of M^(Bc+b) x;
// a jump is then 64/B table lookups, and p_k is one 64-bit word.
//
// Host: q, the low 64 coefficients of P, from the Berlekamp-Massey algorithm
// (Massey, 1969) over one state bit's sequence, checked on every basis vector
// (M^64 e = q(M) e).  Returns 0 if the check fails.
inline uint64_t rng_charpoly() {
  constexpr int N = 128;
  int s[N];
  uint64_t x = 1;
  for (int t = 0; t < N; ++t, x = xorshift(x)) s[t] = (int)(x & 1);
  int C[N + 1] = {1}, B[N + 1] = {1}, T[N + 1];
  int L = 0, m = 1;
  for (int n = 0; n < N; ++n) {
    int d = s[n];
    for (int i = 1; i <= L; ++i) d ^= C[i] & s[n - i];
    if (!d) {
      ++m;
      continue;
    }
    for (int i = 0; i <= N; ++i) T[i] = C[i];
    for (int i = 0; i + m <= N; ++i) C[i + m] ^= B[i];
    if (2 * L <= n) {
      L = n + 1 - L;
      for (int i = 0; i <= N; ++i) B[i] = T[i];
      m = 1;
    } else {
      ++m;
    }
  }
  if (L != 64) return 0;
  uint64_t q = 0;
  for (int j = 0; j < 64; ++j) q |= (uint64_t)C[64 - j] << j;
  for (int e = 0; e < 64; ++e) {
    uint64_t v = 1ull << e, acc = 0;
    for (int j = 0; j < 64; ++j, v = xorshift(v))
      if (q >> j & 1) acc ^= v;
    if (acc != v) return 0;
  }
  return q;
}

// p * z mod P: one more generator step.
__host__ __device__ __forceinline__ uint64_t poly_mulz(uint64_t p, uint64_t q) {
  return (p << 1) ^ ((p >> 63) ? q : 0ull);
}

// Entry e = c * 2^B + n of the chunk tables of the states M^j x, j < 64, held
// in `states`.
template <int B>
__device__ __forceinline__ uint64_t jump_entry(const uint64_t* states, uint32_t e) {
  const uint64_t* s = states + (e >> B) * B;
  uint64_t v = 0;
#pragma unroll
  for (int b = 0; b < B; ++b)
    if (e >> b & 1u) v ^= s[b];
  return v;
}

// M^k x for p = z^k mod P, from the chunk tables of x.
template <int B>
__device__ __forceinline__ uint64_t jump_poly(uint64_t p, const uint64_t* tab) {
  uint64_t r = 0;
#pragma unroll
  for (int c = 0; c < 64 / B; ++c)
    r ^= tab[(c << B) + (uint32_t)((p >> (B * c)) & ((1u << B) - 1))];
  return r;
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
