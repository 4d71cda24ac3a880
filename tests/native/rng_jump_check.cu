// Host-only check of the generator jumps in lgx_rng.cuh: the characteristic
// polynomial found by Berlekamp-Massey, jump polynomials z^k mod P applied to
// a state (as the byte and fill kernels apply them through their tables), and
// the matrix jumps, all against stepping the generator k times.  Prints "ok"
// and exits 0, or names the first mismatch and exits 1.
#include <stdint.h>
#include <stdio.h>

#include "lgx_rng.cuh"

using namespace lgx;

static uint64_t apply_poly(uint64_t p, uint64_t x) {
  uint64_t r = 0;
  for (int j = 0; j < 64; ++j, x = xorshift(x))
    if (p >> j & 1) r ^= x;
  return r;
}

static uint64_t apply_matrices(const std::vector<uint64_t>& J, uint64_t x, uint64_t k) {
  for (int i = 0; k; ++i, k >>= 1) {
    if (!(k & 1)) continue;
    uint64_t r = 0;
    for (int j = 0; j < 64; ++j)
      if (x >> j & 1) r ^= J[(size_t)i * 64 + j];
    x = r;
  }
  return x;
}

int main() {
  const uint64_t q = rng_charpoly();
  if (!q) {
    printf("characteristic polynomial check failed\n");
    return 1;
  }
  const std::vector<uint64_t> J = build_jumps();
  const uint64_t seeds[3] = {rng_seed(0x5EED), rng_seed(12345), rng_seed(~0ull)};
  for (uint64_t x0 : seeds) {
    uint64_t serial = x0, p = 1;
    for (uint64_t k = 0; k <= 70000; ++k) {
      if (k % 997 == 0 || k < 200) {
        if (apply_poly(p, x0) != serial) {
          printf("jump polynomial differs at k = %llu\n", (unsigned long long)k);
          return 1;
        }
        if (apply_matrices(J, x0, k) != serial) {
          printf("matrix jump differs at k = %llu\n", (unsigned long long)k);
          return 1;
        }
      }
      serial = xorshift(serial);
      p = poly_mulz(p, q);
    }
  }
  // a long jump: 2^40 + 12345 steps by matrices equals the polynomial built by
  // squaring (z^(2^i) mod P from repeated doubling of exponents)
  const uint64_t k = (1ull << 40) + 12345;
  uint64_t pk = 1, zpow = 2;  // zpow = z^(2^i) mod P
  auto mulmod = [&](uint64_t a, uint64_t b) {  // a * b mod P, shift-and-add
    uint64_t r = 0;
    for (int i = 63; i >= 0; --i) {
      r = poly_mulz(r, q);
      if (b >> i & 1) r ^= a;
    }
    return r;
  };
  for (uint64_t e = k; e; e >>= 1) {
    if (e & 1) pk = mulmod(pk, zpow);
    zpow = mulmod(zpow, zpow);
  }
  if (apply_poly(pk, seeds[0]) != apply_matrices(J, seeds[0], k)) {
    printf("long jump differs\n");
    return 1;
  }
  printf("ok\n");
  return 0;
}
