// Generated by lattice-gas_gb300/gen/collide_gen.py -- do not edit.
//
// The FHP collision rule as three-input lookup tables, one lop3.b32 each.
// Inputs: seven planes n[0..6] (six directions, then rest), the fair bit s2,
// one-hot selectors s3[0..2] and s5[0..4].  Output: seven planes o[0..6].
// Semantics (class pick by selector) follow the reference's known-answer
// specification, src/gpu.rs:799-817; classes come from src/collision.rs:62-69.
#pragma once
#include <stdint.h>

#ifndef LGX_HD_INLINE
#if defined(__CUDACC__)
#define LGX_HD_INLINE __host__ __device__ __forceinline__
#else
#define LGX_HD_INLINE static inline
#endif
#endif

#define LGX_LOP3(a, b, c, lut) lgx_lop3_host((a), (b), (c), (lut))

// Host evaluation of a three-input table: bit i of lut is f(a_i, b_i, c_i)
// with i = 4a + 2b + c (the lop3 convention: a = 0xF0, b = 0xCC, c = 0xAA).
static inline uint32_t lgx_lop3_host(uint32_t a, uint32_t b, uint32_t c, uint32_t lut) {
  uint32_t r = 0;
  for (int i = 0; i < 8; ++i) {
    if ((lut >> i) & 1u) {
      uint32_t ta = (i & 4) ? a : ~a, tb = (i & 2) ? b : ~b, tc = (i & 1) ? c : ~c;
      r |= ta & tb & tc;
    }
  }
  return r;
}


#if defined(__CUDA_ARCH__)
__device__ __forceinline__ uint32_t lgx_lop3_0x01(uint32_t a, uint32_t b, uint32_t c) {
  uint32_t r;
  asm("lop3.b32 %0, %1, %2, %3, 0x01;" : "=r"(r) : "r"(a), "r"(b), "r"(c));
  return r;
}
__device__ __forceinline__ uint32_t lgx_lop3_0x02(uint32_t a, uint32_t b, uint32_t c) {
  uint32_t r;
  asm("lop3.b32 %0, %1, %2, %3, 0x02;" : "=r"(r) : "r"(a), "r"(b), "r"(c));
  return r;
}
__device__ __forceinline__ uint32_t lgx_lop3_0x03(uint32_t a, uint32_t b, uint32_t c) {
  uint32_t r;
  asm("lop3.b32 %0, %1, %2, %3, 0x03;" : "=r"(r) : "r"(a), "r"(b), "r"(c));
  return r;
}
__device__ __forceinline__ uint32_t lgx_lop3_0x04(uint32_t a, uint32_t b, uint32_t c) {
  uint32_t r;
  asm("lop3.b32 %0, %1, %2, %3, 0x04;" : "=r"(r) : "r"(a), "r"(b), "r"(c));
  return r;
}
__device__ __forceinline__ uint32_t lgx_lop3_0x07(uint32_t a, uint32_t b, uint32_t c) {
  uint32_t r;
  asm("lop3.b32 %0, %1, %2, %3, 0x07;" : "=r"(r) : "r"(a), "r"(b), "r"(c));
  return r;
}
__device__ __forceinline__ uint32_t lgx_lop3_0x08(uint32_t a, uint32_t b, uint32_t c) {
  uint32_t r;
  asm("lop3.b32 %0, %1, %2, %3, 0x08;" : "=r"(r) : "r"(a), "r"(b), "r"(c));
  return r;
}
__device__ __forceinline__ uint32_t lgx_lop3_0x0c(uint32_t a, uint32_t b, uint32_t c) {
  uint32_t r;
  asm("lop3.b32 %0, %1, %2, %3, 0x0c;" : "=r"(r) : "r"(a), "r"(b), "r"(c));
  return r;
}
__device__ __forceinline__ uint32_t lgx_lop3_0x0f(uint32_t a, uint32_t b, uint32_t c) {
  uint32_t r;
  asm("lop3.b32 %0, %1, %2, %3, 0x0f;" : "=r"(r) : "r"(a), "r"(b), "r"(c));
  return r;
}
__device__ __forceinline__ uint32_t lgx_lop3_0x10(uint32_t a, uint32_t b, uint32_t c) {
  uint32_t r;
  asm("lop3.b32 %0, %1, %2, %3, 0x10;" : "=r"(r) : "r"(a), "r"(b), "r"(c));
  return r;
}
__device__ __forceinline__ uint32_t lgx_lop3_0x13(uint32_t a, uint32_t b, uint32_t c) {
  uint32_t r;
  asm("lop3.b32 %0, %1, %2, %3, 0x13;" : "=r"(r) : "r"(a), "r"(b), "r"(c));
  return r;
}
__device__ __forceinline__ uint32_t lgx_lop3_0x15(uint32_t a, uint32_t b, uint32_t c) {
  uint32_t r;
  asm("lop3.b32 %0, %1, %2, %3, 0x15;" : "=r"(r) : "r"(a), "r"(b), "r"(c));
  return r;
}
__device__ __forceinline__ uint32_t lgx_lop3_0x17(uint32_t a, uint32_t b, uint32_t c) {
  uint32_t r;
  asm("lop3.b32 %0, %1, %2, %3, 0x17;" : "=r"(r) : "r"(a), "r"(b), "r"(c));
  return r;
}
__device__ __forceinline__ uint32_t lgx_lop3_0x18(uint32_t a, uint32_t b, uint32_t c) {
  uint32_t r;
  asm("lop3.b32 %0, %1, %2, %3, 0x18;" : "=r"(r) : "r"(a), "r"(b), "r"(c));
  return r;
}
__device__ __forceinline__ uint32_t lgx_lop3_0x1b(uint32_t a, uint32_t b, uint32_t c) {
  uint32_t r;
  asm("lop3.b32 %0, %1, %2, %3, 0x1b;" : "=r"(r) : "r"(a), "r"(b), "r"(c));
  return r;
}
__device__ __forceinline__ uint32_t lgx_lop3_0x1f(uint32_t a, uint32_t b, uint32_t c) {
  uint32_t r;
  asm("lop3.b32 %0, %1, %2, %3, 0x1f;" : "=r"(r) : "r"(a), "r"(b), "r"(c));
  return r;
}
__device__ __forceinline__ uint32_t lgx_lop3_0x20(uint32_t a, uint32_t b, uint32_t c) {
  uint32_t r;
  asm("lop3.b32 %0, %1, %2, %3, 0x20;" : "=r"(r) : "r"(a), "r"(b), "r"(c));
  return r;
}
__device__ __forceinline__ uint32_t lgx_lop3_0x24(uint32_t a, uint32_t b, uint32_t c) {
  uint32_t r;
  asm("lop3.b32 %0, %1, %2, %3, 0x24;" : "=r"(r) : "r"(a), "r"(b), "r"(c));
  return r;
}
__device__ __forceinline__ uint32_t lgx_lop3_0x27(uint32_t a, uint32_t b, uint32_t c) {
  uint32_t r;
  asm("lop3.b32 %0, %1, %2, %3, 0x27;" : "=r"(r) : "r"(a), "r"(b), "r"(c));
  return r;
}
__device__ __forceinline__ uint32_t lgx_lop3_0x2a(uint32_t a, uint32_t b, uint32_t c) {
  uint32_t r;
  asm("lop3.b32 %0, %1, %2, %3, 0x2a;" : "=r"(r) : "r"(a), "r"(b), "r"(c));
  return r;
}
__device__ __forceinline__ uint32_t lgx_lop3_0x2e(uint32_t a, uint32_t b, uint32_t c) {
  uint32_t r;
  asm("lop3.b32 %0, %1, %2, %3, 0x2e;" : "=r"(r) : "r"(a), "r"(b), "r"(c));
  return r;
}
__device__ __forceinline__ uint32_t lgx_lop3_0x2f(uint32_t a, uint32_t b, uint32_t c) {
  uint32_t r;
  asm("lop3.b32 %0, %1, %2, %3, 0x2f;" : "=r"(r) : "r"(a), "r"(b), "r"(c));
  return r;
}
__device__ __forceinline__ uint32_t lgx_lop3_0x30(uint32_t a, uint32_t b, uint32_t c) {
  uint32_t r;
  asm("lop3.b32 %0, %1, %2, %3, 0x30;" : "=r"(r) : "r"(a), "r"(b), "r"(c));
  return r;
}
__device__ __forceinline__ uint32_t lgx_lop3_0x31(uint32_t a, uint32_t b, uint32_t c) {
  uint32_t r;
  asm("lop3.b32 %0, %1, %2, %3, 0x31;" : "=r"(r) : "r"(a), "r"(b), "r"(c));
  return r;
}
__device__ __forceinline__ uint32_t lgx_lop3_0x35(uint32_t a, uint32_t b, uint32_t c) {
  uint32_t r;
  asm("lop3.b32 %0, %1, %2, %3, 0x35;" : "=r"(r) : "r"(a), "r"(b), "r"(c));
  return r;
}
__device__ __forceinline__ uint32_t lgx_lop3_0x3c(uint32_t a, uint32_t b, uint32_t c) {
  uint32_t r;
  asm("lop3.b32 %0, %1, %2, %3, 0x3c;" : "=r"(r) : "r"(a), "r"(b), "r"(c));
  return r;
}
__device__ __forceinline__ uint32_t lgx_lop3_0x40(uint32_t a, uint32_t b, uint32_t c) {
  uint32_t r;
  asm("lop3.b32 %0, %1, %2, %3, 0x40;" : "=r"(r) : "r"(a), "r"(b), "r"(c));
  return r;
}
__device__ __forceinline__ uint32_t lgx_lop3_0x42(uint32_t a, uint32_t b, uint32_t c) {
  uint32_t r;
  asm("lop3.b32 %0, %1, %2, %3, 0x42;" : "=r"(r) : "r"(a), "r"(b), "r"(c));
  return r;
}
__device__ __forceinline__ uint32_t lgx_lop3_0x45(uint32_t a, uint32_t b, uint32_t c) {
  uint32_t r;
  asm("lop3.b32 %0, %1, %2, %3, 0x45;" : "=r"(r) : "r"(a), "r"(b), "r"(c));
  return r;
}
__device__ __forceinline__ uint32_t lgx_lop3_0x4f(uint32_t a, uint32_t b, uint32_t c) {
  uint32_t r;
  asm("lop3.b32 %0, %1, %2, %3, 0x4f;" : "=r"(r) : "r"(a), "r"(b), "r"(c));
  return r;
}
__device__ __forceinline__ uint32_t lgx_lop3_0x50(uint32_t a, uint32_t b, uint32_t c) {
  uint32_t r;
  asm("lop3.b32 %0, %1, %2, %3, 0x50;" : "=r"(r) : "r"(a), "r"(b), "r"(c));
  return r;
}
__device__ __forceinline__ uint32_t lgx_lop3_0x54(uint32_t a, uint32_t b, uint32_t c) {
  uint32_t r;
  asm("lop3.b32 %0, %1, %2, %3, 0x54;" : "=r"(r) : "r"(a), "r"(b), "r"(c));
  return r;
}
__device__ __forceinline__ uint32_t lgx_lop3_0x69(uint32_t a, uint32_t b, uint32_t c) {
  uint32_t r;
  asm("lop3.b32 %0, %1, %2, %3, 0x69;" : "=r"(r) : "r"(a), "r"(b), "r"(c));
  return r;
}
__device__ __forceinline__ uint32_t lgx_lop3_0x70(uint32_t a, uint32_t b, uint32_t c) {
  uint32_t r;
  asm("lop3.b32 %0, %1, %2, %3, 0x70;" : "=r"(r) : "r"(a), "r"(b), "r"(c));
  return r;
}
__device__ __forceinline__ uint32_t lgx_lop3_0x73(uint32_t a, uint32_t b, uint32_t c) {
  uint32_t r;
  asm("lop3.b32 %0, %1, %2, %3, 0x73;" : "=r"(r) : "r"(a), "r"(b), "r"(c));
  return r;
}
__device__ __forceinline__ uint32_t lgx_lop3_0x7c(uint32_t a, uint32_t b, uint32_t c) {
  uint32_t r;
  asm("lop3.b32 %0, %1, %2, %3, 0x7c;" : "=r"(r) : "r"(a), "r"(b), "r"(c));
  return r;
}
__device__ __forceinline__ uint32_t lgx_lop3_0x80(uint32_t a, uint32_t b, uint32_t c) {
  uint32_t r;
  asm("lop3.b32 %0, %1, %2, %3, 0x80;" : "=r"(r) : "r"(a), "r"(b), "r"(c));
  return r;
}
__device__ __forceinline__ uint32_t lgx_lop3_0x81(uint32_t a, uint32_t b, uint32_t c) {
  uint32_t r;
  asm("lop3.b32 %0, %1, %2, %3, 0x81;" : "=r"(r) : "r"(a), "r"(b), "r"(c));
  return r;
}
__device__ __forceinline__ uint32_t lgx_lop3_0x87(uint32_t a, uint32_t b, uint32_t c) {
  uint32_t r;
  asm("lop3.b32 %0, %1, %2, %3, 0x87;" : "=r"(r) : "r"(a), "r"(b), "r"(c));
  return r;
}
__device__ __forceinline__ uint32_t lgx_lop3_0x8a(uint32_t a, uint32_t b, uint32_t c) {
  uint32_t r;
  asm("lop3.b32 %0, %1, %2, %3, 0x8a;" : "=r"(r) : "r"(a), "r"(b), "r"(c));
  return r;
}
__device__ __forceinline__ uint32_t lgx_lop3_0x8e(uint32_t a, uint32_t b, uint32_t c) {
  uint32_t r;
  asm("lop3.b32 %0, %1, %2, %3, 0x8e;" : "=r"(r) : "r"(a), "r"(b), "r"(c));
  return r;
}
__device__ __forceinline__ uint32_t lgx_lop3_0x8f(uint32_t a, uint32_t b, uint32_t c) {
  uint32_t r;
  asm("lop3.b32 %0, %1, %2, %3, 0x8f;" : "=r"(r) : "r"(a), "r"(b), "r"(c));
  return r;
}
__device__ __forceinline__ uint32_t lgx_lop3_0xa3(uint32_t a, uint32_t b, uint32_t c) {
  uint32_t r;
  asm("lop3.b32 %0, %1, %2, %3, 0xa3;" : "=r"(r) : "r"(a), "r"(b), "r"(c));
  return r;
}
__device__ __forceinline__ uint32_t lgx_lop3_0xa8(uint32_t a, uint32_t b, uint32_t c) {
  uint32_t r;
  asm("lop3.b32 %0, %1, %2, %3, 0xa8;" : "=r"(r) : "r"(a), "r"(b), "r"(c));
  return r;
}
__device__ __forceinline__ uint32_t lgx_lop3_0xac(uint32_t a, uint32_t b, uint32_t c) {
  uint32_t r;
  asm("lop3.b32 %0, %1, %2, %3, 0xac;" : "=r"(r) : "r"(a), "r"(b), "r"(c));
  return r;
}
__device__ __forceinline__ uint32_t lgx_lop3_0xb3(uint32_t a, uint32_t b, uint32_t c) {
  uint32_t r;
  asm("lop3.b32 %0, %1, %2, %3, 0xb3;" : "=r"(r) : "r"(a), "r"(b), "r"(c));
  return r;
}
__device__ __forceinline__ uint32_t lgx_lop3_0xb5(uint32_t a, uint32_t b, uint32_t c) {
  uint32_t r;
  asm("lop3.b32 %0, %1, %2, %3, 0xb5;" : "=r"(r) : "r"(a), "r"(b), "r"(c));
  return r;
}
__device__ __forceinline__ uint32_t lgx_lop3_0xbc(uint32_t a, uint32_t b, uint32_t c) {
  uint32_t r;
  asm("lop3.b32 %0, %1, %2, %3, 0xbc;" : "=r"(r) : "r"(a), "r"(b), "r"(c));
  return r;
}
__device__ __forceinline__ uint32_t lgx_lop3_0xc0(uint32_t a, uint32_t b, uint32_t c) {
  uint32_t r;
  asm("lop3.b32 %0, %1, %2, %3, 0xc0;" : "=r"(r) : "r"(a), "r"(b), "r"(c));
  return r;
}
__device__ __forceinline__ uint32_t lgx_lop3_0xc3(uint32_t a, uint32_t b, uint32_t c) {
  uint32_t r;
  asm("lop3.b32 %0, %1, %2, %3, 0xc3;" : "=r"(r) : "r"(a), "r"(b), "r"(c));
  return r;
}
__device__ __forceinline__ uint32_t lgx_lop3_0xc8(uint32_t a, uint32_t b, uint32_t c) {
  uint32_t r;
  asm("lop3.b32 %0, %1, %2, %3, 0xc8;" : "=r"(r) : "r"(a), "r"(b), "r"(c));
  return r;
}
__device__ __forceinline__ uint32_t lgx_lop3_0xca(uint32_t a, uint32_t b, uint32_t c) {
  uint32_t r;
  asm("lop3.b32 %0, %1, %2, %3, 0xca;" : "=r"(r) : "r"(a), "r"(b), "r"(c));
  return r;
}
__device__ __forceinline__ uint32_t lgx_lop3_0xe5(uint32_t a, uint32_t b, uint32_t c) {
  uint32_t r;
  asm("lop3.b32 %0, %1, %2, %3, 0xe5;" : "=r"(r) : "r"(a), "r"(b), "r"(c));
  return r;
}
__device__ __forceinline__ uint32_t lgx_lop3_0xe8(uint32_t a, uint32_t b, uint32_t c) {
  uint32_t r;
  asm("lop3.b32 %0, %1, %2, %3, 0xe8;" : "=r"(r) : "r"(a), "r"(b), "r"(c));
  return r;
}
#endif

#if defined(__CUDA_ARCH__)

#undef LGX_LOP3

#define LGX_LOP3(a, b, c, lut) lgx_lop3_##lut(a, b, c)

#endif

// lgx_collide_rest: 161 lop3 per 32-cell word (rest particles: yes)
LGX_HD_INLINE void lgx_collide_rest(const uint32_t n[7], uint32_t s2, const uint32_t s3[3],
                      const uint32_t s5[5], uint32_t o[7]) {
  const uint32_t n0 = n[0];
  const uint32_t n1 = n[1];
  const uint32_t n2 = n[2];
  const uint32_t n3 = n[3];
  const uint32_t n4 = n[4];
  const uint32_t n5 = n[5];
  const uint32_t n6 = n[6];
  const uint32_t s3_0 = s3[0];
  const uint32_t s3_1 = s3[1];
  const uint32_t s3_2 = s3[2];
  const uint32_t s5_0 = s5[0];
  const uint32_t s5_1 = s5[1];
  const uint32_t s5_2 = s5[2];
  const uint32_t s5_3 = s5[3];
  const uint32_t s5_4 = s5[4];
  const uint32_t t22 = LGX_LOP3(n0, n1, n2, 0x69);
  const uint32_t t26 = LGX_LOP3(n0, n1, n2, 0x17);
  const uint32_t t32 = LGX_LOP3(n3, n4, n5, 0x69);
  const uint32_t t36 = LGX_LOP3(n3, n4, n5, 0x17);
  const uint32_t t40 = LGX_LOP3(n6, t22, t32, 0x8e);
  const uint32_t t44 = LGX_LOP3(t26, t36, t40, 0xe8);
  const uint32_t t65 = LGX_LOP3(n6, t44, 0u, 0x3c);
  const uint32_t t68 = LGX_LOP3(s2, t44, 0u, 0x3c);
  const uint32_t t71 = LGX_LOP3(s3_0, s3_2, t44, 0x1b);
  const uint32_t t74 = LGX_LOP3(s3_1, t44, 0u, 0x0f);
  const uint32_t t77 = LGX_LOP3(s3_0, s3_2, t44, 0x27);
  const uint32_t t80 = LGX_LOP3(s5_0, s5_4, t44, 0x1b);
  const uint32_t t83 = LGX_LOP3(s5_1, s5_3, t44, 0x1b);
  const uint32_t t89 = LGX_LOP3(s5_1, s5_3, t44, 0x27);
  const uint32_t t92 = LGX_LOP3(s5_0, s5_4, t44, 0x27);
  const uint32_t t93 = LGX_LOP3(n0, n3, t44, 0x42);
  const uint32_t t94 = LGX_LOP3(n0, n3, t44, 0x24);
  const uint32_t t95 = LGX_LOP3(n0, n3, t44, 0x18);
  const uint32_t t96 = LGX_LOP3(n0, n3, t44, 0x81);
  const uint32_t t97 = LGX_LOP3(n1, n4, t44, 0x42);
  const uint32_t t98 = LGX_LOP3(n1, n4, t44, 0x24);
  const uint32_t t99 = LGX_LOP3(n1, n4, t44, 0x18);
  const uint32_t t100 = LGX_LOP3(n1, n4, t44, 0x81);
  const uint32_t t101 = LGX_LOP3(n2, n5, t44, 0x42);
  const uint32_t t102 = LGX_LOP3(n2, n5, t44, 0x24);
  const uint32_t t103 = LGX_LOP3(n2, n5, t44, 0x18);
  const uint32_t t104 = LGX_LOP3(n2, n5, t44, 0x81);
  const uint32_t t105 = LGX_LOP3(t93, t99, 0u, 0xc0);
  const uint32_t t106 = LGX_LOP3(t102, t105, 0u, 0xc0);
  const uint32_t t107 = LGX_LOP3(t95, t97, 0u, 0xc0);
  const uint32_t t108 = LGX_LOP3(t101, t107, 0u, 0xc0);
  const uint32_t t111 = LGX_LOP3(t65, t106, t108, 0x35);
  const uint32_t t112 = LGX_LOP3(t103, t107, 0u, 0xc0);
  const uint32_t t113 = LGX_LOP3(t101, t105, 0u, 0xc0);
  const uint32_t t116 = LGX_LOP3(t65, t112, t113, 0x35);
  const uint32_t t118 = LGX_LOP3(t95, t98, t101, 0x80);
  const uint32_t t119 = LGX_LOP3(t93, t97, 0u, 0xc0);
  const uint32_t t120 = LGX_LOP3(t102, t119, 0u, 0xc0);
  const uint32_t t123 = LGX_LOP3(t65, t118, t120, 0x35);
  const uint32_t t124 = LGX_LOP3(t96, t97, 0u, 0xc0);
  const uint32_t t126 = LGX_LOP3(t93, t100, 0u, 0xc0);
  const uint32_t t129 = LGX_LOP3(t101, t124, t126, 0x1f);
  const uint32_t t130 = LGX_LOP3(t104, t119, t129, 0x2a);
  const uint32_t t131 = LGX_LOP3(t65, t130, 0u, 0x30);
  const uint32_t t132 = LGX_LOP3(t94, t99, 0u, 0xc0);
  const uint32_t t133 = LGX_LOP3(t94, t99, t101, 0x80);
  const uint32_t t134 = LGX_LOP3(t103, t119, 0u, 0xc0);
  const uint32_t t137 = LGX_LOP3(t65, t133, t134, 0x35);
  const uint32_t t138 = LGX_LOP3(t94, t97, 0u, 0xc0);
  const uint32_t t139 = LGX_LOP3(t102, t138, 0u, 0xc0);
  const uint32_t t140 = LGX_LOP3(t93, t98, 0u, 0xc0);
  const uint32_t t141 = LGX_LOP3(t101, t140, 0u, 0xc0);
  const uint32_t t144 = LGX_LOP3(t65, t139, t141, 0x35);
  const uint32_t t145 = LGX_LOP3(t103, t140, 0u, 0xc0);
  const uint32_t t146 = LGX_LOP3(t101, t138, 0u, 0xc0);
  const uint32_t t149 = LGX_LOP3(t65, t145, t146, 0x35);
  const uint32_t t151 = LGX_LOP3(t95, t100, t101, 0x80);
  const uint32_t t153 = LGX_LOP3(t104, t107, t151, 0x15);
  const uint32_t t156 = LGX_LOP3(t65, t106, t153, 0xa3);
  const uint32_t t158 = LGX_LOP3(t96, t99, t101, 0x80);
  const uint32_t t160 = LGX_LOP3(t104, t105, t158, 0x15);
  const uint32_t t163 = LGX_LOP3(t65, t112, t160, 0xa3);
  const uint32_t t166 = LGX_LOP3(t102, t124, t126, 0x1f);
  const uint32_t t169 = LGX_LOP3(t65, t118, t166, 0xa3);
  const uint32_t t171 = LGX_LOP3(t95, t98, t103, 0x80);
  const uint32_t t172 = LGX_LOP3(t102, t132, t171, 0x15);
  const uint32_t t175 = LGX_LOP3(t65, t130, t172, 0xac);
  const uint32_t t178 = LGX_LOP3(t103, t124, t126, 0x1f);
  const uint32_t t181 = LGX_LOP3(t65, t133, t178, 0xa3);
  const uint32_t t183 = LGX_LOP3(t96, t98, t101, 0x80);
  const uint32_t t185 = LGX_LOP3(t104, t140, t183, 0x15);
  const uint32_t t188 = LGX_LOP3(t65, t139, t185, 0xa3);
  const uint32_t t190 = LGX_LOP3(t94, t100, t101, 0x80);
  const uint32_t t192 = LGX_LOP3(t104, t138, t190, 0x15);
  const uint32_t t195 = LGX_LOP3(t65, t145, t192, 0xa3);
  const uint32_t t197 = LGX_LOP3(s3_0, s3_1, s3_2, 0x01);
  const uint32_t t199 = LGX_LOP3(s5_2, s5_3, 0u, 0x03);
  const uint32_t t200 = LGX_LOP3(s5_0, s5_1, t199, 0x02);
  const uint32_t t202 = LGX_LOP3(t111, t116, 0u, 0xc0);
  const uint32_t t205 = LGX_LOP3(t123, t137, t202, 0x80);
  const uint32_t t206 = LGX_LOP3(t144, t149, t205, 0x80);
  const uint32_t t207 = LGX_LOP3(t131, t156, 0u, 0x0c);
  const uint32_t t208 = LGX_LOP3(t163, t169, 0u, 0xc0);
  const uint32_t t209 = LGX_LOP3(t181, t188, 0u, 0xc0);
  const uint32_t t210 = LGX_LOP3(t207, t208, 0u, 0xc0);
  const uint32_t t212 = LGX_LOP3(t195, t209, t210, 0x80);
  const uint32_t t214 = LGX_LOP3(s5_4, t175, t200, 0x31);
  const uint32_t t215 = LGX_LOP3(t197, t206, t212, 0xc8);
  const uint32_t t216 = LGX_LOP3(t214, t215, 0u, 0x0c);
  const uint32_t t217 = LGX_LOP3(t137, t144, 0u, 0xc0);
  const uint32_t t220 = LGX_LOP3(t68, t149, t217, 0xca);
  const uint32_t t221 = LGX_LOP3(t131, t163, 0u, 0x0c);
  const uint32_t t222 = LGX_LOP3(t169, t181, 0u, 0xc0);
  const uint32_t t223 = LGX_LOP3(t188, t195, 0u, 0xc0);
  const uint32_t t224 = LGX_LOP3(t221, t222, 0u, 0xc0);
  const uint32_t t226 = LGX_LOP3(t71, t223, t224, 0x07);
  const uint32_t t229 = LGX_LOP3(t80, t175, 0u, 0x03);
  const uint32_t t230 = LGX_LOP3(s5_2, t44, t175, 0x50);
  const uint32_t t231 = LGX_LOP3(t77, t209, t229, 0x54);
  const uint32_t t232 = LGX_LOP3(t74, t195, t226, 0x54);
  const uint32_t t234 = LGX_LOP3(t230, t231, t232, 0x08);
  const uint32_t t238 = LGX_LOP3(t44, t220, t234, 0x87);
  const uint32_t t241 = LGX_LOP3(n0, t216, t238, 0x2e);
  const uint32_t t242 = LGX_LOP3(t123, t149, 0u, 0xc0);
  const uint32_t t245 = LGX_LOP3(t68, t144, t242, 0xca);
  const uint32_t t247 = LGX_LOP3(t156, t188, t195, 0x80);
  const uint32_t t250 = LGX_LOP3(t131, t169, t209, 0x08);
  const uint32_t t251 = LGX_LOP3(s3_1, t44, t250, 0x50);
  const uint32_t t253 = LGX_LOP3(t77, t169, t195, 0x07);
  const uint32_t t254 = LGX_LOP3(t83, t175, 0u, 0x03);
  const uint32_t t255 = LGX_LOP3(t89, t175, 0u, 0x03);
  const uint32_t t256 = LGX_LOP3(t71, t247, t251, 0x54);
  const uint32_t t257 = LGX_LOP3(t254, t255, 0u, 0x03);
  const uint32_t t259 = LGX_LOP3(t253, t256, t257, 0x08);
  const uint32_t t263 = LGX_LOP3(t44, t245, t259, 0x87);
  const uint32_t t266 = LGX_LOP3(n1, t216, t263, 0x2e);
  const uint32_t t267 = LGX_LOP3(t111, t144, 0u, 0xc0);
  const uint32_t t270 = LGX_LOP3(t68, t123, t267, 0xca);
  const uint32_t t272 = LGX_LOP3(t156, t163, 0u, 0xc0);
  const uint32_t t274 = LGX_LOP3(t169, t188, t272, 0x80);
  const uint32_t t276 = LGX_LOP3(t74, t195, t274, 0x07);
  const uint32_t t278 = LGX_LOP3(t77, t188, t207, 0x07);
  const uint32_t t279 = LGX_LOP3(t92, t175, 0u, 0x03);
  const uint32_t t281 = LGX_LOP3(t71, t169, t276, 0x54);
  const uint32_t t282 = LGX_LOP3(t229, t278, t281, 0x02);
  const uint32_t t284 = LGX_LOP3(t270, t279, t282, 0x20);
  const uint32_t t287 = LGX_LOP3(t44, t284, 0u, 0xc3);
  const uint32_t t290 = LGX_LOP3(n2, t216, t287, 0x2e);
  const uint32_t t291 = LGX_LOP3(t116, t123, 0u, 0xc0);
  const uint32_t t294 = LGX_LOP3(t68, t111, t291, 0xca);
  const uint32_t t296 = LGX_LOP3(t71, t209, t210, 0x07);
  const uint32_t t300 = LGX_LOP3(t74, t156, t296, 0x54);
  const uint32_t t301 = LGX_LOP3(t77, t208, t300, 0xa8);
  const uint32_t t302 = LGX_LOP3(t230, t254, t301, 0x02);
  const uint32_t t306 = LGX_LOP3(t44, t294, t302, 0x87);
  const uint32_t t309 = LGX_LOP3(n3, t216, t306, 0x2e);
  const uint32_t t310 = LGX_LOP3(t111, t137, 0u, 0xc0);
  const uint32_t t313 = LGX_LOP3(t68, t116, t310, 0xca);
  const uint32_t t315 = LGX_LOP3(t71, t195, t272, 0x07);
  const uint32_t t318 = LGX_LOP3(t77, t156, t181, 0x07);
  const uint32_t t320 = LGX_LOP3(t74, t224, t315, 0x54);
  const uint32_t t321 = LGX_LOP3(t229, t318, t320, 0x02);
  const uint32_t t323 = LGX_LOP3(t255, t313, t321, 0x08);
  const uint32_t t326 = LGX_LOP3(t44, t323, 0u, 0xc3);
  const uint32_t t329 = LGX_LOP3(n4, t216, t326, 0x2e);
  const uint32_t t330 = LGX_LOP3(t116, t149, 0u, 0xc0);
  const uint32_t t333 = LGX_LOP3(t68, t137, t330, 0xca);
  const uint32_t t336 = LGX_LOP3(t195, t209, t272, 0x80);
  const uint32_t t337 = LGX_LOP3(s3_1, t44, t336, 0x50);
  const uint32_t t339 = LGX_LOP3(t77, t195, t221, 0x07);
  const uint32_t t340 = LGX_LOP3(t71, t181, t337, 0x54);
  const uint32_t t341 = LGX_LOP3(t254, t279, 0u, 0x03);
  const uint32_t t343 = LGX_LOP3(t339, t340, t341, 0x08);
  const uint32_t t347 = LGX_LOP3(t44, t333, t343, 0x87);
  const uint32_t t350 = LGX_LOP3(n5, t216, t347, 0x2e);
  const uint32_t t353 = LGX_LOP3(t222, t223, t272, 0x80);
  const uint32_t t356 = LGX_LOP3(t230, t255, t279, 0x01);
  const uint32_t t357 = LGX_LOP3(t77, t353, t356, 0xa8);
  const uint32_t t358 = LGX_LOP3(t68, t206, t357, 0x8a);
  const uint32_t t361 = LGX_LOP3(t44, t358, 0u, 0xc3);
  const uint32_t t364 = LGX_LOP3(n6, t216, t361, 0x2e);
  o[0] = ~t241;
  o[1] = ~t266;
  o[2] = ~t290;
  o[3] = ~t309;
  o[4] = ~t329;
  o[5] = ~t350;
  o[6] = ~t364;
}

// lgx_collide_norest: 83 lop3 per 32-cell word (rest particles: no)
LGX_HD_INLINE void lgx_collide_norest(const uint32_t n[7], uint32_t s2, const uint32_t s3[3],
                      const uint32_t s5[5], uint32_t o[7]) {
  const uint32_t n0 = n[0];
  const uint32_t n1 = n[1];
  const uint32_t n2 = n[2];
  const uint32_t n3 = n[3];
  const uint32_t n4 = n[4];
  const uint32_t n5 = n[5];
  const uint32_t n6 = n[6];
  const uint32_t s3_0 = s3[0];
  const uint32_t s3_1 = s3[1];
  const uint32_t s3_2 = s3[2];
  (void)s5;
  const uint32_t t17 = LGX_LOP3(n0, n3, 0u, 0x03);
  const uint32_t t18 = LGX_LOP3(n0, n3, 0u, 0x30);
  const uint32_t t19 = LGX_LOP3(n0, n3, 0u, 0x0c);
  const uint32_t t20 = LGX_LOP3(n0, n3, 0u, 0xc0);
  const uint32_t t21 = LGX_LOP3(n1, n4, 0u, 0x03);
  const uint32_t t22 = LGX_LOP3(n1, n4, 0u, 0x30);
  const uint32_t t23 = LGX_LOP3(n1, n4, 0u, 0x0c);
  const uint32_t t24 = LGX_LOP3(n1, n4, 0u, 0xc0);
  const uint32_t t25 = LGX_LOP3(n2, n5, 0u, 0x03);
  const uint32_t t26 = LGX_LOP3(n2, n5, 0u, 0x30);
  const uint32_t t27 = LGX_LOP3(n2, n5, 0u, 0x0c);
  const uint32_t t28 = LGX_LOP3(n2, n5, 0u, 0xc0);
  const uint32_t t30 = LGX_LOP3(t20, t21, t25, 0x80);
  const uint32_t t31 = LGX_LOP3(n1, n4, t25, 0x80);
  const uint32_t t33 = LGX_LOP3(n1, n4, t28, 0x02);
  const uint32_t t35 = LGX_LOP3(t17, t30, t31, 0x13);
  const uint32_t t36 = LGX_LOP3(t17, t33, t35, 0x2a);
  const uint32_t t39 = LGX_LOP3(t19, t31, t33, 0x1f);
  const uint32_t t40 = LGX_LOP3(n1, n4, t25, 0x08);
  const uint32_t t43 = LGX_LOP3(t17, t23, t28, 0x80);
  const uint32_t t44 = LGX_LOP3(t20, t40, t43, 0x15);
  const uint32_t t46 = LGX_LOP3(t20, t21, t26, 0x80);
  const uint32_t t47 = LGX_LOP3(n2, n5, t24, 0x20);
  const uint32_t t49 = LGX_LOP3(t17, t46, t47, 0x13);
  const uint32_t t50 = LGX_LOP3(n1, n4, t26, 0x08);
  const uint32_t t53 = LGX_LOP3(t19, t22, t27, 0x80);
  const uint32_t t54 = LGX_LOP3(t18, t50, t53, 0x15);
  const uint32_t t55 = LGX_LOP3(n2, n5, t21, 0x08);
  const uint32_t t58 = LGX_LOP3(t17, t24, t27, 0x80);
  const uint32_t t59 = LGX_LOP3(t20, t55, t58, 0x15);
  const uint32_t t60 = LGX_LOP3(n1, n4, t25, 0x20);
  const uint32_t t63 = LGX_LOP3(t17, t22, t28, 0x80);
  const uint32_t t64 = LGX_LOP3(t20, t60, t63, 0x15);
  const uint32_t t67 = LGX_LOP3(t18, t31, t33, 0x1f);
  const uint32_t t70 = LGX_LOP3(n1, n4, t28, 0x80);
  const uint32_t t72 = LGX_LOP3(t20, t31, t33, 0x1f);
  const uint32_t t73 = LGX_LOP3(t17, t70, t72, 0x2a);
  const uint32_t t75 = LGX_LOP3(s3_0, s3_1, s3_2, 0x01);
  const uint32_t t80 = LGX_LOP3(t39, t44, 0u, 0xc0);
  const uint32_t t81 = LGX_LOP3(t49, t54, 0u, 0xc0);
  const uint32_t t82 = LGX_LOP3(t59, t64, 0u, 0xc0);
  const uint32_t t84 = LGX_LOP3(t67, t82, 0u, 0xc0);
  const uint32_t t85 = LGX_LOP3(t80, t81, t84, 0x80);
  const uint32_t t86 = LGX_LOP3(t36, t73, 0u, 0xc0);
  const uint32_t t88 = LGX_LOP3(t75, t85, t86, 0xc8);
  const uint32_t t90 = LGX_LOP3(t44, t49, 0u, 0xc0);
  const uint32_t t91 = LGX_LOP3(t54, t59, 0u, 0xc0);
  const uint32_t t92 = LGX_LOP3(t64, t67, 0u, 0xc0);
  const uint32_t t94 = LGX_LOP3(t90, t91, t92, 0x80);
  const uint32_t t97 = LGX_LOP3(s2, t67, t94, 0xac);
  const uint32_t t99 = LGX_LOP3(s3_1, t73, 0u, 0x30);
  const uint32_t t100 = LGX_LOP3(n0, t88, t97, 0x2a);
  const uint32_t t101 = LGX_LOP3(s3_0, t86, t99, 0x45);
  const uint32_t t102 = LGX_LOP3(t100, t101, 0u, 0xc0);
  const uint32_t t105 = LGX_LOP3(t39, t64, t67, 0x80);
  const uint32_t t106 = LGX_LOP3(t81, t82, 0u, 0xc0);
  const uint32_t t109 = LGX_LOP3(s2, t105, t106, 0xca);
  const uint32_t t110 = LGX_LOP3(s3_0, t73, 0u, 0x30);
  const uint32_t t112 = LGX_LOP3(s3_2, t73, 0u, 0x30);
  const uint32_t t113 = LGX_LOP3(n1, t88, t109, 0x2a);
  const uint32_t t114 = LGX_LOP3(s3_1, t36, t110, 0x45);
  const uint32_t t116 = LGX_LOP3(t112, t113, t114, 0x08);
  const uint32_t t119 = LGX_LOP3(t49, t64, t80, 0x80);
  const uint32_t t120 = LGX_LOP3(t67, t119, 0u, 0xc0);
  const uint32_t t123 = LGX_LOP3(s2, t81, t120, 0xca);
  const uint32_t t124 = LGX_LOP3(s3_2, t86, 0u, 0x30);
  const uint32_t t125 = LGX_LOP3(n2, t88, t123, 0x2a);
  const uint32_t t127 = LGX_LOP3(t99, t124, t125, 0x02);
  const uint32_t t128 = LGX_LOP3(n3, t88, 0u, 0xc0);
  const uint32_t t130 = LGX_LOP3(t49, t59, t80, 0x80);
  const uint32_t t133 = LGX_LOP3(s2, t64, t130, 0x70);
  const uint32_t t134 = LGX_LOP3(s2, t39, t54, 0x07);
  const uint32_t t136 = LGX_LOP3(t128, t133, t134, 0x01);
  const uint32_t t137 = LGX_LOP3(t101, t136, 0u, 0xc0);
  const uint32_t t140 = LGX_LOP3(t54, t67, t80, 0x80);
  const uint32_t t143 = LGX_LOP3(s2, t59, t90, 0x07);
  const uint32_t t144 = LGX_LOP3(s2, t140, t143, 0x45);
  const uint32_t t145 = LGX_LOP3(n4, t88, t144, 0x2a);
  const uint32_t t147 = LGX_LOP3(t112, t114, t145, 0x08);
  const uint32_t t150 = LGX_LOP3(t80, t91, t92, 0x80);
  const uint32_t t153 = LGX_LOP3(s2, t59, t150, 0xca);
  const uint32_t t154 = LGX_LOP3(n5, t88, t153, 0x2a);
  const uint32_t t156 = LGX_LOP3(t99, t124, t154, 0x02);
  o[0] = ~t102;
  o[1] = ~t116;
  o[2] = ~t127;
  o[3] = ~t137;
  o[4] = ~t147;
  o[5] = ~t156;
  o[6] = n6;
}

// lgx_selectors: 44 lop3; r[0..17] are hashes 2..19 of the chain
LGX_HD_INLINE void lgx_selectors(const uint32_t r[18], uint32_t s3[3], uint32_t s5[5]) {
  const uint32_t r1 = r[0];
  const uint32_t r2 = r[1];
  const uint32_t r3 = r[2];
  const uint32_t r4 = r[3];
  const uint32_t r5 = r[4];
  const uint32_t r6 = r[5];
  const uint32_t r7 = r[6];
  const uint32_t r8 = r[7];
  const uint32_t r9 = r[8];
  const uint32_t r10 = r[9];
  const uint32_t r11 = r[10];
  const uint32_t r12 = r[11];
  const uint32_t r13 = r[12];
  const uint32_t r14 = r[13];
  const uint32_t r15 = r[14];
  const uint32_t r16 = r[15];
  const uint32_t r17 = r[16];
  const uint32_t r18 = r[17];
  const uint32_t t19 = LGX_LOP3(r5, r6, 0u, 0x03);
  const uint32_t t23 = LGX_LOP3(r3, r4, t19, 0x7c);
  const uint32_t t27 = LGX_LOP3(r1, r2, t23, 0xbc);
  const uint32_t t28 = LGX_LOP3(r5, r6, 0u, 0x30);
  const uint32_t t31 = LGX_LOP3(r3, r4, t28, 0x4f);
  const uint32_t t34 = LGX_LOP3(r1, r2, t31, 0x8f);
  const uint32_t t35 = LGX_LOP3(r5, r6, 0u, 0x0c);
  const uint32_t t38 = LGX_LOP3(r3, r4, t35, 0x73);
  const uint32_t t41 = LGX_LOP3(r1, r2, t38, 0xb3);
  const uint32_t t43 = LGX_LOP3(r16, r17, r18, 0x01);
  const uint32_t t44 = LGX_LOP3(r13, r14, 0u, 0x03);
  const uint32_t t46 = LGX_LOP3(r13, r14, r15, 0xa8);
  const uint32_t t48 = LGX_LOP3(r15, t43, t44, 0xb5);
  const uint32_t t49 = LGX_LOP3(r10, r11, 0u, 0x03);
  const uint32_t t51 = LGX_LOP3(r10, r11, r12, 0xa8);
  const uint32_t t53 = LGX_LOP3(r12, t48, t49, 0xe5);
  const uint32_t t54 = LGX_LOP3(r7, r8, 0u, 0x03);
  const uint32_t t56 = LGX_LOP3(r7, r8, r9, 0xa8);
  const uint32_t t58 = LGX_LOP3(r9, t53, t54, 0xe5);
  const uint32_t t60 = LGX_LOP3(r16, r17, r18, 0x10);
  const uint32_t t62 = LGX_LOP3(r13, r14, r15, 0x10);
  const uint32_t t64 = LGX_LOP3(t46, t60, t62, 0x15);
  const uint32_t t66 = LGX_LOP3(r10, r11, r12, 0x10);
  const uint32_t t68 = LGX_LOP3(t51, t64, t66, 0x45);
  const uint32_t t70 = LGX_LOP3(r7, r8, r9, 0x10);
  const uint32_t t72 = LGX_LOP3(t56, t68, t70, 0x45);
  const uint32_t t74 = LGX_LOP3(r16, r17, r18, 0x04);
  const uint32_t t76 = LGX_LOP3(r13, r14, r15, 0x04);
  const uint32_t t78 = LGX_LOP3(t46, t74, t76, 0x15);
  const uint32_t t80 = LGX_LOP3(r10, r11, r12, 0x04);
  const uint32_t t82 = LGX_LOP3(t51, t78, t80, 0x45);
  const uint32_t t84 = LGX_LOP3(r7, r8, r9, 0x04);
  const uint32_t t86 = LGX_LOP3(t56, t82, t84, 0x45);
  const uint32_t t88 = LGX_LOP3(r16, r17, r18, 0x40);
  const uint32_t t90 = LGX_LOP3(r13, r14, r15, 0x40);
  const uint32_t t92 = LGX_LOP3(t46, t88, t90, 0x15);
  const uint32_t t94 = LGX_LOP3(r10, r11, r12, 0x40);
  const uint32_t t96 = LGX_LOP3(t51, t92, t94, 0x45);
  const uint32_t t98 = LGX_LOP3(r7, r8, r9, 0x40);
  const uint32_t t100 = LGX_LOP3(t56, t96, t98, 0x45);
  const uint32_t t101 = LGX_LOP3(r16, r17, r18, 0x02);
  const uint32_t t104 = LGX_LOP3(r15, t44, t101, 0x1f);
  const uint32_t t107 = LGX_LOP3(r12, t49, t104, 0x2f);
  const uint32_t t110 = LGX_LOP3(r9, t54, t107, 0x2f);
  s3[0] = ~t27;
  s3[1] = ~t34;
  s3[2] = ~t41;
  s5[0] = ~t58;
  s5[1] = ~t72;
  s5[2] = ~t86;
  s5[3] = ~t100;
  s5[4] = ~t110;
}

// stats: lgx_collide_rest {'aig_ands': 348, 'lop3': 161, 'checked': 6144}; lgx_collide_norest {'aig_ands': 140, 'lop3': 83, 'checked': 6144}; lgx_selectors {'aig_ands': 92, 'lop3': 44, 'checked': 4096}
