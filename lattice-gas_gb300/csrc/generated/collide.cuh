// Generated by lattice-gas_gb300/gen/collide_gen.py -- do not edit.
//
// The FHP collision rule as three-input lookup tables, one lop3.b32 each.
// Inputs: seven planes n[0..6] (six directions, then rest), the fair bit s2,
// one-hot selectors s3[0..2] and s5[0..4].  Output: seven planes o[0..6].
// Semantics (class pick by selector) follow the reference's known-answer
// specification, src/gpu.rs:799-817; classes come from src/collision.rs:152-159.
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
__device__ __forceinline__ uint32_t lgx_lop3_0x23(uint32_t a, uint32_t b, uint32_t c) {
  uint32_t r;
  asm("lop3.b32 %0, %1, %2, %3, 0x23;" : "=r"(r) : "r"(a), "r"(b), "r"(c));
  return r;
}
__device__ __forceinline__ uint32_t lgx_lop3_0x2a(uint32_t a, uint32_t b, uint32_t c) {
  uint32_t r;
  asm("lop3.b32 %0, %1, %2, %3, 0x2a;" : "=r"(r) : "r"(a), "r"(b), "r"(c));
  return r;
}
__device__ __forceinline__ uint32_t lgx_lop3_0x30(uint32_t a, uint32_t b, uint32_t c) {
  uint32_t r;
  asm("lop3.b32 %0, %1, %2, %3, 0x30;" : "=r"(r) : "r"(a), "r"(b), "r"(c));
  return r;
}
__device__ __forceinline__ uint32_t lgx_lop3_0x35(uint32_t a, uint32_t b, uint32_t c) {
  uint32_t r;
  asm("lop3.b32 %0, %1, %2, %3, 0x35;" : "=r"(r) : "r"(a), "r"(b), "r"(c));
  return r;
}
__device__ __forceinline__ uint32_t lgx_lop3_0x3a(uint32_t a, uint32_t b, uint32_t c) {
  uint32_t r;
  asm("lop3.b32 %0, %1, %2, %3, 0x3a;" : "=r"(r) : "r"(a), "r"(b), "r"(c));
  return r;
}
__device__ __forceinline__ uint32_t lgx_lop3_0x40(uint32_t a, uint32_t b, uint32_t c) {
  uint32_t r;
  asm("lop3.b32 %0, %1, %2, %3, 0x40;" : "=r"(r) : "r"(a), "r"(b), "r"(c));
  return r;
}
__device__ __forceinline__ uint32_t lgx_lop3_0x45(uint32_t a, uint32_t b, uint32_t c) {
  uint32_t r;
  asm("lop3.b32 %0, %1, %2, %3, 0x45;" : "=r"(r) : "r"(a), "r"(b), "r"(c));
  return r;
}
__device__ __forceinline__ uint32_t lgx_lop3_0x51(uint32_t a, uint32_t b, uint32_t c) {
  uint32_t r;
  asm("lop3.b32 %0, %1, %2, %3, 0x51;" : "=r"(r) : "r"(a), "r"(b), "r"(c));
  return r;
}
__device__ __forceinline__ uint32_t lgx_lop3_0x53(uint32_t a, uint32_t b, uint32_t c) {
  uint32_t r;
  asm("lop3.b32 %0, %1, %2, %3, 0x53;" : "=r"(r) : "r"(a), "r"(b), "r"(c));
  return r;
}
__device__ __forceinline__ uint32_t lgx_lop3_0x54(uint32_t a, uint32_t b, uint32_t c) {
  uint32_t r;
  asm("lop3.b32 %0, %1, %2, %3, 0x54;" : "=r"(r) : "r"(a), "r"(b), "r"(c));
  return r;
}
__device__ __forceinline__ uint32_t lgx_lop3_0x70(uint32_t a, uint32_t b, uint32_t c) {
  uint32_t r;
  asm("lop3.b32 %0, %1, %2, %3, 0x70;" : "=r"(r) : "r"(a), "r"(b), "r"(c));
  return r;
}
__device__ __forceinline__ uint32_t lgx_lop3_0x80(uint32_t a, uint32_t b, uint32_t c) {
  uint32_t r;
  asm("lop3.b32 %0, %1, %2, %3, 0x80;" : "=r"(r) : "r"(a), "r"(b), "r"(c));
  return r;
}
__device__ __forceinline__ uint32_t lgx_lop3_0x8a(uint32_t a, uint32_t b, uint32_t c) {
  uint32_t r;
  asm("lop3.b32 %0, %1, %2, %3, 0x8a;" : "=r"(r) : "r"(a), "r"(b), "r"(c));
  return r;
}
__device__ __forceinline__ uint32_t lgx_lop3_0xab(uint32_t a, uint32_t b, uint32_t c) {
  uint32_t r;
  asm("lop3.b32 %0, %1, %2, %3, 0xab;" : "=r"(r) : "r"(a), "r"(b), "r"(c));
  return r;
}
__device__ __forceinline__ uint32_t lgx_lop3_0xac(uint32_t a, uint32_t b, uint32_t c) {
  uint32_t r;
  asm("lop3.b32 %0, %1, %2, %3, 0xac;" : "=r"(r) : "r"(a), "r"(b), "r"(c));
  return r;
}
__device__ __forceinline__ uint32_t lgx_lop3_0xc0(uint32_t a, uint32_t b, uint32_t c) {
  uint32_t r;
  asm("lop3.b32 %0, %1, %2, %3, 0xc0;" : "=r"(r) : "r"(a), "r"(b), "r"(c));
  return r;
}
__device__ __forceinline__ uint32_t lgx_lop3_0xc5(uint32_t a, uint32_t b, uint32_t c) {
  uint32_t r;
  asm("lop3.b32 %0, %1, %2, %3, 0xc5;" : "=r"(r) : "r"(a), "r"(b), "r"(c));
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
__device__ __forceinline__ uint32_t lgx_lop3_0xd0(uint32_t a, uint32_t b, uint32_t c) {
  uint32_t r;
  asm("lop3.b32 %0, %1, %2, %3, 0xd0;" : "=r"(r) : "r"(a), "r"(b), "r"(c));
  return r;
}
#endif

#if defined(__CUDA_ARCH__)

#undef LGX_LOP3

#define LGX_LOP3(a, b, c, lut) lgx_lop3_##lut(a, b, c)

#endif

// lgx_collide_rest: 261 lop3 per 32-cell word (rest particles: yes)
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
  const uint32_t t17 = LGX_LOP3(n0, n3, 0u, 0x03);
  const uint32_t t18 = LGX_LOP3(n0, n3, 0u, 0x30);
  const uint32_t t19 = LGX_LOP3(n0, n3, 0u, 0x0c);
  const uint32_t t20 = LGX_LOP3(n0, n3, 0u, 0xc0);
  const uint32_t t21 = LGX_LOP3(n1, n4, 0u, 0x03);
  const uint32_t t22 = LGX_LOP3(n1, n4, 0u, 0x30);
  const uint32_t t24 = LGX_LOP3(n1, n4, 0u, 0xc0);
  const uint32_t t25 = LGX_LOP3(n2, n5, 0u, 0x03);
  const uint32_t t26 = LGX_LOP3(n2, n5, 0u, 0x30);
  const uint32_t t28 = LGX_LOP3(n2, n5, 0u, 0xc0);
  const uint32_t t29 = LGX_LOP3(n1, n4, t26, 0x08);
  const uint32_t t30 = LGX_LOP3(n0, n3, t29, 0x02);
  const uint32_t t31 = LGX_LOP3(n1, n4, t25, 0x02);
  const uint32_t t32 = LGX_LOP3(n0, n3, t31, 0x08);
  const uint32_t t35 = LGX_LOP3(n6, t30, t32, 0x53);
  const uint32_t t36 = LGX_LOP3(n2, n5, t21, 0x08);
  const uint32_t t37 = LGX_LOP3(n0, n3, t36, 0x08);
  const uint32_t t38 = LGX_LOP3(n1, n4, t25, 0x08);
  const uint32_t t39 = LGX_LOP3(n0, n3, t38, 0x02);
  const uint32_t t42 = LGX_LOP3(n6, t37, t39, 0x53);
  const uint32_t t43 = LGX_LOP3(n1, n4, t25, 0x20);
  const uint32_t t44 = LGX_LOP3(n0, n3, t43, 0x08);
  const uint32_t t45 = LGX_LOP3(n2, n5, t21, 0x20);
  const uint32_t t46 = LGX_LOP3(n0, n3, t45, 0x02);
  const uint32_t t49 = LGX_LOP3(n6, t44, t46, 0x53);
  const uint32_t t51 = LGX_LOP3(n1, n4, t25, 0x80);
  const uint32_t t52 = LGX_LOP3(n0, n3, t51, 0x02);
  const uint32_t t53 = LGX_LOP3(n1, n4, t28, 0x02);
  const uint32_t t55 = LGX_LOP3(t20, t31, t52, 0x15);
  const uint32_t t56 = LGX_LOP3(t17, t53, t55, 0x2a);
  const uint32_t t57 = LGX_LOP3(n6, t56, 0u, 0x03);
  const uint32_t t58 = LGX_LOP3(n0, n3, t38, 0x20);
  const uint32_t t59 = LGX_LOP3(n0, n3, t36, 0x02);
  const uint32_t t62 = LGX_LOP3(n6, t58, t59, 0x53);
  const uint32_t t63 = LGX_LOP3(n0, n3, t45, 0x20);
  const uint32_t t64 = LGX_LOP3(n0, n3, t43, 0x02);
  const uint32_t t67 = LGX_LOP3(n6, t63, t64, 0x53);
  const uint32_t t68 = LGX_LOP3(n2, n5, t22, 0x08);
  const uint32_t t69 = LGX_LOP3(n0, n3, t68, 0x02);
  const uint32_t t70 = LGX_LOP3(n0, n3, t31, 0x20);
  const uint32_t t73 = LGX_LOP3(n6, t69, t70, 0x53);
  const uint32_t t76 = LGX_LOP3(t19, t51, t53, 0x1f);
  const uint32_t t79 = LGX_LOP3(n6, t30, t76, 0x3a);
  const uint32_t t80 = LGX_LOP3(n0, n3, t38, 0x80);
  const uint32_t t81 = LGX_LOP3(n1, n4, t28, 0x08);
  const uint32_t t83 = LGX_LOP3(t17, t80, t81, 0x13);
  const uint32_t t86 = LGX_LOP3(n6, t37, t83, 0x3a);
  const uint32_t t88 = LGX_LOP3(n2, n5, t24, 0x20);
  const uint32_t t89 = LGX_LOP3(n0, n3, t88, 0x02);
  const uint32_t t90 = LGX_LOP3(t20, t45, t89, 0x15);
  const uint32_t t93 = LGX_LOP3(n6, t44, t90, 0x3a);
  const uint32_t t95 = LGX_LOP3(n0, n3, t68, 0x08);
  const uint32_t t96 = LGX_LOP3(t18, t29, t95, 0x15);
  const uint32_t t99 = LGX_LOP3(n6, t56, t96, 0xca);
  const uint32_t t101 = LGX_LOP3(n2, n5, t24, 0x08);
  const uint32_t t102 = LGX_LOP3(n0, n3, t101, 0x02);
  const uint32_t t103 = LGX_LOP3(t20, t36, t102, 0x15);
  const uint32_t t106 = LGX_LOP3(n6, t58, t103, 0x3a);
  const uint32_t t108 = LGX_LOP3(n1, n4, t28, 0x20);
  const uint32_t t109 = LGX_LOP3(n0, n3, t108, 0x02);
  const uint32_t t110 = LGX_LOP3(t20, t43, t109, 0x15);
  const uint32_t t113 = LGX_LOP3(n6, t63, t110, 0x3a);
  const uint32_t t116 = LGX_LOP3(t18, t51, t53, 0x1f);
  const uint32_t t119 = LGX_LOP3(n6, t69, t116, 0x3a);
  const uint32_t t120 = LGX_LOP3(n0, n3, t29, 0x80);
  const uint32_t t123 = LGX_LOP3(n6, t76, t120, 0xc5);
  const uint32_t t124 = LGX_LOP3(n0, n3, t101, 0x08);
  const uint32_t t127 = LGX_LOP3(n6, t83, t124, 0xc5);
  const uint32_t t128 = LGX_LOP3(n0, n3, t108, 0x08);
  const uint32_t t131 = LGX_LOP3(n6, t90, t128, 0xc5);
  const uint32_t t134 = LGX_LOP3(n1, n4, t28, 0x80);
  const uint32_t t136 = LGX_LOP3(t20, t51, t53, 0x1f);
  const uint32_t t137 = LGX_LOP3(t17, t134, t136, 0x2a);
  const uint32_t t140 = LGX_LOP3(n6, t96, t137, 0xca);
  const uint32_t t141 = LGX_LOP3(n0, n3, t81, 0x20);
  const uint32_t t144 = LGX_LOP3(n6, t103, t141, 0xc5);
  const uint32_t t145 = LGX_LOP3(n0, n3, t88, 0x20);
  const uint32_t t148 = LGX_LOP3(n6, t110, t145, 0xc5);
  const uint32_t t149 = LGX_LOP3(n0, n3, t68, 0x80);
  const uint32_t t152 = LGX_LOP3(n6, t116, t149, 0xc5);
  const uint32_t t153 = LGX_LOP3(n0, n3, t134, 0x08);
  const uint32_t t156 = LGX_LOP3(n6, t120, t153, 0x35);
  const uint32_t t157 = LGX_LOP3(n0, n3, t81, 0x80);
  const uint32_t t160 = LGX_LOP3(n6, t124, t157, 0x35);
  const uint32_t t161 = LGX_LOP3(n0, n3, t88, 0x80);
  const uint32_t t164 = LGX_LOP3(n6, t128, t161, 0x35);
  const uint32_t t165 = LGX_LOP3(n6, t137, 0u, 0x30);
  const uint32_t t166 = LGX_LOP3(n0, n3, t101, 0x80);
  const uint32_t t169 = LGX_LOP3(n6, t141, t166, 0x35);
  const uint32_t t170 = LGX_LOP3(n0, n3, t108, 0x80);
  const uint32_t t173 = LGX_LOP3(n6, t145, t170, 0x35);
  const uint32_t t174 = LGX_LOP3(n0, n3, t134, 0x20);
  const uint32_t t177 = LGX_LOP3(n6, t149, t174, 0x35);
  const uint32_t t179 = LGX_LOP3(s3_0, s3_1, s3_2, 0x01);
  const uint32_t t181 = LGX_LOP3(s5_2, s5_3, 0u, 0x03);
  const uint32_t t182 = LGX_LOP3(s5_0, s5_1, t181, 0x02);
  const uint32_t t185 = LGX_LOP3(t49, t62, 0u, 0xc0);
  const uint32_t t187 = LGX_LOP3(t156, t160, 0u, 0xc0);
  const uint32_t t188 = LGX_LOP3(t164, t169, 0u, 0xc0);
  const uint32_t t190 = LGX_LOP3(t35, t42, t185, 0x80);
  const uint32_t t191 = LGX_LOP3(t67, t73, t187, 0x80);
  const uint32_t t192 = LGX_LOP3(t173, t177, t188, 0x80);
  const uint32_t t194 = LGX_LOP3(t190, t191, t192, 0x80);
  const uint32_t t195 = LGX_LOP3(t57, t79, 0u, 0x0c);
  const uint32_t t196 = LGX_LOP3(t86, t93, 0u, 0xc0);
  const uint32_t t197 = LGX_LOP3(t106, t113, 0u, 0xc0);
  const uint32_t t198 = LGX_LOP3(t119, t123, 0u, 0xc0);
  const uint32_t t199 = LGX_LOP3(t127, t131, 0u, 0xc0);
  const uint32_t t200 = LGX_LOP3(t144, t148, 0u, 0xc0);
  const uint32_t t201 = LGX_LOP3(t152, t165, 0u, 0x30);
  const uint32_t t202 = LGX_LOP3(t195, t196, 0u, 0xc0);
  const uint32_t t205 = LGX_LOP3(t197, t198, t202, 0x80);
  const uint32_t t206 = LGX_LOP3(t199, t200, t201, 0x80);
  const uint32_t t208 = LGX_LOP3(t179, t205, t206, 0x07);
  const uint32_t t209 = LGX_LOP3(t99, t140, 0u, 0xc0);
  const uint32_t t210 = LGX_LOP3(s5_4, t182, t209, 0x51);
  const uint32_t t212 = LGX_LOP3(t194, t208, t210, 0x10);
  const uint32_t t213 = LGX_LOP3(n0, t212, 0u, 0xc0);
  const uint32_t t215 = LGX_LOP3(t160, t164, 0u, 0xc0);
  const uint32_t t216 = LGX_LOP3(t169, t173, 0u, 0xc0);
  const uint32_t t217 = LGX_LOP3(t62, t67, t215, 0x80);
  const uint32_t t218 = LGX_LOP3(t177, t216, 0u, 0xc0);
  const uint32_t t221 = LGX_LOP3(t73, t156, t216, 0x80);
  const uint32_t t223 = LGX_LOP3(s2, t217, t218, 0x70);
  const uint32_t t224 = LGX_LOP3(s2, t177, t221, 0x07);
  const uint32_t t226 = LGX_LOP3(t57, t86, 0u, 0x0c);
  const uint32_t t227 = LGX_LOP3(t93, t106, 0u, 0xc0);
  const uint32_t t228 = LGX_LOP3(t113, t119, 0u, 0xc0);
  const uint32_t t230 = LGX_LOP3(t148, t152, 0u, 0xc0);
  const uint32_t t231 = LGX_LOP3(t226, t227, 0u, 0xc0);
  const uint32_t t232 = LGX_LOP3(t123, t144, t228, 0x80);
  const uint32_t t233 = LGX_LOP3(t165, t230, 0u, 0x0c);
  const uint32_t t235 = LGX_LOP3(t231, t232, t233, 0x80);
  const uint32_t t237 = LGX_LOP3(t119, t127, 0u, 0xc0);
  const uint32_t t238 = LGX_LOP3(t131, t144, 0u, 0xc0);
  const uint32_t t240 = LGX_LOP3(t233, t237, t238, 0x80);
  const uint32_t t241 = LGX_LOP3(s3_1, t240, 0u, 0x30);
  const uint32_t t243 = LGX_LOP3(s3_2, t152, t197, 0x70);
  const uint32_t t244 = LGX_LOP3(s5_0, t209, 0u, 0x30);
  const uint32_t t245 = LGX_LOP3(s5_1, t140, 0u, 0x30);
  const uint32_t t246 = LGX_LOP3(s5_2, t99, 0u, 0x30);
  const uint32_t t247 = LGX_LOP3(s5_3, t140, 0u, 0x30);
  const uint32_t t248 = LGX_LOP3(t213, t223, t224, 0x01);
  const uint32_t t249 = LGX_LOP3(s3_0, t235, t241, 0x45);
  const uint32_t t250 = LGX_LOP3(s5_0, t209, t243, 0x45);
  const uint32_t t253 = LGX_LOP3(t245, t246, t250, 0x02);
  const uint32_t t254 = LGX_LOP3(t248, t249, t253, 0x80);
  const uint32_t t255 = LGX_LOP3(s5_3, t140, t254, 0x8a);
  const uint32_t t258 = LGX_LOP3(t156, t164, 0u, 0xc0);
  const uint32_t t259 = LGX_LOP3(t49, t73, t258, 0x80);
  const uint32_t t262 = LGX_LOP3(t164, t173, 0u, 0xc0);
  const uint32_t t263 = LGX_LOP3(t67, t160, t262, 0x80);
  const uint32_t t265 = LGX_LOP3(s2, t218, t259, 0x70);
  const uint32_t t266 = LGX_LOP3(s2, t177, t263, 0x07);
  const uint32_t t267 = LGX_LOP3(t265, t266, 0u, 0x03);
  const uint32_t t270 = LGX_LOP3(t79, t113, t237, 0x80);
  const uint32_t t271 = LGX_LOP3(t131, t148, t201, 0x80);
  const uint32_t t273 = LGX_LOP3(s3_0, t270, t271, 0x70);
  const uint32_t t276 = LGX_LOP3(t57, t93, t197, 0x08);
  const uint32_t t277 = LGX_LOP3(t123, t148, t152, 0x80);
  const uint32_t t279 = LGX_LOP3(s3_1, t276, t277, 0x70);
  const uint32_t t281 = LGX_LOP3(t148, t165, 0u, 0x30);
  const uint32_t t282 = LGX_LOP3(t93, t119, t238, 0x80);
  const uint32_t t284 = LGX_LOP3(s3_2, t281, t282, 0x70);
  const uint32_t t285 = LGX_LOP3(s5_0, t140, 0u, 0x30);
  const uint32_t t287 = LGX_LOP3(s5_2, t140, 0u, 0x30);
  const uint32_t t289 = LGX_LOP3(s5_4, t140, 0u, 0x30);
  const uint32_t t290 = LGX_LOP3(n1, t212, t267, 0x2a);
  const uint32_t t293 = LGX_LOP3(s5_1, t99, t287, 0x45);
  const uint32_t t294 = LGX_LOP3(s5_3, t99, t289, 0x45);
  const uint32_t t295 = LGX_LOP3(t273, t279, t290, 0x02);
  const uint32_t t296 = LGX_LOP3(t284, t285, t293, 0x02);
  const uint32_t t298 = LGX_LOP3(t294, t295, t296, 0x80);
  const uint32_t t301 = LGX_LOP3(t35, t67, t187, 0x80);
  const uint32_t t303 = LGX_LOP3(t177, t262, t301, 0x80);
  const uint32_t t305 = LGX_LOP3(t49, t156, t188, 0x80);
  const uint32_t t306 = LGX_LOP3(t173, t305, 0u, 0xc0);
  const uint32_t t309 = LGX_LOP3(s2, t303, t306, 0xca);
  const uint32_t t311 = LGX_LOP3(t93, t123, t238, 0x80);
  const uint32_t t313 = LGX_LOP3(s3_0, t148, t311, 0x70);
  const uint32_t t314 = LGX_LOP3(t79, t86, 0u, 0xc0);
  const uint32_t t317 = LGX_LOP3(t93, t113, t314, 0x80);
  const uint32_t t318 = LGX_LOP3(t119, t131, t165, 0x40);
  const uint32_t t320 = LGX_LOP3(s3_1, t317, t318, 0x70);
  const uint32_t t322 = LGX_LOP3(t113, t123, t195, 0x80);
  const uint32_t t324 = LGX_LOP3(t199, t230, t322, 0x80);
  const uint32_t t326 = LGX_LOP3(s3_2, t165, t324, 0xd0);
  const uint32_t t329 = LGX_LOP3(n2, t212, t309, 0x2a);
  const uint32_t t331 = LGX_LOP3(s5_0, t99, t326, 0x45);
  const uint32_t t333 = LGX_LOP3(s5_4, t99, t247, 0x45);
  const uint32_t t334 = LGX_LOP3(t313, t320, t329, 0x02);
  const uint32_t t335 = LGX_LOP3(t245, t287, t331, 0x02);
  const uint32_t t337 = LGX_LOP3(t333, t334, t335, 0x80);
  const uint32_t t340 = LGX_LOP3(t42, t49, t187, 0x80);
  const uint32_t t342 = LGX_LOP3(t173, t188, t340, 0x80);
  const uint32_t t344 = LGX_LOP3(t35, t156, t215, 0x80);
  const uint32_t t345 = LGX_LOP3(t177, t344, 0u, 0xc0);
  const uint32_t t348 = LGX_LOP3(s2, t342, t345, 0xca);
  const uint32_t t349 = LGX_LOP3(t123, t127, 0u, 0xc0);
  const uint32_t t352 = LGX_LOP3(t131, t152, t165, 0x40);
  const uint32_t t353 = LGX_LOP3(t197, t202, t349, 0x80);
  const uint32_t t355 = LGX_LOP3(s3_0, t352, t353, 0x70);
  const uint32_t t357 = LGX_LOP3(t79, t123, t199, 0x80);
  const uint32_t t359 = LGX_LOP3(t165, t200, t357, 0x08);
  const uint32_t t362 = LGX_LOP3(s3_2, t123, t196, 0x70);
  const uint32_t t363 = LGX_LOP3(s5_1, t209, 0u, 0x30);
  const uint32_t t364 = LGX_LOP3(n3, t212, t348, 0x2a);
  const uint32_t t365 = LGX_LOP3(s3_1, t355, t359, 0x23);
  const uint32_t t367 = LGX_LOP3(s5_1, t209, t246, 0x45);
  const uint32_t t369 = LGX_LOP3(t285, t362, t367, 0x02);
  const uint32_t t370 = LGX_LOP3(t364, t365, t369, 0x80);
  const uint32_t t371 = LGX_LOP3(s5_4, t140, t370, 0x8a);
  const uint32_t t374 = LGX_LOP3(t35, t62, t187, 0x80);
  const uint32_t t376 = LGX_LOP3(t177, t188, t374, 0x80);
  const uint32_t t377 = LGX_LOP3(t42, t156, 0u, 0xc0);
  const uint32_t t379 = LGX_LOP3(t160, t169, t377, 0x80);
  const uint32_t t380 = LGX_LOP3(t173, t379, 0u, 0xc0);
  const uint32_t t383 = LGX_LOP3(s2, t376, t380, 0xca);
  const uint32_t t384 = LGX_LOP3(t127, t144, 0u, 0xc0);
  const uint32_t t386 = LGX_LOP3(t148, t165, t384, 0x20);
  const uint32_t t387 = LGX_LOP3(t198, t314, t386, 0x80);
  const uint32_t t388 = LGX_LOP3(s3_0, t387, 0u, 0x30);
  const uint32_t t390 = LGX_LOP3(t152, t231, t349, 0x80);
  const uint32_t t394 = LGX_LOP3(t79, t106, t199, 0x80);
  const uint32_t t395 = LGX_LOP3(t144, t165, t394, 0x20);
  const uint32_t t398 = LGX_LOP3(n4, t212, t383, 0x2a);
  const uint32_t t399 = LGX_LOP3(s3_1, t388, t390, 0x23);
  const uint32_t t400 = LGX_LOP3(s3_2, t244, t395, 0x23);
  const uint32_t t401 = LGX_LOP3(t398, t399, 0u, 0xc0);
  const uint32_t t403 = LGX_LOP3(t287, t400, t401, 0x08);
  const uint32_t t404 = LGX_LOP3(s5_3, t209, t403, 0x8a);
  const uint32_t t405 = LGX_LOP3(n5, t212, 0u, 0xc0);
  const uint32_t t407 = LGX_LOP3(t42, t73, t187, 0x80);
  const uint32_t t410 = LGX_LOP3(t62, t160, t188, 0x80);
  const uint32_t t412 = LGX_LOP3(s2, t218, t407, 0x70);
  const uint32_t t413 = LGX_LOP3(s2, t177, t410, 0x07);
  const uint32_t t416 = LGX_LOP3(t106, t127, t238, 0x80);
  const uint32_t t418 = LGX_LOP3(s3_0, t152, t416, 0x70);
  const uint32_t t421 = LGX_LOP3(t119, t144, t165, 0x40);
  const uint32_t t422 = LGX_LOP3(t197, t314, t421, 0x80);
  const uint32_t t425 = LGX_LOP3(t230, t384, 0u, 0xc0);
  const uint32_t t426 = LGX_LOP3(t198, t226, t425, 0x80);
  const uint32_t t428 = LGX_LOP3(s3_2, t165, t426, 0xd0);
  const uint32_t t430 = LGX_LOP3(t405, t412, t413, 0x01);
  const uint32_t t431 = LGX_LOP3(s3_1, t418, t422, 0x23);
  const uint32_t t434 = LGX_LOP3(t287, t363, t428, 0x01);
  const uint32_t t435 = LGX_LOP3(t430, t431, t434, 0x80);
  const uint32_t t436 = LGX_LOP3(s5_4, t209, t435, 0x8a);
  const uint32_t t437 = LGX_LOP3(n6, t212, 0u, 0xc0);
  const uint32_t t439 = LGX_LOP3(s3_0, t165, 0u, 0xc0);
  const uint32_t t441 = LGX_LOP3(t233, t238, t349, 0x80);
  const uint32_t t444 = LGX_LOP3(t228, t349, 0u, 0xc0);
  const uint32_t t446 = LGX_LOP3(t227, t314, t444, 0x80);
  const uint32_t t447 = LGX_LOP3(t165, t230, t238, 0x08);
  const uint32_t t449 = LGX_LOP3(s3_2, t446, t447, 0x70);
  const uint32_t t450 = LGX_LOP3(s2, t194, t437, 0x54);
  const uint32_t t451 = LGX_LOP3(s3_1, t439, t441, 0x23);
  const uint32_t t452 = LGX_LOP3(s5_3, s5_4, t209, 0xab);
  const uint32_t t454 = LGX_LOP3(t246, t449, 0u, 0x03);
  const uint32_t t455 = LGX_LOP3(t450, t451, t454, 0x80);
  const uint32_t t456 = LGX_LOP3(t452, t455, 0u, 0xc0);
  o[0] = ~t255;
  o[1] = ~t298;
  o[2] = ~t337;
  o[3] = ~t371;
  o[4] = ~t404;
  o[5] = ~t436;
  o[6] = ~t456;
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

// stats: lgx_collide_rest {'aig_ands': 440, 'lop3': 261, 'checked': 6144}; lgx_collide_norest {'aig_ands': 140, 'lop3': 83, 'checked': 6144}
