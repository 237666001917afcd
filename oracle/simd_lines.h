// Vector primitives of the reference's NEON line kernels
// (src/pixie/simd/neon.nim:6-28, used by the kernels of :427-700), restated
// with GCC vector extensions so the same source compiles to NEON on
// an aarch64 host and to SSE on x86.  TIMED CPU BASELINE ONLY: the bytes are
// those of a NEON pixie build (a multiply by alpha rounds, neon.nim:6-8),
// not the scalar semantics the oracle and the CUDA library share, and no
// parity claim rests on them.  Included by pxo.cpp, which holds the kernels.
//
// Each kernel keeps the reference's structure: scalar pixels until the line
// pointer is 16-byte aligned, blocks of 16 pixels while i < len - 16, then a
// scalar tail.  The 16-pixel blocks are held as four 16-byte vectors of
// interleaved RGBX (the reference de-interleaves with vld4q_u8; the per-byte
// arithmetic is the same, with each pixel's alpha broadcast to its bytes).
#pragma once
#include <cstdint>
#include <cstring>

namespace simd {

typedef uint8_t u8x16 __attribute__((vector_size(16)));
typedef uint16_t u16x8 __attribute__((vector_size(16)));

static inline u8x16 load16(const void* p) {
  u8x16 v;
  std::memcpy(&v, p, 16);
  return v;
}
static inline void store16(void* p, u8x16 v) { std::memcpy(p, &v, 16); }

// multiplyDiv255 (neon.nim:6-8): vraddhn_u16(ca, vrshrq_n_u16(ca, 8)), i.e.
// (ca + ((ca + 128) >> 8) + 128) >> 8 per byte, ca = c * a
static inline u8x16 mul_div255(u8x16 c, u8x16 a) {
  const u16x8 c0 = __builtin_convertvector(__builtin_shufflevector(c, c, 0, 1, 2, 3, 4, 5, 6, 7), u16x8);
  const u16x8 c1 = __builtin_convertvector(__builtin_shufflevector(c, c, 8, 9, 10, 11, 12, 13, 14, 15), u16x8);
  const u16x8 a0 = __builtin_convertvector(__builtin_shufflevector(a, a, 0, 1, 2, 3, 4, 5, 6, 7), u16x8);
  const u16x8 a1 = __builtin_convertvector(__builtin_shufflevector(a, a, 8, 9, 10, 11, 12, 13, 14, 15), u16x8);
  u16x8 p0 = c0 * a0, p1 = c1 * a1;
  p0 = (p0 + ((p0 + 128) >> 8) + 128) >> 8;
  p1 = (p1 + ((p1 + 128) >> 8) + 128) >> 8;
  typedef uint8_t u8x8 __attribute__((vector_size(8)));
  const u8x8 n0 = __builtin_convertvector(p0, u8x8), n1 = __builtin_convertvector(p1, u8x8);
  return __builtin_shufflevector(n0, n1, 0, 1, 2, 3, 4, 5, 6, 7, 8, 9, 10, 11, 12, 13, 14, 15);
}
// each pixel's alpha byte in all four of its bytes
static inline u8x16 alpha_bcast(u8x16 v) {
  return __builtin_shufflevector(v, v, 3, 3, 3, 3, 7, 7, 7, 7, 11, 11, 11, 11, 15, 15, 15, 15);
}
static inline bool all_alpha(u8x16 v, uint8_t x) {
  const u8x16 a = alpha_bcast(v);
  for (int i = 0; i < 16; i += 4)
    if (a[i] != x) return false;
  return true;
}
// blendNormalSimd (neon.nim:16-28): backdrop * (255 - source.a) / 255 + source
static inline u8x16 normal4(u8x16 bd, u8x16 src) {
  const u8x16 k = (u8x16{} + 255) - alpha_bcast(src);
  return mul_div255(bd, k) + src;
}

}  // namespace simd
