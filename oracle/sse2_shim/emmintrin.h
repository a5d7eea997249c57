/* emmintrin.h -- the SSE2 subset the reference's CPU aligner uses, for hosts without SSE2.
 *
 * TEST INFRASTRUCTURE ONLY (the timed CPU baseline and its parity check).  The
 * reference's striped Smith-Waterman (src/ssw/ssw_core.cpp) has only an x86_64 (SSE2)
 * and a PowerPC (AltiVec) branch; the GB300's host is aarch64.  This header stands in
 * for <emmintrin.h> when oracle/Makefile compiles that source for such a host: on
 * aarch64 every operation is one or a few NEON instructions; elsewhere it is written
 * with portable GCC vector extensions, which lets the x86_64 container check the
 * shim's semantics against the genuine SSE2 build bit for bit.
 *
 * The 18 operations and __m128i, with SSE2's semantics (Intel's intrinsics guide):
 *   saturating adds/subtracts: adds_epi16, adds_epu8, subs_epu8, subs_epu16;
 *   lane compares giving all-ones masks: cmpeq_epi8, cmpeq_epi16, cmpgt_epi16;
 *   lane maxima: max_epi16, max_epu8;  broadcasts: set1_epi8/16/32;
 *   whole-register byte shifts filling zeros: slli_si128 (towards higher lanes),
 *   srli_si128 (towards lower lanes);  movemask_epi8 (bit i = top bit of byte i);
 *   extract_epi16 (lane, zero-extended);  aligned load/store.
 */
#ifndef MHSW_SSE2_SHIM_EMMINTRIN_H
#define MHSW_SSE2_SHIM_EMMINTRIN_H

#include <stdint.h>
#include <string.h>

#if defined(__aarch64__)
#include <arm_neon.h>

typedef uint8x16_t __m128i;

#define MHSW_S16(x) vreinterpretq_s16_u8(x)
#define MHSW_U16(x) vreinterpretq_u16_u8(x)
#define MHSW_B(x) vreinterpretq_u8_s16(x)
#define MHSW_BU(x) vreinterpretq_u8_u16(x)

static inline __m128i _mm_adds_epi16(__m128i a, __m128i b) { return MHSW_B(vqaddq_s16(MHSW_S16(a), MHSW_S16(b))); }
static inline __m128i _mm_adds_epu8(__m128i a, __m128i b) { return vqaddq_u8(a, b); }
static inline __m128i _mm_subs_epu8(__m128i a, __m128i b) { return vqsubq_u8(a, b); }
static inline __m128i _mm_subs_epu16(__m128i a, __m128i b) { return MHSW_BU(vqsubq_u16(MHSW_U16(a), MHSW_U16(b))); }
static inline __m128i _mm_cmpeq_epi8(__m128i a, __m128i b) { return vceqq_u8(a, b); }
static inline __m128i _mm_cmpeq_epi16(__m128i a, __m128i b) { return MHSW_BU(vceqq_s16(MHSW_S16(a), MHSW_S16(b))); }
static inline __m128i _mm_cmpgt_epi16(__m128i a, __m128i b) { return MHSW_BU(vcgtq_s16(MHSW_S16(a), MHSW_S16(b))); }
static inline __m128i _mm_max_epi16(__m128i a, __m128i b) { return MHSW_B(vmaxq_s16(MHSW_S16(a), MHSW_S16(b))); }
static inline __m128i _mm_max_epu8(__m128i a, __m128i b) { return vmaxq_u8(a, b); }
static inline __m128i _mm_set1_epi8(char v) { return vdupq_n_u8((uint8_t)v); }
static inline __m128i _mm_set1_epi16(short v) { return MHSW_B(vdupq_n_s16(v)); }
static inline __m128i _mm_set1_epi32(int v) { return vreinterpretq_u8_s32(vdupq_n_s32(v)); }
static inline __m128i _mm_load_si128(const __m128i *p) { return vld1q_u8((const uint8_t *)p); }
static inline void _mm_store_si128(__m128i *p, __m128i a) { vst1q_u8((uint8_t *)p, a); }
static inline int _mm_movemask_epi8(__m128i a) {
  /* each byte's top bit moved to bit (i mod 8), then the two halves summed */
  static const int8_t kShift[16] = {0, 1, 2, 3, 4, 5, 6, 7, 0, 1, 2, 3, 4, 5, 6, 7};
  const uint8x16_t bits = vshlq_u8(vshrq_n_u8(a, 7), vld1q_s8(kShift));
  return (int)vaddv_u8(vget_low_u8(bits)) | ((int)vaddv_u8(vget_high_u8(bits)) << 8);
}
/* byte shifts by a constant 1..15: vext takes the top bytes of its first operand and
 * the low bytes of its second */
#define _mm_slli_si128(a, imm) vextq_u8(vdupq_n_u8(0), (a), 16 - (imm))
#define _mm_srli_si128(a, imm) vextq_u8((a), vdupq_n_u8(0), (imm))
#define _mm_extract_epi16(a, imm) ((int)vgetq_lane_u16(MHSW_U16(a), (imm)))

#else /* portable GCC vectors */

typedef long long __m128i __attribute__((__vector_size__(16), __may_alias__));
typedef uint8_t mhsw_u8x16 __attribute__((__vector_size__(16), __may_alias__));
typedef int8_t mhsw_s8x16 __attribute__((__vector_size__(16), __may_alias__));
typedef uint16_t mhsw_u16x8 __attribute__((__vector_size__(16), __may_alias__));
typedef int16_t mhsw_s16x8 __attribute__((__vector_size__(16), __may_alias__));
typedef int32_t mhsw_s32x4 __attribute__((__vector_size__(16), __may_alias__));

static inline __m128i _mm_adds_epi16(__m128i a, __m128i b) {
  const mhsw_s16x8 x = (mhsw_s16x8)a, y = (mhsw_s16x8)b;
  mhsw_s16x8 r;
  for (int i = 0; i < 8; i++) {
    const int v = (int)x[i] + (int)y[i];
    r[i] = (int16_t)(v > 32767 ? 32767 : (v < -32768 ? -32768 : v));
  }
  return (__m128i)r;
}
static inline __m128i _mm_adds_epu8(__m128i a, __m128i b) {
  const mhsw_u8x16 x = (mhsw_u8x16)a, y = (mhsw_u8x16)b, s = x + y;
  return (__m128i)(s | (mhsw_u8x16)(s < x));
}
static inline __m128i _mm_subs_epu8(__m128i a, __m128i b) {
  const mhsw_u8x16 x = (mhsw_u8x16)a, y = (mhsw_u8x16)b;
  return (__m128i)((x - y) & (mhsw_u8x16)(x > y));
}
static inline __m128i _mm_subs_epu16(__m128i a, __m128i b) {
  const mhsw_u16x8 x = (mhsw_u16x8)a, y = (mhsw_u16x8)b;
  return (__m128i)((x - y) & (mhsw_u16x8)(x > y));
}
static inline __m128i _mm_cmpeq_epi8(__m128i a, __m128i b) { return (__m128i)((mhsw_s8x16)a == (mhsw_s8x16)b); }
static inline __m128i _mm_cmpeq_epi16(__m128i a, __m128i b) { return (__m128i)((mhsw_s16x8)a == (mhsw_s16x8)b); }
static inline __m128i _mm_cmpgt_epi16(__m128i a, __m128i b) { return (__m128i)((mhsw_s16x8)a > (mhsw_s16x8)b); }
static inline __m128i _mm_max_epi16(__m128i a, __m128i b) {
  const mhsw_s16x8 x = (mhsw_s16x8)a, y = (mhsw_s16x8)b;
  return (__m128i)(x > y ? x : y);
}
static inline __m128i _mm_max_epu8(__m128i a, __m128i b) {
  const mhsw_u8x16 x = (mhsw_u8x16)a, y = (mhsw_u8x16)b;
  return (__m128i)(x > y ? x : y);
}
static inline __m128i _mm_set1_epi8(char v) {
  mhsw_u8x16 r;
  for (int i = 0; i < 16; i++) r[i] = (uint8_t)v;
  return (__m128i)r;
}
static inline __m128i _mm_set1_epi16(short v) {
  mhsw_s16x8 r;
  for (int i = 0; i < 8; i++) r[i] = v;
  return (__m128i)r;
}
static inline __m128i _mm_set1_epi32(int v) {
  mhsw_s32x4 r;
  for (int i = 0; i < 4; i++) r[i] = v;
  return (__m128i)r;
}
static inline __m128i _mm_load_si128(const __m128i *p) { return *p; }
static inline void _mm_store_si128(__m128i *p, __m128i a) { *p = a; }
static inline int _mm_movemask_epi8(__m128i a) {
  const mhsw_u8x16 x = (mhsw_u8x16)a;
  int m = 0;
  for (int i = 0; i < 16; i++) m |= (int)(x[i] >> 7) << i;
  return m;
}
static inline __m128i mhsw_bytes_shift(__m128i a, int left, int n) {
  uint8_t in[16], out[16];
  memcpy(in, &a, 16);
  for (int i = 0; i < 16; i++) {
    const int from = left ? i - n : i + n;
    out[i] = (from >= 0 && from < 16) ? in[from] : 0;
  }
  __m128i r;
  memcpy(&r, out, 16);
  return r;
}
#define _mm_slli_si128(a, imm) mhsw_bytes_shift((a), 1, (imm))
#define _mm_srli_si128(a, imm) mhsw_bytes_shift((a), 0, (imm))
#define _mm_extract_epi16(a, imm) ((int)(uint16_t)((mhsw_s16x8)(a))[(imm)])

#endif
#endif /* MHSW_SSE2_SHIM_EMMINTRIN_H */
