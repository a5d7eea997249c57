// mhsw_types.h -- plain data types shared by the kernels and the host driver.
#pragma once
#include <cstdint>

namespace mhsw {

// Codes 0..3 = A, C, G, T; 4 = N (any other byte); 5 = PAD (outside the matrix);
// 6 = zero score (SSW's query padding, score2 mode of the generic engine).
enum : int { kCodeN = 4, kCodePad = 5, kCodeZeroPad = 6, kNumCodes = 7 };

// Penalties are positive magnitudes (klign passes them negated; the driver flips them).
struct Scoring {
  int match, mismatch, gap_open, gap_extend, ambiguity;
};

// Result record flags.
enum : uint32_t {
  kFlagOverflow16 = 1u,   // int16 ceiling crossed: forward pass re-run in int32
  kFlagRevWide = 2u,      // reverse band wider than the banded kernel's limit
  kFlagTooLong = 4u,      // sequence beyond the engine limits (error)
};

struct PairSet {  // device pointers; A = SSW ref (rows), B = SSW query (columns)
  const char *a_seq;
  const int64_t *a_off;
  const int32_t *a_len;
  const char *b_seq;
  const int64_t *b_off;
  const int32_t *b_len;
  int64_t n;
  // Base codes (0..4, SSW's translation) at the same offsets as the raw bytes; filled
  // once per batch by the translation kernel and read by every alignment kernel.
  const uint8_t *a_code = nullptr;
  const uint8_t *b_code = nullptr;
  // Score2 mode (null otherwise): per A row of each pair, at the A offsets, the row's
  // maximum over B padded as SSW's byte path (rowmax16) and word path (rowmax8) pad it.
  int32_t *rowmax16 = nullptr;
  int32_t *rowmax8 = nullptr;
};

struct ResultSet {  // device pointers, one entry per pair
  int32_t *score, *a_end, *b_end, *a_beg, *b_beg;
  uint32_t *flag;
  int32_t *score2 = nullptr, *a_end2 = nullptr;  // score2 mode: SSW's second-best score and its A row
};

// SSW's byte-path bias (-min of its score matrix) and its query padding: the byte path
// pads B to a multiple of 16, the word path (scores + bias >= 255) to a multiple of 8
// (ssw_core.cpp:178, :549, :476, :1129-1133).
__host__ __device__ inline int ssw_bias(const Scoring &s) {
  const int b = s.mismatch > s.ambiguity ? s.mismatch : s.ambiguity;
  return b > 0 ? b : 0;
}
__host__ __device__ inline int ssw_pad16(int n) { return (n + 15) / 16 * 16; }
__host__ __device__ inline int ssw_pad8(int n) { return (n + 7) / 8 * 8; }

}  // namespace mhsw
