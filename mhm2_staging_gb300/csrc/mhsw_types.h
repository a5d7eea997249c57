// mhsw_types.h -- plain data types shared by the kernels and the host driver.
#pragma once
#include <cstdint>

namespace mhsw {

enum : int { kCodeN = 4, kCodePad = 5, kNumCodes = 6 };

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
  const uint8_t *a_code;
  const uint8_t *b_code;
};

struct ResultSet {  // device pointers, one entry per pair
  int32_t *score, *a_end, *b_end, *a_beg, *b_beg;
  uint32_t *flag;
};

}  // namespace mhsw
