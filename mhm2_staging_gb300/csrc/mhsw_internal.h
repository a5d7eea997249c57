// mhsw_internal.h -- entry points shared between the library's own translation units
// (not part of the C ABI).
#pragma once
#include <cstdint>
#include <mutex>

#include "../../include/mhsw.h"
#include "mhsw_types.h"

namespace mhsw {

// Aligns a device-resident batch on a driver handle whose A side is raw bytes
// (ps.a_seq, translated here into the handle's code buffer) and whose B side is an
// already translated code arena that stays resident across calls (ps.b_code; ps.b_seq
// is not read).  Forward and begin passes run on the handle's stream; out5_dev (device,
// 5 int32 per pair: score, a_begin, a_end, b_begin, b_end) is written by the last
// kernel.  Returns without waiting: the caller synchronises the handle's stream.
int align_resident(mhsw_driver *d, const PairSet &ps, int64_t a_bytes, int max_a, int max_b, int form,
                   int32_t *out5_dev);

// The handle's stream (cudaStream_t) and device.
void *driver_stream(mhsw_driver *d);
int driver_device(mhsw_driver *d);
// The handle's form for batch calls (MHSW_FORM_*) and match score.
int driver_form(mhsw_driver *d);
int driver_match(mhsw_driver *d);
// The handle's gap penalties as positive magnitudes.
void driver_gaps(mhsw_driver *d, int *gap_open, int *gap_extend);
// CIGAR mode: runs the CIGAR pass over the batch of the last align_resident call (after
// its stream work; synchronous); its CIGARs are then what mhsw_last_cigar returns.
// Returns MHSW_ERR_STATE when the handle is not in CIGAR mode.
int cigar_resident(mhsw_driver *d, const PairSet &ps);
bool driver_cigar(mhsw_driver *d);
// After the stream work of an align_resident call (and its CIGAR pass) completed: its
// device times into the handle's mhsw_timing (translation to end of the begin pass).
void resident_timing(mhsw_driver *d);
// Device arena of at least `bytes` for one call's own arrays (the caller side, the protein
// entry point), kept on the handle between calls (grown when a batch needs more, never
// shrunk); nullptr when the allocation fails.  Its contents are only valid during one call.
unsigned char *driver_call_arena(mhsw_driver *d, size_t bytes);
// Held by a call that uses the call arena, for the whole call (taken before the handle's
// own lock, which the resident-batch functions above take inside), so calls that share a
// handle stay serialised.
std::mutex &driver_call_mutex(mhsw_driver *d);
// Lays arrays out back to back at 256-byte boundaries: with base == nullptr it only sums
// their sizes (off), otherwise it also hands out the pointers.
struct Carve {
  size_t off = 0;
  unsigned char *base = nullptr;
  template <class T>
  void take(T **p, size_t count) {
    const size_t at = off;
    off += ((count > 0 ? count : 1) * sizeof(T) + 255) & ~size_t(255);
    *p = base ? reinterpret_cast<T *>(base + at) : nullptr;
  }
};
// The A codes the last align_resident call translated (device).
const uint8_t *driver_a_codes(mhsw_driver *d);
// Second-best scores (device, n entries) of the last align_resident call when the handle
// is in score2 mode, else null.
const int32_t *driver_score2(mhsw_driver *d, int64_t n);

}  // namespace mhsw
