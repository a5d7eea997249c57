// mhsw_batch.h -- the batched (length-bucketed, persistent, work-stealing) forward form.
#pragma once
#include <cstdint>
#include <string>
#include <cuda_runtime.h>

#include "mhsw_types.h"

namespace mhsw {

struct WorkLists;
struct Forks;

// One tuned configuration of the persistent kernels.
struct BatchShape {
  int groups_per_block = 16;  // block size in units of 8 threads
  int blocks_per_sm = 0;      // 0 = occupancy maximum
  int lane_rows = 160;        // longest A (rows) given to 8-lane groups; longer A runs in 16-lane groups
  bool wide_try16 = false;    // pairs whose score bound exceeds the int16 keys: int16 first (re-run on
                              // overflow) instead of straight to int32
};

// What the tuner keys on: the batch's A-length mix over the kernels' row classes (fractions
// of a sample of the lengths; all -1 when the lengths are not visible to the host, i.e. a
// device batch with size hints), the row class of its longest A, its longest B and its
// size.  Two signatures describe the same workload when the longest A falls in the same
// row class, the longest B within a factor of 2, the sizes within a factor of 8 (any two
// of at most 65,536 pairs count as alike) and, where both mixes are known, no class fraction
// moved by more than 0.15; ratios rather than fixed class edges keep batches that
// straddle an edge (serving micro-batches of 1k..64k pairs) from re-tuning in turn.
constexpr int kSigClasses = 8;
struct BatchSignature {
  float a_mix[kSigClasses] = {-1, -1, -1, -1, -1, -1, -1, -1};
  int max_a_class = -1, max_a = 0, max_b = 0;
  int64_t n = 0;
  static constexpr float kTolerance = 0.15f;
  bool close_to(const BatchSignature &o) const;
};
// Row class of an A length for the signature (0..7: up to 64, 96, 128, 160, 192, 256,
// 1024 rows, longer).
int signature_class(int a_len);
// Signature from host-visible lengths (a strided sample of at most 4096 pairs), or from
// the longest lengths alone when a_len is null.
BatchSignature batch_signature(const int32_t *a_len, int64_t n, int max_a, int max_b);

// Result of the last tuning (diagnostics, also returned through the C ABI).
struct TuneRecord {
  int trials = 0;
  int64_t sample_pairs = 0;
  double wall_ms = 0;  // host wall time the tuning added to its call
  float trial_ms[16] = {0};
  int64_t tunings = 0;  // tunings by this handle so far
  bool last_call_tuned = false;
};

struct BatchState {
  std::string err;
  uint32_t *keys_in = nullptr, *keys_out = nullptr;
  uint32_t *idx_in = nullptr, *idx_out = nullptr;
  void *temp = nullptr;
  size_t temp_bytes = 0;
  size_t cap = 0;
  // the tuner's sample of the batch (sorted like the batch), its sort space
  uint32_t *s_keys_in = nullptr, *s_keys_out = nullptr, *s_idx_in = nullptr, *s_idx_out = nullptr;
  void *s_temp = nullptr;
  size_t s_temp_bytes = 0;
  int *s_hist = nullptr;  // bucket counts of the sample (device), read by the tuner
  int *queue = nullptr;
  void *scratch = nullptr;  // strip scratch for A longer than one strip
  size_t scratch_bytes = 0;
  BatchShape shape;
  BatchSignature tuned_for;
  bool tuned = false;
  bool autotune = true;
  // the last kCached tuned configurations, taken back without trials for a batch whose
  // signature is close to one of theirs
  struct Tuned {
    BatchSignature sig;
    BatchShape shape;
  };
  static constexpr int kCached = 8;
  Tuned cached[kCached];
  int n_cached = 0, next_cached = 0;
  TuneRecord tune;
  void release();
};

// Forward pass of the batched form: computes bucket keys (rows-per-lane class of A,
// then descending B length), sorts the pair order on the device, and runs the
// persistent kernel whose lane groups claim pairs from one atomic queue.  Pairs whose
// score could exceed the int16 ceiling go straight to the int32 list wl.ovf.
// A call whose batch signature differs from the one the handle last tuned for takes back
// the configuration of a close earlier signature (the last eight are kept), or else runs
// the tuner first: timed trials of the persistent kernels on a strided sample of the batch
// (at most 256k pairs) over the launch shape (groups per block, blocks per SM), the row
// threshold between 8- and 16-lane groups (the rows each lane holds follow from it), and,
// when the sample holds pairs whose score bound exceeds the int16 keys, their int16/int32
// split; the fastest configuration is kept.
// With side streams (fk), the two persistent launches (8-lane and 16-lane groups) run
// concurrently, so the tail of one fills with the other.
int batched_forward(BatchState &bs, int device, const PairSet &ps, const ResultSet &rs, const WorkLists &wl,
                    const Scoring &sc, int ceiling, int max_a, int max_b, const BatchSignature &sig,
                    cudaStream_t st, int64_t *launches, const Forks *fk = nullptr);

}  // namespace mhsw
