// mhsw_batch.h -- the batched (length-bucketed, persistent, work-stealing) forward form.
#pragma once
#include <cstdint>
#include <string>
#include <cuda_runtime.h>

#include "mhsw_types.h"

namespace mhsw {

struct WorkLists;
struct Forks;

// One tuned launch shape of the persistent kernel.
struct BatchShape {
  int groups_per_block = 16;  // block size in units of 8 threads
  int blocks_per_sm = 0;      // 0 = occupancy maximum
};

struct BatchState {
  std::string err;
  uint32_t *keys_in = nullptr, *keys_out = nullptr;
  uint32_t *idx_in = nullptr, *idx_out = nullptr;
  void *temp = nullptr;
  size_t temp_bytes = 0;
  size_t cap = 0;
  int *queue = nullptr;
  void *scratch = nullptr;  // strip scratch for A longer than one strip
  size_t scratch_bytes = 0;
  BatchShape shape;
  bool tuned = false;
  bool autotune = true;
  double tune_ms[8] = {0};  // measured candidates (diagnostics)
  int tune_n = 0;
  void release();
};

// Forward pass of the batched form: computes bucket keys (rows-per-lane class of A,
// then descending B length), sorts the pair order on the device, and runs the
// persistent kernel whose lane groups claim pairs from one atomic queue.  Pairs whose
// score could exceed the int16 ceiling go straight to the int32 list wl.ovf.
// The first call tunes the launch shape (groups per block, blocks per SM) on the batch.
// With side streams (fk), the two persistent launches (8-lane and 16-lane groups) run
// concurrently, so the tail of one fills with the other.
int batched_forward(BatchState &bs, int device, const PairSet &ps, const ResultSet &rs, const WorkLists &wl,
                    const Scoring &sc, int ceiling, int max_a, int max_b, cudaStream_t st, int64_t *launches,
                    const Forks *fk = nullptr);

}  // namespace mhsw
