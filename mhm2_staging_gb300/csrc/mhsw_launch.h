// mhsw_launch.h -- host-side launch entry points of the alignment kernels (internal).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace mhsw {

struct Scoring;
struct PairSet;
struct ResultSet;

constexpr int kBandClasses = 7;  // banded begin-pass instantiations (half-widths 3 .. 31)

// Work lists built on the device (no host round trip between passes).
struct WorkLists {
  int64_t *ovf;       // pairs whose int16 forward pass crossed the ceiling
  int *ovf_count;
  int64_t *wide;      // pairs whose reverse band is wider than the banded kernels handle
  int *wide_count;
  int64_t *bands;     // begin-pass pairs grouped by band class (one segment per class)
  int *band_counts;   // kBandClasses pair counts, then kBandClasses scatter cursors
  int64_t cap;        // capacity of each list
};

struct FwdConfig {
  int K;              // packed cell pairs per lane (rows per lane = 2K)
  int G;              // lanes per pair
  int groups_per_block;
  int bcap;           // per-group B code buffer bytes (>= pad + maxB + 2G)
  int pad;            // leading PAD entries
  int grid;           // blocks (grid-stride over pairs)
  size_t smem;        // dynamic shared memory bytes
  bool keyed;         // int16 forward uses the keyed engine (mhsw_engine16.cuh)
};

// Upper bound of B length the forward kernels accept (shared-memory code buffer).
constexpr int kMaxB = 65000;

// Side streams of one driver handle, for launches that may overlap on the device (the
// two persistent forward launches; the band classes of the begin pass).  Work forked
// onto them waits for everything issued on the main stream before the fork, and the
// main stream waits for all of it at the join, so the main stream's order is kept.
constexpr int kSideStreams = 8;
struct Forks {
  cudaStream_t side[kSideStreams] = {};
  cudaEvent_t fork = nullptr;
  cudaEvent_t join[kSideStreams] = {};
};
cudaError_t forks_create(Forks &f);
void forks_destroy(Forks &f);
// Side streams 0 .. k-1 wait for the work issued so far on st.
cudaError_t fork_to(const Forks &f, cudaStream_t st, int k);
// st waits for the work issued so far on side streams 0 .. k-1.
cudaError_t join_from(const Forks &f, cudaStream_t st, int k);

// Raises a kernel's dynamic shared-memory limit to at least `bytes` on the current
// device (no-op at or below the 48 KB default).  The limit only ever grows, so host
// threads launching the same kernel with different block shapes never lower it under
// one another's launch.
cudaError_t raise_smem_limit(const void *func, size_t bytes);

// Chooses K/G/grid/smem for a forward launch over pairs whose A (rows) lengths are at
// most max_a and B lengths at most max_b.  wide32 selects the int32 engine.
// s2: score2 mode (the keyed profile table gains the zero-score code).
cudaError_t plan_forward(int device, int max_a, int max_b, bool wide32, FwdConfig *cfg, bool keyed = false,
                         bool s2 = false);
// Second-best scores (score2 mode) from the row maxima the forward pass wrote.
cudaError_t launch_score2(const PairSet &ps, const ResultSet &rs, const Scoring &sc, cudaStream_t st);

// Bytes of strip scratch a forward launch needs (0 when A fits one strip).
size_t forward_scratch_bytes(const FwdConfig &cfg, int max_a, int max_b, bool wide32);

// Forward pass (int16, or int32 when wide32) over pairs [0, n) or over the device list
// (list != nullptr, count read on the device).  Writes score, a_end, b_end, flag.
cudaError_t launch_forward(const FwdConfig &cfg, bool wide32, const PairSet &ps, const ResultSet &rs,
                           const Scoring &sc, const int64_t *list, const int *list_count, int ceiling,
                           void *scratch, const WorkLists &wl, cudaStream_t st);

// True when the keyed int16 engine (mhsw_engine16.cuh) can run this scoring: every
// substitution score plus the gap-open penalty is non-negative.
bool keyed_scoring(const Scoring &sc);

// Begin pass: banded thread-per-pair kernels (bands of up to 16, 32, 64 cells, each
// escalating to the next), then the wavefront kernel on reversed prefixes for the pairs
// left in wl.wide.  order (may be null) is the pair order of the first kernel.
cudaError_t launch_reverse(int device, const PairSet &ps, const ResultSet &rs, const Scoring &sc, int max_a,
                           int max_b, void *scratch, size_t scratch_bytes, const WorkLists &wl, cudaStream_t st,
                           const uint32_t *order, const Forks *fk = nullptr);

// Raw bytes -> base codes (0..4) for one arena.
cudaError_t launch_translate(const char *src, uint8_t *dst, int64_t nbytes, cudaStream_t st);

// Clears the device work-list counters.
cudaError_t reset_lists(const WorkLists &wl, cudaStream_t st);

// Output views in the caller's orientation (see mhsw.h).  out_* may be null.
struct OutViews {
  int16_t *s_score, *s_ref_beg, *s_ref_end, *s_qry_beg, *s_qry_end;
  int32_t *w_score, *w_ref_beg, *w_ref_end, *w_qry_beg, *w_qry_end;
};
// a_is_query: A (SSW ref) is the caller's query (klign: reads); else A is the caller's ref.
// part: 1 = ends + score, 2 = begins, 3 = all.
cudaError_t launch_finalize(const ResultSet &rs, int64_t n, bool a_is_query, int part, const OutViews &ov,
                            cudaStream_t st);

// Packs results into n x 5 int32 rows (score, a_beg, a_end, b_beg, b_end).
cudaError_t launch_pack5(const ResultSet &rs, int64_t n, int32_t *out5, cudaStream_t st);

// ---- CIGAR pass (mhsw_cigar.cu) ----------------------------------------------------
constexpr int kCigarClasses = 6;     // register-band traceback kernels, half-widths 1, 2, 4, 8, 16, 31
constexpr int kCigarRowCap = 512;    // box rows those kernels keep directions for
// Counters: [0] diagonal boxes (their CIGAR needs no DP; the first segment of the sorted
// pair order), [1 .. kCigarClasses] the pairs each register kernel takes first (its
// segment), then the generic list size, pairs that found the arena full, tracebacks that
// left the computed band, and [kCigarEsc ..] each register kernel's escalation list size
// (pairs whose band outgrew a narrower kernel).
constexpr int kCigarSegments = kCigarClasses + 1;
constexpr int kCigarGeneric = kCigarSegments;
constexpr int kCigarArenaFull = kCigarSegments + 1;
constexpr int kCigarWalkErrors = kCigarSegments + 2;
constexpr int kCigarEsc = kCigarSegments + 3;
constexpr int kCigarCounters = kCigarEsc + kCigarClasses;
constexpr size_t kCigarDirBudget = size_t(256) << 20;  // direction scratch of the register kernels

// Generic-kernel slice of one pair at half-width w: H and E rows plus 4-bit directions.
__host__ __device__ inline size_t cigar_slice_bytes(int w, int rows) {
  return 4 * (2 * (size_t)(2 * w + 2) + (size_t)rows * (size_t)((2 * w + 1 + 7) / 8));
}

struct CigarBufs {           // device buffers of the CIGAR pass
  int32_t *nops, *mism;      // per pair: op count (0 none, -1 not computed) and mismatches
  int64_t *op_off;           // per pair: first op in the arena
  uint32_t *arena;           // BAM-encoded ops, in completion order
  int64_t arena_cap;
  unsigned long long *cursor;
  int *counts;               // kCigarCounters
  uint32_t *keys_in, *keys_out, *idx_in, *idx_out;  // n each: (class, rows) sort of the pairs
  void *sort_temp;
  size_t sort_temp_bytes;
  int2 *lists;               // kCigarClasses escalation lists of list_cap (pair, half-width) entries
  int64_t list_cap;
  int4 *generic;             // generic list: (pair, half-width, rows, columns), list_cap entries
  uint32_t *dirs;            // direction scratch, dirs_bytes
  size_t dirs_bytes;
};

// Classification and the register-band kernels (no host synchronisation).  Pairs left
// for the generic kernel are in cb.generic (count in cb.counts[kCigarGeneric]).  order
// (may be null): a pair order to classify in (the batched forward pass's sorted order).
cudaError_t launch_cigar(const PairSet &ps, const ResultSet &rs, const Scoring &sc, const CigarBufs &cb, int sms,
                         const uint32_t *order, cudaStream_t st, int64_t *launches);
// Temporary bytes of the (class, rows) sort of n pairs.
cudaError_t cigar_sort_temp_bytes(int64_t n, size_t *bytes);
// Generic kernel over `count` entries (device copy), `threads` threads with a slice of
// `slice` bytes each in `pool`.
cudaError_t launch_cigar_generic(const PairSet &ps, const ResultSet &rs, const Scoring &sc, const CigarBufs &cb,
                                 const int4 *entries, int count, int threads, size_t slice, void *pool,
                                 cudaStream_t st);
// Pair-order copy: ord_off[0..n] = exclusive sum of the op counts, ord_ops = the ops in
// pair order (ord_ops may be null to get the offsets only).  c64: n + 1 int64 scratch.
cudaError_t cigar_gather_temp_bytes(int64_t n, size_t *bytes);
cudaError_t launch_cigar_gather(const CigarBufs &cb, int64_t n, int64_t *c64, int64_t *ord_off, uint32_t *ord_ops,
                                void *temp, size_t temp_bytes, cudaStream_t st);

int launches_per_batch();

}  // namespace mhsw
