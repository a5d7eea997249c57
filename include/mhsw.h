/*
 * mhsw.h -- C ABI of the GB300 read-to-contig Smith-Waterman driver.
 *
 * It replaces MHM2's ADEPT GPU aligner behind klign (reference
 * src/adept-sw/driver.hpp:14-57, src/adept-sw/driver.cpp:28-417) with results that
 * are bit-exact against the reference's CPU aligner
 * (StripedSmithWaterman::Aligner::Align with Filter(true, false, 0, 32767),
 * src/ssw/ssw.cpp:431-469, as klign calls it at src/klign.cpp:257).
 *
 * Conventions
 *   - Every call returns an int status (MHSW_OK == 0); nothing throws across the ABI.
 *     mhsw_driver_last_error() gives the message of the last failure on a handle.
 *   - Scores are passed the way klign passes them to the reference GPU driver
 *     (src/klign.cpp:464-465): match positive, penalties negated (e.g. 1, -3, -5, -2).
 *   - "A" is the sequence SSW treats as its reference (the outer loop of
 *     sw_sse2_byte, src/ssw/ssw_core.cpp:296) and "B" the one it profiles (its query).
 *     klign calls Align(contig, read, ...) (src/klign.cpp:257), so in klign's
 *     orientation A = read and B = contig window.  Tie-breaks follow SSW's roles.
 *   - A handle serialises its own calls; use one handle per host thread.  Calls that
 *     keep device state on the handle between their own steps (mhsw_klign_align and the
 *     protein entry point) also hold the handle for their whole call, so two threads may
 *     share a handle for those; mixing them on a shared handle with the batch calls
 *     (mhsw_align_pairs and its result readers) is not supported.
 *   - Result arrays returned by mhsw_get_aln_results() are owned by the handle and stay
 *     valid until the next mhsw_run_kernel_* call or mhsw_driver_destroy().
 */
#ifndef MHSW_H_
#define MHSW_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ---------------------------------------------------------- */
#define MHSW_OK 0
#define MHSW_ERR_CUDA 1      /* a CUDA runtime call failed */
#define MHSW_ERR_ARG 2       /* invalid argument */
#define MHSW_ERR_STATE 3     /* call out of order (e.g. backwards before forwards) */
#define MHSW_ERR_NOMEM 4     /* host or device allocation failed */
#define MHSW_ERR_LIMIT 5     /* a sequence exceeds the engine limits (see mhsw_limits) */
#define MHSW_ERR_NO_GPU 6    /* no CUDA device */
#define MHSW_ERR_INTERNAL 7  /* internal consistency check failed */
#define MHSW_ERR_BUSY 8      /* serving queue full (submit with MHSW_SUBMIT_NOWAIT) */

/* ---- orientation ----------------------------------------------------------- */
/* klign (default): reads are SSW's ref (A), contigs its query (B); results map
 * query_* <- read coordinates, ref_* <- contig coordinates (src/klign.cpp:369-376). */
#define MHSW_ORIENT_KLIGN 0
/* test/ssw-test.cpp: the driver's "contigs" argument is SSW's ref (A) and "reads"
 * its query (B) (test/ssw-test.cpp:44-66 with translate_adept_to_ssw, :22-40). */
#define MHSW_ORIENT_REF_IS_A 1

/* ---- forms ----------------------------------------------------------------- */
#define MHSW_FORM_PLAIN 0    /* one wavefront group per pair, input order */
#define MHSW_FORM_BATCHED 1  /* length-bucketed, sorted, persistent work-stealing launch */

typedef struct mhsw_driver mhsw_driver;

/* Result views, as in adept_sw::AlignmentResults (src/adept-sw/driver.hpp:17-23),
 * plus exact int32 copies (the short views saturate beyond 32767). */
typedef struct {
  int16_t *ref_begin, *query_begin, *ref_end, *query_end, *top_scores;
  int32_t *ref_begin32, *query_begin32, *ref_end32, *query_end32, *top_scores32;
  int32_t n;
  /* score2 mode only (else NULL; see mhsw_driver_set_score2): SSW's second-best score
   * (sw_score_next_best) and its A row (ref_end_next_best: the read row in klign's
   * orientation), filled by run_kernel_forwards. */
  int32_t *score2_32, *a_end2_32;
} mhsw_aln_results;

/* Device-timed figures of the last mhsw_align_pairs / run_kernel_* call, or of the
 * aligned candidates of the last mhsw_klign_align call (n_pairs = those aligned; total_ms
 * from their translation to the end of the begin pass; fwd_cells and the counters of
 * re-runs left 0). */
typedef struct {
  double fwd_ms;      /* forward kernels (incl. int32 re-runs) */
  double rev_ms;      /* begin (reverse) kernels */
  double total_ms;    /* all device work of the call incl. copies */
  double fwd_cells;   /* sum over pairs of len(A) * len(B) */
  int64_t n_pairs;
  int64_t n_overflow16;  /* pairs re-run in int32 */
  int64_t n_rev_wide;    /* begin searches that used the wavefront path */
  int64_t launches;      /* kernels launched by the call (a graph replay counts its kernels) */
  int64_t graph_replays; /* CUDA graph launches by this handle so far: a device-resident batch
                          * aligned again with the same pointers, sizes and settings is
                          * captured on its second call and replayed from then on */
  double cigar_ms;          /* CIGAR mode: the CIGAR pass (device kernels plus the host-driven
                             * rounds for wide bands), 0 otherwise */
  int64_t n_cigar_generic;  /* CIGAR mode: pairs whose band or box exceeded the register
                             * kernels and took the generic kernel */
} mhsw_timing;

/* The batched form's tuning (no counterpart in the reference, whose launch shape follows
 * the batch's longest sequences, src/adept-sw/driver.cpp:343-368): the configuration the
 * handle's persistent forward kernels run with, and what its last tuning cost.  A batched
 * call whose length signature (the A-length mix over the kernels' row classes, sampled
 * where the host sees the lengths, and the classes of the longest A and B and of the
 * batch size) moved away from the one the handle last tuned for re-tunes on a strided
 * sample of at most 256k pairs of its batch before aligning it. */
typedef struct {
  int32_t threads_per_block;  /* persistent kernels' block size */
  int32_t blocks_per_sm;      /* 0 = the occupancy limit */
  int32_t lane_rows;          /* longest A (rows) aligned by 8-lane groups; longer A by 16-lane groups */
  int32_t wide_try16;         /* 1: pairs whose score bound exceeds the int16 keys run int16 first */
  int32_t last_call_tuned;    /* 1 when the last batched call ran the tuner */
  int32_t trials;             /* timed trials of the last tuning */
  int64_t sample_pairs;       /* pairs the last tuning's trials ran on */
  int64_t tunings;            /* tunings by this handle so far */
  double tune_wall_ms;        /* host wall time the last tuning added to its call */
  float trial_ms[16];         /* the trials' device times, in trial order */
} mhsw_tuning;

/* One completed mhsw_align_pairs / mhsw_align_pairs_async call, its device times in ms
 * since the handle's initialisation (no counterpart in the reference).  The kernels of a
 * call start once both its copies in have ended and the handle's stream has reached it
 * (the previous call's kernels are done); copies in wait only for their input set's call
 * four calls back and for the previous call's copies. */
typedef struct {
  uint64_t seq;            /* call number on this handle */
  int64_t n_pairs;
  double copy_in_start;    /* host batches: the first copy in starts (-1 for device batches) */
  double copy_in_end;      /* the last copy in ends (-1 for device batches) */
  double stream_ready;     /* the handle's stream reached the call */
  double translated;       /* translation to base codes done */
  double forward_done;     /* forward pass done */
  double begin_done;       /* begin pass done */
  double done;             /* results copied out: the call is complete */
} mhsw_call_record;

typedef struct {
  int32_t max_b_len;       /* longest B (SSW query) the kernels accept */
  int32_t max_coord;       /* coordinates and lengths must stay below this */
  int32_t int16_ceiling;   /* score ceiling of the packed int16 engine for scorings whose
                            * mismatch and ambiguity penalties do not exceed the gap-open
                            * penalty (the others use the unkeyed int16 engine, ceiling 16319) */
} mhsw_limits_t;

/* A batch as concatenated bytes with per-pair offsets and lengths.  Pointers are
 * host or device pointers depending on the call. */
typedef struct {
  const char *a_seq;
  const int64_t *a_off;
  const int32_t *a_len;
  const char *b_seq;
  const int64_t *b_off;
  const int32_t *b_len;
  int64_t n;
  /* Optional hints (0 = unknown): the longest A and B, the sum of len(A)*len(B), and
   * the byte extents of the two arenas (max over pairs of off + len).  With all four of
   * max_a_len, max_b_len, a_bytes and b_bytes given, a device batch is launched without
   * reading its lengths or offsets back, and a host batch without scanning them on the
   * host; the caller then vouches that they bound every pair. */
  int32_t max_a_len;
  int32_t max_b_len;
  double cells;
  int64_t a_bytes;
  int64_t b_bytes;
} mhsw_pairs;

/* ---- free functions (src/adept-sw/driver.hpp:25-35, driver.cpp:28-77) ------- */
/* get_num_node_gpus (driver.cpp:47-52): 0 when no device or the runtime fails. */
int mhsw_get_num_node_gpus(int *count);
/* get_tot_gpu_mem (driver.cpp:41-45): totalGlobalMem of device 0. */
int mhsw_get_tot_gpu_mem(size_t *bytes);
/* get_avail_gpu_mem_per_rank (driver.cpp:28-33): 0.8 * total / (tot_ranks / devices). */
int mhsw_get_avail_gpu_mem_per_rank(int tot_ranks, int num_devices, size_t *bytes);
/* get_device_name (driver.cpp:35-39): the PCI bus id string. */
int mhsw_get_device_name(int device_id, char *buf, size_t buflen);
/* initialize_gpu (driver.cpp:54-77): first-touch of pinned memory, timed. */
int mhsw_initialize_gpu(double *seconds, int *device_count, size_t *total_mem);
int mhsw_limits(mhsw_limits_t *out);

/* ---- driver handle (adept_sw::GPUDriver, driver.hpp:37-55) ------------------ */
int mhsw_driver_create(mhsw_driver **out);
/* ~GPUDriver (driver.cpp:249-268). */
void mhsw_driver_destroy(mhsw_driver *drv);
const char *mhsw_driver_last_error(const mhsw_driver *drv);

/* GPUDriver::init (driver.cpp:198-247): device = rank_me % device_count; scores
 * as klign passes them (negated penalties).  rlen_limit only pre-sizes buffers;
 * batches of any size and length (up to mhsw_limits) are accepted.
 * *seconds (may be NULL) receives the time spent. */
int mhsw_driver_init(mhsw_driver *drv, int rank_me, int rank_n, short match_score, short mismatch_score,
                     short gap_opening_score, short gap_extending_score, int rlen_limit, double *seconds);
/* SSW's ambiguity penalty (N against anything), negated like the others.  The
 * reference GPU driver has no such parameter (ADEPT compares raw bytes,
 * src/adept-sw/kernel.cpp:308); klign's CPU path passes ALN_AMBIGUITY_COST
 * (src/klign.cpp:423-424).  Default: -1 (ALN_AMBIGUITY_COST in CMakeDefinitions.txt:117). */
int mhsw_driver_set_ambiguity(mhsw_driver *drv, short ambiguity_score);
int mhsw_driver_set_orientation(mhsw_driver *drv, int orientation);
/* Form used by run_kernel_forwards (default MHSW_FORM_PLAIN). */
int mhsw_driver_set_form(mhsw_driver *drv, int form);
/* Debug knob: pairs whose score exceeds `ceiling` in the packed int16 engine are
 * re-run in int32 (default and maximum: mhsw_limits().int16_ceiling). */
int mhsw_driver_set_int16_ceiling(mhsw_driver *drv, int ceiling);
/* The CUDA stream (cudaStream_t) the handle launches on. */
int mhsw_driver_stream(mhsw_driver *drv, void **stream);
/* Score2 mode (default off).  klign's CPU path keeps SSW's second-best score
 * (aln.score2 = sw_score_next_best, src/klign.cpp:267); the reference GPU driver has no
 * such output and klign writes 0 (src/klign.cpp:377-378).  With the mode on, the forward
 * pass also computes it exactly as SSW does (ssw_core.cpp:513-536, :825-847, :1154-1160,
 * maskLen = max(len(A)/2, 15) as klign passes it, SSW's zero-score query padding
 * included); it costs one extra add-max per cell pair.  Results: mhsw_last_score2 and,
 * for the drop-in protocol, mhsw_aln_results.score2_32 / a_end2_32. */
int mhsw_driver_set_score2(mhsw_driver *drv, int on);
/* Second-best scores of the last batch aligned in score2 mode: score2[i] and its A row
 * a_end2[i] (0 and 0 when no row qualifies), host or device pointers as host_io says. */
int mhsw_last_score2(mhsw_driver *drv, int32_t *score2, int32_t *a_end2, int host_io);

/* CIGAR mode (default off).  klign's post-assembly alignment asks SSW for CIGARs
 * (ssw_filter.report_cigar, src/klign.cpp:435; Filter(true, true, 0, 32767)) and writes
 * cigar_string and mismatches into the SAM record (src/klign.cpp:257-271, :178-205); the
 * reference GPU driver has none and klign falls back to the CPU aligner whenever CIGARs
 * are wanted (src/klign.cpp:589-600).  With the mode on, mhsw_align_pairs and the
 * run_kernel_backwards / kernel_block round also compute, per pair, exactly what
 * StripedSmithWaterman::Aligner::Align returns with report_cigar: banded_sw's traceback
 * (src/ssw/ssw_core.cpp:854-1053) with the soft clips of ConvertAlignment and the =/X
 * split and mismatch count of CalculateNumberMismatch (src/ssw/ssw.cpp:57-254).  No CIGAR
 * (0 ops) for score 0 -- SSW then compares a base outside its reference buffer -- or when
 * a span exceeds SSW's distance filter of 32767.  Results: mhsw_last_cigar. */
int mhsw_driver_set_cigar(mhsw_driver *drv, int on);
/* CIGARs of the last batch aligned in CIGAR mode, in pair order: nops[i] ops (0: none;
 * -1: not computed, the box or band beyond the kernels' scratch) of pair i at
 * ops[op_off[i] .. op_off[i] + nops[i]), BAM-encoded (length << 4 | op, op 0..8 of
 * "MIDNSHP=X"); op_off has n + 1 entries (op_off[n] = total); mismatches[i] as SSW's
 * Alignment::mismatches.  Any output may be NULL; *ops_total receives the total op count.
 * ops_cap < total with ops non-NULL fails with MHSW_ERR_ARG (after filling the rest), so
 * a first call with ops = NULL sizes the buffer.  host_io as in mhsw_last_score2. */
int mhsw_last_cigar(mhsw_driver *drv, int32_t *nops, int32_t *mismatches, int64_t *op_off, uint32_t *ops,
                    int64_t ops_cap, int64_t *ops_total, int host_io);
/* SAM text of nops BAM-encoded ops (Alignment::cigar_string): returns its length, or -1
 * when buf (cap bytes, NUL included) is too small. */
int64_t mhsw_cigar_format(const uint32_t *ops, int32_t nops, char *buf, int64_t cap);

/* GPUDriver::run_kernel_forwards (driver.cpp:281-375): copies the batch, launches
 * the forward pass and the copy of the end coordinates and scores; returns without
 * waiting.  reads[i]/contigs[i] are byte strings of read_lens[i]/contig_lens[i]
 * bytes.  max_read_size / max_contig_size are accepted for signature parity and
 * checked as upper bounds. */
int mhsw_run_kernel_forwards(mhsw_driver *drv, const char *const *reads, const int32_t *read_lens,
                             const char *const *contigs, const int32_t *contig_lens, int32_t n,
                             uint32_t max_read_size, uint32_t max_contig_size);
/* GPUDriver::run_kernel_backwards (driver.cpp:377-417): launches the begin pass for
 * the batch of the preceding run_kernel_forwards (same arguments) and the copy of
 * begins; returns without waiting.  Unlike the reference, no host-side reduction
 * (get_new_min_length, driver.cpp:170-180) runs between the passes. */
int mhsw_run_kernel_backwards(mhsw_driver *drv, const char *const *reads, const int32_t *read_lens,
                              const char *const *contigs, const int32_t *contig_lens, int32_t n,
                              uint32_t max_read_size, uint32_t max_contig_size);
/* GPUDriver::kernel_is_done (driver.cpp:270-274): *done = 1 when the last
 * run_kernel_* call has completed. */
int mhsw_kernel_is_done(mhsw_driver *drv, int *done);
/* GPUDriver::kernel_block (driver.cpp:276-279). */
int mhsw_kernel_block(mhsw_driver *drv);
/* GPUDriver::get_aln_results (driver.hpp:54). */
int mhsw_get_aln_results(mhsw_driver *drv, mhsw_aln_results *out);

/* ---- batch entry points (the batched form and the benchmarks) --------------- */
/* Aligns a whole batch synchronously: forward + begin pass.  host_io != 0: the
 * pairs and out5 are host pointers (copies are part of the call); host_io == 0:
 * they are device pointers already resident on the handle's device.
 * out5[5*i .. 5*i+4] = score, a_begin, a_end, b_begin, b_end (SSW ref = A,
 * SSW query = B; score 0 gives -1, -1, 0, 0 as SSW does). */
int mhsw_align_pairs(mhsw_driver *drv, const mhsw_pairs *pairs, int32_t *out5, int host_io, int form);
/* mhsw_align_pairs in two halves, for callers that overlap one batch's copies with
 * another's work (klign overlaps its blocks the same way, src/klign.cpp:552-606): the
 * first enqueues the whole call -- copies in, kernels, the copy of out5 -- and returns;
 * mhsw_align_wait completes every call still pending (errors, timing, CIGAR rounds) and
 * must come before their out5 are read.  A handle keeps up to four host batches in
 * flight on four device input sets (each reserved when first used): a batch's copies wait
 * only for the call four back and for the previous call's copies, so they run while
 * earlier calls' kernels do (kernels stay in call order), and a copy the host runs slowly
 * is absorbed by the calls queued behind it; a fifth call first completes the oldest.
 * Host arrays and out5 stay untouched by the caller until completed, and should be pinned
 * for the copies to run asynchronously.  In score2 or CIGAR mode, for
 * device batches, and on any other call on the handle, pending calls complete first. */
int mhsw_align_pairs_async(mhsw_driver *drv, const mhsw_pairs *pairs, int32_t *out5, int host_io, int form);
/* The records of the handle's last completed batch calls (at most 64 kept), oldest first:
 * min(max_records, kept) records into out, their number into *count.  Completes pending
 * calls first. */
int mhsw_call_history(mhsw_driver *drv, mhsw_call_record *out, int max_records, int *count);
/* The batched form's current configuration and last tuning (mhsw_tuning above). */
int mhsw_last_tuning(mhsw_driver *drv, mhsw_tuning *out);
/* Fixes the batched form's configuration and turns the tuner off: threads_per_block 64,
 * 128 or 256; blocks_per_sm 0 (occupancy limit) or a cap; lane_rows 128 or 160;
 * wide_try16 0 or 1 (mhsw_tuning).  threads_per_block 0 turns the tuner back on (the next
 * batched call re-tunes; the configurations kept from earlier tunings are dropped).
 * MHSW_ERR_ARG for other values. */
int mhsw_driver_fix_batch_config(mhsw_driver *drv, int threads_per_block, int blocks_per_sm, int lane_rows,
                                 int wide_try16);
int mhsw_align_wait(mhsw_driver *drv);
int mhsw_last_timing(mhsw_driver *drv, mhsw_timing *out);

/* ---- serving form (no counterpart in the reference) ------------------------ */
/* Contigs stay resident on the device (translated once); alignment requests -- a read
 * plus the contig and position its k-mer seed hit points to -- arrive in uneven batches
 * from any number of host threads.  Each request's pair is the read against the contig
 * window [max(0, pos - flank), min(contig_len, pos + read_len + flank)), the window klign
 * cuts around a seed hit (src/klign.cpp:670-739).  Worker slots, each with its own stream
 * and device buffers sized from the device-memory budget, pack whatever requests are
 * waiting into the next micro-batch as soon as they free up (continuous batching), so
 * requests that arrive while others are on the GPU join the next free slot and the slots'
 * work overlaps on the device.  Results are those of mhsw_align_pairs on the same pairs,
 * whatever else shares the micro-batch. */
typedef struct mhsw_server mhsw_server;

typedef struct {
  int device;                   /* CUDA device */
  int slots;                    /* micro-batches in flight at once (0: 3) */
  int32_t max_pairs_per_batch;  /* pairs per micro-batch (0: 65536) */
  int32_t flank;                /* window flank in bases (negative: 200) */
  size_t hbm_budget;            /* device bytes for contigs plus slots (0: half the free memory) */
  size_t queue_budget;          /* host bytes of admitted requests not yet finished (0: 1 GiB) */
  short match_score, mismatch_score, gap_opening_score, gap_extending_score, ambiguity_score; /* as klign passes them */
  int form;                     /* MHSW_FORM_BATCHED or MHSW_FORM_PLAIN */
} mhsw_server_config;

typedef struct {   /* host pointers; offsets, lengths, ids and positions are copied by
                    * mhsw_server_submit, the read bytes are read until the ticket completes */
  const char *read_seq;
  const int64_t *read_off;
  const int32_t *read_len;
  const int32_t *contig_id;   /* index into the loaded contigs */
  const int32_t *contig_pos;  /* seed-hit position in the contig, 0 <= pos < contig_len */
  int32_t n;
} mhsw_requests;

typedef struct {
  int64_t submitted, completed;   /* request batches */
  int64_t pairs_done;
  double cells_done;              /* sum of read_len * window_len over finished pairs */
  int64_t micro_batches;
  int64_t queued_pairs;           /* admitted, not yet on a slot */
  size_t admitted_bytes;          /* host bytes of admitted, unfinished requests */
  int slots, busy_slots;
  int32_t slot_pairs;             /* pairs per micro-batch */
  size_t device_bytes;            /* contig store + slot buffers */
} mhsw_server_stats;

#define MHSW_SUBMIT_NOWAIT 1       /* fail with MHSW_ERR_BUSY instead of waiting for queue room */

/* Creates a server (no device memory yet).  errbuf (may be NULL) receives a message. */
int mhsw_server_create(const mhsw_server_config *cfg, mhsw_server **out, char *errbuf, size_t errlen);
/* Stops the slots after their current micro-batch; unfinished requests fail. */
void mhsw_server_destroy(mhsw_server *s);
const char *mhsw_server_last_error(const mhsw_server *s);
/* Uploads and translates the contigs (host pointers), then sizes and starts the slots
 * from what is left of the budget.  Once per server. */
int mhsw_server_load_contigs(mhsw_server *s, const char *seq, const int64_t *off, const int32_t *len, int64_t count);
/* Admits a request batch once the queue budget has room; results go to out5
 * (5 * n int32: score, a_begin, a_end, b_begin, b_end, B coordinates relative to the
 * window) and win_start (n int64, may be NULL: contig offset of each window) when the
 * ticket completes; they and req->read_seq must stay valid until mhsw_server_wait returns.
 * A batch whose reads lie back to back in read_seq (each read_off the previous one's end)
 * is packed for the device with one copy per micro-batch piece; others read by read. */
int mhsw_server_submit(mhsw_server *s, const mhsw_requests *req, int32_t *out5, int64_t *win_start, int flags,
                       uint64_t *ticket);
/* *done = 1 once the ticket's results are written. */
int mhsw_server_test(mhsw_server *s, uint64_t ticket, int *done);
/* Waits for the ticket, returns its status and releases it.  times (may be NULL)
 * receives submit, first dispatch and completion times in seconds (steady clock). */
int mhsw_server_wait(mhsw_server *s, uint64_t ticket, double *times3);
int mhsw_server_stats_get(mhsw_server *s, mhsw_server_stats *out);

/* ---- klign's caller side on the device ---------------------------------------- */
/* What klign does around each aligner call, for a batch of seed-hit candidates against
 * contigs resident on the device (klign keeps them in a DHT and caches fetched windows,
 * src/klign.cpp:670-739):
 *   orientation  '-' when the contig's seed k-mer and the read's differ in strand; the
 *                read is then reverse-complemented (utils.cpp revcomp: ACGTN, IUPAC codes
 *                to N, any other byte is an error) and the seed position mirrored
 *                (pos_in_read = rlen - (kmer_len + pos_in_read), :684-689);
 *   window       the read's footprint on the seed diagonal, clipped to the contig:
 *                left = min(pos_in_read, pos_in_ctg), right = min(rlen - kmer_len -
 *                pos_in_read, clen - pos_in_ctg - kmer_len), cstart = pos_in_ctg - left,
 *                rstart = pos_in_read - left, overlap = left + kmer_len + right (:690-701);
 *   perfect      window bytes equal to the read's overlap (raw byte compare, :220): no
 *                alignment; score1 = overlap * match, rstop = rstart + overlap, cstop =
 *                cstart + overlap (:220-230);
 *   otherwise    the whole oriented read against the window (SSW ref = read, query =
 *                window, :239-241 and :257), mapped as klign maps either aligner's result
 *                (:260-263, :372-376): rstart = read begin, rstop = read end + 1, cstart =
 *                cstart + window begin, cstop = cstart + window end + 1;
 *   then         '-' switches the read coordinates (start = rlen - stop, stop = rlen -
 *                start, utils.cpp switch_orient) and identity = 100 * score1 / match /
 *                rlen (integer arithmetic, :226, :266).
 * score2 is SSW's second-best score when the driver is in score2 mode (klign's CPU path,
 * :267), else 0 (its GPU path, :377-378); 0 for perfect matches. */
typedef struct mhsw_contigs mhsw_contigs;

/* Uploads contigs (host pointers: bytes, offsets, lengths) to the device and translates
 * them once; raw bytes stay for the perfect-match compare. */
int mhsw_contigs_create(int device, const char *seq, const int64_t *off, const int32_t *len, int64_t count,
                        mhsw_contigs **out);
void mhsw_contigs_destroy(mhsw_contigs *c);

typedef struct {   /* host pointers */
  const char *read_seq;       /* reads as found (before orientation), concatenated */
  const int64_t *read_off;
  const int32_t *read_len;
  const int32_t *contig_id;   /* contig of the seed hit */
  const int32_t *pos_in_ctg;  /* CtgLoc::pos_in_ctg: the seed k-mer's start in the contig */
  const int32_t *pos_in_read; /* the seed k-mer's start in the read as found */
  const uint8_t *strand;      /* bit 0: the read's k-mer was reverse-complemented; bit 1: the contig's (CtgLoc::is_rc) */
  int64_t n;
  int32_t kmer_len;
} mhsw_candidates;

typedef struct {   /* host pointers, n each: klign's Aln fields */
  int32_t *rstart, *rstop, *cstart, *cstop;
  int32_t *score1, *score2, *identity;
  char *orient;               /* '+' or '-' */
  uint8_t *perfect;           /* 1: taken by the perfect-match shortcut (no alignment) */
  int32_t *cigar_slot;        /* may be NULL.  In CIGAR mode: the candidate's index in the CIGAR
                               * batch mhsw_last_cigar then returns (the aligned candidates), -1
                               * for a perfect match, whose SAM CIGAR klign writes as
                               * "<rstop - rstart>=" with 0 mismatches (src/klign.cpp:229);
                               * left unwritten outside CIGAR mode */
} mhsw_alns;

/* Runs the whole caller side plus the alignments for a candidate batch with the driver's
 * scoring, form and score2 mode; synchronous.  Fails with MHSW_ERR_ARG (nothing written)
 * when a candidate's seed lies outside its read or contig or its read has a byte revcomp
 * rejects; *n_aligned (may be NULL) receives how many candidates needed an alignment.
 * The call's device arrays live in an arena kept on the handle (grown for a larger batch,
 * freed with the handle), so repeated calls allocate nothing. */
int mhsw_klign_align(mhsw_driver *drv, const mhsw_contigs *contigs, const mhsw_candidates *cand, mhsw_alns *out,
                     int64_t *n_aligned);

/* ---- protein alignment ---------------------------------------------------------- */
/* The reference declares protein kernels (src/adept-sw/kernel.cpp:510-899,
 * sequence_aa_kernel / sequence_aa_reverse) that take a 24 x 24 scoring matrix and a
 * 91-entry ASCII encoding (byte -> matrix index) from their caller; nothing in MHM2
 * launches them.  mhsw_align_protein computes their outputs -- score, a_begin, a_end,
 * b_begin, b_end per pair, laid out as mhsw_align_pairs -- with SSW's result rules (the
 * DNA path's) and the handle's gap penalties: matrix[a * 24 + b] scores A's code a against
 * B's code b.  Bytes >= 91 or encodings outside [0, 24) fail with MHSW_ERR_ARG.  Pairs
 * and out5 are host or device pointers as host_io says; synchronous. */
int mhsw_align_protein(mhsw_driver *drv, const mhsw_pairs *pairs, const int16_t *scoring_matrix,
                       const int16_t *encoding, int32_t *out5, int host_io);

/* ---- allocation-free forward pass (no counterpart in the reference) ---------- */
/* Forward pass only -- score, a_end, b_end per pair, the same values as columns 0, 2
 * and 4 of mhsw_align_pairs -- for callers that must not have the library allocate
 * device memory: a process that has handed its device memory to its own pool up front,
 * or a pipelined loop that cannot take the device-wide synchronisation cudaMalloc and
 * cudaFree may imply.  Nothing in this call allocates (no cudaMalloc, cudaFree or
 * allocating library routine); all scratch lives in one fixed 32 MiB device array inside
 * the library, one per device.  No handle: the current device is used.
 *   pairs : DEVICE pointers of a batch on the current device (raw bytes, any case, as
 *           mhsw_align_pairs takes them); pairs->max_a_len and pairs->max_b_len are
 *           required and must bound every pair (a pair beyond them gets -1, -1, -1).
 *           Each lane group takes about 9 * max_b_len + max_a_len bytes of the scratch
 *           array; a batch with max_b_len above 65000, max_a_len of 2^20 or more, or a
 *           share beyond the whole array is rejected with MHSW_ERR_LIMIT.
 *   scores: as mhsw_driver_init (match positive, penalties negated), plus ambiguity.
 *   out3  : device array of 3 * n int32: score, a_end, b_end (score 0: 0, -1, 0).
 *   stream: cudaStream_t to launch on (NULL: the default stream); returns without waiting.
 *   errbuf: (may be NULL) receives a message when the call fails.
 * The first call on a device does a one-time set-up with that device current (the
 * scratch array's address, the kernel's attributes); make it before any stream capture.
 * Calls race on the shared scratch array: two calls on one device must not overlap in
 * time (issue them on one stream, or order them with events).  Nothing in the scratch
 * array needs to start at zero. */
int mhsw_forward_noalloc(const mhsw_pairs *pairs, short match_score, short mismatch_score, short gap_opening_score,
                         short gap_extending_score, short ambiguity_score, int32_t *out3, void *stream, char *errbuf,
                         size_t errlen);

/* ---- diagnostics ----------------------------------------------------------- */
/* Measures the device's packed int16 DPX add-max throughput (__viaddmax_s16x2 on
 * independent chains, all SMs busy): *ops_per_s = packed instructions per second over
 * the whole GPU, *sm_hz = SM cycles per second seen by the probe.  Basis of the
 * cell-update roofline. */
int mhsw_probe_dpx_rate(int device, double *ops_per_s, double *sm_hz);
/* Throughput of one instruction form (lane operations per second, all SMs busy):
 * op 0 __viaddmax_s16x2, 1 __vimax3_s16x2, 2 __viaddmax_s16x2_relu,
 * 3 __vimax_s16x2_relu, 4 three-operand integer add, 5 integer multiply-add. */
int mhsw_probe_op_rate(int device, int op, double *ops_per_s);

#ifdef __cplusplus
}
#endif
#endif /* MHSW_H_ */
