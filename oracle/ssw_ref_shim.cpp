// ssw_ref_shim.cpp -- extern "C" wrapper around the reference's own CPU aligner.
//
// TEST INFRASTRUCTURE ONLY.  It is compiled by oracle/Makefile together with the
// reference sources src/ssw/ssw.cpp and src/ssw/ssw_core.cpp, read where they lie
// in the reference checkout, into oracle/_ref/libssw_ref.so (git-ignored).  No
// reference source is copied into this repository.
//
// The call is the one klign makes on its CPU path (src/klign.cpp:257):
//   Aligner(match, mismatch, gap_open, gap_extend, ambiguity)
//     .Align(query, ref, ref_len, Filter(true, false, 0, 32767), &aln, maskLen)
// with query = SSW query (B) and ref = SSW ref (A).  maskLen = max(ref_len/2, 15)
// as klign passes it (klign.cpp:257) unless the caller gives one.
#include <pthread.h>
#include <stdint.h>
#include <string>
#include <vector>

#include "ssw.hpp"

using StripedSmithWaterman::Aligner;
using StripedSmithWaterman::Alignment;
using StripedSmithWaterman::Filter;

extern "C" {

// out[0..7] = sw_score, ref_begin, ref_end, query_begin, query_end,
//             sw_score_next_best, ref_end_next_best, mismatches
int ssw_ref_align(const char *query, int query_len, const char *ref, int ref_len, int match, int mismatch, int gap_open,
                  int gap_extend, int ambiguity, int mask_len, int32_t *out) {
  Aligner aligner((uint8_t)match, (uint8_t)mismatch, (uint8_t)gap_open, (uint8_t)gap_extend, (uint8_t)ambiguity);
  Filter filter(true, false, 0, 32767);
  Alignment aln;
  aln.Clear();
  std::string q(query, (size_t)query_len);
  if (mask_len < 0) mask_len = ref_len / 2 > 15 ? ref_len / 2 : 15;
  bool ok = aligner.Align(q.c_str(), ref, ref_len, filter, &aln, mask_len);
  out[0] = aln.sw_score;
  out[1] = aln.ref_begin;
  out[2] = aln.ref_end;
  out[3] = aln.query_begin;
  out[4] = aln.query_end;
  out[5] = aln.sw_score_next_best;
  out[6] = aln.ref_end_next_best;
  out[7] = aln.mismatches;
  return ok ? 0 : 1;
}

struct RefBatch {
  const char *a_seqs, *b_seqs;
  const int64_t *a_off, *b_off;
  const int32_t *a_len, *b_len;
  int64_t n;
  int match, mismatch, gO, gE, amb;
  int32_t *out;
  int64_t next;
  int width;  // 5: score and coordinates; 7: plus sw_score_next_best and ref_end_next_best
  pthread_mutex_t mu;
};

static void *ref_worker(void *arg) {
  RefBatch *bt = (RefBatch *)arg;
  // One Aligner per thread, as klign keeps one per block (AlignBlockData copies it).
  Aligner aligner((uint8_t)bt->match, (uint8_t)bt->mismatch, (uint8_t)bt->gO, (uint8_t)bt->gE, (uint8_t)bt->amb);
  Filter filter(true, false, 0, 32767);
  Alignment aln;
  std::string q;
  for (;;) {
    pthread_mutex_lock(&bt->mu);
    int64_t lo = bt->next;
    bt->next += 64;
    pthread_mutex_unlock(&bt->mu);
    if (lo >= bt->n) break;
    int64_t hi = lo + 64 < bt->n ? lo + 64 : bt->n;
    for (int64_t p = lo; p < hi; p++) {
      // A = SSW ref (the read in klign's call), B = SSW query (the contig window).
      q.assign(bt->b_seqs + bt->b_off[p], (size_t)bt->b_len[p]);
      int rl = bt->a_len[p];
      int mask_len = rl / 2 > 15 ? rl / 2 : 15;
      aln.Clear();
      aligner.Align(q.c_str(), bt->a_seqs + bt->a_off[p], rl, filter, &aln, mask_len);
      int32_t *o = bt->out + bt->width * p;
      o[0] = aln.sw_score;
      o[1] = aln.ref_begin;
      o[2] = aln.ref_end;
      o[3] = aln.query_begin;
      o[4] = aln.query_end;
      if (bt->width == 7) {
        o[5] = aln.sw_score_next_best;
        o[6] = aln.ref_end_next_best;
      }
    }
  }
  return nullptr;
}

static int ref_batch_run(const char *a_seqs, const int64_t *a_off, const int32_t *a_len, const char *b_seqs,
                         const int64_t *b_off, const int32_t *b_len, int64_t n, int match, int mismatch, int gap_open,
                         int gap_extend, int ambiguity, int nthreads, int32_t *out, int width) {
  RefBatch bt;
  bt.width = width;
  bt.a_seqs = a_seqs;
  bt.b_seqs = b_seqs;
  bt.a_off = a_off;
  bt.b_off = b_off;
  bt.a_len = a_len;
  bt.b_len = b_len;
  bt.n = n;
  bt.match = match;
  bt.mismatch = mismatch;
  bt.gO = gap_open;
  bt.gE = gap_extend;
  bt.amb = ambiguity;
  bt.out = out;
  bt.next = 0;
  pthread_mutex_init(&bt.mu, nullptr);
  if (nthreads < 1) nthreads = 1;
  std::vector<pthread_t> th((size_t)nthreads);
  for (int t = 1; t < nthreads; t++) pthread_create(&th[t], nullptr, ref_worker, &bt);
  ref_worker(&bt);
  for (int t = 1; t < nthreads; t++) pthread_join(th[t], nullptr);
  pthread_mutex_destroy(&bt.mu);
  return 0;
}

// Same layout as sw_oracle_align_batch: out[5p..5p+4] = score, a_begin, a_end, b_begin, b_end.
int ssw_ref_align_batch(const char *a_seqs, const int64_t *a_off, const int32_t *a_len, const char *b_seqs,
                        const int64_t *b_off, const int32_t *b_len, int64_t n, int match, int mismatch, int gap_open,
                        int gap_extend, int ambiguity, int nthreads, int32_t *out) {
  return ref_batch_run(a_seqs, a_off, a_len, b_seqs, b_off, b_len, n, match, mismatch, gap_open, gap_extend, ambiguity,
                       nthreads, out, 5);
}

// As sw_oracle_align_batch7: out[7p..7p+6] adds sw_score_next_best and ref_end_next_best.
int ssw_ref_align_batch7(const char *a_seqs, const int64_t *a_off, const int32_t *a_len, const char *b_seqs,
                         const int64_t *b_off, const int32_t *b_len, int64_t n, int match, int mismatch, int gap_open,
                         int gap_extend, int ambiguity, int nthreads, int32_t *out) {
  return ref_batch_run(a_seqs, a_off, a_len, b_seqs, b_off, b_len, n, match, mismatch, gap_open, gap_extend, ambiguity,
                       nthreads, out, 7);
}

// With report_cigar (Filter(true, true, 0, 32767), the filter klign's post-assembly
// alignment asks for): out[6p..6p+5] = score, a_begin, a_end, b_begin, b_end, mismatches;
// ops[ops_cap*p ..] = the BAM-encoded CIGAR, nops[p] its length (-1: more than ops_cap).
struct RefCigarBatch {
  const char *a_seqs, *b_seqs;
  const int64_t *a_off, *b_off;
  const int32_t *a_len, *b_len;
  int64_t n;
  int match, mismatch, gO, gE, amb;
  int32_t *out;
  uint32_t *ops;
  int32_t *nops;
  int ops_cap;
  int64_t next;
  pthread_mutex_t mu;
};

static void *ref_cigar_worker(void *arg) {
  RefCigarBatch *bt = (RefCigarBatch *)arg;
  Aligner aligner((uint8_t)bt->match, (uint8_t)bt->mismatch, (uint8_t)bt->gO, (uint8_t)bt->gE, (uint8_t)bt->amb);
  Filter filter(true, true, 0, 32767);
  Alignment aln;
  std::string q;
  for (;;) {
    pthread_mutex_lock(&bt->mu);
    int64_t lo = bt->next;
    bt->next += 64;
    pthread_mutex_unlock(&bt->mu);
    if (lo >= bt->n) break;
    int64_t hi = lo + 64 < bt->n ? lo + 64 : bt->n;
    for (int64_t p = lo; p < hi; p++) {
      q.assign(bt->b_seqs + bt->b_off[p], (size_t)bt->b_len[p]);
      int rl = bt->a_len[p];
      int mask_len = rl / 2 > 15 ? rl / 2 : 15;
      aln.Clear();
      aligner.Align(q.c_str(), bt->a_seqs + bt->a_off[p], rl, filter, &aln, mask_len);
      int32_t *o = bt->out + 6 * p;
      o[0] = aln.sw_score;
      o[1] = aln.ref_begin;
      o[2] = aln.ref_end;
      o[3] = aln.query_begin;
      o[4] = aln.query_end;
      o[5] = aln.mismatches;
      if ((int64_t)aln.cigar.size() > bt->ops_cap) {
        bt->nops[p] = -1;
      } else {
        bt->nops[p] = (int32_t)aln.cigar.size();
        for (size_t k = 0; k < aln.cigar.size(); k++) bt->ops[(int64_t)bt->ops_cap * p + (int64_t)k] = aln.cigar[k];
      }
    }
  }
  return nullptr;
}

int ssw_ref_cigar_batch(const char *a_seqs, const int64_t *a_off, const int32_t *a_len, const char *b_seqs,
                        const int64_t *b_off, const int32_t *b_len, int64_t n, int match, int mismatch, int gap_open,
                        int gap_extend, int ambiguity, int nthreads, int32_t *out, uint32_t *ops, int32_t *nops,
                        int ops_cap) {
  RefCigarBatch bt;
  bt.a_seqs = a_seqs;
  bt.b_seqs = b_seqs;
  bt.a_off = a_off;
  bt.b_off = b_off;
  bt.a_len = a_len;
  bt.b_len = b_len;
  bt.n = n;
  bt.match = match;
  bt.mismatch = mismatch;
  bt.gO = gap_open;
  bt.gE = gap_extend;
  bt.amb = ambiguity;
  bt.out = out;
  bt.ops = ops;
  bt.nops = nops;
  bt.ops_cap = ops_cap;
  bt.next = 0;
  pthread_mutex_init(&bt.mu, nullptr);
  if (nthreads < 1) nthreads = 1;
  std::vector<pthread_t> th((size_t)nthreads);
  for (int t = 1; t < nthreads; t++) pthread_create(&th[t], nullptr, ref_cigar_worker, &bt);
  ref_cigar_worker(&bt);
  for (int t = 1; t < nthreads; t++) pthread_join(th[t], nullptr);
  pthread_mutex_destroy(&bt.mu);
  return 0;
}

// Protein: Aligner(score_matrix, 24, translation, 128) with SetGapPenalty, the SSW API
// for other alphabets (ssw.hpp: "If you target for other character aligners ... pass the
// corresponding matrix in").  out[5p..5p+4] = score, a_begin, a_end, b_begin, b_end.
int ssw_ref_protein_batch(const char *a_seqs, const int64_t *a_off, const int32_t *a_len, const char *b_seqs,
                          const int64_t *b_off, const int32_t *b_len, int64_t n, const int8_t *mat24,
                          const int8_t *trans128, int gap_open, int gap_extend, int32_t *out) {
  Aligner aligner(mat24, 24, trans128, 128);
  aligner.SetGapPenalty((uint8_t)gap_open, (uint8_t)gap_extend);
  Filter filter(true, false, 0, 32767);
  Alignment aln;
  std::string q;
  for (int64_t p = 0; p < n; p++) {
    q.assign(b_seqs + b_off[p], (size_t)b_len[p]);
    const int rl = a_len[p];
    aln.Clear();
    aligner.Align(q.c_str(), a_seqs + a_off[p], rl, filter, &aln, rl / 2 > 15 ? rl / 2 : 15);
    int32_t *o = out + 5 * p;
    o[0] = aln.sw_score;
    o[1] = aln.ref_begin;
    o[2] = aln.ref_end;
    o[3] = aln.query_begin;
    o[4] = aln.query_end;
  }
  return 0;
}

}  // extern "C"
