/*
 * sw_oracle.c -- CPU oracle for the read-to-contig Smith-Waterman hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the product path links or calls this
 * file: only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg
 * use it, as the checker.  Parity pinned against the reference's own SSW
 * (src/ssw/ssw.cpp + src/ssw/ssw_core.cpp, compiled from the reference
 * sources by oracle/Makefile into oracle/_ref/) and against the known-answer
 * cases of test/ssw-test.cpp:151-238 (fixtures in tests/golden/).
 *
 * What it restates (the result contract of StripedSmithWaterman::Aligner::Align
 * with Filter(report_begin_position=true, report_cigar=false), ssw.cpp:431-469):
 *
 *   A = SSW "ref"   (outer loop of sw_sse2_byte/word, ssw_core.cpp:296-493)
 *   B = SSW "query" (the striped profile dimension, ssw_core.cpp:173-197)
 *
 *   Gotoh local alignment, H = max(0, H(i-1,j-1)+s, E, F) with
 *   E(i,j) = max(E(i-1,j)-gE, H(i-1,j)-gO) and F(i,j) = max(F(i,j-1)-gE, H(i,j-1)-gO).
 *
 *   score          = max H (ssw_core.cpp:474-485: max only grows on a strict increase)
 *   (a_end, b_end) = lexicographically smallest (i, j) holding the score: the first
 *                    A column whose max reaches the score (end_ref, ssw_core.cpp:480)
 *                    and in it the smallest B index (end_read, ssw_core.cpp:496-506).
 *   (a_begin, b_begin) = the same rule run on A[0..a_end] and B[0..b_end], both
 *                    reversed, stopping at the first row that reaches the score
 *                    (ssw_align's reverse pass with terminate=score1, ssw_core.cpp:1166-1178).
 *   score 0        -> a_end = a_begin = -1, b_end = b_begin = 0 (end_ref starts at -1,
 *                    ssw_core.cpp:241; the reverse pass then runs on an empty A).
 *   score2, a_end2 = the second-best score SSW reports (ssw_core.cpp:513-536 byte path,
 *                    :825-847 word path, :1154-1160).  SSW's maxColumn[i] is the max of H
 *                    over its striped query, which is padded to a multiple of 16 (byte
 *                    path) or 8 (word path) positions that score 0 against every base
 *                    (qP_byte / qP_word, ssw_core.cpp:191, :559): rowmax(i) = max over
 *                    j < P of H(i, j) on B extended by P - N zero-score columns (the real
 *                    cells are unchanged: the extra columns lie right of them).  score2 is
 *                    the largest rowmax(i), first i on ties, over i < max(a_end - maskLen, 0)
 *                    and over i >= min(a_end + maskLen, M) (+1 on the byte path).  The byte
 *                    path held the score iff score + bias < 255 with bias = -min(matrix)
 *                    (ssw_core.cpp:476, :1129-1133).  0 and 0 when no row qualifies; 0 and
 *                    -1 when maskLen < 15.
 *
 * Substitution scores follow BuildSwScoreMatrix (ssw.cpp:28-55): +match on equal
 * ACGT codes, -mismatch on different ACGT codes, -ambiguity whenever either code
 * is 4 (N or any non-ACGT byte, including N against N).  ASCII is translated by
 * the table of ssw.cpp:13-26 ('U'/'u' map to code 0 there, lowercase folds).
 *
 * SSW's lazy-F loop skips the I-then-D update (ssw_core.cpp:381); it cannot
 * change H when mismatch and ambiguity are <= min(2*gE, gO+gE, 2*gO), which
 * holds for every scoring the reference uses.  SSW's 16-bit path saturates at
 * 32767; this oracle uses int32 and stays exact beyond that.
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <pthread.h>

#define SWO_NEG (-(1 << 29))

/* ASCII -> code table restated from ssw.cpp:13-26 (codes 0..3 = ACGT, 4 = other). */
static int8_t swo_code_of(unsigned char c) {
  switch (c) {
    case 'A': case 'a': case 'U': case 'u': return 0;
    case 'C': case 'c': return 1;
    case 'G': case 'g': return 2;
    case 'T': case 't': return 3;
    default: return 4;
  }
}

void sw_oracle_encode(const char *ascii, int64_t len, uint8_t *codes) {
  for (int64_t i = 0; i < len; i++) codes[i] = (uint8_t)swo_code_of((unsigned char)ascii[i]);
}

/* 5x5 matrix laid out like BuildSwScoreMatrix (ssw.cpp:28-55). */
void sw_oracle_matrix(int match, int mismatch, int ambiguity, int8_t *mat) {
  for (int a = 0; a < 5; a++)
    for (int b = 0; b < 5; b++) {
      int s;
      if (a == 4 || b == 4) s = -ambiguity;
      else s = (a == b) ? match : -mismatch;
      mat[a * 5 + b] = (int8_t)s;
    }
}

/* Row-major Gotoh sweep: rows over A (outer), columns over B.  Records the first
 * cell (in row-major order) where the running max strictly grows.  If stop_at > 0,
 * stops after the first row whose max reaches stop_at. */
/* B codes >= 5 score 0 against every A code (SSW's query padding). */
static void swo_sweep(const uint8_t *A, int M, const uint8_t *B, int N, const int8_t *mat, int gO, int gE, int stop_at,
                      int32_t *Hrow, int32_t *Erow, int *best, int *bi, int *bj, int32_t *rowmax) {
  int b = 0, ii = -1, jj = 0;
  for (int j = 0; j < N; j++) {
    Hrow[j] = 0;
    Erow[j] = -gO; /* E(0,j) = H(-1,j) - gO */
  }
  for (int i = 0; i < M; i++) {
    const int8_t *srow = mat + 5 * A[i];
    int32_t diag = 0; /* H(i-1,-1) */
    int32_t f = -gO;  /* F(i,0) = H(i,-1) - gO */
    int32_t rm = 0;
    for (int j = 0; j < N; j++) {
      int32_t e = Erow[j];
      int32_t h = diag + (B[j] < 5 ? srow[B[j]] : 0);
      if (e > h) h = e;
      if (f > h) h = f;
      if (h < 0) h = 0;
      diag = Hrow[j];
      Hrow[j] = h;
      int32_t hg = h - gO;
      int32_t en = e - gE;
      Erow[j] = en > hg ? en : hg;
      int32_t fn = f - gE;
      f = fn > hg ? fn : hg;
      if (h > b) {
        b = h;
        ii = i;
        jj = j;
      }
      if (h > rm) rm = h;
    }
    if (rowmax) rowmax[i] = rm;
    if (stop_at > 0 && b >= stop_at) break;
  }
  *best = b;
  *bi = ii;
  *bj = jj;
}

/* out[0..4] = score, a_begin, a_end, b_begin, b_end.  Returns cells swept (fwd + rev). */
int64_t sw_oracle_align_codes(const uint8_t *A, int M, const uint8_t *B, int N, const int8_t *mat, int gO, int gE,
                              int32_t *out) {
  out[0] = 0;
  out[1] = -1;
  out[2] = -1;
  out[3] = 0;
  out[4] = 0;
  if (M <= 0 || N <= 0) return 0;
  int32_t *work = (int32_t *)malloc(sizeof(int32_t) * 2 * (size_t)N + 16);
  int32_t *Hrow = work, *Erow = work + N;
  int S, ie, je;
  swo_sweep(A, M, B, N, mat, gO, gE, 0, Hrow, Erow, &S, &ie, &je, NULL);
  int64_t cells = (int64_t)M * N;
  if (S > 0) {
    int Mr = ie + 1, Nr = je + 1;
    uint8_t *ra = (uint8_t *)malloc((size_t)Mr + (size_t)Nr + 16);
    uint8_t *rb = ra + Mr;
    for (int i = 0; i < Mr; i++) ra[i] = A[ie - i];
    for (int j = 0; j < Nr; j++) rb[j] = B[je - j];
    int S2, ir, jr;
    swo_sweep(ra, Mr, rb, Nr, mat, gO, gE, S, Hrow, Erow, &S2, &ir, &jr, NULL);
    cells += (int64_t)(ir + 1) * Nr;
    free(ra);
    out[0] = S;
    out[1] = ie - ir;
    out[2] = ie;
    out[3] = je - jr;
    out[4] = je;
  }
  free(work);
  return cells;
}

/* Second-best score from the forward pass's row maxima (SSW's maxColumn over its ref). */
static void swo_second_best(const int32_t *rowmax, int M, int S, int a_end, int mask_len, int bias, int32_t *score2,
                            int32_t *a_end2) {
  *score2 = 0;
  *a_end2 = 0;
  if (mask_len < 15) {
    *a_end2 = -1;
    return;
  }
  const int word = S + bias >= 255;
  int32_t best = 0, at = 0;
  int edge = a_end - mask_len > 0 ? a_end - mask_len : 0;
  for (int i = 0; i < edge; i++)
    if (rowmax[i] > best) {
      best = rowmax[i];
      at = i;
    }
  edge = a_end + mask_len > M ? M : a_end + mask_len;
  for (int i = word ? edge : edge + 1; i < M; i++)
    if (rowmax[i] > best) {
      best = rowmax[i];
      at = i;
    }
  *score2 = best;
  *a_end2 = at;
}

/* out[0..6] = score, a_begin, a_end, b_begin, b_end, score2, a_end2 (maskLen as given;
 * klign passes max(len(A)/2, 15)). */
int64_t sw_oracle_align_codes7(const uint8_t *A, int M, const uint8_t *B, int N, const int8_t *mat, int gO, int gE,
                               int mask_len, int32_t *out) {
  int64_t cells = sw_oracle_align_codes(A, M, B, N, mat, gO, gE, out);
  out[5] = 0;
  out[6] = mask_len < 15 ? -1 : 0;
  if (M <= 0 || N <= 0) return cells;
  int bias = 0;
  for (int k = 0; k < 25; k++)
    if (mat[k] < bias) bias = mat[k];
  bias = -bias;
  const int S = out[0], ie = out[2];
  const int word = S + bias >= 255;
  const int P = word ? (N + 7) / 8 * 8 : (N + 15) / 16 * 16;  /* SSW's padded query length */
  int32_t *work = (int32_t *)malloc(sizeof(int32_t) * (2 * (size_t)P + (size_t)M) + 16);
  int32_t *Hrow = work, *Erow = work + P, *rowmax = work + 2 * P;
  uint8_t *Bp = (uint8_t *)malloc((size_t)P + 16);
  memcpy(Bp, B, (size_t)N);
  memset(Bp + N, 5, (size_t)(P - N));
  int S2, i2, j2;
  swo_sweep(A, M, Bp, P, mat, gO, gE, 0, Hrow, Erow, &S2, &i2, &j2, rowmax);
  swo_second_best(rowmax, M, S, ie, mask_len, bias, out + 5, out + 6);
  free(Bp);
  free(work);
  return cells + (int64_t)M * P;
}

typedef struct {
  const char *a_seqs, *b_seqs;
  const int64_t *a_off, *b_off;
  const int32_t *a_len, *b_len;
  int64_t n;
  int8_t mat[25];
  int gO, gE;
  int32_t *out;
  int64_t next;
  int64_t chunk;
  int width; /* 5: score and coordinates; 7: plus score2 and a_end2 */
  pthread_mutex_t mu;
} swo_batch;

static void *swo_worker(void *arg) {
  swo_batch *bt = (swo_batch *)arg;
  uint8_t *ca = NULL, *cb = NULL;
  int64_t cap_a = 0, cap_b = 0;
  for (;;) {
    pthread_mutex_lock(&bt->mu);
    int64_t lo = bt->next;
    bt->next += bt->chunk;
    pthread_mutex_unlock(&bt->mu);
    if (lo >= bt->n) break;
    int64_t hi = lo + bt->chunk < bt->n ? lo + bt->chunk : bt->n;
    for (int64_t p = lo; p < hi; p++) {
      int32_t la = bt->a_len[p], lb = bt->b_len[p];
      if (la > cap_a) {
        free(ca);
        cap_a = la + 64;
        ca = (uint8_t *)malloc((size_t)cap_a);
      }
      if (lb > cap_b) {
        free(cb);
        cap_b = lb + 64;
        cb = (uint8_t *)malloc((size_t)cap_b);
      }
      sw_oracle_encode(bt->a_seqs + bt->a_off[p], la, ca);
      sw_oracle_encode(bt->b_seqs + bt->b_off[p], lb, cb);
      if (bt->width == 7) {
        const int mask_len = la / 2 > 15 ? la / 2 : 15;
        sw_oracle_align_codes7(ca, la, cb, lb, bt->mat, bt->gO, bt->gE, mask_len, bt->out + 7 * p);
      } else {
        sw_oracle_align_codes(ca, la, cb, lb, bt->mat, bt->gO, bt->gE, bt->out + 5 * p);
      }
    }
  }
  free(ca);
  free(cb);
  return NULL;
}

/* Batch over concatenated ASCII sequences.  A_p = a_seqs[a_off[p] .. +a_len[p]),
 * B_p likewise.  out is n*5 int32 (score, a_begin, a_end, b_begin, b_end). */
static int swo_batch_run(const char *a_seqs, const int64_t *a_off, const int32_t *a_len, const char *b_seqs,
                         const int64_t *b_off, const int32_t *b_len, int64_t n, int match, int mismatch, int gap_open,
                         int gap_extend, int ambiguity, int nthreads, int32_t *out, int width) {
  swo_batch bt;
  bt.width = width;
  bt.a_seqs = a_seqs;
  bt.b_seqs = b_seqs;
  bt.a_off = a_off;
  bt.b_off = b_off;
  bt.a_len = a_len;
  bt.b_len = b_len;
  bt.n = n;
  sw_oracle_matrix(match, mismatch, ambiguity, bt.mat);
  bt.gO = gap_open;
  bt.gE = gap_extend;
  bt.out = out;
  bt.next = 0;
  bt.chunk = 64;
  pthread_mutex_init(&bt.mu, NULL);
  if (nthreads < 1) nthreads = 1;
  if (nthreads > 512) nthreads = 512;
  pthread_t th[512];
  for (int t = 1; t < nthreads; t++) pthread_create(&th[t], NULL, swo_worker, &bt);
  swo_worker(&bt);
  for (int t = 1; t < nthreads; t++) pthread_join(th[t], NULL);
  pthread_mutex_destroy(&bt.mu);
  return 0;
}

int sw_oracle_align_batch(const char *a_seqs, const int64_t *a_off, const int32_t *a_len, const char *b_seqs,
                          const int64_t *b_off, const int32_t *b_len, int64_t n, int match, int mismatch, int gap_open,
                          int gap_extend, int ambiguity, int nthreads, int32_t *out) {
  return swo_batch_run(a_seqs, a_off, a_len, b_seqs, b_off, b_len, n, match, mismatch, gap_open, gap_extend, ambiguity,
                       nthreads, out, 5);
}

/* As sw_oracle_align_batch with out = n*7 int32: score, a_begin, a_end, b_begin, b_end,
 * score2, a_end2 (maskLen = max(len(A)/2, 15), as klign passes it, klign.cpp:257). */
int sw_oracle_align_batch7(const char *a_seqs, const int64_t *a_off, const int32_t *a_len, const char *b_seqs,
                           const int64_t *b_off, const int32_t *b_len, int64_t n, int match, int mismatch, int gap_open,
                           int gap_extend, int ambiguity, int nthreads, int32_t *out) {
  return swo_batch_run(a_seqs, a_off, a_len, b_seqs, b_off, b_len, n, match, mismatch, gap_open, gap_extend, ambiguity,
                       nthreads, out, 7);
}
