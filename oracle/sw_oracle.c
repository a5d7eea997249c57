/*
 * sw_oracle.c -- CPU oracle for the read-to-contig Smith-Waterman hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the product path links or calls this
 * file: only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg
 * use it, to check results and as the timed CPU baseline.  Parity pinned against the reference's own SSW
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
  int width; /* 5: score and coordinates; 7: plus score2 and a_end2; 6: plus mismatches, with CIGARs */
  uint32_t *ops;  /* width 6: ops_cap BAM-encoded CIGAR ops per pair */
  int32_t *nops;  /* width 6: op count per pair, -1 when more than ops_cap */
  int ops_cap;
  pthread_mutex_t mu;
} swo_batch;

int sw_oracle_cigar(const uint8_t *A, int M, const uint8_t *B, int N, const int8_t *mat, int gO, int gE,
                    const int32_t *res5, uint32_t *ops, int cap, int32_t *mismatches);

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
      if (bt->width == 6) {
        int32_t *o = bt->out + 6 * p;
        sw_oracle_align_codes(ca, la, cb, lb, bt->mat, bt->gO, bt->gE, o);
        bt->nops[p] = sw_oracle_cigar(ca, la, cb, lb, bt->mat, bt->gO, bt->gE, o, bt->ops + (int64_t)bt->ops_cap * p,
                                      bt->ops_cap, o + 5);
      } else if (bt->width == 7) {
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
                         int gap_extend, int ambiguity, int nthreads, int32_t *out, int width, uint32_t *ops,
                         int32_t *nops, int ops_cap) {
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
  bt.ops = ops;
  bt.nops = nops;
  bt.ops_cap = ops_cap;
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
                       nthreads, out, 5, NULL, NULL, 0);
}

/* As sw_oracle_align_batch with out = n*7 int32: score, a_begin, a_end, b_begin, b_end,
 * score2, a_end2 (maskLen = max(len(A)/2, 15), as klign passes it, klign.cpp:257). */
int sw_oracle_align_batch7(const char *a_seqs, const int64_t *a_off, const int32_t *a_len, const char *b_seqs,
                           const int64_t *b_off, const int32_t *b_len, int64_t n, int match, int mismatch, int gap_open,
                           int gap_extend, int ambiguity, int nthreads, int32_t *out) {
  return swo_batch_run(a_seqs, a_off, a_len, b_seqs, b_off, b_len, n, match, mismatch, gap_open, gap_extend, ambiguity,
                       nthreads, out, 7, NULL, NULL, 0);
}

/* ---- CIGAR (report_cigar = true) ----------------------------------------------------
 * Restates what SSW returns when the filter asks for a CIGAR:
 *  1. banded_sw (ssw_core.cpp:854-1053) on the aligned boxes A[a_begin..a_end] (its "ref",
 *     columns j) and B[b_begin..b_end] (its "read", rows i): a banded DP whose band
 *     half-width starts at |lenA - lenB| + 1 and doubles until the box's maximum reaches
 *     the score, with the band kept left-aligned per row (index j - max(i - w, 0) + 1,
 *     ssw_core.cpp:99-102) and its edge cell cleared at each row start exactly as SSW
 *     does; three direction codes per cell; a traceback from the box's last cell that
 *     stops at row 0 and closes with an M of one more (or a separate 1M);
 *  2. ConvertAlignment (ssw.cpp:57-93): soft clips for the unaligned ends of B;
 *  3. CalculateNumberMismatch (ssw.cpp:129-254): every M split into = / X by comparing
 *     base codes (N against N counts as equal there), mismatches = X + I + D lengths.
 * Ops are BAM-encoded, length << 4 | op with M=0 I=1 D=2 S=4 '='=7 X=8. */
enum { SWO_OP_M = 0, SWO_OP_I = 1, SWO_OP_D = 2, SWO_OP_S = 4, SWO_OP_EQ = 7, SWO_OP_X = 8 };

static int swo_push(uint32_t *ops, int cap, int *n, uint32_t len, int op) {
  if (*n >= cap) return -1;
  ops[(*n)++] = (len << 4) | (uint32_t)op;
  return 0;
}

/* banded_sw's raw CIGAR (M/I/D, in order) for the boxes; returns the op count or -1. */
static int swo_banded(const uint8_t *ref, int refLen, const uint8_t *read, int readLen, int score, const int8_t *mat,
                      int gO, int gE, uint32_t *raw, int cap) {
  int w = refLen > readLen ? refLen - readLen : readLen - refLen;
  w += 1;
  int max = 0;
  int32_t *hb = NULL, *eb = NULL, *hc = NULL;
  int8_t *dir = NULL;
  int last_w = w;
  for (;;) {
    const int width = 2 * w + 3, width_d = 2 * w + 1;
    free(hb);
    free(eb);
    free(hc);
    free(dir);
    hb = (int32_t *)calloc((size_t)width + 1, sizeof(int32_t));
    eb = (int32_t *)calloc((size_t)width + 1, sizeof(int32_t));
    hc = (int32_t *)calloc((size_t)width + 1, sizeof(int32_t));
    dir = (int8_t *)calloc((size_t)width_d * 3 * (size_t)readLen + 16, 1);
    for (int i = 0; i < readLen; i++) {
      const int x0 = i - w > 0 ? i - w : 0;               /* band start (left-aligned storage) */
      const int jb = x0, je = refLen - 1 < i + w ? refLen - 1 : i + w;
      const int edge = je + 1 < width - 1 ? je + 1 : width - 1;
      int f = 0;
      hb[0] = eb[0] = hb[edge] = eb[edge] = hc[0] = 0;
      int8_t *line = dir + (size_t)width_d * 3 * i;
      const int xp = i - 1 - w > 0 ? i - 1 - w : 0;      /* previous row's band start */
      int u = 0;
      for (int j = jb; j <= je; j++) {
        u = j - x0 + 1;
        const int e = j - xp + 1, b = u - 1, d = e - 1;
        const int dbase = (j - x0) * 3;
        int t1 = i == 0 ? -gO : hb[e] - gO;
        int t2 = i == 0 ? -gE : eb[e] - gE;
        eb[u] = t1 > t2 ? t1 : t2;
        line[dbase + 0] = (int8_t)(t1 > t2 ? 3 : 2);
        t1 = hc[b] - gO;
        t2 = f - gE;
        f = t1 > t2 ? t1 : t2;
        line[dbase + 1] = (int8_t)(t1 > t2 ? 5 : 4);
        const int e1 = eb[u] > 0 ? eb[u] : 0, f1 = f > 0 ? f : 0;
        t1 = e1 > f1 ? e1 : f1;
        t2 = hb[d] + mat[ref[j] * 5 + read[i]];
        hc[u] = t1 > t2 ? t1 : t2;
        if (hc[u] > max) max = hc[u];
        line[dbase + 2] = (int8_t)(t1 <= t2 ? 1 : (e1 > f1 ? line[dbase + 0] : line[dbase + 1]));
      }
      for (int k = 1; k <= u; k++) hb[k] = hc[k];
    }
    last_w = w;
    w *= 2;
    if (max >= score) break;
    if (last_w > refLen + readLen + 2) { /* the full box never reaches the score: inconsistent input */
      free(hb);
      free(eb);
      free(hc);
      free(dir);
      return -1;
    }
  }
  const int bw = last_w, width_d = 2 * bw + 1;
  /* traceback, ops collected last-to-first */
  uint32_t *rev = (uint32_t *)malloc(sizeof(uint32_t) * ((size_t)readLen + (size_t)refLen + 4));
  int nrev = 0;
  int i = readLen - 1, j = refLen - 1, cnt = 0, state = 2;
  char op = 'M', prev = 'M';
  int ok = 1;
  while (i > 0) {
    const int x0 = i - bw > 0 ? i - bw : 0;
    const int8_t code = dir[(size_t)width_d * 3 * i + (size_t)(j - x0) * 3 + state];
    switch (code) {
      case 1: --i; --j; state = 2; op = 'M'; break;
      case 2: --i; state = 0; op = 'I'; break;
      case 3: --i; state = 2; op = 'I'; break;
      case 4: --j; state = 1; op = 'D'; break;
      case 5: --j; state = 2; op = 'D'; break;
      default: ok = 0; break;
    }
    if (!ok) break;
    if (op == prev) {
      ++cnt;
    } else {
      rev[nrev++] = ((uint32_t)cnt << 4) | (uint32_t)(prev == 'M' ? SWO_OP_M : prev == 'I' ? SWO_OP_I : SWO_OP_D);
      prev = op;
      cnt = 1;
    }
  }
  int n = -1;
  if (ok) {
    if (op == 'M') {
      rev[nrev++] = ((uint32_t)(cnt + 1) << 4) | SWO_OP_M;
    } else {
      rev[nrev++] = ((uint32_t)cnt << 4) | (uint32_t)(op == 'I' ? SWO_OP_I : SWO_OP_D);
      rev[nrev++] = (1u << 4) | SWO_OP_M;
    }
    if (nrev <= cap) {
      for (int k = 0; k < nrev; k++) raw[k] = rev[nrev - 1 - k];
      n = nrev;
    }
  }
  free(rev);
  free(hb);
  free(eb);
  free(hc);
  free(dir);
  return n;
}

/* Final CIGAR and mismatch count of an alignment res5 = (score, a_begin, a_end, b_begin,
 * b_end) of A (SSW ref, M codes) and B (SSW query, N codes).  Returns the op count
 * (0: no CIGAR, score 0) or -1 when cap is too small. */
int sw_oracle_cigar(const uint8_t *A, int M, const uint8_t *B, int N, const int8_t *mat, int gO, int gE,
                    const int32_t *res5, uint32_t *ops, int cap, int32_t *mismatches) {
  *mismatches = 0;
  const int S = res5[0], ab = res5[1], ae = res5[2], bb = res5[3], be = res5[4];
  /* no CIGAR for score 0 (SSW then compares a base before its ref, out of bounds) nor past
   * SSW's distance filter 32767 (ssw_core.cpp:1180) */
  if (S <= 0 || M <= 0 || N <= 0 || ae - ab > 32767 || be - bb > 32767) return 0;
  uint32_t *raw = (uint32_t *)malloc(sizeof(uint32_t) * ((size_t)M + (size_t)N + 8));
  const int nraw = swo_banded(A + ab, ae - ab + 1, B + bb, be - bb + 1, S, mat, gO, gE, raw, M + N + 8);
  if (nraw < 0) {
    free(raw);
    return -1;
  }
  int n = 0, mm = 0;
  const uint8_t *r = A + ab, *q = B + bb;
  if (bb > 0 && swo_push(ops, cap, &n, (uint32_t)bb, SWO_OP_S)) goto full;
  for (int k = 0; k < nraw; k++) {
    const int op = (int)(raw[k] & 0xfu);
    const uint32_t len = raw[k] >> 4;
    if (op == SWO_OP_M) {
      int run_op = -1;
      uint32_t run = 0;
      for (uint32_t t = 0; t < len; t++) {
        const int o = (*r != *q) ? SWO_OP_X : SWO_OP_EQ;
        if (o == SWO_OP_X) ++mm;
        if (o != run_op && run > 0) {
          if (swo_push(ops, cap, &n, run, run_op)) goto full;
          run = 0;
        }
        run_op = o;
        ++run;
        ++r;
        ++q;
      }
      if (run > 0 && swo_push(ops, cap, &n, run, run_op)) goto full;
    } else if (op == SWO_OP_I) {
      q += len;
      mm += (int)len;
      if (swo_push(ops, cap, &n, len, op)) goto full;
    } else {
      r += len;
      mm += (int)len;
      if (swo_push(ops, cap, &n, len, op)) goto full;
    }
  }
  if (N - be - 1 > 0 && swo_push(ops, cap, &n, (uint32_t)(N - be - 1), SWO_OP_S)) goto full;
  free(raw);
  *mismatches = mm;
  return n;
full:
  free(raw);
  return -1;
}

/* As sw_oracle_align_batch with a CIGAR per pair (Filter(true, true, 0, 32767)):
 * out = n*6 int32 (score, a_begin, a_end, b_begin, b_end, mismatches), ops = n*ops_cap
 * BAM-encoded ops, nops[p] = op count of pair p (0: none, -1: more than ops_cap). */
int sw_oracle_cigar_batch(const char *a_seqs, const int64_t *a_off, const int32_t *a_len, const char *b_seqs,
                          const int64_t *b_off, const int32_t *b_len, int64_t n, int match, int mismatch, int gap_open,
                          int gap_extend, int ambiguity, int nthreads, int32_t *out, uint32_t *ops, int32_t *nops,
                          int ops_cap) {
  return swo_batch_run(a_seqs, a_off, a_len, b_seqs, b_off, b_len, n, match, mismatch, gap_open, gap_extend, ambiguity,
                       nthreads, out, 6, ops, nops, ops_cap);
}

/* ---- protein (an nc x nc substitution matrix) ------------------------------------------
 * The same result rules as sw_oracle_align_codes (score, lexicographically smallest end,
 * begin by the reversed sweep that stops at the first row reaching the score), with
 * scores mat[a * nc + b] for codes a (A) and b (B) below nc.  The reference's protein
 * kernels (src/adept-sw/kernel.cpp:510-899, sequence_aa_kernel / sequence_aa_reverse) take
 * a 24 x 24 scoring matrix and a 91-entry ASCII encoding from their caller. */
static void swo_sweep_mat(const uint8_t *A, int M, const uint8_t *B, int N, const int16_t *mat, int nc, int gO, int gE,
                          int stop_at, int32_t *Hrow, int32_t *Erow, int *best, int *bi, int *bj) {
  int b = 0, ii = -1, jj = 0;
  for (int j = 0; j < N; j++) {
    Hrow[j] = 0;
    Erow[j] = -gO;
  }
  for (int i = 0; i < M; i++) {
    const int16_t *srow = mat + nc * A[i];
    int32_t diag = 0, f = -gO;
    for (int j = 0; j < N; j++) {
      int32_t e = Erow[j];
      int32_t h = diag + srow[B[j]];
      if (e > h) h = e;
      if (f > h) h = f;
      if (h < 0) h = 0;
      diag = Hrow[j];
      Hrow[j] = h;
      int32_t hg = h - gO, en = e - gE, fn = f - gE;
      Erow[j] = en > hg ? en : hg;
      f = fn > hg ? fn : hg;
      if (h > b) {
        b = h;
        ii = i;
        jj = j;
      }
    }
    if (stop_at > 0 && b >= stop_at) break;
  }
  *best = b;
  *bi = ii;
  *bj = jj;
}

int sw_oracle_align_protein(const uint8_t *A, int M, const uint8_t *B, int N, const int16_t *mat, int nc, int gO, int gE,
                            int32_t *out) {
  out[0] = 0;
  out[1] = -1;
  out[2] = -1;
  out[3] = 0;
  out[4] = 0;
  if (M <= 0 || N <= 0) return 0;
  int32_t *work = (int32_t *)malloc(sizeof(int32_t) * 2 * (size_t)N + 16);
  int S, ie, je;
  swo_sweep_mat(A, M, B, N, mat, nc, gO, gE, 0, work, work + N, &S, &ie, &je);
  if (S > 0) {
    const int Mr = ie + 1, Nr = je + 1;
    uint8_t *ra = (uint8_t *)malloc((size_t)Mr + (size_t)Nr + 16);
    uint8_t *rb = ra + Mr;
    for (int i = 0; i < Mr; i++) ra[i] = A[ie - i];
    for (int j = 0; j < Nr; j++) rb[j] = B[je - j];
    int S2, ir, jr;
    swo_sweep_mat(ra, Mr, rb, Nr, mat, nc, gO, gE, S, work, work + N, &S2, &ir, &jr);
    free(ra);
    out[0] = S;
    out[1] = ie - ir;
    out[2] = ie;
    out[3] = je - jr;
    out[4] = je;
  }
  free(work);
  return 0;
}

typedef struct {
  const char *a_seqs, *b_seqs;
  const int64_t *a_off, *b_off;
  const int32_t *a_len, *b_len;
  int64_t n;
  const int16_t *mat, *enc;
  int gO, gE;
  int32_t *out;
  int64_t next;
  pthread_mutex_t mu;
} swo_pbatch;

static void *swo_pworker(void *arg) {
  swo_pbatch *bt = (swo_pbatch *)arg;
  uint8_t *ca = NULL, *cb = NULL;
  int64_t cap_a = 0, cap_b = 0;
  for (;;) {
    pthread_mutex_lock(&bt->mu);
    const int64_t lo = bt->next;
    bt->next += 64;
    pthread_mutex_unlock(&bt->mu);
    if (lo >= bt->n) break;
    const int64_t hi = lo + 64 < bt->n ? lo + 64 : bt->n;
    for (int64_t p = lo; p < hi; p++) {
      const int32_t la = bt->a_len[p], lb = bt->b_len[p];
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
      for (int i = 0; i < la; i++) ca[i] = (uint8_t)bt->enc[(unsigned char)bt->a_seqs[bt->a_off[p] + i]];
      for (int j = 0; j < lb; j++) cb[j] = (uint8_t)bt->enc[(unsigned char)bt->b_seqs[bt->b_off[p] + j]];
      sw_oracle_align_protein(ca, la, cb, lb, bt->mat, 24, bt->gO, bt->gE, bt->out + 5 * p);
    }
  }
  free(ca);
  free(cb);
  return NULL;
}

/* Protein batch: bytes below 91 encoded by enc (ADEPT's 91-entry table, indices < 24),
 * mat = 24 x 24 scores; the caller checks the bytes.  out = n x 5 as the DNA batch. */
int sw_oracle_protein_batch(const char *a_seqs, const int64_t *a_off, const int32_t *a_len, const char *b_seqs,
                            const int64_t *b_off, const int32_t *b_len, int64_t n, const int16_t *mat,
                            const int16_t *enc, int gap_open, int gap_extend, int nthreads, int32_t *out) {
  swo_pbatch bt;
  bt.a_seqs = a_seqs;
  bt.b_seqs = b_seqs;
  bt.a_off = a_off;
  bt.b_off = b_off;
  bt.a_len = a_len;
  bt.b_len = b_len;
  bt.n = n;
  bt.mat = mat;
  bt.enc = enc;
  bt.gO = gap_open;
  bt.gE = gap_extend;
  bt.out = out;
  bt.next = 0;
  pthread_mutex_init(&bt.mu, NULL);
  if (nthreads < 1) nthreads = 1;
  if (nthreads > 512) nthreads = 512;
  pthread_t th[512];
  for (int t = 1; t < nthreads; t++) pthread_create(&th[t], NULL, swo_pworker, &bt);
  swo_pworker(&bt);
  for (int t = 1; t < nthreads; t++) pthread_join(th[t], NULL);
  pthread_mutex_destroy(&bt.mu);
  return 0;
}
