/*
 * sw_lanes.cpp -- the CPU oracle's result contract, vectorised across pairs.
 *
 * TEST INFRASTRUCTURE ONLY, like sw_oracle.c: the CPU baseline that bench.py times
 * (and a second route to the same results that the tests compare with the scalar
 * restatement).  It computes exactly what sw_oracle_align_codes computes -- the same
 * int Gotoh recurrence, the same strict row-major arg-max for the end and the same
 * "first cell reaching the score" rule on the reversed prefixes for the begin -- but
 * eight pairs per 128-bit GCC vector, one pair per int16 lane (portable:
 * the compiler emits SSE2 on x86_64 and NEON on aarch64; no intrinsics headers).  C++ for
 * the vector conditional operator.
 *
 * Pairs are sorted by (len A, len B) so the eight of a group have similar shapes;
 * each group is padded to its longest A and B.  Padding positions score like N
 * (-ambiguity): with ambiguity > 0 and gap open > 0, a padded cell is at most a
 * neighbouring cell's value minus a positive penalty (or equal to a real cell of an
 * earlier row along its diagonal), so it never raises the running maximum (strict >)
 * and never reaches the score before the real cell that does, and no real cell reads a
 * padded one (real cells read only columns to their left and rows above).  Pairs whose
 * score could leave int16 (min(len A, len B) * match >= 30000), and scorings outside
 * those conditions, go through the scalar restatement instead.
 *
 * Codes: A uses 0..3 for ACGT and 4 for any other byte or padding, B uses 0..3 and 8,
 * so A == B only for equal ACGT bases; each row and column also carries its per-lane
 * substitution base (-ambiguity for N, -mismatch otherwise).
 */
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define SWL_LANES 8
/* Vectors of pairs swept side by side: on aarch64 (measured on 16 Grace cores: 19.1, 30.6
 * and 33.0 GCUPS for 1, 2 and 4) the independent F chains along the rows need the
 * interleaving; on x86_64 it gains nothing. */
#ifndef SWL_NV
#if defined(__aarch64__)
#define SWL_NV 4
#else
#define SWL_NV 1
#endif
#endif
typedef int16_t swl_v __attribute__((vector_size(16)));

extern "C" {
void sw_oracle_encode(const char *ascii, int64_t len, uint8_t *codes);
void sw_oracle_matrix(int match, int mismatch, int ambiguity, int8_t *mat);
int64_t sw_oracle_align_codes(const uint8_t *A, int M, const uint8_t *B, int N, const int8_t *mat, int gO, int gE,
                              int32_t *out);
int sw_oracle_align_batch_lanes(const char *a_seqs, const int64_t *a_off, const int32_t *a_len, const char *b_seqs,
                                const int64_t *b_off, const int32_t *b_len, int64_t n, int match, int mismatch,
                                int gap_open, int gap_extend, int ambiguity, int nthreads, int32_t *out);
}

static swl_v swl_splat(int x) {
  swl_v v;
  for (int k = 0; k < SWL_LANES; k++) v[k] = (int16_t)x;
  return v;
}

typedef struct {
  int m, x, amb, gO, gE;
} swl_score;

/* One group's sweep over NV vectors of lanes side by side (independent dependency
 * chains, interleaved by the compiler).  Position p of A / B holds NV vectors
 * A[p * NV + v]; RB / CB likewise: per-lane codes (A: 0..4, B: 0..3 or 8) and the
 * per-lane substitution base of each row and column, -ambiguity for N and -mismatch
 * otherwise, combined with max (ambiguity <= mismatch) or min (ambiguity > mismatch), so
 * s = (A == B ? match + mismatch : 0) + base.  mode 0: forward arg-max (strict >,
 * row-major) into best / bi / bj.  mode 1: first cell with H >= S per lane (row-major)
 * into bi / bj, stopping once every lane has one. */
template <int NV, bool AMB_LE_MIS>
static void swl_sweep(const swl_v *A, const swl_v *RB, int Mg, const swl_v *B, const swl_v *CB, int Ng,
                      const swl_score *sc, int mode, const swl_v *S, swl_v *Hrow, swl_v *Erow, swl_v *best_out,
                      swl_v *bi_out, swl_v *bj_out, swl_v *found) {
  const swl_v zero = swl_splat(0), one = swl_splat(1), vgO = swl_splat(sc->gO), vgE = swl_splat(sc->gE);
  const swl_v mx = swl_splat(sc->m + sc->x);
  for (int j = 0; j < Ng * NV; j++) {
    Hrow[j] = zero;
    Erow[j] = -vgO;
  }
  swl_v best[NV], bi[NV], bj[NV], Sm1[NV];
  for (int v = 0; v < NV; v++) {
    best[v] = zero;
    bi[v] = swl_splat(-1);
    bj[v] = zero;
    Sm1[v] = S[v] - one;
  }
  for (int i = 0; i < Mg; i++) {
    swl_v a[NV], rb[NV], diag[NV], f[NV], mark[NV];
    for (int v = 0; v < NV; v++) {
      a[v] = A[i * NV + v];
      rb[v] = RB[i * NV + v];
      diag[v] = zero;
      f[v] = -vgO;
      mark[v] = zero;
    }
    swl_v j1 = zero;
    for (int j = 0; j < Ng; j++) {
      j1 += one;
#pragma GCC unroll 4
      for (int v = 0; v < NV; v++) {
        const int x = j * NV + v;
        const swl_v cb = CB[x];
        const swl_v base = AMB_LE_MIS ? (rb[v] > cb ? rb[v] : cb) : (rb[v] < cb ? rb[v] : cb);
        const swl_v s = ((swl_v)(a[v] == B[x]) & mx) + base;
        const swl_v e = Erow[x];
        swl_v h = diag[v] + s;
        h = h > e ? h : e;
        h = h > f[v] ? h : f[v];
        h = h > zero ? h : zero;
        diag[v] = Hrow[x];
        Hrow[x] = h;
        const swl_v hg = h - vgO;
        const swl_v en = e - vgE;
        Erow[x] = en > hg ? en : hg;
        const swl_v fn = f[v] - vgE;
        f[v] = fn > hg ? fn : hg;
        if (mode == 0) {
          const swl_v gt = (swl_v)(h > best[v]);
          best[v] = h > best[v] ? h : best[v];
          const swl_v c = gt & j1; /* j + 1 where the running max grows; later cells of a row have larger j */
          mark[v] = mark[v] > c ? mark[v] : c;
        } else {
          mark[v] |= (swl_v)(h > Sm1[v]);
        }
      }
    }
    const swl_v iv = swl_splat(i);
    if (mode == 0) {
      for (int v = 0; v < NV; v++) {
        const swl_v grew = (swl_v)(mark[v] > zero);
        bj[v] = (grew & (mark[v] - one)) | (~grew & bj[v]);
        bi[v] = (grew & iv) | (~grew & bi[v]);
      }
    } else {
      int any = 0;
      swl_v fresh[NV];
      for (int v = 0; v < NV; v++) {
        fresh[v] = mark[v] & ~found[v];
        for (int k = 0; k < SWL_LANES; k++) any |= (fresh[v][k] != 0);
      }
      if (any) { /* the first column of this row holding the score, for the lanes that reached it */
        int all = 1;
        for (int v = 0; v < NV; v++) {
          swl_v first = swl_splat(0x7fff);
          for (int j = Ng - 1; j >= 0; j--) {
            const swl_v hit = (swl_v)(Hrow[j * NV + v] > Sm1[v]) & fresh[v];
            const swl_v jv = swl_splat(j);
            first = (hit & jv) | (~hit & first);
          }
          bj[v] = (fresh[v] & first) | (~fresh[v] & bj[v]);
          bi[v] = (fresh[v] & iv) | (~fresh[v] & bi[v]);
          found[v] |= fresh[v];
          for (int k = 0; k < SWL_LANES; k++) all &= (found[v][k] != 0);
        }
        if (all) break;
      }
    }
  }
  for (int v = 0; v < NV; v++) {
    best_out[v] = best[v];
    bi_out[v] = bi[v];
    bj_out[v] = bj[v];
  }
}

/* Per-row and per-column substitution bases (see swl_sweep). */
static void swl_bases(const swl_v *A, swl_v *RB, int Mg, const swl_v *B, swl_v *CB, int Ng, const swl_score *sc) {
  /* Mg, Ng: counts of vectors */
  const swl_v three = swl_splat(3), nx = swl_splat(-sc->x), na = swl_splat(-sc->amb);
  for (int i = 0; i < Mg; i++) {
    const swl_v n = (swl_v)(A[i] > three);
    RB[i] = (n & na) | (~n & nx);
  }
  for (int j = 0; j < Ng; j++) {
    const swl_v n = (swl_v)(B[j] > three);
    CB[j] = (n & na) | (~n & nx);
  }
}

typedef struct {
  const char *a_seqs, *b_seqs;
  const int64_t *a_off, *b_off;
  const int32_t *a_len, *b_len;
  const int64_t *order; /* lane pairs, sorted by shape */
  int64_t n_lanes;
  const int64_t *scalar; /* pairs for the scalar restatement */
  int64_t n_scalar;
  swl_score sc;
  int8_t mat[25];
  int32_t *out;
  int64_t next_group, next_scalar;
  pthread_mutex_t mu;
} swl_batch;

static void *swl_worker(void *arg) {
  swl_batch *bt = (swl_batch *)arg;
  constexpr int NV = SWL_NV, L = SWL_LANES * SWL_NV;
  uint8_t *ca = NULL, *cb = NULL;
  int64_t cap_a = 0, cap_b = 0, cap_v = 0;
  swl_v *A = NULL, *B = NULL, *H = NULL, *E = NULL, *RB = NULL, *CB = NULL;
  const int64_t groups = (bt->n_lanes + L - 1) / L;
  /* lane k of a group: vector k / SWL_LANES, element k % SWL_LANES */
  auto at = [](swl_v *X, int pos, int k) -> int16_t & { return X[pos * NV + k / SWL_LANES][k % SWL_LANES]; };
  for (;;) {
    pthread_mutex_lock(&bt->mu);
    const int64_t g = bt->next_group++;
    int64_t sp = -1;
    if (g >= groups && bt->next_scalar < bt->n_scalar) sp = bt->next_scalar++;
    pthread_mutex_unlock(&bt->mu);
    if (g >= groups && sp < 0) break;
    if (sp >= 0) { /* scalar restatement */
      const int64_t p = bt->scalar[sp];
      const int32_t la = bt->a_len[p], lb = bt->b_len[p];
      uint8_t *xa = (uint8_t *)malloc((size_t)la + (size_t)lb + 16);
      sw_oracle_encode(bt->a_seqs + bt->a_off[p], la, xa);
      sw_oracle_encode(bt->b_seqs + bt->b_off[p], lb, xa + la);
      sw_oracle_align_codes(xa, la, xa + la, lb, bt->mat, bt->sc.gO, bt->sc.gE, bt->out + 5 * p);
      free(xa);
      continue;
    }
    const int64_t lo = g * L, hi = lo + L < bt->n_lanes ? lo + L : bt->n_lanes;
    int Mg = 0, Ng = 0;
    for (int64_t q = lo; q < hi; q++) {
      const int64_t p = bt->order[q];
      if (bt->a_len[p] > Mg) Mg = bt->a_len[p];
      if (bt->b_len[p] > Ng) Ng = bt->b_len[p];
    }
    const int64_t need = ((Mg > Ng ? Mg : Ng) + 1) * NV;
    if (need > cap_v) {
      free(A);
      cap_v = need + 64 * NV;
      A = (swl_v *)aligned_alloc(16, sizeof(swl_v) * 6 * (size_t)cap_v);
      B = A + cap_v;
      H = B + cap_v;
      E = H + cap_v;
      RB = E + cap_v;
      CB = RB + cap_v;
    }
    if (Mg > cap_a) {
      free(ca);
      cap_a = Mg + 64;
      ca = (uint8_t *)malloc((size_t)cap_a);
    }
    if (Ng > cap_b) {
      free(cb);
      cap_b = Ng + 64;
      cb = (uint8_t *)malloc((size_t)cap_b);
    }
    /* forward: lane k = pair order[lo + k] (empty lanes stay padding) */
    int32_t M[L], N[L];
    for (int i = 0; i < Mg * NV; i++) A[i] = swl_splat(4);
    for (int j = 0; j < Ng * NV; j++) B[j] = swl_splat(8);
    for (int k = 0; k < L; k++) {
      M[k] = N[k] = 0;
      if (lo + k >= hi) continue;
      const int64_t p = bt->order[lo + k];
      M[k] = bt->a_len[p];
      N[k] = bt->b_len[p];
      sw_oracle_encode(bt->a_seqs + bt->a_off[p], M[k], ca);
      sw_oracle_encode(bt->b_seqs + bt->b_off[p], N[k], cb);
      for (int i = 0; i < M[k]; i++) at(A, i, k) = ca[i];
      for (int j = 0; j < N[k]; j++) at(B, j, k) = cb[j] < 4 ? cb[j] : 8;
    }
    swl_v best[NV], bi[NV], bj[NV], S[NV], found[NV];
    for (int v = 0; v < NV; v++) {
      S[v] = swl_splat(0);
      found[v] = swl_splat(0);
    }
    swl_bases(A, RB, Mg * NV, B, CB, Ng * NV, &bt->sc);
    if (bt->sc.amb <= bt->sc.x)
      swl_sweep<NV, true>(A, RB, Mg, B, CB, Ng, &bt->sc, 0, S, H, E, best, bi, bj, found);
    else
      swl_sweep<NV, false>(A, RB, Mg, B, CB, Ng, &bt->sc, 0, S, H, E, best, bi, bj, found);
    /* reverse: A[0..a_end] and B[0..b_end] reversed; lanes with score 0 start found */
    int32_t ie[L], je[L], sc0[L];
    int Mr = 0, Nr = 0;
    for (int k = 0; k < L; k++) {
      const int v = k / SWL_LANES, e = k % SWL_LANES;
      ie[k] = bi[v][e];
      je[k] = bj[v][e];
      sc0[k] = best[v][e];
      S[v][e] = (int16_t)sc0[k];
      if (lo + k >= hi || sc0[k] <= 0) {
        S[v][e] = 32767;
        found[v][e] = -1;
        continue;
      }
      if (ie[k] + 1 > Mr) Mr = ie[k] + 1;
      if (je[k] + 1 > Nr) Nr = je[k] + 1;
    }
    swl_v rbi[NV], rbj[NV], rbest[NV];
    for (int v = 0; v < NV; v++) {
      rbi[v] = swl_splat(-1);
      rbj[v] = swl_splat(0);
    }
    if (Mr > 0) {
      for (int i = 0; i < Mr * NV; i++) A[i] = swl_splat(4);
      for (int j = 0; j < Nr * NV; j++) B[j] = swl_splat(8);
      for (int k = 0; k < L; k++) {
        if (found[k / SWL_LANES][k % SWL_LANES]) continue;
        const int64_t p = bt->order[lo + k];
        sw_oracle_encode(bt->a_seqs + bt->a_off[p], M[k], ca);
        sw_oracle_encode(bt->b_seqs + bt->b_off[p], N[k], cb);
        for (int i = 0; i <= ie[k]; i++) at(A, i, k) = ca[ie[k] - i];
        for (int j = 0; j <= je[k]; j++) at(B, j, k) = cb[je[k] - j] < 4 ? cb[je[k] - j] : 8;
      }
      swl_bases(A, RB, Mr * NV, B, CB, Nr * NV, &bt->sc);
      if (bt->sc.amb <= bt->sc.x)
        swl_sweep<NV, true>(A, RB, Mr, B, CB, Nr, &bt->sc, 1, S, H, E, rbest, rbi, rbj, found);
      else
        swl_sweep<NV, false>(A, RB, Mr, B, CB, Nr, &bt->sc, 1, S, H, E, rbest, rbi, rbj, found);
    }
    for (int k = 0; k < L; k++) {
      if (lo + k >= hi) continue;
      const int v = k / SWL_LANES, e = k % SWL_LANES;
      int32_t *o = bt->out + 5 * bt->order[lo + k];
      if (sc0[k] <= 0) {
        o[0] = 0;
        o[1] = -1;
        o[2] = -1;
        o[3] = 0;
        o[4] = 0;
      } else {
        o[0] = sc0[k];
        o[1] = ie[k] - rbi[v][e];
        o[2] = ie[k];
        o[3] = je[k] - rbj[v][e];
        o[4] = je[k];
      }
    }
  }
  free(A);
  free(ca);
  free(cb);
  return NULL;
}

typedef struct {
  int32_t key_a, key_b;
  int64_t p;
} swl_key;

static int swl_cmp(const void *x, const void *y) {
  const swl_key *a = (const swl_key *)x, *b = (const swl_key *)y;
  if (a->key_a != b->key_a) return a->key_a < b->key_a ? -1 : 1;
  if (a->key_b != b->key_b) return a->key_b < b->key_b ? -1 : 1;
  return a->p < b->p ? -1 : (a->p > b->p);
}

/* Same arguments and output as sw_oracle_align_batch (n x 5: score, a_begin, a_end,
 * b_begin, b_end). */
int sw_oracle_align_batch_lanes(const char *a_seqs, const int64_t *a_off, const int32_t *a_len, const char *b_seqs,
                                const int64_t *b_off, const int32_t *b_len, int64_t n, int match, int mismatch,
                                int gap_open, int gap_extend, int ambiguity, int nthreads, int32_t *out) {
  swl_batch bt;
  memset(&bt, 0, sizeof(bt));
  bt.a_seqs = a_seqs;
  bt.b_seqs = b_seqs;
  bt.a_off = a_off;
  bt.b_off = b_off;
  bt.a_len = a_len;
  bt.b_len = b_len;
  bt.out = out;
  bt.sc.m = match;
  bt.sc.x = mismatch;
  bt.sc.amb = ambiguity;
  bt.sc.gO = gap_open;
  bt.sc.gE = gap_extend;
  sw_oracle_matrix(match, mismatch, ambiguity, bt.mat);
  const int lanes_ok = ambiguity > 0 && gap_open > 0 && gap_extend >= 0 && match > 0 && match <= 127 &&
                       mismatch >= 0 && mismatch <= 127 && ambiguity <= 127 && gap_open <= 127 && gap_extend <= 127;
  swl_key *keys = (swl_key *)malloc(sizeof(swl_key) * (size_t)(n > 0 ? n : 1));
  int64_t *scalar = (int64_t *)malloc(sizeof(int64_t) * (size_t)(n > 0 ? n : 1));
  int64_t *order = (int64_t *)malloc(sizeof(int64_t) * (size_t)(n > 0 ? n : 1));
  int64_t nk = 0, ns = 0;
  for (int64_t p = 0; p < n; p++) {
    const int32_t la = a_len[p], lb = b_len[p];
    int32_t *o = out + 5 * p;
    o[0] = 0;
    o[1] = -1;
    o[2] = -1;
    o[3] = 0;
    o[4] = 0;
    if (la <= 0 || lb <= 0) continue;
    const int64_t mn = la < lb ? la : lb;
    if (!lanes_ok || mn * match >= 30000) {
      scalar[ns++] = p;
    } else {
      keys[nk].key_a = la;
      keys[nk].key_b = lb;
      keys[nk].p = p;
      nk++;
    }
  }
  qsort(keys, (size_t)nk, sizeof(swl_key), swl_cmp);
  for (int64_t q = 0; q < nk; q++) order[q] = keys[q].p;
  free(keys);
  bt.order = order;
  bt.n_lanes = nk;
  bt.scalar = scalar;
  bt.n_scalar = ns;
  pthread_mutex_init(&bt.mu, NULL);
  if (nthreads < 1) nthreads = 1;
  if (nthreads > 512) nthreads = 512;
  pthread_t th[512];
  for (int t = 1; t < nthreads; t++) pthread_create(&th[t], NULL, swl_worker, &bt);
  swl_worker(&bt);
  for (int t = 1; t < nthreads; t++) pthread_join(th[t], NULL);
  pthread_mutex_destroy(&bt.mu);
  free(order);
  free(scalar);
  return 0;
}
