// mhsw_cigar.cu -- CIGAR pass: SSW's report_cigar output (banded traceback, soft clips,
// =/X split and mismatch count) computed on the device after the begin pass.
//
// What SSW does (ssw_core.cpp:1180-1198 calls banded_sw, ssw_core.cpp:854-1053; then
// ConvertAlignment and CalculateNumberMismatch, ssw.cpp:57-254):
//   box      A[a_beg..a_end] (SSW ref, columns j) x B[b_beg..b_end] (SSW query, rows i);
//            no CIGAR for score 0 or when either span exceeds 32767 (the distance filter);
//   band     half-width w = |lenA - lenB| + 1, doubled until the band's maximum reaches
//            the score; cell (i, j) is in the band when |j - i| <= w;
//   cell     E = max(H_up - gO, E_up - gE), F = max(H_left - gO, F_left - gE) with F
//            starting at 0 in each row, H = max(max(E, 0), max(F, 0), H_diag + s), and the
//            direction of H = diagonal when that max is not below the diagonal term, else
//            E when max(E,0) > max(F,0), else F; cells outside the band read H = E = 0;
//   quirk    SSW clears one edge cell of its row buffers at each row start by an index
//            that, for rows i <= w + 1, lands on the previous row's last-column cell once
//            the band reaches the box's last column (lenA <= i + w): that cell's "up"
//            neighbour then reads H = E = 0;
//   trace    from (lenB - 1, lenA - 1) while i > 0, following the direction states; the
//            cell where the walk stops counts as one more M;
//   output   [S(b_beg)] + ops + [S(lenB_total - 1 - b_end)], every M split into runs of =
//            and X by comparing base codes along the CIGAR's own walk from the box's
//            start (N against N counts as =), mismatches = X + I + D lengths.
//
// GB300 mapping.  One thread per pair; the band is kept diagonal-indexed (k = j - i + w)
// so the rows slide without moving data: H and E of the previous row live in registers
// at fixed indices, the A codes of the band in a nibble-packed register window shifted
// one code per row.  Five instantiations hold half-widths up to 1, 3, 7, 15 and 31
// (cells per row 3 .. 63); a pair whose band doubles past its kernel's width moves to the
// next list, and boxes longer than kCigarRowCap rows or bands wider than 31 go to the
// generic kernel (rows and directions in global memory, host-driven rounds).  Directions
// take 4 bits per cell (E open/extend, F open/extend, H source) written one row word at
// a time, coalesced across the warp ([row][word][thread] layout).  The traceback walks
// the stored directions once, streaming the rows it visits through a ring of prefetched
// row words and recording its steps (2 bits each) in thread-local memory; replaying the
// record counts the ops and mismatches, then writes the ops back to front straight to
// their place in a shared arena reserved with one atomic per warp.  (The generic kernel,
// whose walks are unbounded, walks its stored directions three times instead.)
#include <cub/cub.cuh>

#include <algorithm>
#include <cstdint>

#include "mhsw_launch.h"
#include "mhsw_types.h"

namespace mhsw {

namespace {

enum : uint32_t { kOpM = 0, kOpI = 1, kOpD = 2, kOpS = 4, kOpEq = 7, kOpX = 8 };

struct CigarArgs {
  const uint8_t *a_code, *b_code;
  const int64_t *a_off, *b_off;
  const int32_t *b_len;
  const int32_t *score, *a_beg, *a_end, *b_beg, *b_end;
  int match, mismatch, amb, gO, gE;
  int32_t *nops, *mism;
  int64_t *op_off;
  uint32_t *arena;
  int64_t arena_cap;
  unsigned long long *cursor;
  int *counts;
  uint32_t *keys, *idx;           // classification output (sort input)
  const uint32_t *sorted;         // pairs in (class, rows descending) order
  int2 *lists;
  int64_t list_cap;
  int4 *generic;
  uint32_t *dirs;
};

__host__ __device__ constexpr int cigar_half(int c) { return c == 0 ? 1 : c == 1 ? 3 : c == 2 ? 7 : c == 3 ? 15 : 31; }

__device__ __forceinline__ int list_for(int w, int rows) {
  if (rows > kCigarRowCap) return kCigarGeneric;
#pragma unroll
  for (int c = 0; c < kCigarClasses; c++)
    if (w <= cigar_half(c)) return c;
  return kCigarGeneric;
}

__device__ __forceinline__ int sub_score(const CigarArgs &g, int a, int b) {
  return (a == kCodeN || b == kCodeN) ? -g.amb : (a == b ? g.match : -g.mismatch);
}

// Appends (p, w) to the generic list or to register kernel c's escalation list.
__device__ __forceinline__ void list_push(const CigarArgs &g, int c, int p, int w, int rows, int ref_len) {
  if (c == kCigarGeneric) {
    const int at = atomicAdd(&g.counts[kCigarGeneric], 1);
    g.generic[at] = make_int4(p, w, rows, ref_len);
    return;
  }
  const int at = atomicAdd(&g.counts[kCigarEsc + c], 1);
  g.lists[(int64_t)c * g.list_cap + at] = make_int2(p, w);
}

constexpr uint32_t kKeyNone = (1u << 13) - 1;  // sorts after every (class, rows) key

// order (may be null): the batched forward pass's length-sorted pair order, so pairs of
// similar length share warps in every list.
// Per pair: the register kernel its first band fits (key = class, then box rows
// descending, so a warp's lanes take boxes of about the same height, longest first), or
// the generic list.  order (may be null): the batched forward pass's pair order.
__global__ void k_cigar_classify(CigarArgs g, int64_t n, const uint32_t *__restrict__ order) {
  const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= n) return;
  const int64_t p = order ? (int64_t)order[idx] : idx;
  g.nops[p] = 0;
  g.mism[p] = 0;
  g.op_off[p] = 0;
  uint32_t key = kKeyNone;
  const int S = g.score[p], ab = g.a_beg[p], ae = g.a_end[p], bb = g.b_beg[p], be = g.b_end[p];
  if (S > 0 && ab >= 0 && bb >= 0 && ae - ab <= 32767 && be - bb <= 32767) {
    const int ref_len = ae - ab + 1, rows = be - bb + 1;
    const int w = abs(ref_len - rows) + 1;
    const int c = list_for(w, rows);
    if (c == kCigarGeneric) {
      list_push(g, c, (int)p, w, rows, ref_len);
    } else {
      key = ((uint32_t)c << 10) | (uint32_t)(1023 - rows);
      const unsigned act = __activemask();  // the lanes on this path only
      const unsigned peers = __match_any_sync(act, c);
      const int leader = __ffs(peers) - 1;
      if ((int)(threadIdx.x & 31) == leader) atomicAdd(&g.counts[c], __popc(peers));
    }
  }
  g.keys[idx] = key;
  g.idx[idx] = (uint32_t)p;
}

// ---- traceback (shared by the register and the generic kernels) ----------------------

// One step from (i, j) in state st (0 = E, 1 = F, 2 = H); returns the op (kOpM/I/D) or
// -1 when the walk leaves the cells the final pass computed.
template <class Dir>
__device__ __forceinline__ int tb_step(const Dir &dir, int w, int &i, int &j, int &st) {
  if (j < 0) return -1;
  const int k = j - i + w;
  if (k < 0 || k > 2 * w) return -1;
  const uint32_t nib = dir(i, k);
  int code;
  if (st == 0) {
    code = 2 + (int)(nib & 1u);
  } else if (st == 1) {
    code = 4 + (int)((nib >> 1) & 1u);
  } else {
    const uint32_t hs = nib >> 2;
    code = hs == 0 ? 1 : hs == 1 ? 2 + (int)(nib & 1u) : hs == 2 ? 4 + (int)((nib >> 1) & 1u) : 0;
  }
  switch (code) {
    case 1: --i; --j; st = 2; return kOpM;
    case 2: --i; st = 0; return kOpI;
    case 3: --i; st = 2; return kOpI;
    case 4: --j; st = 1; return kOpD;
    case 5: --j; st = 2; return kOpD;
    default: return -1;
  }
}

struct Box {
  const uint8_t *A, *B;  // codes at the box start
  int ref_len, rows;     // box extents (A columns, B rows)
  int bb, tail;          // soft clips: leading B bases, trailing B bases
};

// Walk the stored directions.  mode 0: returns the end column j_end; mode 1: counts the
// final ops (*nops) and mismatches; mode 2: writes the ops to out[0 .. nops) back to
// front.  Returns false when the walk leaves the computed cells.
template <class Dir>
__device__ bool tb_walk(const Dir &dir, const Box &bx, int w, int mode, int j_end, int *res, int *mm, uint32_t *out,
                        int nops) {
  int t = 0, run_kind = -1, run_len = 0, mis = 0;
  auto emit = [&](uint32_t kind, int len) {
    if (mode == 2) out[nops - 1 - t] = ((uint32_t)len << 4) | kind;
    ++t;
  };
  auto cell = [&](int kind) {
    if (kind == run_kind) {
      ++run_len;
    } else {
      if (run_len > 0) emit((uint32_t)run_kind, run_len);
      run_kind = kind;
      run_len = 1;
    }
  };
  if (mode > 0 && bx.tail > 0) emit(kOpS, bx.tail);
  int i = bx.rows - 1, j = bx.ref_len - 1, st = 2;
  while (i > 0) {
    const int ci = i, cj = j;
    const int op = tb_step(dir, w, i, j, st);
    if (op < 0) return false;
    if (mode == 0) continue;
    if (op == kOpM) {
      const bool x = bx.A[cj - j_end] != bx.B[ci];
      mis += x;
      cell(x ? kOpX : kOpEq);
    } else {
      ++mis;
      cell(op);
    }
  }
  if (mode == 0) {
    *res = j;
    return true;
  }
  // the cell where the walk stopped: one more M, at the CIGAR's first column
  const bool x = bx.A[0] != bx.B[0];
  mis += x;
  cell(x ? kOpX : kOpEq);
  if (run_len > 0) emit((uint32_t)run_kind, run_len);
  if (bx.bb > 0) emit(kOpS, bx.bb);
  *res = t;
  *mm = mis;
  return true;
}

// Arena space for `want` ops.  warp_sync: every lane of the warp calls together and the
// warp reserves its total with one atomic (lanes with nothing to write pass 0).
__device__ __forceinline__ int64_t reserve_arena(const CigarArgs &g, int want, bool warp_sync) {
  if (!warp_sync) return want > 0 ? (int64_t)atomicAdd(g.cursor, (unsigned long long)want) : 0;
  const int lane = threadIdx.x & 31;
  int incl = want;
#pragma unroll
  for (int s = 1; s < 32; s <<= 1) {
    const int v = __shfl_up_sync(0xffffffffu, incl, s);
    if (lane >= s) incl += v;
  }
  unsigned long long wb = 0;
  if (lane == 31 && incl > 0) wb = atomicAdd(g.cursor, (unsigned long long)incl);
  wb = __shfl_sync(0xffffffffu, wb, 31);
  return (int64_t)wb + incl - want;
}

// Three walks: end column, count, then (after the arena reservation) the ops.  Lanes of
// a warp reserve their arena space with one atomic; `valid` lanes with nothing to write
// join the reservation with 0 ops.
template <class Dir>
__device__ void traceback_and_emit(const CigarArgs &g, const Dir &dir, const Box &bx, int w, int p, bool valid,
                                   bool warp_sync) {
  int j_end = 0, nops = 0, mm = 0;
  bool ok = valid;
  if (ok) ok = tb_walk(dir, bx, w, 0, 0, &j_end, nullptr, nullptr, 0);
  if (ok) ok = tb_walk(dir, bx, w, 1, j_end, &nops, &mm, nullptr, 0);
  if (valid && !ok) {
    g.nops[p] = -1;
    atomicAdd(&g.counts[kCigarWalkErrors], 1);
  }
  const int want = ok ? nops : 0;
  const int64_t base = reserve_arena(g, want, warp_sync);
  if (!ok) return;
  if (base + want > g.arena_cap) {  // arena full: the host grows it and runs the pass again
    g.nops[p] = -1;
    atomicAdd(&g.counts[kCigarArenaFull], 1);
    return;
  }
  int t2 = 0, mm2 = 0;
  tb_walk(dir, bx, w, 2, j_end, &t2, &mm2, g.arena + base, nops);
  g.op_off[p] = base;
  g.nops[p] = nops;
  g.mism[p] = mm;
}

// ---- register-band kernels ------------------------------------------------------------

// Register kernels' traceback.  The direction walk is a chain of dependent loads (each
// step's position comes from the previous step's nibble), so it runs once: the rows it
// visits stream through a ring of prefetched row words (P rows of NW words, P * NW = 8,
// loaded P rows ahead of the walk), and its steps are recorded, 2 bits each, in a
// thread-local array.  Counting and writing the ops then replay the record.
constexpr int kPathWords = 68;  // 16 steps a word; a walk takes at most
                                // (kCigarRowCap - 1) + (kCigarRowCap + 30 - 1) steps

template <int NW>
struct RowRing {
  static constexpr int P = 8 / NW;
  uint32_t r[P][NW];
  const uint32_t *base;
  int64_t stride;
  __device__ __forceinline__ void load(uint32_t (&dst)[NW], int i) const {
#pragma unroll
    for (int q = 0; q < NW; q++) dst[q] = i >= 0 ? __ldcg(base + ((int64_t)i * NW + q) * stride) : 0u;
  }
  __device__ __forceinline__ void init(int top) {
#pragma unroll
    for (int p = 0; p < P; p++) load(r[p], top - p);
  }
  __device__ __forceinline__ void down(int new_top) {  // the walk moved from row new_top + 1
#pragma unroll
    for (int p = 0; p + 1 < P; p++)
#pragma unroll
      for (int q = 0; q < NW; q++) r[p][q] = r[p + 1][q];
    load(r[P - 1], new_top - (P - 1));
  }
  __device__ __forceinline__ uint32_t nib(int k) const {
    uint32_t w = r[0][0];
#pragma unroll
    for (int q = 1; q < NW; q++)
      if ((k >> 3) == q) w = r[0][q];
    return (w >> ((k & 7) * 4)) & 15u;
  }
};

// Walk 1: returns false when the walk leaves the computed band (or outgrows the record).
template <int NW>
__device__ bool walk_record(RowRing<NW> &ring, const Box &bx, int w, uint32_t *path, int *nsteps, int *j_end) {
  int i = bx.rows - 1, j = bx.ref_len - 1, st = 2, n = 0;
  ring.init(i);
  while (i > 0) {
    if (j < 0 || n >= kPathWords * 16) return false;
    const int k = j - i + w;
    if (k < 0 || k > 2 * w) return false;
    const uint32_t nb = ring.nib(k);
    int code;
    if (st == 0) {
      code = 2 + (int)(nb & 1u);
    } else if (st == 1) {
      code = 4 + (int)((nb >> 1) & 1u);
    } else {
      const uint32_t hs = nb >> 2;
      code = hs == 0 ? 1 : hs == 1 ? 2 + (int)(nb & 1u) : hs == 2 ? 4 + (int)((nb >> 1) & 1u) : 0;
    }
    uint32_t op;
    switch (code) {
      case 1: --i; --j; st = 2; op = kOpM; break;
      case 2: --i; st = 0; op = kOpI; break;
      case 3: --i; st = 2; op = kOpI; break;
      case 4: --j; st = 1; op = kOpD; break;
      case 5: --j; st = 2; op = kOpD; break;
      default: return false;
    }
    if ((n & 15) == 0) path[n >> 4] = 0u;
    path[n >> 4] |= op << ((n & 15) * 2);
    ++n;
    if (op != kOpD) ring.down(i);
  }
  *nsteps = n;
  *j_end = j;
  return true;
}

// Replays the record.  mode 1: counts ops (*res) and mismatches (*mm), comparing the
// bases of the M steps with loads issued 8 steps at a time, and keeps each M step's
// =/X outcome in xf (1 bit a step); mode 2: writes the ops to out[0 .. nops) back to
// front from the record and xf alone.
__device__ void replay_path(const Box &bx, const uint32_t *path, uint32_t *xf, int nsteps, int j_end, int mode,
                            int *res, int *mm, uint32_t *out, int nops) {
  int t = 0, run_kind = -1, run_len = 0, mis = 0;
  auto emit = [&](uint32_t kind, int len) {
    if (mode == 2) out[nops - 1 - t] = ((uint32_t)len << 4) | kind;
    ++t;
  };
  auto cell = [&](int kind) {
    if (kind == run_kind) {
      ++run_len;
    } else {
      if (run_len > 0) emit((uint32_t)run_kind, run_len);
      run_kind = kind;
      run_len = 1;
    }
  };
  if (bx.tail > 0) emit(kOpS, bx.tail);
  int ci = bx.rows - 1, cj = bx.ref_len - 1;
  for (int s0 = 0; s0 < nsteps; s0 += 8) {
    uint32_t xbits = 0;
    if (mode == 1) {
      uint32_t av[8], bv[8];
      int i = ci, j = cj;
#pragma unroll
      for (int u = 0; u < 8; u++) {  // positions and independent loads of up to 8 steps
        const int st = s0 + u;
        const uint32_t op = st < nsteps ? (path[st >> 4] >> ((st & 15) * 2)) & 3u : kOpD;
        av[u] = bv[u] = 0;
        if (st < nsteps && op == kOpM) {
          av[u] = bx.A[j - j_end];
          bv[u] = bx.B[i];
        }
        i -= op != kOpD;
        j -= op != kOpI;
      }
#pragma unroll
      for (int u = 0; u < 8; u++) xbits |= (uint32_t)(av[u] != bv[u]) << u;
      if ((s0 & 31) == 0) xf[s0 >> 5] = 0u;
      xf[s0 >> 5] |= xbits << (s0 & 31);
    } else {
      xbits = (xf[s0 >> 5] >> (s0 & 31)) & 0xffu;
    }
#pragma unroll
    for (int u = 0; u < 8; u++) {
      const int st = s0 + u;
      if (st >= nsteps) break;
      const uint32_t op = (path[st >> 4] >> ((st & 15) * 2)) & 3u;
      if (op == kOpM) {
        const bool x = (xbits >> u) & 1u;
        mis += x;
        cell(x ? kOpX : kOpEq);
        --ci;
        --cj;
      } else if (op == kOpI) {
        ++mis;
        cell(kOpI);
        --ci;
      } else {
        ++mis;
        cell(kOpD);
        --cj;
      }
    }
  }
  const bool x = bx.A[0] != bx.B[0];  // the cell where the walk stopped: one more M
  mis += x;
  cell(x ? kOpX : kOpEq);
  if (run_len > 0) emit((uint32_t)run_kind, run_len);
  if (bx.bb > 0) emit(kOpS, bx.bb);
  *res = t;
  *mm = mis;
}

template <int NW>
__device__ void traceback_reg(const CigarArgs &g, const uint32_t *dcol, int64_t stride, const Box &bx, int w, int p,
                              bool valid) {
  uint32_t path[kPathWords], xf[kPathWords / 2];
  int nsteps = 0, j_end = 0, nops = 0, mm = 0;
  bool ok = valid;
  if (ok) {
    RowRing<NW> ring;
    ring.base = dcol;
    ring.stride = stride;
    ok = walk_record(ring, bx, w, path, &nsteps, &j_end);
    if (!ok) {
      g.nops[p] = -1;
      atomicAdd(&g.counts[kCigarWalkErrors], 1);
    } else {
      replay_path(bx, path, xf, nsteps, j_end, 1, &nops, &mm, nullptr, 0);
    }
  }
  const int want = ok ? nops : 0;
  const int64_t base = reserve_arena(g, want, true);
  if (!ok) return;
  if (base + want > g.arena_cap) {  // arena full: the host grows it and runs the pass again
    g.nops[p] = -1;
    atomicAdd(&g.counts[kCigarArenaFull], 1);
    return;
  }
  int t2 = 0, mm2 = 0;
  replay_path(bx, path, xf, nsteps, j_end, 2, &t2, &mm2, g.arena + base, nops);
  g.op_off[p] = base;
  g.nops[p] = nops;
  g.mism[p] = mm;
}

// One banded DP pass at half-width w <= W; returns the band's maximum.
template <int W>
__device__ int band_pass(const CigarArgs &g, const Box &bx, int w, uint32_t *dcol, int64_t stride) {
  constexpr int K = 2 * W + 1;
  constexpr int NW = (K + 7) / 8;  // direction words per row (8 nibbles each)
  constexpr int NC = (K + 7) / 8;  // A-code window words (8 nibbles each)
  int H[K + 1], E[K + 1];
#pragma unroll
  for (int k = 0; k <= K; k++) H[k] = E[k] = 0;
  uint32_t win[NC];
#pragma unroll
  for (int q = 0; q < NC; q++) win[q] = 0;
#pragma unroll
  for (int k = 0; k < K; k++) {
    const int pos = k - w;
    const uint32_t c = (pos >= 0 && pos < bx.ref_len) ? bx.A[pos] : 0u;
    win[k >> 3] |= c << ((k & 7) * 4);
  }
  int mx = 0;
  for (int i = 0; i < bx.rows; i++) {
    const int qb = bx.B[i];
    const int kstart = max(0, w - i), kend = min(2 * w, bx.ref_len - 1 - i + w);
    const bool clob = i >= 1 && i <= w + 1 && bx.ref_len <= i + w;
    int f = 0, hl = 0;
    uint32_t dw[NW];
#pragma unroll
    for (int q = 0; q < NW; q++) dw[q] = 0;
#pragma unroll
    for (int k = 0; k < K; k++) {
      if (k >= kstart && k <= kend) {
        int hu = H[k + 1], eu = E[k + 1];
        if (clob && k == kend) hu = eu = 0;
        int t1 = hu - g.gO, t2 = eu - g.gE;
        const int e = max(t1, t2);
        const uint32_t de = t1 > t2;
        t1 = hl - g.gO;
        t2 = f - g.gE;
        f = max(t1, t2);
        const uint32_t df = t1 > t2;
        const int e1 = max(e, 0), f1 = max(f, 0), m1 = max(e1, f1);
        const int ac = (int)((win[k >> 3] >> ((k & 7) * 4)) & 15u);
        const int dg = H[k] + sub_score(g, ac, qb);
        const int h = max(m1, dg);
        const uint32_t hs = m1 <= dg ? 0u : (e1 > f1 ? 1u : 2u);
        H[k] = h;
        E[k] = e;
        hl = h;
        mx = max(mx, h);
        dw[k >> 3] |= (de | (df << 1) | (hs << 2)) << ((k & 7) * 4);
      }
    }
#pragma unroll
    for (int q = 0; q < NW; q++) __stcg(dcol + ((int64_t)i * NW + q) * stride, dw[q]);
    // slide the window one code: new k = old k + 1; the last slot takes A[i + 1 - w + K - 1]
#pragma unroll
    for (int q = 0; q < NC; q++) win[q] = (win[q] >> 4) | (q + 1 < NC ? (win[q + 1] << 28) : 0u);
    const int pos = i + 1 - w + K - 1;
    const uint32_t c = (pos >= 0 && pos < bx.ref_len) ? bx.A[pos] : 0u;
    win[(K - 1) >> 3] |= c << (((K - 1) & 7) * 4);
  }
  return mx;
}

__device__ __forceinline__ Box make_box(const CigarArgs &g, int p) {
  Box bx;
  const int ab = g.a_beg[p], ae = g.a_end[p], bb = g.b_beg[p], be = g.b_end[p];
  bx.A = g.a_code + g.a_off[p] + ab;
  bx.B = g.b_code + g.b_off[p] + bb;
  bx.ref_len = ae - ab + 1;
  bx.rows = be - bb + 1;
  bx.bb = bb;
  bx.tail = g.b_len[p] - 1 - be;
  return bx;
}

template <int C>
__global__ void __launch_bounds__(128) k_cigar_band(CigarArgs g) {
  constexpr int W = cigar_half(C);
  constexpr int NW = (2 * W + 1 + 7) / 8;
  const int64_t T = (int64_t)gridDim.x * blockDim.x;
  const int64_t tid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  // this kernel's segment of the sorted pairs, then its escalation list
  int seg0 = 0;
#pragma unroll
  for (int c = 0; c < C; c++) seg0 += g.counts[c];
  const int seg_n = g.counts[C];
  const int count = seg_n + g.counts[kCigarEsc + C];
  const int2 *list = g.lists + (int64_t)C * g.list_cap;
  uint32_t *dcol = g.dirs + tid;
  // warp-uniform trip count: every lane reaches the arena reservation together
  for (int64_t base = tid - (threadIdx.x & 31); base < count; base += T) {
    const int64_t e = base + (threadIdx.x & 31);
    bool valid = e < count;
    int p = 0, w = 0;
    Box bx{};
    if (valid) {
      if (e < seg_n) {
        p = (int)g.sorted[seg0 + e];
        bx = make_box(g, p);
        w = abs(bx.ref_len - bx.rows) + 1;
      } else {
        const int2 ent = list[e - seg_n];
        p = ent.x;
        w = ent.y;
        bx = make_box(g, p);
      }
      const int S = g.score[p];
      for (;;) {
        if (w > W) {
          list_push(g, list_for(w, bx.rows), p, w, bx.rows, bx.ref_len);
          valid = false;
          break;
        }
        if (band_pass<W>(g, bx, w, dcol, T) >= S) break;
        w *= 2;
      }
    }
    __syncwarp();
    traceback_reg<NW>(g, dcol, T, bx, w, p, valid);
  }
}

// ---- generic kernel (any band, any box): rows and directions in a global slice --------

struct SliceDir {
  const uint32_t *d;
  int nw;
  __device__ __forceinline__ uint32_t operator()(int i, int k) const {
    return (d[(int64_t)i * nw + (k >> 3)] >> ((k & 7) * 4)) & 15u;
  }
};

__device__ int any_pass(const CigarArgs &g, const Box &bx, int w, int *Hs, int *Es, uint32_t *D) {
  const int nw = (2 * w + 1 + 7) / 8;
  for (int k = 0; k <= 2 * w + 1; k++) Hs[k] = Es[k] = 0;
  int mx = 0;
  for (int i = 0; i < bx.rows; i++) {
    const int qb = bx.B[i];
    const int kstart = max(0, w - i), kend = min(2 * w, bx.ref_len - 1 - i + w);
    const bool clob = i >= 1 && i <= w + 1 && bx.ref_len <= i + w;
    uint32_t *row = D + (int64_t)i * nw;
    for (int q = 0; q < nw; q++) row[q] = 0;
    int f = 0, hl = 0;
    uint32_t word = 0;
    int wq = kstart >> 3;
    for (int k = kstart; k <= kend; k++) {
      if ((k >> 3) != wq) {
        row[wq] = word;
        word = 0;
        wq = k >> 3;
      }
      int hu = Hs[k + 1], eu = Es[k + 1];
      if (clob && k == kend) hu = eu = 0;
      int t1 = hu - g.gO, t2 = eu - g.gE;
      const int e = max(t1, t2);
      const uint32_t de = t1 > t2;
      t1 = hl - g.gO;
      t2 = f - g.gE;
      f = max(t1, t2);
      const uint32_t df = t1 > t2;
      const int e1 = max(e, 0), f1 = max(f, 0), m1 = max(e1, f1);
      const int dg = Hs[k] + sub_score(g, bx.A[i - w + k], qb);
      const int h = max(m1, dg);
      const uint32_t hs = m1 <= dg ? 0u : (e1 > f1 ? 1u : 2u);
      Hs[k] = h;
      Es[k] = e;
      hl = h;
      mx = max(mx, h);
      word |= (de | (df << 1) | (hs << 2)) << ((k & 7) * 4);
    }
    if (kstart <= kend) row[wq] = word;
  }
  return mx;
}

__global__ void k_cigar_any(CigarArgs g, const int4 *entries, int count, int threads, unsigned char *pool,
                            size_t slice) {
  const int64_t T = threads;  // the pool holds `threads` slices; the grid may round up past it
  const int64_t tid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (tid >= T) return;
  unsigned char *my = pool + (size_t)tid * slice;
  for (int64_t e = tid; e < count; e += T) {
    const int4 ent = entries[e];
    const int p = ent.x;
    int w = ent.y;
    const Box bx = make_box(g, p);
    const int S = g.score[p];
    bool ok = true;
    for (;;) {
      const size_t need = cigar_slice_bytes(w, bx.rows);
      if (need > slice) {  // the host sized slices for the widest band a box can need
        ok = false;
        break;
      }
      int *Hs = reinterpret_cast<int *>(my);
      int *Es = Hs + (2 * w + 2);
      uint32_t *D = reinterpret_cast<uint32_t *>(Es + (2 * w + 2));
      if (any_pass(g, bx, w, Hs, Es, D) >= S) break;
      w *= 2;
    }
    if (!ok) {
      g.nops[p] = -1;
      atomicAdd(&g.counts[kCigarWalkErrors], 1);
      continue;
    }
    int *Hs = reinterpret_cast<int *>(my);
    const SliceDir dir{reinterpret_cast<const uint32_t *>(Hs + 2 * (2 * w + 2)), (2 * w + 1 + 7) / 8};
    traceback_and_emit(g, dir, bx, w, p, true, false);
  }
}

// ---- pair-order gather ----------------------------------------------------------------

__global__ void k_cigar_counts64(const int32_t *nops, int64_t n, int64_t *c64) {
  const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p < n) c64[p] = nops[p] > 0 ? nops[p] : 0;
  if (p == n) c64[p] = 0;
}

__global__ void k_cigar_gather(const int32_t *nops, const int64_t *op_off, const uint32_t *arena, int64_t n,
                               const int64_t *ord_off, uint32_t *ord_ops) {
  const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  const int k = nops[p];
  const uint32_t *src = arena + op_off[p];
  uint32_t *dst = ord_ops + ord_off[p];
  for (int t = 0; t < k; t++) dst[t] = src[t];
}

__global__ void k_cigar_reset(int *counts, unsigned long long *cursor) {
  if (threadIdx.x < kCigarCounters) counts[threadIdx.x] = 0;
  if (threadIdx.x == 0) *cursor = 0ull;
}

CigarArgs make_args(const PairSet &ps, const ResultSet &rs, const Scoring &sc, const CigarBufs &cb) {
  CigarArgs g;
  g.a_code = ps.a_code;
  g.b_code = ps.b_code;
  g.a_off = ps.a_off;
  g.b_off = ps.b_off;
  g.b_len = ps.b_len;
  g.score = rs.score;
  g.a_beg = rs.a_beg;
  g.a_end = rs.a_end;
  g.b_beg = rs.b_beg;
  g.b_end = rs.b_end;
  g.match = sc.match;
  g.mismatch = sc.mismatch;
  g.amb = sc.ambiguity;
  g.gO = sc.gap_open;
  g.gE = sc.gap_extend;
  g.nops = cb.nops;
  g.mism = cb.mism;
  g.op_off = cb.op_off;
  g.arena = cb.arena;
  g.arena_cap = cb.arena_cap;
  g.cursor = cb.cursor;
  g.counts = cb.counts;
  g.keys = cb.keys_in;
  g.idx = cb.idx_in;
  g.sorted = cb.idx_out;
  g.lists = cb.lists;
  g.list_cap = cb.list_cap;
  g.generic = cb.generic;
  g.dirs = cb.dirs;
  return g;
}

template <int C>
cudaError_t launch_band(const CigarArgs &g, int sms, size_t dirs_bytes, cudaStream_t st) {
  constexpr int W = cigar_half(C);
  constexpr int NW = (2 * W + 1 + 7) / 8;
  const int64_t per_thread = (int64_t)kCigarRowCap * NW * 4;
  int64_t threads = std::min<int64_t>((int64_t)dirs_bytes / per_thread, (int64_t)sms * 8 * 128);
  const int blocks = (int)std::max<int64_t>(1, threads / 128);
  k_cigar_band<C><<<blocks, 128, 0, st>>>(g);
  return cudaGetLastError();
}

}  // namespace

cudaError_t launch_cigar(const PairSet &ps, const ResultSet &rs, const Scoring &sc, const CigarBufs &cb, int sms,
                         const uint32_t *order, cudaStream_t st, int64_t *launches) {
  const CigarArgs g = make_args(ps, rs, sc, cb);
  k_cigar_reset<<<1, 32, 0, st>>>(cb.counts, cb.cursor);
  const int64_t n = ps.n;
  if (n > 0) k_cigar_classify<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(g, n, order);
  cudaError_t e = cudaGetLastError();
  if (e) return e;
  if (n > 0) {
    size_t tb = cb.sort_temp_bytes;
    e = cub::DeviceRadixSort::SortPairs(cb.sort_temp, tb, cb.keys_in, cb.keys_out, cb.idx_in, cb.idx_out, (int)n, 0,
                                        13, st);
    if (e) return e;
  }
  if ((e = launch_band<0>(g, sms, cb.dirs_bytes, st))) return e;
  if ((e = launch_band<1>(g, sms, cb.dirs_bytes, st))) return e;
  if ((e = launch_band<2>(g, sms, cb.dirs_bytes, st))) return e;
  if ((e = launch_band<3>(g, sms, cb.dirs_bytes, st))) return e;
  if ((e = launch_band<4>(g, sms, cb.dirs_bytes, st))) return e;
  if (launches) *launches += 2 + kCigarClasses + 4;  // + the radix sort's passes (approximate)
  return cudaSuccess;
}

cudaError_t launch_cigar_generic(const PairSet &ps, const ResultSet &rs, const Scoring &sc, const CigarBufs &cb,
                                 const int4 *entries, int count, int threads, size_t slice, void *pool,
                                 cudaStream_t st) {
  if (count <= 0) return cudaSuccess;
  const CigarArgs g = make_args(ps, rs, sc, cb);
  const int block = threads < 64 ? threads : 64;
  const int blocks = (threads + block - 1) / block;
  k_cigar_any<<<blocks, block, 0, st>>>(g, entries, count, threads, static_cast<unsigned char *>(pool), slice);
  return cudaGetLastError();
}

cudaError_t cigar_sort_temp_bytes(int64_t n, size_t *bytes) {
  *bytes = 0;
  return cub::DeviceRadixSort::SortPairs(nullptr, *bytes, (const uint32_t *)nullptr, (uint32_t *)nullptr,
                                         (const uint32_t *)nullptr, (uint32_t *)nullptr, (int)std::max<int64_t>(n, 1),
                                         0, 13);
}

cudaError_t cigar_gather_temp_bytes(int64_t n, size_t *bytes) {
  *bytes = 0;
  return cub::DeviceScan::ExclusiveSum(nullptr, *bytes, (const int64_t *)nullptr, (int64_t *)nullptr, (int)(n + 1));
}

cudaError_t launch_cigar_gather(const CigarBufs &cb, int64_t n, int64_t *c64, int64_t *ord_off, uint32_t *ord_ops,
                                void *temp, size_t temp_bytes, cudaStream_t st) {
  k_cigar_counts64<<<(unsigned)((n + 1 + 255) / 256), 256, 0, st>>>(cb.nops, n, c64);
  cudaError_t e = cub::DeviceScan::ExclusiveSum(temp, temp_bytes, c64, ord_off, (int)(n + 1), st);
  if (e) return e;
  if (ord_ops && n > 0)
    k_cigar_gather<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(cb.nops, cb.op_off, cb.arena, n, ord_off, ord_ops);
  return cudaGetLastError();
}

}  // namespace mhsw
