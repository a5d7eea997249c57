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
// one code per row.  Six instantiations hold half-widths up to 1, 2, 4, 8, 16 and 31
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

// Half-widths of the register kernels: escalation doubles a band, so chains that start
// at 1, 2 or 4 land on full-width kernels.
__host__ __device__ constexpr int cigar_half(int c) {
  return c == 0 ? 1 : c == 1 ? 2 : c == 2 ? 4 : c == 3 ? 8 : c == 4 ? 16 : 31;
}

// The register kernel a band of half-width w over `rows` rows fits, or kCigarClasses
// (the generic kernel).
__device__ __forceinline__ int list_for(int w, int rows) {
  if (rows > kCigarRowCap) return kCigarClasses;
#pragma unroll
  for (int c = 0; c < kCigarClasses; c++)
    if (w <= cigar_half(c)) return c;
  return kCigarClasses;
}

__device__ __forceinline__ int sub_score(const CigarArgs &g, int a, int b) {
  return (a == kCodeN || b == kCodeN) ? -g.amb : (a == b ? g.match : -g.mismatch);
}

// Appends (p, w) to register kernel c's escalation list, or (c == kCigarClasses) to the
// generic list.
__device__ __forceinline__ void list_push(const CigarArgs &g, int c, int p, int w, int rows, int ref_len) {
  if (c == kCigarClasses) {
    const int at = atomicAdd(&g.counts[kCigarGeneric], 1);
    g.generic[at] = make_int4(p, w, rows, ref_len);
    return;
  }
  const int at = atomicAdd(&g.counts[kCigarEsc + c], 1);
  g.lists[(int64_t)c * g.list_cap + at] = make_int2(p, w);
}

constexpr uint32_t kKeyNone = (1u << 13) - 1;  // sorts after every (class, rows) key

struct Box {
  const uint8_t *A, *B;  // codes at the box start
  int ref_len, rows;     // box extents (A columns, B rows)
  int bb, tail;          // soft clips: leading B bases, trailing B bases
};

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

// A code stream read through registers: 16-byte loads, one vector ahead of use, so the
// DP's rows never wait on a byte load.  Loads start at 16-byte boundaries and never past
// the vector that holds the stream's last code (the code arenas keep 16 bytes of slack).
struct CodeStream {
  const uint8_t *next_vec, *lim;  // the next vector to load; one past the stream's last code
  uint4 cur, nxt;
  int o;     // byte offset of the next code in cur
  int left;  // codes left (0 is returned after the last)
  __device__ __forceinline__ static uint4 ld(const uint8_t *v, const uint8_t *lim) {
    return v < lim ? __ldg(reinterpret_cast<const uint4 *>(v)) : make_uint4(0u, 0u, 0u, 0u);
  }
  __device__ __forceinline__ void init(const uint8_t *start, int len) {
    const uint8_t *v = reinterpret_cast<const uint8_t *>(reinterpret_cast<uintptr_t>(start) & ~uintptr_t(15));
    lim = start + (len > 0 ? len : 0);
    cur = ld(v, lim);
    nxt = ld(v + 16, lim);
    next_vec = v + 32;
    o = (int)(reinterpret_cast<uintptr_t>(start) & 15);
    left = len;
  }
  __device__ __forceinline__ uint32_t next() {
    const uint32_t w = o < 8 ? (o < 4 ? cur.x : cur.y) : (o < 12 ? cur.z : cur.w);
    const uint32_t b = left > 0 ? (w >> ((o & 3) * 8)) & 0xffu : 0u;
    --left;
    if (++o == 16) {
      cur = nxt;
      nxt = ld(next_vec, lim);
      next_vec += 16;
      o = 0;
    }
    return b;
  }
};

// A box as high as wide whose diagonal scores the full score needs no DP: every cell
// of the diagonal then holds exactly the diagonal's prefix score (a higher value there
// would give the corner more than the maximum), so banded_sw's traceback, which takes the
// diagonal on ties, follows it from corner to corner.  Its CIGAR is the diagonal's runs
// of = and X between the soft clips.  Returns whether the box is such a box, with the op
// count and the mismatches (X count).
__device__ bool diagonal_box(const CigarArgs &g, const Box &bx, int S, int *nops, int *mism) {
  if (bx.ref_len != bx.rows) return false;
  CodeStream as, bs;
  as.init(bx.A, bx.rows);
  bs.init(bx.B, bx.rows);
  int sum = 0, runs = 0, mis = 0, lk = -1;
  for (int t = 0; t < bx.rows; t++) {
    const int a = (int)as.next(), b = (int)bs.next();
    sum += sub_score(g, a, b);
    const int kind = a == b ? 0 : 1;
    runs += kind != lk;
    lk = kind;
    mis += kind;
  }
  if (sum != S) return false;
  *nops = runs + (bx.tail > 0) + (bx.bb > 0);
  *mism = mis;
  return true;
}

// Writes a diagonal box's ops to out[0 .. nops), front to back.
__device__ void emit_diagonal(const Box &bx, uint32_t *out) {
  int t = 0;
  if (bx.bb > 0) out[t++] = ((uint32_t)bx.bb << 4) | kOpS;
  CodeStream as, bs;
  as.init(bx.A, bx.rows);
  bs.init(bx.B, bx.rows);
  uint32_t rk = 0;
  int rl = 0;
  for (int u = 0; u < bx.rows; u++) {
    const uint32_t op = as.next() == bs.next() ? kOpEq : kOpX;
    if (op == rk) {
      ++rl;
    } else {
      if (rl > 0) out[t++] = ((uint32_t)rl << 4) | rk;
      rk = op;
      rl = 1;
    }
  }
  out[t++] = ((uint32_t)rl << 4) | rk;
  if (bx.tail > 0) out[t++] = ((uint32_t)bx.tail << 4) | kOpS;
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

// Per pair: a diagonal box (segment 0, its op count and mismatches found here), the
// register kernel its first band fits (segment 1 + class), or the generic list.  The sort
// key is the segment, then box rows descending, so a warp's lanes take boxes of about the
// same height, longest first.  order (may be null): the batched forward pass's pair order.
__global__ void k_cigar_classify(CigarArgs g, int64_t n, const uint32_t *__restrict__ order) {
  const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= n) return;
  const int64_t p = order ? (int64_t)order[idx] : idx;
  int nops = 0, mism = 0;
  uint32_t key = kKeyNone;
  const int S = g.score[p], ab = g.a_beg[p], ae = g.a_end[p], bb = g.b_beg[p], be = g.b_end[p];
  if (S > 0 && ab >= 0 && bb >= 0 && ae - ab <= 32767 && be - bb <= 32767) {
    const Box bx = make_box(g, (int)p);
    const int w = abs(bx.ref_len - bx.rows) + 1;
    // the register kernels' lazy F needs gap open >= gap extend, their score table int8
    const bool reg_ok = g.gO >= g.gE && g.match <= 127 && g.mismatch <= 128 && g.amb <= 128;
    const int c = reg_ok ? list_for(w, bx.rows) : kCigarClasses;
    if (c == kCigarClasses) {
      list_push(g, c, (int)p, w, bx.rows, bx.ref_len);
    } else {
      const int seg = (c == 0 && diagonal_box(g, bx, S, &nops, &mism)) ? 0 : 1 + c;
      key = ((uint32_t)seg << 10) | (uint32_t)(1023 - bx.rows);
      const unsigned act = __activemask();  // the lanes on this path only
      const unsigned peers = __match_any_sync(act, seg);
      const int leader = __ffs(peers) - 1;
      if ((int)(threadIdx.x & 31) == leader) atomicAdd(&g.counts[seg], __popc(peers));
    }
  }
  g.nops[p] = nops;
  g.mism[p] = mism;
  g.op_off[p] = 0;
  g.keys[idx] = key;
  g.idx[idx] = (uint32_t)p;
}

// Diagonal boxes (segment 0): reserve and write their ops.
__global__ void __launch_bounds__(128) k_cigar_diag(CigarArgs g) {
  const int64_t T = (int64_t)gridDim.x * blockDim.x;
  const int64_t tid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int count = g.counts[0];
  for (int64_t base = tid - (threadIdx.x & 31); base < count; base += T) {
    const int64_t e = base + (threadIdx.x & 31);
    const bool valid = e < count;
    int p = 0, nops = 0;
    Box bx{};
    if (valid) {
      p = (int)g.sorted[e];
      bx = make_box(g, p);
      nops = g.nops[p];
    }
    const int64_t at = reserve_arena(g, nops, true);
    if (!valid) continue;
    if (at + nops > g.arena_cap) {  // arena full: the host grows it and runs the pass again
      g.nops[p] = -1;
      atomicAdd(&g.counts[kCigarArenaFull], 1);
      continue;
    }
    emit_diagonal(bx, g.arena + at);
    g.op_off[p] = at;
  }
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

// Direction rows of the register kernels: four bit-planes of PB bits (PB = the band's
// cells rounded up to 8, 16, 32 or 64), bit (plane * PB + k) of the row's words: E opened
// (not extended), F opened, and a 2-bit H source in planes 2-3 -- 1 = E, 2 = F, 0 = the
// diagonal with different bases, 3 = the diagonal with equal codes (the =/X of an M step
// read straight from the directions).
template <int W>
struct Planes {
  static constexpr int K = 2 * W + 1;
  static constexpr int PB = K <= 8 ? 8 : K <= 16 ? 16 : K <= 32 ? 32 : 64;
  static constexpr int NW = 4 * PB / 32;  // words per row
};

template <int W>
struct RowRing {
  static constexpr int PB = Planes<W>::PB, NW = Planes<W>::NW;
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
  __device__ __forceinline__ uint32_t bit(int plane, int k) const {
    const int b = plane * PB + k;
    uint32_t w = r[0][0];
#pragma unroll
    for (int q = 1; q < NW; q++)
      if ((b >> 5) == q) w = r[0][q];
    return (w >> (b & 31)) & 1u;
  }
  // the cell's directions as one nibble: E open | F open << 1 | H source << 2
  __device__ __forceinline__ uint32_t nib(int k) const {
    return bit(0, k) | (bit(1, k) << 1) | (bit(2, k) << 2) | (bit(3, k) << 3);
  }
};

// Step kinds of the record: = (0), I (1), D (2), X (3); an M step's =/X comes from the
// direction it was taken from.
enum : uint32_t { kKindEq = 0, kKindI = 1, kKindD = 2, kKindX = 3 };

// The direction walk.  Records each step's kind, counts the runs of equal kinds and the
// mismatches (X, I and D steps) on the way; returns false when it leaves the band the
// final pass computed (or outgrows the record).
template <int W>
__device__ bool walk_record(RowRing<W> &ring, const Box &bx, int w, uint32_t *path, int *nsteps, int *j_end,
                            int *runs, int *last_kind, int *mism) {
  int i = bx.rows - 1, j = bx.ref_len - 1, st = 2, n = 0, nr = 0, lk = -1, mis = 0;
  uint32_t cur = 0;
  ring.init(i);
  while (i > 0) {
    if (j < 0 || n >= kPathWords * 16) return false;
    const int k = j - i + w;
    if (k < 0 || k > 2 * w) return false;
    const uint32_t nb = ring.nib(k);
    const uint32_t hs = nb >> 2;
    // effective state at this cell: 0 = E (an I step), 1 = F (a D step), 2 = diagonal (M)
    const int eff = st != 2 ? st : (hs == 1u ? 0 : hs == 2u ? 1 : 2);
    const uint32_t kind = eff == 0 ? kKindI : eff == 1 ? kKindD : (hs == 3u ? kKindEq : kKindX);
    st = eff == 0 ? ((nb & 1u) ? 2 : 0) : eff == 1 ? ((nb & 2u) ? 2 : 1) : 2;
    i -= eff != 1;
    j -= eff != 0;
    nr += (int)kind != lk;
    lk = (int)kind;
    mis += kind != kKindEq;
    cur |= kind << ((n & 15) * 2);
    if ((n & 15) == 15) {
      path[n >> 4] = cur;
      cur = 0;
    }
    ++n;
    if (eff != 1) ring.down(i);
  }
  if (n & 15) path[n >> 4] = cur;
  *nsteps = n;
  *j_end = j;
  *runs = nr;
  *last_kind = lk;
  *mism = mis;
  return true;
}

// Writes the ops of a walk that ended in column 0 to out[0 .. nops) back to front: the
// runs of the record, then the stopping cell's M (=/X given), between the soft clips.
__device__ void emit_kinds(const Box &bx, const uint32_t *path, int nsteps, uint32_t last_cell_kind, uint32_t *out,
                           int nops) {
  int t = 0;
  auto emit = [&](uint32_t kind, int len) {
    out[nops - 1 - t] = ((uint32_t)len << 4) | kind;
    ++t;
  };
  static constexpr uint32_t kOpOf = (kOpEq << 0) | (kOpI << 8) | (kOpD << 16) | (kOpX << 24);
  if (bx.tail > 0) emit(kOpS, bx.tail);
  uint32_t rk = 4;
  int rl = 0;
  for (int s = 0; s < nsteps; s++) {
    const uint32_t kind = (path[s >> 4] >> ((s & 15) * 2)) & 3u;
    if (kind == rk) {
      ++rl;
    } else {
      if (rl > 0) emit((kOpOf >> (8 * rk)) & 0xffu, rl);
      rk = kind;
      rl = 1;
    }
  }
  if (last_cell_kind == rk) {
    ++rl;
  } else {
    if (rl > 0) emit((kOpOf >> (8 * rk)) & 0xffu, rl);
    rk = last_cell_kind;
    rl = 1;
  }
  emit((kOpOf >> (8 * rk)) & 0xffu, rl);
  if (bx.bb > 0) emit(kOpS, bx.bb);
}

// Replays the record of a walk that stopped short of column 0 (its M steps' =/X then
// compares bases shifted by the stopping column, as SSW's CalculateNumberMismatch walks
// the CIGAR from the box's start).  mode 1: counts ops (*res) and mismatches (*mm),
// comparing the bases of the M steps with loads issued 8 steps at a time, and keeps each
// M step's =/X outcome in xf (1 bit a step); mode 2: writes the ops to out[0 .. nops)
// back to front from the record and xf alone.
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
        uint32_t op = st < nsteps ? (path[st >> 4] >> ((st & 15) * 2)) & 3u : kOpD;
        if (op == kKindX) op = kOpM;
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
      uint32_t op = (path[st >> 4] >> ((st & 15) * 2)) & 3u;
      if (op == kKindX) op = kOpM;
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

template <int W>
__device__ void traceback_reg(const CigarArgs &g, const uint32_t *dcol, int64_t stride, const Box &bx, int w, int p,
                              bool valid) {
  uint32_t path[kPathWords], xf[kPathWords / 2];
  int nsteps = 0, j_end = 0, nops = 0, mm = 0, runs = 0, last = -1;
  uint32_t last_cell = 0;
  bool ok = valid;
  if (ok) {
    RowRing<W> ring;
    ring.base = dcol;
    ring.stride = stride;
    ok = walk_record(ring, bx, w, path, &nsteps, &j_end, &runs, &last, &mm);
    if (!ok) {
      g.nops[p] = -1;
      atomicAdd(&g.counts[kCigarWalkErrors], 1);
    } else if (j_end == 0) {
      last_cell = bx.A[0] != bx.B[0] ? kKindX : kKindEq;  // the stopping cell (0, 0)
      mm += last_cell == kKindX;
      nops = runs + ((int)last_cell != last) + (bx.tail > 0) + (bx.bb > 0);
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
  if (j_end == 0) {
    emit_kinds(bx, path, nsteps, last_cell, g.arena + base, nops);
  } else {
    int t2 = 0, mm2 = 0;
    replay_path(bx, path, xf, nsteps, j_end, 2, &t2, &mm2, g.arena + base, nops);
  }
  g.op_off[p] = base;
  g.nops[p] = nops;
  g.mism[p] = mm;
}

// One banded DP pass at half-width w <= W; returns the band's maximum.
//
// F runs from H before F's own contribution ("lazy F"): with gap open >= gap extend,
// max(H(k-1) - gO, F(k-1) - gE) equals max(H'(k-1) - gO, F(k-1) - gE) for H' = max(E, 0,
// diagonal), and so do their open/extend choices -- when F made H(k-1), H(k-1) - gO =
// F(k-1) - gO <= F(k-1) - gE -- so the serial chain along a row is one add-max per cell.
// The classifier sends other scorings to the generic kernel.  Substitution scores come
// from one byte permute per 4 cells: the window's nibble codes select bytes of a per-row
// table of the 5 scores of the row's B base.
template <int W>
__device__ int band_pass(const CigarArgs &g, const Box &bx, int w, uint32_t *dcol, int64_t stride) {
  constexpr int K = 2 * W + 1;
  constexpr int PB = Planes<W>::PB, NW = Planes<W>::NW;
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
  const uint32_t mis8 = ((uint32_t)(-g.mismatch) & 0xffu) * 0x01010101u;
  const uint32_t amb8 = ((uint32_t)(-g.amb) & 0xffu) * 0x01010101u;
  const uint32_t mat1 = (uint32_t)g.match & 0xffu;
  const int gO = g.gO, gE = g.gE;
  CodeStream bs, as;  // B codes of the rows; the A code entering the window after each row
  bs.init(bx.B, bx.rows);
  as.init(bx.A + (K - w), bx.ref_len - (K - w));
  int mx = 0;
  for (int i = 0; i < bx.rows; i++) {
    const uint32_t qb = bs.next();
    // nibble k of ne[k >> 3] is nonzero where the window's code differs from qb
    uint32_t ne[NC];
#pragma unroll
    for (int q = 0; q < NC; q++) {
      const uint32_t x = win[q] ^ (qb * 0x11111111u);
      ne[q] = (x | (x >> 1) | (x >> 2) | (x >> 3)) & 0x11111111u;
    }
    // bytes 0..4 = score of codes 0..4 against qb
    const uint32_t t_lo = qb < 4 ? (mis8 & ~(0xffu << (8 * qb))) | (mat1 << (8 * qb)) : amb8;
    const int kstart = max(0, w - i), kend = min(2 * w, bx.ref_len - 1 - i + w);
    const bool clob = i >= 1 && i <= w + 1 && bx.ref_len <= i + w;
    int f = 0, hpl = 0;  // F and H' of the previous cell (0 before the band's first cell)
    uint32_t pl[NW];
#pragma unroll
    for (int q = 0; q < NW; q++) pl[q] = 0;
    uint32_t sc4 = 0;
#pragma unroll
    for (int k = 0; k < K; k++) {
      if ((k & 3) == 0) sc4 = __byte_perm(t_lo, amb8, win[k >> 3] >> (16 * ((k >> 2) & 1)));
      if (k >= kstart && k <= kend) {
        int hu = H[k + 1], eu = E[k + 1];
        if (clob && k == kend) hu = eu = 0;
        const int a = hu - gO, b = eu - gE;
        const int e = max(a, b);
        if (a > b) pl[(0 * PB + k) >> 5] |= 1u << ((0 * PB + k) & 31);
        const int fo = hpl - gO, fe = f - gE;
        f = max(fo, fe);
        if (fo > fe) pl[(1 * PB + k) >> 5] |= 1u << ((1 * PB + k) & 31);
        const int sv = (int)(signed char)(sc4 >> (8 * (k & 3)));
        const int dg = H[k] + sv;
        const int hp = __vimax_s32_relu(e, dg);  // H' = max(E, 0, diagonal)
        const int h = __vimax_s32_relu(hp, f);
        const int m1 = __vimax_s32_relu(e, f);
        if (m1 > dg) {
          if (e > max(f, 0)) {
            pl[(2 * PB + k) >> 5] |= 1u << ((2 * PB + k) & 31);
          } else {
            pl[(3 * PB + k) >> 5] |= 1u << ((3 * PB + k) & 31);
          }
        } else if (!((ne[k >> 3] >> ((k & 7) * 4)) & 1u)) {  // diagonal, equal codes
          pl[(2 * PB + k) >> 5] |= 1u << ((2 * PB + k) & 31);
          pl[(3 * PB + k) >> 5] |= 1u << ((3 * PB + k) & 31);
        }
        H[k] = h;
        E[k] = e;
        hpl = hp;
        mx = max(mx, h);
      }
    }
#pragma unroll
    for (int q = 0; q < NW; q++) __stcg(dcol + ((int64_t)i * NW + q) * stride, pl[q]);
    // slide the window one code: new k = old k + 1; the last slot takes A[i + 1 - w + K - 1]
#pragma unroll
    for (int q = 0; q < NC; q++) win[q] = (win[q] >> 4) | (q + 1 < NC ? (win[q + 1] << 28) : 0u);
    win[(K - 1) >> 3] |= as.next() << (((K - 1) & 7) * 4);
  }
  return mx;
}

template <int C>
__global__ void __launch_bounds__(128) k_cigar_band(CigarArgs g) {
  constexpr int W = cigar_half(C);
  const int64_t T = (int64_t)gridDim.x * blockDim.x;
  const int64_t tid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  // this kernel's segment of the sorted pairs, then its escalation list
  int seg0 = 0;
#pragma unroll
  for (int c = 0; c <= C; c++) seg0 += g.counts[c];
  const int seg_n = g.counts[1 + C];
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
    traceback_reg<W>(g, dcol, T, bx, w, p, valid);
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
  constexpr int NW = Planes<cigar_half(C)>::NW;
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
  k_cigar_diag<<<sms * 8, 128, 0, st>>>(g);
  if ((e = cudaGetLastError())) return e;
  if ((e = launch_band<0>(g, sms, cb.dirs_bytes, st))) return e;
  if ((e = launch_band<1>(g, sms, cb.dirs_bytes, st))) return e;
  if ((e = launch_band<2>(g, sms, cb.dirs_bytes, st))) return e;
  if ((e = launch_band<3>(g, sms, cb.dirs_bytes, st))) return e;
  if ((e = launch_band<4>(g, sms, cb.dirs_bytes, st))) return e;
  if ((e = launch_band<5>(g, sms, cb.dirs_bytes, st))) return e;
  if (launches) *launches += 3 + kCigarClasses + 4;  // + the radix sort's passes (approximate)
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
