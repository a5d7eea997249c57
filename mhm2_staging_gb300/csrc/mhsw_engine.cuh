// mhsw_engine.cuh -- anti-diagonal wavefront Smith-Waterman engine for sm_103a.
//
// Computes, for one pair, the local affine-gap alignment score and the
// lexicographically first cell (smallest A row, then smallest B column) that holds
// it -- the forward-pass result of StripedSmithWaterman's sw_sse2_byte/word
// (reference src/ssw/ssw_core.cpp:296-506), with A = SSW "ref" and B = SSW "query".
// The reverse (begin) pass runs the same engine on reversed prefixes
// (ssw_core.cpp:1166-1178), or the banded kernel in mhsw_kernels.cu.
//
// Layout ("lanes along A, sweep B"):
//   * a group of G lanes owns one pair; lane L holds A rows [L*2K, L*2K+2K) of the
//     current row strip (2K*G rows per strip; longer A uses several strips);
//   * each lane register packs two cells as int16x2 (V16) or two int32 (V32):
//     the low half is row L*2K+k at column j, the high half row L*2K+K+k at column
//     j-1 (one step behind), so the two halves never depend on each other in a step
//     and the DPX packed-int16 max/add instructions update both at once;
//   * lane L runs two steps behind lane L-1 (column j = t - 2L); lane L-1 hands its
//     last row's H and vertical-gap value to lane L through one __shfl_up_sync;
//   * the substitution score comes from a per-lane table T[c][k] in shared memory
//     (c = B code incl. N and PAD), one vector load per step; the two halves of a
//     packed score are merged with one byte-permute.
//
// DP (int, exact): H = max(0, Hdiag + s, E, F); E (gap along A, flows down the rows of
// a column) and F (gap along B, carried per row across steps) use
// X' = max(X - gE, H - gO).  Gap values are kept within [true, max(true,0)], which
// leaves every H unchanged.  Positions outside the matrix use code PAD (score -BIG),
// so every step is branch-free; their values stay below the pair's maximum and never
// win the arg-max.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "mhsw_types.h"

namespace mhsw {

// ASCII -> code table: the reference's base translation (src/ssw/ssw.cpp:13-26) restated: A/a/U/u -> 0,
// C/c -> 1, G/g -> 2, T/t -> 3, every other byte -> 4.
#define MHSW_R16(x) x, x, x, x, x, x, x, x, x, x, x, x, x, x, x, x
static __constant__ uint8_t c_code[256] = {
    MHSW_R16(4), MHSW_R16(4), MHSW_R16(4), MHSW_R16(4),
    // 64..79: @ A B C D E F G H I J K L M N O
    4, 0, 4, 1, 4, 4, 4, 2, 4, 4, 4, 4, 4, 4, 4, 4,
    // 80..95: P Q R S T U V W X Y Z [ \ ] ^ _
    4, 4, 4, 4, 3, 0, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4,
    // 96..111: ` a b c d e f g h i j k l m n o
    4, 0, 4, 1, 4, 4, 4, 2, 4, 4, 4, 4, 4, 4, 4, 4,
    // 112..127: p q r s t u v w x y z { | } ~ DEL
    4, 4, 4, 4, 3, 0, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4,
    MHSW_R16(4), MHSW_R16(4), MHSW_R16(4), MHSW_R16(4), MHSW_R16(4), MHSW_R16(4), MHSW_R16(4), MHSW_R16(4)};
#undef MHSW_R16
// (bytes >= 128, which the reference indexes with a negative char, map to 4 here.)

__host__ __device__ inline int sub_score(int a, int b, const Scoring &s, int big) {
  if (a == kCodePad || b == kCodePad) return -big;
  if (b == kCodeZeroPad) return 0;
  if (a == kCodeN || b == kCodeN) return -s.ambiguity;
  return a == b ? s.match : -s.mismatch;
}

// ---------------------------------------------------------------------------------
// Packed value types.
// ---------------------------------------------------------------------------------
struct V16 {
  using T = uint32_t;
  using Pay = uint32_t;                  // what a lane hands to the next lane per step
  static constexpr int kBig = 16384;     // PAD penalty; valid while every H <= kBig-1
  static constexpr int kWordsPerT = 1;
  __device__ static __forceinline__ T pack(int lo, int hi) {
    return (uint32_t)(uint16_t)(int16_t)lo | ((uint32_t)(uint16_t)(int16_t)hi << 16);
  }
  __device__ static __forceinline__ T splat(int v) { return pack(v, v); }
  __device__ static __forceinline__ int lo(T x) { return (int)(int16_t)(x & 0xffffu); }
  __device__ static __forceinline__ int hi(T x) { return (int)(int16_t)(x >> 16); }
  __device__ static __forceinline__ T max_relu(T a, T b) { return __vimax_s16x2_relu(a, b); }
  __device__ static __forceinline__ T addmax_relu(T a, T b, T c) { return __viaddmax_s16x2_relu(a, b, c); }
  __device__ static __forceinline__ T addmax(T a, T b, T c) { return __viaddmax_s16x2(a, b, c); }
  __device__ static __forceinline__ T add(T a, T b) { return __viaddmax_s16x2(a, b, 0x80008000u); }
  // low half from cur, high half from prev
  __device__ static __forceinline__ T mix(T cur, T prev) { return __byte_perm(cur, prev, 0x7610); }
  // (lo: h.hi, hi: e.hi)
  __device__ static __forceinline__ Pay payload(T h, T e) { return __byte_perm(h, e, 0x7632); }
  __device__ static __forceinline__ Pay pay_make(int h, int e) { return pack(h, e); }
  // E entering the first row of each half: lo from the left lane, hi from own lo half.
  __device__ static __forceinline__ T etop(Pay z, T own_e) { return __byte_perm(z, own_e, 0x5432); }
  __device__ static __forceinline__ T htop(Pay z, T own_h) { return __byte_perm(z, own_h, 0x5410); }
  template <int W>
  __device__ static __forceinline__ Pay shfl_up(unsigned mask, Pay p) {
    return __shfl_up_sync(mask, p, 1, W);
  }
};

struct V32 {
  struct T {
    int lo, hi;
  };
  struct Pay {
    int h, e;
  };
  static constexpr int kBig = 1 << 28;
  static constexpr int kWordsPerT = 2;
  __device__ static __forceinline__ T pack(int lo, int hi) { return T{lo, hi}; }
  __device__ static __forceinline__ T splat(int v) { return T{v, v}; }
  __device__ static __forceinline__ int lo(T x) { return x.lo; }
  __device__ static __forceinline__ int hi(T x) { return x.hi; }
  __device__ static __forceinline__ T max_relu(T a, T b) {
    return T{__vimax_s32_relu(a.lo, b.lo), __vimax_s32_relu(a.hi, b.hi)};
  }
  __device__ static __forceinline__ T addmax_relu(T a, T b, T c) {
    return T{__viaddmax_s32_relu(a.lo, b.lo, c.lo), __viaddmax_s32_relu(a.hi, b.hi, c.hi)};
  }
  __device__ static __forceinline__ T addmax(T a, T b, T c) {
    return T{__viaddmax_s32(a.lo, b.lo, c.lo), __viaddmax_s32(a.hi, b.hi, c.hi)};
  }
  __device__ static __forceinline__ T add(T a, T b) { return T{a.lo + b.lo, a.hi + b.hi}; }
  __device__ static __forceinline__ T mix(T cur, T prev) { return T{cur.lo, prev.hi}; }
  __device__ static __forceinline__ Pay payload(T h, T e) { return Pay{h.hi, e.hi}; }
  __device__ static __forceinline__ Pay pay_make(int h, int e) { return Pay{h, e}; }
  __device__ static __forceinline__ T etop(Pay z, T own_e) { return T{z.e, own_e.lo}; }
  __device__ static __forceinline__ T htop(Pay z, T own_h) { return T{z.h, own_h.lo}; }
  template <int W>
  __device__ static __forceinline__ Pay shfl_up(unsigned mask, Pay p) {
    return Pay{__shfl_up_sync(mask, p.h, 1, W), __shfl_up_sync(mask, p.e, 1, W)};
  }
};

// ---------------------------------------------------------------------------------
// Shared-memory profile table.  Per lane and code c it holds K packed words
// T[c][k] = (lo: s(A[row0+k], c), hi: s(A[row0+K+k], c)), stored as vectors of VW
// 32-bit words in [c][q][lane] order so a warp's vector loads are bank-conflict free.
// ---------------------------------------------------------------------------------
template <class VT, int K>
struct ProfileLayout {
  static constexpr int kWords = K * VT::kWordsPerT;                 // words per (lane, code)
#ifndef MHSW_PROFILE_VW_MAX
#define MHSW_PROFILE_VW_MAX 4
#endif
  static constexpr int kVW = (kWords % 4 == 0 && MHSW_PROFILE_VW_MAX >= 4) ? 4
                             : ((kWords % 2 == 0 && MHSW_PROFILE_VW_MAX >= 2) ? 2 : 1);
  static constexpr int kNQ = kWords / kVW;                          // vectors per (lane, code)
  // bytes for `lanes` lanes
  __host__ __device__ static constexpr size_t bytes(int lanes) {
    return (size_t)kNumCodes * kNQ * lanes * kVW * 4;
  }
};

template <int VW>
struct VecW;
template <>
struct VecW<4> {
  using type = uint4;
};
template <>
struct VecW<2> {
  using type = uint2;
};
template <>
struct VecW<1> {
  using type = uint32_t;
};

template <class VT, int K>
__host__ __device__ __forceinline__ void load_profile(const uint32_t *__restrict__ tab, int lanes, int lane_in_block, int c,
                                             typename VT::T (&P)[K]) {
  using L = ProfileLayout<VT, K>;
  using Vec = typename VecW<L::kVW>::type;
  uint32_t w[L::kWords];
#pragma unroll
  for (int q = 0; q < L::kNQ; q++) {
    const Vec *src = reinterpret_cast<const Vec *>(tab) + ((size_t)(c * L::kNQ + q) * lanes + lane_in_block);
    Vec v = *src;
    const uint32_t *vv = reinterpret_cast<const uint32_t *>(&v);
#pragma unroll
    for (int x = 0; x < L::kVW; x++) w[q * L::kVW + x] = vv[x];
  }
#pragma unroll
  for (int k = 0; k < K; k++) {
    if constexpr (VT::kWordsPerT == 1) {
      P[k] = *reinterpret_cast<typename VT::T *>(&w[k]);
    } else {
      P[k] = typename VT::T{(int)w[2 * k], (int)w[2 * k + 1]};
    }
  }
}

template <class VT, int K>
__host__ __device__ __forceinline__ void store_profile_entry(uint32_t *tab, int lanes, int lane_in_block, int c, int k, int lo,
                                                    int hi) {
  using L = ProfileLayout<VT, K>;
  int word, nw;
  uint32_t vals[2];
  if constexpr (VT::kWordsPerT == 1) {
    word = k;
    nw = 1;
    vals[0] = (uint32_t)(uint16_t)(int16_t)lo | ((uint32_t)(uint16_t)(int16_t)hi << 16);
  } else {
    word = 2 * k;
    nw = 2;
    vals[0] = (uint32_t)lo;
    vals[1] = (uint32_t)hi;
  }
  for (int x = 0; x < nw; x++) {
    int wi = word + x;
    int q = wi / L::kVW, r = wi % L::kVW;
    tab[((size_t)(c * L::kNQ + q) * lanes + lane_in_block) * L::kVW + r] = vals[x];
  }
}

// Packs (value, row, col) into a key whose unsigned max is the lexicographic best:
// larger value, then smaller row, then smaller column.  Key 0 = nothing positive.
__host__ __device__ __forceinline__ unsigned long long best_key(int v, int row, int col) {
  if (v <= 0) return 0ull;
  return ((unsigned long long)(unsigned)v << 40) | ((unsigned long long)(0xFFFFFu - (unsigned)row) << 20) |
         (unsigned long long)(0xFFFFFu - (unsigned)col);
}
__host__ __device__ __forceinline__ int key_value(unsigned long long k) { return (int)(k >> 40); }
__host__ __device__ __forceinline__ int key_row(unsigned long long k) { return (int)(0xFFFFFu - (unsigned)((k >> 20) & 0xFFFFFu)); }
__host__ __device__ __forceinline__ int key_col(unsigned long long k) { return (int)(0xFFFFFu - (unsigned)(k & 0xFFFFFu)); }

// Sequence view over base codes with a direction: seq[i] = base[dir * i].
struct SeqView {
  const uint8_t *base;
  int dir;  // +1 forward, -1 reversed prefix
  int len;
  __device__ __forceinline__ int code(int i) const {
    return (i >= 0 && i < len) ? (int)base[(ptrdiff_t)dir * i] : kCodePad;
  }
};

// Per-group shared state handed to the engine.
struct GroupSmem {
  uint32_t *prof;   // this group's profile table ([c][q][lane] vectors, lane in group)
  int prof_lanes;   // lanes in the group (table stride)
  uint8_t *bcodes;  // this group's B code buffer: bcodes[pad + j]
  int pad;          // leading PAD entries (>= 2G)
  int bcap;         // capacity of bcodes in bytes
};

// Shared memory of one group: its profile table (sized for the largest K the kernel
// may run, so groups of a block can run different K) followed by the B code buffer.
template <class VT, int KMAX, int G>
__host__ __device__ constexpr size_t group_prof_bytes() {
  return (ProfileLayout<VT, KMAX>::bytes(G) + 15) / 16 * 16;
}

// Result of one forward sweep.
struct SweepOut {
  unsigned long long key;  // best_key of the lexicographic best cell
  int overflow;            // 1 if the int16 ceiling was crossed
};

// ---------------------------------------------------------------------------------
// One pair through the wavefront.  All G lanes of the group call this together.
//   lane       : 0..G-1 within the group
//   gmask      : the group's lanes within the warp (for shuffles / syncwarp)
//   bnd        : global scratch of >= N payloads for multi-strip A (may be null if
//                A fits one strip)
//   ceiling    : int16 overflow ceiling (values above it flag overflow)
// ---------------------------------------------------------------------------------
// Score2 mode of the generic engine: the sweep covers P16 columns ([N, P16) score 0, SSW's
// byte-path query padding) and keeps two maxima per A row, over columns [0, P16) and over
// [0, P8) (the word path pads to a multiple of 8); both are written, and the second-best
// score reads the one of the path SSW took.
struct RowMaxOut2 {
  int32_t *rowmax16, *rowmax8;
  int P16, P8;
};

template <class VT, int K, int G, bool S2 = false>
__device__ void sweep_pair(const SeqView &A, const SeqView &B, const Scoring &sc, const GroupSmem &gs, int lane,
                           unsigned gmask, typename VT::Pay *bnd, int ceiling, SweepOut &out,
                           const RowMaxOut2 &rm2 = RowMaxOut2{nullptr, nullptr, 0, 0}) {
  const int lane_in_block = lane;  // table column: lane within the group
  using T = typename VT::T;
  using Pay = typename VT::Pay;
  constexpr int RS = 2 * K * G;  // rows per strip
  const int M = A.len, N = B.len;
  const T NGO = VT::splat(-sc.gap_open);
  const T NGE = VT::splat(-sc.gap_extend);

  const int NP = S2 ? rm2.P16 : N;  // columns swept
  // B codes into shared memory: bcodes[pad + j] for j in [-pad, NP + 2G); PAD outside
  // [0, N) except the zero-score columns [N, NP) of score2 mode.
  const int fill = gs.pad + NP + 2 * G < gs.bcap ? gs.pad + NP + 2 * G : gs.bcap;
  for (int x = lane; x < fill; x += G) {
    int j = x - gs.pad;
    gs.bcodes[x] = (uint8_t)((S2 && j >= N && j < NP) ? kCodeZeroPad : B.code(j));
  }
  __syncwarp(gmask);

  unsigned long long best = 0ull;
  int overflow = 0;
  const int nstrips = (M + RS - 1) / RS;
  const int T_end = NP + 2 * G - 1;  // steps per strip

  for (int s = 0; s < nstrips; s++) {
    const int row0 = s * RS + lane * 2 * K;
    // Profile table for this lane's rows.
    __syncwarp(gmask);
    for (int c = 0; c < kNumCodes; c++) {
#pragma unroll
      for (int k = 0; k < K; k++) {
        int alo = A.code(row0 + k), ahi = A.code(row0 + K + k);
        store_profile_entry<VT, K>(gs.prof, gs.prof_lanes, lane_in_block, c, k, sub_score(alo, c, sc, VT::kBig),
                                   sub_score(ahi, c, sc, VT::kBig));
      }
    }
    __syncwarp(gmask);

    T H[K], F[K], V[K], Pprev[K];
    int Jlo[K], Jhi[K];
    int R16lo[K], R16hi[K], R8lo[K], R8hi[K];  // score2 mode: row maxima over valid columns
#pragma unroll
    for (int k = 0; k < K; k++) {
      H[k] = VT::splat(0);
      F[k] = NGO;
      V[k] = VT::splat(0);
      Jlo[k] = -1;
      Jhi[k] = -1;
      R16lo[k] = R16hi[k] = R8lo[k] = R8hi[k] = 0;
    }
    load_profile<VT, K>(gs.prof, gs.prof_lanes, lane_in_block, kCodePad, Pprev);
    T Hlast = VT::splat(0);
    T Ecout = NGO;
    T HtopPrev = VT::splat(0);
    Pay Zout = VT::pay_make(0, -sc.gap_open);
    const Pay ztop0 = VT::pay_make(0, -sc.gap_open);
    const bool first_strip = (s == 0);
    const bool last_strip = (s == nstrips - 1);

    // four steps per loop iteration: the loop's own instructions and the register moves at
    // its back edge are paid once per four steps (3-4% on the int32 and non-keyed passes)
#pragma unroll 4
    for (int t = 0; t < T_end; t++) {
      const int j = t - 2 * lane;  // lo-half column
      const int c = gs.bcodes[gs.pad + j];
      T Pcur[K];
      load_profile<VT, K>(gs.prof, gs.prof_lanes, lane_in_block, c, Pcur);

      Pay z = VT::template shfl_up<G>(gmask, Zout);
      if (lane == 0) {
        // Top boundary: row -1 for the first strip, else the previous strip's last row.
        z = ztop0;
        if (!first_strip && j < NP) z = bnd[j];
      }
      T Ev = VT::etop(z, Ecout);
      T Htop = VT::htop(z, Hlast);
      T Hd = HtopPrev;
      HtopPrev = Htop;
      const bool ok16l = (unsigned)j < (unsigned)rm2.P16, ok16h = (unsigned)(j - 1) < (unsigned)rm2.P16;
      const bool ok8l = (unsigned)j < (unsigned)rm2.P8, ok8h = (unsigned)(j - 1) < (unsigned)rm2.P8;

#pragma unroll
      for (int k = 0; k < K; k++) {
        const T P = VT::mix(Pcur[k], Pprev[k]);
        const T t1 = VT::max_relu(Ev, F[k]);
        const T Hn = VT::addmax_relu(Hd, P, t1);
        const T Hg = VT::add(Hn, NGO);
        Ev = VT::addmax(Ev, NGE, Hg);
        F[k] = VT::addmax(F[k], NGE, Hg);
        Hd = H[k];
        H[k] = Hn;
        {
          // Strict increase of the row's running max records the step (first column).
          // (Written as plain compares: the __vibmax_s16x2 form miscompiled once 14 or
          // more copies were unrolled per step.)
          const int hl = VT::lo(Hn), hh = VT::hi(Hn), vl = VT::lo(V[k]), vh = VT::hi(V[k]);
          Jlo[k] = hl > vl ? t : Jlo[k];
          Jhi[k] = hh > vh ? t : Jhi[k];
          V[k] = VT::max_relu(V[k], Hn);
          if constexpr (S2) {
            R16lo[k] = ok16l && hl > R16lo[k] ? hl : R16lo[k];
            R16hi[k] = ok16h && hh > R16hi[k] ? hh : R16hi[k];
            R8lo[k] = ok8l && hl > R8lo[k] ? hl : R8lo[k];
            R8hi[k] = ok8h && hh > R8hi[k] ? hh : R8hi[k];
          }
        }
        Pprev[k] = Pcur[k];
      }
      Zout = VT::payload(H[K - 1], Ev);
      Hlast = H[K - 1];
      Ecout = Ev;
      if (!last_strip && lane == G - 1) {
        const int jh = t - 2 * lane - 1;  // hi-half column of the last lane
        if (jh >= 0 && jh < NP) bnd[jh] = Zout;
      }
    }

    if constexpr (S2) {
#pragma unroll
      for (int k = 0; k < K; k++) {
        const int rl = row0 + k, rh = row0 + K + k;
        if (rl < M) {
          rm2.rowmax16[rl] = R16lo[k];
          rm2.rowmax8[rl] = R8lo[k];
        }
        if (rh < M) {
          rm2.rowmax16[rh] = R16hi[k];
          rm2.rowmax8[rh] = R8hi[k];
        }
      }
    }

    // Lane-local best over its rows (ascending row order), then the group max.
    unsigned long long kbest = 0ull;
    int vmax_lane = 0;
#pragma unroll
    for (int k = 0; k < K; k++) {
      const int r = row0 + k;
      const int v = VT::lo(V[k]);
      if (r < M && Jlo[k] >= 0) {
        unsigned long long kk = best_key(v, r, Jlo[k] - 2 * lane);
        if (kk > kbest) kbest = kk;
      }
      if (r < M && v > vmax_lane) vmax_lane = v;
    }
#pragma unroll
    for (int k = 0; k < K; k++) {
      const int r = row0 + K + k;
      const int v = VT::hi(V[k]);
      if (r < M && Jhi[k] >= 0) {
        unsigned long long kk = best_key(v, r, Jhi[k] - 2 * lane - 1);
        if (kk > kbest) kbest = kk;
      }
      if (r < M && v > vmax_lane) vmax_lane = v;
    }
    if (vmax_lane > ceiling) overflow = 1;
#pragma unroll
    for (int o = G / 2; o > 0; o >>= 1) {
      unsigned long long other = __shfl_xor_sync(gmask, kbest, o, G);
      kbest = other > kbest ? other : kbest;
      overflow |= __shfl_xor_sync(gmask, overflow, o, G);
    }
    if (kbest > best) best = kbest;
    __syncwarp(gmask);
  }
  out.key = best;
  out.overflow = overflow;
}

}  // namespace mhsw
