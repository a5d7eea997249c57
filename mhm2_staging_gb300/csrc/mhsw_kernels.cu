// mhsw_kernels.cu -- forward, begin and output kernels of the alignment path (sm_103a).
//
// Forward  : k_fwd<V16|V32, K, G>  -- the wavefront engine of mhsw_engine.cuh, one
//            G-lane group per pair (the reference's one-block-per-pair
//            sequence_dna_kernel, src/adept-sw/kernel.cpp:160-333, replaced).
// Begin    : k_rev_banded          -- one thread per pair, banded DP on the reversed
//            prefixes A[0..a_end], B[0..b_end] (the reference's reverse pass,
//            src/ssw/ssw_core.cpp:1166-1178 and src/adept-sw/kernel.cpp:335-509).
//            Exact: every cell holding the score lies on an alignment from the end
//            cell whose total gap length g obeys
//            g*min(gO,gE) + max(gO-gE, 0) <= D*match - score with
//            D <= min(a_end+1, b_end+1) diagonal steps,
//            so the band |j - i| <= g contains it and banding only lowers other cells.
//            k_rev_wave runs the wavefront engine on the reversed box for the rare
//            pairs whose band is wider than the widest banded instantiation.
// Output   : k_finalize / k_pack5  -- orientation mapping into the caller's arrays.
#include <algorithm>
#include <cstdio>
#include <map>
#include <mutex>
#include <utility>

#include "mhsw_engine.cuh"
#include "mhsw_engine16.cuh"
#include "mhsw_launch.h"

namespace mhsw {


namespace {

constexpr int kG = 16;  // lanes per pair in every forward instantiation

__device__ __forceinline__ unsigned group_mask(int G) {
  if (G == 32) return 0xffffffffu;
  const int lane32 = threadIdx.x & 31;
  return ((1u << G) - 1u) << ((lane32 / G) * G);
}

template <class VT, int K, int G, bool S2 = false>
__global__ void __launch_bounds__(256) k_fwd(PairSet ps, ResultSet rs, Scoring sc, const int64_t *__restrict__ list,
                                             const int *__restrict__ list_count, int ceiling,
                                             typename VT::Pay *scratch, int scratch_stride, WorkLists wl, int pad,
                                             int bcap) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int lanes = blockDim.x;
  const int gpb = lanes / G;
  const int grp = threadIdx.x / G;
  const int lane = threadIdx.x % G;
  const unsigned gmask = group_mask(G);
  constexpr size_t kProf = group_prof_bytes<VT, K, G>();
  unsigned char *gbase = smem + (size_t)grp * (kProf + (size_t)bcap);
  GroupSmem gs;
  gs.prof = reinterpret_cast<uint32_t *>(gbase);
  gs.prof_lanes = G;
  gs.bcodes = gbase + kProf;
  gs.pad = pad;
  gs.bcap = bcap;
  constexpr int RS = 2 * K * G;
  constexpr bool kWide = (VT::kWordsPerT == 2);

  int64_t total = ps.n;
  if (list) {
    total = (int64_t)(*list_count);
    if (total > wl.cap) total = wl.cap;
  }
  const int64_t gid = (int64_t)blockIdx.x * gpb + grp;
  const int64_t gstride = (int64_t)gridDim.x * gpb;
  typename VT::Pay *bnd = scratch ? scratch + gid * (int64_t)scratch_stride : nullptr;

  for (int64_t i = gid; i < total; i += gstride) {
    const int64_t p = list ? list[i] : i;
    const int M = ps.a_len[p], N = ps.b_len[p];
    const int NP = S2 ? ssw_pad16(N) : N;  // columns swept (score2 mode adds SSW's padding)
    const bool too_long = (NP > bcap - pad - 2 * G) || (M > RS && (bnd == nullptr || NP > scratch_stride));
    if (M <= 0 || N <= 0 || too_long) {
      if (lane == 0) {
        rs.score[p] = 0;
        rs.a_end[p] = -1;
        rs.b_end[p] = 0;
        rs.flag[p] = too_long ? kFlagTooLong : 0u;
      }
      continue;
    }
    SeqView A{ps.a_code + ps.a_off[p], 1, M};
    SeqView B{ps.b_code + ps.b_off[p], 1, N};
    SweepOut so;
    RowMaxOut2 rm2{nullptr, nullptr, 0, 0};
    if constexpr (S2) rm2 = RowMaxOut2{ps.rowmax16 + ps.a_off[p], ps.rowmax8 + ps.a_off[p], NP, ssw_pad8(N)};
    sweep_pair<VT, K, G, S2>(A, B, sc, gs, lane, gmask, bnd, ceiling, so, rm2);
    if (lane == 0) {
      const int S = key_value(so.key);
      if (!kWide && so.overflow) {
        rs.flag[p] = kFlagOverflow16;
        const int slot = atomicAdd(wl.ovf_count, 1);
        if (slot < wl.cap) wl.ovf[slot] = p;
        rs.score[p] = S;
        rs.a_end[p] = -1;
        rs.b_end[p] = 0;
      } else {
        rs.flag[p] = 0u;
        rs.score[p] = S;
        rs.a_end[p] = S > 0 ? key_row(so.key) : -1;
        rs.b_end[p] = S > 0 ? key_col(so.key) : 0;
      }
    }
  }
}

// Plain forward pass with the keyed int16 engine (mhsw_engine16.cuh): one G-lane group
// per pair, grid-stride over [0, n).
template <int K, int G, bool S2 = false>
__global__ void __launch_bounds__(256) k_fwd16(PairSet ps, ResultSet rs, Scoring sc, int ceiling, V16::Pay *scratch,
                                               int scratch_stride, WorkLists wl, int pad, int bcap) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int gpb = blockDim.x / G;
  const int grp = threadIdx.x / G;
  const int lane = threadIdx.x % G;
  const unsigned gmask = group_mask(G);
  constexpr size_t kProf = group_prof16_bytes<K, G, S2 ? kCode16Zero + 1 : kCodeN + 1>();
  unsigned char *gbase = smem + (size_t)grp * kProf;  // keyed engine: profile table only
  GroupSmem gs;
  gs.prof = reinterpret_cast<uint32_t *>(gbase);
  gs.prof_lanes = G;
  gs.bcodes = nullptr;
  gs.pad = pad;
  gs.bcap = bcap;
  constexpr int RS = 2 * K * G;
  const int64_t gid = (int64_t)blockIdx.x * gpb + grp;
  const int64_t gstride = (int64_t)gridDim.x * gpb;
  V16::Pay *bnd = scratch ? scratch + gid * (int64_t)scratch_stride : nullptr;
  for (int64_t p = gid; p < ps.n; p += gstride) {
    const int M = ps.a_len[p], N = ps.b_len[p];
    const int NP = S2 ? ssw_pad16(N) : N;
    const bool too_long = (N > kMaxB) || (M > RS && (bnd == nullptr || NP > scratch_stride));
    if (M <= 0 || N <= 0 || too_long) {
      if (lane == 0) {
        rs.score[p] = 0;
        rs.a_end[p] = -1;
        rs.b_end[p] = 0;
        rs.flag[p] = too_long ? kFlagTooLong : 0u;
      }
      continue;
    }
    SeqView A{ps.a_code + ps.a_off[p], 1, M};
    SeqView B{ps.b_code + ps.b_off[p], 1, N};
    SweepOut so;
    RowMaxOut rmo{nullptr, 0};
    if constexpr (S2) rmo = RowMaxOut{ps.rowmax16 + ps.a_off[p], NP};
    sweep16<K, G, S2>(A, B, sc, gs, lane, gmask, bnd, ceiling, so, rmo);
    if (lane == 0) {
      const int S = key_value(so.key);
      // score2 mode: SSW's word path pads B to a multiple of 8; where that differs from
      // the byte-path padding swept here, the int32 pass recomputes the row maxima.
      const bool word_redo = S2 && S + ssw_bias(sc) >= 255 && ssw_pad8(N) != NP;
      if (so.overflow || word_redo) {
        rs.flag[p] = kFlagOverflow16;
        const int slot = atomicAdd(wl.ovf_count, 1);
        if (slot < wl.cap) wl.ovf[slot] = p;
        rs.score[p] = S;
        rs.a_end[p] = -1;
        rs.b_end[p] = 0;
      } else {
        rs.flag[p] = 0u;
        rs.score[p] = S;
        rs.a_end[p] = S > 0 ? key_row(so.key) : -1;
        rs.b_end[p] = S > 0 ? key_col(so.key) : 0;
      }
    }
  }
}

// Begin pass, banded.  Each pair's search is first assigned a band class: the
// narrowest instantiation whose width holds the alignment's largest drift to each side
// of the end cell's diagonal at the first row cap (band_sides: vertical gaps also cost
// rows, so that side's bound is the tighter one; the band sits asymmetrically around the
// diagonal) (k_rev_count / k_rev_scatter group the pairs into one segment per class), so
// every thread of a class kernel has a pair to work on.  One thread per pair: the band is
// WB-1 = 2G+1 cells wide and lives in registers, fully unrolled; the codes
// of a row's band are loaded before its dependency chain starts.  Rows whose band lies
// inside [0, N2) run without bound checks.  The row cap t starts at 2*score/match + 16
// and doubles until a row reaches the score, so short low-score alignments stay in a
// narrow band; a pair whose bound outgrows its class when t doubles goes to the
// wavefront list.
__host__ __device__ constexpr int band_half(int c) {  // half-widths 3, 5, 7, 11, 15, 23, 31
  return c == 0 ? 3 : c == 1 ? 5 : c == 2 ? 7 : c == 3 ? 11 : c == 4 ? 15 : c == 5 ? 23 : 31;
}

__host__ __device__ __forceinline__ int band_first_cap(int S, int mt, int M2) {
  const long long tt = 2ll * S / (mt > 0 ? mt : 1) + 16;
  return (int)(tt < M2 ? tt : M2);
}

// Total gap length g (inserted plus deleted cells) of an alignment that scores S with at
// most dmax diagonal steps.  Each diagonal step scores at most match, and g gap cells in
// r >= 1 runs cost r*gO + (g - r)*gE >= g*min(gO, gE) + max(gO - gE, 0), so
// g*min(gO, gE) + max(gO - gE, 0) <= dmax*match - S (g = 0 when that leaves no room for
// one gap cell).  (dmax <= 65000 and match <= 127 keep the product inside 32 bits.)
__host__ __device__ __forceinline__ int gap_cells_bound(int dmax, int S, const Scoring &sc) {
  const int gmin = sc.gap_open < sc.gap_extend ? sc.gap_open : sc.gap_extend;
  const int g1 = gmin > 0 ? gmin : 1;
  const int slack = dmax * sc.match - S - (sc.gap_open > sc.gap_extend ? sc.gap_open - sc.gap_extend : 0);
  return slack < g1 ? 0 : slack / g1;
}

// Total gap length any alignment reaching the score within the first t rows can have:
// its diagonal steps D <= min(t, N2).
__host__ __device__ __forceinline__ int band_gap_bound(int t, int N2, int S, const Scoring &sc) {
  return gap_cells_bound(t < N2 ? t : N2, S, sc);
}

// How far such an alignment can drift from the end cell's diagonal to either side.  I
// vertical gap cells (a row each, no column) leave at most t - I diagonal steps:
// S <= (t - I)*match - I*gmin - c, c = max(gO - gE, 0) once, so
// I <= (t*match - S - c) / (match + gmin); likewise J horizontal gap cells leave at most
// N2 - J, so J <= (N2*match - S - c) / (match + gmin).  Both are at most the total g.  A
// band over columns [row - L, row - L + W) holds every such alignment when I <= L and
// J <= W - 1 - L.
__host__ __device__ __forceinline__ void band_sides(int t, int N2, int S, const Scoring &sc, int &I, int &J) {
  const int g = band_gap_bound(t, N2, S, sc);
  const int gmin = sc.gap_open < sc.gap_extend ? sc.gap_open : sc.gap_extend;
  const int mg = sc.match + (gmin > 0 ? gmin : 1);
  const int c = sc.gap_open > sc.gap_extend ? sc.gap_open - sc.gap_extend : 0;
  const int st = t * sc.match - S - c, sn = N2 * sc.match - S - c;
  I = st < mg ? 0 : st / mg;
  J = sn < mg ? 0 : sn / mg;
  if (I > g) I = g;
  if (J > g) J = g;
}

// The narrowest band class whose width holds both sides at the first row cap
// (kBandClasses: none does).
__host__ __device__ __forceinline__ int band_fit(int S, int M2, int N2, const Scoring &sc) {
  int I, J;
  band_sides(band_first_cap(S, sc.match, M2), N2, S, sc, I, J);
  int c = kBandClasses;
#pragma unroll
  for (int k = kBandClasses - 1; k >= 0; k--)
    if (I + J <= 2 * band_half(k)) c = k;
  return c;
}

// The band's left extent for a pair of class half-width G: its vertical bound at the first
// row cap, with the room the class leaves beyond both bounds split between the sides.
__device__ __forceinline__ int band_left(int S, int M2, int N2, const Scoring &sc, int G) {
  int I, J;
  band_sides(band_first_cap(S, sc.match, M2), N2, S, sc, I, J);
  return I + (2 * G - I - J) / 2;
}

// True when an alignment reaching S within t rows may leave the band [row - L, row - L + 2G].
__device__ __forceinline__ bool band_outgrown(int t, int N2, int S, const Scoring &sc, int L, int G) {
  int I, J;
  band_sides(t, N2, S, sc, I, J);
  return I > L || J > 2 * G - L;
}

// Band class of pair p (0 .. kBandClasses-1), kBandClasses for the wavefront, or -1 when
// there is nothing to search (score 0, or a pair the forward pass rejected); those get
// their begin written here.
// s_cap: the largest score the band kernels take (the packed int16 kernels hold scores up
// to kBand16Score); pairs above it go to the wavefront list too.
__device__ __forceinline__ int band_class(const ResultSet &rs, const Scoring &sc, int64_t p, int s_cap) {
  const int S = rs.score[p];
  if ((rs.flag[p] & kFlagTooLong) || S <= 0) {
    rs.a_beg[p] = -1;
    rs.b_beg[p] = 0;
    return -1;
  }
  if (S > s_cap) return kBandClasses;
  return band_fit(S, rs.a_end[p] + 1, rs.b_end[p] + 1, sc);
}

// Warp-aggregated append of p to list[*count] (one atomic per distinct counter).
__device__ __forceinline__ void append_agg(int64_t *list, int *count, int64_t cap, int64_t p, bool want) {
  const unsigned act = __activemask();
  const unsigned sel = __ballot_sync(act, want);
  if (!sel) return;
  const int leader = __ffs(sel) - 1;
  const int lane32 = threadIdx.x & 31;
  int base = 0;
  if (lane32 == leader) base = atomicAdd(count, __popc(sel));
  base = __shfl_sync(act, base, leader);
  if (want) {
    const int slot = base + __popc(sel & ((1u << lane32) - 1u));
    if (slot < cap) list[slot] = p;
  }
}

// Pass 1: count the pairs of each band class.
__global__ void __launch_bounds__(256) k_rev_count(ResultSet rs, Scoring sc, const uint32_t *__restrict__ order,
                                                   int64_t n, int *band_counts, int s_cap) {
  __shared__ int cnt[kBandClasses];
  if (threadIdx.x < kBandClasses) cnt[threadIdx.x] = 0;
  __syncthreads();
  for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < n; idx += (int64_t)gridDim.x * blockDim.x) {
    const int64_t p = order ? (int64_t)order[idx] : idx;
    const int c = band_class(rs, sc, p, s_cap);
    if (c >= 0 && c < kBandClasses) atomicAdd(&cnt[c], 1);
  }
  __syncthreads();
  if (threadIdx.x < kBandClasses && cnt[threadIdx.x]) atomicAdd(&band_counts[threadIdx.x], cnt[threadIdx.x]);
}

// Pass 2: place each pair in its class segment (segments in class order, each filled in
// the batch's order); wider pairs go to the wavefront list.
__global__ void __launch_bounds__(256) k_rev_scatter(ResultSet rs, Scoring sc, const uint32_t *__restrict__ order,
                                                     int64_t n, WorkLists wl, int s_cap) {
  int off[kBandClasses];
  int acc = 0;
#pragma unroll
  for (int c = 0; c < kBandClasses; c++) {
    off[c] = acc;
    acc += wl.band_counts[c];
  }
  int *cursor = wl.band_counts + kBandClasses;
  for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < n; idx += (int64_t)gridDim.x * blockDim.x) {
    const int64_t p = order ? (int64_t)order[idx] : idx;
    const int S = rs.score[p];
    int c = -1;
    if (!((rs.flag[p] & kFlagTooLong) || S <= 0)) {
      c = S <= s_cap ? band_fit(S, rs.a_end[p] + 1, rs.b_end[p] + 1, sc) : kBandClasses;
    }
    // one append per class present in the warp: lanes of a class share one atomic
    const unsigned act = __activemask();
    const unsigned same = __match_any_sync(act, c);
    const int lane32 = threadIdx.x & 31;
    const int leader = __ffs(same) - 1;
    int64_t *list = nullptr;
    int *cnt = nullptr;
    int64_t cap = 0;
    if (c == kBandClasses) {
      list = wl.wide;
      cnt = wl.wide_count;
      cap = wl.cap;
    } else if (c >= 0) {
      int o = 0;
#pragma unroll
      for (int k = 0; k < kBandClasses; k++) o = k == c ? off[k] : o;
      list = wl.bands + o;
      cnt = cursor + c;
      cap = wl.cap - o;
    }
    int base = 0;
    if (c >= 0 && lane32 == leader) base = atomicAdd(cnt, __popc(same));
    base = __shfl_sync(act, base, leader);
    if (c >= 0) {
      const int slot = base + __popc(same & ((1u << lane32) - 1u));
      if (slot < cap) list[slot] = p;
    }
  }
}

// Band cells, two rows at a time.  Gap values are kept biased by +gO (E^ = E + gO,
// F^ = F + gO) so H feeds their updates directly.  cb[u + d] holds the code of band cell
// d's column OR 0x7770 (a byte_perm selector: byte 0 picks the row's score for that
// code, bytes 1-3 read zero); columns outside [0, N2) carry the PAD code, which scores
// -128: cells left of column 0 then stay exactly at the boundary values and cells right
// of the last column stay below the score, so the band needs no per-cell bound checks.
// BI: the table bytes already hold s + gO (every score >= -gO; PAD scores -gO), and
// Hdiag + byte is a multiply-add by a runtime 1 (bias then carries that 1), which issues
// on the FMA pipe instead of the integer ALU pipe the band saturates.  A PAD score of -gO
// keeps the cells left of column 0 at exactly 0 (their diagonal, above and left values
// are 0) and every cell right of the last column at most a real cell's H - gO.
template <bool BI>
__device__ __forceinline__ int band_q(int hd, uint32_t byte, int bias) {
  if constexpr (BI) return (int)mad_u32((uint32_t)hd, (uint32_t)bias, byte);
  else return hd + (int)byte + bias;
}

// Rows A (window offset u) and the row below it, B (offset u + 1), two cells behind.  B's
// cell d reads A's cells d (diagonal) and d + 1 (above), written at the two steps before,
// and overwrites A's cell d, which nothing needs any more; A's cell s reads only cells
// >= s of the row above.  The two rows' dependency chains (F along each row) are
// independent within a step, so they interleave.
// Returns the largest cell key of the two rows, key = H * 128 + (64 for row A) + 63 - d
// (W <= 63): its H is the larger row maximum, and among cells holding it the key picks
// the upper row first, then its leftmost cell -- the first cell SSW's reverse scan meets
// (rows = A positions before B positions).  The multiply-adds forming the keys issue on
// the FMA pipe; one three-way max per step folds both rows' keys.
template <int W, int NC, bool BI>
__device__ __forceinline__ int band_pair(const int (&cb)[NC], int u, uint32_t ra0, uint32_t ra1, uint32_t rb0,
                                         uint32_t rb1, int bias, int ngo, int nge, uint32_t k128, int (&H)[W + 1],
                                         int (&E)[W + 1]) {
  constexpr int NEG = -(1 << 28);
  static_assert(W <= 63, "cell index must fit the key's six bits");
  int FA = NEG, FB = NEG;
  int km = 0;
#pragma unroll
  for (int s = 0; s < W + 2; s++) {
    int ka = 0, kb = 0;
    if (s < W) {
      const int q = band_q<BI>(H[s], __byte_perm(ra0, ra1, (uint32_t)cb[u + s]), bias);
      const int e = __viaddmax_s32(E[s + 1], nge, H[s + 1]);
      const int ha = __viaddmax_s32_relu(__vimax3_s32(q, e, FA), ngo, 0);
      FA = __viaddmax_s32(FA, nge, ha);
      E[s] = e;
      H[s] = ha;
      ka = (int)mad_u32((uint32_t)ha, k128, (uint32_t)(64 + 63 - s));
    }
    if (s >= 2) {
      const int d = s - 2;
      const int q = band_q<BI>(H[d], __byte_perm(rb0, rb1, (uint32_t)cb[u + 1 + d]), bias);
      const int e = __viaddmax_s32(E[d + 1], nge, H[d + 1]);
      const int hb = __viaddmax_s32_relu(__vimax3_s32(q, e, FB), ngo, 0);
      FB = __viaddmax_s32(FB, nge, hb);
      E[d] = e;
      H[d] = hb;
      kb = (int)mad_u32((uint32_t)hb, k128, (uint32_t)(63 - d));
    }
    km = __vimax3_s32(km, ka, kb);
  }
  return km;
}

// Pass 3 (one launch per class C): the banded search over the class's segment.  Rows go
// in pairs, in blocks of U; the band's codes live in a register window of W + U columns
// that slides by U columns per block (one load per new column), and the rows' scores
// come from a per-block table indexed by the A code.  No cell of the reversed box exceeds
// the score, so the first cell reaching S in scan order is the largest key of the first
// row pair whose key reaches S * 128: every thread runs the same row-pair code whether or
// not its pair is about to reach the score.  A row past the box's last (an odd box) gets
// the PAD row, whose cells stay below S, and its upper row wins every tie anyway.
template <int WB, int C, bool BI>
__global__ void __launch_bounds__(128) k_rev_band(PairSet ps, ResultSet rs, Scoring sc, WorkLists wl) {
  constexpr int NEG = -(1 << 28);
  constexpr int G = WB / 2 - 1;
  constexpr int W = 2 * G + 1;
  constexpr int U = W <= 15 ? 8 : (W <= 31 ? 4 : 2);
  constexpr int NC = W + U;
  static_assert(G == band_half(C), "band class and width disagree");
  static_assert(U % 2 == 0, "rows go in pairs within a block");
  // per A code 0..4: s(a, c) + off as bytes c = 0..3 | c = 4, PAD; off = gO (BI) or 128;
  // code 5 (PAD, rows past the box): every column scores -off
  __shared__ uint32_t rptab[2 * 8];
  const int toff = BI ? sc.gap_open : 128;
  if (threadIdx.x < 6) {
    const int a = threadIdx.x;
    uint32_t r0 = 0, r1 = 0;
    for (int c = 0; c < 5 && a < kCodePad; c++) {
      const uint32_t v = (uint32_t)(sub_score(a, c, sc, 128) + toff) & 0xffu;
      if (c < 4) r0 |= v << (8 * c);
      else r1 = v;  // byte 1 (PAD) and above stay 0: score -off
    }
    rptab[2 * a] = r0;
    rptab[2 * a + 1] = r1;
  }
  __syncthreads();
  const int mt = sc.match;
  // BI: bias is a 1 the compiler cannot fold (gap_open is positive and below 2^30); k128
  // likewise a 128, so the key multiply-adds stay on the FMA pipe
  const int bias = BI ? (sc.gap_open >> 30) + 1 : sc.gap_open - 128, ngo = -sc.gap_open, nge = -sc.gap_extend;
  const uint32_t k128 = (uint32_t)(sc.gap_open >> 30) + 128u;
  int64_t off = 0;
#pragma unroll
  for (int c = 0; c < C; c++) off += wl.band_counts[c];
  int64_t total = wl.band_counts[C];
  if (off + total > wl.cap) total = wl.cap - off;
  // A pair's fields are loaded one grid-stride iteration ahead of its search (their
  // chain of dependent loads then overlaps the previous pair's rows), and the A codes of
  // each block's first row pair one block ahead (the other rows' codes are loaded at the
  // block's start and used after the first pair; the window's new columns are first read
  // at the end of a row).
  struct Meta {
    int64_t p = -1;
    int S = 0, ie = 0, je = 0;
    int64_t aoff = 0, boff = 0;
  };
  auto load_meta = [&](int64_t idx) {
    Meta m;
    if (idx < total) {
      m.p = wl.bands[off + idx];
      m.S = rs.score[m.p];
      m.ie = rs.a_end[m.p];
      m.je = rs.b_end[m.p];
      m.aoff = ps.a_off[m.p];
      m.boff = ps.b_off[m.p];
    }
    return m;
  };
  const int64_t gstride = (int64_t)gridDim.x * blockDim.x;
  int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  Meta cur = load_meta(idx);
  for (; idx < total; idx += gstride) {
    const Meta nxt = load_meta(idx + gstride);
    const int64_t p = cur.p;
    const int S = cur.S;
    const int ie = cur.ie, je = cur.je;
    const int M2 = ie + 1, N2 = je + 1;
    const uint8_t *a = ps.a_code + cur.aoff + ie;  // reversed: a[-i]
    const uint8_t *b = ps.b_code + cur.boff + je;  // reversed: b[-j]
    cur = nxt;
    auto code_at = [&](int j) -> int { return ((unsigned)j < (unsigned)N2 ? (int)b[-j] : kCodePad) | 0x7770; };
    auto row_code = [&](int r) -> int { return r < M2 ? (int)a[-r] : kCodePad; };
    // row caps are kept at multiples of U (or M2) so the window always slides by U
    auto cap_rows = [&](int t) { t = (t + U - 1) / U * U; return t < M2 ? t : M2; };
    int t = cap_rows(band_first_cap(S, mt, M2));
    const int L = band_left(S, M2, N2, sc, G);  // row i's band: columns i - L + [0, W)
    int fi = -1, fj = -1;
    bool escalate = false, found = false;
    int H[W + 1], E[W + 1], cb[NC];
#pragma unroll
    for (int d = 0; d <= W; d++) {
      H[d] = 0;
      E[d] = NEG;
    }
#pragma unroll
    for (int k = 0; k < NC; k++) cb[k] = code_at(k - L);
    int a0 = row_code(0), a1 = row_code(1);  // the block's first row pair
    int i = 0;  // first row of the current block; the window covers columns i - L + [0, NC)
    for (;;) {
      if (band_outgrown(t, N2, S, sc, L, G)) {
        escalate = true;
        break;
      }
      while (i < t && !found) {
        // the next block's first row pair
        const int n0 = row_code(i + U), n1 = row_code(i + U + 1);
        // t is a multiple of U below M2, so a row pair starting below t ends below t
        // unless t == M2 (its lower row is then the PAD row)
#pragma unroll
        for (int u = 0; u < U; u += 2) {
          const int row = i + u;
          if (!found && row < t) {
            const int ca = u == 0 ? a0 : row_code(row), cc = u == 0 ? a1 : row_code(row + 1);
            const int km = band_pair<W, NC, BI>(cb, u, rptab[2 * ca], rptab[2 * ca + 1], rptab[2 * cc],
                                                rptab[2 * cc + 1], bias, ngo, nge, k128, H, E);
            if ((km >> 7) >= S) {
              found = true;
              fi = row + 1 - ((km >> 6) & 1);
              fj = fi - L + (63 - (km & 63));
            }
          }
        }
        if (found || i + U >= M2) break;
        i += U;
#pragma unroll
        for (int k = 0; k < W; k++) cb[k] = cb[k + U];
#pragma unroll
        for (int k = W; k < NC; k++) cb[k] = code_at(i - L + k);
        a0 = n0;
        a1 = n1;
      }
      if (found || t >= M2) break;
      t = cap_rows(2 * t);
    }
    append_agg(wl.wide, wl.wide_count, wl.cap, p, escalate);
    if (escalate) continue;
    if (!found || fi >= M2 || fj < 0 || fj >= N2) {
      rs.flag[p] |= kFlagTooLong;  // inconsistent; reported as an error by the driver
      rs.a_beg[p] = -1;
      rs.b_beg[p] = 0;
      continue;
    }
    rs.a_beg[p] = ie - fi;
    rs.b_beg[p] = je - fj;
  }
}

// Packed int16x2 form of the row-pair band, for scores up to kBand16Score under the
// gap-open-biased table (klign's scorings).  One register holds a cell of row A (low
// half) and the cell of row B two positions behind it (high half), so each DPX operation
// updates both rows.  After a row pair, P[k] = (H of A's cell k, H of B's cell k - 2) and
// Q[k] likewise for E^; the next pair reads the row above from the high halves (old) and
// its own upper row from the low halves (new), so the "above" operands of a step are
// gathered by one byte permute each, and the diagonal operand of a step is the "above"
// operand of the step before.  F's chain runs along each half on its own.  Halves that are
// no cell (B before its first cell, A past its last) are kept out: A's cells past the band
// hold H = 0 and E^ = NEG for B, and the row maxima skip both.  No cell of the reversed box
// exceeds S (<= 16000), every value stays inside int16, and the low-half sums of the
// multiply-add never carry (all terms are non-negative).
constexpr int kBand16Score = 16000;

template <int W, int NC>
__device__ __forceinline__ uint32_t band_pair16(const int (&cb)[NC], int u, uint32_t ra0, uint32_t ra1,
                                                uint32_t rb0, uint32_t rb1, uint32_t one, uint32_t ngo2,
                                                uint32_t nge2, uint32_t (&P)[W + 3], uint32_t (&Q)[W + 3]) {
  constexpr uint32_t NEG2 = 0xC000C000u;  // -16384 in both halves
  uint32_t F2 = NEG2, rm = 0u, up_prev = 0u;
#pragma unroll
  for (int s = 0; s < W + 2; s++) {
    // above-operands: high halves of the old row at s + 3, low halves of the new row at s - 1
    constexpr int kLast = W + 2;
    const int iu = s + 3 <= kLast ? s + 3 : kLast;
    const uint32_t up2 = __byte_perm(P[iu], s >= 1 ? P[s >= 1 ? s - 1 : 0] : 0u, 0x5432);
    const uint32_t eup2 = __byte_perm(Q[iu], s >= 1 ? Q[s >= 1 ? s - 1 : 0] : NEG2, 0x5432);
    const uint32_t diag2 = s == 0 ? __byte_perm(P[2], 0u, 0x5432) : up_prev;
    // scores (s + gO as bytes): A at window column u + s, B one column to the left
    const uint32_t sa = __byte_perm(ra0, ra1, (uint32_t)cb[u + s]);
    const uint32_t sb = __byte_perm(rb0, rb1, (uint32_t)cb[u + s >= 1 ? u + s - 1 : 0]);
    const uint32_t q2 = mad_u32(diag2, one, __byte_perm(sa, sb, 0x5410));
    const uint32_t e2 = __viaddmax_s16x2(eup2, nge2, up2);
    if (s == 2) F2 = __byte_perm(F2, NEG2, 0x7610);  // B's row starts here
    const uint32_t h2 = __viaddmax_s16x2_relu(__vimax3_s16x2(q2, e2, F2), ngo2, 0u);
    F2 = __viaddmax_s16x2(F2, nge2, h2);
    uint32_t hs = h2, es = e2;
    if (s >= W) {  // A has no cell here: H = 0, E^ = NEG for the cells of B below it
      hs = h2 & 0xffff0000u;
      es = __byte_perm(e2, NEG2, 0x3254);
    }
    P[s] = hs;
    Q[s] = es;
    rm = __vmaxs2(rm, s < 2 ? (h2 & 0xffffu) : hs);
    up_prev = up2;
  }
  return rm;
}

// Pass 3, packed: k_rev_band's search with band_pair16 (klign's scorings, S <= 16000).
template <int WB, int C>
__global__ void __launch_bounds__(128) k_rev_band16(PairSet ps, ResultSet rs, Scoring sc, WorkLists wl) {
  constexpr int G = WB / 2 - 1;
  constexpr int W = 2 * G + 1;
  constexpr int U = W <= 15 ? 8 : (W <= 31 ? 4 : 2);
  constexpr int NC = W + U;
  static_assert(G == band_half(C), "band class and width disagree");
  static_assert(U % 2 == 0, "rows go in pairs within a block");
  __shared__ uint32_t rptab[2 * 8];
  if (threadIdx.x < 6) {
    const int a = threadIdx.x;
    uint32_t r0 = 0, r1 = 0;
    for (int c = 0; c < 5 && a < kCodePad; c++) {
      const uint32_t v = (uint32_t)(sub_score(a, c, sc, 128) + sc.gap_open) & 0xffu;
      if (c < 4) r0 |= v << (8 * c);
      else r1 = v;
    }
    rptab[2 * a] = r0;
    rptab[2 * a + 1] = r1;
  }
  __syncthreads();
  const int mt = sc.match;
  const uint32_t one = (uint32_t)(sc.gap_open >> 30) + 1u;  // a 1 the compiler cannot fold
  const uint32_t ngo2 = (uint32_t)(uint16_t)(-sc.gap_open) * 0x00010001u;
  const uint32_t nge2 = (uint32_t)(uint16_t)(-sc.gap_extend) * 0x00010001u;
  int64_t off = 0;
#pragma unroll
  for (int c = 0; c < C; c++) off += wl.band_counts[c];
  int64_t total = wl.band_counts[C];
  if (off + total > wl.cap) total = wl.cap - off;
  struct Meta {
    int64_t p = -1;
    int S = 0, ie = 0, je = 0;
    int64_t aoff = 0, boff = 0;
  };
  auto load_meta = [&](int64_t idx) {
    Meta m;
    if (idx < total) {
      m.p = wl.bands[off + idx];
      m.S = rs.score[m.p];
      m.ie = rs.a_end[m.p];
      m.je = rs.b_end[m.p];
      m.aoff = ps.a_off[m.p];
      m.boff = ps.b_off[m.p];
    }
    return m;
  };
  const int64_t gstride = (int64_t)gridDim.x * blockDim.x;
  int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  Meta cur = load_meta(idx);
  for (; idx < total; idx += gstride) {
    const Meta nxt = load_meta(idx + gstride);
    const int64_t p = cur.p;
    const int S = cur.S;
    const int ie = cur.ie, je = cur.je;
    const int M2 = ie + 1, N2 = je + 1;
    const uint8_t *a = ps.a_code + cur.aoff + ie;  // reversed: a[-i]
    const uint8_t *b = ps.b_code + cur.boff + je;  // reversed: b[-j]
    cur = nxt;
    auto code_at = [&](int j) -> int { return ((unsigned)j < (unsigned)N2 ? (int)b[-j] : kCodePad) | 0x7770; };
    auto row_code = [&](int r) -> int { return r < M2 ? (int)a[-r] : kCodePad; };
    auto cap_rows = [&](int t) { t = (t + U - 1) / U * U; return t < M2 ? t : M2; };
    int t = cap_rows(band_first_cap(S, mt, M2));
    const int L = band_left(S, M2, N2, sc, G);  // row i's band: columns i - L + [0, W)
    int fi = -1, fj = -1;
    bool escalate = false, found = false;
    uint32_t P[W + 3], Q[W + 3];
    int cb[NC];
#pragma unroll
    for (int d = 0; d < W + 3; d++) {
      P[d] = 0u;
      Q[d] = 0xC000C000u;
    }
#pragma unroll
    for (int k = 0; k < NC; k++) cb[k] = code_at(k - L);
    int a0 = row_code(0), a1 = row_code(1);
    int i = 0;
    for (;;) {
      if (band_outgrown(t, N2, S, sc, L, G)) {
        escalate = true;
        break;
      }
      while (i < t && !found) {
        const int n0 = row_code(i + U), n1 = row_code(i + U + 1);
#pragma unroll
        for (int u = 0; u < U; u += 2) {
          const int row = i + u;
          if (!found && row < t) {
            const int ca = u == 0 ? a0 : row_code(row), cc = u == 0 ? a1 : row_code(row + 1);
            const uint32_t rm = band_pair16<W, NC>(cb, u, rptab[2 * ca], rptab[2 * ca + 1], rptab[2 * cc],
                                                   rptab[2 * cc + 1], one, ngo2, nge2, P, Q);
            if ((int)(rm & 0xffffu) >= S || (int)(rm >> 16) >= S) {
              // the first cell holding S: row A's cells left to right, then row B's
              found = true;
#pragma unroll
              for (int k = 0; k < W; k++)
                if (fi < 0 && (int)(P[k] & 0xffffu) == S) {
                  fi = row;
                  fj = row - L + k;
                }
#pragma unroll
              for (int k = 2; k < W + 2; k++)
                if (fi < 0 && (int)(P[k] >> 16) == S) {
                  fi = row + 1;
                  fj = row + 1 - L + (k - 2);
                }
            }
          }
        }
        if (found || i + U >= M2) break;
        i += U;
#pragma unroll
        for (int k = 0; k < W; k++) cb[k] = cb[k + U];
#pragma unroll
        for (int k = W; k < NC; k++) cb[k] = code_at(i - L + k);
        a0 = n0;
        a1 = n1;
      }
      if (found || t >= M2) break;
      t = cap_rows(2 * t);
    }
    append_agg(wl.wide, wl.wide_count, wl.cap, p, escalate);
    if (escalate) continue;
    if (!found || fi < 0 || fi >= M2 || fj < 0 || fj >= N2) {
      rs.flag[p] |= kFlagTooLong;  // inconsistent; reported as an error by the driver
      rs.a_beg[p] = -1;
      rs.b_beg[p] = 0;
      continue;
    }
    rs.a_beg[p] = ie - fi;
    rs.b_beg[p] = je - fj;
  }
}

// SSW's second-best score (ssw_core.cpp:513-536, :825-847, :1154-1160) from the row
// maxima of the forward pass: the largest row maximum, first row on ties, over rows
// before a_end - maskLen and from a_end + maskLen on (+1 on the byte path), with
// maskLen = max(len(A)/2, 15) as klign passes it (klign.cpp:257).
__global__ void k_score2(PairSet ps, ResultSet rs, Scoring sc, int64_t n) {
  const int bias = ssw_bias(sc);
  for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < n; p += (int64_t)gridDim.x * blockDim.x) {
    const int M = ps.a_len[p], N = ps.b_len[p];
    int best = 0, at = 0;
    if (M > 0 && N > 0 && !(rs.flag[p] & kFlagTooLong)) {
      const int S = rs.score[p], ie = rs.a_end[p];
      const int mask = M / 2 > 15 ? M / 2 : 15;
      const bool word = S + bias >= 255;
      const int32_t *rm = ((word && ssw_pad8(N) != ssw_pad16(N)) ? ps.rowmax8 : ps.rowmax16) + ps.a_off[p];
      const int e1 = ie - mask > 0 ? ie - mask : 0;
      for (int i = 0; i < e1; i++) {
        const int v = rm[i];
        if (v > best) {
          best = v;
          at = i;
        }
      }
      const int e2 = ie + mask > M ? M : ie + mask;
      for (int i = word ? e2 : e2 + 1; i < M; i++) {
        const int v = rm[i];
        if (v > best) {
          best = v;
          at = i;
        }
      }
    }
    rs.score2[p] = best;
    rs.a_end2[p] = at;
  }
}

// Byte arena -> SSW base codes (0..4), 16 bytes per thread step when aligned.
__global__ void k_translate(const char *__restrict__ src, uint8_t *__restrict__ dst, int64_t nbytes, int vec) {
  __shared__ uint8_t tab[256];
  for (int i = threadIdx.x; i < 256; i += blockDim.x) tab[i] = c_code[i];
  __syncthreads();
  const int64_t tid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  int64_t done = 0;
  if (vec) {
    const int64_t n16 = nbytes / 16;
    const uint4 *s4 = reinterpret_cast<const uint4 *>(src);
    uint4 *d4 = reinterpret_cast<uint4 *>(dst);
    for (int64_t i = tid; i < n16; i += stride) {
      uint4 v = s4[i];
      uint32_t w[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
      for (int q = 0; q < 4; q++) {
        const uint32_t x = w[q];
        w[q] = (uint32_t)tab[x & 0xff] | ((uint32_t)tab[(x >> 8) & 0xff] << 8) | ((uint32_t)tab[(x >> 16) & 0xff] << 16) |
               ((uint32_t)tab[x >> 24] << 24);
      }
      d4[i] = make_uint4(w[0], w[1], w[2], w[3]);
    }
    done = n16 * 16;
  }
  for (int64_t i = done + tid; i < nbytes; i += stride) dst[i] = tab[(unsigned char)src[i]];
}

// Wavefront begin search on the reversed box for the pairs listed in wl.wide whose score
// lies in [s_lo, s_hi].  No cell of the reversed box exceeds the score, so int16 values
// (V16) are exact for scores up to kWaveScore16; the int32 instantiation takes the rest.
constexpr int kWaveScore16 = 16000;
template <class VT, int K, int G>
__global__ void __launch_bounds__(256) k_rev_wave(PairSet ps, ResultSet rs, Scoring sc, WorkLists wl,
                                                  typename VT::Pay *scratch, int scratch_stride, int pad, int bcap,
                                                  int s_lo, int s_hi) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int lanes = blockDim.x;
  const int gpb = lanes / G;
  const int grp = threadIdx.x / G;
  const int lane = threadIdx.x % G;
  const unsigned gmask = group_mask(G);
  constexpr size_t kProf = group_prof_bytes<VT, K, G>();
  unsigned char *gbase = smem + (size_t)grp * (kProf + (size_t)bcap);
  GroupSmem gs;
  gs.prof = reinterpret_cast<uint32_t *>(gbase);
  gs.prof_lanes = G;
  gs.bcodes = gbase + kProf;
  gs.pad = pad;
  gs.bcap = bcap;
  constexpr int RS = 2 * K * G;
  const int64_t total = *wl.wide_count < wl.cap ? *wl.wide_count : wl.cap;
  const int64_t gid = (int64_t)blockIdx.x * gpb + grp;
  const int64_t gstride = (int64_t)gridDim.x * gpb;
  typename VT::Pay *bnd = scratch ? scratch + gid * (int64_t)scratch_stride : nullptr;
  for (int64_t i = gid; i < total; i += gstride) {
    const int64_t p = wl.wide[i];
    const int S = rs.score[p];
    if (S < s_lo || S > s_hi) continue;
    const int ie = rs.a_end[p], je = rs.b_end[p];
    const int M2 = ie + 1;
    const int dmax = M2 < je + 1 ? M2 : je + 1;
    const long long gbl = gap_cells_bound(dmax, S, sc);
    long long n2 = (long long)M2 + gbl + 1;
    if (n2 > je + 1) n2 = je + 1;
    const int N2 = (int)n2;
    const bool too_long = (N2 > bcap - pad - 2 * G) || (M2 > RS && (bnd == nullptr || N2 > scratch_stride));
    if (too_long) {
      if (lane == 0) {
        rs.flag[p] |= kFlagTooLong;
        rs.a_beg[p] = -1;
        rs.b_beg[p] = 0;
      }
      continue;
    }
    SeqView A{ps.a_code + ps.a_off[p] + ie, -1, M2};
    SeqView B{ps.b_code + ps.b_off[p] + je, -1, N2};
    SweepOut so;
    sweep_pair<VT, K, G>(A, B, sc, gs, lane, gmask, bnd, 0x7fffffff, so);
    if (lane == 0) {
      if (key_value(so.key) != S) {
        rs.flag[p] |= kFlagTooLong;
        rs.a_beg[p] = -1;
        rs.b_beg[p] = 0;
      } else {
        rs.a_beg[p] = ie - key_row(so.key);
        rs.b_beg[p] = je - key_col(so.key);
      }
    }
  }
}

__device__ __forceinline__ int16_t to_short(int v) {
  return (int16_t)(v > 32767 ? 32767 : (v < -32768 ? -32768 : v));
}

__global__ void k_finalize(ResultSet rs, int64_t n, bool a_is_query, int part, OutViews ov) {
  for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < n; p += (int64_t)gridDim.x * blockDim.x) {
    if (part & 1) {
      const int sc = rs.score[p], ae = rs.a_end[p], be = rs.b_end[p];
      const int re = a_is_query ? be : ae, qe = a_is_query ? ae : be;
      if (ov.s_score) ov.s_score[p] = to_short(sc);
      if (ov.s_ref_end) ov.s_ref_end[p] = to_short(re);
      if (ov.s_qry_end) ov.s_qry_end[p] = to_short(qe);
      if (ov.w_score) ov.w_score[p] = sc;
      if (ov.w_ref_end) ov.w_ref_end[p] = re;
      if (ov.w_qry_end) ov.w_qry_end[p] = qe;
    }
    if (part & 2) {
      const int ab = rs.a_beg[p], bb = rs.b_beg[p];
      const int rb = a_is_query ? bb : ab, qb = a_is_query ? ab : bb;
      if (ov.s_ref_beg) ov.s_ref_beg[p] = to_short(rb);
      if (ov.s_qry_beg) ov.s_qry_beg[p] = to_short(qb);
      if (ov.w_ref_beg) ov.w_ref_beg[p] = rb;
      if (ov.w_qry_beg) ov.w_qry_beg[p] = qb;
    }
  }
}

__global__ void k_pack5(ResultSet rs, int64_t n, int32_t *out5) {
  for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < n; p += (int64_t)gridDim.x * blockDim.x) {
    int32_t *o = out5 + 5 * p;
    o[0] = rs.score[p];
    o[1] = rs.a_beg[p];
    o[2] = rs.a_end[p];
    o[3] = rs.b_beg[p];
    o[4] = rs.b_end[p];
  }
}

__global__ void k_reset_lists(WorkLists wl) {
  *wl.ovf_count = 0;
  *wl.wide_count = 0;
  for (int i = 0; i < 2 * kBandClasses; i++) wl.band_counts[i] = 0;
}

int g_num_sms = 0;

int num_sms(int device) {
  if (g_num_sms == 0) {
    int v = 0;
    cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, device);
    g_num_sms = v > 0 ? v : 1;
  }
  return g_num_sms;
}

template <int C>
size_t group_prof16_rt_c(int K, int G) {
  if (G == kGKShort) {
    switch (K) {
      case 4: return group_prof16_bytes<4, kGKShort, C>();
      case 6: return group_prof16_bytes<6, kGKShort, C>();
      case 8: return group_prof16_bytes<8, kGKShort, C>();
      default: return group_prof16_bytes<10, kGKShort, C>();
    }
  }
  return K == 6 ? group_prof16_bytes<6, kGKLong, C>() : group_prof16_bytes<8, kGKLong, C>();
}

size_t group_prof16_rt(int K, int G, bool s2) {
  return s2 ? group_prof16_rt_c<kCode16Zero + 1>(K, G) : group_prof16_rt_c<kCodeN + 1>(K, G);
}

size_t group_prof_rt(bool wide32, int K) {
  if (wide32) return group_prof_bytes<V32, 4, kG>();
  switch (K) {
    case 2: return group_prof_bytes<V16, 2, kG>();
    case 3: return group_prof_bytes<V16, 3, kG>();
    case 4: return group_prof_bytes<V16, 4, kG>();
    case 5: return group_prof_bytes<V16, 5, kG>();
    case 6: return group_prof_bytes<V16, 6, kG>();
    case 7: return group_prof_bytes<V16, 7, kG>();
    default: return group_prof_bytes<V16, 8, kG>();
  }
}

template <class VT, int K>
cudaError_t launch_fwd_t(const FwdConfig &cfg, const PairSet &ps, const ResultSet &rs, const Scoring &sc,
                         const int64_t *list, const int *list_count, int ceiling, void *scratch, int scratch_stride,
                         const WorkLists &wl, cudaStream_t st) {
  auto kern = ps.rowmax16 ? k_fwd<VT, K, kG, true> : k_fwd<VT, K, kG, false>;
  {
    cudaError_t e = raise_smem_limit(reinterpret_cast<const void *>(kern), cfg.smem);
    if (e != cudaSuccess) return e;
  }
  kern<<<cfg.grid, cfg.groups_per_block * kG, cfg.smem, st>>>(
      ps, rs, sc, list, list_count, ceiling, reinterpret_cast<typename VT::Pay *>(scratch), scratch_stride, wl, cfg.pad,
      cfg.bcap);
  return cudaGetLastError();
}

template <int K, int G>
cudaError_t launch_fwd16_t(const FwdConfig &cfg, const PairSet &ps, const ResultSet &rs, const Scoring &sc,
                           int ceiling, void *scratch, int scratch_stride, const WorkLists &wl, cudaStream_t st) {
  auto kern = ps.rowmax16 ? k_fwd16<K, G, true> : k_fwd16<K, G, false>;
  {
    cudaError_t e = raise_smem_limit(reinterpret_cast<const void *>(kern), cfg.smem);
    if (e != cudaSuccess) return e;
  }
  kern<<<cfg.grid, cfg.groups_per_block * G, cfg.smem, st>>>(ps, rs, sc, ceiling,
                                                              reinterpret_cast<V16::Pay *>(scratch), scratch_stride,
                                                              wl, cfg.pad, cfg.bcap);
  return cudaGetLastError();
}

}  // namespace

bool keyed_scoring(const Scoring &sc) {
  return sc.mismatch <= sc.gap_open && sc.ambiguity <= sc.gap_open && sc.gap_open >= 1 && sc.gap_extend >= 1;
}

cudaError_t plan_forward(int device, int max_a, int max_b, bool wide32, FwdConfig *cfg, bool keyed, bool s2) {
  FwdConfig c{};
  c.G = kG;
  if (keyed && !wide32) {
    c.G = keyed_g_for_rows(max_a);
    c.K = keyed_k_for_rows(max_a);
  } else if (wide32) {
    c.K = 4;
  } else {
    const int need = (max_a + 2 * kG - 1) / (2 * kG);  // K with 2*K*G >= max_a
    if (need <= 2) c.K = 2;
    else if (need <= 3) c.K = 3;
    else if (need <= 4) c.K = 4;
    else if (need <= 5) c.K = 5;
    else if (need <= 6) c.K = 6;
    else if (need <= 7) c.K = 7;
    else c.K = 8;
  }
  c.pad = 2 * c.G;
  if (max_b < 1) max_b = 1;
  if (max_b > kMaxB) return cudaErrorInvalidValue;
  // room for B, the groups' lane skew and SSW's zero-score padding of score2 mode (< 16)
  c.bcap = ((c.pad + max_b + 16 + 2 * c.G) + 15) / 16 * 16;
  const size_t budget = 100 * 1024;  // keep two blocks per SM possible
  // the keyed engine reads B from global memory: its group needs the profile table only
  const size_t per_group =
      (keyed && !wide32) ? group_prof16_rt(c.K, c.G, s2) : group_prof_rt(wide32, c.K) + (size_t)c.bcap;
  int gpb = 8;
  while (gpb > 1 && (size_t)gpb * per_group > budget) gpb /= 2;
  if (c.G < kG) gpb *= kG / c.G;  // same block size (128 threads) with smaller groups
  c.groups_per_block = gpb;
  c.smem = (size_t)gpb * per_group;
  if (c.smem > 220 * 1024) return cudaErrorInvalidValue;
  int sms = num_sms(device);
  c.grid = sms * 8;  // grid-stride; callers may lower it
  c.keyed = keyed && !wide32;
  *cfg = c;
  return cudaSuccess;
}

size_t forward_scratch_bytes(const FwdConfig &cfg, int max_a, int max_b, bool wide32) {
  const int RS = 2 * cfg.K * cfg.G;
  if (max_a <= RS) return 0;
  (void)max_b;
  const size_t pay = wide32 ? sizeof(V32::Pay) : sizeof(V16::Pay);
  return (size_t)cfg.grid * cfg.groups_per_block * (size_t)cfg.bcap * pay;  // stride = bcap payloads per group
}

cudaError_t launch_forward(const FwdConfig &cfg, bool wide32, const PairSet &ps, const ResultSet &rs,
                           const Scoring &sc, const int64_t *list, const int *list_count, int ceiling,
                           void *scratch, const WorkLists &wl, cudaStream_t st) {
  // scratch stride (payloads per group) = B capacity
  const int stride = cfg.bcap;
  if (wide32) return launch_fwd_t<V32, 4>(cfg, ps, rs, sc, list, list_count, ceiling, scratch, stride, wl, st);
  if (cfg.keyed && !list) {
    if (cfg.G == kGKShort) {
      switch (cfg.K) {
        case 4: return launch_fwd16_t<4, kGKShort>(cfg, ps, rs, sc, ceiling, scratch, stride, wl, st);
        case 6: return launch_fwd16_t<6, kGKShort>(cfg, ps, rs, sc, ceiling, scratch, stride, wl, st);
        case 8: return launch_fwd16_t<8, kGKShort>(cfg, ps, rs, sc, ceiling, scratch, stride, wl, st);
        default: return launch_fwd16_t<10, kGKShort>(cfg, ps, rs, sc, ceiling, scratch, stride, wl, st);
      }
    }
    if (cfg.K == 6) return launch_fwd16_t<6, kGKLong>(cfg, ps, rs, sc, ceiling, scratch, stride, wl, st);
    return launch_fwd16_t<8, kGKLong>(cfg, ps, rs, sc, ceiling, scratch, stride, wl, st);
  }
  switch (cfg.K) {
    case 2: return launch_fwd_t<V16, 2>(cfg, ps, rs, sc, list, list_count, ceiling, scratch, stride, wl, st);
    case 3: return launch_fwd_t<V16, 3>(cfg, ps, rs, sc, list, list_count, ceiling, scratch, stride, wl, st);
    case 4: return launch_fwd_t<V16, 4>(cfg, ps, rs, sc, list, list_count, ceiling, scratch, stride, wl, st);
    case 5: return launch_fwd_t<V16, 5>(cfg, ps, rs, sc, list, list_count, ceiling, scratch, stride, wl, st);
    case 6: return launch_fwd_t<V16, 6>(cfg, ps, rs, sc, list, list_count, ceiling, scratch, stride, wl, st);
    case 7: return launch_fwd_t<V16, 7>(cfg, ps, rs, sc, list, list_count, ceiling, scratch, stride, wl, st);
    default: return launch_fwd_t<V16, 8>(cfg, ps, rs, sc, list, list_count, ceiling, scratch, stride, wl, st);
  }
}

cudaError_t forks_create(Forks &f) {
  cudaError_t e = cudaEventCreateWithFlags(&f.fork, cudaEventDisableTiming);
  for (int k = 0; k < kSideStreams && e == cudaSuccess; k++) {
    e = cudaStreamCreateWithFlags(&f.side[k], cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&f.join[k], cudaEventDisableTiming);
  }
  return e;
}

void forks_destroy(Forks &f) {
  for (int k = 0; k < kSideStreams; k++) {
    if (f.side[k]) cudaStreamDestroy(f.side[k]);
    if (f.join[k]) cudaEventDestroy(f.join[k]);
    f.side[k] = nullptr;
    f.join[k] = nullptr;
  }
  if (f.fork) cudaEventDestroy(f.fork);
  f.fork = nullptr;
}

cudaError_t fork_to(const Forks &f, cudaStream_t st, int k) {
  cudaError_t e = cudaEventRecord(f.fork, st);
  for (int i = 0; i < k && e == cudaSuccess; i++) e = cudaStreamWaitEvent(f.side[i], f.fork, 0);
  return e;
}

cudaError_t join_from(const Forks &f, cudaStream_t st, int k) {
  cudaError_t e = cudaSuccess;
  for (int i = 0; i < k && e == cudaSuccess; i++) {
    e = cudaEventRecord(f.join[i], f.side[i]);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(st, f.join[i], 0);
  }
  return e;
}


// Strip plan of a wavefront launch: the grid and the boundary scratch its groups need
// when A is longer than one strip (max_a > 2*K*G).  Returns false when that scratch is
// not available.
template <class VT>
static bool wave_plan(FwdConfig &c, int max_a, void *scratch, size_t scratch_bytes, int sms,
                      typename VT::Pay **scr) {
  *scr = nullptr;
  if (max_a > 2 * c.K * c.G) {
    const size_t per_group = (size_t)c.bcap * sizeof(typename VT::Pay);
    const int groups =
        scratch ? (int)std::min<size_t>(scratch_bytes / per_group, (size_t)c.grid * c.groups_per_block) : 0;
    if (groups < c.groups_per_block) return false;
    c.grid = groups / c.groups_per_block;
    *scr = reinterpret_cast<typename VT::Pay *>(scratch);
  }
  c.grid = std::max(1, std::min(c.grid, sms * 4));
  return true;
}

template <class VT>
static bool wave_launch_ok(FwdConfig c, int max_a, void *scratch, size_t scratch_bytes, int sms) {
  typename VT::Pay *scr;
  return wave_plan<VT>(c, max_a, scratch, scratch_bytes, sms, &scr);
}

template <class VT, int K>
static cudaError_t launch_rev_wave_t(FwdConfig c, const PairSet &ps, const ResultSet &rs, const Scoring &sc,
                                     const WorkLists &wl, void *scratch, size_t scratch_bytes, int max_a, int sms,
                                     int s_lo, int s_hi, cudaStream_t st) {
  typename VT::Pay *scr = nullptr;
  // without scratch, pairs longer than a strip are reported (kFlagTooLong), as before
  wave_plan<VT>(c, max_a, scratch, scratch_bytes, sms, &scr);
  auto kern = k_rev_wave<VT, K, kG>;
  cudaError_t e = raise_smem_limit(reinterpret_cast<const void *>(kern), c.smem);
  if (e != cudaSuccess) return e;
  kern<<<c.grid, c.groups_per_block * kG, c.smem, st>>>(ps, rs, sc, wl, scr, c.bcap, c.pad, c.bcap, s_lo, s_hi);
  return cudaGetLastError();
}

static cudaError_t launch_rev_wave16(const FwdConfig &c, const PairSet &ps, const ResultSet &rs, const Scoring &sc,
                                     const WorkLists &wl, void *scratch, size_t scratch_bytes, int max_a, int sms,
                                     cudaStream_t st) {
  switch (c.K) {
    case 2: return launch_rev_wave_t<V16, 2>(c, ps, rs, sc, wl, scratch, scratch_bytes, max_a, sms, 1, kWaveScore16, st);
    case 3: return launch_rev_wave_t<V16, 3>(c, ps, rs, sc, wl, scratch, scratch_bytes, max_a, sms, 1, kWaveScore16, st);
    case 4: return launch_rev_wave_t<V16, 4>(c, ps, rs, sc, wl, scratch, scratch_bytes, max_a, sms, 1, kWaveScore16, st);
    case 5: return launch_rev_wave_t<V16, 5>(c, ps, rs, sc, wl, scratch, scratch_bytes, max_a, sms, 1, kWaveScore16, st);
    case 6: return launch_rev_wave_t<V16, 6>(c, ps, rs, sc, wl, scratch, scratch_bytes, max_a, sms, 1, kWaveScore16, st);
    case 7: return launch_rev_wave_t<V16, 7>(c, ps, rs, sc, wl, scratch, scratch_bytes, max_a, sms, 1, kWaveScore16, st);
    default: return launch_rev_wave_t<V16, 8>(c, ps, rs, sc, wl, scratch, scratch_bytes, max_a, sms, 1, kWaveScore16, st);
  }
}

cudaError_t launch_reverse(int device, const PairSet &ps, const ResultSet &rs, const Scoring &sc, int max_a,
                           int max_b, void *scratch, size_t scratch_bytes, const WorkLists &wl, cudaStream_t st,
                           const uint32_t *order, const Forks *fk) {
  const int sms = num_sms(device);
  if (ps.n > 0) {
    const int grid = (int)std::min<int64_t>((ps.n + 255) / 256, (int64_t)sms * 8);
    const int gridb = sms * 8;
    // band classes by half-width 3, 5, 7, 11, 15, 23, 31 (band of 7 .. 63 cells); the
    // segments' counts stay on the device.
    // scores s + gO as bytes when no penalty exceeds the gap-open penalty (klign's scorings);
    // then the packed int16 band kernels take scores up to kBand16Score
    const bool bi = sc.gap_open > 0 && sc.mismatch <= sc.gap_open && sc.ambiguity <= sc.gap_open &&
                    sc.match + sc.gap_open <= 255;
    const int s_cap = bi ? kBand16Score : 0x7fffffff;
    k_rev_count<<<grid, 256, 0, st>>>(rs, sc, order, ps.n, wl.band_counts, s_cap);
    k_rev_scatter<<<grid, 256, 0, st>>>(rs, sc, order, ps.n, wl, s_cap);
    // The classes are independent: with side streams they run concurrently, so the
    // latency-bound narrow classes share the SMs with the wide ones.
    cudaStream_t cs[kBandClasses];
    const bool fan = fk && fk->fork;
    if (fan) {
      cudaError_t e = fork_to(*fk, st, kBandClasses);
      if (e != cudaSuccess) return e;
    }
    for (int c = 0; c < kBandClasses; c++) cs[c] = fan ? fk->side[c] : st;
    if (bi) {
      k_rev_band16<64, 6><<<gridb, 128, 0, cs[6]>>>(ps, rs, sc, wl);
      k_rev_band16<48, 5><<<gridb, 128, 0, cs[5]>>>(ps, rs, sc, wl);
      k_rev_band16<32, 4><<<gridb, 128, 0, cs[4]>>>(ps, rs, sc, wl);
      k_rev_band16<24, 3><<<gridb, 128, 0, cs[3]>>>(ps, rs, sc, wl);
      k_rev_band16<16, 2><<<gridb, 128, 0, cs[2]>>>(ps, rs, sc, wl);
      k_rev_band16<12, 1><<<gridb, 128, 0, cs[1]>>>(ps, rs, sc, wl);
      k_rev_band16<8, 0><<<gridb, 128, 0, cs[0]>>>(ps, rs, sc, wl);
    } else {
      k_rev_band<64, 6, false><<<gridb, 128, 0, cs[6]>>>(ps, rs, sc, wl);
      k_rev_band<48, 5, false><<<gridb, 128, 0, cs[5]>>>(ps, rs, sc, wl);
      k_rev_band<32, 4, false><<<gridb, 128, 0, cs[4]>>>(ps, rs, sc, wl);
      k_rev_band<24, 3, false><<<gridb, 128, 0, cs[3]>>>(ps, rs, sc, wl);
      k_rev_band<16, 2, false><<<gridb, 128, 0, cs[2]>>>(ps, rs, sc, wl);
      k_rev_band<12, 1, false><<<gridb, 128, 0, cs[1]>>>(ps, rs, sc, wl);
      k_rev_band<8, 0, false><<<gridb, 128, 0, cs[0]>>>(ps, rs, sc, wl);
    }
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    if (fan) {
      e = join_from(*fk, st, kBandClasses);
      if (e != cudaSuccess) return e;
    }
  }
  // Wide bands: wavefront on the reversed box (count read on the device), in int16 for
  // scores up to kWaveScore16 where a strip plan with scratch exists, int32 otherwise.
  FwdConfig c16, c32;
  cudaError_t e = plan_forward(device, max_a, max_b, false, &c16, false, false);
  if (e != cudaSuccess) return e;
  e = plan_forward(device, max_a, max_b, true, &c32);
  if (e != cudaSuccess) return e;
  int split = 0;  // largest score the int16 launch takes
  if (wave_launch_ok<V16>(c16, max_a, scratch, scratch_bytes, sms)) {
    e = launch_rev_wave16(c16, ps, rs, sc, wl, scratch, scratch_bytes, max_a, sms, st);
    if (e != cudaSuccess) return e;
    split = kWaveScore16;
  }
  return launch_rev_wave_t<V32, 4>(c32, ps, rs, sc, wl, scratch, scratch_bytes, max_a, sms, split + 1, 0x7fffffff, st);
}

cudaError_t raise_smem_limit(const void *func, size_t bytes) {
  if (bytes <= 48 * 1024) return cudaSuccess;
  static std::mutex mu;
  static std::map<std::pair<int, const void *>, size_t> limit;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  std::lock_guard<std::mutex> lk(mu);
  size_t &cur = limit[{dev, func}];
  if (bytes <= cur) return cudaSuccess;
  e = cudaFuncSetAttribute(func, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
  if (e == cudaSuccess) cur = bytes;
  return e;
}

cudaError_t launch_translate(const char *src, uint8_t *dst, int64_t nbytes, cudaStream_t st) {
  if (nbytes <= 0) return cudaSuccess;
  const int vec = ((reinterpret_cast<uintptr_t>(src) | reinterpret_cast<uintptr_t>(dst)) % 16 == 0) ? 1 : 0;
  const int64_t work = vec ? (nbytes / 16 + 1) : nbytes;
  const int grid = (int)std::min<int64_t>((work + 255) / 256, 152 * 16);
  k_translate<<<grid, 256, 0, st>>>(src, dst, nbytes, vec);
  return cudaGetLastError();
}

cudaError_t launch_score2(const PairSet &ps, const ResultSet &rs, const Scoring &sc, cudaStream_t st) {
  if (ps.n <= 0) return cudaSuccess;
  const int grid = (int)std::min<int64_t>((ps.n + 255) / 256, 4096);
  k_score2<<<grid, 256, 0, st>>>(ps, rs, sc, ps.n);
  return cudaGetLastError();
}

cudaError_t reset_lists(const WorkLists &wl, cudaStream_t st) {
  k_reset_lists<<<1, 1, 0, st>>>(wl);
  return cudaGetLastError();
}

cudaError_t launch_finalize(const ResultSet &rs, int64_t n, bool a_is_query, int part, const OutViews &ov,
                            cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  int grid = (int)std::min<int64_t>((n + 255) / 256, 4096);
  k_finalize<<<grid, 256, 0, st>>>(rs, n, a_is_query, part, ov);
  return cudaGetLastError();
}

cudaError_t launch_pack5(const ResultSet &rs, int64_t n, int32_t *out5, cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  int grid = (int)std::min<int64_t>((n + 255) / 256, 4096);
  k_pack5<<<grid, 256, 0, st>>>(rs, n, out5);
  return cudaGetLastError();
}

}  // namespace mhsw
