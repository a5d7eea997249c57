// mhsw_engine16.cuh -- the packed-int16 wavefront engine used for the forward pass.
//
// Same wavefront as sweep_pair in mhsw_engine.cuh (lane L holds rows [2KL, 2KL+2K) of a
// strip, low halves at column j, high halves at column j-1, lane L two steps behind
// lane L-1), with these changes, which take work off the integer ALU pipe and out of the
// issue slots:
//
//  1. Gap values are kept biased by the gap-open penalty: X^ = X + gO for X in {E, F}.
//     Then X^' = max(X^ - gE, H) uses H directly, and
//       H = max(max(Hdiag + s + gO, E^, F^) - gO, 0)
//     is one 3-way max and one add-max-relu.  Hdiag + s + gO is formed with integer
//     multiply-adds (FMA pipe) from two table words, one per half, each already
//     biased by +gO; this needs s + gO >= 0 for every score (mismatch and ambiguity
//     not above the gap-open penalty), which the driver checks before choosing this
//     engine.  Rows past the end of A score -gO (biased 0); columns outside B read as
//     N (score -ambiguity <= 0).  Cells left of column 0 then stay exactly 0, and every
//     cell right of the last column is at most a real cell of a smaller row, so no
//     value outside the matrix can win the arg-max or raise a false overflow.
//  2. The arg-max is tracked per lane half, not per row: each cell contributes the
//     16-bit key H*2^b + (2^b-1-k) (k = row within the half, b = 3 for up to 8 rows
//     per half, else 4), so the maximum key is the
//     largest score at the smallest row; the half's running key is kept with the step
//     at which it last strictly grew.  Because steps are columns, that step is the
//     first column at which that row reached that score -- the lexicographic rule of
//     SSW (ssw_core.cpp:474-506).  Keys need H < 2^(15-b), so this engine flags pairs
//     whose score reaches the ceiling (at most KeyBits::kCap) for the int32 engine.
//  3. The profile table holds separate low-half and high-half words for the five B
//     codes, loaded as 128-bit vectors: K/4 vectors of low words, K/4 of high words and,
//     when K is 2 mod 4, one vector holding the last two low and the last two high
//     words (every load is a full 128-bit vector, conflict-free across the groups of a
//     warp).  The high words loaded at step t serve the high half at step t+1 (the step
//     loop is unrolled by two so the two word sets alternate registers).
//  4. B codes are read from global memory (each loaded two steps before its use) instead
//     of being staged in shared memory, so a group's shared memory is its profile table only.
//     The sweep runs in three phases: the middle one, where every lane's look-ahead column
//     lies inside B, loads codes without the bounds test and the N substitution, eight
//     steps per loop iteration.
//  5. A lane receives its left neighbour's last-row H and E^ words by two shuffles and
//     takes their high halves with one byte permute each, whose selector is a per-lane
//     register; lane 0 of a pair's first strip, whose row above is the zero boundary,
//     holds a sign-replicate selector instead (H and E^ are never negative, so the
//     replicated sign bytes are zero).
//
// Score2 mode (S2) also produces what SSW's second-best score is computed from
// (ssw_core.cpp:489, :513-536): each A row's maximum of H, over B extended to P columns
// by zero-scoring positions -- SSW pads its striped query to a multiple of 16 (byte
// path) with positions that score 0 (qP_byte, ssw_core.cpp:191), and those reach its
// per-row maxima.  The extra columns lie right of the real ones, so score and end are
// unchanged.  The profile table then has a sixth code (zero score), and each row keeps a
// running maximum over the valid columns (one DPX add-max per row and step).
#pragma once
#include <type_traits>

#include "mhsw_engine.cuh"

namespace mhsw {

constexpr int kCeiling16 = 4000;  // largest score the keyed int16 engine accepts (8 or fewer rows per half)
// Lane groups of the keyed kernels: 8 lanes per pair for A up to 160 rows (K = 4, 6, 8, 10
// rows-pairs per lane), 16 lanes for longer A (K = 6, 8; strips of 256 rows beyond).
constexpr int kGKShort = 8;
constexpr int kGKLong = 16;
constexpr int kShortRows = 160;
__host__ __device__ constexpr int keyed_g_for_rows(int rows) { return rows <= kShortRows ? kGKShort : kGKLong; }
__host__ __device__ constexpr int keyed_k_for_rows(int rows) {
  return rows <= 64 ? 4 : rows <= 96 ? 6 : rows <= 128 ? 8 : rows <= 160 ? 10 : rows <= 192 ? 6 : 8;
}
__host__ __device__ constexpr int keyed_cap(int K) { return K <= 8 ? (1 << 12) - 64 : (1 << 11) - 64; }

constexpr int kCode16Zero = 5;  // score2 mode: SSW's zero-scoring query padding

template <int K, int CODES = kCodeN + 1>
struct Prof16 {
  static_assert(K % 2 == 0, "row pairs per lane must be even");
  static constexpr int kCodes = CODES;        // B codes A, C, G, T, N (outside B reads as N) [, zero]
  static constexpr int kQ = K / 4;            // full vectors of low words (and of high words)
  static constexpr bool kRem = (K % 4) != 0;  // one vector: low K-2, K-1, high K-2, K-1
  static constexpr int kNV = 2 * kQ + (kRem ? 1 : 0);  // 128-bit vectors per (code, lane)
  __host__ __device__ static constexpr size_t bytes(int lanes) { return (size_t)kCodes * kNV * lanes * 16; }
  // vector and element of low word w / high word w
  __host__ __device__ static constexpr int lo_vec(int w) { return w < 4 * kQ ? w / 4 : 2 * kQ; }
  __host__ __device__ static constexpr int lo_elem(int w) { return w < 4 * kQ ? w % 4 : w - 4 * kQ; }
  __host__ __device__ static constexpr int hi_vec(int w) { return w < 4 * kQ ? kQ + w / 4 : 2 * kQ; }
  __host__ __device__ static constexpr int hi_elem(int w) { return w < 4 * kQ ? w % 4 : 2 + w - 4 * kQ; }
};

template <int KMAX, int G, int CODES = kCodeN + 1>
__host__ __device__ constexpr size_t group_prof16_bytes() {
  return Prof16<KMAX, CODES>::bytes(G);
}

// Where score2 mode writes the row maxima (rowmax[row] for the pair's A rows) and the
// number of B columns it sweeps (P >= N; columns [N, P) score 0).
struct RowMaxOut {
  int32_t *rowmax;
  int P;
};

__device__ __forceinline__ uint32_t mad_u32(uint32_t a, uint32_t b, uint32_t c) {
  uint32_t r;
  asm("mad.lo.u32 %0, %1, %2, %3;" : "=r"(r) : "r"(a), "r"(b), "r"(c));
  return r;
}

// PRMT with a selector held in a register; unlike __byte_perm (which reads only the low
// three bits of each selector nibble) it keeps the sign-replicate bit.
__device__ __forceinline__ uint32_t prmt_sel(uint32_t a, uint32_t b, uint32_t sel) {
  uint32_t r;
  asm("prmt.b32 %0, %1, %2, %3;" : "=r"(r) : "r"(a), "r"(b), "r"(sel));
  return r;
}

__device__ __forceinline__ uint32_t sign_mask16(uint32_t x) {
  // each 16-bit half -> 0xffff if its bit 15 is set, else 0 (PRMT sign-replicate mode)
  uint32_t r;
  asm("prmt.b32 %0, %1, %2, 0xBB99;" : "=r"(r) : "r"(x), "r"(0u));
  return r;
}

// One wavefront step of the keyed engine for one lane.  W holds this step's profile
// words (lo words used now), Phi the high words of the previous step; both are
// register arrays of the caller, alternated between steps so no copies are needed.
// Arg-max key of a cell: H << kKeyBits | (kKeyMask - k), k = row within the lane half.
template <int K>
struct KeyBits {
  static constexpr int kBits = K <= 8 ? 3 : 4;
  static constexpr uint32_t kMask = (1u << kBits) - 1u;
  static constexpr int kCap = (1 << (15 - kBits)) - 64;  // largest score a key holds, with margin
};

template <int K, int G, bool S2 = false>
struct Step16 {
  using L = Prof16<K, S2 ? kCode16Zero + 1 : kCodeN + 1>;
  static constexpr uint32_t kKeyMask = KeyBits<K>::kMask;
  // S2: Rm[k] keeps each row's running maximum over valid columns; vmask is 0 in a half
  // whose column is valid at this step and -16384 otherwise (an add-max then ignores it).
  __device__ static __forceinline__ void run(int t, uint32_t zH, uint32_t zE, uint32_t sel, const uint32_t (&Wlo)[K],
                                             const uint32_t (&Phi)[K], uint32_t (&H)[K], uint32_t (&F)[K],
                                             uint32_t &Hlast, uint32_t &Ecout, uint32_t &HtopPrev,
                                             uint32_t &Kl, uint32_t &Jp, uint32_t NGE, uint32_t NGO, uint32_t one,
                                             uint32_t eight, uint32_t (&Rm)[K], uint32_t vmask) {
    uint32_t Ev = prmt_sel(zE, Ecout, sel);  // lo: from the left lane, hi: own lo half
    const uint32_t Htop = prmt_sel(zH, Hlast, sel);
    uint32_t Hd = HtopPrev;
    HtopPrev = Htop;
    uint32_t key[K];
#pragma unroll
    for (int k = 0; k < K; k++) {
      // halves never carry: all terms >= 0, sum < 2^15.  Written as multiply-adds by a
      // runtime 1 so they issue on the FMA pipe, not the integer ALU pipe the DP saturates.
      const uint32_t Q = mad_u32(mad_u32(Hd, one, Wlo[k]), one, Phi[k]);
      const uint32_t m = __vimax3_s16x2(Q, Ev, F[k]);
      const uint32_t Hn = __viaddmax_s16x2_relu(m, NGO, 0u);
      Ev = __viaddmax_s16x2(Ev, NGE, Hn);
      F[k] = __viaddmax_s16x2(F[k], NGE, Hn);
      Hd = H[k];
      H[k] = Hn;
      key[k] = mad_u32(Hn, eight, (uint32_t)(kKeyMask - k) * 0x00010001u);
      if constexpr (S2) Rm[k] = __viaddmax_s16x2(Hn, vmask, Rm[k]);
    }
    // running key per half (keys are non-negative int16): K/2 three-way maxima
    uint32_t Kn = Kl;
#pragma unroll
    for (int k = 0; k < K; k += 2) Kn = __vimax3_s16x2(Kn, key[k], key[k + 1]);
    Hlast = H[K - 1];
    Ecout = Ev;
    // record the step where the running key strictly grows
    const uint32_t msk = sign_mask16(Kn - Kl + 0x7fff7fffu);
    const uint32_t tt = (uint32_t)t * 0x00010001u;
    Jp = (msk & tt) | (~msk & Jp);
    Kl = Kn;
  }
  // Words of code c: low words into Wlo (used at this step), high words into Whi (used
  // at the next step by the high half).
  __device__ static __forceinline__ void load(const uint4 *tab, int c, int lane, uint32_t (&Wlo)[K],
                                              uint32_t (&Whi)[K]) {
    const uint4 *b = tab + c * L::kNV * G + lane;
#pragma unroll
    for (int q = 0; q < L::kQ; q++) {
      const uint4 v = b[q * G];
      Wlo[4 * q + 0] = v.x;
      Wlo[4 * q + 1] = v.y;
      Wlo[4 * q + 2] = v.z;
      Wlo[4 * q + 3] = v.w;
      const uint4 u = b[(L::kQ + q) * G];
      Whi[4 * q + 0] = u.x;
      Whi[4 * q + 1] = u.y;
      Whi[4 * q + 2] = u.z;
      Whi[4 * q + 3] = u.w;
    }
    if constexpr (L::kRem) {
      const uint4 v = b[2 * L::kQ * G];
      Wlo[K - 2] = v.x;
      Wlo[K - 1] = v.y;
      Whi[K - 2] = v.z;
      Whi[K - 1] = v.w;
    }
  }
};

// Forward sweep of one pair with the keyed engine.  B is read directly from its code
// array in global memory (one byte per lane per step, loaded two steps ahead); the
// shared memory of the group holds only the profile table.  A must be a forward view.
template <int K, int G, bool MULTI, bool S2 = false>
__device__ void sweep16_impl(const SeqView &A, const SeqView &B, const Scoring &sc, const GroupSmem &gs, int lane,
                             unsigned gmask, V16::Pay *bnd, int ceiling, SweepOut &out, const RowMaxOut &rmo) {
  using ST = Step16<K, G, S2>;
  using L = typename ST::L;
  constexpr int RS = 2 * K * G;
  constexpr int KB = KeyBits<K>::kBits;
  constexpr uint32_t KMASK = KeyBits<K>::kMask;
  const int M = A.len, N = B.len;
  const uint32_t NGE = V16::splat(-sc.gap_extend);
  const uint32_t NGO = V16::splat(-sc.gap_open);
  const uint8_t *bg = B.base;
  if (ceiling > KeyBits<K>::kCap) ceiling = KeyBits<K>::kCap;

  unsigned long long best = 0ull;
  int overflow = 0;
  const int nstrips = (M + RS - 1) / RS;
  const int NP = S2 ? rmo.P : N;  // columns swept ([N, NP) score 0 in score2 mode)
  const int T_end = NP + 2 * G - 1;
  const uint4 *tab = reinterpret_cast<const uint4 *>(gs.prof);
  // 1 and 2^KB as values the compiler cannot fold (gs.pad is a launch argument >= 0)
  const uint32_t one = (uint32_t)(gs.pad >> 30) + 1u;
  const uint32_t scale = one << KB;

  for (int s = 0; s < nstrips; s++) {
    const int row0 = s * RS + lane * 2 * K;
    __syncwarp(gmask);
    // Profile words: lo word k = s(A[row0+k], c) + gO; hi word k = (s(A[row0+K+k], c) + gO) << 16.
    {
      uint32_t *tw = gs.prof;
      for (int c = 0; c < L::kCodes; c++) {
#pragma unroll
        for (int w = 0; w < K; w++) {
          const int alo = A.code(row0 + w), ahi = A.code(row0 + K + w);
          // the zero code scores 0 against real rows (biased gO); rows past A stay at -gO
          const int slo = (S2 && c == kCode16Zero) ? (alo == kCodePad ? -sc.gap_open : 0) : sub_score(alo, c, sc, sc.gap_open);
          const int shi = (S2 && c == kCode16Zero) ? (ahi == kCodePad ? -sc.gap_open : 0) : sub_score(ahi, c, sc, sc.gap_open);
          const uint32_t vlo = (uint32_t)(slo + sc.gap_open) & 0xffffu;
          const uint32_t vhi = ((uint32_t)(shi + sc.gap_open) & 0xffffu) << 16;
          tw[((c * L::kNV + L::lo_vec(w)) * G + lane) * 4 + L::lo_elem(w)] = vlo;
          tw[((c * L::kNV + L::hi_vec(w)) * G + lane) * 4 + L::hi_elem(w)] = vhi;
        }
      }
    }
    __syncwarp(gmask);

    const bool first_strip = (s == 0);
    const bool last_strip = (s == nstrips - 1);
    uint32_t H[K], F[K], Wlo[K], HA[K], HB[K];
#pragma unroll
    for (int k = 0; k < K; k++) {
      H[k] = 0u;
      F[k] = 0u;  // F^ = F + gO with F = -gO before column 0
    }
#pragma unroll
    for (int w = 0; w < K; w++) HB[w] = 0u;  // hi words before column 0 (biased 0)
    uint32_t Hlast = 0u, Ecout = 0u, HtopPrev = 0u;
    // lane 0 of the first strip reads zeros above: the selector replicates the sign of a
    // top byte of its own (non-negative) H and E^ words; other lanes take the left lane's hi halves
    const uint32_t sel = (lane == 0 && first_strip) ? 0x54BBu : 0x5432u;
    uint32_t Kl = 0u;    // running key per half
    uint32_t Jp = 0u;    // step of the last strict increase of Kl, per half
    uint32_t Rm[K];      // score2 mode: running row maxima over valid columns
#pragma unroll
    for (int k = 0; k < K; k++) Rm[k] = 0u;
    const int j0 = -2 * lane;  // lo column at step 0
    auto code_at = [&](int j) -> int {
      if ((unsigned)j < (unsigned)N) return (int)bg[j];
      return (S2 && (unsigned)j < (unsigned)NP) ? kCode16Zero : kCodeN;
    };
    // score2 mode: 0 in a half whose column is inside [0, NP) at step t, else -16384
    auto vmask_at = [&](int t) -> uint32_t {
      if constexpr (!S2) return 0u;
      const int jl = t + j0;
      const uint32_t lo = (unsigned)jl < (unsigned)NP ? 0u : 0x0000C000u;
      const uint32_t hi = (unsigned)(jl - 1) < (unsigned)NP ? 0u : 0xC0000000u;
      return lo | hi;
    };
    // codes of the even and odd steps, each loaded two steps before its use
    int ceven = code_at(j0), codd = code_at(j0 + 1);

    // the left lane's H of its hi-last row and E^ below it (hi halves); lane 0 of a later
    // strip reads them from the boundary row (lo: H, hi: E^), zero past column NP
    auto top = [&](int t, uint32_t &zH, uint32_t &zE) {
      zH = __shfl_up_sync(gmask, Hlast, 1, G);
      zE = __shfl_up_sync(gmask, Ecout, 1, G);
      if (MULTI && lane == 0 && !first_strip) {
        const uint32_t b = t < NP ? bnd[t] : 0u;
        zH = __byte_perm(b, 0u, 0x1000);
        zE = b;
      }
    };
    auto out_bnd = [&](int t) {
      if (MULTI && !last_strip && lane == G - 1) {
        const int jh = t - 2 * lane - 1;  // hi-half column of the last lane
        if (jh >= 0 && jh < NP) bnd[jh] = __byte_perm(Hlast, Ecout, 0x7632);
      }
    };
    int t = 0;
    const uint8_t *bl = bg + j0;
    // Two steps; `guarded` (std::true_type / std::false_type) says whether the look-ahead
    // codes need the bounds test.
    auto two_steps = [&](auto guarded) {
      constexpr bool kGuard = decltype(guarded)::value;
      // even step: hi words into HA; the high half uses HB (previous column)
      int c = ceven;
      ceven = kGuard ? code_at(t + 2 + j0) : (int)bl[t + 2];
      ST::load(tab, c, lane, Wlo, HA);
      uint32_t zH, zE;
      top(t, zH, zE);
      ST::run(t, zH, zE, sel, Wlo, HB, H, F, Hlast, Ecout, HtopPrev, Kl, Jp, NGE, NGO, one, scale, Rm, vmask_at(t));
      out_bnd(t);
      // odd step: hi words into HB; the high half uses HA
      c = codd;
      codd = kGuard ? code_at(t + 3 + j0) : (int)bl[t + 3];
      ST::load(tab, c, lane, Wlo, HB);
      top(t + 1, zH, zE);
      ST::run(t + 1, zH, zE, sel, Wlo, HA, H, F, Hlast, Ecout, HtopPrev, Kl, Jp, NGE, NGO, one, scale, Rm,
              vmask_at(t + 1));
      out_bnd(t + 1);
    };
    // The look-ahead columns t+2+j0 and t+3+j0 lie in [0, N) for every lane of the group
    // (j0 = -2 lane, lane < G) when 2G-4 <= t <= N-4.
    const int tm0 = 2 * G - 4, tm1 = N - 3;
    for (; t + 1 < T_end && t < tm0; t += 2) two_steps(std::true_type{});
    // eight steps per iteration in the middle phase (the loop's own instructions and the
    // register moves at its back edge are paid once per eight steps); its last few steps
    // go to the guarded drain loop, which keeps one copy of the step code fewer
    for (; t + 6 < tm1;) {
#pragma unroll
      for (int u = 0; u < 4; u++) {
        two_steps(std::false_type{});
        t += 2;
      }
    }
    for (; t + 1 < T_end; t += 2) two_steps(std::true_type{});
    if (t < T_end) {
      ST::load(tab, ceven, lane, Wlo, HA);
      uint32_t zH, zE;
      top(t, zH, zE);
      ST::run(t, zH, zE, sel, Wlo, HB, H, F, Hlast, Ecout, HtopPrev, Kl, Jp, NGE, NGO, one, scale, Rm, vmask_at(t));
      out_bnd(t);
    }

    if constexpr (S2) {
#pragma unroll
      for (int k = 0; k < K; k++) {
        const int rl = row0 + k, rh = row0 + K + k;
        if (rl < M) rmo.rowmax[rl] = (int32_t)(Rm[k] & 0xffffu);
        if (rh < M) rmo.rowmax[rh] = (int32_t)(Rm[k] >> 16);
      }
    }
    // Decode the two halves' keys into (value, row, column) and reduce over the group.
    unsigned long long kbest = 0ull;
    int vmax_lane = 0;
#pragma unroll
    for (int half = 0; half < 2; half++) {
      const uint32_t key = half ? (Kl >> 16) : (Kl & 0xffffu);
      const int v = (int)(key >> KB);
      const int k = (int)KMASK - (int)(key & KMASK);
      const int r = row0 + (half ? K : 0) + k;
      const int jstep = (int)(half ? (Jp >> 16) : (Jp & 0xffffu));
      const int col = jstep - 2 * lane - half;
      if (v > vmax_lane) vmax_lane = v;  // every key counts for the overflow test (PAD rows included)
      if (v > 0 && r < M) {
        const unsigned long long kk = best_key(v, r, col);
        if (kk > kbest) kbest = kk;
      }
    }
    if (vmax_lane > ceiling) overflow = 1;
#pragma unroll
    for (int o = G / 2; o > 0; o >>= 1) {
      const unsigned long long other = __shfl_xor_sync(gmask, kbest, o, G);
      kbest = other > kbest ? other : kbest;
      overflow |= __shfl_xor_sync(gmask, overflow, o, G);
    }
    if (kbest > best) best = kbest;
    __syncwarp(gmask);
  }
  out.key = best;
  out.overflow = overflow;
}

template <int K, int G, bool S2 = false>
__device__ __forceinline__ void sweep16(const SeqView &A, const SeqView &B, const Scoring &sc, const GroupSmem &gs,
                                        int lane, unsigned gmask, V16::Pay *bnd, int ceiling, SweepOut &out,
                                        const RowMaxOut &rmo = RowMaxOut{nullptr, 0}) {
  if (A.len > 2 * K * G)
    sweep16_impl<K, G, true, S2>(A, B, sc, gs, lane, gmask, bnd, ceiling, out, rmo);
  else
    sweep16_impl<K, G, false, S2>(A, B, sc, gs, lane, gmask, bnd, ceiling, out, rmo);
}

}  // namespace mhsw
