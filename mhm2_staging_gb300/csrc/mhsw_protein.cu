// mhsw_protein.cu -- protein Smith-Waterman (include/mhsw.h: mhsw_align_protein).
//
// The reference declares protein kernels (src/adept-sw/kernel.cpp:510-899,
// sequence_aa_kernel / sequence_aa_reverse: score and ends, then begins, with a 24 x 24
// scoring matrix and a 91-entry ASCII encoding from the caller) that nothing in MHM2
// launches.  This path computes the same outputs with SSW's result rules, as the DNA
// path does: score = max H of the local affine recurrence (E and F opened at gap_open,
// extended at gap_extend), end = the lexicographically smallest (A row, B column) holding
// it, begin = the same rule on the reversed prefixes A[0..a_end], B[0..b_end].
//
// GB300 mapping: one warp per pair, lanes along A (K rows a lane, 32K rows a strip), B's
// columns swept as a skewed wavefront -- lane l works on column t - l at step t and hands
// its bottom row's H and E to lane l + 1 by shuffle; strips hand their last row to the next
// through a per-warp global row.  int32 cells with DPX add-max / 3-way relu-max; the
// scoring matrix sits in shared memory, indexed by the row's code * 24 + the column's code.
// The begin pass is the same kernel on reversed views of the prefixes ending at the ends.
#include <algorithm>
#include <cstdint>
#include <cstring>
#include <vector>

#include "../../include/mhsw.h"
#include "mhsw_internal.h"
#include "mhsw_launch.h"
#include "mhsw_types.h"

namespace {

constexpr int kAA = 24;              // matrix dimension
constexpr int kEnc = 91;             // encoding entries (bytes 0..90)
constexpr int kPK = 8;               // rows per lane
constexpr int kPRows = 32 * kPK;     // rows per strip
constexpr int kNegBig = -(1 << 28);  // "minus infinity" for E and F at the borders

// bytes -> codes (0..23); any byte >= 91 or encoded outside [0, 24) sets *bad and gets 0
__global__ void k_protein_encode(const char *__restrict__ src, uint8_t *__restrict__ dst, int64_t nbytes,
                                 const int16_t *__restrict__ enc, int *bad) {
  __shared__ int16_t senc[kEnc];
  for (int k = threadIdx.x; k < kEnc; k += blockDim.x) senc[k] = enc[k];
  __syncthreads();
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nbytes; i += (int64_t)gridDim.x * blockDim.x) {
    const unsigned char c = (unsigned char)src[i];
    int v = c < kEnc ? senc[c] : -1;
    if (v < 0 || v >= kAA) {
      atomicOr(bad, 1);
      v = 0;
    }
    dst[i] = (uint8_t)v;
  }
}

struct PArgs {
  const uint8_t *a_code, *b_code;
  const int64_t *a_off, *b_off;
  const int32_t *a_len, *b_len;
  int64_t n;
  const int32_t *mat;  // 24 x 24
  int gO, gE;
  int32_t *score, *a_end, *b_end;  // forward: written; reverse: read (the prefixes) and
  int32_t *a_beg, *b_beg;          // begins written
  int2 *rows;                      // per warp slot: H, E of a strip's last row (max_n each)
  int64_t max_n;
};

// One pass: forward (REV = false) over the whole pairs, or the begin pass (REV = true)
// over the reversed prefixes that end at each pair's end.
template <bool REV>
__global__ void __launch_bounds__(128) k_protein(PArgs g) {
  __shared__ int32_t smat[kAA * kAA];
  for (int k = threadIdx.x; k < kAA * kAA; k += blockDim.x) smat[k] = g.mat[k];
  __syncthreads();
  const int lane = threadIdx.x & 31;
  const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  int2 *bound = g.rows + warp * g.max_n;
  const int gO = g.gO, gE = g.gE;
  for (int64_t p = warp; p < g.n; p += nwarps) {
    int M, N;
    const uint8_t *A = g.a_code + g.a_off[p], *B = g.b_code + g.b_off[p];
    int ie = 0, je = 0;
    if (REV) {
      if (g.score[p] <= 0) {  // score 0: begins as SSW reports them
        if (lane == 0) {
          g.a_beg[p] = -1;
          g.b_beg[p] = 0;
        }
        continue;
      }
      ie = g.a_end[p];
      je = g.b_end[p];
      M = ie + 1;
      N = je + 1;
    } else {
      M = g.a_len[p];
      N = g.b_len[p];
    }
    // codes of the pass: reversed prefixes for the begin pass
    auto acode = [&](int i) -> int { return REV ? A[ie - i] : A[i]; };
    auto bcode = [&](int j) -> int { return REV ? B[je - j] : B[j]; };
    int best = 0, bi = -1, bj = 0;  // running best over the strips done (warp-uniform)
    if (M > 0 && N > 0) {
      const int nstrips = (M + kPRows - 1) / kPRows;
      for (int s = 0; s < nstrips; s++) {
        const int row0 = s * kPRows + lane * kPK;
        int a24[kPK], Hl[kPK], Fl[kPK], rb[kPK], rj[kPK];
#pragma unroll
        for (int k = 0; k < kPK; k++) {
          const int r = row0 + k;
          a24[k] = r < M ? acode(r) * kAA : 0;
          Hl[k] = 0;
          Fl[k] = kNegBig;
          rb[k] = 0;
          rj[k] = 0;
        }
        int recvH = 0, recvE = kNegBig, prevH = 0;  // from the row above: this column, and the last
        int sendH = 0, sendE = kNegBig;
        const bool last_strip = s == nstrips - 1;
        const int steps = N + 31;
        // four steps per loop iteration (the loop's own instructions and register moves
        // are paid once per four steps: ~7% on 100-500-residue pairs)
#pragma unroll 4
        for (int t = 0; t < steps; t++) {
          // what lane l - 1 computed at t - 1 (its bottom row, column t - l)
          const int upH = __shfl_up_sync(0xffffffffu, sendH, 1);
          const int upE = __shfl_up_sync(0xffffffffu, sendE, 1);
          const int j = t - lane;
          prevH = recvH;
          if (lane == 0) {
            if (s == 0 || j >= N) {
              recvH = 0;
              recvE = kNegBig;
            } else {
              const int2 v = bound[j];
              recvH = v.x;
              recvE = v.y;
            }
          } else {
            recvH = upH;
            recvE = upE;
          }
          sendH = 0;
          sendE = kNegBig;
          if (j >= 0 && j < N) {
            const int b = bcode(j);
            int hu = recvH, eu = recvE, hd = prevH;
#pragma unroll
            for (int k = 0; k < kPK; k++) {
              const int e = __viaddmax_s32(eu, -gE, hu - gO);      // E(r, j)
              const int f = __viaddmax_s32(Fl[k], -gE, Hl[k] - gO);  // F(r, j)
              const int h = __vimax3_s32_relu(hd + smat[a24[k] + b], e, f);
              hd = Hl[k];  // H(r, j - 1): the next row's diagonal
              Hl[k] = h;
              Fl[k] = f;
              hu = h;
              eu = e;
              if (h > rb[k]) {  // first column of the row's maximum
                rb[k] = h;
                rj[k] = j;
              }
            }
            sendH = hu;
            sendE = eu;
            if (lane == 31 && !last_strip) bound[j] = make_int2(hu, eu);
          }
        }
        __syncwarp();
        // the strip's best: largest value, then smallest row (rows grow with lane and k)
        int lb = 0, li = -1, lj = 0;
#pragma unroll
        for (int k = 0; k < kPK; k++) {
          if (row0 + k < M && rb[k] > lb) {
            lb = rb[k];
            li = row0 + k;
            lj = rj[k];
          }
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
          const int ob = __shfl_down_sync(0xffffffffu, lb, o);
          const int oi = __shfl_down_sync(0xffffffffu, li, o);
          const int oj = __shfl_down_sync(0xffffffffu, lj, o);
          if (lane + o < 32 && (ob > lb || (ob == lb && ob > 0 && (li < 0 || oi < li)))) {
            lb = ob;
            li = oi;
            lj = oj;
          }
        }
        lb = __shfl_sync(0xffffffffu, lb, 0);
        li = __shfl_sync(0xffffffffu, li, 0);
        lj = __shfl_sync(0xffffffffu, lj, 0);
        if (lb > best) {  // a later strip replaces only with a strictly larger score
          best = lb;
          bi = li;
          bj = lj;
        }
      }
    }
    if (lane == 0) {
      if (!REV) {
        g.score[p] = best;
        g.a_end[p] = best > 0 ? bi : -1;
        g.b_end[p] = best > 0 ? bj : 0;
      } else {
        g.a_beg[p] = ie - bi;
        g.b_beg[p] = je - bj;
      }
    }
  }
}

__global__ void k_protein_pack(const int32_t *score, const int32_t *a_beg, const int32_t *a_end, const int32_t *b_beg,
                               const int32_t *b_end, int64_t n, int32_t *out5) {
  const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  out5[5 * p + 0] = score[p];
  out5[5 * p + 1] = a_beg[p];
  out5[5 * p + 2] = a_end[p];
  out5[5 * p + 3] = b_beg[p];
  out5[5 * p + 4] = b_end[p];
}

}  // namespace

extern "C" {

int mhsw_align_protein(mhsw_driver *d, const mhsw_pairs *pairs, const int16_t *scoring_matrix,
                       const int16_t *encoding, int32_t *out5, int host_io) {
  if (!d || !pairs || !scoring_matrix || !encoding || pairs->n < 0 || (pairs->n > 0 && !out5)) return MHSW_ERR_ARG;
  const int64_t n = pairs->n;
  if (n == 0) return MHSW_OK;
  const int dev = mhsw::driver_device(d);
  if (dev < 0) return MHSW_ERR_STATE;
  for (int k = 0; k < kEnc; k++)
    if (encoding[k] < 0 || encoding[k] >= kAA) return MHSW_ERR_ARG;
  std::lock_guard<std::mutex> call_lk(mhsw::driver_call_mutex(d));
  cudaSetDevice(dev);
  cudaStream_t st = static_cast<cudaStream_t>(mhsw::driver_stream(d));
  int gO = 0, gE = 0;
  mhsw::driver_gaps(d, &gO, &gE);
  // extents: host batches are scanned here; device batches read their lengths back
  std::vector<int32_t> la((size_t)n), lb((size_t)n);
  std::vector<int64_t> oa((size_t)n), ob((size_t)n);
  cudaError_t e = cudaSuccess;
  if (host_io) {
    std::memcpy(la.data(), pairs->a_len, sizeof(int32_t) * n);
    std::memcpy(lb.data(), pairs->b_len, sizeof(int32_t) * n);
    std::memcpy(oa.data(), pairs->a_off, sizeof(int64_t) * n);
    std::memcpy(ob.data(), pairs->b_off, sizeof(int64_t) * n);
  } else {
    e = cudaMemcpyAsync(la.data(), pairs->a_len, sizeof(int32_t) * n, cudaMemcpyDeviceToHost, st);
    if (!e) e = cudaMemcpyAsync(lb.data(), pairs->b_len, sizeof(int32_t) * n, cudaMemcpyDeviceToHost, st);
    if (!e) e = cudaMemcpyAsync(oa.data(), pairs->a_off, sizeof(int64_t) * n, cudaMemcpyDeviceToHost, st);
    if (!e) e = cudaMemcpyAsync(ob.data(), pairs->b_off, sizeof(int64_t) * n, cudaMemcpyDeviceToHost, st);
    if (!e) e = cudaStreamSynchronize(st);
    if (e) return MHSW_ERR_CUDA;
  }
  int64_t ta = 0, tb = 0, max_n = 1;
  for (int64_t i = 0; i < n; i++) {
    if (la[(size_t)i] < 0 || lb[(size_t)i] < 0 || oa[(size_t)i] < 0 || ob[(size_t)i] < 0) return MHSW_ERR_ARG;
    ta = std::max(ta, oa[(size_t)i] + la[(size_t)i]);
    tb = std::max(tb, ob[(size_t)i] + lb[(size_t)i]);
    max_n = std::max<int64_t>(max_n, lb[(size_t)i]);
  }
  char *as = nullptr, *bs = nullptr;
  int64_t *ao = nullptr, *bo = nullptr;
  int32_t *al = nullptr, *bl = nullptr;
  uint8_t *ac = nullptr, *bc = nullptr;
  int16_t *enc = nullptr;
  int32_t *mat = nullptr, *sc = nullptr, *ae = nullptr, *be = nullptr, *ab = nullptr, *bb = nullptr, *o5 = nullptr;
  int *bad = nullptr;
  int2 *rows = nullptr;
  int sms = 152;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  // one warp per pair at a time; 24 resident warps per SM (76 registers x 128 threads
  // fits 6 blocks of 4 warps) to cover the row chain's latency
  const int64_t warps = std::min<int64_t>(n, (int64_t)sms * 24);
  // the call's arrays, laid out in the handle's call arena (sized by a first pass)
  auto lay = [&](mhsw::Carve &c) {
    if (host_io) {
      c.take(&as, (size_t)ta + 16);
      c.take(&bs, (size_t)tb + 16);
      c.take(&ao, (size_t)n);
      c.take(&bo, (size_t)n);
      c.take(&al, (size_t)n);
      c.take(&bl, (size_t)n);
      c.take(&o5, (size_t)n * 5);
    }
    c.take(&ac, (size_t)ta + 16);
    c.take(&bc, (size_t)tb + 16);
    c.take(&enc, kEnc);
    c.take(&mat, kAA * kAA);
    c.take(&sc, (size_t)n);
    c.take(&ae, (size_t)n);
    c.take(&be, (size_t)n);
    c.take(&ab, (size_t)n);
    c.take(&bb, (size_t)n);
    c.take(&bad, 1);
    c.take(&rows, (size_t)(warps * max_n));
  };
  mhsw::Carve sizing;
  lay(sizing);
  mhsw::Carve arena{0, mhsw::driver_call_arena(d, sizing.off)};
  if (!arena.base) return MHSW_ERR_NOMEM;
  lay(arena);
  if (host_io) {
    auto up = [&](void *dst, const void *src, size_t bytes) {
      if (!e && bytes) e = cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, st);
    };
    up(as, pairs->a_seq, (size_t)ta);
    up(bs, pairs->b_seq, (size_t)tb);
    up(ao, pairs->a_off, sizeof(int64_t) * n);
    up(bo, pairs->b_off, sizeof(int64_t) * n);
    up(al, pairs->a_len, sizeof(int32_t) * n);
    up(bl, pairs->b_len, sizeof(int32_t) * n);
  } else {
    as = const_cast<char *>(pairs->a_seq);
    bs = const_cast<char *>(pairs->b_seq);
    ao = const_cast<int64_t *>(pairs->a_off);
    bo = const_cast<int64_t *>(pairs->b_off);
    al = const_cast<int32_t *>(pairs->a_len);
    bl = const_cast<int32_t *>(pairs->b_len);
    o5 = out5;
  }
  int32_t hmat[kAA * kAA];
  for (int k = 0; k < kAA * kAA; k++) hmat[k] = scoring_matrix[k];
  if (!e) e = cudaMemcpyAsync(mat, hmat, sizeof(hmat), cudaMemcpyHostToDevice, st);
  if (!e) e = cudaMemcpyAsync(enc, encoding, sizeof(int16_t) * kEnc, cudaMemcpyHostToDevice, st);
  if (!e) e = cudaMemsetAsync(bad, 0, sizeof(int), st);
  if (!e) {
    k_protein_encode<<<(unsigned)std::max<int64_t>(1, std::min<int64_t>((ta + 255) / 256, 4096)), 256, 0, st>>>(
        as, ac, ta, enc, bad);
    k_protein_encode<<<(unsigned)std::max<int64_t>(1, std::min<int64_t>((tb + 255) / 256, 4096)), 256, 0, st>>>(
        bs, bc, tb, enc, bad);
    e = cudaGetLastError();
  }
  if (!e) {
    PArgs g{ac, bc, ao, bo, al, bl, n, mat, gO, gE, sc, ae, be, ab, bb, rows, max_n};
    const unsigned blocks = (unsigned)((warps * 32 + 127) / 128);
    k_protein<false><<<blocks, 128, 0, st>>>(g);
    k_protein<true><<<blocks, 128, 0, st>>>(g);
    k_protein_pack<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(sc, ab, ae, bb, be, n, o5);
    e = cudaGetLastError();
  }
  if (!e && host_io) e = cudaMemcpyAsync(out5, o5, sizeof(int32_t) * 5 * n, cudaMemcpyDeviceToHost, st);
  int hbad = 0;
  if (!e) e = cudaMemcpyAsync(&hbad, bad, sizeof(int), cudaMemcpyDeviceToHost, st);
  if (!e) e = cudaStreamSynchronize(st);
  if (e) cudaStreamSynchronize(st);  // nothing of a failed call left in flight
  if (e) return e == cudaErrorMemoryAllocation ? MHSW_ERR_NOMEM : MHSW_ERR_CUDA;
  return hbad ? MHSW_ERR_ARG : MHSW_OK;
}

}  // extern "C"
