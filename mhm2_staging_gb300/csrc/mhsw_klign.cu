// mhsw_klign.cu -- klign's caller side on the device (include/mhsw.h: mhsw_contigs_*,
// mhsw_klign_align).
//
// klign turns every seed hit into a candidate (read, contig window) and decides per
// candidate whether it needs an alignment at all (src/klign.cpp:218-241, :670-739); the
// aligner's results are then mapped into its Aln records (:260-266, :369-381).  Here all
// of it runs on the device against a resident contig set:
//   k_klign_prepare   one warp per candidate: orientation and the mirrored seed
//                     position, the diagonal window clipped to the contig, the oriented
//                     read written (reverse complement for '-'), the raw-byte perfect-
//                     match compare 32 bytes at a time; candidates that need an
//                     alignment are appended to a compacted pair list (window = offset
//                     into the resident contig codes, no copy; one list reservation per
//                     block and round) with the batch's longest read and window;
//   alignment         the driver's resident-batch path (forward + begin pass, score2 when
//                     the driver is in score2 mode) over the compacted list;
//   k_klign_finish    one thread per candidate: klign's Aln fields from either the
//                     shortcut or the alignment, switch_orient for '-', identity.
// The host synchronises once between the two kernels (the list's length and longest
// sequences size the alignment launch).
#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <string>
#include <vector>

#include "../../include/mhsw.h"
#include "mhsw_internal.h"
#include "mhsw_launch.h"
#include "mhsw_types.h"

struct mhsw_contigs {
  int device = 0;
  char *raw = nullptr;       // contig bytes (device), kept for the raw perfect-match compare
  uint8_t *codes = nullptr;  // contig codes (device)
  int64_t *off = nullptr;    // device
  int32_t *len = nullptr;    // device
  int64_t count = 0, bytes = 0;
  std::vector<int64_t> h_off;  // host copies for argument checks
  std::vector<int32_t> h_len;
};

namespace {

// utils.cpp revcomp: complement of an upper-case base, IUPAC codes to N, -1 for any other
// byte (revcomp dies on it).
__device__ __forceinline__ int comp_base(unsigned char c) {
  switch (c) {
    case 'A': return 'T';
    case 'C': return 'G';
    case 'G': return 'C';
    case 'T': return 'A';
    case 'N':
    case 'U':
    case 'R':
    case 'Y':
    case 'K':
    case 'M':
    case 'S':
    case 'W':
    case 'B':
    case 'D':
    case 'H':
    case 'V': return 'N';
    default: return -1;
  }
}

struct KArgs {
  // candidates (device)
  const char *read;
  const int64_t *read_off;
  const int32_t *read_len;
  const int32_t *cid, *pic, *pir;
  const uint8_t *strand;
  int64_t n;
  int kmer_len;
  // contigs (device)
  const char *craw;
  const int64_t *coff;
  const int32_t *clen;
  // per candidate state
  char *ori;         // oriented reads, at the candidates' read offsets
  int32_t *wstart;   // window start in the contig
  int32_t *rstart0;  // read start of the overlap (after orientation)
  int32_t *overlap;
  int8_t *orient;    // '+' / '-'
  int32_t *slot;     // index in the aligned list, -1 for a perfect match
  // aligned list
  int64_t *a_off, *b_off;
  int32_t *a_len, *b_len;
  int *counts;       // [0] list length, [1] longest read, [2] longest window, [3] bad reads
};

// One warp per candidate, kPrepWarps candidates per block per round: the warp's lanes
// stride the read and the window 32 bytes at a time (coalesced), the perfect-match compare
// stops at the first round with a differing byte (a warp vote), and the block reserves its
// aligned candidates' list slots with one atomic per round; the longest read and window
// and the bad-read flag are reduced per block.
constexpr int kPrepWarps = 8;

__global__ void __launch_bounds__(kPrepWarps * 32) k_klign_prepare(KArgs g) {
  __shared__ int s_need[kPrepWarps];
  __shared__ int s_base;
  __shared__ int s_max[3][kPrepWarps];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const unsigned full = 0xffffffffu;
  const int K = g.kmer_len;
  int rmax = 0, omax = 0, nbad = 0;  // this warp's, kept by every lane
  for (int64_t base = (int64_t)blockIdx.x * kPrepWarps; base < g.n; base += (int64_t)gridDim.x * kPrepWarps) {
    const int64_t c = base + warp;
    bool need = false;
    int64_t ro = 0, boff = 0;
    int rlen = 0, ov = 0;
    if (c < g.n) {
      rlen = g.read_len[c];
      ro = g.read_off[c];
      const char *r = g.read + ro;
      const int id = g.cid[c];
      const bool minus = ((g.strand[c] >> 1) & 1u) != (g.strand[c] & 1u);
      // the oriented read (klign reverse-complements every read up front, :673)
      bool bad = false;
      for (int t = lane; t < rlen; t += 32) {
        const int cc = comp_base((unsigned char)r[rlen - 1 - t]);
        bad |= cc < 0;
        g.ori[ro + t] = minus ? (char)cc : r[t];
      }
      if (__any_sync(full, bad)) nbad = 1;
      const int pos_in_read = minus ? rlen - (K + g.pir[c]) : g.pir[c];
      const int pos_in_ctg = g.pic[c];
      const int cl = g.clen[id];
      const int left = min(pos_in_read, pos_in_ctg);
      const int right = min(rlen - K - pos_in_read, cl - pos_in_ctg - K);
      const int cstart = pos_in_ctg - left, rstart = pos_in_read - left;
      ov = left + K + right;
      boff = g.coff[id] + cstart;
      if (lane == 0) {
        g.wstart[c] = cstart;
        g.rstart0[c] = rstart;
        g.overlap[c] = ov;
        g.orient[c] = minus ? '-' : '+';
      }
      // perfect match: the window's bytes equal the oriented read's overlap (:220)
      const char *cw = g.craw + boff;
      for (int t0 = 0; t0 < ov; t0 += 32) {
        const int t = t0 + lane;
        bool ok = true;
        if (t < ov) {
          const char rb = minus ? (char)comp_base((unsigned char)r[rlen - 1 - (rstart + t)]) : r[rstart + t];
          ok = cw[t] == rb;
        }
        if (!__all_sync(full, ok)) {
          need = true;
          break;
        }
      }
      if (need) {
        rmax = max(rmax, rlen);
        omax = max(omax, ov);
      } else if (lane == 0) {
        g.slot[c] = -1;
      }
    }
    if (lane == 0) s_need[warp] = need ? 1 : 0;
    __syncthreads();
    if (threadIdx.x == 0) {
      int tot = 0;
      for (int w = 0; w < kPrepWarps; w++) tot += s_need[w];
      s_base = tot ? atomicAdd(&g.counts[0], tot) : 0;
    }
    __syncthreads();
    if (need && lane == 0) {
      int at = s_base;
      for (int w = 0; w < warp; w++) at += s_need[w];
      g.slot[c] = at;
      g.a_off[at] = ro;  // the whole oriented read (:708)
      g.a_len[at] = rlen;
      g.b_off[at] = boff;
      g.b_len[at] = ov;
    }
    __syncthreads();  // s_need and s_base are rewritten next round
  }
  if (lane == 0) {
    s_max[0][warp] = rmax;
    s_max[1][warp] = omax;
    s_max[2][warp] = nbad;
  }
  __syncthreads();
  if (threadIdx.x < 3) {
    int m = 0;
    for (int w = 0; w < kPrepWarps; w++) m = max(m, s_max[threadIdx.x][w]);
    if (threadIdx.x == 2) {
      if (m) atomicAdd(&g.counts[3], 1);
    } else if (m) {
      atomicMax(&g.counts[1 + threadIdx.x], m);
    }
  }
}

struct FArgs {
  const int32_t *read_len;
  const int32_t *wstart, *rstart0, *overlap, *slot;
  const int8_t *orient;
  const int32_t *out5;    // aligned list: score, a_begin, a_end, b_begin, b_end
  const int32_t *score2;  // aligned list, or null
  int match;
  int64_t n;
  int32_t *rstart, *rstop, *cstart, *cstop, *score1, *s2, *identity;
  char *orient_out;
  uint8_t *perfect;
};

__global__ void k_klign_finish(FArgs g) {
  const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= g.n) return;
  const int rlen = g.read_len[c], j = g.slot[c];
  int rs, re, cs, ce, sc, s2 = 0;
  if (j < 0) {  // :221-225
    const int ov = g.overlap[c];
    rs = g.rstart0[c];
    re = rs + ov;
    cs = g.wstart[c];
    ce = cs + ov;
    sc = ov * g.match;
  } else {  // :260-263 (CPU path), :372-375 (GPU path)
    const int32_t *o = g.out5 + 5 * (int64_t)j;
    sc = o[0];
    rs = o[1];
    re = o[2] + 1;
    cs = g.wstart[c] + o[3];
    ce = g.wstart[c] + o[4] + 1;
    if (g.score2) s2 = g.score2[j];
  }
  if (g.orient[c] == '-') {  // utils.cpp switch_orient
    const int t = rs;
    rs = rlen - re;
    re = rlen - t;
  }
  g.rstart[c] = rs;
  g.rstop[c] = re;
  g.cstart[c] = cs;
  g.cstop[c] = ce;
  g.score1[c] = sc;
  g.s2[c] = s2;
  g.identity[c] = 100 * sc / g.match / rlen;  // :226, :266
  g.orient_out[c] = (char)g.orient[c];
  g.perfect[c] = j < 0;
}


}  // namespace

extern "C" {

int mhsw_contigs_create(int device, const char *seq, const int64_t *off, const int32_t *len, int64_t count,
                        mhsw_contigs **out) {
  if (!out || count < 0 || (count > 0 && (!seq || !off || !len))) return MHSW_ERR_ARG;
  *out = nullptr;
  int64_t total = 0;
  for (int64_t i = 0; i < count; i++) {
    if (len[i] < 0 || off[i] < 0) return MHSW_ERR_ARG;
    total = std::max(total, off[i] + len[i]);
  }
  if (cudaSetDevice(device) != cudaSuccess) return MHSW_ERR_CUDA;
  mhsw_contigs *c = new mhsw_contigs;
  c->device = device;
  c->count = count;
  c->bytes = total;
  c->h_off.assign(off, off + count);
  c->h_len.assign(len, len + count);
  cudaError_t e = cudaMalloc(&c->raw, (size_t)total + 16);
  if (!e) e = cudaMalloc(&c->codes, (size_t)total + 16);
  if (!e) e = cudaMalloc(&c->off, sizeof(int64_t) * (size_t)std::max<int64_t>(count, 1));
  if (!e) e = cudaMalloc(&c->len, sizeof(int32_t) * (size_t)std::max<int64_t>(count, 1));
  if (!e && total > 0) e = cudaMemcpy(c->raw, seq, (size_t)total, cudaMemcpyHostToDevice);
  if (!e && count > 0) e = cudaMemcpy(c->off, off, sizeof(int64_t) * count, cudaMemcpyHostToDevice);
  if (!e && count > 0) e = cudaMemcpy(c->len, len, sizeof(int32_t) * count, cudaMemcpyHostToDevice);
  if (!e && total > 0) e = mhsw::launch_translate(c->raw, c->codes, total, nullptr);
  if (!e) e = cudaDeviceSynchronize();
  if (e) {
    mhsw_contigs_destroy(c);
    return e == cudaErrorMemoryAllocation ? MHSW_ERR_NOMEM : MHSW_ERR_CUDA;
  }
  *out = c;
  return MHSW_OK;
}

void mhsw_contigs_destroy(mhsw_contigs *c) {
  if (!c) return;
  cudaSetDevice(c->device);
  cudaFree(c->raw);
  cudaFree(c->codes);
  cudaFree(c->off);
  cudaFree(c->len);
  delete c;
}

int mhsw_klign_align(mhsw_driver *d, const mhsw_contigs *cg, const mhsw_candidates *cand, mhsw_alns *out,
                     int64_t *n_aligned) {
  if (!d || !cg || !cand || !out) return MHSW_ERR_ARG;
  const int64_t n = cand->n;
  if (n_aligned) *n_aligned = 0;
  if (n < 0 || cand->kmer_len <= 0) return MHSW_ERR_ARG;
  if (n == 0) return MHSW_OK;
  if (!cand->read_seq || !cand->read_off || !cand->read_len || !cand->contig_id || !cand->pos_in_ctg ||
      !cand->pos_in_read || !cand->strand || !out->rstart || !out->rstop || !out->cstart || !out->cstop ||
      !out->score1 || !out->score2 || !out->identity || !out->orient || !out->perfect)
    return MHSW_ERR_ARG;
  if (mhsw::driver_device(d) != cg->device) return MHSW_ERR_ARG;
  // argument checks as klign's asserts (:705-706): the seed inside read and contig
  const int K = cand->kmer_len;
  int64_t rbytes = 0;
  for (int64_t i = 0; i < n; i++) {
    const int32_t rl = cand->read_len[i], id = cand->contig_id[i];
    if (rl < K || cand->read_off[i] < 0 || id < 0 || id >= cg->count) return MHSW_ERR_ARG;
    if (cand->pos_in_read[i] < 0 || cand->pos_in_read[i] + K > rl) return MHSW_ERR_ARG;
    if (cand->pos_in_ctg[i] < 0 || cand->pos_in_ctg[i] + K > cg->h_len[(size_t)id]) return MHSW_ERR_ARG;
    rbytes = std::max<int64_t>(rbytes, cand->read_off[i] + rl);
  }
  if (rbytes > INT32_MAX) return MHSW_ERR_LIMIT;
  std::lock_guard<std::mutex> call_lk(mhsw::driver_call_mutex(d));
  cudaStream_t st = static_cast<cudaStream_t>(mhsw::driver_stream(d));
  cudaSetDevice(cg->device);
  KArgs g{};
  FArgs f{};
  int *counts = nullptr;
  int32_t *out5 = nullptr;
  int rc = MHSW_OK;
  cudaError_t e = cudaSuccess;
  char *read = nullptr, *ori = nullptr;
  int64_t *roff = nullptr;
  int32_t *rlen = nullptr, *cid = nullptr, *pic = nullptr, *pir = nullptr;
  uint8_t *strand = nullptr;
  int32_t *wstart = nullptr, *rstart0 = nullptr, *ov = nullptr, *slot = nullptr;
  int8_t *orient = nullptr;
  int64_t *a_off = nullptr, *b_off = nullptr;
  int32_t *a_len = nullptr, *b_len = nullptr;
  int32_t *o_rs = nullptr, *o_re = nullptr, *o_cs = nullptr, *o_ce = nullptr, *o_sc = nullptr, *o_s2 = nullptr,
          *o_id = nullptr;
  char *o_or = nullptr;
  uint8_t *o_pf = nullptr;
  // the call's arrays, laid out in the handle's caller arena (sized by a first pass)
  auto lay = [&](mhsw::Carve &c) {
    c.take(&read, (size_t)rbytes + 16);
    c.take(&ori, (size_t)rbytes + 16);
    c.take(&roff, (size_t)n);
    c.take(&rlen, (size_t)n);
    c.take(&cid, (size_t)n);
    c.take(&pic, (size_t)n);
    c.take(&pir, (size_t)n);
    c.take(&strand, (size_t)n);
    c.take(&wstart, (size_t)n);
    c.take(&rstart0, (size_t)n);
    c.take(&ov, (size_t)n);
    c.take(&slot, (size_t)n);
    c.take(&orient, (size_t)n);
    c.take(&a_off, (size_t)n);
    c.take(&b_off, (size_t)n);
    c.take(&a_len, (size_t)n);
    c.take(&b_len, (size_t)n);
    c.take(&counts, 4);
    c.take(&o_rs, (size_t)n);
    c.take(&o_re, (size_t)n);
    c.take(&o_cs, (size_t)n);
    c.take(&o_ce, (size_t)n);
    c.take(&o_sc, (size_t)n);
    c.take(&o_s2, (size_t)n);
    c.take(&o_id, (size_t)n);
    c.take(&o_or, (size_t)n);
    c.take(&o_pf, (size_t)n);
    c.take(&out5, (size_t)n * 5);  // the aligned candidates' results (at most n)
  };
  mhsw::Carve sizing;
  lay(sizing);
  mhsw::Carve arena{0, mhsw::driver_call_arena(d, sizing.off)};
  if (!arena.base) return MHSW_ERR_NOMEM;
  lay(arena);
  auto up = [&](void *dst, const void *src, size_t bytes) {
    if (!e && bytes) e = cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, st);
  };
  up(read, cand->read_seq, (size_t)rbytes);
  up(roff, cand->read_off, sizeof(int64_t) * n);
  up(rlen, cand->read_len, sizeof(int32_t) * n);
  up(cid, cand->contig_id, sizeof(int32_t) * n);
  up(pic, cand->pos_in_ctg, sizeof(int32_t) * n);
  up(pir, cand->pos_in_read, sizeof(int32_t) * n);
  up(strand, cand->strand, (size_t)n);
  if (!e) e = cudaMemsetAsync(counts, 0, 4 * sizeof(int), st);
  int h_counts[4] = {0, 0, 0, 0};
  if (!e) {
    g = KArgs{read, roff, rlen, cid, pic, pir, strand, n, K, cg->raw, cg->off, cg->len, ori, wstart, rstart0, ov,
              orient, slot, a_off, b_off, a_len, b_len, counts};
    int sms = 152, per_sm = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, cg->device);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_klign_prepare, kPrepWarps * 32, 0);
    const int64_t blocks = std::min<int64_t>((n + kPrepWarps - 1) / kPrepWarps, (int64_t)sms * std::max(per_sm, 1));
    k_klign_prepare<<<(unsigned)blocks, kPrepWarps * 32, 0, st>>>(g);
    e = cudaGetLastError();
  }
  if (!e) e = cudaMemcpyAsync(h_counts, counts, sizeof(h_counts), cudaMemcpyDeviceToHost, st);
  if (!e) e = cudaStreamSynchronize(st);
  const int32_t *s2 = nullptr;
  if (!e && h_counts[3] > 0) rc = MHSW_ERR_ARG;  // a read byte that revcomp rejects
  if (!e && !rc && h_counts[0] > 0) {
    const int64_t m = h_counts[0];
    mhsw::PairSet ps;
    ps.a_seq = ori;
    ps.a_off = a_off;
    ps.a_len = a_len;
    ps.b_seq = cg->raw;
    ps.b_off = b_off;
    ps.b_len = b_len;
    ps.n = m;
    ps.b_code = cg->codes;
    if (!e) {
      rc = mhsw::align_resident(d, ps, rbytes, h_counts[1], h_counts[2], mhsw::driver_form(d), out5);
      if (!rc) s2 = mhsw::driver_score2(d, m);
      // CIGAR mode: SSW's CIGARs of the aligned candidates (the pair set's A and B codes
      // are the translated oriented reads and the resident contig codes)
      if (!rc && out->cigar_slot && mhsw::driver_cigar(d)) {
        ps.a_code = mhsw::driver_a_codes(d);
        rc = mhsw::cigar_resident(d, ps);
      }
    }
    if (n_aligned) *n_aligned = m;
  }
  if (!e && !rc) {
    f = FArgs{rlen, wstart, rstart0, ov, slot, orient, out5, s2, mhsw::driver_match(d), n,
              o_rs, o_re, o_cs, o_ce, o_sc, o_s2, o_id, o_or, o_pf};
    k_klign_finish<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(f);
    e = cudaGetLastError();
    auto down = [&](void *dst, const void *src, size_t bytes) {
      if (!e) e = cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, st);
    };
    down(out->rstart, o_rs, sizeof(int32_t) * n);
    down(out->rstop, o_re, sizeof(int32_t) * n);
    down(out->cstart, o_cs, sizeof(int32_t) * n);
    down(out->cstop, o_ce, sizeof(int32_t) * n);
    down(out->score1, o_sc, sizeof(int32_t) * n);
    down(out->score2, o_s2, sizeof(int32_t) * n);
    down(out->identity, o_id, sizeof(int32_t) * n);
    down(out->orient, o_or, (size_t)n);
    down(out->perfect, o_pf, (size_t)n);
    if (out->cigar_slot && mhsw::driver_cigar(d)) down(out->cigar_slot, slot, sizeof(int32_t) * n);
    if (!e) e = cudaStreamSynchronize(st);
    if (!e && h_counts[0] > 0) mhsw::resident_timing(d);
  }
  if (e || rc) cudaStreamSynchronize(st);  // nothing of a failed call left in flight
  if (e) return e == cudaErrorMemoryAllocation ? MHSW_ERR_NOMEM : MHSW_ERR_CUDA;
  return rc;
}

}  // extern "C"
