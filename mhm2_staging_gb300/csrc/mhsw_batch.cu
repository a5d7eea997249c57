// mhsw_batch.cu -- batched form of the forward pass.
//
// The reference launches one block per pair with the block size fixed by the batch's
// longest sequences (src/adept-sw/driver.cpp:343-368), so uneven batches idle most
// threads.  Here the pair order is sorted on the device by a key
//   bucket(len A) << 17 | (131071 - len B)
// (bucket = rows-per-lane class of the wavefront engine, so a lane group always runs
// the narrowest engine that fits; longest B first inside a bucket), and one
// persistent launch of G-lane groups claims pairs from a single atomic counter
// (work stealing: a group that finishes early takes the next pair).  Pairs whose
// score could exceed the int16 range (min(lenA, lenB) * match above the int16
// capacity) are sent straight to the int32 list.
#include <algorithm>
#include <chrono>
#include <cub/cub.cuh>

#include "mhsw_batch.h"
#include "mhsw_engine.cuh"
#include "mhsw_engine16.cuh"
#include "mhsw_launch.h"

namespace mhsw {

namespace {

constexpr int kKeyShift = 17;
constexpr int kSortBits = 20;  // 3 bucket bits above the 17 B-length bits
// Buckets: 0..3 = A up to 64/96/128/160 rows (8-lane groups, K = 4/6/8/10),
// 4/5 = up to 192/256 rows (16-lane groups, K = 6/8), 6 = longer A (K = 8 strips),
// 7 = could exceed the int16 keys: straight to the int32 list.  The tuned row threshold
// (lane_rows, 160 or 128) moves A of 129..160 rows between bucket 3 and bucket 4.
constexpr int kBucketFirstLong = 4;
constexpr int kBucketStrip = 6;
constexpr int kBucketWide = 7;
constexpr int kBuckets = 8;
constexpr int64_t kTuneSample = 256 * 1024;  // pairs the tuner's trials run on, at most

__host__ __device__ constexpr int bucket_k(int b) {
  return b == 0 ? 4 : b == 1 ? 6 : b == 2 ? 8 : b == 3 ? 10 : b == 4 ? 6 : 8;
}

__device__ __forceinline__ int bucket_of(int M, int N, const Scoring &sc, int lane_rows, bool wide_try16) {
  const int b = M <= lane_rows ? (M <= 64 ? 0 : M <= 96 ? 1 : M <= 128 ? 2 : 3)
                               : (M <= 192 ? 4 : M <= 256 ? 5 : kBucketStrip);
  // wide_try16: the int16 engine's ceiling test sends the pairs that do overflow to int32.
  // That test sees a score cross the keys' capacity only if the first cell above it still
  // fits a 16-bit key: the capacity leaves 64 values of margin and H grows by at most match
  // per step, so it holds for match <= 63; larger matches keep the bound routing.
  const long long bound = (long long)(M < N ? M : N) * sc.match;
  if ((!wide_try16 || sc.match > 63) && bound > keyed_cap(bucket_k(b))) return kBucketWide;
  return b;
}

// Sort keys of items i < m, item i = pair i * stride (stride 1: the whole batch; larger:
// the tuner's sample); hist (the sample) counts the items per bucket.
__global__ void k_keys(PairSet ps, Scoring sc, int lane_rows, bool wide_try16, int64_t m, int64_t stride,
                       uint32_t *keys, uint32_t *idx, int *hist) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < m; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t p = i * stride;
    const int M = ps.a_len[p], N = ps.b_len[p];
    const int b = (M <= 0 || N <= 0) ? 0 : bucket_of(M, N, sc, lane_rows, wide_try16);
    const int nb = N < 0 ? 0 : (N > 131071 ? 131071 : N);
    keys[i] = ((uint32_t)b << kKeyShift) | (uint32_t)(131071 - nb);
    idx[i] = (uint32_t)p;
    if (hist) atomicAdd(&hist[b], 1);
  }
}

__device__ __forceinline__ unsigned group_mask_b(int G) {
  if (G == 32) return 0xffffffffu;
  const int lane32 = threadIdx.x & 31;
  return ((1u << G) - 1u) << ((lane32 / G) * G);
}

// First sorted item of the long-read buckets (the sorted keys are ascending).
__global__ void k_split(const uint32_t *__restrict__ keys, int64_t n, int *split) {
  const uint32_t first = (uint32_t)kBucketFirstLong << kKeyShift;
  int64_t lo = 0, hi = n;
  while (lo < hi) {
    const int64_t mid = (lo + hi) / 2;
    if (keys[mid] < first) lo = mid + 1;
    else hi = mid;
  }
  *split = (int)lo;
}

// Persistent forward kernel over one range of the sorted pair order: 8-lane groups for
// the short-read buckets (items [0, split)), 16-lane groups for the rest ([split, n)).
// A group claims its next pair from the range's atomic counter.
template <int G, bool S2 = false>
__global__ void __launch_bounds__(256) k_fwd_persist(PairSet ps, ResultSet rs, Scoring sc,
                                                     const uint32_t *__restrict__ keys,
                                                     const uint32_t *__restrict__ order, int64_t n, int *queue,
                                                     const int *split, int ceiling, WorkLists wl, int pad, int bcap,
                                                     V16::Pay *scratch, int scratch_stride) {
  constexpr bool kShort = (G == kGKShort);
  extern __shared__ __align__(16) unsigned char smem[];
  const int gpb = blockDim.x / G;
  const int grp = threadIdx.x / G;
  const int lane = threadIdx.x % G;
  const unsigned gmask = group_mask_b(G);
  constexpr int kC = S2 ? kCode16Zero + 1 : kCodeN + 1;
  constexpr size_t kProf = kShort ? group_prof16_bytes<10, G, kC>() : group_prof16_bytes<8, G, kC>();
  unsigned char *gbase = smem + (size_t)grp * kProf;  // keyed engine: profile table only
  GroupSmem gs;
  gs.prof = reinterpret_cast<uint32_t *>(gbase);
  gs.prof_lanes = G;
  gs.bcodes = nullptr;
  gs.pad = pad;
  gs.bcap = bcap;
  const int64_t gid = (int64_t)blockIdx.x * gpb + grp;
  V16::Pay *bnd = scratch ? scratch + gid * (int64_t)scratch_stride : nullptr;
  const int64_t lo = kShort ? 0 : *split;
  const int64_t hi = kShort ? *split : n;
  int *counter = queue + (kShort ? 0 : 1);

  for (;;) {
    int claim = 0;
    if (lane == 0) claim = atomicAdd(counter, 1);
    claim = __shfl_sync(gmask, claim, 0, G);
    const int64_t item = lo + claim;
    if (item >= hi) break;
    const uint32_t key = keys[item];
    const int64_t p = order[item];
    const int bucket = (int)(key >> kKeyShift);
    const int M = ps.a_len[p], N = ps.b_len[p];
    if (bucket == kBucketWide) {
      if (lane == 0) {
        rs.flag[p] = kFlagOverflow16;
        rs.score[p] = 0;
        rs.a_end[p] = -1;
        rs.b_end[p] = 0;
        const int slot = atomicAdd(wl.ovf_count, 1);
        if (slot < wl.cap) wl.ovf[slot] = p;
      }
      continue;
    }
    const int NP = S2 ? ssw_pad16(N) : N;
    const bool too_long = (N > kMaxB) || (bucket == kBucketStrip && (bnd == nullptr || NP > scratch_stride));
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
    if constexpr (kShort) {
      switch (bucket) {
        case 0: sweep16<4, G, S2>(A, B, sc, gs, lane, gmask, bnd, ceiling, so, rmo); break;
        case 1: sweep16<6, G, S2>(A, B, sc, gs, lane, gmask, bnd, ceiling, so, rmo); break;
        case 2: sweep16<8, G, S2>(A, B, sc, gs, lane, gmask, bnd, ceiling, so, rmo); break;
        default: sweep16<10, G, S2>(A, B, sc, gs, lane, gmask, bnd, ceiling, so, rmo); break;
      }
    } else {
      if (bucket == 4) sweep16<6, G, S2>(A, B, sc, gs, lane, gmask, bnd, ceiling, so, rmo);
      else sweep16<8, G, S2>(A, B, sc, gs, lane, gmask, bnd, ceiling, so, rmo);
    }
    if (lane == 0) {
      const int S = key_value(so.key);
      // score2 mode: the word path's padding differs from the one swept here; the int32
      // pass recomputes those row maxima
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

template <class T>
cudaError_t grow(T **p, size_t n) {
  if (*p) cudaFree(*p);
  *p = nullptr;
  return cudaMalloc(p, n * sizeof(T));
}

}  // namespace

void BatchState::release() {
  for (uint32_t **q : {&keys_in, &keys_out, &idx_in, &idx_out, &s_keys_in, &s_keys_out, &s_idx_in, &s_idx_out}) {
    if (*q) cudaFree(*q);
    *q = nullptr;
  }
  for (void **q : {&temp, &s_temp, &scratch}) {
    if (*q) cudaFree(*q);
    *q = nullptr;
  }
  if (queue) cudaFree(queue);
  if (s_hist) cudaFree(s_hist);
  queue = nullptr;
  s_hist = nullptr;
  cap = 0;
  temp_bytes = 0;
  s_temp_bytes = 0;
  scratch_bytes = 0;
}

int signature_class(int a_len) {
  return a_len <= 64 ? 0 : a_len <= 96 ? 1 : a_len <= 128 ? 2 : a_len <= 160 ? 3 : a_len <= 192 ? 4 : a_len <= 256 ? 5
         : a_len <= 1024 ? 6 : 7;
}

BatchSignature batch_signature(const int32_t *a_len, int64_t n, int max_a, int max_b) {
  BatchSignature s;
  s.max_a_class = signature_class(max_a);
  s.max_a = max_a;
  s.max_b = max_b;
  s.n = n;
  if (a_len && n > 0) {
    const int64_t step = n > 4096 ? n / 4096 : 1;
    int cnt[kSigClasses] = {0};
    int64_t k = 0;
    for (int64_t i = 0; i < n; i += step, k++) cnt[signature_class(a_len[i])]++;
    for (int c = 0; c < kSigClasses; c++) s.a_mix[c] = (float)cnt[c] / (float)k;
  }
  return s;
}

static bool within(double x, double y, double factor) {
  x = x > 1 ? x : 1;
  y = y > 1 ? y : 1;
  return x <= y * factor && y <= x * factor;
}

bool BatchSignature::close_to(const BatchSignature &o) const {
  if (max_a_class != o.max_a_class || !within(max_b, o.max_b, 2.0)) return false;
  if (!(n <= 65536 && o.n <= 65536) && !within((double)n, (double)o.n, 8.0)) return false;
  if (a_mix[0] < 0 || o.a_mix[0] < 0) return true;  // a mix the host cannot see is not compared
  for (int c = 0; c < kSigClasses; c++)
    if (a_mix[c] - o.a_mix[c] > kTolerance || o.a_mix[c] - a_mix[c] > kTolerance) return false;
  return true;
}

int batched_forward(BatchState &bs, int device, const PairSet &ps, const ResultSet &rs, const WorkLists &wl,
                    const Scoring &sc, int ceiling, int max_a, int max_b, const BatchSignature &sig,
                    cudaStream_t st, int64_t *launches, const Forks *fk) {
  auto fail = [&](cudaError_t e, const char *what) {
    bs.err = std::string(what) + ": " + cudaGetErrorString(e);
    return 1;
  };
  const int64_t n = ps.n;
  bs.tune.last_call_tuned = false;
  if (n <= 0) return 0;
  if (n > 0x7fffffff) {
    bs.err = "batch larger than 2^31 pairs";
    return 1;
  }
  cudaError_t e;
  if ((size_t)n > bs.cap) {
    size_t c = (size_t)n + (size_t)n / 8 + 1024;
    if ((e = grow(&bs.keys_in, c)) || (e = grow(&bs.keys_out, c)) || (e = grow(&bs.idx_in, c)) ||
        (e = grow(&bs.idx_out, c)))
      return fail(e, "cudaMalloc batch keys");
    size_t tb = 0;
    cub::DeviceRadixSort::SortPairs(nullptr, tb, bs.keys_in, bs.keys_out, bs.idx_in, bs.idx_out, (int)c, 0, kSortBits,
                                    st);
    if (bs.temp) cudaFree(bs.temp);
    bs.temp = nullptr;
    if ((e = cudaMalloc(&bs.temp, tb))) return fail(e, "cudaMalloc sort temp");
    bs.temp_bytes = tb;
    bs.cap = c;
  }
  // queue[0], queue[1]: claim counters of the short and long ranges; queue[2]: split item;
  // queue[4..6]: the same for the tuner's sample
  if (!bs.queue && (e = cudaMalloc(&bs.queue, sizeof(int) * 8))) return fail(e, "cudaMalloc queue");

  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
  if (max_b > kMaxB) {
    bs.err = "B longer than the kernel limit";
    return 1;
  }
  const bool s2 = ps.rowmax16 != nullptr;
  auto kshort = s2 ? k_fwd_persist<kGKShort, true> : k_fwd_persist<kGKShort, false>;
  auto klong = s2 ? k_fwd_persist<kGKLong, true> : k_fwd_persist<kGKLong, false>;
  const size_t prof_short = s2 ? group_prof16_bytes<10, kGKShort, kCode16Zero + 1>() : group_prof16_bytes<10, kGKShort>();
  const size_t prof_long = s2 ? group_prof16_bytes<8, kGKLong, kCode16Zero + 1>() : group_prof16_bytes<8, kGKLong>();
  const int pad = 2 * kGKLong;
  // strip scratch stride: B, the lane skew and score2 mode's zero-score padding (< 16)
  const int bcap = ((pad + std::max(max_b, 1) + 16 + 2 * kGKLong) + 15) / 16 * 16;

  // keys + device sort of m items (pair i * stride), split point into q[2]
  auto sort_items = [&](const BatchShape &sh, int64_t m, int64_t stride, uint32_t *kin, uint32_t *kout, uint32_t *iin,
                        uint32_t *iout, void *temp, size_t temp_bytes, int *q, int *hist) -> int {
    const int grid = (int)std::min<int64_t>((m + 255) / 256, (int64_t)sms * 32);
    if (hist && (e = cudaMemsetAsync(hist, 0, sizeof(int) * kBuckets, st))) return fail(e, "memset");
    k_keys<<<grid, 256, 0, st>>>(ps, sc, sh.lane_rows, sh.wide_try16, m, stride, kin, iin, hist);
    if ((e = cudaGetLastError())) return fail(e, "keys launch");
    size_t tb = temp_bytes;
    e = cub::DeviceRadixSort::SortPairs(temp, tb, kin, kout, iin, iout, (int)m, 0, kSortBits, st);
    if (e) return fail(e, "radix sort");
    k_split<<<1, 1, 0, st>>>(kout, m, q + 2);
    if ((e = cudaGetLastError())) return fail(e, "split launch");
    if (launches) *launches += 2 + 4;  // keys, split, and the radix sort's passes (approximate)
    return 0;
  };

  // the two persistent launches over m sorted items (keys, order), claim counters in q
  auto run = [&](const BatchShape &sh, const uint32_t *keys, const uint32_t *order, int64_t m, int *q,
                 float *ms) -> int {
    const int threads = sh.groups_per_block * 8;  // block size: 8 groups of 8 lanes or 4 of 16, etc.
    const int gpb_s = threads / kGKShort, gpb_l = threads / kGKLong;
    const size_t smem_s = (size_t)gpb_s * prof_short, smem_l = (size_t)gpb_l * prof_long;
    cudaError_t e2;
    if ((e2 = raise_smem_limit(reinterpret_cast<const void *>(kshort), smem_s))) return fail(e2, "smem attribute");
    if ((e2 = raise_smem_limit(reinterpret_cast<const void *>(klong), smem_l))) return fail(e2, "smem attribute");
    int occ_s = 0, occ_l = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ_s, kshort, threads, smem_s);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ_l, klong, threads, smem_l);
    occ_s = std::max(occ_s, 1);
    occ_l = std::max(occ_l, 1);
    const int grid_s = sms * (sh.blocks_per_sm > 0 ? std::min(sh.blocks_per_sm, occ_s) : occ_s);
    const int grid_l = sms * (sh.blocks_per_sm > 0 ? std::min(sh.blocks_per_sm, occ_l) : occ_l);
    V16::Pay *scr = nullptr;
    const int stride = bcap;
    if (max_a > 2 * 8 * kGKLong) {
      const size_t need = (size_t)grid_l * gpb_l * (size_t)stride * sizeof(V16::Pay);
      if (need > bs.scratch_bytes) {
        if (bs.scratch) cudaFree(bs.scratch);
        bs.scratch = nullptr;
        bs.scratch_bytes = 0;
        e2 = cudaMalloc(&bs.scratch, need);
        if (e2) return fail(e2, "cudaMalloc strip scratch");
        bs.scratch_bytes = need;
      }
      scr = reinterpret_cast<V16::Pay *>(bs.scratch);
    }
    cudaEvent_t t0 = nullptr, t1 = nullptr;
    if (ms) {
      cudaEventCreate(&t0);
      cudaEventCreate(&t1);
      cudaEventRecord(t0, st);
    }
    cudaMemsetAsync(q, 0, 2 * sizeof(int), st);
    cudaMemsetAsync(wl.ovf_count, 0, sizeof(int), st);
    const bool fan = fk && fk->fork;
    if (fan && (e2 = fork_to(*fk, st, 1))) return fail(e2, "fork");
    klong<<<grid_l, threads, smem_l, fan ? fk->side[0] : st>>>(ps, rs, sc, keys, order, m, q, q + 2, ceiling, wl, pad,
                                                               bcap, scr, stride);
    kshort<<<grid_s, threads, smem_s, st>>>(ps, rs, sc, keys, order, m, q, q + 2, ceiling, wl, pad, bcap, nullptr,
                                             stride);
    e2 = cudaGetLastError();
    if (e2) return fail(e2, "persistent forward launch");
    if (fan && (e2 = join_from(*fk, st, 1))) return fail(e2, "join");
    if (launches) *launches += 2;
    if (ms) {
      cudaEventRecord(t1, st);
      cudaEventSynchronize(t1);
      cudaEventElapsedTime(ms, t0, t1);
      cudaEventDestroy(t0);
      cudaEventDestroy(t1);
    }
    return 0;
  };

  // a configuration tuned earlier for a signature close to this one is taken back without
  // trials (batches that alternate between workloads, such as full and partial serving
  // micro-batches, tune once each)
  if (bs.autotune && (!bs.tuned || !sig.close_to(bs.tuned_for))) {
    for (int k = 0; k < bs.n_cached; k++)
      if (sig.close_to(bs.cached[k].sig)) {
        bs.shape = bs.cached[k].shape;
        bs.tuned_for = bs.cached[k].sig;
        bs.tuned = true;
        break;
      }
  }
  if (bs.autotune && (!bs.tuned || !sig.close_to(bs.tuned_for))) {
    // Trials on a strided sample of the batch (every stride-th pair, so its length mix is
    // the batch's), sorted as the batch is.  Coordinate descent: the launch shape at the
    // default row threshold; then the 16-lane threshold for A of 129..160 rows; then the
    // int16/int32 split of pairs whose bound exceeds the int16 keys -- each only when the
    // sample has pairs it affects.  Trial results land in the result arrays of the sampled
    // pairs and are overwritten by the batch's own pass.
    const auto t_start = std::chrono::steady_clock::now();
    const int64_t stride = (n + kTuneSample - 1) / kTuneSample;
    const int64_t m = (n + stride - 1) / stride;
    if (!bs.s_keys_in) {
      const size_t c = (size_t)kTuneSample + 1024;
      if ((e = grow(&bs.s_keys_in, c)) || (e = grow(&bs.s_keys_out, c)) || (e = grow(&bs.s_idx_in, c)) ||
          (e = grow(&bs.s_idx_out, c)) || (e = grow(&bs.s_hist, (size_t)kBuckets)))
        return fail(e, "cudaMalloc tuner sample");
      size_t tb = 0;
      cub::DeviceRadixSort::SortPairs(nullptr, tb, bs.s_keys_in, bs.s_keys_out, bs.s_idx_in, bs.s_idx_out, (int)c, 0,
                                      kSortBits, st);
      if ((e = cudaMalloc(&bs.s_temp, tb))) return fail(e, "cudaMalloc tuner sort temp");
      bs.s_temp_bytes = tb;
    }
    int *sq = bs.queue + 4;
    int hist[kBuckets] = {0};
    auto sample_sort = [&](const BatchShape &sh) -> int {
      if (sort_items(sh, m, stride, bs.s_keys_in, bs.s_keys_out, bs.s_idx_in, bs.s_idx_out, bs.s_temp,
                     bs.s_temp_bytes, sq, bs.s_hist))
        return 1;
      if ((e = cudaMemcpyAsync(hist, bs.s_hist, sizeof(hist), cudaMemcpyDeviceToHost, st)) ||
          (e = cudaStreamSynchronize(st)))
        return fail(e, "tuner histogram");
      return 0;
    };
    TuneRecord tr;
    tr.tunings = bs.tune.tunings + 1;
    tr.sample_pairs = m;
    auto trial = [&](const BatchShape &sh, float *ms) -> int {
      if (run(sh, bs.s_keys_out, bs.s_idx_out, m, sq, ms)) return 1;
      if (tr.trials < 16) tr.trial_ms[tr.trials] = *ms;
      tr.trials++;
      return 0;
    };
    BatchShape best;  // defaults: 128-thread blocks, occupancy limit, rows <= 160 in 8-lane groups
    if (sample_sort(best)) return 1;
    float warm = 0.f, best_ms = 1e30f;
    if (run(best, bs.s_keys_out, bs.s_idx_out, m, sq, &warm)) return 1;  // untimed warm-up
    const BatchShape shapes[] = {{8, 0}, {16, 0}, {32, 0}, {16, 2}, {32, 1}};
    for (const BatchShape &c0 : shapes) {
      BatchShape c = best;
      c.groups_per_block = c0.groups_per_block;
      c.blocks_per_sm = c0.blocks_per_sm;
      float ms = 0.f;
      if (trial(c, &ms)) return 1;
      if (ms < best_ms) {
        best_ms = ms;
        best = c;
      }
    }
    if (hist[3] > 0) {  // A of 129..160 rows present: try them in 16-lane groups
      BatchShape c = best;
      c.lane_rows = 128;
      float ms = 0.f;
      if (sample_sort(c) || trial(c, &ms)) return 1;
      if (ms < best_ms) {
        best_ms = ms;
        best = c;
      }
      if (sample_sort(best)) return 1;  // hist of the kept threshold
    }
    if (hist[kBucketWide] > 0 && sc.match <= 63) {  // bound above the int16 keys: try int16 first
      BatchShape c = best;
      c.wide_try16 = true;
      float ms = 0.f;
      if (sample_sort(c) || trial(c, &ms)) return 1;
      if (ms < best_ms) best = c;
    }
    bs.shape = best;
    bs.tuned_for = sig;
    bs.tuned = true;
    bs.cached[bs.next_cached] = BatchState::Tuned{sig, best};
    bs.next_cached = (bs.next_cached + 1) % BatchState::kCached;
    if (bs.n_cached < BatchState::kCached) bs.n_cached++;
    tr.last_call_tuned = true;
    tr.wall_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t_start).count();
    bs.tune = tr;
  }

  // the batch: keys with the kept configuration, sort, the persistent launches
  if (sort_items(bs.shape, n, 1, bs.keys_in, bs.keys_out, bs.idx_in, bs.idx_out, bs.temp, bs.temp_bytes, bs.queue,
                 nullptr))
    return 1;
  return run(bs.shape, bs.keys_out, bs.idx_out, n, bs.queue, nullptr);
}

}  // namespace mhsw
