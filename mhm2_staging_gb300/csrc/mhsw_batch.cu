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
#include <cub/cub.cuh>

#include "mhsw_batch.h"
#include "mhsw_engine.cuh"
#include "mhsw_engine16.cuh"
#include "mhsw_launch.h"

namespace mhsw {

namespace {

constexpr int kGB = 16;
constexpr int kKeyShift = 17;
constexpr int kBucketStrip = 6;  // A longer than one K=8 strip
constexpr int kBucketWide = 7;   // straight to int32
constexpr int kInt16Capacity = kCeiling16;  // keyed int16 engine

__device__ __forceinline__ int bucket_of(int M, int N, const Scoring &sc) {
  const long long bound = (long long)(M < N ? M : N) * sc.match;
  if (bound > kInt16Capacity) return kBucketWide;
  if (M > 2 * 8 * kGB) return kBucketStrip;
  const int need = (M + 2 * kGB - 1) / (2 * kGB);
  if (need <= 2) return 0;
  if (need <= 3) return 1;
  if (need <= 4) return 2;
  if (need <= 5) return 3;
  if (need <= 6) return 4;
  return 5;
}

__global__ void k_keys(PairSet ps, Scoring sc, uint32_t *keys, uint32_t *idx) {
  for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < ps.n; p += (int64_t)gridDim.x * blockDim.x) {
    const int M = ps.a_len[p], N = ps.b_len[p];
    const int b = (M <= 0 || N <= 0) ? 0 : bucket_of(M, N, sc);
    const int nb = N < 0 ? 0 : (N > 131071 ? 131071 : N);
    keys[p] = ((uint32_t)b << kKeyShift) | (uint32_t)(131071 - nb);
    idx[p] = (uint32_t)p;
  }
}

__device__ __forceinline__ unsigned group_mask_b(int G) {
  if (G == 32) return 0xffffffffu;
  const int lane32 = threadIdx.x & 31;
  return ((1u << G) - 1u) << ((lane32 / G) * G);
}

template <int G>
__global__ void __launch_bounds__(256) k_fwd_persist(PairSet ps, ResultSet rs, Scoring sc,
                                                     const uint32_t *__restrict__ keys,
                                                     const uint32_t *__restrict__ order, int64_t n, int *queue,
                                                     int ceiling, WorkLists wl, int pad, int bcap, V16::Pay *scratch,
                                                     int scratch_stride) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int gpb = blockDim.x / G;
  const int grp = threadIdx.x / G;
  const int lane = threadIdx.x % G;
  const unsigned gmask = group_mask_b(G);
  constexpr size_t kProf = group_prof16_bytes<8, G>();
  unsigned char *gbase = smem + (size_t)grp * kProf;  // keyed engine: profile table only
  GroupSmem gs;
  gs.prof = reinterpret_cast<uint32_t *>(gbase);
  gs.prof_lanes = G;
  gs.bcodes = nullptr;
  gs.pad = pad;
  gs.bcap = bcap;
  const int64_t gid = (int64_t)blockIdx.x * gpb + grp;
  V16::Pay *bnd = scratch ? scratch + gid * (int64_t)scratch_stride : nullptr;

  for (;;) {
    int item = 0;
    if (lane == 0) item = atomicAdd(queue, 1);
    item = __shfl_sync(gmask, item, 0, G);
    if (item >= n) break;
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
    const bool too_long = (N > kMaxB) || (bucket == kBucketStrip && (bnd == nullptr || N > scratch_stride));
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
    switch (bucket) {
      case 0: sweep16<2, G>(A, B, sc, gs, lane, gmask, bnd, ceiling, so); break;
      case 1: sweep16<3, G>(A, B, sc, gs, lane, gmask, bnd, ceiling, so); break;
      case 2: sweep16<4, G>(A, B, sc, gs, lane, gmask, bnd, ceiling, so); break;
      case 3: sweep16<5, G>(A, B, sc, gs, lane, gmask, bnd, ceiling, so); break;
      case 4: sweep16<6, G>(A, B, sc, gs, lane, gmask, bnd, ceiling, so); break;
      default: sweep16<8, G>(A, B, sc, gs, lane, gmask, bnd, ceiling, so); break;
    }
    if (lane == 0) {
      const int S = key_value(so.key);
      if (so.overflow) {
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
  if (keys_in) cudaFree(keys_in);
  if (keys_out) cudaFree(keys_out);
  if (idx_in) cudaFree(idx_in);
  if (idx_out) cudaFree(idx_out);
  if (temp) cudaFree(temp);
  if (queue) cudaFree(queue);
  if (scratch) cudaFree(scratch);
  keys_in = keys_out = idx_in = idx_out = nullptr;
  temp = nullptr;
  queue = nullptr;
  scratch = nullptr;
  cap = 0;
  temp_bytes = 0;
  scratch_bytes = 0;
}

int batched_forward(BatchState &bs, int device, const PairSet &ps, const ResultSet &rs, const WorkLists &wl,
                    const Scoring &sc, int ceiling, int max_a, int max_b, cudaStream_t st, int64_t *launches) {
  auto fail = [&](cudaError_t e, const char *what) {
    bs.err = std::string(what) + ": " + cudaGetErrorString(e);
    return 1;
  };
  const int64_t n = ps.n;
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
    cub::DeviceRadixSort::SortPairs(nullptr, tb, bs.keys_in, bs.keys_out, bs.idx_in, bs.idx_out, (int)c, 0, 20, st);
    if (bs.temp) cudaFree(bs.temp);
    bs.temp = nullptr;
    if ((e = cudaMalloc(&bs.temp, tb))) return fail(e, "cudaMalloc sort temp");
    bs.temp_bytes = tb;
    bs.cap = c;
  }
  if (!bs.queue && (e = cudaMalloc(&bs.queue, sizeof(int) * 4))) return fail(e, "cudaMalloc queue");

  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
  const int pad = 2 * kGB;
  const int bcap = ((pad + std::max(max_b, 1) + 2 * kGB) + 15) / 16 * 16;
  if (max_b > kMaxB) {
    bs.err = "B longer than the kernel limit";
    return 1;
  }
  const size_t per_group = group_prof16_bytes<8, kGB>();
  auto kern = k_fwd_persist<kGB>;

  // keys + sort (the order is reused by every tuning trial)
  {
    int grid = (int)std::min<int64_t>((n + 255) / 256, (int64_t)sms * 32);
    k_keys<<<grid, 256, 0, st>>>(ps, sc, bs.keys_in, bs.idx_in);
    if ((e = cudaGetLastError())) return fail(e, "keys launch");
    size_t tb = bs.temp_bytes;
    e = cub::DeviceRadixSort::SortPairs(bs.temp, tb, bs.keys_in, bs.keys_out, bs.idx_in, bs.idx_out, (int)n, 0, 20,
                                        st);
    if (e) return fail(e, "radix sort");
    if (launches) *launches += 2 + 3;  // keys + cub's onesweep passes (approximate)
  }

  auto run = [&](const BatchShape &sh, float *ms) -> int {
    const int gpb = sh.groups_per_block;
    const size_t smem = (size_t)gpb * per_group;
    if (smem > 48 * 1024) {
      cudaError_t e2 = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      if (e2) return fail(e2, "smem attribute");
    }
    int occ = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, gpb * kGB, smem);
    if (occ < 1) occ = 1;
    int bps = sh.blocks_per_sm > 0 ? std::min(sh.blocks_per_sm, occ) : occ;
    int grid = sms * bps;
    V16::Pay *scr = nullptr;
    int stride = bcap;
    if (max_a > 2 * 8 * kGB) {
      size_t need = (size_t)grid * gpb * (size_t)stride * sizeof(V16::Pay);
      if (need > bs.scratch_bytes) {
        if (bs.scratch) cudaFree(bs.scratch);
        bs.scratch = nullptr;
        bs.scratch_bytes = 0;
        cudaError_t e2 = cudaMalloc(&bs.scratch, need);
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
    cudaMemsetAsync(bs.queue, 0, sizeof(int), st);
    cudaMemsetAsync(wl.ovf_count, 0, sizeof(int), st);
    kern<<<grid, gpb * kGB, smem, st>>>(ps, rs, sc, bs.keys_out, bs.idx_out, n, bs.queue, ceiling, wl, pad, bcap, scr,
                                        stride);
    cudaError_t e2 = cudaGetLastError();
    if (e2) return fail(e2, "persistent forward launch");
    if (launches) *launches += 1;
    if (ms) {
      cudaEventRecord(t1, st);
      cudaEventSynchronize(t1);
      cudaEventElapsedTime(ms, t0, t1);
      cudaEventDestroy(t0);
      cudaEventDestroy(t1);
    }
    return 0;
  };

  if (bs.autotune && !bs.tuned) {
    // Candidate launch shapes: groups per block x blocks per SM.
    const BatchShape cands[] = {{2, 0}, {4, 0}, {8, 0}, {4, 2}, {8, 1}};
    float best = 1e30f;
    BatchShape pick = bs.shape;
    bs.tune_n = 0;
    for (const auto &c : cands) {
      float ms = 0.f;
      if (run(c, &ms)) return 1;
      if (bs.tune_n < 8) bs.tune_ms[bs.tune_n++] = ms;
      if (ms < best) {
        best = ms;
        pick = c;
      }
    }
    bs.shape = pick;
    bs.tuned = true;
  }
  return run(bs.shape, nullptr);
}

}  // namespace mhsw
