// mhsw_noalloc.cu -- the allocation-free forward entry point, mhsw_forward_noalloc().
//
// Some callers cannot let a library allocate device memory while they run:
//   * a process whose device memory has been handed, up front, to its own pool or
//     caching allocator (MHM2 sizes its GPU buffers per rank from the free memory it
//     measures at start-up), where a cudaMalloc of ours may fail or squeeze the pool;
//   * a pipelined loop that cannot take the device-wide synchronisation that cudaMalloc
//     and cudaFree may imply, because other streams of the same process must keep
//     running meanwhile.
// This entry point serves them.  It computes what the forward pass of the driver
// computes -- score, A end and B end per pair, bit-exact with SSW -- with one kernel
// whose every piece of scratch memory (per lane group: the translated A and B codes, the
// staged B codes and the strip boundary of long A) lives in one file-scope device array
// of fixed size.  The kernel is a variant of k_fwd<V32, 4, 16> (mhsw_kernels.cu), the
// int32 wavefront forward kernel, grid-stride over the batch, exact at every score.
//
// Nothing here calls cudaMalloc, cudaFree or any library routine that allocates.
// The first call on a device does a one-time set-up with that device current: it looks
// up the scratch array's device address (cudaGetSymbolAddress, which also loads this
// module onto the device) and sets the kernel's shared-memory attribute.  Make that
// first call before any stream capture begins.
#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <cstdarg>
#include <cstdio>
#include <mutex>

#include "../../include/mhsw.h"
#include "mhsw_engine.cuh"
#include "mhsw_launch.h"

namespace mhsw {
namespace {

constexpr int kNaG = 16;  // lanes per pair
constexpr int kNaK = 4;   // row pairs per lane: strips of 2 * 4 * 16 = 128 rows
constexpr int kNaGroupsPerBlock = 8;
constexpr int kNaMaxDevices = 64;

// The scratch array: 32 MiB per device, shared by every call on that device.
constexpr size_t kNoAllocScratchBytes = size_t(32) << 20;
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

__host__ __device__ constexpr size_t round_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

// Layout of one lane group's share of the scratch array, for a batch whose pairs
// have at most max_a A bytes and max_b B bytes:
//   [strip boundary: bcap payloads][A codes][B codes][staged B codes: bcap bytes]
struct NaLayout {
  int pad, bcap;
  size_t bnd_bytes, a_cap, b_cap, stride;
};

__host__ __device__ inline NaLayout na_layout(int max_a, int max_b) {
  NaLayout l;
  l.pad = 2 * kNaG;
  l.bcap = (int)round_up((size_t)l.pad + (size_t)max_b + 2 * kNaG, 16);
  l.bnd_bytes = round_up((size_t)l.bcap * sizeof(V32::Pay), 256);
  l.a_cap = round_up((size_t)max_a, 16);
  l.b_cap = round_up((size_t)max_b, 16);
  l.stride = round_up(l.bnd_bytes + l.a_cap + l.b_cap + (size_t)l.bcap, 256);
  return l;
}

__device__ __forceinline__ unsigned na_group_mask() {
  const int lane32 = threadIdx.x & 31;
  return ((1u << kNaG) - 1u) << ((lane32 / kNaG) * kNaG);
}

// One kNaG-lane group per pair, grid-stride over [0, n).  Group gid owns bytes
// [gid * stride, (gid + 1) * stride) of the scratch array; the host sizes the grid so
// that every group's share lies inside it.  Each pair's scratch is written (codes
// translated, B codes staged, boundary written by strip s before strip s + 1 reads it)
// before it is read, so nothing needs to start at zero.
__global__ void __launch_bounds__(kNaG * kNaGroupsPerBlock)
    k_fwd_noalloc(const char *__restrict__ a_seq, const int64_t *__restrict__ a_off,
                  const int32_t *__restrict__ a_len, const char *__restrict__ b_seq,
                  const int64_t *__restrict__ b_off, const int32_t *__restrict__ b_len, int64_t n, Scoring sc,
                  int max_a, int max_b, unsigned char *scratch, NaLayout lay, int32_t *__restrict__ out3) {
  extern __shared__ __align__(16) unsigned char smem[];
  constexpr size_t kProf = group_prof_bytes<V32, kNaK, kNaG>();
  const int gpb = blockDim.x / kNaG;
  const int grp = threadIdx.x / kNaG;
  const int lane = threadIdx.x % kNaG;
  const unsigned gmask = na_group_mask();
  const int64_t gid = (int64_t)blockIdx.x * gpb + grp;
  const int64_t gstride = (int64_t)gridDim.x * gpb;

  unsigned char *mine = scratch + (size_t)gid * lay.stride;
  V32::Pay *bnd = reinterpret_cast<V32::Pay *>(mine);
  uint8_t *acodes = mine + lay.bnd_bytes;
  uint8_t *bcodes = acodes + lay.a_cap;
  GroupSmem gs;
  gs.prof = reinterpret_cast<uint32_t *>(smem + (size_t)grp * kProf);
  gs.prof_lanes = kNaG;
  gs.bcodes = bcodes + lay.b_cap;
  gs.pad = lay.pad;
  gs.bcap = lay.bcap;

  for (int64_t i = gid; i < n; i += gstride) {
    const int M = a_len[i], N = b_len[i];
    if (M < 0 || N < 0 || M > max_a || N > max_b) {  // outside the stated maxima
      if (lane == 0) {
        out3[3 * i + 0] = -1;
        out3[3 * i + 1] = -1;
        out3[3 * i + 2] = -1;
      }
      continue;
    }
    if (M == 0 || N == 0) {
      if (lane == 0) {
        out3[3 * i + 0] = 0;
        out3[3 * i + 1] = -1;
        out3[3 * i + 2] = 0;
      }
      continue;
    }
    const char *as = a_seq + a_off[i];
    const char *bs = b_seq + b_off[i];
    for (int x = lane; x < M; x += kNaG) acodes[x] = c_code[(uint8_t)as[x]];
    for (int x = lane; x < N; x += kNaG) bcodes[x] = c_code[(uint8_t)bs[x]];
    __syncwarp(gmask);
    SeqView A{acodes, 1, M};
    SeqView B{bcodes, 1, N};
    SweepOut so;
    sweep_pair<V32, kNaK, kNaG>(A, B, sc, gs, lane, gmask, bnd, INT_MAX, so);
    if (lane == 0) {
      const int S = key_value(so.key);
      out3[3 * i + 0] = S;
      out3[3 * i + 1] = S > 0 ? key_row(so.key) : -1;
      out3[3 * i + 2] = S > 0 ? key_col(so.key) : 0;
    }
    __syncwarp(gmask);  // the next pair overwrites this pair's codes
  }
}

struct NaDevice {
  bool ready = false;
  unsigned char *scratch = nullptr;
  int sms = 0;
  int blocks_per_sm = 0;
};

std::mutex g_na_mu;
NaDevice g_na_dev[kNaMaxDevices];

int na_fail(char *errbuf, size_t errlen, int rc, const char *fmt, ...) {
  if (errbuf && errlen) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(errbuf, errlen, fmt, ap);
    va_end(ap);
  }
  return rc;
}

constexpr size_t na_block_smem() { return (size_t)kNaGroupsPerBlock * group_prof_bytes<V32, kNaK, kNaG>(); }

// One-time set-up for the current device: scratch address, kernel attribute, occupancy.
int na_setup(int dev, NaDevice **out, char *errbuf, size_t errlen) {
  std::lock_guard<std::mutex> lk(g_na_mu);
  NaDevice &d = g_na_dev[dev];
  if (!d.ready) {
    void *p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess)
      return na_fail(errbuf, errlen, MHSW_ERR_CUDA, "cudaGetSymbolAddress: %s", cudaGetErrorString(e));
    const size_t smem = na_block_smem();
    if (smem > 48 * 1024) {
      e = cudaFuncSetAttribute(k_fwd_noalloc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      if (e != cudaSuccess)
        return na_fail(errbuf, errlen, MHSW_ERR_CUDA, "cudaFuncSetAttribute: %s", cudaGetErrorString(e));
    }
    int sms = 0, occ = 0;
    e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess)
      return na_fail(errbuf, errlen, MHSW_ERR_CUDA, "cudaDeviceGetAttribute: %s", cudaGetErrorString(e));
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_fwd_noalloc, kNaG * kNaGroupsPerBlock, smem);
    if (e != cudaSuccess)
      return na_fail(errbuf, errlen, MHSW_ERR_CUDA, "occupancy query: %s", cudaGetErrorString(e));
    d.scratch = static_cast<unsigned char *>(p);
    d.sms = sms;
    d.blocks_per_sm = occ > 0 ? occ : 1;
    d.ready = true;
  }
  *out = &d;
  return MHSW_OK;
}

}  // namespace
}  // namespace mhsw

extern "C" int mhsw_forward_noalloc(const mhsw_pairs *pairs, short match_score, short mismatch_score,
                                    short gap_opening_score, short gap_extending_score, short ambiguity_score,
                                    int32_t *out3, void *stream, char *errbuf, size_t errlen) {
  using namespace mhsw;
  if (errbuf && errlen) errbuf[0] = '\0';
  if (!pairs) return na_fail(errbuf, errlen, MHSW_ERR_ARG, "pairs is NULL");
  const int64_t n = pairs->n;
  if (n < 0) return na_fail(errbuf, errlen, MHSW_ERR_ARG, "negative pair count");
  const Scoring sc{match_score, (short)-mismatch_score, (short)-gap_opening_score, (short)-gap_extending_score,
                   (short)-ambiguity_score};
  if (sc.match < 0 || sc.mismatch < 0 || sc.ambiguity < 0 || sc.gap_open < 1 || sc.gap_extend < 1)
    return na_fail(errbuf, errlen, MHSW_ERR_ARG,
                   "scores must be match >= 0 and mismatch/ambiguity <= 0, gap open/extend <= -1 (negated penalties)");
  if (sc.match > 127 || sc.mismatch > 127 || sc.ambiguity > 127 || sc.gap_open > 127 || sc.gap_extend > 127)
    return na_fail(errbuf, errlen, MHSW_ERR_ARG, "score magnitudes above 127 are not supported");
  if (n == 0) return MHSW_OK;
  if (!pairs->a_seq || !pairs->a_off || !pairs->a_len || !pairs->b_seq || !pairs->b_off || !pairs->b_len || !out3)
    return na_fail(errbuf, errlen, MHSW_ERR_ARG, "NULL device pointer in pairs or out3");
  const int max_a = pairs->max_a_len, max_b = pairs->max_b_len;
  if (max_a <= 0 || max_b <= 0)
    return na_fail(errbuf, errlen, MHSW_ERR_ARG, "pairs->max_a_len and pairs->max_b_len are required (> 0)");
  if (max_b > kMaxB || max_a >= (1 << 20))
    return na_fail(errbuf, errlen, MHSW_ERR_LIMIT, "max_a_len %d / max_b_len %d beyond the limits (%d / %d)", max_a,
                   max_b, (1 << 20) - 1, kMaxB);
  const NaLayout lay = na_layout(max_a, max_b);
  const int64_t fit = (int64_t)(kNoAllocScratchBytes / lay.stride);  // lane groups whose scratch fits
  if (fit < 1)
    return na_fail(errbuf, errlen, MHSW_ERR_LIMIT,
                   "one lane group needs %zu scratch bytes for max_a_len %d, max_b_len %d; the fixed scratch is %zu",
                   lay.stride, max_a, max_b, kNoAllocScratchBytes);

  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return na_fail(errbuf, errlen, MHSW_ERR_NO_GPU, "cudaGetDevice: %s", cudaGetErrorString(e));
  if (dev < 0 || dev >= kNaMaxDevices) return na_fail(errbuf, errlen, MHSW_ERR_LIMIT, "device %d beyond %d", dev,
                                                      kNaMaxDevices);
  NaDevice *d = nullptr;
  int rc = na_setup(dev, &d, errbuf, errlen);
  if (rc) return rc;

  // Block size: kNaGroupsPerBlock groups, or fewer when the scratch holds fewer groups.
  const int gpb = (int)std::min<int64_t>(kNaGroupsPerBlock, fit);
  int64_t blocks = std::min<int64_t>(fit / gpb, (int64_t)d->sms * d->blocks_per_sm);
  blocks = std::min<int64_t>(blocks, (n + gpb - 1) / gpb);
  if (blocks < 1) blocks = 1;
  // blocks * gpb <= fit: the last group's share ends inside the scratch array.
  const size_t smem = (size_t)gpb * group_prof_bytes<V32, kNaK, kNaG>();
  k_fwd_noalloc<<<(unsigned)blocks, gpb * kNaG, smem, static_cast<cudaStream_t>(stream)>>>(
      pairs->a_seq, pairs->a_off, pairs->a_len, pairs->b_seq, pairs->b_off, pairs->b_len, n, sc, max_a, max_b,
      d->scratch, lay, out3);
  e = cudaGetLastError();
  if (e != cudaSuccess) return na_fail(errbuf, errlen, MHSW_ERR_CUDA, "launch: %s", cudaGetErrorString(e));
  return MHSW_OK;
}
