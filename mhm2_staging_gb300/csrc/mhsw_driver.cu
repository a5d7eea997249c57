// mhsw_driver.cu -- host driver and C ABI (include/mhsw.h).
//
// Re-creates the call surface of the reference's adept_sw::GPUDriver
// (src/adept-sw/driver.hpp:14-57, driver.cpp:28-417) on top of the GB300 kernels.
// Differences from the reference, all internal:
//   * both passes stay on one stream; the end coordinates feed the begin pass on the
//     device (no host reduction between passes, driver.cpp:170-180);
//   * buffers grow with the batch (no fixed KLIGN_GPU_BLOCK_SIZE cap, driver.cpp:213-242);
//   * sequences travel as raw bytes and are translated on the device with SSW's table.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <functional>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "../../include/mhsw.h"
#include "mhsw_batch.h"
#include "mhsw_engine.cuh"
#include "mhsw_engine16.cuh"
#include "mhsw_internal.h"
#include "mhsw_launch.h"

namespace {

template <class T>
struct DBuf {
  T *p = nullptr;
  size_t cap = 0;
  cudaError_t reserve(size_t n) {
    if (n <= cap) return cudaSuccess;
    if (p) cudaFree(p);
    p = nullptr;
    cap = 0;
    size_t want = std::max<size_t>(n + n / 8, 64);
    cudaError_t e = cudaMalloc(&p, want * sizeof(T));
    if (e != cudaSuccess) {
      p = nullptr;
      return e;
    }
    cap = want;
    return cudaSuccess;
  }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    cap = 0;
  }
};

template <class T>
struct HBuf {
  T *p = nullptr;
  size_t cap = 0;
  cudaError_t reserve(size_t n) {
    if (n <= cap) return cudaSuccess;
    if (p) cudaFreeHost(p);
    p = nullptr;
    cap = 0;
    size_t want = std::max<size_t>(n + n / 8, 64);
    cudaError_t e = cudaMallocHost(&p, want * sizeof(T));
    if (e != cudaSuccess) {
      p = nullptr;
      return e;
    }
    cap = want;
    return cudaSuccess;
  }
  void release() {
    if (p) cudaFreeHost(p);
    p = nullptr;
    cap = 0;
  }
};

constexpr int kInt16Ceiling = mhsw::V16::kBig - 1 - 64;  // leaves room for one match step

}  // namespace

// A few host threads a handle keeps for copying a batch's strings into its pinned staging
// buffers: klign hands each block over as std::vector<std::string> (about 13 MB for
// 20,000 reads and windows), and one thread copying them took longer than the block's
// kernels.  run(parts, fn) calls fn(0 .. parts-1) on the pool's threads and the caller's
// and returns when every part is done and no pool thread is still inside the job.
class CopyPool {
 public:
  ~CopyPool() {
    {
      std::lock_guard<std::mutex> lk(m_);
      quit_ = true;
    }
    cv_.notify_all();
    for (std::thread &t : th_) t.join();
  }
  static int threads_wanted() {
    const unsigned hw = std::thread::hardware_concurrency();
    return hw > 2 ? (int)std::min(8u, hw - 1) : 0;
  }
  void run(int parts, const std::function<void(int)> &fn) {
    if (th_.empty()) {
      const int k = threads_wanted();
      for (int i = 0; i < k; i++) th_.emplace_back([this] { loop(); });
    }
    if (th_.empty() || parts <= 1) {
      for (int p = 0; p < parts; p++) fn(p);
      return;
    }
    {
      std::lock_guard<std::mutex> lk(m_);
      job_ = &fn;
      total_ = parts;
      next_.store(0);
      finished_.store(0);
      gen_++;
    }
    cv_.notify_all();
    work();
    std::unique_lock<std::mutex> lk(m_);
    done_cv_.wait(lk, [this] { return finished_.load() == total_ && busy_ == 0; });
    job_ = nullptr;
  }

 private:
  void work() {
    for (;;) {
      const int p = next_.fetch_add(1);
      if (p >= total_) return;
      (*job_)(p);
      if (finished_.fetch_add(1) + 1 == total_) {
        std::lock_guard<std::mutex> lk(m_);
        done_cv_.notify_all();
      }
    }
  }
  void loop() {
    uint64_t seen = 0;
    for (;;) {
      {
        std::unique_lock<std::mutex> lk(m_);
        cv_.wait(lk, [&] { return quit_ || gen_ != seen; });
        if (quit_) return;
        seen = gen_;
        busy_++;
      }
      work();
      {
        std::lock_guard<std::mutex> lk(m_);
        busy_--;
      }
      done_cv_.notify_all();
    }
  }
  std::mutex m_;
  std::condition_variable cv_, done_cv_;
  std::vector<std::thread> th_;
  const std::function<void(int)> *job_ = nullptr;
  int total_ = 0, busy_ = 0;
  std::atomic<int> next_{0}, finished_{0};
  uint64_t gen_ = 0;
  bool quit_ = false;
};

struct mhsw_driver {
  std::mutex mu;
  std::mutex call_mu;  // calls on the call arena (caller side, protein), whole-call
  std::string err;
  bool inited = false;
  int device = 0;
  mhsw::Scoring sc{1, 1, 1, 1, 1};
  int orientation = MHSW_ORIENT_KLIGN;
  int form = MHSW_FORM_PLAIN;
  int ceiling16 = kInt16Ceiling;
  cudaStream_t st = nullptr;
  cudaEvent_t ev_done = nullptr;
  bool ev_live = false;
  cudaEvent_t ev_t[6] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};

  // device batch
  DBuf<char> a_seq, b_seq;
  DBuf<int64_t> a_off, b_off;
  DBuf<int32_t> a_len, b_len;
  DBuf<int32_t> r_score, r_aend, r_bend, r_abeg, r_bbeg;
  DBuf<uint32_t> r_flag;
  DBuf<int64_t> l_ovf, l_wide, l_bands;
  DBuf<int> l_counts;
  DBuf<uint8_t> a_code, b_code;  // base codes of the current batch
  DBuf<unsigned char> scratch;
  DBuf<unsigned char> call_arena;  // one call's own arrays (caller side, protein), kept between calls
  DBuf<unsigned char> outv;  // 5 x int16 + 5 x int32 arrays
  DBuf<int32_t> out5;
  mhsw::BatchState batch;     // batched-form work buffers
  CopyPool copy_pool;         // host threads for staging a block's strings
  mhsw::BatchSignature sig;   // length signature of the batch being aligned (the tuner's key)
  // score2 mode: SSW's second-best score per pair (row maxima arenas, results)
  bool score2 = false;
  int64_t score2_n = -1;  // pairs of the last batch whose second-best scores are in r_score2
  DBuf<int32_t> rowmax16, rowmax8, r_score2, r_aend2;
  HBuf<int32_t> h_score2;  // drop-in protocol: score2 then a_end2, n each
  mhsw::Forks forks;          // side streams for launches that overlap on the device
  // CIGAR mode: SSW's report_cigar output per pair (ops arena, lists, scratch)
  bool cigar = false;
  int64_t cigar_n = -1;        // pairs of the last batch whose CIGARs are in the arena
  int64_t cigar_total = -1;    // ops in pair order (after the ordered copy), -1 before it
  double cigar_ms = 0;
  int64_t cigar_generic = 0;   // pairs of the last batch that took the generic kernel
  int sms = 152;
  DBuf<int32_t> c_nops, c_mism;
  DBuf<int64_t> c_off, c_ordoff, c_c64;
  DBuf<uint32_t> c_arena, c_ordops, c_dirs;
  DBuf<unsigned long long> c_cursor;
  DBuf<int> c_counts;
  DBuf<int2> c_lists;
  DBuf<int4> c_generic, c_gsorted;
  DBuf<uint32_t> c_keys_in, c_keys_out, c_idx_in, c_idx_out;
  DBuf<unsigned char> c_sort_temp;
  DBuf<unsigned char> c_pool, c_temp;
  HBuf<int> h_ccounts;
  cudaEvent_t ev_c[2] = {nullptr, nullptr};
  // Batch calls enqueued (mhsw_align_pairs_async) and not yet completed: up to kSlots,
  // in slots used in turn.  A host batch copies into its slot's input set on the copy
  // streams, which wait only for that set's previous call (kSlots calls back), so its
  // copies run while earlier calls' kernels do, and a copy that runs slow (the host's copy
  // rate drops on some calls) is absorbed by the calls queued behind it; kernels stay in
  // order on the handle's stream.
  static constexpr int kSlots = 4;
  struct Pending {
    bool active = false;
    int64_t n = 0;
    double cells = 0;
    uint64_t seq = 0;
    mhsw::PairSet ps;
  } pend[kSlots];
  struct InSet {
    DBuf<char> a_seq, b_seq;
    DBuf<int64_t> a_off, b_off;
    DBuf<int32_t> a_len, b_len;
    cudaEvent_t free_ev = nullptr;  // recorded after the kernels of the set's last call
    bool used = false;
  } in_sets[kSlots];
  static constexpr int kCopyStreams = 4;
  cudaStream_t copy_st[kCopyStreams] = {};
  cudaEvent_t copy_ev[kCopyStreams] = {};
  cudaEvent_t ev_p[kSlots][5] = {};  // per slot: phase events of its call
  // per slot: its copies in start (copy stream 0) and end (one per copy stream); the
  // handle's epoch (recorded at init) that the call records are timed from
  cudaEvent_t ev_cin[kSlots][1 + kCopyStreams] = {};
  bool cin_recorded[kSlots] = {};
  cudaEvent_t ev_epoch = nullptr;
  static constexpr int kHistory = 64;
  mhsw_call_record history[kHistory] = {};
  int64_t history_n = 0;  // records written so far (the ring keeps the last kHistory)
  HBuf<int> h_counts_p[kSlots];  // per slot: the call's counters
  int next_slot = 0;
  uint64_t call_seq = 0;

  // CUDA graph of a device-resident batch: captured the second time the same batch
  // (same pointers, sizes and settings) is aligned, replayed from then on.
  struct GraphKey {
    const void *ptr[7];
    int64_t n, a_bytes, b_bytes;
    int32_t max_a, max_b;
    int form, ceiling, match, mismatch, gap_open, gap_extend, ambiguity, score2, cigar;
    bool operator==(const GraphKey &o) const { return std::memcmp(this, &o, sizeof(GraphKey)) == 0; }
  };
  GraphKey gkey{};
  bool gkey_seen = false;
  cudaGraphExec_t gexec = nullptr;
  bool use_graphs = true;
  int64_t graph_launches = 0;  // replays so far (diagnostics)

  // pinned host staging
  HBuf<char> h_a, h_b;
  HBuf<int64_t> h_aoff, h_boff;
  HBuf<int32_t> h_alen, h_blen;
  HBuf<unsigned char> h_outv;
  HBuf<int> h_counts;

  // drop-in protocol state
  int64_t n_batch = 0;
  int max_a = 0, max_b = 0;
  int64_t a_bytes = 0, b_bytes = 0;  // arena extents of the staged batch
  bool fwd_issued = false;
  bool rev_issued = false;
  double fwd_cells = 0;
  int64_t launches = 0;
  // Pair order of the last forward pass when it ran the batched form (its sorted
  // order, reused by the begin pass for coherent warps); null after a plain pass.
  const uint32_t *fwd_order = nullptr;
  mhsw_timing timing{};

  int fail(int code, const char *fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    err = buf;
    return code;
  }
  int cuda_fail(cudaError_t e, const char *what) {
    return fail(MHSW_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
  }

  ~mhsw_driver() {
    if (inited) cudaSetDevice(device);
    if (st) cudaStreamSynchronize(st);
    a_seq.release();
    b_seq.release();
    a_off.release();
    b_off.release();
    a_len.release();
    b_len.release();
    r_score.release();
    r_aend.release();
    r_bend.release();
    r_abeg.release();
    r_bbeg.release();
    r_flag.release();
    l_ovf.release();
    l_wide.release();
    l_bands.release();
    a_code.release();
    b_code.release();
    l_counts.release();
    scratch.release();
    call_arena.release();
    outv.release();
    out5.release();
    batch.release();
    rowmax16.release();
    rowmax8.release();
    r_score2.release();
    r_aend2.release();
    h_score2.release();
    c_nops.release();
    c_mism.release();
    c_off.release();
    c_ordoff.release();
    c_c64.release();
    c_arena.release();
    c_ordops.release();
    c_dirs.release();
    c_cursor.release();
    c_counts.release();
    c_lists.release();
    c_generic.release();
    c_gsorted.release();
    c_keys_in.release();
    c_keys_out.release();
    c_idx_in.release();
    c_idx_out.release();
    c_sort_temp.release();
    c_pool.release();
    c_temp.release();
    h_ccounts.release();
    for (auto &e : ev_c)
      if (e) cudaEventDestroy(e);
    for (auto &in : in_sets) {
      in.a_seq.release();
      in.b_seq.release();
      in.a_off.release();
      in.b_off.release();
      in.a_len.release();
      in.b_len.release();
      if (in.free_ev) cudaEventDestroy(in.free_ev);
    }
    for (auto &c : copy_st)
      if (c) cudaStreamDestroy(c);
    for (auto &e : copy_ev)
      if (e) cudaEventDestroy(e);
    for (auto &row : ev_p)
      for (auto &e : row)
        if (e) cudaEventDestroy(e);
    for (auto &row : ev_cin)
      for (auto &e : row)
        if (e) cudaEventDestroy(e);
    if (ev_epoch) cudaEventDestroy(ev_epoch);
    for (auto &h : h_counts_p) h.release();
    h_a.release();
    h_b.release();
    h_aoff.release();
    h_boff.release();
    h_alen.release();
    h_blen.release();
    h_outv.release();
    h_counts.release();
    if (gexec) cudaGraphExecDestroy(gexec);
    mhsw::forks_destroy(forks);
    for (auto &e : ev_t)
      if (e) cudaEventDestroy(e);
    if (ev_done) cudaEventDestroy(ev_done);
    if (st) cudaStreamDestroy(st);
  }
};

#define MHSW_CK(expr, what)                              \
  do {                                                   \
    cudaError_t _e = (expr);                             \
    if (_e != cudaSuccess) return d->cuda_fail(_e, what); \
  } while (0)

namespace {

int finish_pending(mhsw_driver *d);

// Device buffers for n pairs and the byte totals; result arrays; lists.
int ensure_device(mhsw_driver *d, int64_t n, int64_t a_bytes, int64_t b_bytes) {
  MHSW_CK(d->a_seq.reserve((size_t)a_bytes + 16), "cudaMalloc A");
  MHSW_CK(d->b_seq.reserve((size_t)b_bytes + 16), "cudaMalloc B");
  MHSW_CK(d->a_off.reserve((size_t)n + 1), "cudaMalloc offsets");
  MHSW_CK(d->b_off.reserve((size_t)n + 1), "cudaMalloc offsets");
  MHSW_CK(d->a_len.reserve((size_t)n + 1), "cudaMalloc lengths");
  MHSW_CK(d->b_len.reserve((size_t)n + 1), "cudaMalloc lengths");
  return MHSW_OK;
}

int ensure_results(mhsw_driver *d, int64_t n) {
  MHSW_CK(d->r_score.reserve((size_t)n + 1), "cudaMalloc results");
  MHSW_CK(d->r_aend.reserve((size_t)n + 1), "cudaMalloc results");
  MHSW_CK(d->r_bend.reserve((size_t)n + 1), "cudaMalloc results");
  MHSW_CK(d->r_abeg.reserve((size_t)n + 1), "cudaMalloc results");
  MHSW_CK(d->r_bbeg.reserve((size_t)n + 1), "cudaMalloc results");
  MHSW_CK(d->r_flag.reserve((size_t)n + 1), "cudaMalloc results");
  MHSW_CK(d->l_ovf.reserve((size_t)n + 1), "cudaMalloc lists");
  MHSW_CK(d->l_wide.reserve((size_t)n + 1), "cudaMalloc lists");
  MHSW_CK(d->l_bands.reserve((size_t)n + 1), "cudaMalloc lists");
  MHSW_CK(d->l_counts.reserve(2 + 2 * mhsw::kBandClasses), "cudaMalloc lists");
  return MHSW_OK;
}

mhsw::ResultSet result_set(mhsw_driver *d) {
  mhsw::ResultSet rs;
  rs.score = d->r_score.p;
  rs.a_end = d->r_aend.p;
  rs.b_end = d->r_bend.p;
  rs.a_beg = d->r_abeg.p;
  rs.b_beg = d->r_bbeg.p;
  rs.flag = d->r_flag.p;
  if (d->score2) {
    rs.score2 = d->r_score2.p;
    rs.a_end2 = d->r_aend2.p;
  }
  return rs;
}

// Score2 mode: row-maxima arenas at the A offsets and the result arrays; the pair set
// then selects the forward kernels' score2 variants.
int attach_score2(mhsw_driver *d, mhsw::PairSet *ps, int64_t n, int64_t a_bytes) {
  ps->rowmax16 = ps->rowmax8 = nullptr;
  if (!d->score2 || n <= 0) return MHSW_OK;
  MHSW_CK(d->rowmax16.reserve((size_t)a_bytes + 16), "cudaMalloc row maxima");
  MHSW_CK(d->rowmax8.reserve((size_t)a_bytes + 16), "cudaMalloc row maxima");
  MHSW_CK(d->r_score2.reserve((size_t)n + 1), "cudaMalloc results");
  MHSW_CK(d->r_aend2.reserve((size_t)n + 1), "cudaMalloc results");
  ps->rowmax16 = d->rowmax16.p;
  ps->rowmax8 = d->rowmax8.p;
  return MHSW_OK;
}

float elapsed(cudaEvent_t a, cudaEvent_t b) {
  float ms = 0.f;
  if (cudaEventElapsedTime(&ms, a, b) != cudaSuccess) {
    cudaGetLastError();  // not sticky: keep it from surfacing as a later call's error
    return 0.f;
  }
  return ms;
}

// ---- CIGAR mode ------------------------------------------------------------------

int ensure_cigar(mhsw_driver *d, int64_t n) {
  MHSW_CK(d->c_nops.reserve((size_t)n + 1), "cudaMalloc CIGAR");
  MHSW_CK(d->c_mism.reserve((size_t)n + 1), "cudaMalloc CIGAR");
  MHSW_CK(d->c_off.reserve((size_t)n + 1), "cudaMalloc CIGAR");
  MHSW_CK(d->c_lists.reserve((size_t)mhsw::kCigarClasses * ((size_t)n + 1)), "cudaMalloc CIGAR lists");
  MHSW_CK(d->c_generic.reserve((size_t)n + 1), "cudaMalloc CIGAR lists");
  MHSW_CK(d->c_counts.reserve(mhsw::kCigarCounters), "cudaMalloc CIGAR");
  MHSW_CK(d->c_cursor.reserve(1), "cudaMalloc CIGAR");
  MHSW_CK(d->c_dirs.reserve(mhsw::kCigarDirBudget / sizeof(uint32_t)), "cudaMalloc CIGAR scratch");
  // 32 ops per pair on average before the arena has to grow (finish_cigar grows it)
  MHSW_CK(d->c_arena.reserve(std::max<size_t>((size_t)n * 32, 1 << 16)), "cudaMalloc CIGAR arena");
  MHSW_CK(d->h_ccounts.reserve(mhsw::kCigarCounters + 2), "cudaMallocHost");
  MHSW_CK(d->c_keys_in.reserve((size_t)n + 1), "cudaMalloc CIGAR sort");
  MHSW_CK(d->c_keys_out.reserve((size_t)n + 1), "cudaMalloc CIGAR sort");
  MHSW_CK(d->c_idx_in.reserve((size_t)n + 1), "cudaMalloc CIGAR sort");
  MHSW_CK(d->c_idx_out.reserve((size_t)n + 1), "cudaMalloc CIGAR sort");
  size_t tb = 0;
  MHSW_CK(mhsw::cigar_sort_temp_bytes(n, &tb), "CIGAR sort size");
  MHSW_CK(d->c_sort_temp.reserve(tb + 256), "cudaMalloc CIGAR sort");
  return MHSW_OK;
}

mhsw::CigarBufs cigar_bufs(mhsw_driver *d, int64_t n) {
  mhsw::CigarBufs cb;
  cb.nops = d->c_nops.p;
  cb.mism = d->c_mism.p;
  cb.op_off = d->c_off.p;
  cb.arena = d->c_arena.p;
  cb.arena_cap = (int64_t)d->c_arena.cap;
  cb.cursor = d->c_cursor.p;
  cb.counts = d->c_counts.p;
  cb.keys_in = d->c_keys_in.p;
  cb.keys_out = d->c_keys_out.p;
  cb.idx_in = d->c_idx_in.p;
  cb.idx_out = d->c_idx_out.p;
  cb.sort_temp = d->c_sort_temp.p;
  cb.sort_temp_bytes = d->c_sort_temp.cap;
  cb.lists = d->c_lists.p;
  cb.list_cap = n + 1;
  cb.generic = d->c_generic.p;
  cb.dirs = d->c_dirs.p;
  cb.dirs_bytes = d->c_dirs.cap * sizeof(uint32_t);
  return cb;
}

// Classification and the register-band kernels, then the counters' copy to the host
// (all stream-ordered; part of a captured graph when the batch is captured).
int enqueue_cigar(mhsw_driver *d, const mhsw::PairSet &ps) {
  MHSW_CK(mhsw::launch_cigar(ps, result_set(d), d->sc, cigar_bufs(d, ps.n), d->sms, d->fwd_order, d->st,
                              &d->launches),
          "CIGAR launch");
  MHSW_CK(cudaMemcpyAsync(d->h_ccounts.p, d->c_counts.p, sizeof(int) * mhsw::kCigarCounters, cudaMemcpyDeviceToHost,
                          d->st),
          "D2H CIGAR counters");
  return MHSW_OK;
}

// After the batch's stream work completed: grows the arena and runs the pass again when
// it filled up, and runs the generic kernel over the pairs the register kernels left
// (bands wider than 31 or boxes longer than kCigarRowCap rows), in rounds sized to a
// scratch budget.  Synchronous; rare work outside the captured graph.
int finish_cigar(mhsw_driver *d, const mhsw::PairSet &ps) {
  const int64_t n = ps.n;
  const auto t0 = std::chrono::steady_clock::now();
  d->cigar_generic = 0;
  bool generic_done = false;
  for (int round = 0; round < 4; round++) {
    const int *cnt = d->h_ccounts.p;
    if (cnt[mhsw::kCigarArenaFull] > 0) {  // arena full: grow to what was asked for, run again
      unsigned long long need = 0;
      MHSW_CK(cudaMemcpy(&need, d->c_cursor.p, sizeof(need), cudaMemcpyDeviceToHost), "D2H cursor");
      MHSW_CK(d->c_arena.reserve((size_t)need + (size_t)n * 8 + 1024), "cudaMalloc CIGAR arena");
      int rc = enqueue_cigar(d, ps);
      if (rc) return rc;
      MHSW_CK(cudaStreamSynchronize(d->st), "sync");
      generic_done = false;
      continue;
    }
    const int ng = cnt[mhsw::kCigarGeneric];
    if (ng > 0 && !generic_done) {
      generic_done = true;
      d->cigar_generic = ng;
      std::vector<int4> ent((size_t)ng);
      MHSW_CK(cudaMemcpy(ent.data(), d->c_generic.p, sizeof(int4) * ng, cudaMemcpyDeviceToHost), "D2H generic list");
      // the widest band a box can need: doubling from w stops once it covers the box
      auto slice_of = [](const int4 &e) {
        int w = e.y;
        while (w < std::max(e.z, e.w)) w *= 2;
        return (mhsw::cigar_slice_bytes(w, e.z) + 15) / 16 * 16;
      };
      std::sort(ent.begin(), ent.end(), [&](const int4 &a, const int4 &b) { return slice_of(a) > slice_of(b); });
      MHSW_CK(d->c_gsorted.reserve((size_t)ng), "cudaMalloc generic list");
      MHSW_CK(cudaMemcpy(d->c_gsorted.p, ent.data(), sizeof(int4) * ng, cudaMemcpyHostToDevice), "H2D generic list");
      const size_t budget = size_t(1) << 30;
      size_t at = 0;
      while (at < (size_t)ng) {
        const size_t slice = slice_of(ent[at]);
        size_t end = at + 1;
        while (end < (size_t)ng && slice_of(ent[end]) * 2 > slice) end++;  // same size class
        const size_t pool = std::max(budget, slice);
        const int threads = (int)std::max<size_t>(1, std::min<size_t>({end - at, pool / slice, 8192}));
        MHSW_CK(d->c_pool.reserve(slice * (size_t)threads), "cudaMalloc CIGAR pool");
        MHSW_CK(mhsw::launch_cigar_generic(ps, result_set(d), d->sc, cigar_bufs(d, n), d->c_gsorted.p + at,
                                           (int)(end - at), threads, slice, d->c_pool.p, d->st),
                "CIGAR generic launch");
        d->launches += 1;
        at = end;
      }
      MHSW_CK(cudaMemcpyAsync(d->h_ccounts.p, d->c_counts.p, sizeof(int) * mhsw::kCigarCounters,
                              cudaMemcpyDeviceToHost, d->st),
              "D2H CIGAR counters");
      MHSW_CK(cudaStreamSynchronize(d->st), "sync");
      continue;  // the generic kernel may have found the arena full
    }
    break;
  }
  if (d->h_ccounts.p[mhsw::kCigarArenaFull] > 0)
    return d->fail(MHSW_ERR_INTERNAL, "CIGAR arena still full after growing it");
  d->cigar_n = n;
  d->cigar_total = -1;
  d->cigar_ms = elapsed(d->ev_c[0], d->ev_c[1]) +
                std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  return MHSW_OK;
}

mhsw::WorkLists work_lists(mhsw_driver *d, int64_t n) {
  mhsw::WorkLists wl;
  wl.ovf = d->l_ovf.p;
  wl.wide = d->l_wide.p;
  wl.ovf_count = d->l_counts.p;
  wl.wide_count = d->l_counts.p + 1;
  wl.bands = d->l_bands.p;
  wl.band_counts = d->l_counts.p + 2;
  wl.cap = n;
  return wl;
}

// Scratch for multi-strip A (rows longer than one wavefront strip).
int ensure_scratch(mhsw_driver *d, int max_a, int max_b, mhsw::FwdConfig *c16, mhsw::FwdConfig *c32, size_t *bytes) {
  size_t need16 = mhsw::forward_scratch_bytes(*c16, max_a, max_b, false);
  // the int32 paths (re-runs, wide begins) use a smaller grid when strips are needed
  c32->grid = std::min(c32->grid, 152 * 2);
  size_t need32 = mhsw::forward_scratch_bytes(*c32, max_a, max_b, true);
  size_t need = std::max(need16, need32);
  if (need > 0) MHSW_CK(d->scratch.reserve(need), "cudaMalloc scratch");
  *bytes = need > 0 ? d->scratch.cap : 0;
  return MHSW_OK;
}

// Translates both arenas of a batch into base codes (driver-owned buffers) and points
// the PairSet at them.
int translate_batch(mhsw_driver *d, mhsw::PairSet *ps, int64_t a_bytes, int64_t b_bytes) {
  MHSW_CK(d->a_code.reserve((size_t)a_bytes + 16), "cudaMalloc codes");
  MHSW_CK(d->b_code.reserve((size_t)b_bytes + 16), "cudaMalloc codes");
  MHSW_CK(mhsw::launch_translate(ps->a_seq, d->a_code.p, a_bytes, d->st), "translate A");
  MHSW_CK(mhsw::launch_translate(ps->b_seq, d->b_code.p, b_bytes, d->st), "translate B");
  d->launches += 2;
  ps->a_code = d->a_code.p;
  ps->b_code = d->b_code.p;
  return MHSW_OK;
}

// Forward pass over the staged PairSet: int16 engine, then int32 re-runs of the pairs
// whose score crossed the ceiling.  Device-side lists; no host synchronisation.
// Effective int16 ceiling: the keyed engine holds scores below mhsw::kCeiling16.
int ceiling_for(mhsw_driver *d) {
  return mhsw::keyed_scoring(d->sc) ? std::min(d->ceiling16, mhsw::kCeiling16) : d->ceiling16;
}

int run_forward(mhsw_driver *d, const mhsw::PairSet &ps, int max_a, int max_b, bool persistent_grid) {
  mhsw::FwdConfig c16, c32;
  cudaError_t e = mhsw::plan_forward(d->device, max_a, max_b, false, &c16, mhsw::keyed_scoring(d->sc),
                                     ps.rowmax16 != nullptr);
  if (e != cudaSuccess) return d->fail(MHSW_ERR_LIMIT, "B length %d exceeds the kernel limit %d", max_b, mhsw::kMaxB);
  e = mhsw::plan_forward(d->device, max_a, max_b, true, &c32);
  if (e != cudaSuccess) return d->fail(MHSW_ERR_LIMIT, "B length %d exceeds the kernel limit %d", max_b, mhsw::kMaxB);
  const bool strips16 = max_a > 2 * c16.K * c16.G;
  if (!persistent_grid && !strips16) {
    int64_t g = (ps.n + c16.groups_per_block - 1) / c16.groups_per_block;
    c16.grid = (int)std::max<int64_t>(1, std::min<int64_t>(g, 1 << 30));
  }
  size_t scr_bytes = 0;
  int rc = ensure_scratch(d, max_a, max_b, &c16, &c32, &scr_bytes);
  if (rc) return rc;
  mhsw::ResultSet rs = result_set(d);
  mhsw::WorkLists wl = work_lists(d, ps.n);
  MHSW_CK(mhsw::reset_lists(wl, d->st), "reset lists");
  MHSW_CK(mhsw::launch_forward(c16, false, ps, rs, d->sc, nullptr, nullptr, ceiling_for(d), d->scratch.p, wl, d->st),
          "forward int16 launch");
  MHSW_CK(mhsw::launch_forward(c32, true, ps, rs, d->sc, wl.ovf, wl.ovf_count, 0x7fffffff, d->scratch.p, wl, d->st),
          "forward int32 launch");
  d->launches += 3;
  return MHSW_OK;
}

// Forward pass in either form; lists are reset first so both passes see fresh counters.
int forward_passes(mhsw_driver *d, const mhsw::PairSet &ps, int max_a, int max_b, int form);

// Forward pass, then (score2 mode) the second-best scores from the row maxima it wrote.
int forward_any(mhsw_driver *d, const mhsw::PairSet &ps, int max_a, int max_b, int form) {
  d->score2_n = -1;
  int rc = forward_passes(d, ps, max_a, max_b, form);
  if (rc || !ps.rowmax16) return rc;
  MHSW_CK(mhsw::launch_score2(ps, result_set(d), d->sc, d->st), "score2 launch");
  d->launches += 1;
  d->score2_n = ps.n;
  return MHSW_OK;
}

int forward_passes(mhsw_driver *d, const mhsw::PairSet &ps, int max_a, int max_b, int form) {
  // The batched form runs the keyed int16 engine; scorings it cannot hold (a mismatch or
  // ambiguity penalty above the gap-open penalty) use the plain form.
  d->fwd_order = nullptr;
  if (form != MHSW_FORM_BATCHED || !mhsw::keyed_scoring(d->sc)) return run_forward(d, ps, max_a, max_b, false);
  mhsw::WorkLists wl = work_lists(d, ps.n);
  MHSW_CK(mhsw::reset_lists(wl, d->st), "reset lists");
  d->launches += 1;
  if (mhsw::batched_forward(d->batch, d->device, ps, result_set(d), wl, d->sc, ceiling_for(d), max_a, max_b, d->sig,
                            d->st, &d->launches, &d->forks))
    return d->fail(MHSW_ERR_CUDA, "batched forward: %s", d->batch.err.c_str());
  d->fwd_order = d->batch.idx_out;
  // int32 pass over the pairs the int16 engine could not hold
  mhsw::FwdConfig c16, c32;
  if (mhsw::plan_forward(d->device, max_a, max_b, false, &c16, false, ps.rowmax16 != nullptr) != cudaSuccess ||
      mhsw::plan_forward(d->device, max_a, max_b, true, &c32) != cudaSuccess)
    return d->fail(MHSW_ERR_LIMIT, "B length %d exceeds the kernel limit %d", max_b, mhsw::kMaxB);
  size_t sb = 0;
  int rc = ensure_scratch(d, max_a, max_b, &c16, &c32, &sb);
  if (rc) return rc;
  MHSW_CK(mhsw::launch_forward(c32, true, ps, result_set(d), d->sc, wl.ovf, wl.ovf_count, 0x7fffffff, d->scratch.p,
                               wl, d->st),
          "forward int32 launch");
  d->launches += 1;
  return MHSW_OK;
}

int run_reverse(mhsw_driver *d, const mhsw::PairSet &ps, int max_a, int max_b, const uint32_t *order) {
  mhsw::ResultSet rs = result_set(d);
  mhsw::WorkLists wl = work_lists(d, ps.n);
  MHSW_CK(mhsw::launch_reverse(d->device, ps, rs, d->sc, max_a, max_b, d->scratch.p,
                               d->scratch.p ? d->scratch.cap : 0, wl, d->st, order, &d->forks),
          "begin pass launch");
  d->launches += 10;
  return MHSW_OK;
}

// Output views on the device: [5 x int16 arrays][5 x int32 arrays], n each.
int ensure_outviews(mhsw_driver *d, int64_t n, mhsw::OutViews *dv, mhsw::OutViews *hv) {
  size_t bytes = (size_t)n * (5 * sizeof(int16_t) + 5 * sizeof(int32_t)) + 64;
  MHSW_CK(d->outv.reserve(bytes), "cudaMalloc outputs");
  MHSW_CK(d->h_outv.reserve(bytes), "cudaMallocHost outputs");
  auto carve = [n](unsigned char *base, mhsw::OutViews *v) {
    int16_t *s = reinterpret_cast<int16_t *>(base);
    v->s_score = s;
    v->s_ref_beg = s + n;
    v->s_ref_end = s + 2 * n;
    v->s_qry_beg = s + 3 * n;
    v->s_qry_end = s + 4 * n;
    size_t off = ((size_t)n * 5 * sizeof(int16_t) + 15) / 16 * 16;
    int32_t *w = reinterpret_cast<int32_t *>(base + off);
    v->w_score = w;
    v->w_ref_beg = w + n;
    v->w_ref_end = w + 2 * n;
    v->w_qry_beg = w + 3 * n;
    v->w_qry_end = w + 4 * n;
  };
  carve(d->outv.p, dv);
  carve(d->h_outv.p, hv);
  return MHSW_OK;
}

int check_scoring(mhsw_driver *d, const mhsw::Scoring &s) {
  if (s.match < 0 || s.mismatch < 0 || s.ambiguity < 0 || s.gap_open < 1 || s.gap_extend < 1)
    return d->fail(MHSW_ERR_ARG,
                   "scores must be match >= 0 and mismatch/ambiguity <= 0, gap open/extend <= -1 (negated penalties)");
  if (s.match > 127 || s.mismatch > 127 || s.ambiguity > 127 || s.gap_open > 127 || s.gap_extend > 127)
    return d->fail(MHSW_ERR_ARG, "score magnitudes above 127 are not supported");
  return MHSW_OK;
}

// Stage a drop-in batch (pointer arrays) into pinned memory and on to the device.
int stage_strings(mhsw_driver *d, const char *const *reads, const int32_t *read_lens, const char *const *contigs,
                  const int32_t *contig_lens, int32_t n) {
  const bool a_is_read = d->orientation == MHSW_ORIENT_KLIGN;
  const char *const *as = a_is_read ? reads : contigs;
  const int32_t *al = a_is_read ? read_lens : contig_lens;
  const char *const *bs = a_is_read ? contigs : reads;
  const int32_t *bl = a_is_read ? contig_lens : read_lens;
  int64_t ta = 0, tb = 0;
  int ma = 0, mb = 0;
  for (int32_t i = 0; i < n; i++) {
    if (al[i] < 0 || bl[i] < 0) return d->fail(MHSW_ERR_ARG, "negative length at pair %d", i);
    ta += al[i];
    tb += bl[i];
    ma = std::max(ma, (int)al[i]);
    mb = std::max(mb, (int)bl[i]);
  }
  if (mb > mhsw::kMaxB) return d->fail(MHSW_ERR_LIMIT, "sequence of %d bytes exceeds the limit %d", mb, mhsw::kMaxB);
  MHSW_CK(d->h_a.reserve((size_t)ta + 16), "cudaMallocHost");
  MHSW_CK(d->h_b.reserve((size_t)tb + 16), "cudaMallocHost");
  MHSW_CK(d->h_aoff.reserve((size_t)n + 1), "cudaMallocHost");
  MHSW_CK(d->h_boff.reserve((size_t)n + 1), "cudaMallocHost");
  MHSW_CK(d->h_alen.reserve((size_t)n + 1), "cudaMallocHost");
  MHSW_CK(d->h_blen.reserve((size_t)n + 1), "cudaMallocHost");
  int64_t oa = 0, ob = 0;
  for (int32_t i = 0; i < n; i++) {
    d->h_aoff.p[i] = oa;
    d->h_boff.p[i] = ob;
    d->h_alen.p[i] = al[i];
    d->h_blen.p[i] = bl[i];
    oa += al[i];
    ob += bl[i];
  }
  // the bytes, in parts of about 1 MB on the handle's copy threads
  const int parts = (int)std::min<int64_t>(std::max<int64_t>((ta + tb) >> 20, 1), std::max(n, 1));
  const std::function<void(int)> copy_part = [&](int part) {
    const int32_t lo = (int32_t)((int64_t)n * part / parts), hi = (int32_t)((int64_t)n * (part + 1) / parts);
    for (int32_t i = lo; i < hi; i++) {
      if (al[i]) memcpy(d->h_a.p + d->h_aoff.p[i], as[i], (size_t)al[i]);
      if (bl[i]) memcpy(d->h_b.p + d->h_boff.p[i], bs[i], (size_t)bl[i]);
    }
  };
  d->copy_pool.run(parts, copy_part);
  int rc = ensure_device(d, n, ta, tb);
  if (rc) return rc;
  rc = ensure_results(d, n);
  if (rc) return rc;
  MHSW_CK(cudaMemcpyAsync(d->a_seq.p, d->h_a.p, (size_t)ta, cudaMemcpyHostToDevice, d->st), "H2D");
  MHSW_CK(cudaMemcpyAsync(d->b_seq.p, d->h_b.p, (size_t)tb, cudaMemcpyHostToDevice, d->st), "H2D");
  MHSW_CK(cudaMemcpyAsync(d->a_off.p, d->h_aoff.p, sizeof(int64_t) * n, cudaMemcpyHostToDevice, d->st), "H2D");
  MHSW_CK(cudaMemcpyAsync(d->b_off.p, d->h_boff.p, sizeof(int64_t) * n, cudaMemcpyHostToDevice, d->st), "H2D");
  MHSW_CK(cudaMemcpyAsync(d->a_len.p, d->h_alen.p, sizeof(int32_t) * n, cudaMemcpyHostToDevice, d->st), "H2D");
  MHSW_CK(cudaMemcpyAsync(d->b_len.p, d->h_blen.p, sizeof(int32_t) * n, cudaMemcpyHostToDevice, d->st), "H2D");
  d->max_a = ma;
  d->max_b = mb;
  d->n_batch = n;
  d->a_bytes = ta;
  d->b_bytes = tb;
  double cells = 0;
  for (int32_t i = 0; i < n; i++) cells += (double)al[i] * (double)bl[i];
  d->fwd_cells = cells;
  return MHSW_OK;
}

mhsw::PairSet staged_pairs(mhsw_driver *d) {
  mhsw::PairSet ps;
  ps.a_seq = d->a_seq.p;
  ps.a_off = d->a_off.p;
  ps.a_len = d->a_len.p;
  ps.b_seq = d->b_seq.p;
  ps.b_off = d->b_off.p;
  ps.b_len = d->b_len.p;
  ps.n = d->n_batch;
  ps.a_code = d->a_code.p;
  ps.b_code = d->b_code.p;
  return ps;
}

// A host batch into input set `in`: arenas in 64 MB pieces and the offsets and lengths,
// spread over the copy streams; the handle's stream waits for all of them.  after_free:
// the copy streams wait only for the set's previous call (its free event), not for the
// work on the handle's stream, so the copies overlap the previous call's kernels;
// otherwise they wait for everything issued on the handle's stream so far.
int copy_batch_in(mhsw_driver *d, mhsw_driver::InSet &in, const mhsw_pairs *pairs, int64_t n, int64_t ta,
                  int64_t tb, bool after_free, int slot) {
  constexpr size_t kPiece = size_t(64) << 20;
  constexpr int kLanes = mhsw_driver::kCopyStreams;
  if (!after_free) MHSW_CK(cudaEventRecord(d->copy_ev[0], d->st), "event");
  for (int k = 0; k < kLanes; k++) {
    if (after_free) {
      if (in.used) MHSW_CK(cudaStreamWaitEvent(d->copy_st[k], in.free_ev, 0), "wait input set");
      // calls copy in one after another: the first of several calls enqueued together
      // then gets the whole copy bandwidth instead of sharing it, and its kernels start
      // as early as they can (the later calls' copies still run under its kernels)
      for (int m = 0; m < kLanes; m++)
        if (m != k) MHSW_CK(cudaStreamWaitEvent(d->copy_st[k], d->copy_ev[m], 0), "wait previous copies");
    } else {
      MHSW_CK(cudaStreamWaitEvent(d->copy_st[k], d->copy_ev[0], 0), "wait stream");
    }
  }
  MHSW_CK(cudaEventRecord(d->ev_cin[slot][0], d->copy_st[0]), "event");
  int lane = 0;
  auto put = [&](void *dst, const void *src, size_t len) -> cudaError_t {
    for (size_t o = 0; o < len; o += kPiece) {
      const size_t k = std::min(kPiece, len - o);
      cudaError_t e = cudaMemcpyAsync(static_cast<char *>(dst) + o, static_cast<const char *>(src) + o, k,
                                      cudaMemcpyHostToDevice, d->copy_st[lane]);
      if (e) return e;
      lane = (lane + 1) % kLanes;
    }
    return cudaSuccess;
  };
  MHSW_CK(put(in.a_seq.p, pairs->a_seq, (size_t)ta), "H2D");
  MHSW_CK(put(in.b_seq.p, pairs->b_seq, (size_t)tb), "H2D");
  MHSW_CK(put(in.a_off.p, pairs->a_off, sizeof(int64_t) * n), "H2D");
  MHSW_CK(put(in.b_off.p, pairs->b_off, sizeof(int64_t) * n), "H2D");
  MHSW_CK(put(in.a_len.p, pairs->a_len, sizeof(int32_t) * n), "H2D");
  MHSW_CK(put(in.b_len.p, pairs->b_len, sizeof(int32_t) * n), "H2D");
  for (int k = 0; k < kLanes; k++) {
    MHSW_CK(cudaEventRecord(d->ev_cin[slot][1 + k], d->copy_st[k]), "event");
    MHSW_CK(cudaEventRecord(d->copy_ev[k], d->copy_st[k]), "event");
    MHSW_CK(cudaStreamWaitEvent(d->st, d->copy_ev[k], 0), "wait copies");
  }
  d->cin_recorded[slot] = true;
  return MHSW_OK;
}

int ready(mhsw_driver *d) {
  if (!d) return MHSW_ERR_ARG;
  if (!d->inited) return d->fail(MHSW_ERR_STATE, "driver not initialised (call mhsw_driver_init)");
  MHSW_CK(cudaSetDevice(d->device), "cudaSetDevice");
  return MHSW_OK;
}

}  // namespace

extern "C" {

int mhsw_get_num_node_gpus(int *count) {
  if (!count) return MHSW_ERR_ARG;
  int c = 0;
  if (cudaGetDeviceCount(&c) != cudaSuccess) {
    cudaGetLastError();
    c = 0;
  }
  *count = c;
  return MHSW_OK;
}

int mhsw_get_tot_gpu_mem(size_t *bytes) {
  if (!bytes) return MHSW_ERR_ARG;
  cudaDeviceProp prop;
  cudaError_t e = cudaGetDeviceProperties(&prop, 0);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return MHSW_ERR_CUDA;
  }
  *bytes = prop.totalGlobalMem;
  return MHSW_OK;
}

int mhsw_get_avail_gpu_mem_per_rank(int tot_ranks, int num_devices, size_t *bytes) {
  if (!bytes) return MHSW_ERR_ARG;
  *bytes = 0;
  if (num_devices == 0) mhsw_get_num_node_gpus(&num_devices);
  if (num_devices <= 0) return MHSW_OK;
  int ranks_per_device = tot_ranks / num_devices;
  if (ranks_per_device < 1) ranks_per_device = 1;
  size_t tot = 0;
  int rc = mhsw_get_tot_gpu_mem(&tot);
  if (rc) return rc;
  *bytes = (size_t)((double)tot * 0.8) / (size_t)ranks_per_device;
  return MHSW_OK;
}

int mhsw_get_device_name(int device_id, char *buf, size_t buflen) {
  if (!buf || buflen == 0) return MHSW_ERR_ARG;
  cudaError_t e = cudaDeviceGetPCIBusId(buf, (int)buflen, device_id);
  if (e != cudaSuccess) {
    cudaGetLastError();
    buf[0] = 0;
    return MHSW_ERR_CUDA;
  }
  return MHSW_OK;
}

int mhsw_initialize_gpu(double *seconds, int *device_count, size_t *total_mem) {
  auto t0 = std::chrono::steady_clock::now();
  int c = 0;
  mhsw_get_num_node_gpus(&c);
  size_t tot = 0;
  if (c > 0) {
    mhsw_get_tot_gpu_mem(&tot);
    double *first_touch = nullptr;
    if (cudaMallocHost(&first_touch, sizeof(double)) == cudaSuccess) cudaFreeHost(first_touch);
  }
  if (seconds) *seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  if (device_count) *device_count = c;
  if (total_mem) *total_mem = tot;
  return c > 0 ? MHSW_OK : MHSW_ERR_NO_GPU;
}

int mhsw_limits(mhsw_limits_t *out) {
  if (!out) return MHSW_ERR_ARG;
  out->max_b_len = mhsw::kMaxB;
  out->max_coord = 0xFFFFF;
  out->int16_ceiling = mhsw::kCeiling16;
  return MHSW_OK;
}

int mhsw_driver_create(mhsw_driver **out) {
  if (!out) return MHSW_ERR_ARG;
  *out = new (std::nothrow) mhsw_driver();
  return *out ? MHSW_OK : MHSW_ERR_NOMEM;
}

void mhsw_driver_destroy(mhsw_driver *drv) { delete drv; }

const char *mhsw_driver_last_error(const mhsw_driver *drv) { return drv ? drv->err.c_str() : "null driver"; }

int mhsw_driver_init(mhsw_driver *d, int rank_me, int rank_n, short match_score, short mismatch_score,
                     short gap_opening_score, short gap_extending_score, int rlen_limit, double *seconds) {
  if (!d) return MHSW_ERR_ARG;
  std::lock_guard<std::mutex> lk(d->mu);
  auto t0 = std::chrono::steady_clock::now();
  (void)rank_n;
  mhsw::Scoring s{match_score, -mismatch_score, -gap_opening_score, -gap_extending_score, d->sc.ambiguity};
  int rc = check_scoring(d, s);
  if (rc) return rc;
  int count = 0;
  mhsw_get_num_node_gpus(&count);
  if (count <= 0) return d->fail(MHSW_ERR_NO_GPU, "no CUDA device");
  if (d->inited) return d->fail(MHSW_ERR_STATE, "driver already initialised");
  d->device = (rank_me < 0 ? 0 : rank_me) % count;
  MHSW_CK(cudaSetDevice(d->device), "cudaSetDevice");
  MHSW_CK(cudaStreamCreateWithFlags(&d->st, cudaStreamNonBlocking), "cudaStreamCreate");
  MHSW_CK(cudaEventCreateWithFlags(&d->ev_done, cudaEventDisableTiming), "cudaEventCreate");
  MHSW_CK(mhsw::forks_create(d->forks), "side streams");
  for (auto &e : d->ev_t) MHSW_CK(cudaEventCreate(&e), "cudaEventCreate");
  for (auto &e : d->ev_c) MHSW_CK(cudaEventCreate(&e), "cudaEventCreate");
  for (auto &row : d->ev_p)
    for (auto &e : row) MHSW_CK(cudaEventCreate(&e), "cudaEventCreate");
  for (auto &row : d->ev_cin)
    for (auto &e : row) MHSW_CK(cudaEventCreate(&e), "cudaEventCreate");
  MHSW_CK(cudaEventCreate(&d->ev_epoch), "cudaEventCreate");
  MHSW_CK(cudaEventRecord(d->ev_epoch, d->st), "event");
  for (auto &in : d->in_sets) MHSW_CK(cudaEventCreateWithFlags(&in.free_ev, cudaEventDisableTiming), "cudaEventCreate");
  for (auto &c : d->copy_st) MHSW_CK(cudaStreamCreateWithFlags(&c, cudaStreamNonBlocking), "cudaStreamCreate");
  for (auto &e : d->copy_ev) MHSW_CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming), "cudaEventCreate");
  MHSW_CK(cudaDeviceGetAttribute(&d->sms, cudaDevAttrMultiProcessorCount, d->device), "device attribute");
  d->sc = s;
  d->inited = true;
  // Pre-size for a reference-sized block (KLIGN_GPU_BLOCK_SIZE = 20000 pairs).
  if (rlen_limit > 0) {
    const int64_t n = 20000;
    int r2 = ensure_device(d, n, (int64_t)rlen_limit * n, (int64_t)2 * rlen_limit * n);
    if (r2) return r2;
    r2 = ensure_results(d, n);
    if (r2) return r2;
  }
  if (seconds) *seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  return MHSW_OK;
}

int mhsw_driver_set_ambiguity(mhsw_driver *d, short ambiguity_score) {
  if (!d) return MHSW_ERR_ARG;
  std::lock_guard<std::mutex> lk(d->mu);
  mhsw::Scoring s = d->sc;
  s.ambiguity = -ambiguity_score;
  if (!d->inited) {
    // allow setting before init: validate the ambiguity alone
    if (s.ambiguity < 0 || s.ambiguity > 127) return d->fail(MHSW_ERR_ARG, "ambiguity score must be in [-127, 0]");
    d->sc.ambiguity = s.ambiguity;
    return MHSW_OK;
  }
  int rc = check_scoring(d, s);
  if (rc) return rc;
  d->sc = s;
  return MHSW_OK;
}

int mhsw_driver_set_orientation(mhsw_driver *d, int orientation) {
  if (!d) return MHSW_ERR_ARG;
  if (orientation != MHSW_ORIENT_KLIGN && orientation != MHSW_ORIENT_REF_IS_A)
    return d->fail(MHSW_ERR_ARG, "unknown orientation %d", orientation);
  std::lock_guard<std::mutex> lk(d->mu);
  d->orientation = orientation;
  return MHSW_OK;
}

int mhsw_driver_set_form(mhsw_driver *d, int form) {
  if (!d) return MHSW_ERR_ARG;
  if (form != MHSW_FORM_PLAIN && form != MHSW_FORM_BATCHED) return d->fail(MHSW_ERR_ARG, "unknown form %d", form);
  std::lock_guard<std::mutex> lk(d->mu);
  d->form = form;
  return MHSW_OK;
}

int mhsw_driver_set_int16_ceiling(mhsw_driver *d, int ceiling) {
  if (!d) return MHSW_ERR_ARG;
  if (ceiling < 0 || ceiling > kInt16Ceiling)
    return d->fail(MHSW_ERR_ARG, "ceiling must be in [0, %d]", kInt16Ceiling);
  std::lock_guard<std::mutex> lk(d->mu);
  d->ceiling16 = ceiling;
  return MHSW_OK;
}

int mhsw_driver_stream(mhsw_driver *d, void **stream) {
  if (!d || !stream) return MHSW_ERR_ARG;
  if (!d->inited) return d->fail(MHSW_ERR_STATE, "driver not initialised");
  *stream = (void *)d->st;
  return MHSW_OK;
}

int mhsw_run_kernel_forwards(mhsw_driver *d, const char *const *reads, const int32_t *read_lens,
                             const char *const *contigs, const int32_t *contig_lens, int32_t n,
                             uint32_t max_read_size, uint32_t max_contig_size) {
  int rc = ready(d);
  if (rc) return rc;
  std::lock_guard<std::mutex> lk(d->mu);
  if (int rcp = finish_pending(d)) return rcp;
  if (n < 0 || (n > 0 && (!reads || !read_lens || !contigs || !contig_lens)))
    return d->fail(MHSW_ERR_ARG, "bad batch arguments");
  for (int32_t i = 0; i < n; i++)
    if ((uint32_t)read_lens[i] > max_read_size || (uint32_t)contig_lens[i] > max_contig_size)
      return d->fail(MHSW_ERR_ARG, "pair %d longer than max_read_size/max_contig_size", i);
  if (d->ev_live) MHSW_CK(cudaEventSynchronize(d->ev_done), "wait previous batch");
  d->ev_live = false;
  d->fwd_issued = d->rev_issued = false;
  d->launches = 0;
  d->cigar_n = -1;
  MHSW_CK(cudaEventRecord(d->ev_t[0], d->st), "event");
  rc = stage_strings(d, reads, read_lens, contigs, contig_lens, n);
  if (rc) return rc;
  d->sig = mhsw::batch_signature(d->orientation == MHSW_ORIENT_KLIGN ? read_lens : contig_lens, n, d->max_a,
                                 d->max_b);
  mhsw::PairSet ps = staged_pairs(d);
  if (n > 0) {
    rc = translate_batch(d, &ps, d->a_bytes, d->b_bytes);
    if (rc) return rc;
  }
  rc = attach_score2(d, &ps, n, d->a_bytes);
  if (rc) return rc;
  MHSW_CK(cudaEventRecord(d->ev_t[1], d->st), "event");
  if (n > 0) {
    rc = forward_any(d, ps, d->max_a, d->max_b, d->form);
    if (rc) return rc;
    if (ps.rowmax16) {
      MHSW_CK(d->h_score2.reserve(2 * (size_t)n), "cudaMallocHost");
      MHSW_CK(cudaMemcpyAsync(d->h_score2.p, d->r_score2.p, sizeof(int32_t) * n, cudaMemcpyDeviceToHost, d->st),
              "D2H");
      MHSW_CK(cudaMemcpyAsync(d->h_score2.p + n, d->r_aend2.p, sizeof(int32_t) * n, cudaMemcpyDeviceToHost, d->st),
              "D2H");
    }
  }
  MHSW_CK(cudaEventRecord(d->ev_t[2], d->st), "event");
  mhsw::OutViews dv, hv;
  rc = ensure_outviews(d, std::max<int64_t>(n, 1), &dv, &hv);
  if (rc) return rc;
  const bool a_is_query = d->orientation == MHSW_ORIENT_KLIGN;
  if (n > 0) {
    MHSW_CK(mhsw::launch_finalize(result_set(d), n, a_is_query, 1, dv, d->st), "finalize");
    d->launches += 1;
    int16_t *srcs[3] = {dv.s_score, dv.s_ref_end, dv.s_qry_end};
    int16_t *dsts[3] = {hv.s_score, hv.s_ref_end, hv.s_qry_end};
    for (int k = 0; k < 3; k++)
      MHSW_CK(cudaMemcpyAsync(dsts[k], srcs[k], sizeof(int16_t) * n, cudaMemcpyDeviceToHost, d->st), "D2H");
    int32_t *wsrc[3] = {dv.w_score, dv.w_ref_end, dv.w_qry_end};
    int32_t *wdst[3] = {hv.w_score, hv.w_ref_end, hv.w_qry_end};
    for (int k = 0; k < 3; k++)
      MHSW_CK(cudaMemcpyAsync(wdst[k], wsrc[k], sizeof(int32_t) * n, cudaMemcpyDeviceToHost, d->st), "D2H");
  }
  MHSW_CK(cudaEventRecord(d->ev_t[3], d->st), "event");
  MHSW_CK(cudaEventRecord(d->ev_done, d->st), "event");
  d->ev_live = true;
  d->fwd_issued = true;
  return MHSW_OK;
}

int mhsw_run_kernel_backwards(mhsw_driver *d, const char *const *reads, const int32_t *read_lens,
                              const char *const *contigs, const int32_t *contig_lens, int32_t n,
                              uint32_t max_read_size, uint32_t max_contig_size) {
  int rc = ready(d);
  if (rc) return rc;
  std::lock_guard<std::mutex> lk(d->mu);
  if (int rcp = finish_pending(d)) return rcp;
  (void)reads;
  (void)read_lens;
  (void)contigs;
  (void)contig_lens;
  (void)max_read_size;
  (void)max_contig_size;
  if (!d->fwd_issued) return d->fail(MHSW_ERR_STATE, "run_kernel_backwards without a preceding run_kernel_forwards");
  if ((int64_t)n != d->n_batch)
    return d->fail(MHSW_ERR_ARG, "batch size %d differs from the forward batch (%lld)", n, (long long)d->n_batch);
  mhsw::PairSet ps = staged_pairs(d);
  MHSW_CK(cudaEventRecord(d->ev_t[4], d->st), "event");
  d->cigar_n = -1;
  if (n > 0) {
    rc = run_reverse(d, ps, d->max_a, d->max_b, d->fwd_order);
    if (rc) return rc;
    if (d->cigar) {
      rc = ensure_cigar(d, n);
      if (rc) return rc;
      MHSW_CK(cudaEventRecord(d->ev_c[0], d->st), "event");
      rc = enqueue_cigar(d, ps);
      if (rc) return rc;
      MHSW_CK(cudaEventRecord(d->ev_c[1], d->st), "event");
    }
  }
  mhsw::OutViews dv, hv;
  rc = ensure_outviews(d, std::max<int64_t>(n, 1), &dv, &hv);
  if (rc) return rc;
  const bool a_is_query = d->orientation == MHSW_ORIENT_KLIGN;
  if (n > 0) {
    MHSW_CK(mhsw::launch_finalize(result_set(d), n, a_is_query, 2, dv, d->st), "finalize");
    d->launches += 1;
    int16_t *srcs[2] = {dv.s_ref_beg, dv.s_qry_beg};
    int16_t *dsts[2] = {hv.s_ref_beg, hv.s_qry_beg};
    for (int k = 0; k < 2; k++)
      MHSW_CK(cudaMemcpyAsync(dsts[k], srcs[k], sizeof(int16_t) * n, cudaMemcpyDeviceToHost, d->st), "D2H");
    int32_t *wsrc[2] = {dv.w_ref_beg, dv.w_qry_beg};
    int32_t *wdst[2] = {hv.w_ref_beg, hv.w_qry_beg};
    for (int k = 0; k < 2; k++)
      MHSW_CK(cudaMemcpyAsync(wdst[k], wsrc[k], sizeof(int32_t) * n, cudaMemcpyDeviceToHost, d->st), "D2H");
    MHSW_CK(cudaMemcpyAsync(d->h_counts.reserve(4) == cudaSuccess ? d->h_counts.p : nullptr, d->l_counts.p,
                            2 * sizeof(int), cudaMemcpyDeviceToHost, d->st),
            "D2H counters");
  }
  MHSW_CK(cudaEventRecord(d->ev_t[5], d->st), "event");
  MHSW_CK(cudaEventRecord(d->ev_done, d->st), "event");
  d->ev_live = true;
  d->rev_issued = true;
  return MHSW_OK;
}

int mhsw_kernel_is_done(mhsw_driver *d, int *done) {
  if (!d || !done) return MHSW_ERR_ARG;
  std::lock_guard<std::mutex> lk(d->mu);
  if (!d->ev_live) {
    *done = 1;
    return MHSW_OK;
  }
  cudaError_t e = cudaEventQuery(d->ev_done);
  if (e == cudaErrorNotReady) {
    *done = 0;
    return MHSW_OK;
  }
  if (e != cudaSuccess) return d->cuda_fail(e, "cudaEventQuery");
  *done = 1;
  return MHSW_OK;
}

int mhsw_kernel_block(mhsw_driver *d) {
  if (!d) return MHSW_ERR_ARG;
  std::lock_guard<std::mutex> lk(d->mu);
  if (!d->ev_live) return MHSW_OK;
  MHSW_CK(cudaEventSynchronize(d->ev_done), "cudaEventSynchronize");
  if (d->rev_issued && d->cigar && d->n_batch > 0 && d->cigar_n < 0) {
    const int rc = finish_cigar(d, staged_pairs(d));
    if (rc) return rc;
  }
  if (d->rev_issued && d->n_batch > 0 && d->h_counts.p) {
    // timing of the completed protocol round
    d->timing.fwd_ms = elapsed(d->ev_t[1], d->ev_t[2]);
    d->timing.rev_ms = elapsed(d->ev_t[4], d->ev_t[5]);
    d->timing.total_ms = elapsed(d->ev_t[0], d->ev_t[5]);
    d->timing.fwd_cells = d->fwd_cells;
    d->timing.n_pairs = d->n_batch;
    d->timing.n_overflow16 = d->h_counts.p[0];
    d->timing.n_rev_wide = d->h_counts.p[1];
    d->timing.launches = d->launches;
  }
  return MHSW_OK;
}

int mhsw_get_aln_results(mhsw_driver *d, mhsw_aln_results *out) {
  if (!d || !out) return MHSW_ERR_ARG;
  std::lock_guard<std::mutex> lk(d->mu);
  if (!d->fwd_issued || !d->h_outv.p) return d->fail(MHSW_ERR_STATE, "no results yet");
  mhsw::OutViews hv;
  const int64_t n = std::max<int64_t>(d->n_batch, 1);
  int16_t *s = reinterpret_cast<int16_t *>(d->h_outv.p);
  hv.s_score = s;
  hv.s_ref_beg = s + n;
  hv.s_ref_end = s + 2 * n;
  hv.s_qry_beg = s + 3 * n;
  hv.s_qry_end = s + 4 * n;
  size_t off = ((size_t)n * 5 * sizeof(int16_t) + 15) / 16 * 16;
  int32_t *w = reinterpret_cast<int32_t *>(d->h_outv.p + off);
  out->top_scores = hv.s_score;
  out->ref_begin = hv.s_ref_beg;
  out->ref_end = hv.s_ref_end;
  out->query_begin = hv.s_qry_beg;
  out->query_end = hv.s_qry_end;
  out->top_scores32 = w;
  out->ref_begin32 = w + n;
  out->ref_end32 = w + 2 * n;
  out->query_begin32 = w + 3 * n;
  out->query_end32 = w + 4 * n;
  out->n = (int32_t)d->n_batch;
  const bool s2 = d->score2 && d->h_score2.p && d->n_batch > 0;
  out->score2_32 = s2 ? d->h_score2.p : nullptr;
  out->a_end2_32 = s2 ? d->h_score2.p + d->n_batch : nullptr;
  return MHSW_OK;
}

}  // extern "C"

namespace {

// Completes the pending batch call of a slot, if any (the caller holds d->mu): waits for
// its stream work, surfaces asynchronous faults, runs the CIGAR pass's host-driven rounds
// and records the timing.
int finish_slot(mhsw_driver *d, int s) {
  mhsw_driver::Pending &pd = d->pend[s];
  if (!pd.active) return MHSW_OK;
  pd.active = false;
  const int64_t n = pd.n;
  cudaEvent_t *ev = d->ev_p[s];
  MHSW_CK(cudaEventSynchronize(ev[4]), "sync");
  // Surface any asynchronous kernel fault as an error status.
  MHSW_CK(cudaGetLastError(), "kernel execution");
  d->cigar_ms = 0;
  d->cigar_generic = 0;
  if (n > 0 && d->cigar) {
    const int rc = finish_cigar(d, pd.ps);
    if (rc) return rc;
  }
  const int *hc = d->h_counts_p[s].p;
  d->timing.fwd_ms = elapsed(ev[1], ev[2]);
  d->timing.rev_ms = elapsed(ev[2], ev[3]);
  d->timing.total_ms = elapsed(ev[0], ev[4]);
  d->timing.fwd_cells = pd.cells;
  d->timing.n_pairs = n;
  d->timing.n_overflow16 = n > 0 && hc ? hc[0] : 0;
  d->timing.n_rev_wide = n > 0 && hc ? hc[1] : 0;
  d->timing.launches = d->launches;
  d->timing.graph_replays = d->graph_launches;
  d->timing.cigar_ms = d->cigar_ms;
  d->timing.n_cigar_generic = d->cigar_generic;
  // the call's record, ms since the handle's epoch
  mhsw_call_record r{};
  r.seq = pd.seq;
  r.n_pairs = n;
  r.copy_in_start = r.copy_in_end = -1;
  if (d->cin_recorded[s]) {
    r.copy_in_start = elapsed(d->ev_epoch, d->ev_cin[s][0]);
    for (int k = 0; k < mhsw_driver::kCopyStreams; k++)
      r.copy_in_end = std::max(r.copy_in_end, (double)elapsed(d->ev_epoch, d->ev_cin[s][1 + k]));
  }
  r.stream_ready = elapsed(d->ev_epoch, ev[0]);
  r.translated = elapsed(d->ev_epoch, ev[1]);
  r.forward_done = elapsed(d->ev_epoch, ev[2]);
  r.begin_done = elapsed(d->ev_epoch, ev[3]);
  r.done = elapsed(d->ev_epoch, ev[4]);
  d->history[d->history_n % mhsw_driver::kHistory] = r;
  d->history_n++;
  return MHSW_OK;
}

// Completes every pending batch call, oldest first.
int finish_pending(mhsw_driver *d) {
  for (;;) {
    int oldest = -1;
    for (int k = 0; k < mhsw_driver::kSlots; k++)
      if (d->pend[k].active && (oldest < 0 || d->pend[k].seq < d->pend[oldest].seq)) oldest = k;
    if (oldest < 0) return MHSW_OK;
    const int rc = finish_slot(d, oldest);
    if (rc) return rc;
  }
}

// Everything of a batch call up to its completion event, enqueued on the handle's stream;
// leaves the call pending (finish_pending completes it).
int align_pairs_begin(mhsw_driver *d, const mhsw_pairs *pairs, int32_t *out5, int host_io, int form) {
  // Host batches take the slots in turn and overlap; score2 and CIGAR outputs live in one
  // set of buffers, and device batches may be captured into a graph with slot 0's events,
  // so those complete everything pending first and use slot 0.
  const bool overlap = host_io && !d->score2 && !d->cigar;
  int slot = 0;
  int rc = MHSW_OK;
  if (overlap) {
    // slots go round in call order, so the slot taken holds the oldest call in flight
    slot = d->next_slot;
    d->next_slot = (d->next_slot + 1) % mhsw_driver::kSlots;
    rc = finish_slot(d, slot);
  } else {
    rc = finish_pending(d);
    d->next_slot = 1;
  }
  if (rc) return rc;
  cudaEvent_t *ev = d->ev_p[slot];
  d->cin_recorded[slot] = false;
  if (!pairs || pairs->n < 0 || (pairs->n > 0 && !out5)) return d->fail(MHSW_ERR_ARG, "bad pairs");
  if (form != MHSW_FORM_PLAIN && form != MHSW_FORM_BATCHED) return d->fail(MHSW_ERR_ARG, "unknown form %d", form);
  if (d->ev_live) MHSW_CK(cudaEventSynchronize(d->ev_done), "wait previous batch");
  d->ev_live = false;
  d->fwd_issued = d->rev_issued = false;
  const int64_t n = pairs->n;
  d->launches = 0;
  int ma = 0, mb = 0;
  double cells = 0;
  int64_t ta = 0, tb = 0;
  mhsw::PairSet ps;
  MHSW_CK(cudaEventRecord(ev[0], d->st), "event");
  const bool hinted_sizes =
      pairs->max_a_len > 0 && pairs->max_b_len > 0 && pairs->a_bytes > 0 && pairs->b_bytes > 0;
  if (host_io) {
    if (hinted_sizes) {
      // the caller states the batch's extents (as klign states its longest read and contig)
      ma = pairs->max_a_len;
      mb = pairs->max_b_len;
      ta = pairs->a_bytes;
      tb = pairs->b_bytes;
      cells = pairs->cells;
    } else {
      for (int64_t i = 0; i < n; i++) {
        const int32_t la = pairs->a_len[i], lb = pairs->b_len[i];
        if (la < 0 || lb < 0) return d->fail(MHSW_ERR_ARG, "negative length at pair %lld", (long long)i);
        ma = std::max(ma, (int)la);
        mb = std::max(mb, (int)lb);
        ta = std::max(ta, pairs->a_off[i] + la);
        tb = std::max(tb, pairs->b_off[i] + lb);
        cells += (double)la * (double)lb;
      }
    }
    mhsw_driver::InSet &in = d->in_sets[slot];
    MHSW_CK(in.a_seq.reserve((size_t)ta + 16), "cudaMalloc A");
    MHSW_CK(in.b_seq.reserve((size_t)tb + 16), "cudaMalloc B");
    MHSW_CK(in.a_off.reserve((size_t)n + 1), "cudaMalloc offsets");
    MHSW_CK(in.b_off.reserve((size_t)n + 1), "cudaMalloc offsets");
    MHSW_CK(in.a_len.reserve((size_t)n + 1), "cudaMalloc lengths");
    MHSW_CK(in.b_len.reserve((size_t)n + 1), "cudaMalloc lengths");
    if (n > 0) {
      rc = copy_batch_in(d, in, pairs, n, ta, tb, overlap, slot);
      if (rc) return rc;
    }
    ps.a_seq = in.a_seq.p;
    ps.a_off = in.a_off.p;
    ps.a_len = in.a_len.p;
    ps.b_seq = in.b_seq.p;
    ps.b_off = in.b_off.p;
    ps.b_len = in.b_len.p;
  } else if (hinted_sizes) {
    // device-resident inputs with size hints: no host round trip
    ma = pairs->max_a_len;
    mb = pairs->max_b_len;
    cells = pairs->cells;
    ta = pairs->a_bytes;
    tb = pairs->b_bytes;
    ps.a_seq = pairs->a_seq;
    ps.a_off = pairs->a_off;
    ps.a_len = pairs->a_len;
    ps.b_seq = pairs->b_seq;
    ps.b_off = pairs->b_off;
    ps.b_len = pairs->b_len;
  } else {
    // device-resident inputs: lengths and offsets are read back once to size the launch
    std::vector<int32_t> la((size_t)n), lb((size_t)n);
    std::vector<int64_t> oa((size_t)n), ob((size_t)n);
    if (n > 0) {
      MHSW_CK(cudaMemcpyAsync(la.data(), pairs->a_len, sizeof(int32_t) * n, cudaMemcpyDeviceToHost, d->st), "D2H");
      MHSW_CK(cudaMemcpyAsync(lb.data(), pairs->b_len, sizeof(int32_t) * n, cudaMemcpyDeviceToHost, d->st), "D2H");
      MHSW_CK(cudaMemcpyAsync(oa.data(), pairs->a_off, sizeof(int64_t) * n, cudaMemcpyDeviceToHost, d->st), "D2H");
      MHSW_CK(cudaMemcpyAsync(ob.data(), pairs->b_off, sizeof(int64_t) * n, cudaMemcpyDeviceToHost, d->st), "D2H");
      MHSW_CK(cudaStreamSynchronize(d->st), "sync");
    }
    for (int64_t i = 0; i < n; i++) {
      ma = std::max(ma, (int)la[(size_t)i]);
      mb = std::max(mb, (int)lb[(size_t)i]);
      ta = std::max(ta, oa[(size_t)i] + la[(size_t)i]);
      tb = std::max(tb, ob[(size_t)i] + lb[(size_t)i]);
      cells += (double)la[(size_t)i] * (double)lb[(size_t)i];
    }
    ps.a_seq = pairs->a_seq;
    ps.a_off = pairs->a_off;
    ps.a_len = pairs->a_len;
    ps.b_seq = pairs->b_seq;
    ps.b_off = pairs->b_off;
    ps.b_len = pairs->b_len;
    d->sig = mhsw::batch_signature(la.data(), n, ma, mb);
  }
  if (host_io) d->sig = mhsw::batch_signature(pairs->a_len, n, ma, mb);
  else if (hinted_sizes) d->sig = mhsw::batch_signature(nullptr, n, ma, mb);
  ps.n = n;
  if (mb > mhsw::kMaxB) return d->fail(MHSW_ERR_LIMIT, "sequence of %d bytes exceeds the limit %d", mb, mhsw::kMaxB);
  rc = ensure_results(d, n);
  if (rc) return rc;
  if (n > 0) {
    MHSW_CK(d->a_code.reserve((size_t)ta + 16), "cudaMalloc codes");
    MHSW_CK(d->b_code.reserve((size_t)tb + 16), "cudaMalloc codes");
    MHSW_CK(d->h_counts.reserve(4), "cudaMallocHost");
    MHSW_CK(d->h_counts_p[slot].reserve(4), "cudaMallocHost");
    if (host_io) MHSW_CK(d->out5.reserve((size_t)n * 5), "cudaMalloc out5");
  }
  rc = attach_score2(d, &ps, n, ta);
  if (rc) return rc;
  d->cigar_n = -1;
  if (d->cigar && n > 0) {
    rc = ensure_cigar(d, n);
    if (rc) return rc;
  }
  // Everything from translation to the result copy, on the handle's stream.
  // Phase events recorded inside a capture become external event nodes, so a replayed
  // graph still records them and the phase timings stay available.
  bool capturing = false;
  auto mark = [&](cudaEvent_t ev) {
    return capturing ? cudaEventRecordWithFlags(ev, d->st, cudaEventRecordExternal) : cudaEventRecord(ev, d->st);
  };
  auto enqueue = [&]() -> int {
    if (n > 0) {
      int r = translate_batch(d, &ps, ta, tb);
      if (r) return r;
    }
    MHSW_CK(mark(ev[1]), "event");
    if (n > 0) {
      int r = forward_any(d, ps, ma, mb, form);
      if (r) return r;
    }
    MHSW_CK(mark(ev[2]), "event");
    if (n > 0) {
      int r = run_reverse(d, ps, ma, mb, d->fwd_order);
      if (r) return r;
    }
    MHSW_CK(mark(ev[3]), "event");
    if (n > 0 && d->cigar) {
      MHSW_CK(mark(d->ev_c[0]), "event");
      int r = enqueue_cigar(d, ps);
      if (r) return r;
      MHSW_CK(mark(d->ev_c[1]), "event");
    }
    if (n > 0) {
      if (host_io) {
        MHSW_CK(mhsw::launch_pack5(result_set(d), n, d->out5.p, d->st), "pack5");
        MHSW_CK(cudaMemcpyAsync(out5, d->out5.p, sizeof(int32_t) * 5 * n, cudaMemcpyDeviceToHost, d->st), "D2H");
      } else {
        MHSW_CK(mhsw::launch_pack5(result_set(d), n, out5, d->st), "pack5");
      }
      d->launches += 1;
      MHSW_CK(cudaMemcpyAsync(d->h_counts_p[slot].p, d->l_counts.p, 2 * sizeof(int), cudaMemcpyDeviceToHost, d->st),
              "D2H");
    }
    return MHSW_OK;
  };
  // A device-resident batch with all size hints is graph-eligible: the second identical
  // call captures the enqueued work into a CUDA graph, later identical calls replay it.
  const bool hinted = !host_io && pairs->max_a_len > 0 && pairs->max_b_len > 0 && pairs->a_bytes > 0 &&
                      pairs->b_bytes > 0;
  mhsw_driver::GraphKey key{};
  if (hinted) {
    const void *ptrs[7] = {pairs->a_seq, pairs->a_off, pairs->a_len, pairs->b_seq, pairs->b_off, pairs->b_len, out5};
    for (int k = 0; k < 7; k++) key.ptr[k] = ptrs[k];
    key.n = n;
    key.a_bytes = ta;
    key.b_bytes = tb;
    key.max_a = ma;
    key.max_b = mb;
    key.form = form;
    key.ceiling = d->ceiling16;
    key.match = d->sc.match;
    key.mismatch = d->sc.mismatch;
    key.gap_open = d->sc.gap_open;
    key.gap_extend = d->sc.gap_extend;
    key.ambiguity = d->sc.ambiguity;
    key.score2 = d->score2 ? 1 : 0;
    key.cigar = d->cigar ? 1 : 0;
  }
  const bool same = hinted && d->use_graphs && n > 0 && d->gkey_seen && key == d->gkey;
  if (same && d->gexec) {
    MHSW_CK(cudaGraphLaunch(d->gexec, d->st), "graph launch");
    d->launches = d->timing.launches;  // a replay launches what the captured call launched
    d->graph_launches++;
  } else if (same) {
    // capture (the first identical call sized every buffer and tuned the launch shape)
    d->launches = 0;
    cudaGraph_t graph = nullptr;
    MHSW_CK(cudaStreamBeginCapture(d->st, cudaStreamCaptureModeThreadLocal), "begin capture");
    capturing = true;
    const bool tune_was = d->batch.autotune;
    d->batch.autotune = false;  // the tuner synchronises: never inside a capture
    const int r = enqueue();
    d->batch.autotune = tune_was;
    capturing = false;
    const cudaError_t ce = cudaStreamEndCapture(d->st, &graph);
    if (r || ce != cudaSuccess || !graph) {
      if (graph) cudaGraphDestroy(graph);
      cudaGetLastError();
      d->use_graphs = false;  // this batch does not capture: run it directly from now on
      if (r) return r;
      d->launches = 0;
      rc = enqueue();
      if (rc) return rc;
    } else {
      cudaGraphExec_t ex = nullptr;
      const cudaError_t ie = cudaGraphInstantiate(&ex, graph, 0);
      cudaGraphDestroy(graph);
      if (ie != cudaSuccess) {
        cudaGetLastError();
        d->use_graphs = false;
        d->launches = 0;
        rc = enqueue();
        if (rc) return rc;
      } else {
        if (d->gexec) cudaGraphExecDestroy(d->gexec);
        d->gexec = ex;
        MHSW_CK(cudaGraphLaunch(d->gexec, d->st), "graph launch");
        d->graph_launches++;
      }
    }
  } else {
    if (d->gexec) {
      cudaGraphExecDestroy(d->gexec);
      d->gexec = nullptr;
    }
    d->gkey = key;
    d->gkey_seen = hinted;
    rc = enqueue();
    if (rc) return rc;
  }
  MHSW_CK(cudaEventRecord(ev[4], d->st), "event");
  if (host_io) {
    // the slot's input set is free again once this call's kernels are done
    MHSW_CK(cudaEventRecord(d->in_sets[slot].free_ev, d->st), "event");
    d->in_sets[slot].used = true;
  }
  mhsw_driver::Pending &pd = d->pend[slot];
  pd.active = true;
  pd.n = n;
  pd.cells = cells;
  pd.seq = ++d->call_seq;
  pd.ps = ps;
  return MHSW_OK;
}

}  // namespace

extern "C" {

int mhsw_align_pairs(mhsw_driver *d, const mhsw_pairs *pairs, int32_t *out5, int host_io, int form) {
  int rc = ready(d);
  if (rc) return rc;
  std::lock_guard<std::mutex> lk(d->mu);
  rc = align_pairs_begin(d, pairs, out5, host_io, form);
  if (rc) return rc;
  return finish_pending(d);
}

int mhsw_align_pairs_async(mhsw_driver *d, const mhsw_pairs *pairs, int32_t *out5, int host_io, int form) {
  int rc = ready(d);
  if (rc) return rc;
  std::lock_guard<std::mutex> lk(d->mu);
  return align_pairs_begin(d, pairs, out5, host_io, form);
}

int mhsw_align_wait(mhsw_driver *d) {
  if (!d) return MHSW_ERR_ARG;
  std::lock_guard<std::mutex> lk(d->mu);
  return finish_pending(d);
}

int mhsw_last_timing(mhsw_driver *d, mhsw_timing *out) {
  if (!d || !out) return MHSW_ERR_ARG;
  std::lock_guard<std::mutex> lk(d->mu);
  if (int rcp = finish_pending(d)) return rcp;
  *out = d->timing;
  return MHSW_OK;
}

int mhsw_call_history(mhsw_driver *d, mhsw_call_record *out, int max_records, int *count) {
  if (!d || !count || max_records < 0 || (max_records > 0 && !out)) return MHSW_ERR_ARG;
  std::lock_guard<std::mutex> lk(d->mu);
  if (int rcp = finish_pending(d)) return rcp;
  const int64_t have = std::min<int64_t>(d->history_n, mhsw_driver::kHistory);
  const int64_t k = std::min<int64_t>(have, max_records);
  for (int64_t i = 0; i < k; i++) out[i] = d->history[(d->history_n - k + i) % mhsw_driver::kHistory];
  *count = (int)k;
  return MHSW_OK;
}

int mhsw_last_tuning(mhsw_driver *d, mhsw_tuning *out) {
  if (!d || !out) return MHSW_ERR_ARG;
  std::lock_guard<std::mutex> lk(d->mu);
  if (int rcp = finish_pending(d)) return rcp;
  const mhsw::BatchState &b = d->batch;
  mhsw_tuning t{};
  t.threads_per_block = b.shape.groups_per_block * 8;
  t.blocks_per_sm = b.shape.blocks_per_sm;
  t.lane_rows = b.shape.lane_rows;
  t.wide_try16 = b.shape.wide_try16 ? 1 : 0;
  t.last_call_tuned = b.tune.last_call_tuned ? 1 : 0;
  t.trials = b.tune.trials;
  t.sample_pairs = b.tune.sample_pairs;
  t.tunings = b.tune.tunings;
  t.tune_wall_ms = b.tune.wall_ms;
  for (int k = 0; k < 16; k++) t.trial_ms[k] = b.tune.trial_ms[k];
  *out = t;
  return MHSW_OK;
}

int mhsw_driver_fix_batch_config(mhsw_driver *d, int threads_per_block, int blocks_per_sm, int lane_rows,
                                 int wide_try16) {
  if (!d) return MHSW_ERR_ARG;
  std::lock_guard<std::mutex> lk(d->mu);
  if (int rcp = finish_pending(d)) return rcp;
  if (threads_per_block == 0) {
    d->batch.autotune = true;
    d->batch.tuned = false;
    d->batch.n_cached = d->batch.next_cached = 0;
    return MHSW_OK;
  }
  if ((threads_per_block != 64 && threads_per_block != 128 && threads_per_block != 256) || blocks_per_sm < 0 ||
      blocks_per_sm > 32 || (lane_rows != 128 && lane_rows != 160) || (wide_try16 != 0 && wide_try16 != 1))
    return d->fail(MHSW_ERR_ARG, "batch configuration (%d, %d, %d, %d) not supported", threads_per_block,
                   blocks_per_sm, lane_rows, wide_try16);
  d->batch.autotune = false;
  d->batch.shape.groups_per_block = threads_per_block / 8;
  d->batch.shape.blocks_per_sm = blocks_per_sm;
  d->batch.shape.lane_rows = lane_rows;
  d->batch.shape.wide_try16 = wide_try16 != 0;
  return MHSW_OK;
}

int mhsw_driver_set_score2(mhsw_driver *d, int on) {
  if (!d) return MHSW_ERR_ARG;
  std::lock_guard<std::mutex> lk(d->mu);
  if (int rcp = finish_pending(d)) return rcp;
  d->score2 = on != 0;
  return MHSW_OK;
}

int mhsw_last_score2(mhsw_driver *d, int32_t *score2, int32_t *a_end2, int host_io) {
  int rc = ready(d);
  if (rc) return rc;
  std::lock_guard<std::mutex> lk(d->mu);
  if (int rcp = finish_pending(d)) return rcp;
  const int64_t n = d->score2_n;
  if (n < 0 || !d->r_score2.p) return d->fail(MHSW_ERR_STATE, "score2 mode was off for the last batch");
  if (n > 0 && (!score2 || !a_end2)) return d->fail(MHSW_ERR_ARG, "NULL output");
  if (n <= 0) return MHSW_OK;
  const cudaMemcpyKind k = host_io ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice;
  MHSW_CK(cudaMemcpyAsync(score2, d->r_score2.p, sizeof(int32_t) * n, k, d->st), "copy score2");
  MHSW_CK(cudaMemcpyAsync(a_end2, d->r_aend2.p, sizeof(int32_t) * n, k, d->st), "copy score2");
  MHSW_CK(cudaStreamSynchronize(d->st), "sync");
  return MHSW_OK;
}

int mhsw_driver_set_cigar(mhsw_driver *d, int on) {
  if (!d) return MHSW_ERR_ARG;
  std::lock_guard<std::mutex> lk(d->mu);
  if (int rcp = finish_pending(d)) return rcp;
  d->cigar = on != 0;
  return MHSW_OK;
}

int mhsw_last_cigar(mhsw_driver *d, int32_t *nops, int32_t *mismatches, int64_t *op_off, uint32_t *ops,
                    int64_t ops_cap, int64_t *ops_total, int host_io) {
  int rc = ready(d);
  if (rc) return rc;
  std::lock_guard<std::mutex> lk(d->mu);
  if (int rcp = finish_pending(d)) return rcp;
  const int64_t n = d->cigar_n;
  if (n < 0) return d->fail(MHSW_ERR_STATE, "no CIGARs: CIGAR mode was off for the last batch, or it has not completed");
  if (n == 0) {
    if (ops_total) *ops_total = 0;
    if (op_off) {
      const int64_t z = 0;
      MHSW_CK(cudaMemcpy(op_off, &z, sizeof(z), host_io ? cudaMemcpyHostToHost : cudaMemcpyHostToDevice), "copy");
    }
    return MHSW_OK;
  }
  if (d->cigar_total < 0) {  // pair-order copy of the arena, once per batch
    size_t temp = 0;
    MHSW_CK(mhsw::cigar_gather_temp_bytes(n, &temp), "scan size");
    MHSW_CK(d->c_temp.reserve(temp + 16), "cudaMalloc scan");
    MHSW_CK(d->c_c64.reserve((size_t)n + 1), "cudaMalloc CIGAR");
    MHSW_CK(d->c_ordoff.reserve((size_t)n + 1), "cudaMalloc CIGAR");
    unsigned long long used = 0;
    MHSW_CK(cudaMemcpy(&used, d->c_cursor.p, sizeof(used), cudaMemcpyDeviceToHost), "D2H cursor");
    MHSW_CK(d->c_ordops.reserve((size_t)used + 1), "cudaMalloc CIGAR");
    MHSW_CK(mhsw::launch_cigar_gather(cigar_bufs(d, n), n, d->c_c64.p, d->c_ordoff.p, d->c_ordops.p, d->c_temp.p,
                                      d->c_temp.cap, d->st),
            "CIGAR gather");
    int64_t total = 0;
    MHSW_CK(cudaMemcpyAsync(&total, d->c_ordoff.p + n, sizeof(total), cudaMemcpyDeviceToHost, d->st), "D2H total");
    MHSW_CK(cudaStreamSynchronize(d->st), "sync");
    d->cigar_total = total;
  }
  if (ops_total) *ops_total = d->cigar_total;
  const cudaMemcpyKind k = host_io ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice;
  if (nops) MHSW_CK(cudaMemcpyAsync(nops, d->c_nops.p, sizeof(int32_t) * n, k, d->st), "copy op counts");
  if (mismatches) MHSW_CK(cudaMemcpyAsync(mismatches, d->c_mism.p, sizeof(int32_t) * n, k, d->st), "copy mismatches");
  if (op_off) MHSW_CK(cudaMemcpyAsync(op_off, d->c_ordoff.p, sizeof(int64_t) * (n + 1), k, d->st), "copy offsets");
  if (ops) {
    if (ops_cap < d->cigar_total) {
      cudaStreamSynchronize(d->st);
      return d->fail(MHSW_ERR_ARG, "ops buffer holds %lld ops, the batch has %lld", (long long)ops_cap,
                     (long long)d->cigar_total);
    }
    if (d->cigar_total > 0)
      MHSW_CK(cudaMemcpyAsync(ops, d->c_ordops.p, sizeof(uint32_t) * d->cigar_total, k, d->st), "copy ops");
  }
  MHSW_CK(cudaStreamSynchronize(d->st), "sync");
  return MHSW_OK;
}

int64_t mhsw_cigar_format(const uint32_t *ops, int32_t nops, char *buf, int64_t cap) {
  static const char kOps[] = "MIDNSHP=X";
  if (nops < 0 || (nops > 0 && !ops) || !buf || cap <= 0) return -1;
  int64_t at = 0;
  for (int32_t t = 0; t < nops; t++) {
    const uint32_t c = ops[t], code = c & 15u;
    char tmp[16];
    int k = 0;
    uint32_t len = c >> 4;
    do {
      tmp[k++] = (char)('0' + len % 10);
      len /= 10;
    } while (len);
    if (at + k + 1 >= cap) return -1;
    while (k) buf[at++] = tmp[--k];
    buf[at++] = code <= 8 ? kOps[code] : '?';
  }
  buf[at] = '\0';
  return at;
}

}  // extern "C"

namespace mhsw {

int align_resident(mhsw_driver *d, const PairSet &in, int64_t a_bytes, int max_a, int max_b, int form,
                   int32_t *out5_dev) {
  int rc = ready(d);
  if (rc) return rc;
  std::lock_guard<std::mutex> lk(d->mu);
  if (int rcp = finish_pending(d)) return rcp;
  if (form != MHSW_FORM_PLAIN && form != MHSW_FORM_BATCHED) return d->fail(MHSW_ERR_ARG, "unknown form %d", form);
  if (d->ev_live) MHSW_CK(cudaEventSynchronize(d->ev_done), "wait previous batch");
  d->ev_live = false;
  d->fwd_issued = d->rev_issued = false;
  d->launches = 0;
  const int64_t n = in.n;
  if (n <= 0) return MHSW_OK;
  if (!in.b_code || !out5_dev) return d->fail(MHSW_ERR_ARG, "resident batch needs B codes and an output buffer");
  if (max_b > kMaxB) return d->fail(MHSW_ERR_LIMIT, "sequence of %d bytes exceeds the limit %d", max_b, kMaxB);
  rc = ensure_results(d, n);
  if (rc) return rc;
  MHSW_CK(d->a_code.reserve((size_t)a_bytes + 16), "cudaMalloc codes");
  MHSW_CK(cudaEventRecord(d->ev_t[0], d->st), "event");
  MHSW_CK(launch_translate(in.a_seq, d->a_code.p, a_bytes, d->st), "translate A");
  d->launches += 1;
  PairSet ps = in;
  ps.a_code = d->a_code.p;
  rc = attach_score2(d, &ps, n, a_bytes);
  if (rc) return rc;
  MHSW_CK(cudaEventRecord(d->ev_t[1], d->st), "event");
  d->sig = mhsw::batch_signature(nullptr, ps.n, max_a, max_b);
  rc = forward_any(d, ps, max_a, max_b, form);
  if (rc) return rc;
  MHSW_CK(cudaEventRecord(d->ev_t[2], d->st), "event");
  rc = run_reverse(d, ps, max_a, max_b, d->fwd_order);
  if (rc) return rc;
  MHSW_CK(cudaEventRecord(d->ev_t[3], d->st), "event");
  MHSW_CK(launch_pack5(result_set(d), n, out5_dev, d->st), "pack5");
  d->launches += 1;
  d->timing = mhsw_timing{};
  d->timing.n_pairs = n;
  return MHSW_OK;
}

void resident_timing(mhsw_driver *d) {
  if (!d) return;
  std::lock_guard<std::mutex> lk(d->mu);
  if (d->timing.n_pairs <= 0) return;
  d->timing.fwd_ms = elapsed(d->ev_t[1], d->ev_t[2]);
  d->timing.rev_ms = elapsed(d->ev_t[2], d->ev_t[3]);
  d->timing.total_ms = elapsed(d->ev_t[0], d->ev_t[3]);
  d->timing.launches = d->launches;
  d->timing.cigar_ms = d->cigar ? d->cigar_ms : 0;
  d->timing.n_cigar_generic = d->cigar ? d->cigar_generic : 0;
}

void *driver_stream(mhsw_driver *d) { return d ? static_cast<void *>(d->st) : nullptr; }
int driver_device(mhsw_driver *d) { return d ? d->device : -1; }
int driver_form(mhsw_driver *d) { return d ? d->form : MHSW_FORM_PLAIN; }
bool driver_cigar(mhsw_driver *d) { return d && d->cigar; }
const uint8_t *driver_a_codes(mhsw_driver *d) { return d ? d->a_code.p : nullptr; }

std::mutex &driver_call_mutex(mhsw_driver *d) { return d->call_mu; }

unsigned char *driver_call_arena(mhsw_driver *d, size_t bytes) {
  if (!d) return nullptr;
  if (cudaSetDevice(d->device) != cudaSuccess) return nullptr;
  return d->call_arena.reserve(bytes) == cudaSuccess ? d->call_arena.p : nullptr;
}

int cigar_resident(mhsw_driver *d, const PairSet &ps) {
  int rc = ready(d);
  if (rc) return rc;
  std::lock_guard<std::mutex> lk(d->mu);
  if (!d->cigar) return d->fail(MHSW_ERR_STATE, "CIGAR mode is off");
  d->cigar_n = -1;
  if (ps.n <= 0) {
    d->cigar_n = 0;
    return MHSW_OK;
  }
  rc = ensure_cigar(d, ps.n);
  if (rc) return rc;
  MHSW_CK(cudaEventRecord(d->ev_c[0], d->st), "event");
  rc = enqueue_cigar(d, ps);
  if (rc) return rc;
  MHSW_CK(cudaEventRecord(d->ev_c[1], d->st), "event");
  MHSW_CK(cudaStreamSynchronize(d->st), "sync");
  return finish_cigar(d, ps);
}
int driver_match(mhsw_driver *d) { return d ? d->sc.match : 1; }
void driver_gaps(mhsw_driver *d, int *gap_open, int *gap_extend) {
  *gap_open = d ? d->sc.gap_open : 0;
  *gap_extend = d ? d->sc.gap_extend : 0;
}
const int32_t *driver_score2(mhsw_driver *d, int64_t n) {
  return (d && d->score2 && d->score2_n == n && n > 0) ? d->r_score2.p : nullptr;
}

}  // namespace mhsw
