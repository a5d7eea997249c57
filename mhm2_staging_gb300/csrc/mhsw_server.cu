// mhsw_server.cu -- the serving form: resident contigs, budgeted admission and
// continuous batching over worker slots (C ABI in include/mhsw.h).
//
// klign cuts a contig window around every k-mer seed hit and aligns the read against it
// (src/klign.cpp:670-739, :218-249).  Here the contigs are uploaded and translated once;
// a request names (read, contig id, position) and its pair is the read against the
// window [pos - flank, pos + read_len + flank) clamped to the contig -- the window is an
// offset into the resident code arena, nothing is copied.
//
// Flow.  mhsw_server_submit computes the windows of a request batch (the read bytes stay
// in the caller's buffer until its ticket is waited for) and queues it once the queue
// budget has room (admission).  Each slot -- one driver handle with its own
// stream and device buffers sized from the device-memory budget -- runs a worker thread
// that, whenever it is free, packs the waiting pairs (oldest request first, splitting
// large requests) into one micro-batch, uploads the reads, aligns them against the
// resident windows on its stream, and scatters the results back.  Requests arriving
// while other micro-batches are on the GPU go to the next slot that frees up, and the
// slots' kernels overlap on the device.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <deque>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "../../include/mhsw.h"
#include "mhsw_internal.h"
#include "mhsw_launch.h"

namespace {

double now_s() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

// Device-memory estimate of one micro-batch slot: its own buffers (reads, offsets,
// lengths, windows, results) plus the driver's per-pair buffers (codes, result arrays,
// work lists, sort keys and scratch of the batched form).
constexpr size_t kSlotBytesPerPair = 8 + 4 + 8 + 4 + 20 + 24 + 32 + 48;
constexpr size_t kSlotFixedBytes = size_t(8) << 20;  // strip scratch, sort temporaries, alignment slack
constexpr int32_t kReadBytesPerPair = 256;            // read bytes reserved per pair of capacity

struct Request {
  uint64_t ticket = 0;
  int32_t n = 0;
  const char *src = nullptr;    // the caller's read bytes (valid until the ticket is waited for)
  std::vector<int64_t> src_off; // read offsets into src
  std::vector<int64_t> cum;     // prefix sums of the read lengths (n + 1), for packing
  std::vector<int32_t> len;
  std::vector<int64_t> b_off;   // window offsets into the contig code arena
  std::vector<int32_t> b_len;
  std::vector<int64_t> wstart;  // window start within its contig
  bool contiguous = true;       // each read starts where the previous one ends in src
  int32_t *out5 = nullptr;
  int64_t *win_start = nullptr;
  int32_t next = 0;       // first pair not yet on a slot
  int32_t remaining = 0;  // pairs not yet finished
  size_t bytes = 0;       // admitted host bytes
  int status = MHSW_OK;
  bool done = false;
  double t_submit = 0, t_start = 0, t_done = 0;
};

struct Piece {  // a run of one request's pairs inside a micro-batch
  std::shared_ptr<Request> r;
  int32_t first, count;
  int64_t row;  // first row in the micro-batch
};

template <class T>
struct DevArr {
  T *p = nullptr;
  size_t n = 0;
  cudaError_t alloc(size_t count) {
    n = count;
    return cudaMalloc(&p, std::max<size_t>(count, 1) * sizeof(T));
  }
  void free() {
    if (p) cudaFree(p);
    p = nullptr;
  }
};

template <class T>
struct PinArr {
  T *p = nullptr;
  cudaError_t alloc(size_t count) { return cudaMallocHost(&p, std::max<size_t>(count, 1) * sizeof(T)); }
  void free() {
    if (p) cudaFreeHost(p);
    p = nullptr;
  }
};

struct Slot {
  mhsw_driver *drv = nullptr;
  cudaStream_t st = nullptr;
  DevArr<char> a_seq;
  DevArr<int64_t> a_off, b_off;
  DevArr<int32_t> a_len, b_len, out5;
  PinArr<char> h_seq;
  PinArr<int64_t> h_aoff, h_boff;
  PinArr<int32_t> h_alen, h_blen, h_out5;
  std::thread th;
  bool busy = false;
};

}  // namespace

struct mhsw_server {
  mhsw_server_config cfg{};
  mhsw::Scoring sc{};
  std::string err;
  std::mutex err_mu;

  // contig store (device codes; host offsets and lengths for the windows)
  uint8_t *contig_codes = nullptr;
  size_t contig_bytes = 0;
  std::vector<int64_t> coff;
  std::vector<int32_t> clen;
  bool loaded = false;

  std::vector<std::unique_ptr<Slot>> slots;
  int32_t slot_pairs = 0;
  int64_t slot_read_bytes = 0;
  size_t device_bytes = 0;

  std::mutex mu;
  std::condition_variable cv_work, cv_done, cv_room;
  std::deque<std::shared_ptr<Request>> queue;
  std::unordered_map<uint64_t, std::shared_ptr<Request>> live;
  uint64_t next_ticket = 1;
  size_t admitted_bytes = 0;
  int64_t queued_pairs = 0;
  bool stop = false;
  int busy = 0;
  int64_t submitted = 0, completed = 0, pairs_done = 0, micro_batches = 0;
  double cells_done = 0;

  int fail(int code, const char *fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    std::lock_guard<std::mutex> lk(err_mu);
    err = buf;
    return code;
  }

  void worker(Slot *s);
  int run_micro_batch(Slot *s, std::vector<Piece> &pieces, int64_t rows, int64_t bytes);
  void shutdown();
};

namespace {

int copy_err(char *errbuf, size_t errlen, int rc, const char *msg) {
  if (errbuf && errlen) snprintf(errbuf, errlen, "%s", msg);
  return rc;
}

}  // namespace

// One micro-batch on one slot: pack, upload, align against the resident windows,
// download, scatter.  Runs on the slot's worker thread without the server lock.
int mhsw_server::run_micro_batch(Slot *s, std::vector<Piece> &pieces, int64_t rows, int64_t bytes) {
  int32_t max_a = 1, max_b = 1;
  int64_t ab = 0;
  for (auto &pc : pieces) {
    Request &r = *pc.r;
    if (r.contiguous) {
      // the piece's reads are one run of the caller's buffer: one copy of the bytes, the
      // per-pair fields as array copies
      const int32_t f = pc.first;
      const int64_t base = r.cum[(size_t)f];
      std::memcpy(s->h_seq.p + ab, r.src + r.src_off[(size_t)f], (size_t)(r.cum[(size_t)f + pc.count] - base));
      std::memcpy(s->h_alen.p + pc.row, r.len.data() + f, sizeof(int32_t) * (size_t)pc.count);
      std::memcpy(s->h_boff.p + pc.row, r.b_off.data() + f, sizeof(int64_t) * (size_t)pc.count);
      std::memcpy(s->h_blen.p + pc.row, r.b_len.data() + f, sizeof(int32_t) * (size_t)pc.count);
      const int64_t shift = ab - base;
      for (int32_t k = 0; k < pc.count; k++) {
        s->h_aoff.p[pc.row + k] = r.cum[(size_t)f + k] + shift;
        max_a = std::max(max_a, r.len[(size_t)f + k]);
        max_b = std::max(max_b, r.b_len[(size_t)f + k]);
      }
      ab += r.cum[(size_t)f + pc.count] - base;
      continue;
    }
    for (int32_t k = 0; k < pc.count; k++) {
      const int32_t i = pc.first + k;
      const int64_t row = pc.row + k;
      std::memcpy(s->h_seq.p + ab, r.src + r.src_off[i], (size_t)r.len[i]);
      s->h_aoff.p[row] = ab;
      s->h_alen.p[row] = r.len[i];
      s->h_boff.p[row] = r.b_off[i];
      s->h_blen.p[row] = r.b_len[i];
      max_a = std::max(max_a, r.len[i]);
      max_b = std::max(max_b, r.b_len[i]);
      ab += r.len[i];
    }
  }
  (void)bytes;
  cudaStream_t st = s->st;
  cudaError_t e;
#define SRV_CK(expr, what)                                                                  \
  do {                                                                                      \
    if ((e = (expr)) != cudaSuccess) return fail(MHSW_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e)); \
  } while (0)
  SRV_CK(cudaMemcpyAsync(s->a_seq.p, s->h_seq.p, (size_t)ab, cudaMemcpyHostToDevice, st), "H2D reads");
  SRV_CK(cudaMemcpyAsync(s->a_off.p, s->h_aoff.p, sizeof(int64_t) * rows, cudaMemcpyHostToDevice, st), "H2D");
  SRV_CK(cudaMemcpyAsync(s->a_len.p, s->h_alen.p, sizeof(int32_t) * rows, cudaMemcpyHostToDevice, st), "H2D");
  SRV_CK(cudaMemcpyAsync(s->b_off.p, s->h_boff.p, sizeof(int64_t) * rows, cudaMemcpyHostToDevice, st), "H2D");
  SRV_CK(cudaMemcpyAsync(s->b_len.p, s->h_blen.p, sizeof(int32_t) * rows, cudaMemcpyHostToDevice, st), "H2D");
  mhsw::PairSet ps{};
  ps.a_seq = s->a_seq.p;
  ps.a_off = s->a_off.p;
  ps.a_len = s->a_len.p;
  ps.b_seq = nullptr;
  ps.b_off = s->b_off.p;
  ps.b_len = s->b_len.p;
  ps.n = rows;
  ps.a_code = nullptr;
  ps.b_code = contig_codes;
  int rc = mhsw::align_resident(s->drv, ps, ab, max_a, max_b, cfg.form, s->out5.p);
  if (rc) return fail(rc, "slot alignment: %s", mhsw_driver_last_error(s->drv));
  SRV_CK(cudaMemcpyAsync(s->h_out5.p, s->out5.p, sizeof(int32_t) * 5 * rows, cudaMemcpyDeviceToHost, st), "D2H");
  SRV_CK(cudaStreamSynchronize(st), "slot synchronise");
#undef SRV_CK
  for (auto &pc : pieces) {
    Request &r = *pc.r;
    std::memcpy(r.out5 + 5 * (int64_t)pc.first, s->h_out5.p + 5 * pc.row, sizeof(int32_t) * 5 * (size_t)pc.count);
    if (r.win_start)
      std::memcpy(r.win_start + pc.first, r.wstart.data() + pc.first, sizeof(int64_t) * (size_t)pc.count);
  }
  return MHSW_OK;
}

void mhsw_server::worker(Slot *s) {
  cudaSetDevice(cfg.device);
  std::vector<Piece> pieces;
  for (;;) {
    pieces.clear();
    int64_t rows = 0, bytes = 0;
    {
      std::unique_lock<std::mutex> lk(mu);
      cv_work.wait(lk, [&] { return stop || !queue.empty(); });
      if (stop) return;
      // Continuous batching: take the oldest waiting pairs up to the slot's capacity.
      while (!queue.empty() && rows < slot_pairs) {
        auto r = queue.front();
        int32_t k = 0;
        const int64_t base = r->cum[r->next];
        while (r->next + k < r->n && rows + k < slot_pairs &&
               bytes + (r->cum[r->next + k + 1] - base) <= slot_read_bytes)
          k++;
        if (k == 0) break;  // the next read does not fit the remaining bytes
        if (r->next == 0) r->t_start = now_s();
        pieces.push_back(Piece{r, r->next, k, rows});
        rows += k;
        bytes += r->cum[r->next + k] - base;
        r->next += k;
        queued_pairs -= k;
        if (r->next == r->n) queue.pop_front();
      }
      s->busy = true;
      busy++;
      micro_batches++;
    }
    const int rc = rows > 0 ? run_micro_batch(s, pieces, rows, bytes) : MHSW_OK;
    bool more = false;
    {
      std::lock_guard<std::mutex> lk(mu);
      s->busy = false;
      busy--;
      for (auto &pc : pieces) {
        Request &r = *pc.r;
        if (rc) r.status = rc;
        r.remaining -= pc.count;
        pairs_done += pc.count;
        for (int32_t k = 0; k < pc.count; k++)
          cells_done += (double)r.len[pc.first + k] * (double)r.b_len[pc.first + k];
        if (r.remaining == 0) {
          r.done = true;
          r.t_done = now_s();
          admitted_bytes -= r.bytes;
          completed++;
        }
      }
      more = !queue.empty();
    }
    cv_done.notify_all();
    cv_room.notify_all();
    if (more) cv_work.notify_one();
  }
}

void mhsw_server::shutdown() {
  {
    std::lock_guard<std::mutex> lk(mu);
    stop = true;
  }
  cv_work.notify_all();
  for (auto &s : slots)
    if (s->th.joinable()) s->th.join();
  {
    std::lock_guard<std::mutex> lk(mu);
    for (auto &kv : live) {
      Request &r = *kv.second;
      if (!r.done) {
        r.status = MHSW_ERR_STATE;
        r.done = true;
        r.t_done = now_s();
      }
    }
    queue.clear();
  }
  cv_done.notify_all();
  cv_room.notify_all();
  if (!slots.empty() || contig_codes) cudaSetDevice(cfg.device);
  for (auto &s : slots) {
    if (s->drv) mhsw_driver_destroy(s->drv);
    s->a_seq.free();
    s->a_off.free();
    s->b_off.free();
    s->a_len.free();
    s->b_len.free();
    s->out5.free();
    s->h_seq.free();
    s->h_aoff.free();
    s->h_boff.free();
    s->h_alen.free();
    s->h_blen.free();
    s->h_out5.free();
  }
  slots.clear();
  if (contig_codes) cudaFree(contig_codes);
  contig_codes = nullptr;
}

extern "C" {

int mhsw_server_create(const mhsw_server_config *cfg, mhsw_server **out, char *errbuf, size_t errlen) {
  if (errbuf && errlen) errbuf[0] = '\0';
  if (!cfg || !out) return copy_err(errbuf, errlen, MHSW_ERR_ARG, "cfg and out are required");
  *out = nullptr;
  mhsw::Scoring sc{cfg->match_score, -cfg->mismatch_score, -cfg->gap_opening_score, -cfg->gap_extending_score,
                   -cfg->ambiguity_score};
  if (sc.match < 0 || sc.mismatch < 0 || sc.ambiguity < 0 || sc.gap_open < 1 || sc.gap_extend < 1 || sc.match > 127 ||
      sc.mismatch > 127 || sc.ambiguity > 127 || sc.gap_open > 127 || sc.gap_extend > 127)
    return copy_err(errbuf, errlen, MHSW_ERR_ARG, "scores as klign passes them: match >= 0, penalties <= 0 (gaps <= -1), magnitudes <= 127");
  if (cfg->form != MHSW_FORM_PLAIN && cfg->form != MHSW_FORM_BATCHED)
    return copy_err(errbuf, errlen, MHSW_ERR_ARG, "unknown form");
  int count = 0;
  if (cudaGetDeviceCount(&count) != cudaSuccess || count <= 0) {
    cudaGetLastError();
    return copy_err(errbuf, errlen, MHSW_ERR_NO_GPU, "no CUDA device");
  }
  if (cfg->device < 0 || cfg->device >= count) return copy_err(errbuf, errlen, MHSW_ERR_ARG, "device out of range");
  mhsw_server *s = new (std::nothrow) mhsw_server();
  if (!s) return copy_err(errbuf, errlen, MHSW_ERR_NOMEM, "out of host memory");
  s->cfg = *cfg;
  if (s->cfg.slots <= 0) s->cfg.slots = 3;
  if (s->cfg.max_pairs_per_batch <= 0) s->cfg.max_pairs_per_batch = 65536;
  if (s->cfg.flank < 0) s->cfg.flank = 200;
  if (s->cfg.queue_budget == 0) s->cfg.queue_budget = size_t(1) << 30;
  if (s->cfg.hbm_budget == 0) {
    size_t fr = 0, tot = 0;
    cudaSetDevice(s->cfg.device);
    if (cudaMemGetInfo(&fr, &tot) != cudaSuccess) {
      delete s;
      return copy_err(errbuf, errlen, MHSW_ERR_CUDA, "cudaMemGetInfo failed");
    }
    s->cfg.hbm_budget = fr / 2;
  }
  s->sc = sc;
  *out = s;
  return MHSW_OK;
}

void mhsw_server_destroy(mhsw_server *s) {
  if (!s) return;
  s->shutdown();
  delete s;
}

const char *mhsw_server_last_error(const mhsw_server *s) { return s ? s->err.c_str() : "null server"; }

int mhsw_server_load_contigs(mhsw_server *s, const char *seq, const int64_t *off, const int32_t *len, int64_t count) {
  if (!s) return MHSW_ERR_ARG;
  if (s->loaded) return s->fail(MHSW_ERR_STATE, "contigs already loaded");
  if (count <= 0 || !seq || !off || !len) return s->fail(MHSW_ERR_ARG, "no contigs");
  int64_t total = 0;
  for (int64_t i = 0; i < count; i++) {
    if (len[i] < 0 || off[i] < 0) return s->fail(MHSW_ERR_ARG, "negative offset or length at contig %lld", (long long)i);
    total = std::max(total, off[i] + len[i]);
  }
  const auto &cfg = s->cfg;
  cudaError_t e = cudaSetDevice(cfg.device);
  if (e) return s->fail(MHSW_ERR_CUDA, "cudaSetDevice: %s", cudaGetErrorString(e));
  const size_t contig_dev = (size_t)total + 16;
  if (contig_dev >= cfg.hbm_budget) return s->fail(MHSW_ERR_NOMEM, "contigs (%zu bytes) exceed the budget %zu", contig_dev, cfg.hbm_budget);
  // Slot sizing from what the contigs leave of the budget.
  int32_t pairs = cfg.max_pairs_per_batch;
  auto slot_bytes = [](int32_t p) {
    return (size_t)p * (kSlotBytesPerPair + 2 * (size_t)kReadBytesPerPair) + kSlotFixedBytes;
  };
  const size_t left = cfg.hbm_budget - contig_dev;
  int nslots = (int)std::min<size_t>((size_t)cfg.slots, left / slot_bytes(pairs));
  if (nslots < 1) {
    nslots = 1;
    while (pairs > 256 && slot_bytes(pairs) > left) pairs /= 2;
    if (slot_bytes(pairs) > left) return s->fail(MHSW_ERR_NOMEM, "budget %zu leaves no room for a slot", cfg.hbm_budget);
  }
  // Contig store: upload through a temporary device buffer, translate, keep the codes.
  char *raw = nullptr;
  if ((e = cudaMalloc(&raw, contig_dev))) return s->fail(MHSW_ERR_NOMEM, "cudaMalloc contigs: %s", cudaGetErrorString(e));
  if ((e = cudaMalloc(&s->contig_codes, contig_dev))) {
    cudaFree(raw);
    return s->fail(MHSW_ERR_NOMEM, "cudaMalloc contig codes: %s", cudaGetErrorString(e));
  }
  e = cudaMemcpy(raw, seq, (size_t)total, cudaMemcpyHostToDevice);
  if (!e) e = mhsw::launch_translate(raw, s->contig_codes, total, nullptr);
  if (!e) e = cudaDeviceSynchronize();
  cudaFree(raw);
  if (e) return s->fail(MHSW_ERR_CUDA, "contig upload: %s", cudaGetErrorString(e));
  s->contig_bytes = contig_dev;
  s->coff.assign(off, off + count);
  s->clen.assign(len, len + count);
  s->slot_pairs = pairs;
  s->slot_read_bytes = (int64_t)pairs * kReadBytesPerPair;
  s->device_bytes = contig_dev;
  for (int k = 0; k < nslots; k++) {
    auto sl = std::make_unique<Slot>();
    int rc = mhsw_driver_create(&sl->drv);
    if (!rc) rc = mhsw_driver_init(sl->drv, cfg.device, 1, cfg.match_score, cfg.mismatch_score, cfg.gap_opening_score,
                                   cfg.gap_extending_score, 0, nullptr);
    if (!rc) rc = mhsw_driver_set_ambiguity(sl->drv, cfg.ambiguity_score);
    if (rc) {
      std::string m = sl->drv ? mhsw_driver_last_error(sl->drv) : "create";
      if (sl->drv) mhsw_driver_destroy(sl->drv);
      s->shutdown();
      return s->fail(rc, "slot driver: %s", m.c_str());
    }
    sl->st = static_cast<cudaStream_t>(mhsw::driver_stream(sl->drv));
    const size_t P = (size_t)pairs, B = (size_t)s->slot_read_bytes + 16;
    e = sl->a_seq.alloc(B);
    if (!e) e = sl->a_off.alloc(P);
    if (!e) e = sl->b_off.alloc(P);
    if (!e) e = sl->a_len.alloc(P);
    if (!e) e = sl->b_len.alloc(P);
    if (!e) e = sl->out5.alloc(5 * P);
    if (!e) e = sl->h_seq.alloc(B);
    if (!e) e = sl->h_aoff.alloc(P);
    if (!e) e = sl->h_boff.alloc(P);
    if (!e) e = sl->h_alen.alloc(P);
    if (!e) e = sl->h_blen.alloc(P);
    if (!e) e = sl->h_out5.alloc(5 * P);
    s->slots.push_back(std::move(sl));
    if (e) {
      s->shutdown();
      return s->fail(MHSW_ERR_NOMEM, "slot buffers: %s", cudaGetErrorString(e));
    }
    s->device_bytes += slot_bytes(pairs);
  }
  s->loaded = true;
  for (auto &sl : s->slots) {
    Slot *p = sl.get();
    sl->th = std::thread([s, p] { s->worker(p); });
  }
  return MHSW_OK;
}

int mhsw_server_submit(mhsw_server *s, const mhsw_requests *req, int32_t *out5, int64_t *win_start, int flags,
                       uint64_t *ticket) {
  if (!s || !req || !ticket) return MHSW_ERR_ARG;
  const double t0 = now_s();
  if (!s->loaded) return s->fail(MHSW_ERR_STATE, "load contigs before submitting");
  const int32_t n = req->n;
  if (n < 0 || (n > 0 && (!req->read_seq || !req->read_off || !req->read_len || !req->contig_id ||
                          !req->contig_pos || !out5)))
    return s->fail(MHSW_ERR_ARG, "bad request batch");
  auto r = std::make_shared<Request>();
  r->n = n;
  r->out5 = out5;
  r->win_start = win_start;
  r->src = req->read_seq;
  r->src_off.assign(req->read_off, req->read_off + n);
  r->cum.resize((size_t)n + 1);
  r->len.resize((size_t)n);
  r->b_off.resize((size_t)n);
  r->b_len.resize((size_t)n);
  r->wstart.resize((size_t)n);
  int64_t total = 0;
  const int64_t nc = (int64_t)s->clen.size();
  const int64_t flank = s->cfg.flank;
  for (int32_t i = 0; i < n; i++) {
    const int32_t L = req->read_len[i], cid = req->contig_id[i], pos = req->contig_pos[i];
    if (L < 0 || L > s->slot_read_bytes) return s->fail(MHSW_ERR_LIMIT, "read %d: length %d outside [0, %lld]", i, L, (long long)s->slot_read_bytes);
    if (cid < 0 || cid >= nc) return s->fail(MHSW_ERR_ARG, "read %d: contig id %d out of range", i, cid);
    const int64_t cl = s->clen[(size_t)cid];
    if (pos < 0 || pos >= cl) return s->fail(MHSW_ERR_ARG, "read %d: position %d outside contig %d", i, pos, cid);
    const int64_t ws = std::max<int64_t>(0, pos - flank), we = std::min<int64_t>(cl, pos + L + flank);
    if (we - ws > mhsw::kMaxB) return s->fail(MHSW_ERR_LIMIT, "read %d: window of %lld bases", i, (long long)(we - ws));
    if (i > 0 && req->read_off[i] != req->read_off[i - 1] + req->read_len[i - 1]) r->contiguous = false;
    r->cum[(size_t)i] = total;
    r->len[(size_t)i] = L;
    r->b_off[(size_t)i] = s->coff[(size_t)cid] + ws;
    r->b_len[(size_t)i] = (int32_t)(we - ws);
    r->wstart[(size_t)i] = ws;
    total += L;
  }
  r->cum[(size_t)n] = total;
  r->bytes = (size_t)total + (size_t)n * 48;
  r->remaining = n;
  r->t_submit = t0;
  {
    std::unique_lock<std::mutex> lk(s->mu);
    auto room = [&] { return s->stop || s->admitted_bytes == 0 || s->admitted_bytes + r->bytes <= s->cfg.queue_budget; };
    if (!room()) {
      if (flags & MHSW_SUBMIT_NOWAIT) return MHSW_ERR_BUSY;
      s->cv_room.wait(lk, room);
    }
    if (s->stop) return MHSW_ERR_STATE;
    r->ticket = s->next_ticket++;
    s->admitted_bytes += r->bytes;
    s->submitted++;
    s->live[r->ticket] = r;
    if (n == 0) {
      r->done = true;
      r->t_start = r->t_done = now_s();
      s->admitted_bytes -= r->bytes;
      s->completed++;
    } else {
      s->queue.push_back(r);
      s->queued_pairs += n;
    }
    *ticket = r->ticket;
  }
  s->cv_work.notify_one();
  return MHSW_OK;
}

int mhsw_server_test(mhsw_server *s, uint64_t ticket, int *done) {
  if (!s || !done) return MHSW_ERR_ARG;
  std::lock_guard<std::mutex> lk(s->mu);
  auto it = s->live.find(ticket);
  if (it == s->live.end()) return s->fail(MHSW_ERR_ARG, "unknown ticket %llu", (unsigned long long)ticket);
  *done = it->second->done ? 1 : 0;
  return MHSW_OK;
}

int mhsw_server_wait(mhsw_server *s, uint64_t ticket, double *times3) {
  if (!s) return MHSW_ERR_ARG;
  std::unique_lock<std::mutex> lk(s->mu);
  auto it = s->live.find(ticket);
  if (it == s->live.end()) return s->fail(MHSW_ERR_ARG, "unknown ticket %llu", (unsigned long long)ticket);
  auto r = it->second;
  s->cv_done.wait(lk, [&] { return r->done; });
  if (times3) {
    times3[0] = r->t_submit;
    times3[1] = r->t_start;
    times3[2] = r->t_done;
  }
  s->live.erase(ticket);
  return r->status;
}

int mhsw_server_stats_get(mhsw_server *s, mhsw_server_stats *out) {
  if (!s || !out) return MHSW_ERR_ARG;
  std::lock_guard<std::mutex> lk(s->mu);
  out->submitted = s->submitted;
  out->completed = s->completed;
  out->pairs_done = s->pairs_done;
  out->cells_done = s->cells_done;
  out->micro_batches = s->micro_batches;
  out->queued_pairs = s->queued_pairs;
  out->admitted_bytes = s->admitted_bytes;
  out->slots = (int)s->slots.size();
  out->busy_slots = s->busy;
  out->slot_pairs = s->slot_pairs;
  out->device_bytes = s->device_bytes;
  return MHSW_OK;
}

}  // extern "C"
