// gen_workloads.cpp -- seeded synthetic read/contig-window pairs for the alignment path.
//
// The reference quotes no public dataset for this path; these generators stand in for
// klign's candidate pairs with the shapes of the five workloads the path is measured on
// (lengths, divergence, N content, unrelated fraction).  Every stream is std::mt19937_64
// (its output sequence is fixed by the C++ standard); all distributions are written out
// here so the bytes are identical on x86_64 and aarch64.
//
// Mutation model: per source base, with probability p_sub a substitution to a uniformly
// chosen different base; else with probability p_indel a 1-bp indel, 50/50 an insertion of
// a uniform base (before the source base) or a deletion of the source base.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <random>
#include <string>
#include <thread>
#include <vector>

namespace {

const char kBases[4] = {'A', 'C', 'G', 'T'};

struct Rng {
  std::mt19937_64 eng;
  explicit Rng(uint64_t s) : eng(s) {}
  uint64_t next() { return eng(); }
  double u01() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }
  // inclusive [lo, hi]
  int64_t uint_in(int64_t lo, int64_t hi) { return lo + (int64_t)(u01() * (double)(hi - lo + 1)); }
  double normal() {
    double u1 = u01(), u2 = u01();
    if (u1 < 1e-300) u1 = 1e-300;
    return std::sqrt(-2.0 * std::log(u1)) * std::cos(6.283185307179586 * u2);
  }
  char base() { return kBases[next() >> 62]; }
  char other_base(char b) {
    int c = (b == 'A') ? 0 : (b == 'C') ? 1 : (b == 'G') ? 2 : 3;
    return kBases[(c + 1 + (int)uint_in(0, 2)) & 3];
  }
};

uint64_t splitmix64(uint64_t x) {
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}

void random_seq(Rng &r, int64_t n, std::string &out) {
  out.resize((size_t)n);
  for (int64_t i = 0; i < n; i++) out[(size_t)i] = r.base();
}

void mutate(Rng &r, const std::string &src, double p_sub, double p_indel, std::string &out) {
  out.clear();
  out.reserve(src.size() + 16);
  for (char b : src) {
    double u = r.u01();
    if (u < p_sub) {
      out.push_back(r.other_base(b));
    } else if (u < p_sub + p_indel) {
      if (r.u01() < 0.5) {
        out.push_back(r.base());
        out.push_back(b);
      }  // else: deletion
    } else {
      out.push_back(b);
    }
  }
}

// Embed `core` at a uniform offset in uniform random flank so the result has exactly
// `len` bases; if the core is longer, take a uniform window of it.
void embed(Rng &r, const std::string &core, int64_t len, std::string &out) {
  int64_t c = (int64_t)core.size();
  out.clear();
  if (c >= len) {
    int64_t off = r.uint_in(0, c - len);
    out.assign(core, (size_t)off, (size_t)len);
    return;
  }
  int64_t off = r.uint_in(0, len - c);
  out.reserve((size_t)len);
  for (int64_t i = 0; i < off; i++) out.push_back(r.base());
  out += core;
  while ((int64_t)out.size() < len) out.push_back(r.base());
}

void sprinkle_n(Rng &r, std::string &s, double p) {
  for (auto &ch : s)
    if (r.u01() < p) ch = 'N';
}

struct Chunk {
  std::string reads, refs;
  std::vector<int32_t> rlen, flen;
};

// One pair of configuration `cfg` from stream r.
void gen_pair(int cfg, Rng &r, std::string &read, std::string &ref, std::string &tmp) {
  switch (cfg) {
    case 0: {  // 150 bp read; 300 bp ref; 2% subs, 0.5% indels.
      random_seq(r, 150, read);
      mutate(r, read, 0.02, 0.005, tmp);
      embed(r, tmp, 300, ref);
      break;
    }
    case 1: {  // L~U[100,250]; ref = L + U[50,774] capped at 1024; 30% unrelated; 0.1% N.
      int64_t L = r.uint_in(100, 250);
      int64_t F = r.uint_in(50, 774);
      int64_t rl = std::min<int64_t>(L + F, 1024);
      bool unrelated = r.u01() < 0.30;
      random_seq(r, L, read);
      if (unrelated) {
        random_seq(r, rl, ref);
      } else {
        mutate(r, read, 0.02, 0.005, tmp);
        embed(r, tmp, rl, ref);
      }
      sprinkle_n(r, read, 0.001);
      sprinkle_n(r, ref, 0.001);
      break;
    }
    case 2: {  // 60% 150, 30% 250, 10% U[50,150]; ref lognormal(ln 400, 0.6) in [64,2048].
      double u = r.u01();
      int64_t L = u < 0.6 ? 150 : (u < 0.9 ? 250 : r.uint_in(50, 150));
      double ln = std::log(400.0) + 0.6 * r.normal();
      int64_t rl = (int64_t)std::llround(std::exp(ln));
      rl = std::min<int64_t>(std::max<int64_t>(rl, 64), 2048);
      double ps = 0.01 + 0.03 * r.u01();
      double pi = 0.002 + 0.008 * r.u01();
      random_seq(r, L, read);
      mutate(r, read, ps, pi, tmp);
      embed(r, tmp, rl, ref);
      break;
    }
    case 4: {  // 250 bp reads; ref U[2048,8192]; 20% near-identical (0.1%), rest as config 0.
      int64_t rl = r.uint_in(2048, 8192);
      bool near = r.u01() < 0.20;
      random_seq(r, 250, read);
      if (near)
        mutate(r, read, 0.0008, 0.0002, tmp);
      else
        mutate(r, read, 0.02, 0.005, tmp);
      embed(r, tmp, rl, ref);
      break;
    }
    default:
      read.clear();
      ref.clear();
  }
}

struct PairSet {
  std::string reads, refs;
  std::vector<int64_t> roff, foff;
  std::vector<int32_t> rlen, flen;
};

}  // namespace

extern "C" {

// Generates pairs [first, first + count) of configuration cfg (0, 1, 2 or 4) with the
// given seed.  Pair p draws from stream splitmix64(seed, p / 1024), so any slice of a
// workload is reproducible on its own and independent of the thread count.
void *mhsw_gen_pairs(int cfg, uint64_t seed, int64_t first, int64_t count, int nthreads) {
  const int64_t kChunk = 1024;
  PairSet *ps = new PairSet();
  if (count <= 0) {
    ps->roff.push_back(0);
    ps->foff.push_back(0);
    return ps;
  }
  int64_t c0 = first / kChunk, c1 = (first + count - 1) / kChunk;
  int64_t nchunks = c1 - c0 + 1;
  std::vector<Chunk> chunks((size_t)nchunks);
  if (nthreads < 1) nthreads = 1;
  auto work = [&](int tid) {
    std::string read, ref, tmp;
    for (int64_t ci = tid; ci < nchunks; ci += nthreads) {
      int64_t c = c0 + ci;
      Rng r(splitmix64(seed * 0x100000001B3ull + (uint64_t)c));
      Chunk &ch = chunks[(size_t)ci];
      for (int64_t k = 0; k < kChunk; k++) {
        int64_t p = c * kChunk + k;
        gen_pair(cfg, r, read, ref, tmp);  // always draw, so a pair's bytes do not depend on `first`
        if (p < first || p >= first + count) continue;
        ch.reads += read;
        ch.refs += ref;
        ch.rlen.push_back((int32_t)read.size());
        ch.flen.push_back((int32_t)ref.size());
      }
    }
  };
  std::vector<std::thread> th;
  for (int t = 1; t < nthreads; t++) th.emplace_back(work, t);
  work(0);
  for (auto &t : th) t.join();
  size_t tr = 0, tf = 0;
  for (auto &ch : chunks) {
    tr += ch.reads.size();
    tf += ch.refs.size();
  }
  ps->reads.reserve(tr);
  ps->refs.reserve(tf);
  for (auto &ch : chunks) {
    ps->reads += ch.reads;
    ps->refs += ch.refs;
    ps->rlen.insert(ps->rlen.end(), ch.rlen.begin(), ch.rlen.end());
    ps->flen.insert(ps->flen.end(), ch.flen.begin(), ch.flen.end());
  }
  // offsets[k] = start of pair k; offsets[n] = total bytes
  ps->roff.resize(ps->rlen.size() + 1);
  ps->foff.resize(ps->flen.size() + 1);
  int64_t o = 0, q = 0;
  for (size_t k = 0; k < ps->rlen.size(); k++) {
    ps->roff[k] = o;
    ps->foff[k] = q;
    o += ps->rlen[k];
    q += ps->flen[k];
  }
  ps->roff[ps->rlen.size()] = o;
  ps->foff[ps->flen.size()] = q;
  return ps;
}

int64_t mhsw_gen_count(void *h) { return (int64_t)((PairSet *)h)->rlen.size(); }
const char *mhsw_gen_reads(void *h) { return ((PairSet *)h)->reads.data(); }
const char *mhsw_gen_refs(void *h) { return ((PairSet *)h)->refs.data(); }
const int64_t *mhsw_gen_read_off(void *h) { return ((PairSet *)h)->roff.data(); }
const int64_t *mhsw_gen_ref_off(void *h) { return ((PairSet *)h)->foff.data(); }
const int32_t *mhsw_gen_read_len(void *h) { return ((PairSet *)h)->rlen.data(); }
const int32_t *mhsw_gen_ref_len(void *h) { return ((PairSet *)h)->flen.data(); }
void mhsw_gen_free(void *h) { delete (PairSet *)h; }

// ---- config 3 (serving): a resident contig set and requests against it ------------------

struct ContigSet {
  std::string seq;
  std::vector<int64_t> off;  // count + 1
  std::vector<int32_t> len;
};

// Contigs with lengths round(lognormal(ln 2000, 1.0)) clamped to [200, 200000], drawn from
// one stream until the total reaches total_bytes; the bases of contig c come from stream
// splitmix64(seed, c + 1) (uniform ACGT).
void *mhsw_gen_contigs(uint64_t seed, int64_t total_bytes, int nthreads) {
  ContigSet *cs = new ContigSet();
  Rng r(splitmix64(seed * 0x100000001B3ull));
  int64_t tot = 0;
  while (tot < total_bytes) {
    double ln = std::log(2000.0) + 1.0 * r.normal();
    int64_t L = (int64_t)std::llround(std::exp(ln));
    L = std::min<int64_t>(std::max<int64_t>(L, 200), 200000);
    cs->off.push_back(tot);
    cs->len.push_back((int32_t)L);
    tot += L;
  }
  cs->off.push_back(tot);
  cs->seq.resize((size_t)tot);
  const int64_t nc = (int64_t)cs->len.size();
  if (nthreads < 1) nthreads = 1;
  auto work = [&](int tid) {
    for (int64_t c = tid; c < nc; c += nthreads) {
      Rng g(splitmix64(seed * 0x100000001B3ull + (uint64_t)c + 1));
      char *dst = &cs->seq[(size_t)cs->off[(size_t)c]];
      for (int32_t k = 0; k < cs->len[(size_t)c]; k++) dst[k] = g.base();
    }
  };
  std::vector<std::thread> th;
  for (int t = 1; t < nthreads; t++) th.emplace_back(work, t);
  work(0);
  for (auto &t : th) t.join();
  return cs;
}

int64_t mhsw_gen_contig_count(void *h) { return (int64_t)((ContigSet *)h)->len.size(); }
const char *mhsw_gen_contig_seq(void *h) { return ((ContigSet *)h)->seq.data(); }
const int64_t *mhsw_gen_contig_off(void *h) { return ((ContigSet *)h)->off.data(); }
const int32_t *mhsw_gen_contig_len(void *h) { return ((ContigSet *)h)->len.data(); }
void mhsw_gen_contigs_free(void *h) { delete (ContigSet *)h; }

struct RequestSet {
  std::string reads;
  std::vector<int64_t> off;  // count + 1
  std::vector<int32_t> len, cid, pos;
};

// Requests [first, first + count) against a contig set (bytes, offsets, lengths, as
// host arrays): request q draws from stream
// splitmix64(seed, q / 1024).  L ~ U[100, 250]; a uniform base over the whole set picks
// the contig (length-weighted) and the seed-hit position pos, moved left so the read fits
// when it can; the read is contig[pos, pos + L) (clipped at the contig end) with 1.5%
// substitutions and 0.5% 1-bp indels (2% divergence).
void *mhsw_gen_requests(const char *cseq, const int64_t *coff, const int32_t *clen, int64_t ncontigs, uint64_t seed,
                        int64_t first, int64_t count, int nthreads) {
  const int64_t kChunk = 1024;
  RequestSet *rs = new RequestSet();
  rs->off.push_back(0);
  if (count <= 0 || ncontigs <= 0) return rs;
  std::vector<int64_t> cum((size_t)ncontigs + 1, 0);  // length-weighted choice of the contig
  for (int64_t c = 0; c < ncontigs; c++) cum[(size_t)c + 1] = cum[(size_t)c] + clen[c];
  const int64_t total = cum.back();
  if (total <= 0) return rs;
  int64_t c0 = first / kChunk, c1 = (first + count - 1) / kChunk;
  int64_t nchunks = c1 - c0 + 1;
  struct RChunk {
    std::string reads;
    std::vector<int32_t> len, cid, pos;
  };
  std::vector<RChunk> chunks((size_t)nchunks);
  if (nthreads < 1) nthreads = 1;
  auto work = [&](int tid) {
    std::string src, read;
    for (int64_t ci = tid; ci < nchunks; ci += nthreads) {
      const int64_t c = c0 + ci;
      Rng r(splitmix64((seed + 0x5151) * 0x100000001B3ull + (uint64_t)c));
      RChunk &ch = chunks[(size_t)ci];
      for (int64_t k = 0; k < kChunk; k++) {
        const int64_t q = c * kChunk + k;
        const int64_t L = r.uint_in(100, 250);
        const int64_t u = r.uint_in(0, total - 1);
        const int64_t id = (int64_t)(std::upper_bound(cum.begin(), cum.end(), u) - cum.begin()) - 1;
        const int64_t cl = clen[id];
        int64_t pos = u - cum[(size_t)id];
        pos = std::min<int64_t>(pos, std::max<int64_t>(0, cl - L));
        const int64_t take = std::min<int64_t>(L, cl - pos);
        src.assign(cseq + coff[id] + pos, (size_t)take);
        mutate(r, src, 0.015, 0.005, read);
        if (q < first || q >= first + count) continue;
        ch.reads += read;
        ch.len.push_back((int32_t)read.size());
        ch.cid.push_back((int32_t)id);
        ch.pos.push_back((int32_t)pos);
      }
    }
  };
  std::vector<std::thread> th;
  for (int t = 1; t < nthreads; t++) th.emplace_back(work, t);
  work(0);
  for (auto &t : th) t.join();
  for (auto &ch : chunks) {
    for (size_t k = 0; k < ch.len.size(); k++) rs->off.push_back(rs->off.back() + ch.len[k]);
    rs->reads += ch.reads;
    rs->len.insert(rs->len.end(), ch.len.begin(), ch.len.end());
    rs->cid.insert(rs->cid.end(), ch.cid.begin(), ch.cid.end());
    rs->pos.insert(rs->pos.end(), ch.pos.begin(), ch.pos.end());
  }
  return rs;
}

int64_t mhsw_gen_request_count(void *h) { return (int64_t)((RequestSet *)h)->len.size(); }
const char *mhsw_gen_request_reads(void *h) { return ((RequestSet *)h)->reads.data(); }
const int64_t *mhsw_gen_request_off(void *h) { return ((RequestSet *)h)->off.data(); }
const int32_t *mhsw_gen_request_len(void *h) { return ((RequestSet *)h)->len.data(); }
const int32_t *mhsw_gen_request_cid(void *h) { return ((RequestSet *)h)->cid.data(); }
const int32_t *mhsw_gen_request_pos(void *h) { return ((RequestSet *)h)->pos.data(); }
void mhsw_gen_requests_free(void *h) { delete (RequestSet *)h; }

}  // extern "C"
