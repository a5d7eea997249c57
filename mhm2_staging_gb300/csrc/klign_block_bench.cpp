// klign_block_bench.cpp -- klign's GPU call sequence through the C++ drop-in, timed.
//
// A caller written as klign writes its GPU block (src/klign.cpp:356-388): the block's
// reads and contig windows as std::vector<std::string>, at most KLIGN_GPU_BLOCK_SIZE
// (20,000) pairs, then
//   run_kernel_forwards(reads, ctgs, max_rlen, max_clen); kernel_block();
//   run_kernel_backwards(reads, ctgs, max_rlen, max_clen); kernel_block();
//   get_aln_results() -> klign's Aln fields (rstart/rstop from query_*, cstart/cstop from
//   ref_*, score1 from top_scores, :369-381)
// against include/adept-sw/driver.hpp, the header klign compiles unchanged.
//
// Input: a pair file as written by bench.py (little-endian: int64 n, int64 a_bytes,
// int64 b_bytes, a bytes, b bytes, int64 a_off[n], int64 b_off[n], int32 a_len[n],
// int32 b_len[n]; A = the read, B = the contig window).  The strings are built before
// timing, as klign has them before its call.
//   klign_block_bench <pairs file> [block pairs] [timed passes] [form] [results file]
// form: "plain" (the reference's launch model, the drop-in's default) or "batched"
// (set_form(MHSW_FORM_BATCHED)).  Prints one JSON object: pairs, blocks, seconds,
// alignments_per_s, gcups, the block times and their phases; with a results file, also
// writes n x 5 int32 (top_scores, query_begin, query_end, ref_begin, ref_end) of the last
// pass.
#include <algorithm>
#include <chrono>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

#include "adept-sw/driver.hpp"

namespace {

template <class T>
bool read_vec(std::FILE *f, std::vector<T> &v, size_t n) {
  v.resize(n);
  return n == 0 || std::fread(v.data(), sizeof(T), n, f) == n;
}

}  // namespace

int main(int argc, char **argv) {
  if (argc < 2) {
    std::fprintf(stderr, "usage: %s <pairs file> [block pairs] [timed passes] [plain|batched] [results file]\n",
                 argv[0]);
    return 2;
  }
  const size_t block = argc > 2 ? (size_t)std::atol(argv[2]) : (size_t)KLIGN_GPU_BLOCK_SIZE;
  const int passes = argc > 3 ? std::atoi(argv[3]) : 1;
  const bool batched = argc > 4 && std::string(argv[4]) == "batched";
  std::FILE *f = std::fopen(argv[1], "rb");
  if (!f || block == 0 || passes < 1) {
    std::fprintf(stderr, "cannot read %s\n", argv[1]);
    return 2;
  }
  int64_t hdr[3] = {0, 0, 0};
  std::vector<char> a, b;
  std::vector<int64_t> aoff, boff;
  std::vector<int32_t> alen, blen;
  bool ok = std::fread(hdr, sizeof(int64_t), 3, f) == 3;
  const size_t n = ok ? (size_t)hdr[0] : 0;
  ok = ok && read_vec(f, a, (size_t)hdr[1]) && read_vec(f, b, (size_t)hdr[2]) && read_vec(f, aoff, n) &&
       read_vec(f, boff, n) && read_vec(f, alen, n) && read_vec(f, blen, n);
  std::fclose(f);
  if (!ok) {
    std::fprintf(stderr, "short pair file %s\n", argv[1]);
    return 2;
  }
  // the blocks as klign holds them
  struct Block {
    std::vector<std::string> reads, ctgs;
    unsigned max_rlen = 0, max_clen = 0;
    double cells = 0;
  };
  std::vector<Block> blocks;
  for (size_t lo = 0; lo < n; lo += block) {
    Block bk;
    const size_t hi = std::min(n, lo + block);
    for (size_t i = lo; i < hi; i++) {
      bk.reads.emplace_back(a.data() + aoff[i], (size_t)alen[i]);
      bk.ctgs.emplace_back(b.data() + boff[i], (size_t)blen[i]);
      bk.max_rlen = std::max(bk.max_rlen, (unsigned)alen[i]);
      bk.max_clen = std::max(bk.max_clen, (unsigned)blen[i]);
      bk.cells += (double)alen[i] * (double)blen[i];
    }
    blocks.push_back(std::move(bk));
  }
  double cells = 0;
  for (const Block &bk : blocks) cells += bk.cells;

  adept_sw::GPUDriver drv;
  unsigned rlen_limit = 0;
  for (const Block &bk : blocks) rlen_limit = std::max(rlen_limit, bk.max_rlen);
  drv.init(0, 1, 1, -3, -5, -2, (int)rlen_limit);  // klign's scoring, negated penalties (klign.cpp:464-465)
  drv.set_ambiguity(-2);
  if (batched) drv.set_form(MHSW_FORM_BATCHED);

  std::vector<int32_t> out(n * 5);
  int64_t checksum = 0;
  // host time per phase of a block (summed over the timed blocks): the forwards call
  // (string staging, copies and launches enqueued), its kernel_block wait, the
  // backwards call, its wait, and the result mapping
  double phase_ms[5] = {0, 0, 0, 0, 0};
  bool timing_phases = false;
  auto now = [] { return std::chrono::steady_clock::now(); };
  auto run_block = [&](size_t k, bool keep) {
    Block &bk = blocks[k];
    auto t = now();
    auto lap = [&](int ph) {
      const auto u = now();
      if (timing_phases) phase_ms[ph] += std::chrono::duration<double, std::milli>(u - t).count();
      t = u;
    };
    drv.run_kernel_forwards(bk.reads, bk.ctgs, bk.max_rlen, bk.max_clen);
    lap(0);
    drv.kernel_block();
    lap(1);
    drv.run_kernel_backwards(bk.reads, bk.ctgs, bk.max_rlen, bk.max_clen);
    lap(2);
    drv.kernel_block();
    lap(3);
    adept_sw::AlignmentResults &r = drv.get_aln_results();
    // klign's mapping (klign.cpp:369-381): every pair's five fields are read
    for (size_t i = 0; i < bk.reads.size(); i++) {
      checksum += (int64_t)r.top_scores[i] + r.query_begin[i] + r.query_end[i] + r.ref_begin[i] + r.ref_end[i];
      if (keep) {
        const size_t p = k * block + i;
        int32_t *o = out.data() + 5 * p;
        o[0] = r.top_scores[i];
        o[1] = r.query_begin[i];
        o[2] = r.query_end[i];
        o[3] = r.ref_begin[i];
        o[4] = r.ref_end[i];
      }
    }
    lap(4);
  };
  // warm-up: the first blocks (buffers sized, launch shapes chosen)
  for (size_t k = 0; k < std::min<size_t>(2, blocks.size()); k++) run_block(k, false);
  std::vector<double> block_ms;
  timing_phases = true;
  const auto t0 = std::chrono::steady_clock::now();
  for (int pass = 0; pass < passes; pass++) {
    for (size_t k = 0; k < blocks.size(); k++) {
      const auto b0 = std::chrono::steady_clock::now();
      run_block(k, pass == passes - 1);
      block_ms.push_back(std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - b0).count());
    }
  }
  const double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  if (argc > 5) {
    std::FILE *o = std::fopen(argv[5], "wb");
    if (!o || std::fwrite(out.data(), sizeof(int32_t), out.size(), o) != out.size()) return 3;
    std::fclose(o);
  }
  std::vector<double> sorted = block_ms;
  std::sort(sorted.begin(), sorted.end());
  auto pct = [&](double q) { return sorted.empty() ? 0.0 : sorted[(size_t)(q * (double)(sorted.size() - 1))]; };
  const double nb = (double)(block_ms.empty() ? 1 : block_ms.size());
  std::printf(
      "{\"form\": \"%s\", \"pairs\": %zu, \"block_pairs\": %zu, \"blocks\": %zu, \"passes\": %d, "
      "\"seconds\": %.6f, "
      "\"alignments_per_s\": %.1f, \"gcups\": %.3f, \"block_ms_p50\": %.4f, \"block_ms_p99\": %.4f, "
      "\"block_ms_mean\": %.4f, \"phase_ms_mean\": {\"run_kernel_forwards\": %.4f, \"kernel_block_1\": %.4f, "
      "\"run_kernel_backwards\": %.4f, \"kernel_block_2\": %.4f, \"results\": %.4f}, \"checksum\": %lld}\n",
      batched ? "batched" : "plain", n, block, blocks.size(), passes, secs, (double)n * passes / secs, cells * passes / secs / 1e9, pct(0.5),
      pct(0.99), secs * 1e3 / (double)block_ms.size(), phase_ms[0] / nb, phase_ms[1] / nb, phase_ms[2] / nb,
      phase_ms[3] / nb, phase_ms[4] / nb, (long long)checksum);
  return 0;
}
