// adept-sw/driver.hpp -- header-only drop-in for the reference's GPU aligner class.
//
// Same namespace, class and signatures as the reference header src/adept-sw/driver.hpp
// (lines 14-57), implemented over the C ABI of include/mhsw.h (libmhsw.so).  A caller
// such as klign (src/klign.cpp:361-367, :449-466) compiles unchanged against this file;
// results follow the reference's CPU aligner (StripedSmithWaterman::Aligner::Align with
// Filter(true, false, 0, 32767)), including SSW's tie-breaks and its handling of N.
//
// Behaviour kept from the reference:
//   * scores are passed as klign passes them: match positive, penalties negated;
//   * errors throw std::runtime_error (the reference's cudaErrchk, driver.cpp:17-26);
//   * get_aln_results() returns driver-owned arrays valid until the next run_kernel_*.
// Additions (defaults keep the reference behaviour of klign's CPU path):
//   * the ambiguity (N) penalty, -ALN_AMBIGUITY_COST unless set_ambiguity() is called;
//   * set_orientation() for callers that pass SSW's ref as "contigs" (test/ssw-test.cpp).
#pragma once

#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

#include "../mhsw.h"

#ifndef KLIGN_GPU_BLOCK_SIZE
#define KLIGN_GPU_BLOCK_SIZE 20000
#endif

#ifndef ALN_AMBIGUITY_COST
#define ALN_AMBIGUITY_COST 1
#endif

namespace adept_sw {

// for storing the alignment results (driver.hpp:17-23)
struct AlignmentResults {
  short *ref_begin = nullptr;
  short *query_begin = nullptr;
  short *ref_end = nullptr;
  short *query_end = nullptr;
  short *top_scores = nullptr;
};

namespace detail {
inline void check(int rc, const mhsw_driver *d, const char *what) {
  if (rc != MHSW_OK) {
    std::string msg = std::string("GPU aligner: ") + what + " failed (status " + std::to_string(rc) + ")";
    if (d) msg += std::string(": ") + mhsw_driver_last_error(d);
    throw std::runtime_error(msg);
  }
}
}  // namespace detail

inline size_t get_tot_gpu_mem() {
  size_t b = 0;
  detail::check(mhsw_get_tot_gpu_mem(&b), nullptr, "get_tot_gpu_mem");
  return b;
}

inline size_t get_avail_gpu_mem_per_rank(int totRanks, int numDevices = 0) {
  size_t b = 0;
  detail::check(mhsw_get_avail_gpu_mem_per_rank(totRanks, numDevices, &b), nullptr, "get_avail_gpu_mem_per_rank");
  return b;
}

inline std::string get_device_name(int device_id) {
  char buf[256];
  detail::check(mhsw_get_device_name(device_id, buf, sizeof(buf)), nullptr, "get_device_name");
  return std::string(buf);
}

inline int get_num_node_gpus() {
  int c = 0;
  mhsw_get_num_node_gpus(&c);
  return c;
}

// The first cudaMallocHost can take seconds; the reference starts it early (driver.hpp:31-33).
inline bool initialize_gpu(double &time_to_initialize, int &device_count, size_t &total_mem) {
  return mhsw_initialize_gpu(&time_to_initialize, &device_count, &total_mem) == MHSW_OK;
}

inline bool initialize_gpu() {
  double t;
  int c;
  size_t m;
  return initialize_gpu(t, c, m);
}

class GPUDriver {
  mhsw_driver *drv_ = nullptr;
  AlignmentResults alignments;
  std::vector<const char *> rp_, cp_;
  std::vector<int32_t> rl_, cl_;

  void marshal(std::vector<std::string> &reads, std::vector<std::string> &contigs) {
    const size_t n = contigs.size();  // the reference takes the pair count from contigs (driver.cpp:284)
    rp_.resize(n);
    cp_.resize(n);
    rl_.resize(n);
    cl_.resize(n);
    for (size_t i = 0; i < n; i++) {
      rp_[i] = reads[i].data();
      rl_[i] = (int32_t)reads[i].size();
      cp_[i] = contigs[i].data();
      cl_[i] = (int32_t)contigs[i].size();
    }
  }

 public:
  GPUDriver() { detail::check(mhsw_driver_create(&drv_), nullptr, "create"); }
  ~GPUDriver() { mhsw_driver_destroy(drv_); }
  GPUDriver(const GPUDriver &) = delete;
  GPUDriver &operator=(const GPUDriver &) = delete;

  // returns the time to execute (driver.cpp:198-247)
  double init(int upcxx_rank_me, int upcxx_rank_n, short match_score, short mismatch_score, short gap_opening_score,
              short gap_extending_score, int rlen_limit) {
    detail::check(mhsw_driver_set_ambiguity(drv_, (short)-ALN_AMBIGUITY_COST), drv_, "set_ambiguity");
    double secs = 0;
    detail::check(mhsw_driver_init(drv_, upcxx_rank_me, upcxx_rank_n, match_score, mismatch_score, gap_opening_score,
                                   gap_extending_score, rlen_limit, &secs),
                  drv_, "init");
    return secs;
  }

  void set_ambiguity(short ambiguity_score) {
    detail::check(mhsw_driver_set_ambiguity(drv_, ambiguity_score), drv_, "set_ambiguity");
  }
  void set_orientation(int orientation) {
    detail::check(mhsw_driver_set_orientation(drv_, orientation), drv_, "set_orientation");
  }
  void set_form(int form) { detail::check(mhsw_driver_set_form(drv_, form), drv_, "set_form"); }
  // Score2 mode: also compute SSW's second-best score per pair (klign's aln.score2, which
  // its GPU path otherwise sets to 0, src/klign.cpp:377-378).
  void set_score2(bool on) { detail::check(mhsw_driver_set_score2(drv_, on ? 1 : 0), drv_, "set_score2"); }
  // After run_kernel_forwards in score2 mode: the batch's second-best scores (driver-owned,
  // valid until the next run_kernel_*); nullptr when the mode is off.
  const int32_t *get_score2() {
    mhsw_aln_results r;
    detail::check(mhsw_get_aln_results(drv_, &r), drv_, "get_aln_results");
    return r.score2_32;
  }

  // CIGAR mode: the run_kernel_backwards / kernel_block round also computes what SSW's
  // Aligner::Align returns with report_cigar (klign's post-assembly SAM output,
  // src/klign.cpp:257-271, which its GPU path cannot produce, src/klign.cpp:589-600).
  void set_cigar(bool on) { detail::check(mhsw_driver_set_cigar(drv_, on ? 1 : 0), drv_, "set_cigar"); }
  // After kernel_block in CIGAR mode: SSW's cigar_string and mismatches per pair ("" and 0
  // for a score of 0).
  void get_cigars(std::vector<std::string> &cigars, std::vector<int32_t> &mismatches) {
    int64_t total = 0;
    detail::check(mhsw_last_cigar(drv_, nullptr, nullptr, nullptr, nullptr, 0, &total, 1), drv_, "last_cigar");
    const size_t n = rl_.size();
    std::vector<int32_t> nops(n);
    std::vector<int64_t> off(n + 1);
    std::vector<uint32_t> ops((size_t)total + 1);
    mismatches.resize(n);
    detail::check(mhsw_last_cigar(drv_, nops.data(), mismatches.data(), off.data(), ops.data(), (int64_t)ops.size(),
                                  &total, 1),
                  drv_, "last_cigar");
    cigars.assign(n, std::string());
    std::vector<char> buf;
    for (size_t i = 0; i < n; i++) {
      if (nops[i] <= 0) continue;
      buf.resize((size_t)nops[i] * 12 + 1);
      const int64_t len = mhsw_cigar_format(ops.data() + off[i], nops[i], buf.data(), (int64_t)buf.size());
      if (len < 0) throw std::runtime_error("adept_sw::GPUDriver::get_cigars: format failed");
      cigars[i].assign(buf.data(), (size_t)len);
    }
  }

  void run_kernel_forwards(std::vector<std::string> &reads, std::vector<std::string> &contigs, unsigned maxReadSize,
                           unsigned maxContigSize) {
    marshal(reads, contigs);
    detail::check(mhsw_run_kernel_forwards(drv_, rp_.data(), rl_.data(), cp_.data(), cl_.data(), (int32_t)cp_.size(),
                                           maxReadSize, maxContigSize),
                  drv_, "run_kernel_forwards");
  }

  void run_kernel_backwards(std::vector<std::string> &reads, std::vector<std::string> &contigs, unsigned maxReadSize,
                            unsigned maxContigSize) {
    marshal(reads, contigs);
    detail::check(mhsw_run_kernel_backwards(drv_, rp_.data(), rl_.data(), cp_.data(), cl_.data(), (int32_t)cp_.size(),
                                            maxReadSize, maxContigSize),
                  drv_, "run_kernel_backwards");
  }

  bool kernel_is_done() {
    int done = 0;
    detail::check(mhsw_kernel_is_done(drv_, &done), drv_, "kernel_is_done");
    return done != 0;
  }

  void kernel_block() { detail::check(mhsw_kernel_block(drv_), drv_, "kernel_block"); }

  AlignmentResults &get_aln_results() {
    mhsw_aln_results r;
    detail::check(mhsw_get_aln_results(drv_, &r), drv_, "get_aln_results");
    alignments.ref_begin = r.ref_begin;
    alignments.query_begin = r.query_begin;
    alignments.ref_end = r.ref_end;
    alignments.query_end = r.query_end;
    alignments.top_scores = r.top_scores;
    return alignments;
  }
};

}  // namespace adept_sw
