// mhsw_probe.cu -- throughput probe of the packed int16 DPX add-max instruction.
//
// The alignment kernels are bound by integer issue, not by HBM or tensor cores; their
// roofline is the device's cell-update rate, derived from the measured rate of the
// DPX instruction every DP cell update is built from (__viaddmax_s16x2).
#include <cuda_runtime.h>

#include <cstdint>

#include "../../include/mhsw.h"

namespace {

constexpr int kChains = 8;
constexpr int kIters = 4096;

__global__ void __launch_bounds__(256) k_dpx_probe(unsigned seed, unsigned *sink, long long *cycles) {
  unsigned acc[kChains];
#pragma unroll
  for (int c = 0; c < kChains; c++) acc[c] = seed * (threadIdx.x + 1u) + (unsigned)c;
  const unsigned b = seed | 0x00010001u;
  const long long t0 = clock64();
  for (int it = 0; it < kIters; it++) {
#pragma unroll
    for (int c = 0; c < kChains; c++) acc[c] = __viaddmax_s16x2(acc[c], b, acc[(c + 1) % kChains]);
  }
  const long long t1 = clock64();
  unsigned x = 0;
#pragma unroll
  for (int c = 0; c < kChains; c++) x ^= acc[c];
  if (x == 0x12345678u) sink[0] = x;  // keeps the chains live
  if (threadIdx.x == 0) cycles[blockIdx.x] = t1 - t0;
}

// Per-intrinsic probe: op 0 = __viaddmax_s16x2, 1 = __vimax3_s16x2, 2 = __viaddmax_s16x2_relu,
// 3 = __vimax_s16x2_relu, 4 = 32-bit integer add of three operands, 5 = integer multiply-add.
template <int OP>
__global__ void __launch_bounds__(256) k_op_probe(unsigned seed, unsigned *sink) {
  unsigned acc[kChains];
#pragma unroll
  for (int c = 0; c < kChains; c++) acc[c] = seed * (threadIdx.x + 1u) + (unsigned)c;
  const unsigned b = seed | 0x00010001u;
  for (int it = 0; it < kIters; it++) {
#pragma unroll
    for (int c = 0; c < kChains; c++) {
      const unsigned x = acc[(c + 1) % kChains];
      if (OP == 0) acc[c] = __viaddmax_s16x2(acc[c], b, x);
      if (OP == 1) acc[c] = __vimax3_s16x2(acc[c], b, x);
      if (OP == 2) acc[c] = __viaddmax_s16x2_relu(acc[c], b, x);
      if (OP == 3) acc[c] = __vimax_s16x2_relu(acc[c], x);
      if (OP == 4) acc[c] = acc[c] + b + x;
      if (OP == 5) acc[c] = acc[c] * b + x;
    }
  }
  unsigned x = 0;
#pragma unroll
  for (int c = 0; c < kChains; c++) x ^= acc[c];
  if (x == 0x12345678u) sink[0] = x;
}

template <int OP>
double time_op(int blocks, unsigned *sink) {
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  k_op_probe<OP><<<blocks, 256>>>(3u, sink);
  cudaEventRecord(e0);
  for (int r = 0; r < 3; r++) k_op_probe<OP><<<blocks, 256>>>(5u + r, sink);
  cudaEventRecord(e1);
  cudaEventSynchronize(e1);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return ms > 0.f ? (double)blocks * 256 * kIters * kChains * 3 / (ms * 1e-3) : 0.0;
}

}  // namespace

extern "C" int mhsw_probe_op_rate(int device, int op, double *ops_per_s) {
  if (!ops_per_s || op < 0 || op > 5) return MHSW_ERR_ARG;
  if (cudaSetDevice(device) != cudaSuccess) return MHSW_ERR_CUDA;
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
  unsigned *sink = nullptr;
  if (cudaMalloc(&sink, 4) != cudaSuccess) return MHSW_ERR_NOMEM;
  const int blocks = sms * 8;
  double r = 0;
  switch (op) {
    case 0: r = time_op<0>(blocks, sink); break;
    case 1: r = time_op<1>(blocks, sink); break;
    case 2: r = time_op<2>(blocks, sink); break;
    case 3: r = time_op<3>(blocks, sink); break;
    case 4: r = time_op<4>(blocks, sink); break;
    default: r = time_op<5>(blocks, sink); break;
  }
  cudaFree(sink);
  if (cudaGetLastError() != cudaSuccess || r <= 0) return MHSW_ERR_CUDA;
  *ops_per_s = r;
  return MHSW_OK;
}

extern "C" int mhsw_probe_dpx_rate(int device, double *ops_per_s, double *sm_hz) {
  if (!ops_per_s || !sm_hz) return MHSW_ERR_ARG;
  if (cudaSetDevice(device) != cudaSuccess) return MHSW_ERR_CUDA;
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
  const int blocks = sms * 8, threads = 256;
  unsigned *sink = nullptr;
  long long *cyc = nullptr;
  if (cudaMalloc(&sink, 4) != cudaSuccess) return MHSW_ERR_NOMEM;
  if (cudaMalloc(&cyc, sizeof(long long) * blocks) != cudaSuccess) {
    cudaFree(sink);
    return MHSW_ERR_NOMEM;
  }
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  k_dpx_probe<<<blocks, threads>>>(3u, sink, cyc);  // warm-up
  cudaEventRecord(e0);
  const int reps = 5;
  for (int r = 0; r < reps; r++) k_dpx_probe<<<blocks, threads>>>(5u + r, sink, cyc);
  cudaEventRecord(e1);
  cudaEventSynchronize(e1);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  long long hc[4096];
  int nb = blocks < 4096 ? blocks : 4096;
  cudaMemcpy(hc, cyc, sizeof(long long) * nb, cudaMemcpyDeviceToHost);
  double mean_cyc = 0;
  for (int i = 0; i < nb; i++) mean_cyc += (double)hc[i];
  mean_cyc /= nb;
  cudaError_t err = cudaGetLastError();
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(sink);
  cudaFree(cyc);
  if (err != cudaSuccess || ms <= 0.f) return MHSW_ERR_CUDA;
  const double ops = (double)blocks * threads * kIters * kChains * reps / 32.0;  // warp instructions
  const double secs = ms * 1e-3;
  *ops_per_s = ops * 32.0 / secs;  // lane-level packed instructions per second
  // blocks run in waves when fewer than 8 fit on an SM: each block's cycles cover one wave
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_dpx_probe, threads, 0);
  const int waves = per_sm > 0 ? (blocks + sms * per_sm - 1) / (sms * per_sm) : 1;
  *sm_hz = mean_cyc * waves / (secs / reps);
  return MHSW_OK;
}
