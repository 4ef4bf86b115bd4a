// hoe_calib.cu — throughput of the special-function unit (sin/cos) on the
// current device, the denominator of the phase generator's ceiling.
//
// Blocks of 256 threads, 4 per SM on average; every thread runs 8 independent
// chains x <- sin(x) + cos(x) (__sincosf: one sin and one cos each), so the
// unit, not latency or issue, sets the rate.  Each block records its SM and
// clock64 before and after its loop.  The block scheduler need not place the
// same number of blocks on every SM, so the rate is taken per SM: the lane
// operations of the blocks an SM ran over the span from its first block's
// start to its last block's end (one SM's clock64 counter), summed over SMs.
// It is in SM cycles, independent of the clock.
#include "hoe_internal.cuh"

#include <algorithm>
#include <array>
#include <map>
#include <vector>

namespace hoe {
namespace {

constexpr int kChains = 8;
constexpr int kBlocksPerSm = 4;
constexpr int kThreads = 256;
constexpr int kIters = 2048;

__global__ void __launch_bounds__(kThreads) k_sfu_rate(float *sink, long long *rec, int iters) {
  float x[kChains];
#pragma unroll
  for (int j = 0; j < kChains; ++j) x[j] = 1e-3f * (float)(threadIdx.x + j);
  const long long t0 = clock64();
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int j = 0; j < kChains; ++j) {
      float s, c;
      __sincosf(x[j], &s, &c);
      x[j] = s + c;
    }
  }
  const long long t1 = clock64();
  float acc = 0.f;
#pragma unroll
  for (int j = 0; j < kChains; ++j) acc += x[j];
  sink[(int64_t)blockIdx.x * blockDim.x + threadIdx.x] = acc;   // keeps the chains live
  if (threadIdx.x == 0) {
    uint32_t sm;
    asm volatile("mov.u32 %0, %%smid;" : "=r"(sm));
    rec[3 * blockIdx.x] = t0;
    rec[3 * blockIdx.x + 1] = t1;
    rec[3 * blockIdx.x + 2] = (long long)sm;
  }
}

}  // namespace

cudaError_t sfu_rate(double *lanesPerClkPerSm, cudaStream_t st) {
  int dev = 0, nsm = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  if (e != cudaSuccess) return e;
  const int blocks = nsm * kBlocksPerSm;
  float *sink = nullptr;
  long long *cyc = nullptr;
  e = cudaMallocAsync(&sink, sizeof(float) * (size_t)blocks * kThreads, st);
  if (e == cudaSuccess) e = cudaMallocAsync(&cyc, sizeof(long long) * 3 * (size_t)blocks, st);
  std::vector<long long> h(3 * (size_t)blocks, 0);
  if (e == cudaSuccess) {
    k_sfu_rate<<<blocks, kThreads, 0, st>>>(sink, cyc, 16);      // warm-up
    k_sfu_rate<<<blocks, kThreads, 0, st>>>(sink, cyc, kIters);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(h.data(), cyc, sizeof(long long) * 3 * (size_t)blocks, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (sink) cudaFreeAsync(sink, st);
  if (cyc) cudaFreeAsync(cyc, st);
  if (e != cudaSuccess) return e;
  // per SM: first start, last end, blocks run
  std::map<long long, std::array<long long, 3>> bySm;
  for (int b = 0; b < blocks; ++b) {
    const long long t0 = h[3 * b], t1 = h[3 * b + 1], sm = h[3 * b + 2];
    auto it = bySm.find(sm);
    if (it == bySm.end()) bySm[sm] = {t0, t1, 1};
    else {
      it->second[0] = std::min(it->second[0], t0);
      it->second[1] = std::max(it->second[1], t1);
      ++it->second[2];
    }
  }
  const double perBlock = (double)kThreads * kIters * kChains * 2.0;   // sin + cos lane operations
  double ops = 0.0, cycles = 0.0;
  for (const auto &kv : bySm) {
    ops += perBlock * (double)kv.second[2];
    cycles += (double)(kv.second[1] - kv.second[0]);
  }
  *lanesPerClkPerSm = cycles > 0.0 ? ops / cycles : 0.0;
  return cudaSuccess;
}

}  // namespace hoe
