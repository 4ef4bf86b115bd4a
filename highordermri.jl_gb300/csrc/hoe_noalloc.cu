// hoe_forward_noalloc: an allocation-free forward product E x.
//
// For callers that cannot allocate device memory at all: code running where
// cudaMalloc is forbidden or unavailable (a pre-allocated real-time
// reconstruction pipeline, a host framework that owns every device byte
// through its own pool, a library loaded into a process whose allocator must
// not be bypassed).  Such a caller cannot create a handle, because hoe_create
// uploads the model and allocates scratch.  This entry point therefore takes
// the model as caller-owned device arrays in the reference layout and keeps
// its only scratch (the split-K partial sums) in one file-scope
// `static __device__` array of fixed size, allocated by the CUDA runtime
// when the library's device code is loaded and held on every GPU that loads
// it until the process exits.
//
// The kernel is a variant of the plain FP32 forward (hoe_simt.cu): the same
// anchored phase (FP64 tile anchors range-reduced to [-1/2,1/2] cycles,
// FP32 residual, FP32 sincos of an argument in [-pi,pi]) and FP32
// accumulation, but the anchors are formed inside the kernel from the raw
// FP64 model instead of precomputed tables, and voxels are taken in the
// caller's mask order (chunks of consecutive masked voxels).
#include <cuda_runtime.h>
#include <cmath>
#include <cstdio>
#include <mutex>

#include "hoe_internal.cuh"

namespace {

constexpr int kT = 128;             // samples per CTA, voxels per chunk
constexpr int kMaxR = 21;           // 16 terms + 4 concomitant + fieldmap
constexpr int kRP = 24;             // padded component count
constexpr float kTwoPi = 6.28318530717958647692f;

// Static scratch: split-K partial sums [split][nSamPad][nChaPad] (complex).
constexpr size_t kScratchElems = size_t(1) << 21;  // 2 Mi complex64 = 16 MiB
static __device__ __align__(256) float2 g_noalloc_scratch[kScratchElems];

std::mutex g_mu;
void *g_scratch_ptr[64] = {};       // device address of the scratch, per device

template <int NC>
constexpr size_t noalloc_smem_bytes() {
  return sizeof(double) * (kMaxR * kT + 2 * kMaxR) + sizeof(float) * kT * kRP +
         sizeof(float2) * kT * NC + sizeof(float) * kT;
}

template <int NC>
__global__ void __launch_bounds__(128, 2)
k_fwd_noalloc(const int *__restrict__ mask_idx, const double *__restrict__ bf,
              const double *__restrict__ kspha, const double *__restrict__ times,
              const double *__restrict__ fieldmap, const float2 *__restrict__ csm,
              const float2 *__restrict__ x, float2 *__restrict__ part, int nVox, int nSam,
              int nCha, int nChaPad, int R0, int nSamPad, int chunksPerSplit) {
  // dynamic shared memory (noalloc_smem_bytes<NC>() bytes):
  //   sG   double [kMaxR][kT]  gamma of this CTA's samples, then beta of a chunk
  //   sBar double [2][kMaxR]   gammabar, betabar
  //   sD   float  [kT][kRP]    dbeta of the chunk
  //   sZ   float2 [kT][NC]     x .* csm of the chunk
  //   sB   float  [kT]         range-reduced beta . gammabar
  extern __shared__ __align__(16) unsigned char smem[];
  double(*sG)[kT] = reinterpret_cast<double(*)[kT]>(smem);
  double(*sBar)[kMaxR] = reinterpret_cast<double(*)[kMaxR]>(smem + sizeof(double) * kMaxR * kT);
  float *sD = reinterpret_cast<float *>(smem + sizeof(double) * (kMaxR * kT + 2 * kMaxR));
  float2 *sZ = reinterpret_cast<float2 *>(sD + kT * kRP);
  float *sB = reinterpret_cast<float *>(sZ + kT * NC);
  const int R = R0 + 1;
  const int tid = threadIdx.x;
  const int st = blockIdx.x, split = blockIdx.y, c0 = blockIdx.z * NC;
  const int s = st * kT + tid;
  const bool sv = s < nSam;
  const int s0 = st * kT, sn = min(kT, nSam - s0);

  // gamma_s = [kspha[:,s], times[s]] and its tile midrange gammabar
  for (int l = 0; l < R; ++l)
    sG[l][tid] = sv ? (l < R0 ? kspha[(int64_t)s * R0 + l] : times[s]) : 0.0;
  __syncthreads();
  if (tid < R) {
    double lo = sG[tid][0], hi = lo;
    for (int j = 1; j < sn; ++j) { lo = fmin(lo, sG[tid][j]); hi = fmax(hi, sG[tid][j]); }
    sBar[0][tid] = 0.5 * (lo + hi);
  }
  __syncthreads();
  double kap64[kMaxR];
  float kap[kRP];
#pragma unroll
  for (int l = 0; l < kRP; ++l) {
    double v = (l < R && sv) ? sG[l < kMaxR ? l : 0][tid] - sBar[0][l < kMaxR ? l : 0] : 0.0;
    if (l < kMaxR) kap64[l] = v;
    kap[l] = (float)v;
  }
  float accR[NC], accI[NC];
#pragma unroll
  for (int c = 0; c < NC; ++c) accR[c] = accI[c] = 0.f;

  const int nChunks = (nVox + kT - 1) / kT;
  const int ch0 = split * chunksPerSplit, ch1 = min(nChunks, ch0 + chunksPerSplit);
  for (int ch = ch0; ch < ch1; ++ch) {
    const int v0 = ch * kT, vn = min(kT, nVox - v0);
    const int v = v0 + tid;
    const bool vv = tid < vn;
    __syncthreads();  // sG / sD / sZ / sB reuse
    for (int l = 0; l < R; ++l)
      sG[l][tid] = vv ? (l < R0 ? bf[(int64_t)l * nVox + v] : (fieldmap ? fieldmap[v] : 0.0)) : 0.0;
    for (int i = tid; i < kT * NC; i += kT) {
      int j = i / NC, c = c0 + i % NC;
      float2 z = make_float2(0.f, 0.f);
      if (j < vn && c < nCha) {
        float2 xv = x[mask_idx[v0 + j]], m = csm[(int64_t)c * nVox + v0 + j];
        z = make_float2(xv.x * m.x - xv.y * m.y, xv.x * m.y + xv.y * m.x);
      }
      sZ[i] = z;
    }
    __syncthreads();
    if (tid < R) {
      double lo = sG[tid][0], hi = lo;
      for (int j = 1; j < vn; ++j) { lo = fmin(lo, sG[tid][j]); hi = fmax(hi, sG[tid][j]); }
      sBar[1][tid] = 0.5 * (lo + hi);
    }
    __syncthreads();
    {
      double b = 0.0;
      for (int l = 0; l < R; ++l) {
        b = fma(sG[l][tid], sBar[0][l], b);
        sD[tid * kRP + l] = vv ? (float)(sG[l][tid] - sBar[1][l]) : 0.f;
      }
      for (int l = R; l < kRP; ++l) sD[tid * kRP + l] = 0.f;
      sB[tid] = (float)(b - rint(b));
    }
    double a64 = 0.0;
#pragma unroll
    for (int l = 0; l < kMaxR; ++l)
      if (l < R) a64 = fma(sBar[1][l], kap64[l], a64);
    const float a = (float)(a64 - rint(a64));
    __syncthreads();
    float tR[NC], tI[NC];
#pragma unroll
    for (int c = 0; c < NC; ++c) tR[c] = tI[c] = 0.f;
    for (int j = 0; j < vn; ++j) {
      float ph = a + sB[j];
      const float4 *d4 = reinterpret_cast<const float4 *>(sD + j * kRP);
#pragma unroll
      for (int q = 0; q < kRP / 4; ++q) {
        float4 d = d4[q];
        ph = fmaf(kap[4 * q], d.x, ph);
        ph = fmaf(kap[4 * q + 1], d.y, ph);
        ph = fmaf(kap[4 * q + 2], d.z, ph);
        ph = fmaf(kap[4 * q + 3], d.w, ph);
      }
      float f = ph - rintf(ph), sn_, cs;
      __sincosf(kTwoPi * f, &sn_, &cs);
#pragma unroll
      for (int c = 0; c < NC; ++c) {
        float2 z = sZ[j * NC + c];
        tR[c] = fmaf(cs, z.x, fmaf(-sn_, z.y, tR[c]));
        tI[c] = fmaf(cs, z.y, fmaf(sn_, z.x, tI[c]));
      }
    }
#pragma unroll
    for (int c = 0; c < NC; ++c) { accR[c] += tR[c]; accI[c] += tI[c]; }
  }
  // every (split, sample, coil) slot is written, so the scratch needs no clearing
  float2 *dst = part + ((int64_t)split * nSamPad + s) * nChaPad + c0;
#pragma unroll
  for (int c = 0; c < NC; ++c) dst[c] = make_float2(accR[c], accI[c]);
}

__global__ void k_reduce_noalloc(const float2 *__restrict__ part, int nSplit, int nSamPad,
                                 int nChaPad, int nSam, int nCha, float scale,
                                 float2 *__restrict__ y) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (int64_t)nSam * nCha) return;
  int c = (int)(i / nSam), s = (int)(i % nSam);
  float sr = 0.f, si = 0.f;
  for (int k = 0; k < nSplit; ++k) {
    float2 v = part[((int64_t)k * nSamPad + s) * nChaPad + c];
    sr += v.x; si += v.y;
  }
  y[i] = make_float2(sr * scale, si * scale);
}

int noalloc_fail(int code, const char *msg) {
  char buf[320];
  snprintf(buf, sizeof(buf), "hoe_forward_noalloc: %s", msg);
  hoe::record_error(buf);  // reported by hoe_last_error(NULL)
  return code;
}

}  // namespace

extern "C" {

int hoe_forward_noalloc(const hoe_raw_model *m, const void *x_dev, void *y_dev, void *stream) {
  if (!m || !x_dev || !y_dev) return noalloc_fail(HOE_ERR_ARG, "model, x and y must be given");
  if (m->nTermEff < 1 || m->nTermEff > kMaxR - 1)
    return noalloc_fail(HOE_ERR_ARG, "nTermEff must be in 1..20");
  if (m->nVox <= 0 || m->nSam <= 0 || m->nCha <= 0)
    return noalloc_fail(HOE_ERR_ARG, "nVox, nSam and nCha must be positive");
  if (!m->mask_idx || !m->bf || !m->kspha || !m->times || !m->csm)
    return noalloc_fail(HOE_ERR_ARG, "mask_idx, bf, kspha, times and csm are required");
  const int nChaPad = m->nCha <= 4 ? 4 : (m->nCha <= 8 ? 8 : (m->nCha + 15) / 16 * 16);
  const int nSt = (m->nSam + kT - 1) / kT;
  const size_t perSplit = (size_t)nSt * kT * nChaPad;
  if (perSplit > kScratchElems)
    return noalloc_fail(HOE_ERR_DIM,
                        "ceil(nSam/128)*128 * nChaPad exceeds the static scratch of 2^21 "
                        "complex partial sums (for example nSam*nCha <= 2,097,152 with nCha a "
                        "multiple of 16)");
  // an error left by earlier work on this thread is reported as such, not as
  // a failure of this call's launches
  cudaError_t e = cudaPeekAtLastError();
  if (e != cudaSuccess) {
    char buf[200];
    snprintf(buf, sizeof(buf), "an earlier CUDA error is pending on this thread (%s)", cudaGetErrorString(e));
    return noalloc_fail(HOE_ERR_CUDA, buf);
  }
  int dev = -1;
  e = cudaGetDevice(&dev);
  if (e != cudaSuccess || dev < 0 || dev >= 64) return noalloc_fail(HOE_ERR_CUDA, "no current device");
  void *scratch = nullptr;
  {
    // one-time set-up per device, on the first call with that device current:
    // the device address of the static scratch and the kernels' shared-memory
    // limit.  With lazy module loading (the CUDA default) this first call is
    // also what loads the module, and with it the static scratch, onto the
    // device.  The cached address is not refreshed: after cudaDeviceReset
    // this entry point must not be used again in the process.
    std::lock_guard<std::mutex> lock(g_mu);
    if (!g_scratch_ptr[dev]) {
      void *ptr = nullptr;
      e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
      if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_fwd_noalloc<4>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)noalloc_smem_bytes<4>());
      if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_fwd_noalloc<8>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)noalloc_smem_bytes<8>());
      if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_fwd_noalloc<16>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)noalloc_smem_bytes<16>());
      if (e != cudaSuccess) return noalloc_fail(HOE_ERR_CUDA, cudaGetErrorString(e));
      g_scratch_ptr[dev] = ptr;
    }
    scratch = g_scratch_ptr[dev];
  }
  int numSMs = 0;
  e = cudaDeviceGetAttribute(&numSMs, cudaDevAttrMultiProcessorCount, dev);
  if (e != cudaSuccess) return noalloc_fail(HOE_ERR_CUDA, cudaGetErrorString(e));
  const int nChunks = (m->nVox + kT - 1) / kT;
  const int nCC = nChaPad <= 8 ? 1 : nChaPad / 16;
  int maxSplit = (int)(kScratchElems / perSplit);
  int want = (4 * (numSMs > 0 ? numSMs : 148) + nSt * nCC - 1) / (nSt * nCC);
  int nSplit = want < 1 ? 1 : want;
  if (nSplit > maxSplit) nSplit = maxSplit;
  if (nSplit > nChunks) nSplit = nChunks;
  int cps = (nChunks + nSplit - 1) / nSplit;
  nSplit = (nChunks + cps - 1) / cps;
  cudaStream_t st = (cudaStream_t)stream;
  dim3 grid(nSt, nSplit, nCC);
  const int nSamPad = nSt * kT;
  float2 *part = (float2 *)scratch;
#define HOE_NOALLOC(NCV)                                                                       \
  k_fwd_noalloc<NCV><<<grid, kT, noalloc_smem_bytes<NCV>(), st>>>(m->mask_idx, m->bf, m->kspha, m->times, m->fieldmap, \
                                          (const float2 *)m->csm, (const float2 *)x_dev, part,  \
                                          m->nVox, m->nSam, m->nCha, nChaPad, m->nTermEff,      \
                                          nSamPad, cps)
  if (nChaPad == 4) HOE_NOALLOC(4);
  else if (nChaPad == 8) HOE_NOALLOC(8);
  else HOE_NOALLOC(16);
#undef HOE_NOALLOC
  e = cudaGetLastError();
  if (e != cudaSuccess) return noalloc_fail(HOE_ERR_CUDA, cudaGetErrorString(e));
  int64_t n = (int64_t)m->nSam * m->nCha;
  k_reduce_noalloc<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(
      part, nSplit, nSamPad, nChaPad, m->nSam, m->nCha, (float)(1.0 / sqrt((double)m->nVox)),
      (float2 *)y_dev);
  e = cudaGetLastError();
  if (e != cudaSuccess) return noalloc_fail(HOE_ERR_CUDA, cudaGetErrorString(e));
  return HOE_OK;
}

}  // extern "C"
