// Plain FP32 CUDA-core engine: direct summation with the anchored phase
// (FP64 anchors, FP32 residual, range reduction before sincos), plus the
// prologue/epilogue kernels shared with the tensor-core engine, the
// derivative (kspha_dt) forward and the backward pass.
//
// Forward   y[s,c] = scale * sum_v e^{+i2pi phi[s,v]} Z[v,c],   Z = x .* csm
//           (explicit_array_forward, array_operator.jl:241-288)
// Adjoint   x[v]   = scale * sum_c conj(csm[v,c]) sum_s e^{-i2pi phi[s,v]} y[s,c]
//           (explicit_array_adjoint, array_operator.jl:294-348)
// Derivative (B x)[s,c] = scale * sum_v e^{i2pi phi} 2pi i (sum_l bf[v,l] kdot[l,s]) Z[v,c]
//           (explicit_array_derivative, array_operator.jl:216-218; no fieldmap term,
//            no concomitant term)
//
// Work decomposition: one CTA of 128 threads per (sample tile, split, coil
// chunk) in the forward, one thread per sample; per (voxel tile, split, coil
// chunk) in the adjoint, one thread per voxel.  Split-K partial sums are
// written to scratch and reduced in a fixed order, so results are
// deterministic run to run.
#include <cuda_runtime.h>
#include <algorithm>
#include "hoe_internal.cuh"

namespace hoe {
namespace {

constexpr float kTwoPi = 6.28318530717958647692f;

// e^{i 2 pi f} for f already range-reduced to [-1/2, 1/2]: |argument| <= pi.
__device__ __forceinline__ void cis_reduced(float ph, float &c, float &s) {
  float f = ph - rintf(ph);
  __sincosf(kTwoPi * f, &s, &c);
}

__global__ void k_prep_Z(const float2 *__restrict__ x, const int *__restrict__ perm,
                         const float2 *__restrict__ csm, float2 *__restrict__ Z, int nVoxPad,
                         int nChaPad) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (int64_t)nVoxPad * nChaPad) return;
  int p = (int)(i / nChaPad);
  int g = perm[p];
  float2 out = make_float2(0.f, 0.f);
  if (g >= 0) {
    float2 xv = x[g], cv = csm[i];
    out = make_float2(xv.x * cv.x - xv.y * cv.y, xv.x * cv.y + xv.y * cv.x);
  }
  Z[i] = out;
}

__global__ void k_prep_Yt(const float2 *__restrict__ y, const float *__restrict__ D,
                          float2 *__restrict__ Yt, int nSam, int nCha, int nSamPad, int nChaPad) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (int64_t)nSamPad * nChaPad) return;
  int s = (int)(i / nChaPad), c = (int)(i % nChaPad);
  float2 v = make_float2(0.f, 0.f);
  if (s < nSam && c < nCha) {
    int64_t o = (int64_t)c * nSam + s;
    v = y[o];
    if (D) { float w = D[o]; v.x *= w; v.y *= w; }
  }
  Yt[i] = v;
}

template <int NC, int RP, bool DERIV>
__global__ void __launch_bounds__(128, 4)
k_fwd_simt(const float *__restrict__ kappa, const float *__restrict__ dbeta,
           const float *__restrict__ Atab, const float *__restrict__ Btab,
           const float2 *__restrict__ Z, const float *__restrict__ bfraw,
           const float *__restrict__ kdot, float2 *__restrict__ part, int nSamPad, int nVoxPad,
           int nChaPad, int nVt, int tps, int nTerm) {
  constexpr int T = kTileV;
  __shared__ __align__(16) float sD[T * RP];
  __shared__ __align__(16) float2 sZ[T * NC];
  __shared__ float sB[T];
  __shared__ __align__(16) float sR[DERIV ? T * kRF : 4];
  const int st = blockIdx.x, split = blockIdx.y, c0 = blockIdx.z * NC;
  const int tid = threadIdx.x;
  const int s = st * kTileS + tid;

  float kap[RP];
#pragma unroll
  for (int l = 0; l < RP; l += 4) {
    float4 v = *reinterpret_cast<const float4 *>(kappa + (int64_t)s * RP + l);
    kap[l] = v.x; kap[l + 1] = v.y; kap[l + 2] = v.z; kap[l + 3] = v.w;
  }
  float kd[DERIV ? kRF : 1];
  if (DERIV) {
#pragma unroll
    for (int l = 0; l < kRF; ++l) kd[l] = kdot[(int64_t)s * kRF + l];
  }
  float accR[NC], accI[NC];
#pragma unroll
  for (int c = 0; c < NC; ++c) accR[c] = accI[c] = 0.f;

  const int vt0 = split * tps, vt1 = min(nVt, vt0 + tps);
  for (int vt = vt0; vt < vt1; ++vt) {
    const float a = Atab[(int64_t)vt * nSamPad + s];
    __syncthreads();
    {
      const float4 *src = reinterpret_cast<const float4 *>(dbeta + (int64_t)vt * T * RP);
      float4 *dst = reinterpret_cast<float4 *>(sD);
      for (int i = tid; i < T * RP / 4; i += 128) dst[i] = src[i];
      if (DERIV) {
        const float4 *srcr = reinterpret_cast<const float4 *>(bfraw + (int64_t)vt * T * kRF);
        float4 *dstr = reinterpret_cast<float4 *>(sR);
        for (int i = tid; i < T * kRF / 4; i += 128) dstr[i] = srcr[i];
      }
      for (int i = tid; i < T * NC; i += 128) {
        int j = i / NC, c = i % NC;
        sZ[i] = Z[((int64_t)vt * T + j) * nChaPad + c0 + c];
      }
      sB[tid] = Btab[(int64_t)st * nVoxPad + (int64_t)vt * T + tid];
    }
    __syncthreads();
    float tR[NC], tI[NC];
#pragma unroll
    for (int c = 0; c < NC; ++c) tR[c] = tI[c] = 0.f;
#pragma unroll 2
    for (int j = 0; j < T; ++j) {
      float ph = a + sB[j];
      const float4 *d4 = reinterpret_cast<const float4 *>(sD + j * RP);
#pragma unroll
      for (int q = 0; q < RP / 4; ++q) {
        float4 d = d4[q];
        ph = fmaf(kap[4 * q], d.x, ph);
        ph = fmaf(kap[4 * q + 1], d.y, ph);
        ph = fmaf(kap[4 * q + 2], d.z, ph);
        ph = fmaf(kap[4 * q + 3], d.w, ph);
      }
      float cs, sn;
      cis_reduced(ph, cs, sn);
      if (DERIV) {
        float g = 0.f;
#pragma unroll
        for (int l = 0; l < kRF; ++l)
          if (l < nTerm) g = fmaf(kd[l], sR[j * kRF + l], g);
        float w = kTwoPi * g;
        float ncs = -w * sn, nsn = w * cs;
        cs = ncs; sn = nsn;
      }
      const float4 *z4 = reinterpret_cast<const float4 *>(sZ + j * NC);
#pragma unroll
      for (int q = 0; q < NC / 2; ++q) {
        float4 z = z4[q];
        tR[2 * q] = fmaf(cs, z.x, fmaf(-sn, z.y, tR[2 * q]));
        tI[2 * q] = fmaf(cs, z.y, fmaf(sn, z.x, tI[2 * q]));
        tR[2 * q + 1] = fmaf(cs, z.z, fmaf(-sn, z.w, tR[2 * q + 1]));
        tI[2 * q + 1] = fmaf(cs, z.w, fmaf(sn, z.z, tI[2 * q + 1]));
      }
    }
#pragma unroll
    for (int c = 0; c < NC; ++c) { accR[c] += tR[c]; accI[c] += tI[c]; }
  }
  float2 *dst = part + ((int64_t)split * nSamPad + s) * nChaPad + c0;
#pragma unroll
  for (int c = 0; c < NC; ++c) dst[c] = make_float2(accR[c], accI[c]);
}

template <int NC, int RP>
__global__ void __launch_bounds__(128, 4)
k_adj_simt(const float *__restrict__ kappa, const float *__restrict__ dbeta,
           const float *__restrict__ Atab, const float *__restrict__ Btab,
           const float2 *__restrict__ Yt, float2 *__restrict__ part, int nSamPad, int nVoxPad,
           int nChaPad, int nSt, int tps) {
  constexpr int T = kTileS;
  __shared__ __align__(16) float sK[T * RP];
  __shared__ __align__(16) float2 sY[T * NC];
  __shared__ float sA[T];
  const int vt = blockIdx.x, split = blockIdx.y, c0 = blockIdx.z * NC;
  const int tid = threadIdx.x;
  const int p = vt * kTileV + tid;

  float db[RP];
#pragma unroll
  for (int l = 0; l < RP; l += 4) {
    float4 v = *reinterpret_cast<const float4 *>(dbeta + (int64_t)p * RP + l);
    db[l] = v.x; db[l + 1] = v.y; db[l + 2] = v.z; db[l + 3] = v.w;
  }
  float accR[NC], accI[NC];
#pragma unroll
  for (int c = 0; c < NC; ++c) accR[c] = accI[c] = 0.f;

  const int st0 = split * tps, st1 = min(nSt, st0 + tps);
  for (int st = st0; st < st1; ++st) {
    const float b = Btab[(int64_t)st * nVoxPad + p];
    __syncthreads();
    {
      const float4 *src = reinterpret_cast<const float4 *>(kappa + (int64_t)st * T * RP);
      float4 *dst = reinterpret_cast<float4 *>(sK);
      for (int i = tid; i < T * RP / 4; i += 128) dst[i] = src[i];
      for (int i = tid; i < T * NC; i += 128) {
        int j = i / NC, c = i % NC;
        sY[i] = Yt[((int64_t)st * T + j) * nChaPad + c0 + c];
      }
      sA[tid] = Atab[(int64_t)vt * nSamPad + (int64_t)st * T + tid];
    }
    __syncthreads();
    float tR[NC], tI[NC];
#pragma unroll
    for (int c = 0; c < NC; ++c) tR[c] = tI[c] = 0.f;
#pragma unroll 2
    for (int j = 0; j < T; ++j) {
      float ph = sA[j] + b;
      const float4 *k4 = reinterpret_cast<const float4 *>(sK + j * RP);
#pragma unroll
      for (int q = 0; q < RP / 4; ++q) {
        float4 k = k4[q];
        ph = fmaf(k.x, db[4 * q], ph);
        ph = fmaf(k.y, db[4 * q + 1], ph);
        ph = fmaf(k.z, db[4 * q + 2], ph);
        ph = fmaf(k.w, db[4 * q + 3], ph);
      }
      float cs, sn;
      cis_reduced(ph, cs, sn);
      const float4 *y4 = reinterpret_cast<const float4 *>(sY + j * NC);
#pragma unroll
      for (int q = 0; q < NC / 2; ++q) {
        float4 y = y4[q];
        tR[2 * q] = fmaf(cs, y.x, fmaf(sn, y.y, tR[2 * q]));
        tI[2 * q] = fmaf(cs, y.y, fmaf(-sn, y.x, tI[2 * q]));
        tR[2 * q + 1] = fmaf(cs, y.z, fmaf(sn, y.w, tR[2 * q + 1]));
        tI[2 * q + 1] = fmaf(cs, y.w, fmaf(-sn, y.z, tI[2 * q + 1]));
      }
    }
#pragma unroll
    for (int c = 0; c < NC; ++c) { accR[c] += tR[c]; accI[c] += tI[c]; }
  }
  float2 *dst = part + ((int64_t)split * nVoxPad + p) * nChaPad + c0;
#pragma unroll
  for (int c = 0; c < NC; ++c) dst[c] = make_float2(accR[c], accI[c]);
}

// Sum split-K partials of the forward; write y (samples fastest) or the
// weighted, transposed Yt that feeds the adjoint of a normal application.
__global__ void k_fwd_reduce(const float2 *__restrict__ part, int nSplit, int nSamPad, int nChaPad,
                             int nSam, int nCha, float scale, const float *__restrict__ D,
                             float2 *__restrict__ y, float2 *__restrict__ Yt) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (int64_t)nSamPad * nChaPad) return;
  int s = (int)(i / nChaPad), c = (int)(i % nChaPad);
  float sr = 0.f, si = 0.f;
  for (int k = 0; k < nSplit; ++k) {
    float2 v = part[(int64_t)k * nSamPad * nChaPad + i];
    sr += v.x; si += v.y;
  }
  sr *= scale; si *= scale;
  bool valid = s < nSam && c < nCha;
  int64_t o = (int64_t)c * nSam + s;
  if (y) {
    if (valid) y[o] = make_float2(sr, si);
  } else {
    float w = (valid && D) ? D[o] : 1.f;
    Yt[i] = valid ? make_float2(sr * w, si * w) : make_float2(0.f, 0.f);
  }
}

// Sum split-K partials of the adjoint, apply conj(csm), sum coils, scale and
// scatter into the full grid (zeroed beforehand).
__global__ void k_adj_reduce(const float2 *__restrict__ part, int nSplit, int nVoxPad, int nChaPad,
                             int nCha, const float2 *__restrict__ csm, const int *__restrict__ perm,
                             float scale, float2 *__restrict__ x) {
  int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= nVoxPad) return;
  int g = perm[p];
  if (g < 0) return;
  float xr = 0.f, xi = 0.f;
  for (int c = 0; c < nCha; ++c) {
    float qr = 0.f, qi = 0.f;
    for (int k = 0; k < nSplit; ++k) {
      float2 v = part[((int64_t)k * nVoxPad + p) * nChaPad + c];
      qr += v.x; qi += v.y;
    }
    float2 m = csm[(int64_t)p * nChaPad + c];
    xr += m.x * qr + m.y * qi;   // conj(m) * q
    xi += m.x * qi - m.y * qr;
  }
  x[g] = make_float2(xr * scale, xi * scale);
}

// ---------------------------------------------------------------------------
// Backward pass.  With r = E x - y and w'[s,v] = sum_c conj(r[s,c]) Z[v,c],
//   G[s,v] = dL/dphi[s,v] = -(2 pi / sqrt(nVox)) Im(e^{i2pi phi[s,v]} w'[s,v])
//   dL/dkspha[l,s] = sum_v G bf[v,l];  dL/dfieldmap[v] = sum_s G t_s;
//   dL/dt0 = -sum_v fieldmap[v] sum_s G  -  sum_{l<nTerm,s} kdot[l,s] dL/dkspha[l,s]
// The phase is recomputed, never stored.
template <int NC, int RP>
__global__ void __launch_bounds__(128, 2)
k_bwd_simt(const float *__restrict__ kappa, const float *__restrict__ dbeta,
           const float *__restrict__ Atab, const float *__restrict__ Btab,
           const float2 *__restrict__ Z, const float2 *__restrict__ Rt,
           const float *__restrict__ bfraw, const float *__restrict__ times,
           float *__restrict__ dkpart, float *__restrict__ g1part, float *__restrict__ gtpart,
           int nSamPad, int nVoxPad, int nChaPad, int nVt, int tps, float scaleG) {
  constexpr int T = kTileV;
  __shared__ __align__(16) float sD[T * RP];
  __shared__ __align__(16) float sF[T * kRF];
  __shared__ __align__(16) float2 sZ[T * NC];
  __shared__ float sB[T];
  __shared__ float sW1[4][T];
  __shared__ float sWt[4][T];
  const int st = blockIdx.x, split = blockIdx.y;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int s = st * kTileS + tid;

  float kap[RP];
#pragma unroll
  for (int l = 0; l < RP; ++l) kap[l] = kappa[(int64_t)s * RP + l];
  float rr[NC], ri[NC];
#pragma unroll
  for (int c = 0; c < NC; ++c) {
    float2 v = Rt[(int64_t)s * nChaPad + c];
    rr[c] = v.x; ri[c] = v.y;
  }
  const float ts = times[s];
  float dk[kRF];
#pragma unroll
  for (int l = 0; l < kRF; ++l) dk[l] = 0.f;

  const int vt0 = split * tps, vt1 = min(nVt, vt0 + tps);
  for (int vt = vt0; vt < vt1; ++vt) {
    const float a = Atab[(int64_t)vt * nSamPad + s];
    __syncthreads();
    {
      const float4 *src = reinterpret_cast<const float4 *>(dbeta + (int64_t)vt * T * RP);
      const float4 *srf = reinterpret_cast<const float4 *>(bfraw + (int64_t)vt * T * kRF);
      for (int i = tid; i < T * RP / 4; i += 128) reinterpret_cast<float4 *>(sD)[i] = src[i];
      for (int i = tid; i < T * kRF / 4; i += 128) reinterpret_cast<float4 *>(sF)[i] = srf[i];
      for (int i = tid; i < T * NC; i += 128) {
        int j = i / NC, c = i % NC;
        sZ[i] = Z[((int64_t)vt * T + j) * nChaPad + c];
      }
      sB[tid] = Btab[(int64_t)st * nVoxPad + (int64_t)vt * T + tid];
    }
    __syncthreads();
    for (int j = 0; j < T; ++j) {
      float ph = a + sB[j];
#pragma unroll
      for (int l = 0; l < RP; ++l) ph = fmaf(kap[l], sD[j * RP + l], ph);
      float cs, sn;
      cis_reduced(ph, cs, sn);
      float wr = 0.f, wi = 0.f;
#pragma unroll
      for (int c = 0; c < NC; ++c) {
        float2 z = sZ[j * NC + c];
        wr = fmaf(rr[c], z.x, fmaf(ri[c], z.y, wr));
        wi = fmaf(rr[c], z.y, fmaf(-ri[c], z.x, wi));
      }
      float G = -scaleG * (cs * wi + sn * wr);
#pragma unroll
      for (int l = 0; l < kRF; ++l) dk[l] = fmaf(G, sF[j * kRF + l], dk[l]);
      float g1 = G, gt = G * ts;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        g1 += __shfl_xor_sync(0xffffffffu, g1, o);
        gt += __shfl_xor_sync(0xffffffffu, gt, o);
      }
      if (lane == 0) { sW1[warp][j] = g1; sWt[warp][j] = gt; }
    }
    __syncthreads();
    {
      int64_t o = (int64_t)st * nVoxPad + (int64_t)vt * T + tid;
      g1part[o] = (sW1[0][tid] + sW1[1][tid]) + (sW1[2][tid] + sW1[3][tid]);
      gtpart[o] = (sWt[0][tid] + sWt[1][tid]) + (sWt[2][tid] + sWt[3][tid]);
    }
  }
  float *dst = dkpart + ((int64_t)split * nSamPad + s) * kRF;
#pragma unroll
  for (int l = 0; l < kRF; ++l) dst[l] = dk[l];
}

// dL/dkspha from the split partials (dk, when given) and, when coefPart is
// given, the coefficient part of dL/dt0, -sum_{l < nTerm, s} kdot[l,s] dk[l,s],
// as one FP64 partial per block (summed in a fixed order by k_bwd_t0).
__global__ void __launch_bounds__(256) k_bwd_dk(const float *__restrict__ dkpart, int nSplit, int nSamPad, int R0,
                                                int nSam, float *__restrict__ dk, const float *__restrict__ kdot,
                                                int nTerm, double *__restrict__ coefPart) {
  pdl_wait();
  pdl_trigger();
  __shared__ double red[256];
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  double c = 0.0;
  if (i < (int64_t)nSam * R0) {
    const int s = (int)(i / R0), l = (int)(i % R0);
    float acc = 0.f;
    for (int k = 0; k < nSplit; ++k) acc += dkpart[((int64_t)k * nSamPad + s) * kRF + l];
    if (dk) dk[(int64_t)s * R0 + l] = acc;  // [nTermEff x nSam] column-major
    if (coefPart && l < nTerm) c = -(double)kdot[(int64_t)s * kRF + l] * (double)acc;
  }
  if (!coefPart) return;   // uniform over the block
  red[threadIdx.x] = c;
  __syncthreads();
  for (int o = 128; o > 0; o >>= 1) {
    if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) coefPart[blockIdx.x] = red[0];
}

// Per voxel: dL/dfieldmap and the fieldmap part of dL/dt0 (block partials in FP64).
// Sums of the partial rows [nRows][nVoxPad] per voxel in kBwdVoxSplit row
// ranges (grid.y): vpart[0][split][p] (sum_s G), vpart[1][split][p] (sum_s G t).
// A range holds a few dozen rows, summed in FP32 (GB300's FP64 add rate would
// bound this pass); the ranges are added in FP64 by k_bwd_vox.  With ddf
// given, the first range's threads also write the zeros of dL/dfieldmap
// outside the mask (k_bwd_vox writes the voxels).
__global__ void k_bwd_rows(const float *__restrict__ g1part, const float *__restrict__ gtpart, int nRows,
                           int nVoxPad, double *__restrict__ vpart, float *__restrict__ ddf,
                           const int *__restrict__ unmasked, int nUnmasked) {
  pdl_wait();
  pdl_trigger();
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= nVoxPad) return;
  if (ddf && blockIdx.y == 0)
    for (int z = p; z < nUnmasked; z += nVoxPad) ddf[unmasked[z]] = 0.f;
  const int per = (nRows + kBwdVoxSplit - 1) / kBwdVoxSplit;
  const int k0 = blockIdx.y * per, k1 = min(nRows, k0 + per);
  float a1 = 0.f, at = 0.f;
  for (int k = k0; k < k1; ++k) {
    a1 += g1part[(int64_t)k * nVoxPad + p];
    at += gtpart[(int64_t)k * nVoxPad + p];
  }
  vpart[(int64_t)blockIdx.y * nVoxPad + p] = (double)a1;
  vpart[((int64_t)kBwdVoxSplit + blockIdx.y) * nVoxPad + p] = (double)at;
}

__global__ void k_bwd_vox(const double *__restrict__ vpart, int nVoxPad, const int *__restrict__ perm,
                          const float *__restrict__ bfraw, int R0, float *__restrict__ ddf,
                          double *__restrict__ blockAcc) {
  pdl_wait();
  pdl_trigger();
  __shared__ double red[256];
  int p = blockIdx.x * blockDim.x + threadIdx.x;
  double contrib = 0.0;
  if (p < nVoxPad && perm[p] >= 0) {
    double g1 = 0.0, gt = 0.0;
    for (int k = 0; k < kBwdVoxSplit; ++k) {
      g1 += vpart[(int64_t)k * nVoxPad + p];
      gt += vpart[((int64_t)kBwdVoxSplit + k) * nVoxPad + p];
    }
    if (ddf) ddf[perm[p]] = (float)gt;
    contrib = -(double)bfraw[(int64_t)p * kRF + R0] * g1;
  }
  red[threadIdx.x] = contrib;
  __syncthreads();
  for (int o = 128; o > 0; o >>= 1) {
    if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) blockAcc[blockIdx.x] = red[0];
}

// dL/dt0: the fieldmap part from k_bwd_vox's block partials (useB0) plus
// the coefficient part from k_bwd_dk's block partials (nCoef > 0), summed by
// one block in a fixed order.
__global__ void k_bwd_t0(const double *__restrict__ blockAcc, int nBlocks, int useB0,
                         const double *__restrict__ coefPart, int nCoef, double *__restrict__ dt0) {
  pdl_wait();
  pdl_trigger();
  __shared__ double red[256];
  double acc = 0.0;
  if (useB0)
    for (int i = threadIdx.x; i < nBlocks; i += blockDim.x) acc += blockAcc[i];
  for (int i = threadIdx.x; i < nCoef; i += blockDim.x) acc += coefPart[i];
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int o = 128; o > 0; o >>= 1) {
    if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) dt0[0] = red[0];
}

template <int NC, int RP, bool DERIV>
void launch_fwd(const hoe_handle *h, int nCC, cudaStream_t st) {
  const auto &t = h->t;
  int tps = (t.nVt + h->splitF - 1) / h->splitF;
  dim3 grid(t.nSt, h->splitF, nCC);
  k_fwd_simt<NC, RP, DERIV><<<grid, 128, 0, st>>>(t.kappa, t.dbeta, t.Atab, t.Btab, h->s.Z,
                                                   t.bfraw, t.kdot, h->s.part, t.nSamPad,
                                                   t.nVoxPad, t.nChaPad, t.nVt, tps, t.nTerm);
}

template <int NC, int RP>
void launch_adj(const hoe_handle *h, int nCC, cudaStream_t st) {
  const auto &t = h->t;
  int tps = (t.nSt + h->splitA - 1) / h->splitA;
  dim3 grid(t.nVt, h->splitA, nCC);
  k_adj_simt<NC, RP><<<grid, 128, 0, st>>>(t.kappa, t.dbeta, t.Atab, t.Btab, h->s.Yt, h->s.part,
                                           t.nSamPad, t.nVoxPad, t.nChaPad, t.nSt, tps);
}

template <int NC, bool DERIV>
void dispatch_fwd_rp(const hoe_handle *h, int nCC, cudaStream_t st) {
  switch (h->t.Rp) {
    case 8: launch_fwd<NC, 8, DERIV>(h, nCC, st); break;
    case 12: launch_fwd<NC, 12, DERIV>(h, nCC, st); break;
    case 16: launch_fwd<NC, 16, DERIV>(h, nCC, st); break;
    default: launch_fwd<NC, 24, DERIV>(h, nCC, st); break;
  }
}

template <int NC>
void dispatch_adj_rp(const hoe_handle *h, int nCC, cudaStream_t st) {
  switch (h->t.Rp) {
    case 8: launch_adj<NC, 8>(h, nCC, st); break;
    case 12: launch_adj<NC, 12>(h, nCC, st); break;
    case 16: launch_adj<NC, 16>(h, nCC, st); break;
    default: launch_adj<NC, 24>(h, nCC, st); break;
  }
}

template <int NC>
void launch_bwd(const hoe_handle *h, float scaleG, cudaStream_t st) {
  const auto &t = h->t;
  int tps = (t.nVt + h->splitF - 1) / h->splitF;
  dim3 grid(t.nSt, h->splitF, 1);
  float *dkpart = h->s.gpart;
  float *g1 = dkpart + (size_t)h->splitF * t.nSamPad * kRF;
  float *gt = g1 + (size_t)t.nSt * t.nVoxPad;
#define HOE_BWD(RPV)                                                                          \
  k_bwd_simt<NC, RPV><<<grid, 128, 0, st>>>(t.kappa, t.dbeta, t.Atab, t.Btab, h->s.Z, h->s.Yt, \
                                            t.bfraw, t.times, dkpart, g1, gt, t.nSamPad,      \
                                            t.nVoxPad, t.nChaPad, t.nVt, tps, scaleG)
  switch (t.Rp) {
    case 8: HOE_BWD(8); break;
    case 12: HOE_BWD(12); break;
    case 16: HOE_BWD(16); break;
    default: HOE_BWD(24); break;
  }
#undef HOE_BWD
}

}  // namespace

cudaError_t prep_Z(const hoe_handle *h, const float2 *x, cudaStream_t st) {
  const auto &t = h->t;
  int64_t n = (int64_t)t.nVoxPad * t.nChaPad;
  k_prep_Z<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(x, t.perm, t.csm, h->s.Z, t.nVoxPad, t.nChaPad);
  h->launches += 1;
  return cudaGetLastError();
}

cudaError_t prep_Yt(const hoe_handle *h, const float2 *y, const float *D, cudaStream_t st) {
  const auto &t = h->t;
  int64_t n = (int64_t)t.nSamPad * t.nChaPad;
  k_prep_Yt<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(y, D, h->s.Yt, t.nSam, t.nCha, t.nSamPad, t.nChaPad);
  h->launches += 1;
  return cudaGetLastError();
}

cudaError_t simt_forward(const hoe_handle *h, const float2 *, float2 *y, const float *D, int mode,
                         cudaStream_t st) {
  const auto &t = h->t;
  const bool deriv = mode == FWD_DERIV_TO_Y;
  trace(h, EV_FK0, st);
  if (t.nChaPad == 4) {
    deriv ? dispatch_fwd_rp<4, true>(h, 1, st) : dispatch_fwd_rp<4, false>(h, 1, st);
  } else if (t.nChaPad == 8) {
    deriv ? dispatch_fwd_rp<8, true>(h, 1, st) : dispatch_fwd_rp<8, false>(h, 1, st);
  } else {
    int nCC = t.nChaPad / 16;
    deriv ? dispatch_fwd_rp<16, true>(h, nCC, st) : dispatch_fwd_rp<16, false>(h, nCC, st);
  }
  trace(h, EV_FK1, st);
  h->launches += 1;
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  return simt_reduce_forward(h, h->s.part, h->splitF, y, D, mode, st);
}

cudaError_t simt_reduce_forward(const hoe_handle *h, const float2 *part, int splits, float2 *y,
                                const float *D, int mode, cudaStream_t st) {
  const auto &t = h->t;
  int64_t n = (int64_t)t.nSamPad * t.nChaPad;
  float scale = (float)(1.0 / sqrt((double)t.nVox));
  bool toY = (mode == FWD_TO_Y || mode == FWD_DERIV_TO_Y);
  k_fwd_reduce<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(part, splits, t.nSamPad, t.nChaPad,
                                                          t.nSam, t.nCha, scale, D,
                                                          toY ? y : nullptr, toY ? nullptr : h->s.Yt);
  h->launches += 1;
  return cudaGetLastError();
}

cudaError_t simt_adjoint_from_Yt(const hoe_handle *h, float2 *x, cudaStream_t st) {
  const auto &t = h->t;
  trace(h, EV_AK0, st);
  if (t.nChaPad == 4) dispatch_adj_rp<4>(h, 1, st);
  else if (t.nChaPad == 8) dispatch_adj_rp<8>(h, 1, st);
  else dispatch_adj_rp<16>(h, t.nChaPad / 16, st);
  trace(h, EV_AK1, st);
  h->launches += 1;
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  return simt_reduce_adjoint(h, h->s.part, h->splitA, x, st);
}

cudaError_t simt_reduce_adjoint(const hoe_handle *h, const float2 *part, int splits, float2 *x,
                                cudaStream_t st) {
  const auto &t = h->t;
  cudaError_t e = cudaMemsetAsync(x, 0, (size_t)t.nFull * sizeof(float2), st);
  if (e != cudaSuccess) return e;
  float scale = (float)(1.0 / sqrt((double)t.nVox));
  k_adj_reduce<<<(t.nVoxPad + 255) / 256, 256, 0, st>>>(part, splits, t.nVoxPad, t.nChaPad, t.nCha,
                                                       t.csm, t.perm, scale, x);
  h->launches += 1;
  return cudaGetLastError();
}

cudaError_t simt_backward(const hoe_handle *hc, const float2 *, const float2 *r, float *dk,
                          float *ddf, double *dt0, int flags, cudaStream_t st) {
  hoe_handle *h = const_cast<hoe_handle *>(hc);
  const auto &t = h->t;
  if (t.nChaPad > 16) return cudaErrorNotSupported;
  // scratch for the gradient partials, allocated on first use (the last
  // 4 * kBwdVoxSplit * nVoxPad floats hold the FP64 voxel partial sums)
  size_t need = (size_t)h->splitF * t.nSamPad * kRF + 2 * (size_t)t.nSt * t.nVoxPad +
                4 * (size_t)kBwdVoxSplit * t.nVoxPad;
  int nVB = (t.nVoxPad + 255) / 256;
  if (h->s.gpartElems < need || !h->s.dred) {
    if (h->s.gpart) cudaFree(h->s.gpart);
    if (h->s.dred) cudaFree(h->s.dred);
    h->s.gpart = nullptr; h->s.dred = nullptr; h->s.gpartElems = 0;
    cudaError_t e = cudaMalloc(&h->s.gpart, need * sizeof(float));
    if (e != cudaSuccess) return e;
    e = cudaMalloc(&h->s.dred, (size_t)bwd_red_slots(t) * sizeof(double));
    if (e != cudaSuccess) return e;
    h->s.gpartElems = need;
    h->bytes += (int64_t)(need * sizeof(float) + bwd_red_slots(t) * sizeof(double));
  }
  cudaError_t e = prep_Yt(h, r, nullptr, st);
  if (e != cudaSuccess) return e;
  float scaleG = (float)(2.0 * 3.14159265358979323846 / sqrt((double)t.nVox));
  if (t.nChaPad == 4) launch_bwd<4>(h, scaleG, st);
  else if (t.nChaPad == 8) launch_bwd<8>(h, scaleG, st);
  else launch_bwd<16>(h, scaleG, st);
  h->launches += 1;
  e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  float *dkpart = h->s.gpart;
  float *g1 = dkpart + (size_t)h->splitF * t.nSamPad * kRF;
  float *gt = g1 + (size_t)t.nSt * t.nVoxPad;
  double *vpart = reinterpret_cast<double *>(gt + (size_t)t.nSt * t.nVoxPad);
  return bwd_finish(h, dkpart, h->splitF, g1, gt, t.nSt, vpart, h->s.dred, dk, ddf, dt0, flags, st);
}

cudaError_t bwd_finish(hoe_handle *h, const float *dkpart, int nSplit, const float *g1, const float *gt, int nRows,
                       double *vpart, double *dred, float *dk, float *ddf, double *dt0, int flags, cudaStream_t st) {
  const auto &t = h->t;
  const int nVB = (t.nVoxPad + 255) / 256;
  cudaError_t e = cudaSuccess;
  const bool coef = (flags & HOE_GRAD_T0_COEF) != 0;
  h->launches += 2 + ((flags & HOE_GRAD_KSPHA) || coef ? 1 : 0) + ((flags & (HOE_GRAD_T0_B0 | HOE_GRAD_T0_COEF)) ? 1 : 0);
  // programmatic dependent launches: each kernel waits for its predecessor
  // before its first global access (pdl_wait)
  auto ok = [&](cudaError_t r) { if (e == cudaSuccess) e = r; };
  const int64_t nDk = (int64_t)t.nSam * t.R0;
  const int nCoef = coef ? (int)((nDk + 255) / 256) : 0;   // block partials after the nVB voxel ones
  if ((flags & HOE_GRAD_KSPHA) || coef)
    ok(launch_pdl(k_bwd_dk, dim3((unsigned)((nDk + 255) / 256)), dim3(256), 0, st, dkpart, nSplit, t.nSamPad, t.R0,
                  t.nSam, (flags & HOE_GRAD_KSPHA) ? dk : (float *)nullptr, (const float *)t.kdot, t.nTerm,
                  coef ? dred + nVB : (double *)nullptr));
  float *ddfOut = (flags & HOE_GRAD_FIELDMAP) ? ddf : nullptr;
  ok(launch_pdl(k_bwd_rows, dim3(nVB, kBwdVoxSplit), dim3(256), 0, st, g1, gt, nRows, t.nVoxPad, vpart, ddfOut,
                (const int *)t.unmasked, t.nUnmasked));
  ok(launch_pdl(k_bwd_vox, dim3(nVB), dim3(256), 0, st, vpart, t.nVoxPad, (const int *)t.perm,
                (const float *)t.bfraw, t.R0, ddfOut, dred));
  if (flags & (HOE_GRAD_T0_B0 | HOE_GRAD_T0_COEF))
    ok(launch_pdl(k_bwd_t0, dim3(1), dim3(256), 0, st, (const double *)dred, nVB, (flags & HOE_GRAD_T0_B0) ? 1 : 0,
                  (const double *)(dred + nVB), nCoef, dt0));
  return e;
}

}  // namespace hoe
