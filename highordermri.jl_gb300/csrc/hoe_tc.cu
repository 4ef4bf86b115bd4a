// Tensor-core engine, host side and helper kernels: B operands, reductions,
// anchor tables, plans for single operators and batches, the derivative
// product.  The contraction kernel itself is in hoe_tc_kernel.cuh.
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <algorithm>
#include <cstdint>
#include <cstdlib>
#include <string>
#include <vector>

#include "hoe_internal.cuh"
#include "hoe_tcgen05.cuh"
#include "hoe_tc_kernel.cuh"

namespace hoe {
namespace {

// B operand tiles are written in 16-byte units: unit u of a hi tile holds
// row n, k = 8*kg .. 8*kg+7 (kmajor_off), and consecutive units are
// consecutive addresses, so consecutive threads store contiguously.
__device__ __forceinline__ void bop_unit(int u, int &n, int &kg) {
  n = (u / (8 * (TK / 8))) * 8 + u % 8;
  kg = (u / 8) % (TK / 8);
}
__device__ __forceinline__ int bop_unit_of(int n, int kg) { return ((n / 8) * (TK / 8) + kg) * 8 + n % 8; }

// Eight values of one unit split into BF16 hi + lo (the lo tile follows the
// hi tile, per elements further on).
__device__ __forceinline__ void store_bop8(uint16_t *tile, int64_t per, int u, const float *v) {
  uint32_t h[4], l[4];
#pragma unroll
  for (int j = 0; j < 4; ++j) split_bf16x2(v[2 * j], v[2 * j + 1], h[j], l[j]);
  reinterpret_cast<uint4 *>(tile)[u] = make_uint4(h[0], h[1], h[2], h[3]);
  reinterpret_cast<uint4 *>(tile + per)[u] = make_uint4(l[0], l[1], l[2], l[3]);
}

// (re, im) of a complex value v in row n = 2*c + q at k = 2*j + r of the
// forward B operand: [Re, Im; -Im, Re] (r = 0, 1) by q.
__device__ __forceinline__ void bop_fwd_pair(float2 z, int q, float *v) {
  v[0] = q == 0 ? z.x : z.y;
  v[1] = q == 0 ? -z.y : z.x;
}
// ... and of the adjoint B operand: [Re, Im; Im, -Re].
__device__ __forceinline__ void bop_adj_pair(float2 z, int q, float *v) {
  v[0] = q == 0 ? z.x : z.y;
  v[1] = q == 0 ? z.y : -z.x;
}

// B operand of the forward straight from the image: chunk i covers
// tile-order voxels [i*TV, (i+1)*TV); element (n, k) with k = 2*v_local + r
// and n = 2*c + q holds (re, im) of Z = x[perm[v]] * csm[v][c].  One thread
// per 16-byte unit (4 voxels of one row n).
__global__ void k_tc_bop_forward(const float2 *__restrict__ x, const int *__restrict__ perm,
                                 const float2 *__restrict__ csm, uint16_t *__restrict__ Bop, int nChunks, int N,
                                 int nChaPad) {
  pdl_wait();
  pdl_trigger();
  const int units = N * (TK / 8);
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (int64_t)nChunks * units) return;
  const int ch = (int)(i / units), u = (int)(i % units);
  int n, kg;
  bop_unit(u, n, kg);
  const int c = n / 2, q = n & 1;
  float v[8];
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    const int vx = ch * TV + kg * 4 + j;
    float2 z = make_float2(0.f, 0.f);
    const int g = perm[vx];
    // csm rows exist for every tile-order voxel (zero padding), so its load
    // does not wait for perm
    const float2 cv = c < nChaPad ? csm[(int64_t)vx * nChaPad + c] : make_float2(0.f, 0.f);
    if (g >= 0) {
      const float2 xv = x[g];
      z = make_float2(xv.x * cv.x - xv.y * cv.y, xv.x * cv.y + xv.y * cv.x);
    }
    bop_fwd_pair(z, q, v + 2 * j);
  }
  const int64_t per = (int64_t)N * TK;
  store_bop8(Bop + (size_t)ch * 2 * per, per, u, v);
}

// B operand of the adjoint straight from the data y (samples fastest, then
// coils), weighted by D (NULL: ones): chunk i covers samples [i*TV, (i+1)*TV).
// One thread per 16-byte unit (4 samples of one row n).
__global__ void k_tc_bop_adjoint(const float2 *__restrict__ y, const float *__restrict__ D,
                                 uint16_t *__restrict__ Bop, int nChunks, int N, int nSam, int nCha) {
  pdl_wait();
  pdl_trigger();
  const int units = N * (TK / 8);
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (int64_t)nChunks * units) return;
  const int ch = (int)(i / units), u = (int)(i % units);
  int n, kg;
  bop_unit(u, n, kg);
  const int c = n / 2, q = n & 1;
  float v[8];
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    const int s = ch * TV + kg * 4 + j;
    float2 yv = make_float2(0.f, 0.f);
    if (s < nSam && c < nCha) {
      const int64_t o = (int64_t)c * nSam + s;
      yv = y[o];
      if (D) { const float w = D[o]; yv.x *= w; yv.y *= w; }
    }
    bop_adj_pair(yv, q, v + 2 * j);
  }
  const int64_t per = (int64_t)N * TK;
  store_bop8(Bop + (size_t)ch * 2 * per, per, u, v);
}

// The slots a row tile's partial sums occupy: the CTAs that own any of its
// work items, in schedule order (work items [first + r*C, first + (r+1)*C)).
struct SlotMap {
  int64_t first, W;
  int C, G;
  __device__ __forceinline__ int slots(int r) const {
    return work_owner(first + (int64_t)(r + 1) * C - 1, W, G) - work_owner(first + (int64_t)r * C, W, G) + 1;
  }
};

// Forward reduction over the written slots: y[c*nSam + s] = scale * sum, or
// (bopA != NULL) the adjoint's B operand of D * (scale * sum) for the normal
// operator.  A block takes FR_S samples and all nChaTC coils (one row tile:
// FR_S divides TM): it reads the
// slots with coils fastest, transposes through shared memory and writes y
// with samples fastest (or whole 16-byte units of the B operand).
constexpr int FR_S = 16;
__global__ void __launch_bounds__(256) k_tc_fwd_reduce(const float2 *__restrict__ part, int nSamPad, int nChaPad,
                                                       int nChaTC, int nSam, int nCha, float scale, SlotMap m,
                                                       float2 *__restrict__ y, const float *__restrict__ D,
                                                       uint16_t *__restrict__ bopA, int N) {
  pdl_wait();
  pdl_trigger();
  __shared__ float2 tile[64][FR_S + 1];
  const int s0 = blockIdx.x * FR_S;
  __shared__ int sns;
  if (threadIdx.x == 0) sns = m.slots(s0 / TM);
  __syncthreads();
  const int ns = sns;
  for (int e = threadIdx.x; e < FR_S * nChaTC; e += blockDim.x) {
    const int sl = e / nChaTC, c = e % nChaTC, s = s0 + sl;
    float sr = 0.f, si = 0.f;
    if (c < nChaPad) {
      for (int k = 0; k < ns; ++k) {
        const float2 v = part[((int64_t)k * nSamPad + s) * nChaPad + c];
        sr += v.x;
        si += v.y;
      }
    }
    tile[c][sl] = make_float2(sr * scale, si * scale);
  }
  __syncthreads();
  if (!bopA) {
    for (int e = threadIdx.x; e < FR_S * nChaTC; e += blockDim.x) {
      const int c = e / FR_S, sl = e % FR_S, s = s0 + sl;
      if (s < nSam && c < nCha) y[(int64_t)c * nSam + s] = tile[c][sl];
    }
    return;
  }
  // B operand units of these samples: rows n < N, k-groups of 4 samples
  const int64_t per = (int64_t)N * TK;
  uint16_t *t = bopA + (size_t)(s0 / TV) * 2 * per;
  const int kg0 = (s0 % TV) / 4;
  for (int e = threadIdx.x; e < N * (FR_S / 4); e += blockDim.x) {
    const int n = (e / (8 * (FR_S / 4))) * 8 + e % 8, kgl = (e / 8) % (FR_S / 4);
    const int c = n / 2, q = n & 1;
    float v[8];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int sl = kgl * 4 + j, s = s0 + sl;
      float2 z = tile[c][sl];
      const float w = (s < nSam && c < nCha) ? (D ? D[(int64_t)c * nSam + s] : 1.f) : 0.f;
      z.x *= w;
      z.y *= w;
      bop_adj_pair(z, q, v + 2 * j);
    }
    store_bop8(t, per, bop_unit_of(n, kg0 + kgl), v);
  }
}

// Derivative mode (kspha_dt), array_operator.jl:187-235:
//   (B x)[s,c] = scale sum_v e^{i phi} 2 pi i (sum_l bf[v,l] kdot[l,s]) Z[v,c]
//              = 2 pi i sum_l kdot[l,s] (E (bf_l . x))[s,c]
// so B x is formed from forward products of the 128-wide instance, each
// carrying 64 virtual coils cv = lt*CP + c: TP = 64/CP terms (l = l0 + lt)
// times the CP = nCha real coils (columns cv >= TP*CP stay zero).  One pass's
// B operand: Z[v, cv] = bf[v, l] x[perm[v]] csm[v][c] (zero for lt >= TP,
// l >= nTerm or c >= nCha).  One thread per 16-byte unit.
__global__ void k_tc_bop_deriv(const float2 *__restrict__ x, const int *__restrict__ perm,
                               const float2 *__restrict__ csm, const float *__restrict__ bfraw,
                               uint16_t *__restrict__ Bop, int nChunks, int nChaPad, int nCha, int CP, int TP,
                               int l0, int nTerm) {
  pdl_wait();
  pdl_trigger();
  constexpr int ND = 128;
  const int units = ND * (TK / 8);
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (int64_t)nChunks * units) return;
  const int ch = (int)(i / units), u = (int)(i % units);
  int n, kg;
  bop_unit(u, n, kg);
  const int cv = n / 2, q = n & 1, c = cv % CP, lt = cv / CP, l = l0 + lt;
  const bool on = lt < TP && l < nTerm && c < nCha;
  float v[8];
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    const int vx = ch * TV + kg * 4 + j;
    float2 z = make_float2(0.f, 0.f);
    const int g = perm[vx];
    if (on && g >= 0) {
      const float2 xv = x[g], cw = csm[(int64_t)vx * nChaPad + c];
      const float b = bfraw[(int64_t)vx * kRF + l];
      z = make_float2(b * (xv.x * cw.x - xv.y * cw.y), b * (xv.x * cw.y + xv.y * cw.x));
    }
    bop_fwd_pair(z, q, v + 2 * j);
  }
  const int64_t per = (int64_t)ND * TK;
  store_bop8(Bop + (size_t)ch * 2 * per, per, u, v);
}

// One derivative pass: y[c*nSam + s] (+)= scale2pi * i * sum_{lt < TP}
// kdot[s][l0 + lt] * (sum over the written slots of part[.][s][lt*CP + c]).
// The first pass writes y, later passes add to it (fixed order).
__global__ void k_tc_deriv_reduce(const float2 *__restrict__ part, int nSamPad, int nSam, int nCha, int CP, int l0,
                                  int TP, int nTerm, const float *__restrict__ kdot, float scale2pi, SlotMap m,
                                  float2 *__restrict__ y, int accumulate) {
  pdl_wait();
  pdl_trigger();
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (int64_t)nSamPad * CP) return;
  const int s = (int)(i / CP), c = (int)(i % CP);
  if (s >= nSam || c >= nCha) return;
  const int ns = m.slots(s / TM);
  float rr = 0.f, ri = 0.f;
  for (int lt = 0; lt < TP && l0 + lt < nTerm; ++lt) {
    float ar = 0.f, ai = 0.f;
    for (int k = 0; k < ns; ++k) {
      const float2 v = part[((int64_t)k * nSamPad + s) * 64 + lt * CP + c];
      ar += v.x;
      ai += v.y;
    }
    const float kd = kdot[(int64_t)s * kRF + l0 + lt];
    rr = fmaf(kd, ar, rr);
    ri = fmaf(kd, ai, ri);
  }
  const int64_t o = (int64_t)c * nSam + s;
  float2 out = make_float2(-scale2pi * ri, scale2pi * rr);   // i * (rr + i ri)
  if (accumulate) {
    const float2 old = y[o];
    out.x += old.x;
    out.y += old.y;
  }
  y[o] = out;
}

// Adjoint reduction over the written slots: conj(csm), sum over coils,
// scale, scatter into the full grid; the threads after the voxels' write
// zeros to the grid points outside the mask.  L = min(nChaPad,
// 32) consecutive lanes take one voxel, coils innermost, so that the slot
// and csm loads are coalesced; the coil sum is a shuffle reduction over the
// L lanes (every lane of the warp takes part).  A block of 256 threads
// covers 256 / L voxels of one row tile (L divides 32, TM = 128), so the
// slot count is computed once per block.  Padding voxels have slot and csm
// rows too, so those loads do not wait for perm.
__global__ void __launch_bounds__(256) k_tc_adj_reduce(const float2 *__restrict__ part, int nVoxPad, int nChaPad,
                                                       int nCha, const float2 *__restrict__ csm,
                                                       const int *__restrict__ perm, float scale, SlotMap m,
                                                       const int *__restrict__ unmasked, int nUnmasked,
                                                       float2 *__restrict__ x) {
  pdl_wait();
  pdl_trigger();
  const int L = nChaPad < 32 ? nChaPad : 32;
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int p = (int)(i / L), l = (int)(i % L);
  __shared__ int sns;
  if (threadIdx.x == 0) {
    const int p0 = (int)((int64_t)blockIdx.x * blockDim.x / L);
    sns = p0 < nVoxPad ? m.slots(p0 / TM) : 0;
  }
  __syncthreads();
  const int g = p < nVoxPad ? perm[p] : -1;
  float xr = 0.f, xi = 0.f;
  if (p < nVoxPad) {
    const int ns = sns;
    for (int c = l; c < nCha; c += L) {
      float qr = 0.f, qi = 0.f;
      for (int k = 0; k < ns; ++k) {
        const float2 v = part[((int64_t)k * nVoxPad + p) * nChaPad + c];
        qr += v.x;
        qi += v.y;
      }
      const float2 w = csm[(int64_t)p * nChaPad + c];
      xr += w.x * qr + w.y * qi;   // conj(w) * q
      xi += w.x * qi - w.y * qr;
    }
  }
  for (int o = L / 2; o > 0; o >>= 1) {
    xr += __shfl_down_sync(0xffffffffu, xr, o, L);
    xi += __shfl_down_sync(0xffffffffu, xi, o, L);
  }
  if (l == 0 && g >= 0) x[g] = make_float2(xr * scale, xi * scale);   // padding voxels (g < 0) are dropped
  const int64_t z = i - (int64_t)nVoxPad * L;   // nVoxPad * L is a multiple of 32: whole warps
  if (z >= 0 && z < nUnmasked) x[unmasked[z]] = make_float2(0.f, 0.f);
}

// Anchor tables of the anchor k-step: v = 2*pi*tab[i] (radians) split into
// TF32 hi + lo, stored as [hi, lo] (8 bytes; the kernels supply the
// constant halves of the k-step operands in shared memory).
__device__ __forceinline__ float tf32_rn(float f) {
  uint32_t b = __float_as_uint(f);
  if ((b & 0x7f800000u) != 0x7f800000u) {
    b += 0x00000fffu + ((b >> 13) & 1u);
    b &= 0xffffe000u;
  }
  return __uint_as_float(b);
}

__global__ void k_tc_anchor_tf32(const float *__restrict__ tab, int64_t n, float2 *__restrict__ out) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double v = 6.283185307179586476925 * (double)tab[i];
  const float h = tf32_rn((float)v);
  const float l = tf32_rn((float)(v - (double)h));
  out[i] = make_float2(h, l);
}

int tc_ncha(int nCha) {
  int n = 8;
  while (n < nCha) n *= 2;
  return n;  // 8, 16, 32 or 64 coils per MMA: N = 16, 32, 64, 128
}


}  // namespace

bool tc_supported(const hoe_handle *h, std::string *why) {
  int dev = h->device, major = 0, minor = 0;
  cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev);
  cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, dev);
  if (major != 10 || minor != 3) {
    if (why) *why = "tcgen05 kernels are built for sm_103a (GB300) only";
    return false;
  }
  if (tc_ncha(h->t.nCha) > 64) {
    if (why) *why = "the tensor-core engine supports up to 64 coils";
    return false;
  }
  if (!(h->t.residBound <= kTcMaxPhaseBound)) {
    if (why) *why = "the residual phase bound of this plan exceeds the tensor-core engine's 1024 cycles";
    return false;
  }
  return true;
}

cudaError_t tc_prepare(hoe_handle *h) {
  if (h->tc.ready) return cudaSuccess;
  const auto &t = h->t;
  TcBuffers b;
  b.nChaTC = tc_ncha(t.nCha);
  b.N = 2 * b.nChaTC;
  const int bps = configure_kernel<1>(t.KP, b.N);
  if (bps < 1) return cudaErrorInvalidConfiguration;
  const int chunksF = t.nVoxPad / TV, chunksA = t.nSamPad / TV;
  const int G = h->numSMs * bps;
  b.gridF = (int)std::min<int64_t>(G, (int64_t)t.nSt * chunksF);
  b.gridA = (int)std::min<int64_t>(G, (int64_t)t.nVt * chunksA);
  b.slotsF = max_slots(t.nSt, chunksF, b.gridF);
  b.slotsA = max_slots(t.nVt, chunksA, b.gridA);
  b.bopFElems = (size_t)chunksF * 2 * b.N * TK;
  b.bopAElems = (size_t)chunksA * 2 * b.N * TK;
  b.partElems = std::max((size_t)b.slotsF * t.nSamPad, (size_t)b.slotsA * t.nVoxPad) * t.nChaPad;
  const size_t nAP = (size_t)t.nVt * t.nSamPad, nBQ = (size_t)t.nSt * t.nVoxPad;
  size_t bytes = b.bopFElems * 2 + 256 + b.bopAElems * 2 + 256 + b.partElems * sizeof(float2) + 256 + 256 +
                 (nAP + nBQ) * 8 + 512;
  unsigned char *buf = nullptr;
  cudaError_t e = cudaMalloc(&buf, bytes);
  if (e != cudaSuccess) return e;
  size_t off = 0;
  auto take = [&](size_t n) { unsigned char *p = buf + off; off = (off + n + 255) / 256 * 256; return p; };
  b.bopF = (uint16_t *)take(b.bopFElems * 2);
  b.bopA = (uint16_t *)take(b.bopAElems * 2);
  b.part = (float2 *)take(b.partElems * sizeof(float2));
  b.err = (int *)take(sizeof(int));
  b.AtabP = (float *)take(nAP * 8);
  b.BtabQ = (float *)take(nBQ * 8);
  e = cudaMemset(b.err, 0, sizeof(int));
  if (e != cudaSuccess) { cudaFree(buf); return e; }
  h->tc.buf = buf;
  h->tc.bytes = bytes;
  h->tc.ready = true;
  // failure detection test (host-side injection): HOE_INJECT_TC_STALL=k makes
  // the first forward contraction of this operator stall CTA 0 at stage k
  if (const char *inj = getenv("HOE_INJECT_TC_STALL")) b.injectStall1 = atoi(inj) + 1;
  h->tc_host = new TcBuffers(b);
  e = tc_anchor_tables(h, 0);
  if (e == cudaSuccess) e = cudaStreamSynchronize(0);
  if (e == cudaSuccess && h->tcPlan > 0) e = tc_set_plan(h, h->tcPlan);
  return e;
}

void tc_release(hoe_handle *h) {
  if (h->tc.buf) cudaFree(h->tc.buf);
  if (h->tc_host && ((TcBuffers *)h->tc_host)->memD) cudaFree(((TcBuffers *)h->tc_host)->memD);
  delete (TcBuffers *)h->tc_host;
  h->tc_host = nullptr;
  h->tc = TcState();
}

namespace {

// Operands of one operator for one direction.
TcSlice slice_forward(const hoe_handle *h, const TcBuffers &b) {
  const auto &t = h->t;
  TcSlice sl{};
  sl.rowHi = t.kpHi; sl.rowLo = t.kpLo;
  sl.colHi = t.dbHi; sl.colLo = t.dbLo;
  sl.rowX = b.AtabP;
  sl.rowXStride = t.nSamPad;
  sl.colX = b.BtabQ;
  sl.colXStride = t.nVoxPad;
  sl.Bop = b.bopF;
  sl.part = b.part;
  sl.nRowPad = t.nSamPad;
  sl.nColChunks = t.nVoxPad / TV;
  sl.nRowTiles = t.nSt;
  return sl;
}

TcSlice slice_adjoint(const hoe_handle *h, const TcBuffers &b) {
  const auto &t = h->t;
  TcSlice sl{};
  sl.rowHi = t.dbHi; sl.rowLo = t.dbLo;
  sl.colHi = t.kpHi; sl.colLo = t.kpLo;
  sl.rowX = b.BtabQ;
  sl.rowXStride = t.nVoxPad;
  sl.colX = b.AtabP;
  sl.colXStride = t.nSamPad;
  sl.Bop = b.bopA;
  sl.part = b.part;
  sl.nRowPad = t.nVoxPad;
  sl.nColChunks = t.nSamPad / TV;
  sl.nRowTiles = t.nVt;
  return sl;
}

SlotMap slot_map(int64_t first, int C, int64_t W, int G) {
  SlotMap m;
  m.first = first;
  m.W = W;
  m.C = C;
  m.G = G;
  return m;
}

cudaError_t bop_forward(const hoe_handle *h, const TcBuffers &b, const float2 *x, cudaStream_t st) {
  const auto &t = h->t;
  const int chunks = t.nVoxPad / TV;
  const int64_t n = (int64_t)chunks * b.N * (TK / 8);   // 16-byte units
  const cudaError_t e = launch_pdl(k_tc_bop_forward, dim3((unsigned)((n + 255) / 256)), dim3(256), 0, st, x,
                                   t.perm, t.csm, b.bopF, chunks, b.N, t.nChaPad);
  h->launches += 1;
  return e;
}

cudaError_t bop_adjoint(const hoe_handle *h, const TcBuffers &b, const float2 *y, const float *D, cudaStream_t st) {
  const auto &t = h->t;
  const int chunks = t.nSamPad / TV;
  const int64_t n = (int64_t)chunks * b.N * (TK / 8);   // 16-byte units
  const cudaError_t e = launch_pdl(k_tc_bop_adjoint, dim3((unsigned)((n + 255) / 256)), dim3(256), 0, st, y, D,
                                   b.bopA, chunks, b.N, t.nSam, t.nCha);
  h->launches += 1;
  return e;
}

// y = E x (toBop false), or the adjoint B operand of D * E x (toBop true).
cudaError_t reduce_forward(const hoe_handle *h, const TcBuffers &b, const SlotMap &m, float2 *y, const float *D,
                           bool toBop, cudaStream_t st) {
  const auto &t = h->t;
  static_assert(TM % FR_S == 0 && TV % FR_S == 0, "reduction blocks within one row tile and one chunk");
  const float scale = (float)(1.0 / sqrt((double)t.nVox));
  const cudaError_t e = launch_pdl(k_tc_fwd_reduce, dim3((unsigned)(t.nSamPad / FR_S)), dim3(256), 0, st, b.part,
                                   t.nSamPad, t.nChaPad, b.nChaTC, t.nSam, t.nCha, scale, m, y, D,
                                   toBop ? b.bopA : nullptr, b.N);
  h->launches += 1;
  return e;
}

cudaError_t reduce_adjoint(const hoe_handle *h, const TcBuffers &b, const SlotMap &m, float2 *x, cudaStream_t st) {
  const auto &t = h->t;
  const float scale = (float)(1.0 / sqrt((double)t.nVox));
  const int lanes = t.nChaPad < 32 ? t.nChaPad : 32;   // per voxel; divides 32
  const int64_t n = (int64_t)t.nVoxPad * lanes + t.nUnmasked;
  const cudaError_t e2 = launch_pdl(k_tc_adj_reduce, dim3((unsigned)((n + 255) / 256)), dim3(256), 0, st, b.part,
                                    t.nVoxPad, t.nChaPad, t.nCha, t.csm, t.perm, scale, m, t.unmasked,
                                    t.nUnmasked, x);
  h->launches += 1;
  return e2;
}

TcParams<1> single_params(const hoe_handle *h, const TcBuffers &b, const TcSlice &sl) {
  TcParams<1> p{};
  p.err = b.err;
  p.nSlices = 1;
  p.nChaPad = h->t.nChaPad;
  p.nChaTC = b.nChaTC;
  p.s[0] = sl;
  p.s[0].first = 0;
  p.work = (int64_t)sl.nRowTiles * sl.nColChunks;
  return p;
}

// Several operators with the same coil count in one persistent launch per
// direction: slices grouped by residual width KP, at most kBatchSlices per
// launch, work items of a group split evenly over its CTAs.
struct TcBatchPlan {
  struct Group {
    int KP = 0, G_F = 1, G_A = 1;
    std::vector<int> idx;                 // slices of this launch
    TcParams<kBatchSlices> pF{}, pA{};
  };
  std::vector<hoe_handle *> hs;
  std::vector<int> slotsF, slotsA;        // partial slots per slice
  std::vector<SlotMap> mapF, mapA;        // each slice's place in its launch
  std::vector<Group> groups;
  int *err = nullptr;                     // device word shared by the batch's launches
};

int slots_needed(int64_t first, int rowTiles, int C, int64_t W, int G) {
  int J = 1;
  for (int r = 0; r < rowTiles; ++r) {
    int b0 = work_owner(first + (int64_t)r * C, W, G), b1 = work_owner(first + (int64_t)(r + 1) * C - 1, W, G);
    J = std::max(J, b1 - b0 + 1);
  }
  return J;
}

}  // namespace

namespace {

// A single operator's contraction with its execution plan (TcPlan; plans
// above 0 exist for up to 16 coils, N <= 32).
cudaError_t launch_planned(const hoe_handle *h, const TcBuffers &b, const TcParams<1> &p, int G, cudaStream_t st) {
  if (b.plan == 0) return launch(h, p, h->t.KP, b.N, G, st);
  return b.N == 16 ? tc_launch_plan16(h, p, h->t.KP, b.plan, G, st)
                   : tc_launch_plan32(h, p, h->t.KP, b.plan, G, st);
}

cudaError_t contract_forward(const hoe_handle *h, const TcBuffers &b, cudaStream_t st) {
  TcParams<1> p = single_params(h, b, slice_forward(h, b));
  if (b.injectStall1 > 0) {
    // failure detection test: CTA 0 never receives this stage's operands and
    // its waits run out after 1 ms; the kernel reports HOE_ERR_TIMEOUT
    p.stallStage1 = b.injectStall1;
    p.waitNs = 1000000;
    b.injectStall1 = 0;
  }
  trace(h, EV_FK0, st);
  cudaError_t e = launch_planned(h, b, p, b.gridF, st);
  trace(h, EV_FK1, st);
  return e;
}

cudaError_t contract_adjoint(const hoe_handle *h, const TcBuffers &b, cudaStream_t st) {
  const TcParams<1> p = single_params(h, b, slice_adjoint(h, b));
  trace(h, EV_AK0, st);
  cudaError_t e = launch_planned(h, b, p, b.gridA, st);
  trace(h, EV_AK1, st);
  return e;
}

SlotMap single_map_forward(const hoe_handle *h, const TcBuffers &b) {
  const int C = h->t.nVoxPad / TV;
  return slot_map(0, C, (int64_t)h->t.nSt * C, b.gridF);
}

SlotMap single_map_adjoint(const hoe_handle *h, const TcBuffers &b) {
  const int C = h->t.nSamPad / TV;
  return slot_map(0, C, (int64_t)h->t.nVt * C, b.gridA);
}

}  // namespace

cudaError_t tc_forward(const hoe_handle *h, const float2 *x, float2 *y, cudaStream_t st) {
  const TcBuffers &b = *(const TcBuffers *)h->tc_host;
  cudaError_t e = bop_forward(h, b, x, st);
  if (e == cudaSuccess) e = contract_forward(h, b, st);
  if (e == cudaSuccess) e = reduce_forward(h, b, single_map_forward(h, b), y, nullptr, false, st);
  return e;
}

cudaError_t tc_adjoint(const hoe_handle *h, const float2 *y, const float *D, float2 *x, cudaStream_t st) {
  const TcBuffers &b = *(const TcBuffers *)h->tc_host;
  cudaError_t e = bop_adjoint(h, b, y, D, st);
  if (e == cudaSuccess) e = contract_adjoint(h, b, st);
  if (e == cudaSuccess) e = reduce_adjoint(h, b, single_map_adjoint(h, b), x, st);
  return e;
}

cudaError_t tc_normal(const hoe_handle *h, const float *D, const float2 *x, float2 *out, cudaStream_t st) {
  const TcBuffers &b = *(const TcBuffers *)h->tc_host;
  cudaError_t e = bop_forward(h, b, x, st);
  if (e == cudaSuccess) e = contract_forward(h, b, st);
  if (e == cudaSuccess) e = reduce_forward(h, b, single_map_forward(h, b), nullptr, D, true, st);
  if (e == cudaSuccess) e = contract_adjoint(h, b, st);
  if (e == cudaSuccess) e = reduce_adjoint(h, b, single_map_adjoint(h, b), out, st);
  return e;
}

int tc_plan_count(const hoe_handle *h) {
  return h->tc_host && ((const TcBuffers *)h->tc_host)->N <= 32 ? kTcPlans : 1;
}

int tc_get_plan(const hoe_handle *h) { return h->tc_host ? ((const TcBuffers *)h->tc_host)->plan : 0; }

// Selects the contraction's execution plan for this operator's forward and
// adjoint products (batches and the derivative product use plan 0); sets the
// kernel's shared-memory limit on first use.
cudaError_t tc_set_plan(hoe_handle *h, int plan) {
  if (!h->tc_host || plan < 0 || plan >= tc_plan_count(h)) return cudaErrorInvalidValue;
  TcBuffers &b = *(TcBuffers *)h->tc_host;
  if (plan > 0) {
    const int nb = b.N == 16 ? tc_configure_plan16(h->t.KP, plan) : tc_configure_plan32(h->t.KP, plan);
    if (nb < 1) return cudaErrorInvalidConfiguration;
  }
  b.plan = plan;
  return cudaSuccess;
}

bool tc_derivative_supported(const hoe_handle *h) { return h->tc.ready && h->t.hasKdot; }

// B x in derivative mode.  Up to 16 coils (N <= 32) one pass of the forward
// kernel's derivative instance (hoe_tc_deriv.cu): bop_forward, the contraction
// with the phase tile scaled by 2 pi i F, reduce_forward.  Above 16 coils
// ceil(nTerm / TP) passes of the 128-wide instance, TP = 64 / CP terms of
// CP = nCha coils each (k_tc_bop_deriv, k_tc_deriv_reduce).
// tc_derivative_prepare allocates the buffers once (and builds the basis
// tiles); the delay search calls it before its graph capture.
cudaError_t tc_derivative_prepare(hoe_handle *h) {
  TcBuffers &b = *(TcBuffers *)h->tc_host;
  const auto &t = h->t;
  const int chunks = t.nVoxPad / TV;
  constexpr int ND = 128;
  if (b.memD) return cudaSuccess;
  if (b.N <= 32) {
    const size_t bfB = ((size_t)t.nVoxPad * KF * sizeof(float) + 255) / 256 * 256;
    const size_t kdB = ((size_t)t.nSamPad * KF * sizeof(float) + 255) / 256 * 256;
    b.bytesD = bfB + kdB + KF * KF * sizeof(float);
    cudaError_t e = cudaMalloc(&b.memD, b.bytesD);
    if (e != cudaSuccess) { b.memD = nullptr; return e; }
    b.bfT = (float *)b.memD;
    b.kd1 = (float *)((unsigned char *)b.memD + bfB);
    b.Md = (float *)((unsigned char *)b.memD + bfB + kdB);
    h->bytes += (int64_t)b.bytesD;
    // voxel side of the reduced basis: fixed for the operator
    e = tc_deriv_basis(h, b.bfT, b.Md, &b.rankD, &b.kfD);
    if (e == cudaSuccess && tc_configure_deriv(t.KP, b.N, b.kfD) < 1) e = cudaErrorInvalidConfiguration;
    if (e == cudaSuccess) {
      b.fusedD = true;
    } else {
      cudaFree(b.memD);
      h->bytes -= (int64_t)b.bytesD;
      b.memD = nullptr;
      b.bfT = b.kd1 = b.Md = nullptr;
    }
    return e;
  }
  const int bps = configure_kernel<1>(t.KP, ND);
  if (bps < 1) return cudaErrorInvalidConfiguration;
  b.gridD = (int)std::min<int64_t>((int64_t)h->numSMs * bps, (int64_t)t.nSt * chunks);
  b.slotsD = max_slots(t.nSt, chunks, b.gridD);
  const size_t bopB = (size_t)chunks * 2 * ND * TK * 2, partB = (size_t)b.slotsD * t.nSamPad * 64 * sizeof(float2);
  b.bytesD = (bopB + 255) / 256 * 256 + partB;
  cudaError_t e = cudaMalloc(&b.memD, b.bytesD);
  if (e != cudaSuccess) { b.memD = nullptr; return e; }
  b.bopD = (uint16_t *)b.memD;
  b.partD = (float2 *)((unsigned char *)b.memD + (bopB + 255) / 256 * 256);
  h->bytes += (int64_t)b.bytesD;
  return cudaSuccess;
}

cudaError_t tc_derivative(hoe_handle *h, const float2 *x, float2 *y, cudaStream_t st) {
  cudaError_t e = tc_derivative_prepare(h);
  if (e != cudaSuccess) return e;
  const TcBuffers &b = *(const TcBuffers *)h->tc_host;
  const auto &t = h->t;
  if (b.fusedD) {
    // the reduced 2 pi kdot from the current kspha_dt (hoe_set_kspha may replace it)
    e = tc_deriv_kdot(h, b.Md, b.kd1, st);
    if (e == cudaSuccess) e = bop_forward(h, b, x, st);
    if (e == cudaSuccess) {
      TcParams<1> p = single_params(h, b, slice_forward(h, b));
      p.bfT = b.bfT;
      p.kd1 = b.kd1;
      trace(h, EV_FK0, st);
      e = tc_launch_deriv(h, p, t.KP, b.N, b.kfD, b.gridF, st);
      trace(h, EV_FK1, st);
    }
    if (e == cudaSuccess) e = reduce_forward(h, b, single_map_forward(h, b), y, nullptr, false, st);
    return e;
  }
  const int chunks = t.nVoxPad / TV;
  constexpr int ND = 128;
  const int CP = t.nCha, TP = 64 / CP, passes = (t.nTerm + TP - 1) / TP;
  TcSlice sl = slice_forward(h, b);
  sl.Bop = b.bopD;
  sl.part = b.partD;
  TcParams<1> p = single_params(h, b, sl);
  p.nChaPad = 64;   // the slots' row stride: 64 virtual coils
  p.nChaTC = 64;
  const SlotMap m = slot_map(0, chunks, (int64_t)t.nSt * chunks, b.gridD);
  const float scale2pi = (float)(2.0 * 3.14159265358979323846 / sqrt((double)t.nVox));
  const int64_t nU = (int64_t)chunks * ND * (TK / 8), nR = (int64_t)t.nSamPad * CP;
  for (int q = 0; q < passes && e == cudaSuccess; ++q) {
    const int l0 = q * TP;
    e = launch_pdl(k_tc_bop_deriv, dim3((unsigned)((nU + 255) / 256)), dim3(256), 0, st, x, (const int *)t.perm,
                   (const float2 *)t.csm, (const float *)t.bfraw, b.bopD, chunks, t.nChaPad, t.nCha, CP, TP,
                   l0, t.nTerm);
    if (e == cudaSuccess) e = launch(h, p, t.KP, ND, b.gridD, st);
    if (e == cudaSuccess)
      e = launch_pdl(k_tc_deriv_reduce, dim3((unsigned)((nR + 255) / 256)), dim3(256), 0, st,
                     (const float2 *)b.partD, t.nSamPad, t.nSam, t.nCha, CP, l0, TP, t.nTerm,
                     (const float *)t.kdot, scale2pi, m, y, q > 0 ? 1 : 0);
    h->launches += 2;
  }
  return e;
}

void *tc_batch_plan(hoe_handle *const *hs, int n, std::string *why) {
  auto *P = new TcBatchPlan();
  P->hs.assign(hs, hs + n);
  P->slotsF.assign(n, 1);
  P->slotsA.assign(n, 1);
  P->mapF.assign(n, SlotMap{});
  P->mapA.assign(n, SlotMap{});
  const TcBuffers &b0 = *(const TcBuffers *)hs[0]->tc_host;
  // group by KP, in input order, at most kBatchSlices per launch
  for (int KP : {8, 16, 24}) {
    TcBatchPlan::Group g;
    for (int i = 0; i < n; ++i) {
      if (hs[i]->t.KP != KP) continue;
      g.idx.push_back(i);
      if ((int)g.idx.size() == kBatchSlices) { g.KP = KP; P->groups.push_back(g); g = TcBatchPlan::Group(); }
    }
    if (!g.idx.empty()) { g.KP = KP; P->groups.push_back(g); }
  }
  for (auto &g : P->groups) {
    const int bps = configure_kernel<kBatchSlices>(g.KP, b0.N);
    if (bps < 1) { if (why) *why = "batched kernel configuration"; delete P; return nullptr; }
    for (int dir = 0; dir < 2; ++dir) {
      TcParams<kBatchSlices> &p = dir == 0 ? g.pF : g.pA;
      p = TcParams<kBatchSlices>{};
      p.nSlices = (int)g.idx.size();
      p.nChaPad = hs[g.idx[0]]->t.nChaPad;
      p.nChaTC = b0.nChaTC;
      int64_t W = 0;
      for (int k = 0; k < p.nSlices; ++k) {
        const hoe_handle *h = hs[g.idx[k]];
        const TcBuffers &b = *(const TcBuffers *)h->tc_host;
        p.s[k] = dir == 0 ? slice_forward(h, b) : slice_adjoint(h, b);
        p.s[k].first = W;
        W += (int64_t)p.s[k].nRowTiles * p.s[k].nColChunks;
      }
      p.work = W;
      const int G = (int)std::min<int64_t>((int64_t)hs[g.idx[0]]->numSMs * bps, W);
      (dir == 0 ? g.G_F : g.G_A) = G;
      for (int k = 0; k < p.nSlices; ++k) {
        const int i = g.idx[k];
        const hoe_handle *h = hs[i];
        const TcBuffers &b = *(const TcBuffers *)h->tc_host;
        (dir == 0 ? P->mapF : P->mapA)[i] = slot_map(p.s[k].first, p.s[k].nColChunks, W, G);
        const int J = slots_needed(p.s[k].first, p.s[k].nRowTiles, p.s[k].nColChunks, W, G);
        if ((size_t)J * p.s[k].nRowPad * h->t.nChaPad > b.partElems) {
          if (why) *why = "partial-sum buffer of a slice too small for the batched schedule";
          delete P;
          return nullptr;
        }
        (dir == 0 ? P->slotsF : P->slotsA)[i] = J;
      }
    }
  }
  if (cudaMalloc(&P->err, sizeof(int)) != cudaSuccess || cudaMemset(P->err, 0, sizeof(int)) != cudaSuccess) {
    if (P->err) cudaFree(P->err);
    if (why) *why = "device allocation";
    delete P;
    return nullptr;
  }
  for (auto &g : P->groups) { g.pF.err = P->err; g.pA.err = P->err; }
  return P;
}

void tc_batch_plan_free(void *plan) {
  auto *P = (TcBatchPlan *)plan;
  if (!P) return;
  if (P->err) cudaFree(P->err);
  delete P;
}

int *tc_batch_error_word(void *plan) { return plan ? ((TcBatchPlan *)plan)->err : nullptr; }

namespace {

cudaError_t batch_contract(TcBatchPlan *P, bool forward, cudaStream_t st) {
  cudaError_t e = cudaSuccess;
  for (size_t k = 0; k < P->groups.size() && e == cudaSuccess; ++k) {
    const auto &g = P->groups[k];
    const hoe_handle *h0 = P->hs[g.idx[0]];
    e = launch(h0, forward ? g.pF : g.pA, g.KP, ((const TcBuffers *)h0->tc_host)->N, forward ? g.G_F : g.G_A, st);
  }
  return e;
}

const TcBuffers &buffers(const hoe_handle *h) { return *(const TcBuffers *)h->tc_host; }

}  // namespace

cudaError_t tc_batch_forward(void *plan, const float2 *const *x, float2 *const *y, cudaStream_t st) {
  auto *P = (TcBatchPlan *)plan;
  const int n = (int)P->hs.size();
  cudaError_t e = cudaSuccess;
  for (int i = 0; i < n && e == cudaSuccess; ++i) e = bop_forward(P->hs[i], buffers(P->hs[i]), x[i], st);
  if (e == cudaSuccess) e = batch_contract(P, true, st);
  for (int i = 0; i < n && e == cudaSuccess; ++i)
    e = reduce_forward(P->hs[i], buffers(P->hs[i]), P->mapF[i], y[i], nullptr, false, st);
  return e;
}

cudaError_t tc_batch_adjoint(void *plan, const float2 *const *y, const float *const *D, float2 *const *x,
                             cudaStream_t st) {
  auto *P = (TcBatchPlan *)plan;
  const int n = (int)P->hs.size();
  cudaError_t e = cudaSuccess;
  for (int i = 0; i < n && e == cudaSuccess; ++i)
    e = bop_adjoint(P->hs[i], buffers(P->hs[i]), y[i], D ? D[i] : nullptr, st);
  if (e == cudaSuccess) e = batch_contract(P, false, st);
  for (int i = 0; i < n && e == cudaSuccess; ++i) e = reduce_adjoint(P->hs[i], buffers(P->hs[i]), P->mapA[i], x[i], st);
  return e;
}

cudaError_t tc_batch_normal(void *plan, const float *const *D, const float2 *const *x, float2 *const *out,
                            cudaStream_t st) {
  auto *P = (TcBatchPlan *)plan;
  const int n = (int)P->hs.size();
  cudaError_t e = cudaSuccess;
  for (int i = 0; i < n && e == cudaSuccess; ++i) e = bop_forward(P->hs[i], buffers(P->hs[i]), x[i], st);
  if (e == cudaSuccess) e = batch_contract(P, true, st);
  for (int i = 0; i < n && e == cudaSuccess; ++i)
    e = reduce_forward(P->hs[i], buffers(P->hs[i]), P->mapF[i], nullptr, D ? D[i] : nullptr, true, st);
  if (e == cudaSuccess) e = batch_contract(P, false, st);
  for (int i = 0; i < n && e == cudaSuccess; ++i)
    e = reduce_adjoint(P->hs[i], buffers(P->hs[i]), P->mapA[i], out[i], st);
  return e;
}

int tc_batch_launches(void *plan) { return plan ? (int)((TcBatchPlan *)plan)->groups.size() : 0; }

cudaError_t tc_anchor_tables(const hoe_handle *h, cudaStream_t st) {
  if (!h->tc.ready) return cudaSuccess;
  const auto &t = h->t;
  const TcBuffers &b = *(const TcBuffers *)h->tc_host;
  const int64_t nAP = (int64_t)t.nVt * t.nSamPad, nBQ = (int64_t)t.nSt * t.nVoxPad;
  k_tc_anchor_tf32<<<(unsigned)((nAP + 255) / 256), 256, 0, st>>>(t.Atab, nAP, (float2 *)b.AtabP);
  k_tc_anchor_tf32<<<(unsigned)((nBQ + 255) / 256), 256, 0, st>>>(t.Btab, nBQ, (float2 *)b.BtabQ);
  h->launches += 2;
  return cudaGetLastError();
}

int *tc_error_word(const hoe_handle *h) {
  return h->tc_host ? ((const TcBuffers *)h->tc_host)->err : nullptr;
}

}  // namespace hoe
