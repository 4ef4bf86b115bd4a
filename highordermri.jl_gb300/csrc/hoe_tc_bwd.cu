// hoe_tc_bwd.cu — the backward pass of the explicit operator on the tensor
// cores.  With r = E x - y and L = 0.5 ||r||^2 (the same gradient as the
// FP32 kernel k_bwd_simt in hoe_simt.cu):
//
//   W[s,v] = sum_c conj(r[s,c]) Z[v,c],  Z = x * csm (masked voxel order)
//   G[s,v] = -(2 pi / sqrt(nVox)) Im(e^{i phi[s,v]} W[s,v])
//   dL/dkspha[l,s] = sum_v G[s,v] bf[v,l],   g1[v] = sum_s G[s,v],   gt[v] = sum_s G[s,v] t_s
//
// (dL/dfieldmap = gt, dL/dt0 = -sum_v fieldmap[v] g1[v] - sum_{l,s} kdot[l,s] dk[l,s].)
//
// One persistent CTA per SM walks (sample tile of 128 rows, voxel chunk of 64)
// work items in the forward engine's order.  Per stage:
//   * the residual-phase issuer forms phi in radians on the tensor cores, as
//     in the forward engine (TF32 residual products and the anchor k-step);
//   * the W issuer forms W with split-BF16 MMAs, A = [Re r, Im r] per coil
//     (one tile per row tile) and B = Z arranged so that the 128 output
//     columns are (Re W, Im W) per voxel, both from shared memory;
//   * 16 phase warps (two groups on alternate stages) read phi and W from
//     tensor memory, form G, write it as BF16 hi/lo into a shared-memory A
//     tile and sum G and G t over their 32 rows with warp MMAs (mma.sync
//     m16n8k16: A = rows of ones, t_hi and t_lo; B = their part of the G tile
//     read back transposed by ldmatrix); the four row quarters of a tile
//     store separate partial sums, which k_bwd_vox adds in a fixed order (no
//     wait between warps);
//   * the dk issuer contracts G with the basis tile: hi x [bf_hi | bf_lo] as
//     one 64-wide MMA and lo x bf_hi, into one accumulator set that the phase
//     warps add into FP32 registers every 32 stages.
// The stage ring (Z tiles, residual column tiles, anchors) is released as
// soon as the W and residual-phase MMAs have read it; the basis tiles, read
// two or three stages later by the dk MMAs, have a ring of their own that the
// dk issuer fills itself, NF - 1 stages ahead.
// Every mbarrier wait is bounded as in hoe_tc.cu: on timeout the kernel sets
// the engine's error word, stops, drains its own copies and MMAs and frees
// tensor memory.
#include "hoe_tcgen05.cuh"

#include <algorithm>
#include <cmath>

namespace hoe {
namespace {

// Warp roles: 16 phase warps, W issuer, residual-phase issuer (TMEM owner),
// dk issuer, loader.
constexpr int BW_WISS = PHASE_WARPS;
constexpr int BW_PISS = PHASE_WARPS + 1;
constexpr int BW_KISS = PHASE_WARPS + 2;
constexpr int BW_LOAD = PHASE_WARPS + 3;
constexpr int BW_THREADS = (PHASE_WARPS + 4) * 32;
constexpr int BW_GROUP = 32;   // stages per dk accumulator flush
constexpr int BW_NF = 32;      // basis columns per tile (kRF = 24 used, zero padded)
static_assert(kRF <= BW_NF, "basis tile width");

// byte offset of element (r, k) in a no-swizzle K-major BF16 tile with K = KK
__host__ __device__ constexpr uint32_t kmaj(int r, int k, int KK) {
  return (uint32_t)((r / 8) * (KK / 8) * 128 + (k / 8) * 128 + (r % 8) * 16 + (k % 8) * 2);
}

// Tensor memory (512 columns): residual phase 2 x 64 FP32, W 2 x 128 FP32,
// dk accumulators [hi.bf_hi | hi.bf_lo] 64 + lo.bf_hi 32.
constexpr uint32_t BW_P_COL = 0;
constexpr uint32_t BW_W_COL = 2 * TV;
constexpr uint32_t BW_ACC_COL = BW_W_COL + 2 * 2 * TV;
static_assert(BW_ACC_COL + 3 * BW_NF <= 512, "tensor memory plan");

// Shared memory (dynamic, 1024-byte aligned base), KC = 2 * coils (BF16 K of
// the W product), KP = residual width:
//   stage ring [NS]: ZB [hi|lo] 128 x KC, CV [hi|lo] 64 x KP (TF32),
//                    XR [data|0] 128 x 4, XC [data|0] 64 x 4
//   basis ring [NF]: FB [hi|lo] 32 x 64 (NF = 4; 2 at KC = 64, 32 coils)
//   row-tile tables: RV [hi|lo] 128 x KP (TF32), RA [hi|lo] 128 x KC
//   G tiles [2 parities]: [hi|lo] 128 x 64
constexpr int BW_NFB = 4;
template <int KC, int KP, int NS>
struct BwSmem {
  static constexpr int NF = KC > 32 ? 2 : BW_NFB;
  static constexpr int ZB = 128 * KC * 2, FB = BW_NF * TV * 2, CV = TV * KP * 4;
  static constexpr int XR = TM * 4 * 4, XC = TV * 4 * 4;
  static constexpr int RV = TM * KP * 4, RA = TM * KC * 2, GT = TM * TV * 2;
  static constexpr size_t ZB_OFF = 0;
  static constexpr size_t CV_OFF = ZB_OFF + (size_t)NS * 2 * ZB;
  static constexpr size_t XR_OFF = CV_OFF + (size_t)NS * 2 * CV;
  static constexpr size_t XC_OFF = XR_OFF + (size_t)NS * 2 * XR;
  static constexpr size_t FB_OFF = XC_OFF + (size_t)NS * 2 * XC;
  static constexpr size_t RV_OFF = FB_OFF + (size_t)NF * 2 * FB;
  static constexpr size_t RA_OFF = RV_OFF + (size_t)2 * RV;
  static constexpr size_t G_OFF = RA_OFF + (size_t)2 * RA;
  static constexpr size_t BAR_OFF = G_OFF + (size_t)2 * 2 * GT;
  static constexpr int NBAR = 2 * NS + 2 * NF + 16;
  static constexpr size_t MISC_OFF = BAR_OFF + (size_t)NBAR * 8;
  static constexpr size_t BYTES = MISC_OFF + 16 + 1024;
};

template <int KC, int KP>
constexpr int bw_stages() {
  return BwSmem<KC, KP, 4>::BYTES <= 227 * 1024 ? 4 : BwSmem<KC, KP, 3>::BYTES <= 227 * 1024 ? 3 : 2;
}

struct BwParams {
  const float *kpHi, *kpLo, *dbHi, *dbLo;   // TF32 residual tables (row side: samples)
  const float *AtabP, *BtabQ;               // anchor tables (TF32 [hi, lo] pairs)
  const uint16_t *ra;                       // [nSt][hi,lo][128 x KC] A of the W product
  const uint16_t *zb;                       // [nChunks][hi,lo][128 x KC] B of the W product
  const uint16_t *fb;                       // [nChunks][hi,lo][32 x 64] basis tiles
  const float *times;                       // [nSamPad]
  float *dkpart;                            // [slots][nSamPad][kRF]
  float *g1part, *gtpart;                   // [nSt * 4 row quarters][nVoxPad]
  int *err;
  int nSt, nChunks, nSamPad, nVoxPad;
  float scaleG;
};

template <int KC, int KP, int NS>
__global__ void __launch_bounds__(BW_THREADS, 1) k_tc_backward(const __grid_constant__ BwParams p) {
  using S = BwSmem<KC, KP, NS>;
  extern __shared__ unsigned char smem_raw[];
  unsigned char *smem = align_smem_1024(smem_raw);
  constexpr int NF = S::NF;
  uint64_t *full = reinterpret_cast<uint64_t *>(smem + S::BAR_OFF);
  uint64_t *empty = full + NS;        // [NS] stage read by the W and residual-phase MMAs
  uint64_t *ffull = empty + NS;       // [NF] basis tile loaded
  uint64_t *fempty = ffull + NF;      // [NF] basis tile read by the dk MMAs
  uint64_t *rfull = fempty + NF;      // [1] row-tile tables loaded
  uint64_t *rfree = rfull + 1;        // [1] row-tile tables no longer read (residual and W issuers)
  uint64_t *pfull = rfree + 1;        // [2] residual phase of the stage in TMEM
  uint64_t *pfree = pfull + 2;        // [2] ... read by the phase warps
  uint64_t *wfull = pfree + 2;        // [2] W of the stage in TMEM
  uint64_t *wfree = wfull + 2;        // [2] ... read by the phase warps
  uint64_t *gfull = wfree + 2;        // [2] G tile written (8 phase warps)
  uint64_t *gfree = gfull + 2;        // [2] G tile read by the dk MMAs
  uint64_t *segdone = gfree + 2;      // [1] dk accumulators complete for a group
  uint64_t *tmemfree = segdone + 1;   // [1] dk accumulators read out
  uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(smem + S::MISC_OFF);
  volatile int *abort = reinterpret_cast<volatile int *>(smem + S::MISC_OFF + 8);
  constexpr uint32_t SBO_TF32 = (KP / 4) * 128, SBO_KC = (KC / 8) * 128, SBO_64 = (TV / 8) * 128;

  const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
  const int G = gridDim.x, b = blockIdx.x;
  const int64_t W = (int64_t)p.nSt * p.nChunks;
  const int64_t wb = (int64_t)b * W / G, we = (int64_t)(b + 1) * W / G;
  const int nIter = (int)(we - wb);
  const int rt0 = (int)(wb / p.nChunks), ch0 = (int)(wb % p.nChunks);

  if (threadIdx.x == 0) {
    for (int i = 0; i < NS; ++i) {
      mbar_init(&full[i], 1);
      mbar_init(&empty[i], 2);
    }
    for (int i = 0; i < NF; ++i) {
      mbar_init(&ffull[i], 1);
      mbar_init(&fempty[i], 1);
    }
    mbar_init(&rfull[0], 1);
    mbar_init(&rfree[0], 2);
    for (int i = 0; i < 2; ++i) {
      mbar_init(&pfull[i], 1);
      mbar_init(&pfree[i], GROUP_WARPS);
      mbar_init(&wfull[i], 1);
      mbar_init(&wfree[i], GROUP_WARPS);
      mbar_init(&gfull[i], GROUP_WARPS);
      mbar_init(&gfree[i], 1);
    }
    mbar_init(&segdone[0], 1);
    mbar_init(&tmemfree[0], PHASE_WARPS);
    *abort = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  // anchor k-step operands, per stage slot: row side [a_hi, a_lo, 1, 1 | 0],
  // column side [1, 1, c_hi, c_lo | 0]; the constant halves and the zero
  // core-matrix columns once, the [hi, lo] halves by the loader per stage
  for (int i = threadIdx.x; i < NS * (S::XR + S::XC) / 16; i += BW_THREADS) {
    const int nr = NS * S::XR / 16;
    const bool isRow = i < nr;
    const int slot = isRow ? i / (S::XR / 16) : (i - nr) / (S::XC / 16);
    const int e = isRow ? i % (S::XR / 16) : (i - nr) % (S::XC / 16);
    float4 *base = isRow ? reinterpret_cast<float4 *>(smem + S::XR_OFF + (size_t)slot * 2 * S::XR)
                         : reinterpret_cast<float4 *>(smem + S::XC_OFF + (size_t)slot * 2 * S::XC);
    base[e] = isRow ? make_float4(0.f, 0.f, 1.f, 1.f) : make_float4(1.f, 1.f, 0.f, 0.f);
    base[(isRow ? S::XR : S::XC) / 16 + e] = make_float4(0.f, 0.f, 0.f, 0.f);
  }
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  if (warp == BW_PISS) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                 "r"(512));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;
  // the prologue above touches no global memory; the W operands and the dk
  // slots are written by the kernels before this one in the stream
  pdl_wait();
  pdl_trigger();

  if (warp < PHASE_WARPS) {
    // ---------------- phase warps: rows (warp & 3)*32 + lane, stage columns
    // [half*32, half*32+32) of every other stage (par = warp >> 3)
    const int q = warp & 3, half = (warp >> 2) & 1, par = warp >> 3, qcol = warp >> 2;
    const int row = q * 32 + lane;
    const uint32_t laneBase = (uint32_t)(q * 32) << 16;
    float dkacc[8];
#pragma unroll
    for (int i = 0; i < 8; ++i) dkacc[i] = 0.f;
    int grp = -1, pendGrp = -1, pendRT = -1, pendIt = 0;
    bool pendLast = false, ok = true;
    auto flush = [&]() {
      const int g = pendGrp;
      const bool got = ok && wait_bar(&segdone[0], g & 1, abort, p.err);
      tc_fence_after();
      if (got) {
#pragma unroll
        for (int part = 0; part < 3; ++part) {
          float v[8];
          tmem_ld8(tmem + laneBase + BW_ACC_COL + (uint32_t)(part * BW_NF + qcol * 8), v);
#pragma unroll
          for (int i = 0; i < 8; ++i) dkacc[i] += v[i];
        }
      }
      tc_fence_before();
      __syncwarp();
      if (lane == 0) mbar_arrive(&tmemfree[0]);
      if (pendLast) {
        if (ok && qcol * 8 < kRF) {
          const int slot = b - work_owner((int64_t)pendRT * p.nChunks, W, G);
          float *dst = p.dkpart + ((int64_t)slot * p.nSamPad + (int64_t)pendRT * TM + row) * kRF + qcol * 8;
#pragma unroll
          for (int i = 0; i < 8; ++i)
            if (qcol * 8 + i < kRF) dst[i] = dkacc[i];
        }
#pragma unroll
        for (int i = 0; i < 8; ++i) dkacc[i] = 0.f;
      }
      pendGrp = -1;
    };
    int rt = rt0, ch = ch0;
    // A fragments of the column-sum MMAs (mma.sync m16n8k16, rows = the
    // fragment's groupID lane / 4): row 0 ones, row 1 t_hi(s), row 9 t_lo(s)
    // for the warp's samples s of each 16-sample half kk, so that lanes 0-3
    // end with sum_s G and lanes 4-7 with the hi and lo parts of sum_s G t
    uint32_t ta[2][4];
    const int g4 = lane >> 2, t4 = lane & 3;
    for (int it = 0; it < nIter && ok; ++it) {
      if (it > 0 && ++ch == p.nChunks) { ch = 0; ++rt; }
      if (it == 0 || ch == 0) {
#pragma unroll
        for (int kk = 0; kk < 2; ++kk) {
#pragma unroll
          for (int h8 = 0; h8 < 2; ++h8) {   // k columns 2 t4 + {0, 1} (+ 8 h8)
            const int s0 = q * 32 + kk * 16 + h8 * 8 + 2 * t4;
            uint32_t hi = 0u, lo = 0u;
            if (g4 == 0) {
              hi = 0x3f803f80u;   // (1, 1) in BF16
            } else if (g4 == 1) {
              const float a = p.times[(int64_t)rt * TM + s0], c = p.times[(int64_t)rt * TM + s0 + 1];
              const __nv_bfloat162 th = __floats2bfloat162_rn(a, c);
              const __nv_bfloat162 tl = __floats2bfloat162_rn(a - __low2float(th), c - __high2float(th));
              hi = *reinterpret_cast<const uint32_t *>(&th);
              lo = *reinterpret_cast<const uint32_t *>(&tl);
            }
            ta[kk][2 * h8] = hi;       // rows groupID (0: ones, 1: t_hi)
            ta[kk][2 * h8 + 1] = lo;   // rows groupID + 8 (9: t_lo)
          }
        }
      }
      if (it == 0 || ch % BW_GROUP == 0) ++grp;
      if ((it & 1) == par) {
        const int pb = it & 1, pr = (it >> 1) & 1;
        if (!wait_bar(&pfull[pb], pr, abort, p.err) || !wait_bar(&wfull[pb], pr, abort, p.err)) { ok = false; break; }
        tc_fence_after();
        const uint32_t pBase = tmem + laneBase + BW_P_COL + (uint32_t)(pb * TV + half * 32);
        const uint32_t wBase = tmem + laneBase + BW_W_COL + (uint32_t)(pb * 2 * TV + half * 64);
        float g[32];
#pragma unroll
        for (int j0 = 0; j0 < 32; j0 += 16) {
          // 16 voxels: their phases and (Re W, Im W), three loads and one wait
          uint32_t d[16], w[32];
          tmem_ld16_async(pBase + j0, d);
          tmem_ld16_async(wBase + 2 * j0, w);
          tmem_ld16_async(wBase + 2 * j0 + 16, w + 16);
          tmem_wait_ld(d, w);
#pragma unroll
          for (int j = 0; j < 16; ++j) {
            float sn, cs;
            __sincosf(__uint_as_float(d[j]), &sn, &cs);
            g[j0 + j] = -p.scaleG * (cs * __uint_as_float(w[2 * j + 1]) + sn * __uint_as_float(w[2 * j]));
          }
        }
        tc_fence_before();
        __syncwarp();
        if (lane == 0) {
          mbar_arrive(&pfree[pb]);
          mbar_arrive(&wfree[pb]);
        }
        // G as BF16 hi/lo into the A tile of parity pb, once the dk MMAs of
        // stage it-2 have read it
        if (it >= 2 && !wait_bar(&gfree[pb], ((it >> 1) - 1) & 1, abort, p.err)) { ok = false; break; }
        unsigned char *gHi = smem + S::G_OFF + (size_t)pb * 2 * S::GT;
#pragma unroll
        for (int c8 = 0; c8 < 4; ++c8) {
          uint32_t hw[4], lw[4];
#pragma unroll
          for (int i = 0; i < 4; ++i)
            split_bf16x2(g[c8 * 8 + 2 * i], g[c8 * 8 + 2 * i + 1], hw[i], lw[i]);
          const uint32_t off = kmaj(row, half * 32 + c8 * 8, TV);
          *reinterpret_cast<uint4 *>(gHi + off) = make_uint4(hw[0], hw[1], hw[2], hw[3]);
          *reinterpret_cast<uint4 *>(gHi + S::GT + off) = make_uint4(lw[0], lw[1], lw[2], lw[3]);
        }
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        __syncwarp();
        if (lane == 0) mbar_arrive(&gfull[pb]);
        // column sums of G and G t over the warp's 32 rows on the tensor cores:
        // D[m, v] = sum_s A[m, s] G[s, v] from the G tile just written (BF16
        // hi and lo, read back transposed by ldmatrix), FP32 accumulation
        float acc[4][4];
#pragma unroll
        for (int n = 0; n < 4; ++n)
#pragma unroll
          for (int i = 0; i < 4; ++i) acc[n][i] = 0.f;
#pragma unroll
        for (int kk = 0; kk < 2; ++kk) {
#pragma unroll
          for (int np = 0; np < 2; ++np) {
            // lane L gives row L % 8 of core matrix L / 8: samples of group
            // (L / 8) & 1 of this half, voxels of group L / 16 of this pair
            const int sl = q * 32 + kk * 16 + ((lane >> 3) & 1) * 8 + (lane & 7);
            const int vl = half * 32 + np * 16 + (lane >> 4) * 8;
            const uint32_t off = kmaj(sl, vl, TV);
            uint32_t h0, h1, h2, h3, l0, l1, l2, l3;
            ldmatrix_x4_trans(smem_u32(gHi + off), h0, h1, h2, h3);
            ldmatrix_x4_trans(smem_u32(gHi + S::GT + off), l0, l1, l2, l3);
            mma_bf16_16816(acc[2 * np], ta[kk], h0, h1);
            mma_bf16_16816(acc[2 * np], ta[kk], l0, l1);
            mma_bf16_16816(acc[2 * np + 1], ta[kk], h2, h3);
            mma_bf16_16816(acc[2 * np + 1], ta[kk], l2, l3);
          }
        }
        // lanes 0-3: sum_s G (row 0); lanes 4-7: sum_s G t (rows 1 + 9), for
        // the columns n*8 + 2 t4 + {0, 1} of the warp's 32
        if (g4 < 2) {
          float *dst = (g4 == 0 ? p.g1part : p.gtpart) + ((int64_t)rt * 4 + q) * p.nVoxPad + (int64_t)ch * TV +
                       half * 32 + 2 * t4;
#pragma unroll
          for (int n = 0; n < 4; ++n)
            *reinterpret_cast<float2 *>(dst + n * 8) =
                g4 == 0 ? make_float2(acc[n][0], acc[n][1])
                        : make_float2(acc[n][0] + acc[n][2], acc[n][1] + acc[n][3]);
        }
      }
      if (pendGrp >= 0 && it >= pendIt + 1) flush();
      const bool endRT = (it == nIter - 1) || (ch + 1 == p.nChunks);
      if (endRT || (ch + 1) % BW_GROUP == 0) {
        if (pendGrp >= 0) flush();
        pendGrp = grp;
        pendRT = rt;
        pendLast = endRT;
        pendIt = it;
      }
    }
    if (pendGrp >= 0) flush();
  } else if (warp == BW_WISS) {
    // ---------------- W issuer: W = [Re r, Im r] x Z^T (3 BF16 products)
    if (lane == 0 && nIter > 0) {
      constexpr uint32_t idescW = idesc_bf16(TM, 2 * TV);
      uint64_t *lastBar = nullptr;
      uint32_t lastPar = 0;
      int kj = -1, ch = ch0;
      for (int it = 0; it < nIter; ++it) {
        if (it > 0 && ++ch == p.nChunks) ch = 0;
        if (it == 0 || ch == 0) {
          ++kj;
          if (!wait_bar(&rfull[0], kj & 1, abort, p.err)) break;
        }
        const bool lastOfRow = (it == nIter - 1) || (ch + 1 == p.nChunks);
        const int slot = it % NS, pb = it & 1;
        if (!wait_bar(&full[slot], (it / NS) & 1, abort, p.err)) break;
        if (it >= 2 && !wait_bar(&wfree[pb], ((it >> 1) - 1) & 1, abort, p.err)) break;
        tc_fence_after();
        const uint32_t dt = tmem + BW_W_COL + (uint32_t)(pb * 2 * TV);
        const uint32_t aHi = smem_u32(smem + S::RA_OFF), aLo = aHi + S::RA;
        const uint32_t bHi = smem_u32(smem + S::ZB_OFF + (size_t)slot * 2 * S::ZB), bLo = bHi + S::ZB;
#pragma unroll
        for (int ks = 0; ks < KC / 16; ++ks) {
          const uint32_t ko = ks * 2 * LBO;
          umma_ss(dt, umma_desc(aHi + ko, SBO_KC), umma_desc(bHi + ko, SBO_KC), idescW, ks ? 1u : 0u);
          umma_ss(dt, umma_desc(aHi + ko, SBO_KC), umma_desc(bLo + ko, SBO_KC), idescW, 1u);
          umma_ss(dt, umma_desc(aLo + ko, SBO_KC), umma_desc(bHi + ko, SBO_KC), idescW, 1u);
        }
        umma_commit(&wfull[pb]);
        umma_commit(&empty[slot]);
        lastBar = &wfull[pb];
        lastPar = (it >> 1) & 1;
        if (lastOfRow) umma_commit(&rfree[0]);
      }
      if (*abort && lastBar) drain_bar(lastBar, lastPar);
    }
    __syncwarp();
  } else if (warp == BW_PISS) {
    // ---------------- residual-phase issuer (as in the forward engine)
    if (lane == 0 && nIter > 0) {
      constexpr uint32_t idescP = idesc_tf32(TM, TV);
      uint64_t *lastBar = nullptr;
      uint32_t lastPar = 0;
      int kj = -1, rt = rt0, ch = ch0;
      for (int it = 0; it < nIter; ++it) {
        if (it > 0 && ++ch == p.nChunks) { ch = 0; ++rt; }
        if (it == 0 || ch == 0) {
          ++kj;
          if (!wait_bar(&rfull[0], kj & 1, abort, p.err)) break;
        }
        const bool lastOfRow = (it == nIter - 1) || (ch + 1 == p.nChunks);
        const int s = it % NS, pb = it & 1;
        if (!wait_bar(&full[s], (it / NS) & 1, abort, p.err)) break;
        if (it >= 2 && !wait_bar(&pfree[pb], ((it >> 1) - 1) & 1, abort, p.err)) break;
        tc_fence_after();
        const uint32_t dt = tmem + BW_P_COL + (uint32_t)(pb * TV);
        const uint32_t rHi = smem_u32(smem + S::RV_OFF), rLo = rHi + S::RV;
        const uint32_t cHi = smem_u32(smem + S::CV_OFF + (size_t)s * 2 * S::CV), cLo = cHi + S::CV;
#pragma unroll
        for (int ks = 0; ks < KP / 8; ++ks) {
          const uint32_t ko = ks * 2 * LBO;
          umma_tf32(dt, umma_desc(rHi + ko, SBO_TF32), umma_desc(cHi + ko, SBO_TF32), idescP, ks ? 1u : 0u);
          umma_tf32(dt, umma_desc(rHi + ko, SBO_TF32), umma_desc(cLo + ko, SBO_TF32), idescP, 1u);
          umma_tf32(dt, umma_desc(rLo + ko, SBO_TF32), umma_desc(cHi + ko, SBO_TF32), idescP, 1u);
        }
        umma_tf32(dt, umma_desc(smem_u32(smem + S::XR_OFF + (size_t)s * 2 * S::XR), 128, S::XR),
                  umma_desc(smem_u32(smem + S::XC_OFF + (size_t)s * 2 * S::XC), 128, S::XC), idescP, 1u);
        umma_commit(&pfull[pb]);
        umma_commit(&empty[s]);
        lastBar = &pfull[pb];
        lastPar = (it >> 1) & 1;
        if (lastOfRow) umma_commit(&rfree[0]);
      }
      if (*abort && lastBar) drain_bar(lastBar, lastPar);
    }
    __syncwarp();
  } else if (warp == BW_KISS) {
    // ---------------- dk issuer: D0 += G_hi x [bf_hi | bf_lo], D1 += G_lo x bf_hi.
    // It also loads the basis tiles, NF - 1 stages ahead of its own MMAs.
    if (lane == 0 && nIter > 0) {
      constexpr uint32_t idescW = idesc_bf16(TM, 2 * BW_NF), idescN = idesc_bf16(TM, BW_NF);
      uint64_t *lastBar = nullptr;
      uint32_t lastPar = 0;
      int fIssued = 0, fch = ch0;   // basis tiles requested for stages [0, fIssued); chunk of stage fIssued
      auto load_fb = [&]() -> bool {
        // stage j into slot j % NF, last read by the dk MMAs of stage j - NF
        const int j = fIssued, fs = j % NF;
        if (j >= NF && !wait_bar(&fempty[fs], ((j - NF) / NF) & 1, abort, p.err)) return false;
        mbar_expect_tx(&ffull[fs], 2 * S::FB);
        bulk_g2s(smem + S::FB_OFF + (size_t)fs * 2 * S::FB, p.fb + (size_t)fch * 2 * BW_NF * TV, 2 * S::FB, &ffull[fs]);
        ++fIssued;
        if (++fch == p.nChunks) fch = 0;
        return true;
      };
      bool ok = true;
      while (ok && fIssued < NF - 1 && fIssued < nIter) ok = load_fb();
      int grp = -1, ch = ch0;
      for (int it = 0; it < nIter && ok; ++it) {
        if (it > 0 && ++ch == p.nChunks) ch = 0;
        const bool first = (it == 0) || (ch % BW_GROUP == 0);
        if (first) {
          ++grp;
          // the accumulators were last used by group grp-1: wait until read out
          if (grp >= 1 && !wait_bar(&tmemfree[0], (grp - 1) & 1, abort, p.err)) break;
        }
        const bool last = (it == nIter - 1) || (ch + 1 == p.nChunks) || ((ch + 1) % BW_GROUP == 0);
        const int fs = it % NF, pb = it & 1;
        if (!wait_bar(&ffull[fs], (it / NF) & 1, abort, p.err)) break;
        if (!wait_bar(&gfull[pb], (it >> 1) & 1, abort, p.err)) break;
        tc_fence_after();
        const uint32_t gHi = smem_u32(smem + S::G_OFF + (size_t)pb * 2 * S::GT), gLo = gHi + S::GT;
        const uint32_t fHi = smem_u32(smem + S::FB_OFF + (size_t)fs * 2 * S::FB);
#pragma unroll
        for (int ks = 0; ks < TV / 16; ++ks) {
          const uint32_t ko = ks * 2 * LBO;
          const uint32_t acc = (first && ks == 0) ? 0u : 1u;
          umma_ss(tmem + BW_ACC_COL, umma_desc(gHi + ko, SBO_64), umma_desc(fHi + ko, SBO_64), idescW, acc);
          umma_ss(tmem + BW_ACC_COL + 2 * BW_NF, umma_desc(gLo + ko, SBO_64), umma_desc(fHi + ko, SBO_64), idescN,
                  acc);
        }
        umma_commit(&gfree[pb]);
        umma_commit(&fempty[fs]);
        lastBar = &fempty[fs];
        lastPar = (it / NF) & 1;
        if (last) umma_commit(&segdone[0]);
        if (fIssued < nIter && !load_fb()) break;
      }
      if (*abort) {
        if (lastBar) drain_bar(lastBar, lastPar);   // MMAs done before TMEM is freed
        for (int j = max(0, fIssued - NF); j < fIssued; ++j) drain_bar(&ffull[j % NF], (j / NF) & 1);
      }
    }
    __syncwarp();
  } else if (warp == BW_LOAD) {
    // ---------------- loader: row-tile tables per row tile, stage operands
    // per stage (whole warp; the anchors are fetched one stage ahead by all
    // lanes as TF32 [hi, lo] pairs, the elected lane issues the bulk copies)
    {
      const bool leader = elect_one();
      const uint32_t stageBytes = 2 * S::ZB + 2 * S::CV;
      int issued = 0, kcount = -1, rowIssued = -1, rt = rt0, ch = ch0;
      float2 ar[TM / 32], ac[TV / 32];
      auto fetch = [&](int frt, int fch) {
        const float2 *rx = reinterpret_cast<const float2 *>(p.AtabP) + (int64_t)(fch * TV / 128) * p.nSamPad +
                           (int64_t)frt * TM;
        const float2 *cx = reinterpret_cast<const float2 *>(p.BtabQ) + (int64_t)frt * p.nVoxPad + (int64_t)fch * TV;
#pragma unroll
        for (int j = 0; j < TM / 32; ++j) ar[j] = __ldg(rx + lane + 32 * j);
#pragma unroll
        for (int j = 0; j < TV / 32; ++j) ac[j] = __ldg(cx + lane + 32 * j);
      };
      if (nIter > 0) fetch(rt, ch);
      for (int it = 0; it < nIter; ++it) {
        if (it > 0 && ++ch == p.nChunks) { ch = 0; ++rt; }
        if (it == 0 || ch == 0) {
          // one buffer: the previous row tile's W and residual MMAs must be done
          ++kcount;
          if (kcount >= 1 && !wait_bar_warp(&rfree[0], (kcount - 1) & 1, abort, p.err)) break;
          if (leader) {
            mbar_expect_tx(&rfull[0], 2 * S::RV + 2 * S::RA);
            const size_t ro = (size_t)rt * TM * KP;
            bulk_g2s(smem + S::RV_OFF, p.kpHi + ro, S::RV, &rfull[0]);
            bulk_g2s(smem + S::RV_OFF + S::RV, p.kpLo + ro, S::RV, &rfull[0]);
            bulk_g2s(smem + S::RA_OFF, p.ra + (size_t)rt * 2 * TM * KC, 2 * S::RA, &rfull[0]);
          }
          __syncwarp();
          rowIssued = kcount;
        }
        const int slot = it % NS, round = it / NS;
        if (round > 0 && !wait_bar_warp(&empty[slot], (round - 1) & 1, abort, p.err)) break;
        // anchors into the [hi, lo] halves of the slot's 16-byte rows, made
        // visible to the tensor cores before the stage barrier's arrival
        float2 *xr = reinterpret_cast<float2 *>(smem + S::XR_OFF + (size_t)slot * 2 * S::XR);
        float2 *xc = reinterpret_cast<float2 *>(smem + S::XC_OFF + (size_t)slot * 2 * S::XC);
#pragma unroll
        for (int j = 0; j < TM / 32; ++j) xr[2 * (lane + 32 * j)] = ar[j];
#pragma unroll
        for (int j = 0; j < TV / 32; ++j) xc[2 * (lane + 32 * j) + 1] = ac[j];
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        __syncwarp();
        if (leader) {
          mbar_expect_tx(&full[slot], stageBytes);
          bulk_g2s(smem + S::ZB_OFF + (size_t)slot * 2 * S::ZB, p.zb + (size_t)ch * 2 * TM * KC, 2 * S::ZB,
                   &full[slot]);
          const size_t co = (size_t)ch * TV * KP;
          unsigned char *cv = smem + S::CV_OFF + (size_t)slot * 2 * S::CV;
          bulk_g2s(cv, p.dbHi + co, S::CV, &full[slot]);
          bulk_g2s(cv + S::CV, p.dbLo + co, S::CV, &full[slot]);
        }
        __syncwarp();
        issued = it + 1;
        if (it + 1 < nIter) {
          int nrt = rt, nch = ch + 1;
          if (nch == p.nChunks) { nch = 0; ++nrt; }
          fetch(nrt, nch);
        }
      }
      if (*abort && leader) {
        for (int it = max(0, issued - NS); it < issued; ++it) drain_bar(&full[it % NS], (it / NS) & 1);
        if (rowIssued >= 0) drain_bar(&rfull[0], rowIssued & 1);
      }
    }
    __syncwarp();
  }

  tc_fence_before();
  __syncthreads();
  if (warp == BW_PISS) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(512));
  }
}

// One element of a BF16 hi/lo tile pair (lo tile `per` elements after hi).
__device__ __forceinline__ void store_split(uint16_t *tile, int64_t per, uint32_t byteOff, float val) {
  __nv_bfloat16 h = __float2bfloat16_rn(val);
  __nv_bfloat16 l = __float2bfloat16_rn(val - __bfloat162float(h));
  tile[byteOff / 2] = *reinterpret_cast<uint16_t *>(&h);
  tile[per + byteOff / 2] = *reinterpret_cast<uint16_t *>(&l);
}

// 16-byte unit u of a [TM x KK] K-major tile (kmaj): row n, k = 8*kg ..
// 8*kg+7; consecutive units are consecutive addresses.
__device__ __forceinline__ void bw_unit(int u, int KK, int &n, int &kg) {
  n = (u / (8 * (KK / 8))) * 8 + u % 8;
  kg = (u / 8) % (KK / 8);
}
// Eight values split into BF16 hi + lo, stored as one unit of the hi tile and
// one of the lo tile (per elements further on).
__device__ __forceinline__ void store_split8(uint16_t *tile, int64_t per, int u, const float *v) {
  uint32_t hw[4], lw[4];
#pragma unroll
  for (int j = 0; j < 4; ++j) split_bf16x2(v[2 * j], v[2 * j + 1], hw[j], lw[j]);
  reinterpret_cast<uint4 *>(tile)[u] = make_uint4(hw[0], hw[1], hw[2], hw[3]);
  reinterpret_cast<uint4 *>(tile + per)[u] = make_uint4(lw[0], lw[1], lw[2], lw[3]);
}

// A of the W product: sample tile st, row s, k = 2c + m: (Re r, Im r)[c].
// One thread per 16-byte unit (4 coils of one sample).  The threads also
// zero the dk partial slots (dkz, nz4 float4s) that the backward kernel
// accumulates into.
__global__ void k_bw_ra(const float2 *__restrict__ r, int nSam, int nCha, int nSamPad, int KC,
                        uint16_t *__restrict__ ra, float4 *__restrict__ dkz, int64_t nz4) {
  pdl_wait();
  pdl_trigger();
  const int units = TM * (KC / 8);
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  for (int64_t z = i; z < nz4; z += (int64_t)gridDim.x * blockDim.x) dkz[z] = make_float4(0.f, 0.f, 0.f, 0.f);
  if (i >= (int64_t)(nSamPad / TM) * units) return;
  const int st = (int)(i / units), u = (int)(i % units);
  int n, kg;
  bw_unit(u, KC, n, kg);
  const int s = st * TM + n;
  float v[8];
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    const int c = kg * 4 + j;
    const float2 z = (s < nSam && c < nCha) ? r[(int64_t)c * nSam + s] : make_float2(0.f, 0.f);
    v[2 * j] = z.x;
    v[2 * j + 1] = z.y;
  }
  const int64_t per = (int64_t)TM * KC;
  store_split8(ra + (size_t)st * 2 * per, per, u, v);
}

// B of the W product: chunk ch, row n = 2v + j (voxel v of the chunk), k = 2c + m:
//   j = 0 (Re W): (Re Z, Im Z);   j = 1 (Im W): (Im Z, -Re Z),  Z = x[perm[v]] csm[v, c]
// One thread per 16-byte unit (4 coils of one row).
__global__ void k_bw_zb(const float2 *__restrict__ x, const int *__restrict__ perm, const float2 *__restrict__ csm,
                        int nChunks, int nChaPad, int nCha, int KC, uint16_t *__restrict__ zb) {
  pdl_wait();
  pdl_trigger();
  const int units = TM * (KC / 8);
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (int64_t)nChunks * units) return;
  const int ch = (int)(i / units), u = (int)(i % units);
  int n, kg;
  bw_unit(u, KC, n, kg);
  const int vx = ch * TV + n / 2, jj = n & 1;
  const int g = perm[vx];
  const float2 xv = g >= 0 ? x[g] : make_float2(0.f, 0.f);
  float v[8];
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    const int c = kg * 4 + j;
    // csm rows exist for every tile-order voxel and padded coil (zeros)
    const float2 cv = c < nCha ? csm[(int64_t)vx * nChaPad + c] : make_float2(0.f, 0.f);
    const float2 z = make_float2(xv.x * cv.x - xv.y * cv.y, xv.x * cv.y + xv.y * cv.x);
    v[2 * j] = jj == 0 ? z.x : z.y;
    v[2 * j + 1] = jj == 0 ? z.y : -z.x;
  }
  const int64_t per = (int64_t)TM * KC;
  store_split8(zb + (size_t)ch * 2 * per, per, u, v);
}

// Basis tiles: chunk ch, row l (basis column, kRF used), k = voxel of the chunk.
__global__ void k_bw_fb(const float *__restrict__ bfraw, int nChunks, uint16_t *__restrict__ fb) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t per = (int64_t)BW_NF * TV;
  if (i >= (int64_t)nChunks * per) return;
  const int ch = (int)(i / per), e = (int)(i % per);
  const int l = e / TV, k = e % TV;
  const float v = l < kRF ? bfraw[((int64_t)ch * TV + k) * kRF + l] : 0.f;
  store_split(fb + (size_t)ch * 2 * per, per, kmaj(l, k, TV), v);
}

// Per-operator buffers of the tensor-core backward (allocated on first use).
struct BwBuffers {
  uint16_t *ra = nullptr, *zb = nullptr, *fb = nullptr;
  float *dkpart = nullptr, *g1 = nullptr, *gt = nullptr;
  double *vpart = nullptr, *dred = nullptr;
  void *mem = nullptr;
  size_t bytes = 0;
  int KC = 0, grid = 0, slots = 0;
};

template <int KC, int KP>
int bw_configure() {
  constexpr int NS = bw_stages<KC, KP>();
  using S = BwSmem<KC, KP, NS>;
  static_assert(S::BYTES <= 227 * 1024, "shared memory plan exceeds 227 KB");
  auto kern = k_tc_backward<KC, KP, NS>;
  if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)S::BYTES) != cudaSuccess)
    return 0;
  int nb = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, kern, BW_THREADS, S::BYTES) != cudaSuccess) return 0;
  return nb;
}

template <int KC, int KP>
cudaError_t bw_launch(const BwParams &p, int G, cudaStream_t st) {
  constexpr int NS = bw_stages<KC, KP>();
  static int nb = bw_configure<KC, KP>();
  if (nb < 1) return cudaErrorInvalidConfiguration;
  static_assert(BwSmem<KC, KP, NS>::BYTES <= 227 * 1024, "shared-memory plan");
  return launch_pdl(k_tc_backward<KC, KP, NS>, dim3(G), dim3(BW_THREADS), BwSmem<KC, KP, NS>::BYTES, st, p);
}

cudaError_t bw_dispatch(int KC, int KP, const BwParams &p, int G, cudaStream_t st) {
  if (KC == 16 && KP == 8) return bw_launch<16, 8>(p, G, st);
  if (KC == 16 && KP == 16) return bw_launch<16, 16>(p, G, st);
  if (KC == 32 && KP == 8) return bw_launch<32, 8>(p, G, st);
  if (KC == 32 && KP == 16) return bw_launch<32, 16>(p, G, st);
  if (KC == 16 && KP == 24) return bw_launch<16, 24>(p, G, st);
  if (KC == 32 && KP == 24) return bw_launch<32, 24>(p, G, st);
  if (KC == 64 && KP == 8) return bw_launch<64, 8>(p, G, st);
  if (KC == 64 && KP == 16) return bw_launch<64, 16>(p, G, st);
  return cudaErrorNotSupported;
}

cudaError_t bw_prepare(hoe_handle *h) {
  if (h->tcb_host) return cudaSuccess;
  const auto &t = h->t;
  BwBuffers b;
  b.KC = t.nCha <= 8 ? 16 : (t.nCha <= 16 ? 32 : 64);
  const int nChunks = t.nVoxPad / TV;
  b.grid = std::min<int64_t>(h->numSMs, (int64_t)t.nSt * nChunks);
  b.slots = max_slots(t.nSt, nChunks, b.grid);
  const int nVB = (t.nVoxPad + 255) / 256;
  const size_t raB = (size_t)t.nSamPad * b.KC * 2 * 2, zbB = (size_t)t.nVoxPad * 2 * b.KC * 2 * 2;
  const size_t fbB = (size_t)t.nVoxPad * BW_NF * 2 * 2;
  const size_t dkB = (size_t)b.slots * t.nSamPad * kRF * 4, gB = (size_t)t.nSt * 4 * t.nVoxPad * 4;
  const size_t redB = (size_t)bwd_red_slots(t) * 8, vpB = (size_t)2 * kBwdVoxSplit * t.nVoxPad * 8;
  auto al = [](size_t n) { return (n + 255) / 256 * 256; };
  b.bytes = al(raB) + al(zbB) + al(fbB) + al(dkB) + 2 * al(gB) + al(vpB) + al(redB);
  cudaError_t e = cudaMalloc(&b.mem, b.bytes);
  if (e != cudaSuccess) return e;
  char *m = (char *)b.mem;
  b.ra = (uint16_t *)m; m += al(raB);
  b.zb = (uint16_t *)m; m += al(zbB);
  b.fb = (uint16_t *)m; m += al(fbB);
  b.dkpart = (float *)m; m += al(dkB);
  b.g1 = (float *)m; m += al(gB);
  b.gt = (float *)m; m += al(gB);
  b.vpart = (double *)m; m += al(vpB);
  b.dred = (double *)m;
  const int64_t nF = (int64_t)nChunks * BW_NF * TV;
  k_bw_fb<<<(unsigned)((nF + 255) / 256), 256>>>(t.bfraw, nChunks, b.fb);
  e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaDeviceSynchronize();
  if (e != cudaSuccess) {
    cudaFree(b.mem);
    return e;
  }
  h->tcb_host = new BwBuffers(b);
  h->bytes += (int64_t)b.bytes;
  return cudaSuccess;
}

}  // namespace

bool tc_backward_supported(const hoe_handle *h) {
  // shared memory: up to 16 coils with residual widths up to 24, or up to
  // 32 coils with widths up to 16
  return h->tc.ready && ((h->t.nCha <= 16 && h->t.KP <= 24) || (h->t.nCha <= 32 && h->t.KP <= 16));
}

cudaError_t tc_backward(hoe_handle *h, const float2 *x, const float2 *r, float *dk, float *ddf, double *dt0,
                        int flags, cudaStream_t st) {
  cudaError_t e = bw_prepare(h);
  if (e != cudaSuccess) return e;
  const BwBuffers &b = *(const BwBuffers *)h->tcb_host;
  const TcBuffers &tb = *(const TcBuffers *)h->tc_host;
  const auto &t = h->t;
  const int nChunks = t.nVoxPad / TV;
  const int64_t nR = (int64_t)(t.nSamPad / TM) * TM * (b.KC / 8);   // 16-byte units
  const int64_t nZ = (int64_t)nChunks * TM * (b.KC / 8);
  // programmatic dependent launches (pdl_wait before each kernel's first
  // global access); k_bw_ra also zeroes the dk partial slots
  const int64_t nz4 = (int64_t)b.slots * t.nSamPad * kRF / 4;
  e = launch_pdl(k_bw_ra, dim3((unsigned)((nR + 255) / 256)), dim3(256), 0, st, r, t.nSam, t.nCha, t.nSamPad, b.KC,
                 b.ra, (float4 *)b.dkpart, nz4);
  if (e == cudaSuccess)
    e = launch_pdl(k_bw_zb, dim3((unsigned)((nZ + 255) / 256)), dim3(256), 0, st, x, (const int *)t.perm,
                   (const float2 *)t.csm, nChunks, t.nChaPad, t.nCha, b.KC, b.zb);
  if (e != cudaSuccess) return e;
  BwParams p{};
  p.kpHi = t.kpHi; p.kpLo = t.kpLo; p.dbHi = t.dbHi; p.dbLo = t.dbLo;
  p.AtabP = tb.AtabP; p.BtabQ = tb.BtabQ;
  p.ra = b.ra; p.zb = b.zb; p.fb = b.fb;
  p.times = t.times;
  p.dkpart = b.dkpart; p.g1part = b.g1; p.gtpart = b.gt;
  p.err = tb.err;
  p.nSt = t.nSt; p.nChunks = nChunks; p.nSamPad = t.nSamPad; p.nVoxPad = t.nVoxPad;
  p.scaleG = (float)(2.0 * 3.14159265358979323846 / std::sqrt((double)t.nVox));
  e = bw_dispatch(b.KC, t.KP, p, b.grid, st);
  h->launches += 3;
  if (e != cudaSuccess) return e;
  return bwd_finish(h, b.dkpart, b.slots, b.g1, b.gt, t.nSt * 4, b.vpart, b.dred, dk, ddf, dt0, flags, st);
}

void tc_backward_release(hoe_handle *h) {
  if (!h->tcb_host) return;
  BwBuffers *b = (BwBuffers *)h->tcb_host;
  if (b->mem) cudaFree(b->mem);
  delete b;
  h->tcb_host = nullptr;
}

}  // namespace hoe
