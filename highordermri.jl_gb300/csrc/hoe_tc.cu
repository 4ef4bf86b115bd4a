// Tensor-core engine: the complex contraction on tcgen05 (UMMA) with
// split-BF16 operands (3 products: hi*hi + hi*lo + lo*hi) accumulated in
// FP32 in tensor memory.
//
// Both directions are the same real GEMM shape, D[M=128 rows, N=2*nChaTC] +=
// A[rows, K] * B[K, N], with re/im interleaved along K and along N:
//   forward  rows = samples, columns = voxels:
//            A[s,2v+0] = Re P[s,v], A[s,2v+1] = Im P[s,v]
//            B[2v+0,2c] = Re Z, B[2v+0,2c+1] = Im Z, B[2v+1,2c] = -Im Z, B[2v+1,2c+1] = Re Z
//            so D[s,2c..2c+1] = (Re, Im) of sum_v P[s,v] Z[v,c]
//   adjoint  rows = voxels, columns = samples:
//            A[v,2s+0] = Re P[s,v], A[v,2s+1] = Im P[s,v]
//            B[2s+0,2c] = Re Y, B[2s+0,2c+1] = Im Y, B[2s+1,2c] = Im Y, B[2s+1,2c+1] = -Re Y
//            so D[v,2c..2c+1] = (Re, Im) of sum_s conj(P[s,v]) Y[s,c]
//
// The A operand (the phase tile) never touches global or shared memory.  Per
// stage of 64 columns a residual-phase warp first computes the whole phase of
// the 128 x 64 tile in radians on the tensor cores into a TMEM tile, a few
// stages ahead: the residual dbeta.kappa (TF32, 3 products of hi/lo splits
// made at create time, K = reduced rank) plus one more k-step that adds the
// row and column anchors (see hoe_internal.cuh) as [a_hi, a_lo, 1, 1] .
// [1, 1, c_hi, c_lo].  12 or 16 "phase" warps read it, take the FP32 sincos, split the result
// into BF16 hi/lo and write both into a TMEM A tile with tcgen05.st (lane =
// row, one 32-bit column = one (re, im) pair).  A loader warp streams the
// pre-tiled B operand, the TF32 residual tiles and the anchors with
// cp.async.bulk (TMA bulk copies) onto mbarriers.  Two threads issue the
// contraction with A from TMEM and B from shared memory: one the product
// hi x [B_hi | B_lo] as a single MMA of twice the width, the other lo x B_hi
// (up to 32 coils; beyond that the k-steps are split between them, 3
// products each).  Their FP32 TMEM accumulators are flushed every GROUP
// stages into FP32 register sums.  Every mbarrier wait is bounded in time: on
// timeout the kernel records HOE_ERR_TIMEOUT in a device word, stops
// issuing work, waits (bounded) for its own copies and MMAs and frees TMEM.
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <algorithm>
#include <cstdint>
#include <string>
#include <vector>

#include "hoe_internal.cuh"
#include "hoe_tcgen05.cuh"

namespace hoe {
namespace {

// Warp roles: PW phase warps, two contraction issuers, one residual-phase
// issuer (TF32 MMAs) that also owns the TMEM allocation, and one loader.
// Phase warps form NG groups of GW that take the stages in turn (group
// it % NG), so one group's barrier and tensor-memory latencies overlap the
// others' arithmetic; warp w covers TMEM lane quarter w & 3.
//   N <= 32: 3 groups of 4 (12 warps, 16 in all, 128 registers a thread); a
//     warp covers all 64 columns of its stages.  The role warps then share an
//     SM sub-partition with 3 phase warps instead of 4, which shortens the
//     residual-phase issuer's loop, the chain that sets the stage time.
//   N >= 64: 2 groups of 8 (16 warps, 20 in all, 96 registers, which the
//     wider accumulators need); a warp covers half of the columns.
template <int N>
struct Warps {
  static constexpr int NG = N <= 32 ? 3 : 2;
  static constexpr int GW = N <= 32 ? 4 : 8;
  static constexpr int PW = NG * GW;
  static constexpr bool WIDE = GW == 4;
  // warps that read out the accumulators: 2 or 4 per lane quarter
  static constexpr int FLW = NG == 3 ? 8 : PW;
  static constexpr int CISS = PW;        // contraction issuers: PW, PW + 1
  static constexpr int PISS = PW + 2;    // residual-phase issuer, TMEM owner
  static constexpr int LOAD = PW + 3;
  static constexpr int THREADS = (PW + 4) * 32;
};

// A tensor-core FP32 accumulator sums at most GROUP stages (Tmem<N>::GROUP,
// at most 256 MMAs per accumulator) before it is added, in round-to-nearest
// FP32, into register sums: long accumulation chains in TMEM lose accuracy
// on coherent sums.

// One operator's operands for one direction.  A launch walks the work items
// (row tile, column chunk) of its slices in order: slice si owns the global
// items [first, first + nRowTiles*nColChunks).
struct TcSlice {
  const float *rowHi, *rowLo;   // TF32 row-side residual tables: kappa (forward) / dbeta (adjoint)
  const float *colHi, *colLo;   // TF32 column-side residual tables: dbeta (forward) / kappa (adjoint)
  const float *rowX;            // [colTile][rowXStride][4] TF32 anchor rows: AtabP (forward) / BtabQ (adjoint)
  const float *colX;            // [rowTile][colXStride][4] TF32 anchor columns: BtabQ (forward) / AtabP (adjoint)
  const uint16_t *Bop;          // [nColChunks][hi,lo][N x TK] BF16 tiles, canonical layout
  float2 *part;                 // [slot][nRowPad][nChaPad] partial sums (zeroed before launch)
  int64_t first;                // global index of the slice's first work item
  int rowXStride, colXStride;
  int nRowPad;
  int nColChunks;               // column chunks per row tile (C)
  int nRowTiles;
  int pad;
};

// Up to MS slices per launch (passed by value as a __grid_constant__
// parameter: 96 bytes per slice, 32 slices fit the 4 KB parameter space).
template <int MS>
struct TcParams {
  int *err;
  int64_t work;                 // all slices' work items, split evenly over gridDim.x CTAs
  int nSlices, nChaPad, nChaTC, pad;
  TcSlice s[MS];
  // slice i (a compile-time index for single-slice launches)
  __host__ __device__ __forceinline__ const TcSlice &at(int i) const { return s[MS == 1 ? 0 : i]; }
};
constexpr int kBatchSlices = 32;
static_assert(sizeof(TcParams<kBatchSlices>) <= 4096, "kernel parameter space");

// Position in the work sequence: slice si, row tile rt, column chunk ch.
template <int MS>
struct Cursor {
  int si, rt, ch, C, nRT;
  __device__ __forceinline__ void init(const TcParams<MS> &p, int64_t w) {
    si = 0;
    if constexpr (MS > 1) {
      while (si + 1 < p.nSlices && p.s[si + 1].first <= w) ++si;
    }
    C = p.at(si).nColChunks;
    nRT = p.at(si).nRowTiles;
    const int64_t off = w - p.at(si).first;
    rt = (int)(off / C);
    ch = (int)(off % C);
  }
  __device__ __forceinline__ void next(const TcParams<MS> &p) {
    if (++ch == C) {
      ch = 0;
      ++rt;
      if constexpr (MS > 1) {
        if (rt == nRT && si + 1 < p.nSlices) {
          rt = 0;
          ++si;
          C = p.s[si].nColChunks;
          nRT = p.s[si].nRowTiles;
        }
      }
    }
  }
};

// Tensor-memory plan (512 columns): BF16 phase tiles ABUF x [hi TV | lo TV]
// columns (one 32-bit column per complex element), residual-phase tiles
// PD x TV FP32 columns, ACCBUF accumulator sets of ACCW FP32 columns.
//   PSPLIT (N <= 64): issuer 0 accumulates hi x [B_hi | B_lo] into 2N
//     columns [hi.B_hi | hi.B_lo], issuer 1 lo x B_hi into N more; one set,
//     flushed every 32 stages while the issuers pause (a second set would
//     not leave room for two residual tiles).
//   otherwise (N = 128): one issuer, 3 products per k-step into N columns;
//     one set, flushed every 8 stages, and two phase tiles, so the phase
//     warps write stage s+1 while stage s is multiplied (measured 1.3%
//     faster than two sets with one phase tile; both leave the same PD).
template <int N>
struct Tmem {
  static constexpr bool PSPLIT = N <= 64;
  static constexpr int NISS = PSPLIT ? 2 : 1;
  static constexpr int ABUF = (N <= 32 || N == 128) ? 2 : 1;
  static constexpr int ACCBUF = 1;
  static constexpr int NPART = PSPLIT ? 3 : 1;   // N-wide parts of one set
  static constexpr int ACCW = NPART * N;
  static constexpr int QOFF = 2 * N;             // issuer 1's part of a set (PSPLIT)
  static constexpr int GROUP = PSPLIT ? 32 : 8;
  static constexpr int ACC = ACCBUF * ACCW;
  static constexpr int PD_MAX = (512 - ACC - ABUF * 2 * TV) / TV;
  static constexpr uint32_t A_COL = 0;
  static constexpr uint32_t P_COL = ABUF * 2 * TV;
};

// Shared-memory plan (dynamic, 1024-byte aligned base):
//   B   [NS][hi,lo]   BF16 contraction operand, N x TK
//   CV  [NS][hi,lo]   TF32 column residual tile, TV x KP
//   RV  [2][hi,lo]    TF32 row residual tile, 128 x KP (one per row-tile parity)
//   XR  [NS][data,0]  TF32 anchor k-step, row side: 128 rows x 4, then 128 x 4 zeros
//   XC  [NS][data,0]  TF32 anchor k-step, column side: TV columns x 4, then zeros
//   barriers: full[NS] empty[NS] afull[ABUF] segdone[2]
//             tmemfree[2] pfull[PB] pfree[PB] rfull[2] rfree[2]
// The residual-phase issuer runs up to PD stages ahead of the phase warps.
template <int N, int KP, int NS>
struct Smem {
  static constexpr int ABUF = Tmem<N>::ABUF;
  // Residual widths up to 16: the row tile's TF32 residual vectors (hi, lo)
  // also sit in tensor memory, 2*KP columns after the accumulators, as the A
  // operand of the residual MMAs (written by phase warps 0-3 once per row
  // tile), so that those MMAs read only the column tile from shared memory.
  static constexpr bool RT = KP <= 16;
  static constexpr int R_COLS = RT ? 2 * KP : 0;
  static constexpr int PD_CAP = (512 - Tmem<N>::ACC - ABUF * 2 * TV - R_COLS) / TV;
  static constexpr int PD = (NS - 1) < PD_CAP ? (NS - 1) : (PD_CAP < 3 ? PD_CAP : 3);
  static constexpr int B_TILE = N * TK * 2;
  static constexpr int CV_TILE = TV * KP * 4;
  static constexpr int RV_TILE = TM * KP * 4;
  static constexpr size_t B_OFF = 0;
  static constexpr size_t CV_OFF = B_OFF + (size_t)NS * 2 * B_TILE;
  static constexpr size_t RV_OFF = CV_OFF + (size_t)NS * 2 * CV_TILE;
  static constexpr int XR_BYTES = TM * 4 * 4;    // one core-matrix column of 128 rows
  static constexpr int XC_BYTES = TV * 4 * 4;
  static constexpr size_t XR_OFF = RV_OFF + (size_t)2 * 2 * RV_TILE;
  static constexpr size_t XC_OFF = XR_OFF + (size_t)NS * 2 * XR_BYTES;
  static constexpr size_t BAR_OFF = (XC_OFF + (size_t)NS * 2 * XC_BYTES + 7) / 8 * 8;
  // pfull/pfree barriers: stage s uses barrier s % PB.  A parity wait for s
  // on a barrier whose previous phase (stage s - PB) were still open would
  // see the phase before that and go ahead early.  With PB >= NG that cannot
  // happen: the waiting group has already seen stage s - NG >= s - PB done,
  // and the residual tiles complete in stage order.  With PB >= PD the
  // residual issuer has seen all arrivals for stage s before it writes stage
  // s + PD, so the arrivals for s and s + PB never mix.  Three groups get
  // two barriers each (6; measured 0.7% faster than 3 at 16 coils).
  static constexpr int NG = Warps<N>::NG;
  static constexpr int PB = NG == 3 ? 6 : (PD > NG ? PD : NG);
  static_assert(PB >= NG && PB >= PD, "residual-tile barriers");
  static constexpr int NBAR = 2 * NS + ABUF + 10 + 2 * PB;
  static constexpr size_t MISC_OFF = BAR_OFF + (size_t)NBAR * 8;
  static constexpr size_t BYTES = MISC_OFF + 16 + 1024;  // + alignment slack
};

template <int N, int KP>
constexpr int pick_stages() {
  return Smem<N, KP, 6>::BYTES <= 227 * 1024 ? 6
       : Smem<N, KP, 5>::BYTES <= 227 * 1024 ? 5
       : Smem<N, KP, 4>::BYTES <= 227 * 1024 ? 4
       : Smem<N, KP, 3>::BYTES <= 227 * 1024 ? 3 : 2;
}

template <int N, int KP, int NS, int MS>
__global__ void __launch_bounds__(Warps<N>::THREADS, 1) k_tc_contract(const __grid_constant__ TcParams<MS> p) {
  using S = Smem<N, KP, NS>;
  constexpr int ABUF = S::ABUF, PD = S::PD, PB = S::PB, NISS = Tmem<N>::NISS;
  constexpr int ACCBUF = Tmem<N>::ACCBUF, NPART = Tmem<N>::NPART, ACCW = Tmem<N>::ACCW;
  constexpr int QOFF = Tmem<N>::QOFF, GROUP = Tmem<N>::GROUP;
  constexpr bool PSPLIT = Tmem<N>::PSPLIT;
  using W = Warps<N>;
  constexpr int NG = W::NG, GW = W::GW, PW = W::PW, FLW = W::FLW;
  constexpr int CISS_WARP = W::CISS, PISS_WARP = W::PISS, LOAD_WARP = W::LOAD;
  static_assert(PD >= 1, "residual-phase look-ahead");
  extern __shared__ unsigned char smem_raw[];
  unsigned char *smem = (unsigned char *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  unsigned char *sB = smem + S::B_OFF;
  unsigned char *sCV = smem + S::CV_OFF;
  unsigned char *sRV = smem + S::RV_OFF;
  unsigned char *sXR = smem + S::XR_OFF;
  unsigned char *sXC = smem + S::XC_OFF;
  uint64_t *full = reinterpret_cast<uint64_t *>(smem + S::BAR_OFF);
  uint64_t *empty = full + NS;        // B-ring stage consumed by the contraction MMAs
  uint64_t *afull = empty + NS;       // [ABUF] TMEM phase tile written (one phase-warp group)
  uint64_t *segdone = afull + ABUF;   // [ACCBUF] accumulator set complete (group of stages)
  uint64_t *tmemfree = segdone + 2;   // [ACCBUF] accumulator set read out
  uint64_t *pfull = tmemfree + 2;     // [PB] residual-phase TMEM tile computed
  uint64_t *pfree = pfull + PB;       // [PB] residual-phase TMEM tile read out
  uint64_t *rfull = pfree + PB;       // [2] row residual tile loaded
  uint64_t *rfree = rfull + 2;        // [2] row residual tile no longer read by MMAs
  uint64_t *rtfull = rfree + 2;       // [1] row residual vectors written to TMEM (4 warps)
  uint64_t *rtfree = rtfull + 1;      // [1] ... no longer read by the residual MMAs
  uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(smem + S::MISC_OFF);
  volatile int *abort = reinterpret_cast<volatile int *>(smem + S::MISC_OFF + 8);
  constexpr uint32_t TMEM_COLS = 512;
  constexpr uint32_t A_COL = Tmem<N>::A_COL, P_COL = Tmem<N>::P_COL;
  constexpr uint32_t ACC_COL = P_COL + PD * TV;   // group g, issuer q: ACC_COL + (g%ACCBUF)*ACCW + q*QOFF
  constexpr bool RT = S::RT;
  constexpr uint32_t R_COL = ACC_COL + ACCBUF * ACCW;   // [hi KP | lo KP] when RT
  static_assert(R_COL + S::R_COLS <= TMEM_COLS, "tensor memory plan");
  constexpr uint32_t SBO_TF32 = (KP / 4) * 128;

  const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
  const int G = gridDim.x, b = blockIdx.x;
  const int64_t wb = (int64_t)b * p.work / G, we = (int64_t)(b + 1) * p.work / G;
  const int nIter = (int)(we - wb);
  Cursor<MS> c0;
  c0.init(p, wb);

  if (threadIdx.x == 0) {
    for (int i = 0; i < NS; ++i) {
      mbar_init(&full[i], 1);
      mbar_init(&empty[i], NISS);
    }
    for (int i = 0; i < ABUF; ++i) {
      mbar_init(&afull[i], GW);
    }
    for (int i = 0; i < 2; ++i) {
      mbar_init(&segdone[i], NISS);
      mbar_init(&tmemfree[i], FLW);
      mbar_init(&rfull[i], 1);
      mbar_init(&rfree[i], 1);
    }
    for (int i = 0; i < PB; ++i) {
      mbar_init(&pfull[i], 1);
      mbar_init(&pfree[i], GW);
    }
    mbar_init(&rtfull[0], 4);
    mbar_init(&rtfree[0], 1);
    *abort = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  // the second core-matrix column of every anchor k-step operand is zero
  for (int i = threadIdx.x; i < NS * (S::XR_BYTES + S::XC_BYTES) / 16; i += W::THREADS) {
    const int nr = NS * S::XR_BYTES / 16;
    float4 *dst = i < nr
        ? reinterpret_cast<float4 *>(sXR + (size_t)(i / (S::XR_BYTES / 16)) * 2 * S::XR_BYTES + S::XR_BYTES) + i % (S::XR_BYTES / 16)
        : reinterpret_cast<float4 *>(sXC + (size_t)((i - nr) / (S::XC_BYTES / 16)) * 2 * S::XC_BYTES + S::XC_BYTES) + (i - nr) % (S::XC_BYTES / 16);
    *dst = make_float4(0.f, 0.f, 0.f, 0.f);
  }
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  if (warp == PISS_WARP) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(tmem_slot)),
                 "r"(TMEM_COLS));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;
  // the prologue above touches no global memory; the B operand, the slots
  // and the tables may be written by the previous kernel in the stream
  pdl_wait();
  pdl_trigger();

  if (warp < PW) {
    // ---------------- phase generator: one row x 64 (N <= 32) or 32 columns
    // of every NG-th stage.  FLUSH_LAG stages after a group of GROUP stages
    // closes (or at the end), the first FLW warps add its accumulator set into
    // register sums (columns split by warp >> 2) and, at the end of a row
    // tile, write the sums to the partial slot.  With one set the issuers wait
    // for this, so it comes right after the next stage's tile; with two it
    // waits one stage more, so that the group's MMAs are normally done by then.
    const int row = (warp & 3) * 32 + lane;
    const int qcol = warp >> 2;          // accumulator part (FLW / 4 of them)
    const int half = W::WIDE ? 0 : (warp >> 2) & 1;   // stage columns [half*32, half*32+32) when not WIDE
    const int par = warp / GW;           // stages with it % NG == par
    const uint32_t laneBase = (uint32_t)((warp & 3) * 32) << 16;
    constexpr int NA = N / (FLW / 4);  // accumulator columns owned by this thread
    constexpr int FLUSH_LAG = ACCBUF == 1 ? 1 : 2;
    float acc[NA];
#pragma unroll
    for (int i = 0; i < NA; ++i) acc[i] = 0.f;
    int grp = -1;
    int pendGrp = -1, pendRT = -1, pendSI = 0, pendIt = 0;
    bool pendLast = false;
    bool ok = true;
    auto flush = [&]() {
      // add group pendGrp into acc; write acc out if it closed its row tile
      if (warp >= FLW) { pendGrp = -1; return; }
      const int g = pendGrp, gb = g % ACCBUF, gr = g / ACCBUF;
      bool got = ok && wait_bar(&segdone[gb], gr & 1, abort, p.err);
      tc_fence_after();
      if (got) {
#pragma unroll
        for (int q = 0; q < NPART; ++q) {
          const uint32_t base =
              tmem + laneBase + ACC_COL + (uint32_t)(gb * ACCW + q * N + qcol * NA);
          if constexpr (NA % 16 == 0) {
#pragma unroll
            for (int k0 = 0; k0 < NA; k0 += 16) {
              float v[16];
              tmem_ld16(base + k0, v);
#pragma unroll
              for (int i = 0; i < 16; ++i) acc[k0 + i] += v[i];
            }
          } else if constexpr (NA == 8) {
            float v[8];
            tmem_ld8(base, v);
#pragma unroll
            for (int i = 0; i < 8; ++i) acc[i] += v[i];
          } else {
            static_assert(NA == 4, "accumulator columns per thread");
            float v[4];
            tmem_ld4(base, v);
#pragma unroll
            for (int i = 0; i < 4; ++i) acc[i] += v[i];
          }
        }
      }
      tc_fence_before();
      __syncwarp();
      if (lane == 0) mbar_arrive(&tmemfree[gb]);
      if (pendLast) {
        const TcSlice &ps = p.at(pendSI);
        const int slot = b - work_owner(ps.first + (int64_t)pendRT * ps.nColChunks, p.work, G);
        float2 *dst = ps.part + ((int64_t)slot * ps.nRowPad + (int64_t)pendRT * TM + row) * p.nChaPad;
        const int nOut = min(p.nChaTC, p.nChaPad);
        if (ok) {
#pragma unroll
          for (int i = 0; i < NA; i += 2) {
            int c = (qcol * NA + i) / 2;
            if (c < nOut) dst[c] = make_float2(acc[i], acc[i + 1]);
          }
        }
#pragma unroll
        for (int i = 0; i < NA; ++i) acc[i] = 0.f;
      }
      pendGrp = -1;
    };
    // sincos of 16 phases (radians) -> BF16 hi/lo pairs.  The phase is the
    // sum of two anchors in [-pi, pi] and the residual, which the plan bounds
    // (at most kTcMaxPhaseBound cycles, else the engine is refused).  Over
    // that range the error of the product stays far inside its tolerance
    // (measured 1.3e-5 vs FP64 at a 308-cycle bound).  An explicit Cody-Waite
    // reduction before the sincos measured 32% slower with no accuracy gain
    // up to 79 cycles.  Each (cos, sin) pair becomes one BF16 hi word and one
    // BF16 lo word (low half = cos).
    auto phase16 = [&](const float *d, uint32_t *hi, uint32_t *lo) {
#pragma unroll
      for (int j = 0; j < 16; ++j) {
        float sn, cs;
        __sincosf(d[j], &sn, &cs);
        split_bf16x2(cs, sn, hi[j], lo[j]);
      }
    };
    Cursor<MS> c = c0;
    int kt = -1;   // row tiles whose residual vectors warps 0-3 wrote to TMEM
    for (int it = 0; it < nIter && ok; ++it) {
      if (it > 0) c.next(p);
      if constexpr (RT) {
        if (warp < 4 && (it == 0 || c.ch == 0)) {
          // the new row tile's residual vectors, hi and lo, from the shared
          // tile into TMEM once the previous row tile's residual MMAs are done
          ++kt;
          if ((kt > 0 && !wait_bar_warp(&rtfree[0], (kt - 1) & 1, abort, p.err)) ||
              !wait_bar_warp(&rfull[kt & 1], (kt >> 1) & 1, abort, p.err)) { ok = false; break; }
          tc_fence_after();
          const float4 *rv = reinterpret_cast<const float4 *>(sRV + (size_t)(kt & 1) * 2 * S::RV_TILE);
          uint32_t hv[KP], lv[KP];
#pragma unroll
          for (int kc = 0; kc < KP / 4; ++kc) {
            const int o = ((row / 8) * (KP / 4) + kc) * 8 + (row % 8);   // float4 index
            const float4 h = rv[o], l = rv[S::RV_TILE / 16 + o];
            hv[4 * kc] = __float_as_uint(h.x); hv[4 * kc + 1] = __float_as_uint(h.y);
            hv[4 * kc + 2] = __float_as_uint(h.z); hv[4 * kc + 3] = __float_as_uint(h.w);
            lv[4 * kc] = __float_as_uint(l.x); lv[4 * kc + 1] = __float_as_uint(l.y);
            lv[4 * kc + 2] = __float_as_uint(l.z); lv[4 * kc + 3] = __float_as_uint(l.w);
          }
          const uint32_t rbase = tmem + laneBase + R_COL;
          if constexpr (KP == 16) {
            tmem_st16(rbase, hv);
            tmem_st16(rbase + KP, lv);
          } else {
            tmem_st8(rbase, hv);
            tmem_st8(rbase + KP, lv);
          }
          asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
          tc_fence_before();
          __syncwarp();
          if (lane == 0) mbar_arrive(&rtfull[0]);
        }
      }
      if (it == 0 || c.ch % GROUP == 0) ++grp;
      if (it % NG == par) {
        // phase of this stage in radians (TMEM), then release its buffer
        const int pb = it % PD, pbar = it % PB, pr = it / PB;
        if (!wait_bar(&pfull[pbar], pr & 1, abort, p.err)) { ok = false; break; }
        tc_fence_after();
        const uint32_t pBase = tmem + laneBase + P_COL + (uint32_t)(pb * TV + half * 32);
        const int ab = it % ABUF, ar = it / ABUF;
        const uint32_t aBase = tmem + laneBase + A_COL + (uint32_t)(ab * 2 * TV + half * 32);
        // H blocks of 32 columns, 16 at a time; the residual tile is released
        // once its last 16 columns are in registers
        constexpr int H = W::WIDE ? 2 : 1;
        float d[16];
        uint32_t hi[16], lo[16];
#pragma unroll
        for (int h = 0; h < H; ++h) {
          const uint32_t ph = pBase + (uint32_t)(h * 32), ah = aBase + (uint32_t)(h * 32);
          tmem_ld16(ph, d);
          phase16(d, hi, lo);
          if (h == 0) {
            // TMEM phase tile buffer: free once the contraction of stage
            // it-ABUF is done, which the stage's `empty` barrier records (the
            // slot of stage it-ABUF cannot have been reused: that needs this
            // stage's tile)
            if (ar > 0 && !wait_bar(&empty[(it - ABUF) % NS], ((it - ABUF) / NS) & 1, abort, p.err)) { ok = false; break; }
            tc_fence_after();
          }
          tmem_st16(ah, hi);
          tmem_st16(ah + TV, lo);
          tmem_ld16(ph + 16, d);
          if (h == H - 1) {
            tc_fence_before();
            __syncwarp();
            if (lane == 0) mbar_arrive(&pfree[pbar]);
          }
          phase16(d, hi, lo);
          tmem_st16(ah + 16, hi);
          tmem_st16(ah + TV + 16, lo);
        }
        if (!ok) break;
        asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
        tc_fence_before();
        __syncwarp();
        if (lane == 0) mbar_arrive(&afull[ab]);
      }
      // a closed group is flushed two stages later, when its MMAs are done
      if (pendGrp >= 0 && it >= pendIt + FLUSH_LAG) flush();
      const bool endRT = (it == nIter - 1) || (c.ch + 1 == c.C);
      if (endRT || (c.ch + 1) % GROUP == 0) {
        if (pendGrp >= 0) flush();  // a short group closed within FLUSH_LAG stages of the previous one
        pendGrp = grp;
        pendRT = c.rt;
        pendSI = c.si;
        pendLast = endRT;
        pendIt = it;
      }
    }
    if (pendGrp >= 0) flush();
  } else if (warp == CISS_WARP || warp == CISS_WARP + 1) {
    // ---------------- contraction issuers: with PSPLIT issuer 0 takes
    // hi x [B_hi | B_lo] and issuer 1 lo x B_hi over all k-steps, otherwise
    // issuer q takes k-steps [q*KS, (q+1)*KS) with all 3 products
    const int q = warp - CISS_WARP;
    if (q < NISS && nIter > 0) {
      // the whole warp walks the loop and waits; the elected lane issues
      const bool leader = elect_one();
      constexpr int KS = (TK / 16) / NISS;
      constexpr uint32_t idescC = idesc_bf16(TM, N);
      uint64_t *lastBar = nullptr;
      uint32_t lastPar = 0;
      int grp = -1;
      Cursor<MS> c = c0;
      for (int it = 0; it < nIter; ++it) {
        if (it > 0) c.next(p);
        const int ch = c.ch;
        const bool first = (it == 0) || (ch % GROUP == 0);
        if (first) {
          ++grp;
          // accumulator set grp%ACCBUF was last used by group grp-ACCBUF: wait until it was read out
          if (grp >= ACCBUF &&
              !wait_bar_warp(&tmemfree[grp % ACCBUF], ((grp / ACCBUF) - 1) & 1, abort, p.err)) break;
        }
        const bool last = (it == nIter - 1) || (ch + 1 == c.C) || ((ch + 1) % GROUP == 0);
        const int slot = it % NS, round = it / NS;
        const int ab = it % ABUF, ar = it / ABUF;
        if (!wait_bar_warp(&full[slot], round & 1, abort, p.err)) break;
        if (!wait_bar_warp(&afull[ab], ar & 1, abort, p.err)) break;
        tc_fence_after();
        const uint32_t dt = tmem + ACC_COL + (uint32_t)((grp % ACCBUF) * ACCW + q * QOFF);
        const uint32_t aHi = tmem + A_COL + (uint32_t)(ab * 2 * TV);
        const uint32_t aLo = aHi + TV;
        const uint64_t bHi = umma_desc(smem_u32(sB + (size_t)slot * 2 * S::B_TILE));
        const uint64_t bLo = umma_desc(smem_u32(sB + (size_t)slot * 2 * S::B_TILE + S::B_TILE));
        if (leader) {
        if constexpr (PSPLIT) {
          // B_lo follows B_hi in shared memory as N more rows at the same
          // stride, so [B_hi | B_lo] is one operand of width 2N
          constexpr uint32_t idescW = idesc_bf16(TM, 2 * N);
          const uint32_t aS = q == 0 ? aHi : aLo;
          const uint32_t idS = q == 0 ? idescW : idescC;
#pragma unroll
          for (int ks = 0; ks < TK / 16; ++ks) {
            const uint32_t ka = ks * 8;                          // 16 BF16 = 8 TMEM columns
            const uint64_t kb = (uint64_t)(ks * 2 * LBO) >> 4;   // two core matrices along K
            umma_ta(dt, aS + ka, bHi + kb, idS, (first && ks == 0) ? 0u : 1u);
          }
        } else {
#pragma unroll
          for (int kk = 0; kk < KS; ++kk) {
            const int ks = q * KS + kk;
            const uint32_t ka = ks * 8;
            const uint64_t kb = (uint64_t)(ks * 2 * LBO) >> 4;
            umma_ta(dt, aHi + ka, bHi + kb, idescC, (first && kk == 0) ? 0u : 1u);
            umma_ta(dt, aHi + ka, bLo + kb, idescC, 1u);
            umma_ta(dt, aLo + ka, bHi + kb, idescC, 1u);
          }
        }
        umma_commit(&empty[slot]);
        if (last) umma_commit(&segdone[grp % ACCBUF]);
        }
        __syncwarp();
        lastBar = &empty[slot];
        lastPar = round & 1;
      }
      if (*abort && lastBar) drain_bar(lastBar, lastPar);  // MMAs done before TMEM is freed
    }
    __syncwarp();
  } else if (warp == PISS_WARP) {
    // ---------------- residual-phase issuer: TF32 tile of stage j, up to PD
    // stages ahead of the phase warps (whole warp, elected lane issues)
    if (nIter > 0) {
      const bool leader = elect_one();
      constexpr uint32_t idescP = idesc_tf32(TM, TV);
      uint64_t *lastBar = nullptr;
      uint32_t lastPar = 0;
      int kj = 0;
      Cursor<MS> c = c0;
      for (int j = 0; j < nIter; ++j) {
        if (j > 0) {
          c.next(p);
          if (c.ch == 0) ++kj;
        }
        const bool lastOfRow = (j == nIter - 1) || (c.ch + 1 == c.C);
        const int s = j % NS, r = j / NS;
        if (!wait_bar_warp(&full[s], r & 1, abort, p.err)) break;
        if (!wait_bar_warp(&rfull[kj & 1], (kj >> 1) & 1, abort, p.err)) break;
        if (RT && (j == 0 || c.ch == 0) && !wait_bar_warp(&rtfull[0], kj & 1, abort, p.err)) break;
        const int pb = j % PD, pbar = j % PB, pr = j / PB;
        // tile buffer pb was last used by stage j - PD
        if (j >= PD && !wait_bar_warp(&pfree[(j - PD) % PB], ((j - PD) / PB) & 1, abort, p.err)) break;
        tc_fence_after();
        const uint32_t dt = tmem + P_COL + (uint32_t)(pb * TV);
        const uint32_t rHi = smem_u32(sRV + (size_t)(kj & 1) * 2 * S::RV_TILE);
        const uint32_t rLo = rHi + S::RV_TILE;
        const uint32_t cHi = smem_u32(sCV + (size_t)s * 2 * S::CV_TILE);
        const uint32_t cLo = cHi + S::CV_TILE;
        if (leader) {
#pragma unroll
          for (int ks = 0; ks < KP / 8; ++ks) {
            const uint32_t ko = ks * 2 * LBO;  // 8 TF32 = two core matrices along K
            if constexpr (RT) {
              // A from TMEM: 8 TF32 columns per k-step, hi at R_COL, lo KP further
              const uint32_t ra = tmem + R_COL + (uint32_t)(ks * 8);
              umma_ta_tf32(dt, ra, umma_desc(cHi + ko, SBO_TF32), idescP, ks ? 1u : 0u);
              umma_ta_tf32(dt, ra, umma_desc(cLo + ko, SBO_TF32), idescP, 1u);
              umma_ta_tf32(dt, ra + KP, umma_desc(cHi + ko, SBO_TF32), idescP, 1u);
            } else {
              umma_tf32(dt, umma_desc(rHi + ko, SBO_TF32), umma_desc(cHi + ko, SBO_TF32), idescP, ks ? 1u : 0u);
              umma_tf32(dt, umma_desc(rHi + ko, SBO_TF32), umma_desc(cLo + ko, SBO_TF32), idescP, 1u);
              umma_tf32(dt, umma_desc(rLo + ko, SBO_TF32), umma_desc(cHi + ko, SBO_TF32), idescP, 1u);
            }
          }
          // anchor k-step: [a_hi, a_lo, 1, 1 | 0] . [1, 1, c_hi, c_lo | 0] adds both anchors
          umma_tf32(dt, umma_desc(smem_u32(sXR + (size_t)s * 2 * S::XR_BYTES), 128, S::XR_BYTES),
                    umma_desc(smem_u32(sXC + (size_t)s * 2 * S::XC_BYTES), 128, S::XC_BYTES), idescP, 1u);
          umma_commit(&pfull[pbar]);
          if (lastOfRow) {
            umma_commit(&rfree[kj & 1]);
            if (RT) umma_commit(&rtfree[0]);
          }
        }
        __syncwarp();
        lastBar = &pfull[pbar];
        lastPar = pr & 1;
      }
      if (*abort && lastBar) drain_bar(lastBar, lastPar);
    }
    __syncwarp();
  } else if (warp == LOAD_WARP) {
    // ---------------- loader: row residual tiles per row tile, per stage the
    // B tiles, column residual tiles and column anchors (whole warp, elected
    // lane issues the copies)
    {
      const bool leader = elect_one();
      const uint32_t stageBytes = 2 * S::B_TILE + 2 * S::CV_TILE + S::XR_BYTES + S::XC_BYTES;
      int issued = 0, kcount = -1, rowIssued = -1;
      Cursor<MS> c = c0;
      for (int it = 0; it < nIter; ++it) {
        if (it > 0) c.next(p);
        const TcSlice &sl = p.at(c.si);
        const int rt = c.rt, ch = c.ch;
        if (it == 0 || ch == 0) {
          ++kcount;
          const int rb = kcount & 1;
          if (kcount >= 2 && !wait_bar_warp(&rfree[rb], ((kcount >> 1) - 1) & 1, abort, p.err)) break;
          if (leader) {
            mbar_expect_tx(&rfull[rb], 2 * S::RV_TILE);
            const size_t ro = (size_t)rt * TM * KP;
            bulk_g2s(sRV + (size_t)rb * 2 * S::RV_TILE, sl.rowHi + ro, S::RV_TILE, &rfull[rb]);
            bulk_g2s(sRV + (size_t)rb * 2 * S::RV_TILE + S::RV_TILE, sl.rowLo + ro, S::RV_TILE, &rfull[rb]);
          }
          __syncwarp();
          rowIssued = kcount;
        }
        const int slot = it % NS, round = it / NS;
        if (round > 0 && !wait_bar_warp(&empty[slot], (round - 1) & 1, abort, p.err)) break;
        if (leader) {
          const size_t co = (size_t)ch * TV * KP;
          mbar_expect_tx(&full[slot], stageBytes);
          bulk_g2s(sB + (size_t)slot * 2 * S::B_TILE, sl.Bop + (size_t)ch * 2 * (N * TK), 2 * S::B_TILE, &full[slot]);
          bulk_g2s(sCV + (size_t)slot * 2 * S::CV_TILE, sl.colHi + co, S::CV_TILE, &full[slot]);
          bulk_g2s(sCV + (size_t)slot * 2 * S::CV_TILE + S::CV_TILE, sl.colLo + co, S::CV_TILE, &full[slot]);
          bulk_g2s(sXR + (size_t)slot * 2 * S::XR_BYTES,
                   sl.rowX + ((int64_t)(ch * TV / 128) * sl.rowXStride + (int64_t)rt * TM) * 4, S::XR_BYTES, &full[slot]);
          bulk_g2s(sXC + (size_t)slot * 2 * S::XC_BYTES,
                   sl.colX + ((int64_t)rt * sl.colXStride + (int64_t)ch * TV) * 4, S::XC_BYTES, &full[slot]);
        }
        __syncwarp();
        issued = it + 1;
      }
      if (*abort) {
        // drain the copies still in flight into this CTA's shared memory
        for (int it = max(0, issued - NS); it < issued; ++it)
          drain_bar(&full[it % NS], (it / NS) & 1);
        if (rowIssued >= 0) drain_bar(&rfull[rowIssued & 1], (rowIssued >> 1) & 1);
      }
    }
    __syncwarp();
  }

  tc_fence_before();
  __syncthreads();
  if (warp == PISS_WARP) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TMEM_COLS));
  }
}

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
// TF32 hi + lo, stored as [hi, lo, 1, 1] (format 0) or [1, 1, hi, lo] (format 1).
__device__ __forceinline__ float tf32_rn(float f) {
  uint32_t b = __float_as_uint(f);
  if ((b & 0x7f800000u) != 0x7f800000u) {
    b += 0x00000fffu + ((b >> 13) & 1u);
    b &= 0xffffe000u;
  }
  return __uint_as_float(b);
}

__global__ void k_tc_anchor_tf32(const float *__restrict__ tab, int64_t n, float4 *__restrict__ out, int format) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double v = 6.283185307179586476925 * (double)tab[i];
  const float h = tf32_rn((float)v);
  const float l = tf32_rn((float)(v - (double)h));
  out[i] = format == 0 ? make_float4(h, l, 1.f, 1.f) : make_float4(1.f, 1.f, h, l);
}

int tc_ncha(int nCha) {
  int n = 8;
  while (n < nCha) n *= 2;
  return n;  // 8, 16, 32 or 64 coils per MMA: N = 16, 32, 64, 128
}

template <int N, int KP>
struct Kern {
  static constexpr int NS = pick_stages<N, KP>();
  static_assert(Smem<N, KP, NS>::PD >= 1, "residual-phase look-ahead");
  using S = Smem<N, KP, NS>;
  static_assert(S::BYTES <= 227 * 1024, "shared memory plan exceeds 227 KB");
};

template <int N, int KP, int MS>
cudaError_t launch_contract(const hoe_handle *h, const TcParams<MS> &p, int G, cudaStream_t st) {
  using K = Kern<N, KP>;
  auto kern = k_tc_contract<N, KP, K::NS, MS>;
  const cudaError_t e = launch_pdl(kern, dim3(G), dim3(Warps<N>::THREADS), K::S::BYTES, st, p);
  h->launches += 1;
  return e;
}

// One-time per (process, instantiation): shared-memory limit; returns the
// resident CTAs per SM.
template <int N, int KP, int MS>
int configure() {
  using K = Kern<N, KP>;
  auto kern = k_tc_contract<N, KP, K::NS, MS>;
  if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)K::S::BYTES) != cudaSuccess)
    return 0;
  int nb = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, kern, Warps<N>::THREADS, K::S::BYTES) != cudaSuccess) return 0;
  return nb;
}

template <int KP, int MS>
cudaError_t launch_n(const hoe_handle *h, const TcParams<MS> &p, int N, int G, cudaStream_t st) {
  switch (N) {
    case 16: return launch_contract<16, KP, MS>(h, p, G, st);
    case 32: return launch_contract<32, KP, MS>(h, p, G, st);
    case 64: return launch_contract<64, KP, MS>(h, p, G, st);
    default: return launch_contract<128, KP, MS>(h, p, G, st);
  }
}

template <int MS>
cudaError_t launch(const hoe_handle *h, const TcParams<MS> &p, int KP, int N, int G, cudaStream_t st) {
  switch (KP) {
    case 8: return launch_n<8, MS>(h, p, N, G, st);
    case 16: return launch_n<16, MS>(h, p, N, G, st);
    default: return launch_n<24, MS>(h, p, N, G, st);
  }
}

template <int KP, int MS>
int configure_n(int N) {
  switch (N) {
    case 16: return configure<16, KP, MS>();
    case 32: return configure<32, KP, MS>();
    case 64: return configure<64, KP, MS>();
    default: return configure<128, KP, MS>();
  }
}

template <int MS>
int configure_kernel(int KP, int N) {
  switch (KP) {
    case 8: return configure_n<8, MS>(N);
    case 16: return configure_n<16, MS>(N);
    default: return configure_n<24, MS>(N);
  }
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
                 (nAP + nBQ) * 16 + 512;
  unsigned char *buf = nullptr;
  cudaError_t e = cudaMalloc(&buf, bytes);
  if (e != cudaSuccess) return e;
  size_t off = 0;
  auto take = [&](size_t n) { unsigned char *p = buf + off; off = (off + n + 255) / 256 * 256; return p; };
  b.bopF = (uint16_t *)take(b.bopFElems * 2);
  b.bopA = (uint16_t *)take(b.bopAElems * 2);
  b.part = (float2 *)take(b.partElems * sizeof(float2));
  b.err = (int *)take(sizeof(int));
  b.AtabP = (float *)take(nAP * 16);
  b.BtabQ = (float *)take(nBQ * 16);
  e = cudaMemset(b.err, 0, sizeof(int));
  if (e != cudaSuccess) { cudaFree(buf); return e; }
  h->tc.buf = buf;
  h->tc.bytes = bytes;
  h->tc.ready = true;
  h->tc_host = new TcBuffers(b);
  e = tc_anchor_tables(h, 0);
  if (e == cudaSuccess) e = cudaStreamSynchronize(0);
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

cudaError_t contract_forward(const hoe_handle *h, const TcBuffers &b, cudaStream_t st) {
  const TcParams<1> p = single_params(h, b, slice_forward(h, b));
  trace(h, EV_FK0, st);
  cudaError_t e = launch(h, p, h->t.KP, b.N, b.gridF, st);
  trace(h, EV_FK1, st);
  return e;
}

cudaError_t contract_adjoint(const hoe_handle *h, const TcBuffers &b, cudaStream_t st) {
  const TcParams<1> p = single_params(h, b, slice_adjoint(h, b));
  trace(h, EV_AK0, st);
  cudaError_t e = launch(h, p, h->t.KP, b.N, b.gridA, st);
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

bool tc_derivative_supported(const hoe_handle *h) { return h->tc.ready && h->t.hasKdot; }

// B x in derivative mode: ceil(nTerm / TP) passes of the 128-wide instance,
// TP = 64 / CP terms of CP = nCha coils each (k_tc_bop_deriv,
// k_tc_deriv_reduce).  tc_derivative_prepare allocates the pass buffers
// once; the delay search calls it before its graph capture.
cudaError_t tc_derivative_prepare(hoe_handle *h) {
  TcBuffers &b = *(TcBuffers *)h->tc_host;
  const auto &t = h->t;
  const int chunks = t.nVoxPad / TV;
  constexpr int ND = 128;
  if (!b.memD) {
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
  }
  return cudaSuccess;
}

cudaError_t tc_derivative(hoe_handle *h, const float2 *x, float2 *y, cudaStream_t st) {
  cudaError_t e = tc_derivative_prepare(h);
  if (e != cudaSuccess) return e;
  const TcBuffers &b = *(const TcBuffers *)h->tc_host;
  const auto &t = h->t;
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
  k_tc_anchor_tf32<<<(unsigned)((nAP + 255) / 256), 256, 0, st>>>(t.Atab, nAP, (float4 *)b.AtabP, 0);
  k_tc_anchor_tf32<<<(unsigned)((nBQ + 255) / 256), 256, 0, st>>>(t.Btab, nBQ, (float4 *)b.BtabQ, 1);
  h->launches += 2;
  return cudaGetLastError();
}

int *tc_error_word(const hoe_handle *h) {
  return h->tc_host ? ((const TcBuffers *)h->tc_host)->err : nullptr;
}

}  // namespace hoe
