// hoe_tc_kernel.cuh — the persistent tensor-core contraction kernel
// (k_tc_contract) and its launch helpers, shared by the translation units
// that instantiate it: hoe_tc.cu (forward and adjoint, single operators and
// batches) and hoe_tc_deriv.cu (the derivative product).
//
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
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <algorithm>
#include <cstdint>

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
// Execution plans of the contraction that hoe_autotune times on an operator,
// for up to 16 coils (N <= 32); plan 0 is the default:
//   1: two phase-warp groups (8 phase warps, 12 warps: more registers a thread)
//   2: four phase-warp groups (16 phase warps, 20 warps, 96 registers)
//   3: a stage ring of 4 (phase tiles in flight) instead of the deepest that fits
//   4: accumulators flushed every 16 stages instead of 32
template <int V> struct TcPlan { static constexpr int NG = 0, NS = 0, GROUP = 0; };
template <> struct TcPlan<1> { static constexpr int NG = 2, NS = 0, GROUP = 0; };
template <> struct TcPlan<2> { static constexpr int NG = 4, NS = 0, GROUP = 0; };
template <> struct TcPlan<3> { static constexpr int NG = 0, NS = 4, GROUP = 0; };
template <> struct TcPlan<4> { static constexpr int NG = 0, NS = 0, GROUP = 16; };

template <int N, int V = 0>
struct Warps {
  static constexpr int NG = TcPlan<V>::NG ? TcPlan<V>::NG : (N <= 32 ? 3 : 2);
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

}  // namespace

// One operator's operands for one direction.  A launch walks the work items
// (row tile, column chunk) of its slices in order: slice si owns the global
// items [first, first + nRowTiles*nColChunks).
struct TcSlice {
  const float *rowHi, *rowLo;   // TF32 row-side residual tables: kappa (forward) / dbeta (adjoint)
  const float *colHi, *colLo;   // TF32 column-side residual tables: dbeta (forward) / kappa (adjoint)
  const float *rowX;            // [colTile][rowXStride][2] TF32 [hi, lo] anchor rows: AtabP (forward) / BtabQ (adjoint)
  const float *colX;            // [rowTile][colXStride][2] TF32 [hi, lo] anchor columns: BtabQ (forward) / AtabP (adjoint)
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
  // derivative product only (single slice, rows = samples): the reduced
  // basis of each column chunk, term-major [chunk][KFD][TV] in tile order,
  // and per sample row the reduced 2 pi kdot as [row][KF] (first KFD used)
  const float *bfT;
  const float *kd1;
  // failure detection: every wait's limit in ns (0: the 2 s default), and a
  // stage + 1 (0: none) whose operands CTA 0's loader does not fetch, so that
  // the waits for them run out
  uint64_t waitNs;
  int stallStage1, pad1;
  TcSlice s[MS];
  // slice i (a compile-time index for single-slice launches)
  __host__ __device__ __forceinline__ const TcSlice &at(int i) const { return s[MS == 1 ? 0 : i]; }
};
constexpr int kBatchSlices = 32;
static_assert(sizeof(TcParams<kBatchSlices>) <= 4096, "kernel parameter space");

// Execution plans 1-4 for the autotuner (hoe_tc_plan16.cu, hoe_tc_plan32.cu).
constexpr int kTcPlans = 5;
cudaError_t tc_launch_plan16(const hoe_handle *h, const TcParams<1> &p, int KP, int plan, int G, cudaStream_t st);
cudaError_t tc_launch_plan32(const hoe_handle *h, const TcParams<1> &p, int KP, int plan, int G, cudaStream_t st);
int tc_configure_plan16(int KP, int plan);
int tc_configure_plan32(int KP, int plan);

// The derivative product's instances and tables (hoe_tc_deriv.cu).
cudaError_t tc_launch_deriv(const hoe_handle *h, const TcParams<1> &p, int KP, int N, int KFD, int G,
                            cudaStream_t st);
int tc_configure_deriv(int KP, int N, int KFD);
cudaError_t tc_deriv_basis(const hoe_handle *h, float *bfT, float *Mdev, int *rank, int *kfd);
cudaError_t tc_deriv_kdot(const hoe_handle *h, const float *Mdev, float *kd1, cudaStream_t st);

namespace {

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
template <int N, int V = 0>
struct Tmem {
  static constexpr bool PSPLIT = N <= 64;
  static constexpr int NISS = PSPLIT ? 2 : 1;
  static constexpr int ABUF = (N <= 32 || N == 128) ? 2 : 1;
  static constexpr int ACCBUF = 1;
  static constexpr int NPART = PSPLIT ? 3 : 1;   // N-wide parts of one set
  static constexpr int ACCW = NPART * N;
  static constexpr int QOFF = 2 * N;             // issuer 1's part of a set (PSPLIT)
  static constexpr int GROUP = TcPlan<V>::GROUP ? TcPlan<V>::GROUP : (PSPLIT ? 32 : 8);
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
// Terms of the derivative factor F[s,v] = sum_l 2 pi kdot[l,s] bf[v,l]
// (nTerm <= 16, zero padded).
constexpr int KF = 16;

template <int N, int KP, int NS, int KFD = 0, int V = 0>
struct Smem {
  static constexpr int ABUF = Tmem<N, V>::ABUF;
  // Residual widths up to 16: the row tile's TF32 residual vectors (hi, lo)
  // also sit in tensor memory, 2*KP columns after the accumulators, as the A
  // operand of the residual MMAs (written by phase warps 0-3 once per row
  // tile), so that those MMAs read only the column tile from shared memory.
  static constexpr bool RT = KP <= 16;
  static constexpr int R_COLS = RT ? 2 * KP : 0;
  static constexpr int PD_CAP = (512 - Tmem<N, V>::ACC - ABUF * 2 * TV - R_COLS) / TV;
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
  // derivative product: the stage's basis tile [KF][TV] FP32 (term-major)
  static constexpr int BF_TILE = KFD * TV * 4;
  static constexpr size_t BF_OFF = XC_OFF + (size_t)NS * 2 * XC_BYTES;
  static constexpr size_t BAR_OFF = (BF_OFF + (size_t)NS * BF_TILE + 7) / 8 * 8;
  // pfull/pfree barriers: stage s uses barrier s % PB.  A parity wait for s
  // on a barrier whose previous phase (stage s - PB) were still open would
  // see the phase before that and go ahead early.  With PB >= NG that cannot
  // happen: the waiting group has already seen stage s - NG >= s - PB done,
  // and the residual tiles complete in stage order.  With PB >= PD the
  // residual issuer has seen all arrivals for stage s before it writes stage
  // s + PD, so the arrivals for s and s + PB never mix.  Three groups get
  // two barriers each (6; measured 0.7% faster than 3 at 16 coils).
  static constexpr int NG = Warps<N, V>::NG;
  static constexpr int PB = NG == 3 ? 6 : (PD > NG ? PD : NG);
  static_assert(PB >= NG && PB >= PD, "residual-tile barriers");
  static constexpr int NBAR = 2 * NS + ABUF + 10 + 2 * PB;
  static constexpr size_t MISC_OFF = BAR_OFF + (size_t)NBAR * 8;
  static constexpr size_t BYTES = MISC_OFF + 16 + 1024;  // + alignment slack
};

template <int N, int KP, int KFD = 0, int V = 0>
constexpr int pick_stages() {
  return TcPlan<V>::NS ? TcPlan<V>::NS
       : Smem<N, KP, 6, KFD, V>::BYTES <= 227 * 1024 ? 6
       : Smem<N, KP, 5, KFD, V>::BYTES <= 227 * 1024 ? 5
       : Smem<N, KP, 4, KFD, V>::BYTES <= 227 * 1024 ? 4
       : Smem<N, KP, 3, KFD, V>::BYTES <= 227 * 1024 ? 3 : 2;
}

// DERIV: the derivative product (array_operator.jl:216-218) in one pass of
// the forward: the phase warps scale e^{i phi} by 2 pi i F[s,v] before the
// BF16 split, F formed from the stage's basis tile and the row's kdot.
template <int N, int KP, int NS, int MS, int KFD = 0, int V = 0>
__global__ void __launch_bounds__(Warps<N, V>::THREADS, 1) k_tc_contract(const __grid_constant__ TcParams<MS> p) {
  constexpr bool DERIV = KFD > 0;
  static_assert(!DERIV || MS == 1, "the derivative product serves one operator per launch");
  static_assert(KFD % 2 == 0 && KFD <= KF, "derivative factor terms");
  using S = Smem<N, KP, NS, KFD, V>;
  using TM_ = Tmem<N, V>;
  constexpr int ABUF = S::ABUF, PD = S::PD, PB = S::PB, NISS = TM_::NISS;
  constexpr int ACCBUF = TM_::ACCBUF, NPART = TM_::NPART, ACCW = TM_::ACCW;
  constexpr int QOFF = TM_::QOFF, GROUP = TM_::GROUP;
  constexpr bool PSPLIT = TM_::PSPLIT;
  using W = Warps<N, V>;
  constexpr int NG = W::NG, GW = W::GW, PW = W::PW, FLW = W::FLW;
  constexpr int CISS_WARP = W::CISS, PISS_WARP = W::PISS, LOAD_WARP = W::LOAD;
  static_assert(PD >= 1, "residual-phase look-ahead");
  extern __shared__ unsigned char smem_raw[];
  unsigned char *smem = align_smem_1024(smem_raw);
  unsigned char *sB = smem + S::B_OFF;
  unsigned char *sCV = smem + S::CV_OFF;
  unsigned char *sRV = smem + S::RV_OFF;
  unsigned char *sXR = smem + S::XR_OFF;
  unsigned char *sXC = smem + S::XC_OFF;
  unsigned char *sBF = smem + S::BF_OFF;
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
  constexpr uint32_t A_COL = TM_::A_COL, P_COL = TM_::P_COL;
  constexpr uint32_t ACC_COL = P_COL + PD * TV;   // group g, issuer q: ACC_COL + (g%ACCBUF)*ACCW + q*QOFF
  constexpr bool RT = S::RT;
  constexpr uint32_t R_COL = ACC_COL + ACCBUF * ACCW;   // [hi KP | lo KP] when RT
  static_assert(R_COL + S::R_COLS <= TMEM_COLS, "tensor memory plan");
  constexpr uint32_t SBO_TF32 = (KP / 4) * 128;

  const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
  const int G = gridDim.x, b = blockIdx.x;
  const uint64_t lim = p.waitNs ? p.waitNs : kWaitNs;
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
  // anchor k-step operands, per stage slot: row side [a_hi, a_lo, 1, 1 | 0],
  // column side [1, 1, c_hi, c_lo | 0].  The constant halves and the zero
  // core-matrix columns are written here once; the loader writes the
  // [hi, lo] halves per stage.
  for (int i = threadIdx.x; i < NS * (S::XR_BYTES + S::XC_BYTES) / 16; i += W::THREADS) {
    const int nr = NS * S::XR_BYTES / 16;
    const bool isRow = i < nr;
    const int slot = isRow ? i / (S::XR_BYTES / 16) : (i - nr) / (S::XC_BYTES / 16);
    const int e = isRow ? i % (S::XR_BYTES / 16) : (i - nr) % (S::XC_BYTES / 16);
    float4 *base = isRow ? reinterpret_cast<float4 *>(sXR + (size_t)slot * 2 * S::XR_BYTES)
                         : reinterpret_cast<float4 *>(sXC + (size_t)slot * 2 * S::XC_BYTES);
    base[e] = isRow ? make_float4(0.f, 0.f, 1.f, 1.f) : make_float4(1.f, 1.f, 0.f, 0.f);
    base[(isRow ? S::XR_BYTES : S::XC_BYTES) / 16 + e] = make_float4(0.f, 0.f, 0.f, 0.f);
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
      bool got = ok && wait_bar(&segdone[gb], gr & 1, abort, p.err, lim);
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
    // derivative product: F[j] = sum_l 2 pi kdot[l, s] bf[v_j, l] for 8
    // consecutive columns v_j of the stage (basis tile bcol, term-major with
    // row stride TV, in shared memory; the row's 2 pi kdot in registers kr), as
    // packed FP32x2 FMAs over column pairs; then 2 pi i F e^{i phi} =
    // (-F sin, F cos) -> BF16 hi/lo.  Eight columns a step keep the arrays
    // of the step (phase, factor, hi, lo) in 32 registers.
    auto factor8 = [&](const float *bcol, const float *kr, float *Fv) {
      uint64_t a[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) a[i] = 0ull;   // (0.f, 0.f)
#pragma unroll
      for (int l = 0; l < KFD; ++l) {
        const uint64_t kp = pack_f32x2(kr[l], kr[l]);
        const float4 *b4 = reinterpret_cast<const float4 *>(bcol + l * TV);
#pragma unroll
        for (int q = 0; q < 2; ++q) {
          const float4 bv = b4[q];
          a[2 * q] = fma_f32x2(kp, pack_f32x2(bv.x, bv.y), a[2 * q]);
          a[2 * q + 1] = fma_f32x2(kp, pack_f32x2(bv.z, bv.w), a[2 * q + 1]);
        }
      }
#pragma unroll
      for (int i = 0; i < 4; ++i) unpack_f32x2(a[i], Fv[2 * i], Fv[2 * i + 1]);
    };
    Cursor<MS> c = c0;
    int kt = -1;   // row tiles whose residual vectors warps 0-3 wrote to TMEM
    float kreg[DERIV ? KFD : 1];   // derivative product: this row's reduced 2 pi kdot
    for (int it = 0; it < nIter && ok; ++it) {
      if (it > 0) c.next(p);
      if constexpr (DERIV) {
        if (it == 0 || c.ch == 0) {
          const float2 *k2 = reinterpret_cast<const float2 *>(p.kd1 + ((int64_t)c.rt * TM + row) * KF);
#pragma unroll
          for (int i = 0; i < KFD / 2; ++i) {
            const float2 v = __ldg(k2 + i);
            kreg[2 * i] = v.x;
            kreg[2 * i + 1] = v.y;
          }
        }
      }
      if constexpr (RT) {
        if (warp < 4 && (it == 0 || c.ch == 0)) {
          // the new row tile's residual vectors, hi and lo, from the shared
          // tile into TMEM once the previous row tile's residual MMAs are done
          ++kt;
          if ((kt > 0 && !wait_bar_warp(&rtfree[0], (kt - 1) & 1, abort, p.err, lim)) ||
              !wait_bar_warp(&rfull[kt & 1], (kt >> 1) & 1, abort, p.err, lim)) { ok = false; break; }
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
        if (!wait_bar(&pfull[pbar], pr & 1, abort, p.err, lim)) { ok = false; break; }
        // derivative product: the stage's basis tile (loaded with the stage)
        if (DERIV && !wait_bar(&full[it % NS], (it / NS) & 1, abort, p.err, lim)) { ok = false; break; }
        tc_fence_after();
        const uint32_t pBase = tmem + laneBase + P_COL + (uint32_t)(pb * TV + half * 32);
        const float *bt = reinterpret_cast<const float *>(sBF + (size_t)(it % NS) * S::BF_TILE) + half * 32;

        const int ab = it % ABUF, ar = it / ABUF;
        const uint32_t aBase = tmem + laneBase + A_COL + (uint32_t)(ab * 2 * TV + half * 32);
        // H blocks of 32 columns, 16 at a time; the residual tile is released
        // once its last 16 columns are in registers
        constexpr int H = W::WIDE ? 2 : 1;
        if constexpr (DERIV) {
          // 8 columns a step; the next step's tensor-memory load is in flight
          // while this step's factor, sin/cos and split run (the phase tile is
          // released once its last columns are in registers)
          uint32_t r[8];
          tmem_ld8_async(pBase, r);
          tmem_wait_ld(r);
#pragma unroll 1
          for (int q = 0; q < 4 * H; ++q) {
            const uint32_t ah = aBase + (uint32_t)(q * 8);
            uint32_t rn[8], hv[8], lv[8];
            float Fv[8];
            if (q + 1 < 4 * H) tmem_ld8_async(pBase + (uint32_t)((q + 1) * 8), rn);
            factor8(bt + q * 8, kreg, Fv);
#pragma unroll
            for (int j = 0; j < 8; ++j) {
              float sn, cs;
              __sincosf(__uint_as_float(r[j]), &sn, &cs);
              split_bf16x2(-Fv[j] * sn, Fv[j] * cs, hv[j], lv[j]);
            }
            if (q == 0) {
              if (ar > 0 && !wait_bar(&empty[(it - ABUF) % NS], ((it - ABUF) / NS) & 1, abort, p.err, lim)) { ok = false; break; }
              tc_fence_after();
            }
            tmem_st8(ah, hv);
            tmem_st8(ah + TV, lv);
            if (q + 1 < 4 * H) {
              tmem_wait_ld(rn);
              if (q + 2 == 4 * H) {
                tc_fence_before();
                __syncwarp();
                if (lane == 0) mbar_arrive(&pfree[pbar]);
              }
#pragma unroll
              for (int j = 0; j < 8; ++j) r[j] = rn[j];
            }
          }
        } else {
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
            if (ar > 0 && !wait_bar(&empty[(it - ABUF) % NS], ((it - ABUF) / NS) & 1, abort, p.err, lim)) { ok = false; break; }
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
              !wait_bar_warp(&tmemfree[grp % ACCBUF], ((grp / ACCBUF) - 1) & 1, abort, p.err, lim)) break;
        }
        const bool last = (it == nIter - 1) || (ch + 1 == c.C) || ((ch + 1) % GROUP == 0);
        const int slot = it % NS, round = it / NS;
        const int ab = it % ABUF, ar = it / ABUF;
        if (!wait_bar_warp(&full[slot], round & 1, abort, p.err, lim)) break;
        if (!wait_bar_warp(&afull[ab], ar & 1, abort, p.err, lim)) break;
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
        if (!wait_bar_warp(&full[s], r & 1, abort, p.err, lim)) break;
        if (!wait_bar_warp(&rfull[kj & 1], (kj >> 1) & 1, abort, p.err, lim)) break;
        if (RT && (j == 0 || c.ch == 0) && !wait_bar_warp(&rtfull[0], kj & 1, abort, p.err, lim)) break;
        const int pb = j % PD, pbar = j % PB, pr = j / PB;
        // tile buffer pb was last used by stage j - PD
        if (j >= PD && !wait_bar_warp(&pfree[(j - PD) % PB], ((j - PD) / PB) & 1, abort, p.err, lim)) break;
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
      const uint32_t stageBytes = 2 * S::B_TILE + 2 * S::CV_TILE + S::BF_TILE;
      int issued = 0, kcount = -1, rowIssued = -1;
      const int skip = b == 0 ? p.stallStage1 - 1 : -1;   // failure detection: never fetched
      // the stage's anchors as TF32 [hi, lo] pairs (8 bytes each), fetched
      // one stage ahead into registers: lane l holds rows l + 32 j of the
      // row side and columns l + 32 j of the column side
      float2 ar[TM / 32], ac[TV / 32];
      auto fetch = [&](const Cursor<MS> &cc) {
        const TcSlice &s2 = p.at(cc.si);
        const float2 *rx = reinterpret_cast<const float2 *>(s2.rowX) +
                           (int64_t)(cc.ch * TV / 128) * s2.rowXStride + (int64_t)cc.rt * TM;
        const float2 *cx = reinterpret_cast<const float2 *>(s2.colX) +
                           (int64_t)cc.rt * s2.colXStride + (int64_t)cc.ch * TV;
#pragma unroll
        for (int j = 0; j < TM / 32; ++j) ar[j] = __ldg(rx + lane + 32 * j);
#pragma unroll
        for (int j = 0; j < TV / 32; ++j) ac[j] = __ldg(cx + lane + 32 * j);
      };
      Cursor<MS> c = c0;
      if (nIter > 0) fetch(c);
      for (int it = 0; it < nIter; ++it) {
        if (it > 0) c.next(p);
        const TcSlice &sl = p.at(c.si);
        const int rt = c.rt, ch = c.ch;
        if (it == 0 || ch == 0) {
          ++kcount;
          const int rb = kcount & 1;
          if (kcount >= 2 && !wait_bar_warp(&rfree[rb], ((kcount >> 1) - 1) & 1, abort, p.err, lim)) break;
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
        if (round > 0 && !wait_bar_warp(&empty[slot], (round - 1) & 1, abort, p.err, lim)) break;
        if (it != skip) {
          // anchors into the [hi, lo] halves of the slot's 16-byte rows (row r
          // at byte 16 r, column c's pair at byte 16 c + 8), made visible to
          // the tensor cores before the stage barrier's arrival
          float2 *xr = reinterpret_cast<float2 *>(sXR + (size_t)slot * 2 * S::XR_BYTES);
          float2 *xc = reinterpret_cast<float2 *>(sXC + (size_t)slot * 2 * S::XC_BYTES);
#pragma unroll
          for (int j = 0; j < TM / 32; ++j) xr[2 * (lane + 32 * j)] = ar[j];
#pragma unroll
          for (int j = 0; j < TV / 32; ++j) xc[2 * (lane + 32 * j) + 1] = ac[j];
          asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        }
        __syncwarp();
        if (leader && it != skip) {
          const size_t co = (size_t)ch * TV * KP;
          mbar_expect_tx(&full[slot], stageBytes);
          bulk_g2s(sB + (size_t)slot * 2 * S::B_TILE, sl.Bop + (size_t)ch * 2 * (N * TK), 2 * S::B_TILE, &full[slot]);
          bulk_g2s(sCV + (size_t)slot * 2 * S::CV_TILE, sl.colHi + co, S::CV_TILE, &full[slot]);
          bulk_g2s(sCV + (size_t)slot * 2 * S::CV_TILE + S::CV_TILE, sl.colLo + co, S::CV_TILE, &full[slot]);
          if constexpr (DERIV)
            bulk_g2s(sBF + (size_t)slot * S::BF_TILE, p.bfT + (size_t)ch * KFD * TV, S::BF_TILE, &full[slot]);
        }
        __syncwarp();
        issued = it + 1;
        if (it + 1 < nIter) {
          Cursor<MS> cn = c;
          cn.next(p);
          fetch(cn);
        }
      }
      if (*abort) {
        // drain the copies still in flight into this CTA's shared memory
        for (int it = max(0, issued - NS); it < issued; ++it)
          if (it != skip) drain_bar(&full[it % NS], (it / NS) & 1);
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

// Every launch asks for at least 116 KB of shared memory, more than half of
// an SM's, so that at most one CTA is resident per SM: each CTA allocates all
// 512 tensor-memory columns.
template <int N, int KP, int KFD = 0, int V = 0>
struct Kern {
  static constexpr int NS = pick_stages<N, KP, KFD, V>();
  static_assert(Smem<N, KP, NS, KFD, V>::PD >= 1, "residual-phase look-ahead");
  using S = Smem<N, KP, NS, KFD, V>;
  static_assert(S::BYTES <= 227 * 1024, "shared memory plan exceeds 227 KB");
  static constexpr size_t LAUNCH_BYTES = S::BYTES < 116 * 1024 ? 116 * 1024 : S::BYTES;
};

template <int N, int KP, int MS, int KFD = 0, int V = 0>
cudaError_t launch_contract(const hoe_handle *h, const TcParams<MS> &p, int G, cudaStream_t st) {
  using K = Kern<N, KP, KFD, V>;
  auto kern = k_tc_contract<N, KP, K::NS, MS, KFD, V>;
  const cudaError_t e = launch_pdl(kern, dim3(G), dim3(Warps<N, V>::THREADS), K::LAUNCH_BYTES, st, p);
  h->launches += 1;
  return e;
}

// One-time per (process, instantiation): shared-memory limit; returns the
// resident CTAs per SM.
template <int N, int KP, int MS, int KFD = 0, int V = 0>
int configure() {
  using K = Kern<N, KP, KFD, V>;
  auto kern = k_tc_contract<N, KP, K::NS, MS, KFD, V>;
  if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)K::LAUNCH_BYTES) != cudaSuccess)
    return 0;
  int nb = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, kern, Warps<N, V>::THREADS, K::LAUNCH_BYTES) !=
      cudaSuccess)
    return 0;
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



// Plans 1..kTcPlans-1 of one coil width N (16 or 32) and residual width KP.
template <int N, int KP>
cudaError_t launch_plan_nk(const hoe_handle *h, const TcParams<1> &p, int plan, int G, cudaStream_t st) {
  switch (plan) {
    case 1: return launch_contract<N, KP, 1, 0, 1>(h, p, G, st);
    case 2: return launch_contract<N, KP, 1, 0, 2>(h, p, G, st);
    case 3: return launch_contract<N, KP, 1, 0, 3>(h, p, G, st);
    default: return launch_contract<N, KP, 1, 0, 4>(h, p, G, st);
  }
}
template <int N, int KP>
int configure_plan_nk(int plan) {
  switch (plan) {
    case 1: return configure<N, KP, 1, 0, 1>();
    case 2: return configure<N, KP, 1, 0, 2>();
    case 3: return configure<N, KP, 1, 0, 3>();
    default: return configure<N, KP, 1, 0, 4>();
  }
}

// The derivative product for up to 16 coils (N = 16 or 32), KFD = 6, 10 or
// 16 terms of the reduced factor.
template <int KP, int KFD>
cudaError_t launch_deriv_nk(const hoe_handle *h, const TcParams<1> &p, int N, int G, cudaStream_t st) {
  return N == 16 ? launch_contract<16, KP, 1, KFD>(h, p, G, st) : launch_contract<32, KP, 1, KFD>(h, p, G, st);
}
template <int KP, int KFD>
int configure_deriv_nk(int N) {
  return N == 16 ? configure<16, KP, 1, KFD>() : configure<32, KP, 1, KFD>();
}
}  // namespace
}  // namespace hoe
