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
// The A operand (the phase tile) never touches global memory: 16 "phase"
// warps form it in registers with the anchored FP32 phase of the plain
// engine (identical arithmetic, see hoe_internal.cuh), split it into BF16
// hi/lo and store it in shared memory in the no-swizzle K-major canonical
// layout.  A loader warp streams the pre-tiled B operand and the per-stage
// phase inputs with cp.async.bulk (TMA bulk copies) onto mbarriers; one
// thread of the MMA warp issues tcgen05.mma and commits stage completion
// back to the producers.  Every mbarrier wait is bounded in time: on
// timeout the kernel records HOE_ERR_TIMEOUT in a device word, stops
// issuing work, waits (bounded) for its own copies and MMAs and frees TMEM.
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <algorithm>
#include <cstdint>

#include "hoe_internal.cuh"

namespace hoe {
namespace {

constexpr int TM = 128;             // rows per CTA (one sample tile / one voxel tile)
constexpr int TV = 32;              // complex columns per pipeline stage
constexpr int TK = 2 * TV;          // real K per stage (64 BF16 = 4 UMMA k-steps)
constexpr int PHASE_WARPS = 16;     // four per TMEM lane quarter, a quarter of the stage's columns each
constexpr int MMA_WARP = PHASE_WARPS;
constexpr int LOAD_WARP = PHASE_WARPS + 1;
constexpr int THREADS = (PHASE_WARPS + 2) * 32;
constexpr float kTwoPi = 6.28318530717958647692f;
constexpr uint64_t kWaitNs = 2000000000ull;  // 2 s bound on any single wait

constexpr int A_TILE_BYTES = TM * TK * 2;    // one BF16 A tile (hi or lo): 16 KB
// The tensor-core FP32 accumulator sums at most GROUP chunks (GROUP*12 MMAs)
// before it is added, in round-to-nearest FP32, into register sums: long
// accumulation chains in TMEM lose accuracy on coherent sums.
constexpr int GROUP = 16;

// byte offset of element (r, k) in a no-swizzle K-major tile with K = TK:
// core matrices of 8 rows x 16 B; cores adjacent in K are 128 B apart (LBO),
// 8-row groups are (TK/8)*128 B apart (SBO)
__host__ __device__ constexpr uint32_t kmajor_off(int r, int k) {
  return (uint32_t)((r / 8) * (TK / 8) * 128 + (k / 8) * 128 + (r % 8) * 16 + (k % 8) * 2);
}
constexpr uint32_t LBO = 128;
constexpr uint32_t SBO = (TK / 8) * 128;

__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N) {
  // D = F32 (bits 4-5), A = B = BF16 (bits 7-9, 10-12), K-major, N>>3 at 17, M>>4 at 24
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ uint64_t umma_desc(uint32_t saddr) {
  return (uint64_t)((saddr & 0x3FFFF) >> 4) | ((uint64_t)(LBO >> 4) << 16) |
         ((uint64_t)(SBO >> 4) << 32) | (1ull << 46);
}

__device__ __forceinline__ uint64_t globaltimer() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      " selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// Bounded wait; returns false on timeout or when another role aborted.
__device__ __noinline__ bool wait_bar_slow(uint64_t *bar, uint32_t parity, volatile int *abort,
                                           int *gerr) {
  uint64_t t0 = 0;
  for (uint32_t n = 0;; ++n) {
    if (mbar_try_wait(bar, parity)) return true;
    if (*abort) return false;
    if ((n & 255) == 255) {
      uint64_t t = globaltimer();
      if (t0 == 0) t0 = t;
      else if (t - t0 > kWaitNs) {
        *abort = 1;
        atomicExch(gerr, HOE_ERR_TIMEOUT);
        return false;
      }
    }
  }
}

__device__ __forceinline__ bool wait_bar(uint64_t *bar, uint32_t parity, volatile int *abort,
                                         int *gerr) {
  if (mbar_try_wait(bar, parity)) return true;
  return wait_bar_slow(bar, parity, abort, gerr);
}

// Bounded wait that ignores the abort flag (used to drain in-flight work).
__device__ __noinline__ bool drain_bar(uint64_t *bar, uint32_t parity) {
  uint64_t t0 = globaltimer();
  while (!mbar_try_wait(bar, parity))
    if (globaltimer() - t0 > kWaitNs) return false;
  return true;
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count));
}
__device__ __forceinline__ void mbar_arrive(uint64_t *bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
               "r"(bytes)
               : "memory");
}
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, uint32_t bytes, uint64_t *bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}
__device__ __forceinline__ void umma(uint32_t dtmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                     uint32_t accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(dtmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate));
}
__device__ __forceinline__ void umma_commit(uint64_t *bar) {
  asm volatile(
      "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
          smem_u32(bar))
      : "memory");
}
__device__ __forceinline__ void tc_fence_before() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_after() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float *v) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
        "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ void tmem_ld4(uint32_t taddr, float *v) {
  uint32_t r[4];
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x4.b32 {%0,%1,%2,%3}, [%4];"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
               : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 4; ++i) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ void tmem_ld8(uint32_t taddr, float *v) {
  uint32_t r[8];
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
                 "=r"(r[7])
               : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 8; ++i) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ uint32_t pack_bf16(float lo_elem, float hi_elem) {
  __nv_bfloat162 v = __floats2bfloat162_rn(lo_elem, hi_elem);  // .x (low half) = lo_elem
  return *reinterpret_cast<uint32_t *>(&v);
}

struct TcParams {
  const float *rowvec;     // [nRowPad][RP]: kappa (forward) / dbeta (adjoint)
  const float *rowAnchor;  // [colTile][rowAnchorStride]: Atab (forward) / Btab (adjoint)
  const float *colvec;     // [nColPad][RP]: dbeta (forward) / kappa (adjoint)
  const float *colAnchor;  // [rowTile][colAnchorStride]: Btab (forward) / Atab (adjoint)
  const uint16_t *Bop;     // [nColChunks][hi,lo][N x TK] BF16 tiles, canonical layout
  float2 *part;            // [slot][nRowPad][nChaPad] partial sums (zeroed before launch)
  int *err;
  int rowAnchorStride, colAnchorStride;
  int nRowPad, nChaPad, nChaTC;
  int nColChunks;          // column chunks per row tile (C)
  int64_t work;            // nRowTiles * C work items, split evenly over gridDim.x CTAs
};

// CTA that owns work item w when W items are split into G contiguous ranges
// [b*W/G, (b+1)*W/G).
__host__ __device__ inline int work_owner(int64_t w, int64_t W, int G) {
  return (int)(((w + 1) * (int64_t)G - 1) / W);
}

// Shared-memory plan (dynamic, 1024-byte aligned base):
//   A    [NS][2][A_TILE_BYTES]        phase tile hi / lo
//   B    [NS][2][N*TK*2]              B operand hi / lo
//   CV   [NS][TV][RP] float           column phase vectors
//   CA   [NS][TV] float               column anchors
//   bars full[NS], afull[NS], empty[NS], segdone[2], tmemfree[2]; tmem base; abort flag
template <int N, int RP, int NS>
struct Smem {
  static constexpr int B_TILE = N * TK * 2;
  static constexpr size_t A_OFF = 0;
  static constexpr size_t B_OFF = A_OFF + (size_t)NS * 2 * A_TILE_BYTES;
  static constexpr size_t CV_OFF = B_OFF + (size_t)NS * 2 * B_TILE;
  static constexpr size_t CA_OFF = CV_OFF + (size_t)NS * TV * RP * 4;
  static constexpr size_t BAR_OFF = (CA_OFF + (size_t)NS * TV * 4 + 7) / 8 * 8;
  static constexpr size_t MISC_OFF = BAR_OFF + (size_t)(3 * NS + 4) * 8;
  static constexpr size_t BYTES = MISC_OFF + 16 + 1024;  // + alignment slack
};

template <int N, int RP, int NS>
__global__ void __launch_bounds__(THREADS, 1) k_tc_contract(TcParams p) {
  using S = Smem<N, RP, NS>;
  extern __shared__ unsigned char smem_raw[];
  unsigned char *smem = (unsigned char *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  unsigned char *sA = smem + S::A_OFF;
  unsigned char *sB = smem + S::B_OFF;
  float *sCV = reinterpret_cast<float *>(smem + S::CV_OFF);
  float *sCA = reinterpret_cast<float *>(smem + S::CA_OFF);
  uint64_t *full = reinterpret_cast<uint64_t *>(smem + S::BAR_OFF);
  uint64_t *afull = full + NS;
  uint64_t *empty = afull + NS;
  uint64_t *segdone = empty + NS;   // [2]: accumulator buffer b complete (group of chunks)
  uint64_t *tmemfree = segdone + 2; // [2]: accumulator buffer b read out
  uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(smem + S::MISC_OFF);
  volatile int *abort = reinterpret_cast<volatile int *>(smem + S::MISC_OFF + 8);
  // two accumulator buffers of N FP32 columns
  constexpr uint32_t TMEM_COLS = 2 * N <= 32 ? 32 : (2 * N <= 64 ? 64 : (2 * N <= 128 ? 128 : 256));

  const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
  const int C = p.nColChunks;
  const int G = gridDim.x, b = blockIdx.x;
  const int64_t wb = (int64_t)b * p.work / G, we = (int64_t)(b + 1) * p.work / G;
  const int nIter = (int)(we - wb);

  if (threadIdx.x == 0) {
    for (int i = 0; i < NS; ++i) {
      mbar_init(&full[i], 1);
      mbar_init(&afull[i], PHASE_WARPS);
      mbar_init(&empty[i], 1);
    }
    for (int i = 0; i < 2; ++i) {
      mbar_init(&segdone[i], 1);
      mbar_init(&tmemfree[i], PHASE_WARPS);
    }
    *abort = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == MMA_WARP) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(tmem_slot)),
                 "r"(TMEM_COLS));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;

  // Work item w = (row tile w / C, chunk w % C).  A "group" is a run of at
  // most GROUP consecutive chunks of one row tile; group g accumulates into
  // TMEM buffer g & 1.
  // first (row tile, chunk) of this CTA; later items advance incrementally
  const int rt0 = (int)(wb / C), ch0 = (int)(wb % C);
  if (warp < PHASE_WARPS) {
    // ---------------- phase generator: rows x (a quarter of the stage's columns).
    // After the first stage of group g+1 (or at the end) all 16 warps add
    // group g's accumulator into register sums (columns split by warp
    // quarter) and, at the end of a row tile, write the sums to the partial slot.
    const int row = (warp & 3) * 32 + lane;
    const int qcol = warp >> 2;
    constexpr int NA = N / 4;  // accumulator columns owned by this thread
    float acc[NA];
#pragma unroll
    for (int i = 0; i < NA; ++i) acc[i] = 0.f;
    float rv[RP];
    int curRT = -1, curTile = -1, grp = -1, grow = 0;
    int pendGrp = -1, pendRT = -1;
    bool pendLast = false;
    float a = 0.f;
    bool ok = true;
    auto flush = [&]() {
      // add group pendGrp into acc; write acc out if it closed its row tile
      const int g = pendGrp;
      bool got = ok && wait_bar(&segdone[g & 1], (g >> 1) & 1, abort, p.err);
      tc_fence_after();
      if (got) {
        const uint32_t base = tmem + ((uint32_t)((warp & 3) * 32) << 16) + (uint32_t)((g & 1) * N + qcol * NA);
        if constexpr (NA % 16 == 0) {
#pragma unroll
          for (int c0 = 0; c0 < NA; c0 += 16) {
            float v[16];
            tmem_ld16(base + c0, v);
#pragma unroll
            for (int i = 0; i < 16; ++i) acc[c0 + i] += v[i];
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
      tc_fence_before();
      __syncwarp();
      if (lane == 0) mbar_arrive(&tmemfree[g & 1]);
      if (pendLast) {
        const int slot = b - work_owner((int64_t)pendRT * C, p.work, G);
        float2 *dst = p.part + ((int64_t)slot * p.nRowPad + (int64_t)pendRT * TM + row) * p.nChaPad;
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
    int rt = rt0, ch = ch0;
    // anchor phase of the next anchor tile, loaded one stage ahead
    float aNext = nIter > 0
        ? p.rowAnchor[(int64_t)(ch0 * TV / 128) * p.rowAnchorStride + rt0 * TM + row] : 0.f;
    for (int it = 0; it < nIter && ok; ++it, ++ch) {
      if (ch == C) { ch = 0; ++rt; }
      if (it == 0 || ch % GROUP == 0) ++grp;
      if (rt != curRT) {
        curRT = rt;
        curTile = -1;
        grow = rt * TM + row;
#pragma unroll
        for (int l = 0; l < RP; l += 4) {
          float4 v = *reinterpret_cast<const float4 *>(p.rowvec + (int64_t)grow * RP + l);
          rv[l] = v.x; rv[l + 1] = v.y; rv[l + 2] = v.z; rv[l + 3] = v.w;
        }
      }
      const int slot = it % NS, round = it / NS;
      const int col0 = ch * TV;
      const int colTile = col0 / 128;
      if (colTile != curTile) {
        a = aNext;
        curTile = colTile;
      }
      {
        int nch = ch + 1, nrt = rt;
        if (nch == C) { nch = 0; ++nrt; }
        if (it + 1 < nIter && (nrt != rt || nch * TV / 128 != colTile))
          aNext = p.rowAnchor[(int64_t)(nch * TV / 128) * p.rowAnchorStride + nrt * TM + row];
      }
      if (round > 0 && !wait_bar(&empty[slot], (round - 1) & 1, abort, p.err)) { ok = false; break; }
      if (!wait_bar(&full[slot], round & 1, abort, p.err)) { ok = false; break; }
      const float *cv = sCV + slot * TV * RP;
      const float *ca = sCA + slot * TV;
      unsigned char *aHi = sA + (size_t)slot * 2 * A_TILE_BYTES;
      unsigned char *aLo = aHi + A_TILE_BYTES;
#pragma unroll 1
      for (int cc = 0; cc < 2; ++cc) {
        const int v0 = qcol * 8 + cc * 4;
        const float4 c4 = *reinterpret_cast<const float4 *>(ca + v0);
        float ph[4] = {a + c4.x, a + c4.y, a + c4.z, a + c4.w};
#pragma unroll
        for (int q = 0; q < RP / 4; ++q) {
#pragma unroll
          for (int j = 0; j < 4; ++j) {
            float4 d = reinterpret_cast<const float4 *>(cv + (v0 + j) * RP)[q];
            ph[j] = fmaf(rv[4 * q], d.x, ph[j]);
            ph[j] = fmaf(rv[4 * q + 1], d.y, ph[j]);
            ph[j] = fmaf(rv[4 * q + 2], d.z, ph[j]);
            ph[j] = fmaf(rv[4 * q + 3], d.w, ph[j]);
          }
        }
        uint32_t hi[4], lo[4];
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          float f = ph[j] - rintf(ph[j]);
          float sn, cs;
          __sincosf(kTwoPi * f, &sn, &cs);
          __nv_bfloat162 h = __floats2bfloat162_rn(cs, sn);
          float2 hf = __bfloat1622float2(h);
          hi[j] = *reinterpret_cast<uint32_t *>(&h);
          lo[j] = pack_bf16(cs - hf.x, sn - hf.y);
        }
        const uint32_t off = kmajor_off(row, 2 * v0);
        *reinterpret_cast<uint4 *>(aHi + off) = make_uint4(hi[0], hi[1], hi[2], hi[3]);
        *reinterpret_cast<uint4 *>(aLo + off) = make_uint4(lo[0], lo[1], lo[2], lo[3]);
      }
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      __syncwarp();
      if (lane == 0) mbar_arrive(&afull[slot]);
      // the previous group is flushed one stage late, so its MMAs are done by now
      if (pendGrp >= 0) flush();
      const bool endRT = (it == nIter - 1) || (ch + 1 == C);
      if (endRT || (ch + 1) % GROUP == 0) {
        pendGrp = grp;
        pendRT = rt;
        pendLast = endRT;
      }
    }
    if (pendGrp >= 0) flush();
  } else if (warp == MMA_WARP) {
    // ---------------- MMA issuer (one thread)
    if (lane == 0 && nIter > 0) {
      constexpr uint32_t idesc = idesc_bf16(TM, N);
      int issued = 0, grp = -1;
      int ch = ch0;
      for (int it = 0; it < nIter; ++it, ++ch) {
        if (ch == C) ch = 0;
        const bool first = (it == 0) || (ch % GROUP == 0);
        if (first) {
          ++grp;
          // buffer grp&1 was last used by group grp-2: wait until it was read out
          if (grp >= 2 && !wait_bar(&tmemfree[grp & 1], ((grp >> 1) - 1) & 1, abort, p.err)) break;
        }
        const bool last = (it == nIter - 1) || (ch + 1 == C) || ((ch + 1) % GROUP == 0);
        const int slot = it % NS, round = it / NS;
        if (!wait_bar(&full[slot], round & 1, abort, p.err)) break;
        if (!wait_bar(&afull[slot], round & 1, abort, p.err)) break;
        tc_fence_after();
        const uint32_t dt = tmem + (uint32_t)((grp & 1) * N);
        const uint32_t aHi = smem_u32(sA + (size_t)slot * 2 * A_TILE_BYTES);
        const uint32_t aLo = aHi + A_TILE_BYTES;
        const uint32_t bHi = smem_u32(sB + (size_t)slot * 2 * S::B_TILE);
        const uint32_t bLo = bHi + S::B_TILE;
#pragma unroll
        for (int ks = 0; ks < TK / 16; ++ks) {
          const uint32_t ko = ks * 2 * LBO;  // 16 BF16 = two core matrices along K
          umma(dt, umma_desc(aHi + ko), umma_desc(bHi + ko), idesc, (first && ks == 0) ? 0u : 1u);
          umma(dt, umma_desc(aHi + ko), umma_desc(bLo + ko), idesc, 1u);
          umma(dt, umma_desc(aLo + ko), umma_desc(bHi + ko), idesc, 1u);
        }
        umma_commit(&empty[slot]);
        if (last) umma_commit(&segdone[grp & 1]);
        issued = it + 1;
      }
      if (issued != nIter && issued > 0) {
        // aborted: let the MMAs already issued finish before TMEM is freed
        const int lastIt = issued - 1;
        drain_bar(&empty[lastIt % NS], (lastIt / NS) & 1);
      }
    }
    __syncwarp();
  } else {
    // ---------------- loader (one thread): B tiles + column phase inputs
    if (lane == 0) {
      const uint32_t bBytes = 2 * S::B_TILE, cvBytes = TV * RP * 4, caBytes = TV * 4;
      int issued = 0;
      int rt = rt0, ch = ch0;
      for (int it = 0; it < nIter; ++it, ++ch) {
        if (ch == C) { ch = 0; ++rt; }
        const int slot = it % NS, round = it / NS;
        if (round > 0 && !wait_bar(&empty[slot], (round - 1) & 1, abort, p.err)) break;
        const int col0 = ch * TV;
        mbar_expect_tx(&full[slot], bBytes + cvBytes + caBytes);
        bulk_g2s(sB + (size_t)slot * 2 * S::B_TILE, p.Bop + (size_t)ch * 2 * (N * TK), bBytes, &full[slot]);
        bulk_g2s(sCV + slot * TV * RP, p.colvec + (size_t)col0 * RP, cvBytes, &full[slot]);
        bulk_g2s(sCA + slot * TV, p.colAnchor + (int64_t)rt * p.colAnchorStride + col0, caBytes,
                 &full[slot]);
        issued = it + 1;
      }
      if (*abort) {
        // drain the copies still in flight into this CTA's shared memory
        for (int it = max(0, issued - NS); it < issued; ++it)
          drain_bar(&full[it % NS], (it / NS) & 1);
      }
    }
    __syncwarp();
  }

  tc_fence_before();
  __syncthreads();
  if (warp == MMA_WARP) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TMEM_COLS));
  }
}

// B operand of the forward: chunk i covers voxels [i*TV, (i+1)*TV); element
// (n, k) with k = 2*v_local + r and n = 2*c + q.
__global__ void k_tc_bop_forward(const float2 *__restrict__ Z, uint16_t *__restrict__ Bop,
                                 int nChunks, int N, int nChaPad) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  int64_t per = (int64_t)N * TK;
  if (i >= (int64_t)nChunks * per) return;
  int ch = (int)(i / per), e = (int)(i % per);
  int n = e / TK, k = e % TK;
  int v = ch * TV + k / 2, r = k & 1, c = n / 2, q = n & 1;
  float2 z = c < nChaPad ? Z[(int64_t)v * nChaPad + c] : make_float2(0.f, 0.f);
  float val = r == 0 ? (q == 0 ? z.x : z.y) : (q == 0 ? -z.y : z.x);
  __nv_bfloat16 h = __float2bfloat16_rn(val);
  __nv_bfloat16 l = __float2bfloat16_rn(val - __bfloat162float(h));
  uint16_t *tile = Bop + (size_t)ch * 2 * per;
  uint32_t o = kmajor_off(n, k) / 2;
  tile[o] = *reinterpret_cast<uint16_t *>(&h);
  tile[per + o] = *reinterpret_cast<uint16_t *>(&l);
}

// B operand of the adjoint from Yt [nSamPad][nChaPad]: chunk i covers
// samples [i*TV, (i+1)*TV).
__global__ void k_tc_bop_adjoint(const float2 *__restrict__ Yt, uint16_t *__restrict__ Bop,
                                 int nChunks, int N, int nChaPad) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  int64_t per = (int64_t)N * TK;
  if (i >= (int64_t)nChunks * per) return;
  int ch = (int)(i / per), e = (int)(i % per);
  int n = e / TK, k = e % TK;
  int s = ch * TV + k / 2, r = k & 1, c = n / 2, q = n & 1;
  float2 y = c < nChaPad ? Yt[(int64_t)s * nChaPad + c] : make_float2(0.f, 0.f);
  float val = r == 0 ? (q == 0 ? y.x : y.y) : (q == 0 ? y.y : -y.x);
  __nv_bfloat16 h = __float2bfloat16_rn(val);
  __nv_bfloat16 l = __float2bfloat16_rn(val - __bfloat162float(h));
  uint16_t *tile = Bop + (size_t)ch * 2 * per;
  uint32_t o = kmajor_off(n, k) / 2;
  tile[o] = *reinterpret_cast<uint16_t *>(&h);
  tile[per + o] = *reinterpret_cast<uint16_t *>(&l);
}

int tc_ncha(int nCha) {
  int n = 8;
  while (n < nCha) n *= 2;
  return n;  // 8, 16, 32 or 64 coils per MMA: N = 16, 32, 64, 128
}

template <int N, int RP>
struct Kern {
  static constexpr int NS = N <= 64 ? 4 : 3;
  using S = Smem<N, RP, NS>;
  static_assert(S::BYTES <= 227 * 1024, "shared memory plan exceeds 227 KB");
  static void *fn() { return (void *)k_tc_contract<N, RP, NS>; }
};

template <int N, int RP>
cudaError_t launch_contract(const hoe_handle *h, const TcParams &p, int G, cudaStream_t st) {
  using K = Kern<N, RP>;
  auto kern = k_tc_contract<N, RP, K::NS>;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)K::S::BYTES);
  if (e != cudaSuccess) return e;
  kern<<<G, THREADS, K::S::BYTES, st>>>(p);
  h->launches += 1;
  return cudaGetLastError();
}

// resident CTAs per SM of the instantiation for (N, RP)
template <int N, int RP>
int blocks_per_sm() {
  using K = Kern<N, RP>;
  auto kern = k_tc_contract<N, RP, K::NS>;
  if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)K::S::BYTES) != cudaSuccess)
    return 1;
  int nb = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, kern, THREADS, K::S::BYTES) != cudaSuccess || nb < 1)
    nb = 1;
  return nb;
}


template <int RP>
cudaError_t dispatch_n(const hoe_handle *h, const TcParams &p, int N, int G, cudaStream_t st) {
  switch (N) {
    case 16: return launch_contract<16, RP>(h, p, G, st);
    case 32: return launch_contract<32, RP>(h, p, G, st);
    case 64: return launch_contract<64, RP>(h, p, G, st);
    default: return launch_contract<128, RP>(h, p, G, st);
  }
}

cudaError_t dispatch(const hoe_handle *h, const TcParams &p, int N, int G, cudaStream_t st) {
  switch (h->t.Rp) {
    case 8: return dispatch_n<8>(h, p, N, G, st);
    case 12: return dispatch_n<12>(h, p, N, G, st);
    case 16: return dispatch_n<16>(h, p, N, G, st);
    default: return dispatch_n<24>(h, p, N, G, st);
  }
}

template <int RP>
int bps_n(int N) {
  switch (N) {
    case 16: return blocks_per_sm<16, RP>();
    case 32: return blocks_per_sm<32, RP>();
    case 64: return blocks_per_sm<64, RP>();
    default: return blocks_per_sm<128, RP>();
  }
}

int bps(int Rp, int N) {
  switch (Rp) {
    case 8: return bps_n<8>(N);
    case 12: return bps_n<12>(N);
    case 16: return bps_n<16>(N);
    default: return bps_n<24>(N);
  }
}

// Largest number of CTAs that share one row tile when rowTiles*C work items
// are split evenly over G CTAs.
int max_slots(int rowTiles, int C, int G) {
  const int64_t W = (int64_t)rowTiles * C;
  int J = 1;
  for (int r = 0; r < rowTiles; ++r) {
    int b0 = work_owner((int64_t)r * C, W, G), b1 = work_owner((int64_t)(r + 1) * C - 1, W, G);
    J = std::max(J, b1 - b0 + 1);
  }
  return J;
}

struct TcBuffers {
  uint16_t *bopF = nullptr, *bopA = nullptr;
  float2 *part = nullptr;
  int *err = nullptr;
  int N = 0, nChaTC = 0;
  int gridF = 1, gridA = 1, slotsF = 1, slotsA = 1;
  size_t bopFElems = 0, bopAElems = 0, partElems = 0;
};

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
  return true;
}

cudaError_t tc_prepare(hoe_handle *h) {
  if (h->tc.ready) return cudaSuccess;
  const auto &t = h->t;
  TcBuffers b;
  b.nChaTC = tc_ncha(t.nCha);
  b.N = 2 * b.nChaTC;
  const int chunksF = t.nVoxPad / TV, chunksA = t.nSamPad / TV;
  const int G = h->numSMs * bps(t.Rp, b.N);
  b.gridF = (int)std::min<int64_t>(G, (int64_t)t.nSt * chunksF);
  b.gridA = (int)std::min<int64_t>(G, (int64_t)t.nVt * chunksA);
  b.slotsF = max_slots(t.nSt, chunksF, b.gridF);
  b.slotsA = max_slots(t.nVt, chunksA, b.gridA);
  b.bopFElems = (size_t)chunksF * 2 * b.N * TK;
  b.bopAElems = (size_t)chunksA * 2 * b.N * TK;
  b.partElems = std::max((size_t)b.slotsF * t.nSamPad, (size_t)b.slotsA * t.nVoxPad) * t.nChaPad;
  size_t bytes = b.bopFElems * 2 + 256 + b.bopAElems * 2 + 256 + b.partElems * sizeof(float2) + 256 + 256;
  unsigned char *buf = nullptr;
  cudaError_t e = cudaMalloc(&buf, bytes);
  if (e != cudaSuccess) return e;
  size_t off = 0;
  auto take = [&](size_t n) { unsigned char *p = buf + off; off = (off + n + 255) / 256 * 256; return p; };
  b.bopF = (uint16_t *)take(b.bopFElems * 2);
  b.bopA = (uint16_t *)take(b.bopAElems * 2);
  b.part = (float2 *)take(b.partElems * sizeof(float2));
  b.err = (int *)take(sizeof(int));
  e = cudaMemset(b.err, 0, sizeof(int));
  if (e != cudaSuccess) { cudaFree(buf); return e; }
  h->tc.buf = buf;
  h->tc.bytes = bytes;
  h->tc.ready = true;
  h->tc_host = new TcBuffers(b);
  return cudaSuccess;
}

void tc_release(hoe_handle *h) {
  if (h->tc.buf) cudaFree(h->tc.buf);
  delete (TcBuffers *)h->tc_host;
  h->tc_host = nullptr;
  h->tc = TcState();
}

static TcParams base_params(const hoe_handle *h, const TcBuffers &b) {
  TcParams p{};
  p.part = b.part;
  p.err = b.err;
  p.nChaPad = h->t.nChaPad;
  p.nChaTC = b.nChaTC;
  return p;
}

cudaError_t tc_forward(const hoe_handle *h, const float2 *, float2 *y, const float *D, int mode,
                       cudaStream_t st) {
  const auto &t = h->t;
  const TcBuffers &b = *(const TcBuffers *)h->tc_host;
  const int chunks = t.nVoxPad / TV;
  int64_t n = (int64_t)chunks * b.N * TK;
  k_tc_bop_forward<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(h->s.Z, b.bopF, chunks, b.N, t.nChaPad);
  h->launches += 1;
  TcParams p = base_params(h, b);
  p.rowvec = t.kappa;
  p.rowAnchor = t.Atab;
  p.rowAnchorStride = t.nSamPad;
  p.colvec = t.dbeta;
  p.colAnchor = t.Btab;
  p.colAnchorStride = t.nVoxPad;
  p.Bop = b.bopF;
  p.nRowPad = t.nSamPad;
  p.nColChunks = chunks;
  p.work = (int64_t)t.nSt * chunks;
  cudaError_t e = cudaMemsetAsync(b.part, 0, (size_t)b.slotsF * t.nSamPad * t.nChaPad * sizeof(float2), st);
  if (e != cudaSuccess) return e;
  trace(h, EV_FK0, st);
  e = dispatch(h, p, b.N, b.gridF, st);
  trace(h, EV_FK1, st);
  if (e != cudaSuccess) return e;
  return simt_reduce_forward(h, b.part, b.slotsF, y, D, mode, st);
}

cudaError_t tc_adjoint_from_Yt(const hoe_handle *h, float2 *x, cudaStream_t st) {
  const auto &t = h->t;
  const TcBuffers &b = *(const TcBuffers *)h->tc_host;
  const int chunks = t.nSamPad / TV;
  int64_t n = (int64_t)chunks * b.N * TK;
  k_tc_bop_adjoint<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(h->s.Yt, b.bopA, chunks, b.N, t.nChaPad);
  h->launches += 1;
  TcParams p = base_params(h, b);
  p.rowvec = t.dbeta;
  p.rowAnchor = t.Btab;
  p.rowAnchorStride = t.nVoxPad;
  p.colvec = t.kappa;
  p.colAnchor = t.Atab;
  p.colAnchorStride = t.nSamPad;
  p.Bop = b.bopA;
  p.nRowPad = t.nVoxPad;
  p.nColChunks = chunks;
  p.work = (int64_t)t.nVt * chunks;
  cudaError_t e = cudaMemsetAsync(b.part, 0, (size_t)b.slotsA * t.nVoxPad * t.nChaPad * sizeof(float2), st);
  if (e != cudaSuccess) return e;
  trace(h, EV_AK0, st);
  e = dispatch(h, p, b.N, b.gridA, st);
  trace(h, EV_AK1, st);
  if (e != cudaSuccess) return e;
  return simt_reduce_adjoint(h, b.part, b.slotsA, x, st);
}

int *tc_error_word(const hoe_handle *h) {
  return h->tc_host ? ((const TcBuffers *)h->tc_host)->err : nullptr;
}

}  // namespace hoe
