// hoe_tcgen05.cuh — tcgen05 building blocks shared by the tensor-core
// kernels (hoe_tc.cu: forward/adjoint contraction, hoe_tc_bwd.cu: backward):
// tile shapes, UMMA descriptors and no-swizzle K-major layouts, bounded
// mbarrier waits, bulk copies, MMA and tensor-memory wrappers, the even split
// of work items over CTAs and the engine's per-operator device buffers.
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <algorithm>
#include <cstdint>

#include "hoe_internal.cuh"

namespace hoe {

// Device buffers of the tensor-core engine for one operator (tc_prepare).
struct TcBuffers {
  uint16_t *bopF = nullptr, *bopA = nullptr;
  float *AtabP = nullptr, *BtabQ = nullptr;   // anchors in radians, TF32 [hi, lo] pairs
  float2 *part = nullptr;
  int *err = nullptr;
  int N = 0, nChaTC = 0;
  int plan = 0;                               // execution plan of the contraction (TcPlan)
  // failure detection test: the next forward contraction stalls CTA 0 at
  // this stage + 1 (0: none) with 1 ms waits; set from HOE_INJECT_TC_STALL
  // when the engine is prepared, cleared after one launch
  mutable int injectStall1 = 0;
  int gridF = 1, gridA = 1, slotsF = 1, slotsA = 1;
  size_t bopFElems = 0, bopAElems = 0, partElems = 0;
  // derivative product (kspha_dt mode), allocated on first use.  Up to 16
  // coils one pass (fusedD): basis tiles bfT and 2 pi kdot per sample kd1; above, the
  // 128-wide B operand of 64 virtual coils and its partial slots per pass
  uint16_t *bopD = nullptr;
  float2 *partD = nullptr;
  float *bfT = nullptr;
  float *kd1 = nullptr;
  float *Md = nullptr;      // reduced-basis rotation [KF x KF] of the one-pass path
  int rankD = 0, kfD = 16;  // its rank and the kernel's term count (6, 10 or 16)
  bool fusedD = false;
  void *memD = nullptr;
  size_t bytesD = 0;
  int gridD = 1, slotsD = 1;
};

namespace {

constexpr int TM = 128;             // rows per CTA (one sample tile / one voxel tile)
constexpr int TV = 64;              // complex columns per pipeline stage
constexpr int TK = 2 * TV;          // real K per stage (128 BF16 = 8 UMMA k-steps)

// Phase warps of the backward kernel and of the forward/adjoint kernel above
// 16 coils: two groups of 8 take alternate stages (group = warp >> 3), so one
// group's barrier and tensor-memory latencies overlap the other's
// arithmetic; within a group a warp covers one TMEM lane quarter (warp & 3)
// and half of the stage's columns ((warp >> 2) & 1).  (Up to 16 coils the
// forward/adjoint kernel uses three groups of 4: Warps<N> in hoe_tc.cu.)
constexpr int PHASE_WARPS = 16;
constexpr int GROUP_WARPS = PHASE_WARPS / 2;
constexpr uint64_t kWaitNs = 2000000000ull;  // 2 s bound on any single wait

// byte offset of element (r, k) in a no-swizzle K-major tile with K = TK:
// core matrices of 8 rows x 16 B; cores adjacent in K are 128 B apart (LBO),
// 8-row groups are (TK/8)*128 B apart (SBO)
__host__ __device__ constexpr uint32_t kmajor_off(int r, int k) {
  return (uint32_t)((r / 8) * (TK / 8) * 128 + (k / 8) * 128 + (r % 8) * 16 + (k % 8) * 2);
}
constexpr uint32_t LBO = 128;                 // K-direction core stride (all tiles)
constexpr uint32_t SBO = (TK / 8) * 128;      // 8-row group stride of the BF16 tiles

__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N) {
  // D = F32 (bits 4-5), A = B = BF16 (bits 7-9, 10-12), K-major, N>>3 at 17, M>>4 at 24
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

// The dynamic shared-memory base rounded up to 1024 bytes by pointer
// arithmetic on the shared array itself.  The compiler then keeps the shared
// address space for every pointer derived from it; rounding through an
// integer yields a generic pointer, and each access through that becomes a
// generic load or store (tracked like a global access, with its latency).
__device__ __forceinline__ unsigned char *align_smem_1024(unsigned char *raw) {
  return raw + ((1024u - (smem_u32(raw) & 1023u)) & 1023u);
}

__host__ __device__ constexpr uint32_t idesc_tf32(int M, int N) {
  // D = F32, A = B = TF32 (2 at bits 7-9, 10-12), K-major, N>>3 at 17, M>>4 at 24
  return (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

// Shared-memory matrix descriptor, no swizzle: start address, LBO (K step of
// core matrices), SBO (step of 8-row groups), descriptor version 1.
__device__ __forceinline__ uint64_t umma_desc(uint32_t saddr, uint32_t sbo = SBO, uint32_t lbo = LBO) {
  return (uint64_t)((saddr & 0x3FFFF) >> 4) | ((uint64_t)(lbo >> 4) << 16) |
         ((uint64_t)(sbo >> 4) << 32) | (1ull << 46);
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

// try_wait with a suspend-time hint: a waiting thread sleeps until the phase
// completes (or the hint elapses) instead of spinning on issue slots.
constexpr uint32_t kSuspendNs = 200000;
__device__ __forceinline__ bool mbar_try_wait_sleep(uint64_t *bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n"
      " selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity), "r"(kSuspendNs)
      : "memory");
  return ok != 0;
}

// Bounded wait (at most lim ns); returns false on timeout or when another
// role aborted.
__device__ __noinline__ bool wait_bar_slow(uint64_t *bar, uint32_t parity, volatile int *abort,
                                           int *gerr, uint64_t lim = kWaitNs) {
  const uint64_t t0 = globaltimer();
  for (;;) {
    if (mbar_try_wait_sleep(bar, parity)) return true;
    if (*abort) return false;
    if (globaltimer() - t0 > lim) {
      *abort = 1;
      atomicExch(gerr, HOE_ERR_TIMEOUT);
      return false;
    }
  }
}

__device__ __forceinline__ bool wait_bar(uint64_t *bar, uint32_t parity, volatile int *abort,
                                         int *gerr, uint64_t lim = kWaitNs) {
  if (mbar_try_wait(bar, parity)) return true;
  return wait_bar_slow(bar, parity, abort, gerr, lim);
}

// Bounded wait made by every lane of a converged warp; the result is the same
// in all lanes (any lane's failure counts), so the warp stays converged.
__device__ __forceinline__ bool wait_bar_warp(uint64_t *bar, uint32_t parity, volatile int *abort, int *gerr,
                                              uint64_t lim = kWaitNs) {
  return __all_sync(0xffffffffu, wait_bar(bar, parity, abort, gerr, lim));
}

// One lane of a converged warp (elect.sync).  MMA issuers run their loop with
// the whole warp and let the elected lane issue: issuing back to back from a
// lone active lane costs ~83 cycles per tcgen05.mma, from an elected lane of
// a converged warp ~32 (measured on GB300).
__device__ __forceinline__ bool elect_one() {
  uint32_t pred = 0;
  asm volatile(
      "{\n .reg .pred p;\n .reg .b32 r;\n elect.sync r|p, 0xffffffff;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(pred));
  return pred != 0;
}

// Bounded wait that ignores the abort flag (used to drain in-flight work).
__device__ __noinline__ bool drain_bar(uint64_t *bar, uint32_t parity) {
  uint64_t t0 = globaltimer();
  while (!mbar_try_wait_sleep(bar, parity))
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
__device__ __forceinline__ void umma_tf32(uint32_t dtmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                          uint32_t accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}\n" ::"r"(dtmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate));
}
// D += A(TMEM) * B(SMEM)^T, kind::f16
__device__ __forceinline__ void umma_ta(uint32_t dtmem, uint32_t atmem, uint64_t bdesc, uint32_t idesc,
                                        uint32_t accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], [%1], %2, %3, p;\n}\n" ::"r"(dtmem),
      "r"(atmem), "l"(bdesc), "r"(idesc), "r"(accumulate));
}
__device__ __forceinline__ void tmem_st16(uint32_t taddr, const uint32_t *w) {
  asm volatile(
      "tcgen05.st.sync.aligned.32x32b.x16.b32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16};" ::"r"(
          taddr),
      "r"(w[0]), "r"(w[1]), "r"(w[2]), "r"(w[3]), "r"(w[4]), "r"(w[5]), "r"(w[6]), "r"(w[7]), "r"(w[8]),
      "r"(w[9]), "r"(w[10]), "r"(w[11]), "r"(w[12]), "r"(w[13]), "r"(w[14]), "r"(w[15])
      : "memory");
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

// 16 columns into registers without waiting: call tmem_wait_ld(r) before use.
__device__ __forceinline__ void tmem_ld16_async(uint32_t taddr, uint32_t *r) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
}
// Wait for this thread's tensor-memory loads, then pass each destination
// register through an empty asm after the wait: the registers are outputs of
// the load's asm, so without this the compiler could move arithmetic on them
// (which is not a memory access) above the wait.  Costs no instruction.
template <int K>
__device__ __forceinline__ void tmem_wait_ld(uint32_t (&r)[K]) {
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < K; ++i) asm volatile("" : "+r"(r[i]));
}
template <int K1, int K2>
__device__ __forceinline__ void tmem_wait_ld(uint32_t (&a)[K1], uint32_t (&b)[K2]) {
  tmem_wait_ld(a);
#pragma unroll
  for (int i = 0; i < K2; ++i) asm volatile("" : "+r"(b[i]));
}
// 8 columns into registers without waiting: call tmem_wait_ld(r) before use.
__device__ __forceinline__ void tmem_ld8_async(uint32_t taddr, uint32_t *r) {
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
               : "r"(taddr));
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

// Two FP32 values -> BF16 hi pair (round to nearest) and BF16 lo pair of the
// residuals (a - hi(a), b - hi(b)).  A BF16 value is the upper half of the FP32
// with the same value, so the hi parts are unpacked with a shift and a mask;
// both residuals come from one packed FP32x2 subtraction.
__device__ __forceinline__ void split_bf16x2(float a, float b, uint32_t &hi, uint32_t &lo) {
  __nv_bfloat162 h = __floats2bfloat162_rn(a, b);  // .x (low half) = a
  const uint32_t hb = *reinterpret_cast<uint32_t *>(&h);
  uint64_t v, u, d;
  asm("mov.b64 %0, {%1, %2};" : "=l"(v) : "f"(a), "f"(b));
  asm("mov.b64 %0, {%1, %2};" : "=l"(u) : "r"(hb << 16), "r"(hb & 0xffff0000u));
  asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(v), "l"(u));
  float ra, rb;
  asm("mov.b64 {%0, %1}, %2;" : "=f"(ra), "=f"(rb) : "l"(d));
  hi = hb;
  lo = pack_bf16(ra, rb);
}

// Packed FP32x2 arithmetic (two lanes of one 64-bit register pair).
__device__ __forceinline__ uint64_t pack_f32x2(float a, float b) {
  uint64_t v;
  asm("mov.b64 %0, {%1, %2};" : "=l"(v) : "f"(a), "f"(b));
  return v;
}
__device__ __forceinline__ void unpack_f32x2(uint64_t v, float &a, float &b) {
  asm("mov.b64 {%0, %1}, %2;" : "=f"(a), "=f"(b) : "l"(v));
}
__device__ __forceinline__ uint64_t fma_f32x2(uint64_t a, uint64_t b, uint64_t c) {
  uint64_t d;
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
  return d;
}

// Four 8x8 BF16 matrices from shared memory, transposed (ldmatrix): lanes
// 8j..8j+7 give the 16-byte row addresses of matrix j; register j of lane t
// then holds elements (2(t%4), t/4) and (2(t%4)+1, t/4) of matrix j, which is
// the B fragment of mma.sync m16n8k16 for a matrix stored with K along rows.
__device__ __forceinline__ void ldmatrix_x4_trans(uint32_t saddr, uint32_t &r0, uint32_t &r1, uint32_t &r2,
                                                  uint32_t &r3) {
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 {%0,%1,%2,%3}, [%4];"
               : "=r"(r0), "=r"(r1), "=r"(r2), "=r"(r3)
               : "r"(saddr)
               : "memory");
}

// D[16x8] += A[16x16] B[16x8], BF16 operands, FP32 accumulation (warp MMA).
__device__ __forceinline__ void mma_bf16_16816(float *d, const uint32_t *a, uint32_t b0, uint32_t b1) {
  asm volatile("mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
               "{%0,%1,%2,%3};"
               : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
               : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// CTA that owns work item w when W items are split into G contiguous ranges
// [b*W/G, (b+1)*W/G).
__host__ __device__ inline int work_owner(int64_t w, int64_t W, int G) {
  return (int)(((w + 1) * (int64_t)G - 1) / W);
}

// Largest number of CTAs that share one row tile when rowTiles*C work items
// are split evenly over G CTAs.
inline int max_slots(int rowTiles, int C, int G) {
  const int64_t W = (int64_t)rowTiles * C;
  int J = 1;
  for (int r = 0; r < rowTiles; ++r) {
    int b0 = work_owner((int64_t)r * C, W, G), b1 = work_owner((int64_t)(r + 1) * C - 1, W, G);
    J = std::max(J, b1 - b0 + 1);
  }
  return J;
}

// D += A(TMEM) * B(SMEM)^T, kind::tf32 (one TF32 element per TMEM column)
__device__ __forceinline__ void umma_ta_tf32(uint32_t dtmem, uint32_t atmem, uint64_t bdesc, uint32_t idesc,
                                             uint32_t accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::tf32 [%0], [%1], %2, %3, p;\n}\n" ::"r"(dtmem),
      "r"(atmem), "l"(bdesc), "r"(idesc), "r"(accumulate));
}
__device__ __forceinline__ void tmem_st8(uint32_t taddr, const uint32_t *w) {
  asm volatile("tcgen05.st.sync.aligned.32x32b.x8.b32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8};" ::"r"(taddr), "r"(w[0]),
               "r"(w[1]), "r"(w[2]), "r"(w[3]), "r"(w[4]), "r"(w[5]), "r"(w[6]), "r"(w[7])
               : "memory");
}

// D += A(SMEM) * B(SMEM)^T, kind::f16
__device__ __forceinline__ void umma_ss(uint32_t dtmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                        uint32_t accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(dtmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate));
}

}  // namespace
}  // namespace hoe
