// Internal declarations of libhoexplicit.so (not part of the C ABI).
//
// Phase decomposition used by every engine
// ----------------------------------------
// For voxel v let beta_v = [bf[v,0..R0-1], fieldmap[v]] and for sample s let
// gamma_s = [kspha[0..R0-1,s], times[s]] (R = R0+1 components), so that the
// reference phase (array_operator.jl:269) is phi[s,v] = beta_v . gamma_s in
// cycles.  Voxels are grouped into voxel tiles (compact in space, Morton
// order) and samples into sample tiles (consecutive in time).  With per-tile
// anchors betabar (voxel tile) and gammabar (sample tile), exactly
//
//   phi[s,v] = A[vt(v), s] + B[st(s), v] + dbeta_v . kappa_s
//   A[vt,s]  = betabar_vt . kappa_s            kappa_s = gamma_s - gammabar_st(s)
//   B[st,v]  = beta_v . gammabar_st            dbeta_v = beta_v  - betabar_vt(v)
//
// A and B are evaluated once per operator in FP64 and range-reduced to their
// fractional cycle in [-1/2, 1/2] before being stored as FP32.  Only the
// residual dbeta.kappa, whose magnitude is bounded by the tile extents (a
// few cycles, reported as residual_phase_bound), is formed per (sample,
// voxel) pair in FP32.  The sum is range-reduced again before the FP32
// sine/cosine, so the argument of every sincos is in [-pi, pi].
//
// The voxel-tile anchor of the basis components is the basis of one voxel
// of the tile (the one nearest the tile's centre), so every dbeta_v is a
// difference of basis vectors.  On a 2-D slice the solid harmonics are
// polynomials of degree <= 3 in (x, y) and those differences span at most
// 9 directions (10 with the fieldmap).  The residual is therefore stored in
// a reduced basis: with column balancing S (so dbeta and kappa have equal
// scales per component) and the right singular vectors V_r of the balanced
// dbeta matrix (FP64 Householder QR + one-sided Jacobi SVD),
//   dbeta.kappa = (dbeta S V_r) . (kappa S^-1 V_r) + e,
// where the dropped directions contribute |e| <= 1e-9 cycles per dropped
// direction.  The stored width Rp is r rounded up to 8, 12, 16 or 24.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <complex>
#include <string>
#include <vector>
#include "hoexplicit.h"

#define HOE_MAGIC 0x484f4531  // "HOE1"

namespace hoe {

constexpr int kTileS = 128;   // samples per sample tile (phase anchors, SIMT CTA rows)
constexpr int kTileV = 128;   // voxels per voxel tile
constexpr int kRF = 24;       // stored width of the raw basis / kspha_dt rows
// Largest residual phase bound (cycles) the tensor-core engine accepts.  Its
// phase is formed on the tensor cores (TF32 split products, FP32
// accumulation) and goes to the FP32 sincos without a further reduction, so
// its error grows with the magnitude of the residual: measured on GB300 at
// 5.6e-6 (relative L2 vs FP64) up to 79 cycles and 1.3e-5 at 308 cycles.
// Above this bound the engine refuses the plan and AUTO takes the FP32
// engine, whose phase is range-reduced before every sincos.
constexpr double kTcMaxPhaseBound = 1024.0;

struct Tables {
  // sizes
  int nX = 0, nY = 0, nZ = 0, nFull = 0;
  int nSam = 0, nCha = 0, nTerm = 0, R0 = 0, R = 0, Rp = 0, nVox = 0;
  int ST = kTileS, VT = kTileV;
  int nSt = 0, nVt = 0, nSamPad = 0, nVoxPad = 0, nChaPad = 0;
  int hasKdot = 0;
  double residBound = 0.0;
  // model tables (device)
  int    rank = 0;          // reduced residual dimension r (<= R)
  float  *dbeta = nullptr;   // [nVoxPad][Rp]  reduced, balanced beta_v - betabar
  float  *kappa = nullptr;   // [nSamPad][Rp]  reduced, balanced gamma_s - gammabar
  float  *Atab  = nullptr;   // [nVt][nSamPad] frac(betabar . kappa)
  float  *Btab  = nullptr;   // [nSt][nVoxPad] frac(beta . gammabar)
  float2 *csm   = nullptr;   // [nVoxPad][nChaPad]
  int    *perm  = nullptr;   // [nVoxPad] linear grid index, -1 for padding
  int    *unmasked = nullptr;   // [nUnmasked] linear grid indices outside the mask, ascending
  int    nUnmasked = 0;
  // TF32 hi/lo copies of the reduced residual vectors for the tensor-core
  // phase MMA, in UMMA K-major no-swizzle layout: 8-row groups of KP/4 core
  // matrices (8 rows x 4 TF32 each); width KP = rank rounded up to 8, 16 or 24
  int    KP = 0;
  float  *dbHi = nullptr, *dbLo = nullptr;  // [nVoxPad/8][KP/4][8][4]
  float  *kpHi = nullptr, *kpLo = nullptr;  // [nSamPad/8][KP/4][8][4]
  float  *bfraw = nullptr;   // [nVoxPad][kRF] bf (R0 terms) and fieldmap at slot R0
  float  *kdot  = nullptr;   // [nSamPad][kRF] kspha_dt (nTerm terms), zero elsewhere
  float  *times = nullptr;   // [nSamPad]
  // FP64 planning arrays kept for re-planning the sample side on the device
  // (hoe_set_kspha): beta and its tile anchors, the sample-tile anchors and
  // residuals, times, and the balancing / reduced basis of the residual.
  double *beta64 = nullptr;   // [nVoxPad][R]
  double *betabar = nullptr;  // [nVt][R]
  double *gambar = nullptr;   // [nSt][R]
  double *kap64 = nullptr;    // [nSamPad][R]
  double *times64 = nullptr;  // [nSamPad]
  double *bal = nullptr;      // [R]
  double *Vr = nullptr;       // [R][rank]
};

struct Scratch {
  float2 *Z = nullptr;       // [nVoxPad][nChaPad] x .* csm in tile order
  float2 *Yt = nullptr;      // [nSamPad][nChaPad] data transposed (coil fastest)
  float2 *part = nullptr;    // split-K partial sums
  size_t partElems = 0;
  float  *gpart = nullptr;   // backward partials
  size_t gpartElems = 0;
  double *dred = nullptr;    // backward FP64 reduction slots (bwd_red_slots)
};

// Tensor-core operand staging (built lazily when the TC engine is selected).
struct TcState {
  bool ready = false;
  void *buf = nullptr;       // one allocation for all TC operands
  size_t bytes = 0;
};

// Device-resident CGNR (hoe_cg.cu).
struct CgScalars {            // device scalars of one solve
  double zz0;                 // ‖z₀‖²
  double zz[2];               // ‖zₖ‖², slot k&1
  double pq;                  // Re(pᴴq) of the last iteration
  int status[2];              // 0 running, 1 converged, 2 stopped (pᴴq ≤ 0 / not finite), slot k&1
  int iters;                  // iterations that updated x
  int pad;
};

struct CgRequest {
  int iterations = 0;
  int use_graph = 1;
  double rel_tol = 0.0;
  double lambda = 0.0;
};

// A solve captured as a CUDA graph, replayed while its request is unchanged.
struct CgGraph {
  cudaStream_t cap = nullptr;         // capture stream
  cudaGraphExec_t exec = nullptr;
  int64_t launches = 0;               // kernels per graph launch
  std::vector<const void *> key;      // pointers of the captured request
  int kIters = -1, kEngine = -1;
  double kTol = 0.0, kLambda = 0.0;
};

struct CgState {
  void *base = nullptr;       // one allocation for the buffers below
  size_t bytes = 0;
  float2 *z = nullptr, *p = nullptr, *q = nullptr;   // [nFull] solver vectors
  float *D = nullptr;         // [nSam*nCha] |w|²
  double *part = nullptr;     // [2][304] block partials (pᴴq, ‖z‖²)
  CgScalars *S = nullptr;
  CgGraph graph;
};

// Programmatic dependent launch.  The engine's kernels are launched with
// programmatic stream serialisation (launch_pdl), so a kernel may become
// resident while the previous kernel in the stream is still running.  Each
// kernel calls pdl_wait() before its first global-memory access (it returns
// once the previous grid has completed and its writes are visible) and
// pdl_trigger() only after that, so that kernel k+1 cannot start before
// kernel k-1 has finished.  Without the launch attribute both are no-ops.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

// Launch with programmatic stream serialisation (cudaLaunchKernelEx).
template <typename... KArgs, typename... Args>
cudaError_t launch_pdl(void (*kern)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t st,
                       Args... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, kern, static_cast<KArgs>(args)...);
}

}  // namespace hoe

struct hoe_handle {
  uint32_t magic = HOE_MAGIC;
  // tracing (hoe_set_timing): events 0-3 forward, 4-7 adjoint
  int timing = 0;
  cudaEvent_t ev[8] = {};
  mutable int64_t launches = 0;
  int closed = 0;
  int device = 0;
  int engine = HOE_ENGINE_FP32_SIMT;
  int numSMs = 0;
  int splitF = 1, splitA = 1;
  int tcPlan = 0;                 // tensor-core execution plan requested at create (hoe_desc.tc_plan)
  int64_t bytes = 0;
  std::string err;
  hoe::Tables t;
  hoe::Scratch s;
  hoe::TcState tc;
  void *tc_host = nullptr;   // tensor-core buffer table (hoe_tc.cu)
  void *tcb_host = nullptr;  // tensor-core backward buffers (hoe_tc_bwd.cu), allocated on first use
  hoe::CgState cg;           // device-resident CGNR (hoe_cg.cu)
};

#define HOE_BATCH_MAGIC 0x484f4542u

// Several operators applied together (hoe_batch.cu).  Borrows its members.
struct hoe_batch {
  uint32_t magic = HOE_BATCH_MAGIC;
  int device = 0;
  std::vector<hoe_handle *> hs;
  void *tcplan = nullptr;    // one persistent launch per direction (tensor-core members)
  std::string err;
  int64_t launches = 0;
  hoe::CgGraph graph;        // cached batched CGNR
};

namespace hoe {

// SIMT kernels (hoe_simt.cu).  All launches are asynchronous on `st`.
cudaError_t simt_forward(const hoe_handle *h, const float2 *x, float2 *y,
                         const float *D, int mode, cudaStream_t st);
cudaError_t simt_adjoint_from_Yt(const hoe_handle *h, float2 *x, cudaStream_t st);
cudaError_t prep_Z(const hoe_handle *h, const float2 *x, cudaStream_t st);
cudaError_t prep_Yt(const hoe_handle *h, const float2 *y, const float *D, cudaStream_t st);
// Split-K reductions shared by both engines: sum `splits` partial slices of
// `part` and write y (FWD_TO_Y / FWD_DERIV_TO_Y) or the weighted Yt, resp. the
// coil-combined, scaled, scattered image.
cudaError_t simt_reduce_forward(const hoe_handle *h, const float2 *part, int splits, float2 *y,
                                const float *D, int mode, cudaStream_t st);
cudaError_t simt_reduce_adjoint(const hoe_handle *h, const float2 *part, int splits, float2 *x,
                                cudaStream_t st);
cudaError_t simt_backward(const hoe_handle *h, const float2 *x, const float2 *r,
                          float *dk, float *ddf, double *dt0, int flags, cudaStream_t st);

// Operator applications on the active engine (hoe_api.cu): y = HOOp x,
// out = HOOpᴴ diag(D) HOOp x, and x = HOOpᴴ (D · y) (D = NULL: ones).
cudaError_t apply_forward(hoe_handle *h, const float2 *x, float2 *y, cudaStream_t st);
cudaError_t apply_normal(hoe_handle *h, const float *D, const float2 *x, float2 *out, cudaStream_t st);
cudaError_t apply_adjoint_weighted(hoe_handle *h, const float2 *y, const float *D, float2 *x,
                                   cudaStream_t st);

// Device-resident CGNR (hoe_cg.cu).  cg_solve enqueues a whole solve on st
// (as one cached CUDA graph when r.use_graph); cg_read_stats waits for st.
cudaError_t cg_solve(hoe_handle *h, const float2 *data, const float2 *w, float2 *x, const CgRequest &r,
                     cudaStream_t st);
// The same solve for every member of a batch in lockstep (one graph).
cudaError_t cg_batch_solve(hoe_batch *b, const float2 *const *data, const float2 *const *w, float2 *const *x,
                           const CgRequest &r, cudaStream_t st);
cudaError_t cg_read_stats(const hoe_handle *h, cudaStream_t st, CgScalars *out);
void cg_release(hoe_handle *h);
void cg_graph_release(CgGraph &g);

// Anchor-phase tables Atab/Btab from the FP64 planning arrays (hoe_api.cu).
cudaError_t build_anchor_tables(const hoe_handle *h, cudaStream_t st);

// Sample-side re-plan for new coefficients (hoe_sync.cu): kspha[s*ldk + l]
// (l < R0, FP64), kdot[s*ldd + l] (l < nTerm, FP64) or NULL.  Scaled by
// termMask[l] when given.  Stream-ordered.
cudaError_t replan_samples(hoe_handle *h, const double *kspha, int ldk, const double *kdot, int ldd,
                           const double *termMask, cudaStream_t st);

// Trajectory preprocessing and delay estimation (hoe_sync.cu).
cudaError_t kdot_stencil(const double *traj, int64_t n, int nTerm, double dt, double *out, cudaStream_t st);
cudaError_t sfu_rate(double *lanesPerClkPerSm, cudaStream_t st);
cudaError_t interp_akima(const double *traj, int64_t n, int nTerm, double dt, const double *delTimeDev,
                         double delTimeHost, const double *datatime, int64_t nData, double *out, int layout,
                         int ldo, const double *termMask, cudaStream_t st);
cudaError_t find_delay(hoe_handle *h, hoe_handle *hr, int nShot, const double *startTimes,
                       const hoe_delay_params &q, const float2 *data, const float2 *weights,
                       const double *traj, int64_t nField, float2 *xOut, hoe_delay_result *res, cudaStream_t st);

// Solver building blocks for larger captured sequences (hoe_cg.cu):
// cg_prepare allocates the solver buffers (outside any capture), cg_enqueue
// enqueues one complete solve without a graph of its own.
cudaError_t cg_prepare(hoe_handle *h);
cudaError_t cg_enqueue(hoe_handle *h, const float2 *data, const float2 *w, float2 *x, const CgRequest &r,
                       cudaStream_t st);

// SVD coil compression (hoe_coils.cu).  G is row-major complex128.
cudaError_t coil_gram(const void *A, int doubleInput, int64_t nObs, int nCoil, int center,
                      std::vector<std::complex<double>> &G, cudaStream_t st);
int coil_fit(const void *A, int doubleInput, int64_t nObs, int nCoil, int nVirtual, double energyThreshold,
             const double *noiseCov, double scale, double *matrixOut, double *svOut, int *rankOut,
             double *retainedOut, std::string *why, cudaStream_t st);
cudaError_t coil_apply(const float2 *a, int64_t n, int nCoil, const float2 *M, int nVirt, float2 *out,
                       cudaStream_t st);

// Sets the thread's handle-less error message (hoe_last_error(NULL)).
void record_error(const char *msg);

// Records trace event i on stream st when tracing is enabled.
inline void trace(const hoe_handle *h, int i, cudaStream_t st) {
  if (h->timing && h->ev[i]) cudaEventRecord(h->ev[i], st);
}
enum { EV_F0 = 0, EV_FK0 = 1, EV_FK1 = 2, EV_F1 = 3, EV_A0 = 4, EV_AK0 = 5, EV_AK1 = 6, EV_A1 = 7 };

// forward modes
enum { FWD_TO_Y = 0, FWD_TO_YT_WEIGHTED = 1, FWD_DERIV_TO_Y = 2 };

// Tensor-core kernels (hoe_tc.cu).
cudaError_t tc_prepare(hoe_handle *h);
void tc_release(hoe_handle *h);
// Backward pass on the tensor cores (hoe_tc_bwd.cu): up to 16 coils and a
// residual width of at most 16; otherwise simt_backward.
bool tc_backward_supported(const hoe_handle *h);
cudaError_t tc_backward(hoe_handle *h, const float2 *x, const float2 *r, float *dk, float *ddf, double *dt0,
                        int flags, cudaStream_t st);
void tc_backward_release(hoe_handle *h);
// The reductions after either backward kernel: dk from nSplit partial slots
// [nSplit][nSamPad][kRF], dL/dfieldmap and the fieldmap part of dL/dt0 from
// nRows partial rows [nRows][nVoxPad] of sum_s G and sum_s G t_s, and dL/dt0.
// FP64 block partials of the backward's final reductions: the voxel blocks
// of k_bwd_vox, then the blocks of k_bwd_dk (the t0 coefficient part).
inline int64_t bwd_red_slots(const Tables &t) {
  return (t.nVoxPad + 255) / 256 + ((int64_t)t.nSamPad * kRF + 255) / 256 + 1;
}
cudaError_t bwd_finish(hoe_handle *h, const float *dkpart, int nSplit, const float *g1, const float *gt, int nRows,
                       double *vpart, double *dred, float *dk, float *ddf, double *dt0, int flags, cudaStream_t st);
constexpr int kBwdVoxSplit = 16;   // row ranges of the first voxel reduction pass (vpart: 2 x 16 x nVoxPad)
// Tensor-core applications; each builds its B operand straight from the
// caller's vector (no Z / Yt staging): y = E x; x = E^H (D . y) (D may be
// NULL); out = E^H diag(D) E x.
cudaError_t tc_forward(const hoe_handle *h, const float2 *x, float2 *y, cudaStream_t st);
cudaError_t tc_adjoint(const hoe_handle *h, const float2 *y, const float *D, float2 *x, cudaStream_t st);
cudaError_t tc_normal(const hoe_handle *h, const float *D, const float2 *x, float2 *out, cudaStream_t st);
// B x (kspha_dt mode) on the tensor cores, as forward passes over virtual
// coils (term x coil); buffers on first use.
// Execution plans of the contraction (hoe_autotune): count (5 up to 16
// coils, else 1), current plan, selection (cudaErrorInvalidValue when out of
// range).
int tc_plan_count(const hoe_handle *h);
int tc_get_plan(const hoe_handle *h);
cudaError_t tc_set_plan(hoe_handle *h, int plan);
bool tc_derivative_supported(const hoe_handle *h);
cudaError_t tc_derivative_prepare(hoe_handle *h);
cudaError_t tc_derivative(hoe_handle *h, const float2 *x, float2 *y, cudaStream_t st);
// B x on the operator's engine (the tensor-core passes where supported)
cudaError_t apply_derivative(hoe_handle *h, const float2 *x, float2 *y, cudaStream_t st);
bool tc_supported(const hoe_handle *h, std::string *why);
int *tc_error_word(const hoe_handle *h);   // device word set by a timed-out wait
// Rebuilds the tensor-core anchor tables from Atab/Btab (no-op before tc_prepare).
cudaError_t tc_anchor_tables(const hoe_handle *h, cudaStream_t st);
// Several operators (tensor-core engine, equal coil counts) in one persistent
// launch per direction and residual width.  The plan borrows the handles.
// The batched applications take one device pointer per member; D may be NULL
// (ones) as a whole or per member.
void *tc_batch_plan(hoe_handle *const *hs, int n, std::string *why);
void tc_batch_plan_free(void *plan);
int *tc_batch_error_word(void *plan);
int tc_batch_launches(void *plan);         // contraction launches per direction
cudaError_t tc_batch_forward(void *plan, const float2 *const *x, float2 *const *y, cudaStream_t st);
cudaError_t tc_batch_adjoint(void *plan, const float2 *const *y, const float *const *D, float2 *const *x,
                             cudaStream_t st);
cudaError_t tc_batch_normal(void *plan, const float *const *D, const float2 *const *x, float2 *const *out,
                            cudaStream_t st);

}  // namespace hoe
