// hoe_cg.cu — device-resident weighted CGNR for recon_HOOp.
//
// Restates the solve that recon_HOOp hands to RegularizedLeastSquares
// (src/Recon/recon_HOOp.jl:73-81): with raw complex sample weights w repeated
// over coils, E = W∘HOOp, b = W·vec(Data), and CGNR on the normal equations
//
//     (Eᴴ E + λ I) x = Eᴴ b,      Eᴴ E = HOOpᴴ diag(|w|²) HOOp,  Eᴴ b = HOOpᴴ (|w|² · Data)
//
// starting from x = 0 (RegularizedLeastSquares 0.16.12 `CGNR` with an `AHA`
// normal operator and `L2Regularization(λ)`; that package is not vendored in
// the reference tree, the published conjugate-gradient recurrence is restated):
//
//     z₀ = Eᴴ b,  p₀ = z₀
//     qₖ = (EᴴE + λI) pₖ,  αₖ = ‖zₖ‖² / Re(pₖᴴ qₖ)
//     xₖ₊₁ = xₖ + αₖ pₖ,  zₖ₊₁ = zₖ − αₖ qₖ
//     βₖ = ‖zₖ₊₁‖² / ‖zₖ‖²,  pₖ₊₁ = zₖ₊₁ + βₖ pₖ
//
// stopping after `iterations` updates or once ‖zₖ‖ ≤ rel_tol·‖z₀‖.
//
// Everything stays on the device: the vectors x, z, p, q are complex64 (the
// precision of the operator), the scalars ‖z‖², pᴴq, α and β are FP64 and are
// formed and consumed on the device, so the host never synchronises inside
// the solve.  Reductions are two-level with a fixed block count and a fixed
// summation tree: the same inputs give bitwise the same image, whether the
// iterations run as individual launches or as one captured CUDA graph.
//
// Control on the device: iteration k reads the status and ‖zₖ‖² written by
// iteration k−1 from slot k&1 and writes slot (k+1)&1, so no kernel reads a
// slot that a block of the same kernel writes.  Once the solve has stopped
// (converged, or pᴴq ≤ 0 / not finite), the later iterations of a graph still
// launch but leave x, z and p unchanged.
#include "hoe_internal.cuh"

#include <cmath>

namespace hoe {
namespace {

constexpr int kThreads = 256;
constexpr int kMaxBlocks = 304;  // 2 blocks per SM on 152 SMs

enum { CG_RUNNING = 0, CG_CONVERGED = 1, CG_BREAKDOWN = 2 };

// FP64 sum over a block of kThreads threads with a fixed tree; every thread
// gets the result.
__device__ double block_sum(double v) {
  __shared__ double sh[kThreads / 32];
  __shared__ double total;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x < 32) {
    double r = threadIdx.x < kThreads / 32 ? sh[threadIdx.x] : 0.0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) r += __shfl_down_sync(0xffffffffu, r, o);
    if (threadIdx.x == 0) total = r;
  }
  __syncthreads();
  double r = total;
  __syncthreads();
  return r;
}

// Sum of the G block partials in a fixed order (identical in every block).
__device__ double sum_partials(const double *__restrict__ part, int G) {
  double v = 0.0;
  for (int i = threadIdx.x; i < G; i += kThreads) v += part[i];
  return block_sum(v);
}

__device__ __forceinline__ bool finite_pos(double v) { return v > 0.0 && v < INFINITY; }

// D[s + c*nSam] = |w[s]|² (ones without weights): WᴴW of the weighting operator.
__global__ void k_cg_weights(const float2 *__restrict__ w, float *__restrict__ D, int nSam, int nCha) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (int64_t)nSam * nCha) return;
  float d = 1.f;
  if (w) {
    float2 v = w[i % nSam];
    d = v.x * v.x + v.y * v.y;
  }
  D[i] = d;
}

// p = z, x = 0; partial ‖z‖².
__global__ void __launch_bounds__(kThreads) k_cg_start(const float2 *__restrict__ z, float2 *__restrict__ p,
                                                       float2 *__restrict__ x, int64_t n,
                                                       double *__restrict__ part) {
  double acc = 0.0;
  for (int64_t i = (int64_t)blockIdx.x * kThreads + threadIdx.x; i < n; i += (int64_t)gridDim.x * kThreads) {
    float2 v = z[i];
    p[i] = v;
    x[i] = make_float2(0.f, 0.f);
    acc += (double)v.x * v.x + (double)v.y * v.y;
  }
  double s = block_sum(acc);
  if (threadIdx.x == 0) part[blockIdx.x] = s;
}

__global__ void __launch_bounds__(kThreads) k_cg_start_fin(const double *__restrict__ part, int G,
                                                           CgScalars *S) {
  double zz = sum_partials(part, G);
  if (threadIdx.x == 0) {
    S->zz0 = zz;
    S->zz[0] = zz;
    S->zz[1] = zz;
    S->pq = 0.0;
    S->iters = 0;
    S->status[0] = zz == 0.0 ? CG_CONVERGED : (finite_pos(zz) ? CG_RUNNING : CG_BREAKDOWN);
    S->status[1] = S->status[0];
  }
}

// q += λ p (when λ > 0); partial Re(pᴴ q).
__global__ void __launch_bounds__(kThreads) k_cg_pq(const float2 *__restrict__ p, float2 *__restrict__ q,
                                                    int64_t n, float lambda, double *__restrict__ part) {
  double acc = 0.0;
  for (int64_t i = (int64_t)blockIdx.x * kThreads + threadIdx.x; i < n; i += (int64_t)gridDim.x * kThreads) {
    float2 a = p[i], b = q[i];
    if (lambda != 0.f) {
      b.x = fmaf(lambda, a.x, b.x);
      b.y = fmaf(lambda, a.y, b.y);
      q[i] = b;
    }
    acc += (double)a.x * b.x + (double)a.y * b.y;
  }
  double s = block_sum(acc);
  if (threadIdx.x == 0) part[blockIdx.x] = s;
}

// The decision of iteration k, formed identically by every block of the two
// update kernels from the same FP64 inputs.
struct StepDecision {
  bool update;
  double alpha, zz, pq;
  int status;
};

__device__ StepDecision decide(const double *__restrict__ partPQ, int G, const CgScalars *S, int k) {
  StepDecision d;
  d.pq = sum_partials(partPQ, G);
  d.zz = S->zz[k & 1];
  d.status = S->status[k & 1];
  d.alpha = d.zz / d.pq;
  d.update = d.status == CG_RUNNING && finite_pos(d.pq) && finite_pos(d.alpha);
  return d;
}

// x += α p, z −= α q; partial ‖z‖².
__global__ void __launch_bounds__(kThreads) k_cg_step(float2 *__restrict__ x, float2 *__restrict__ z,
                                                      const float2 *__restrict__ p, const float2 *__restrict__ q,
                                                      int64_t n, const double *__restrict__ partPQ,
                                                      double *__restrict__ partZZ, int G, const CgScalars *S,
                                                      int k) {
  StepDecision d = decide(partPQ, G, S, k);
  double acc = 0.0;
  if (d.update) {
    const float a = (float)d.alpha;
    for (int64_t i = (int64_t)blockIdx.x * kThreads + threadIdx.x; i < n; i += (int64_t)gridDim.x * kThreads) {
      float2 pv = p[i], qv = q[i], xv = x[i], zv = z[i];
      xv.x = fmaf(a, pv.x, xv.x);
      xv.y = fmaf(a, pv.y, xv.y);
      zv.x = fmaf(-a, qv.x, zv.x);
      zv.y = fmaf(-a, qv.y, zv.y);
      x[i] = xv;
      z[i] = zv;
      acc += (double)zv.x * zv.x + (double)zv.y * zv.y;
    }
  }
  double s = block_sum(acc);
  if (threadIdx.x == 0) partZZ[blockIdx.x] = s;
}

// β = ‖zₖ₊₁‖²/‖zₖ‖², p = z + β p; block 0 publishes slot (k+1)&1.
__global__ void __launch_bounds__(kThreads) k_cg_dir(const float2 *__restrict__ z, float2 *__restrict__ p,
                                                     int64_t n, const double *__restrict__ partPQ,
                                                     const double *__restrict__ partZZ, int G, CgScalars *S,
                                                     int k, double tol2) {
  StepDecision d = decide(partPQ, G, S, k);
  double zznew = d.zz;
  if (d.update) {
    zznew = sum_partials(partZZ, G);
    const float b = (float)(zznew / d.zz);
    for (int64_t i = (int64_t)blockIdx.x * kThreads + threadIdx.x; i < n; i += (int64_t)gridDim.x * kThreads) {
      float2 zv = z[i], pv = p[i];
      pv.x = fmaf(b, pv.x, zv.x);
      pv.y = fmaf(b, pv.y, zv.y);
      p[i] = pv;
    }
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    const int nxt = (k + 1) & 1;
    S->pq = d.pq;
    if (d.update) {
      S->zz[nxt] = zznew;
      S->iters = k + 1;
      S->status[nxt] = (zznew <= tol2 * S->zz0) ? CG_CONVERGED : CG_RUNNING;
    } else {
      S->zz[nxt] = d.zz;
      S->status[nxt] = d.status == CG_RUNNING ? CG_BREAKDOWN : d.status;
    }
  }
}

int grid_for(int64_t n) {
  int64_t g = (n + kThreads - 1) / kThreads;
  return (int)(g < kMaxBlocks ? (g > 0 ? g : 1) : kMaxBlocks);
}

cudaError_t ensure_buffers(hoe_handle *h) {
  auto &c = h->cg;
  if (c.z) return cudaSuccess;
  const auto &t = h->t;
  size_t nImg = (size_t)t.nFull;
  size_t bytes = 3 * nImg * sizeof(float2) + (size_t)t.nSam * t.nCha * sizeof(float) +
                 2 * kMaxBlocks * sizeof(double) + sizeof(CgScalars) + 8 * 256;
  char *buf = nullptr;
  cudaError_t e = cudaMalloc(&buf, bytes);
  if (e != cudaSuccess) return e;
  auto carve = [&](size_t b) { char *r = buf; buf += (b + 255) & ~(size_t)255; return r; };
  c.base = nullptr;
  char *start = buf;
  c.z = (float2 *)carve(nImg * sizeof(float2));
  c.p = (float2 *)carve(nImg * sizeof(float2));
  c.q = (float2 *)carve(nImg * sizeof(float2));
  c.D = (float *)carve((size_t)t.nSam * t.nCha * sizeof(float));
  c.part = (double *)carve(2 * kMaxBlocks * sizeof(double));
  c.S = (CgScalars *)carve(sizeof(CgScalars));
  c.base = start;
  c.bytes = bytes;
  h->bytes += (int64_t)bytes;
  return cudaSuccess;
}

// The operators of one solve: a single handle, or the members of a batch
// (with a batched tensor-core plan when every member runs that engine).
struct Members {
  hoe_handle *const *hs;
  int n;
  void *tcplan;
};

// out_i = HOOp_iᴴ diag(D_i) HOOp_i x_i for every member.
cudaError_t normal_all(const Members &m, const std::vector<float2 *> &xs, const std::vector<float2 *> &outs,
                       cudaStream_t st) {
  cudaError_t e = cudaSuccess;
  if (m.tcplan) {
    std::vector<const float *> D(m.n);
    std::vector<const float2 *> xc(xs.begin(), xs.end());
    for (int i = 0; i < m.n; ++i) D[i] = m.hs[i]->cg.D;
    return tc_batch_normal(m.tcplan, D.data(), xc.data(), outs.data(), st);
  }
  for (int i = 0; i < m.n && e == cudaSuccess; ++i) e = apply_normal(m.hs[i], m.hs[i]->cg.D, xs[i], outs[i], st);
  return e;
}

// Enqueues the whole solve of every member on `st` (a capturing stream or an
// ordinary one).  Member i solves for x[i] from data[i] with weights w[i].
cudaError_t enqueue_solve(const Members &m, const float2 *const *data, const float2 *const *w,
                          float2 *const *x, const CgRequest &r, cudaStream_t st) {
  const int n = m.n;
  std::vector<float2 *> zs(n), ps(n), qs(n);
  cudaError_t e = cudaSuccess;
  for (int i = 0; i < n; ++i) {
    hoe_handle *h = m.hs[i];
    const auto &t = h->t;
    zs[i] = h->cg.z; ps[i] = h->cg.p; qs[i] = h->cg.q;
    const int64_t nd = (int64_t)t.nSam * t.nCha;
    k_cg_weights<<<(unsigned)((nd + 255) / 256), 256, 0, st>>>(w[i], h->cg.D, t.nSam, t.nCha);
    h->launches += 1;
  }
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  // z₀ = HOOpᴴ (|w|² · Data)
  if (m.tcplan) {
    std::vector<const float *> D(n);
    for (int i = 0; i < n; ++i) D[i] = m.hs[i]->cg.D;
    e = tc_batch_adjoint(m.tcplan, data, D.data(), zs.data(), st);
  } else {
    for (int i = 0; i < n && e == cudaSuccess; ++i)
      e = apply_adjoint_weighted(m.hs[i], data[i], m.hs[i]->cg.D, zs[i], st);
  }
  if (e != cudaSuccess) return e;
  for (int i = 0; i < n; ++i) {
    hoe_handle *h = m.hs[i];
    const int64_t nv = h->t.nFull;
    const int G = grid_for(nv);
    double *partZZ = h->cg.part + kMaxBlocks;
    k_cg_start<<<G, kThreads, 0, st>>>(h->cg.z, h->cg.p, x[i], nv, partZZ);
    k_cg_start_fin<<<1, kThreads, 0, st>>>(partZZ, G, h->cg.S);
    h->launches += 2;
  }
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  const double tol2 = r.rel_tol * r.rel_tol;
  for (int k = 0; k < r.iterations; ++k) {
    e = normal_all(m, ps, qs, st);
    if (e != cudaSuccess) return e;
    for (int i = 0; i < n; ++i) {
      hoe_handle *h = m.hs[i];
      auto &c = h->cg;
      const int64_t nv = h->t.nFull;
      const int G = grid_for(nv);
      double *partPQ = c.part, *partZZ = c.part + kMaxBlocks;
      k_cg_pq<<<G, kThreads, 0, st>>>(c.p, c.q, nv, (float)r.lambda, partPQ);
      k_cg_step<<<G, kThreads, 0, st>>>(x[i], c.z, c.p, c.q, nv, partPQ, partZZ, G, c.S, k);
      k_cg_dir<<<G, kThreads, 0, st>>>(c.z, c.p, nv, partPQ, partZZ, G, c.S, k, tol2);
      h->launches += 3;
    }
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
  }
  return cudaSuccess;
}

std::vector<const void *> request_key(const Members &m, const float2 *const *data, const float2 *const *w,
                                      float2 *const *x) {
  std::vector<const void *> k;
  k.reserve(4 * m.n);
  for (int i = 0; i < m.n; ++i) {
    k.push_back(m.hs[i]);
    k.push_back(data[i]);
    k.push_back(w[i]);
    k.push_back(x[i]);
  }
  return k;
}

int engine_key(const Members &m) {
  int e = 0;
  for (int i = 0; i < m.n; ++i) e = e * 2 + m.hs[i]->engine;
  return m.tcplan ? -1 - e : e;
}

// Runs the solve through g: captured on the first call for a request,
// replayed afterwards.  Kernel launches are counted into *launches.
cudaError_t run(CgGraph &g, const Members &m, const float2 *const *data, const float2 *const *w,
                float2 *const *x, const CgRequest &r, cudaStream_t st, int64_t *launches) {
  for (int i = 0; i < m.n; ++i) {
    cudaError_t e = ensure_buffers(m.hs[i]);
    if (e != cudaSuccess) return e;
  }
  if (!r.use_graph) {
    int64_t l0 = 0, l1 = 0;
    for (int i = 0; i < m.n; ++i) l0 += m.hs[i]->launches;
    cudaError_t e = enqueue_solve(m, data, w, x, r, st);
    for (int i = 0; i < m.n; ++i) l1 += m.hs[i]->launches;
    *launches += l1 - l0;
    return e;
  }
  std::vector<const void *> key = request_key(m, data, w, x);
  const int ek = engine_key(m);
  cudaError_t e = cudaSuccess;
  if (!(g.exec && g.key == key && g.kIters == r.iterations && g.kTol == r.rel_tol && g.kLambda == r.lambda &&
        g.kEngine == ek)) {
    if (g.exec) cudaGraphExecDestroy(g.exec);
    g.exec = nullptr;
    if (!g.cap) {
      e = cudaStreamCreateWithFlags(&g.cap, cudaStreamNonBlocking);
      if (e != cudaSuccess) return e;
    }
    std::vector<int> timing(m.n);
    std::vector<int64_t> l0(m.n);
    for (int i = 0; i < m.n; ++i) {
      timing[i] = m.hs[i]->timing;
      m.hs[i]->timing = 0;  // no trace events inside a graph
      l0[i] = m.hs[i]->launches;
    }
    e = cudaStreamBeginCapture(g.cap, cudaStreamCaptureModeThreadLocal);
    cudaError_t eq = e == cudaSuccess ? enqueue_solve(m, data, w, x, r, g.cap) : e;
    cudaGraph_t graph = nullptr;
    if (e == cudaSuccess) e = cudaStreamEndCapture(g.cap, &graph);
    int64_t per = 0;
    for (int i = 0; i < m.n; ++i) {
      m.hs[i]->timing = timing[i];
      per += m.hs[i]->launches - l0[i];
      m.hs[i]->launches = l0[i];
    }
    if (eq != cudaSuccess || e != cudaSuccess) {
      if (graph) cudaGraphDestroy(graph);
      cudaGetLastError();
      return eq != cudaSuccess ? eq : e;
    }
    e = cudaGraphInstantiate(&g.exec, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) { g.exec = nullptr; return e; }
    g.launches = per;
    g.key = std::move(key);
    g.kIters = r.iterations; g.kTol = r.rel_tol; g.kLambda = r.lambda; g.kEngine = ek;
  }
  e = cudaGraphLaunch(g.exec, st);
  if (e == cudaSuccess) *launches += g.launches;
  return e;
}

}  // namespace

void cg_graph_release(CgGraph &g) {
  if (g.exec) cudaGraphExecDestroy(g.exec);
  if (g.cap) cudaStreamDestroy(g.cap);
  g = CgGraph{};
}

void cg_release(hoe_handle *h) {
  auto &c = h->cg;
  cg_graph_release(c.graph);
  if (c.base) cudaFree(c.base);
  h->bytes -= (int64_t)c.bytes;
  c = CgState{};
}

cudaError_t cg_solve(hoe_handle *h, const float2 *data, const float2 *w, float2 *x, const CgRequest &r,
                     cudaStream_t st) {
  hoe_handle *hs[1] = {h};
  const Members m{hs, 1, nullptr};
  int64_t launches = 0;
  cudaError_t e = run(h->cg.graph, m, &data, &w, &x, r, st, &launches);
  h->launches += r.use_graph ? launches : 0;
  return e;
}

cudaError_t cg_batch_solve(hoe_batch *b, const float2 *const *data, const float2 *const *w, float2 *const *x,
                           const CgRequest &r, cudaStream_t st) {
  const Members m{b->hs.data(), (int)b->hs.size(), b->tcplan};
  int64_t launches = 0;
  cudaError_t e = run(b->graph, m, data, w, x, r, st, &launches);
  b->launches += launches;
  return e;
}

cudaError_t cg_prepare(hoe_handle *h) { return ensure_buffers(h); }

cudaError_t cg_enqueue(hoe_handle *h, const float2 *data, const float2 *w, float2 *x, const CgRequest &r,
                       cudaStream_t st) {
  hoe_handle *hs[1] = {h};
  const Members m{hs, 1, nullptr};
  return enqueue_solve(m, &data, &w, &x, r, st);
}

cudaError_t cg_read_stats(const hoe_handle *h, cudaStream_t st, CgScalars *out) {
  cudaError_t e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return e;
  return cudaMemcpy(out, h->cg.S, sizeof(CgScalars), cudaMemcpyDeviceToHost);
}

}  // namespace hoe
