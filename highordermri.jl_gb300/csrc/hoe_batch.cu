// hoe_batch.cu — several operators (slices) applied together.
//
// The reference builds one operator per slice and calls its products and
// recon_HOOp slice by slice (explicit_gpu_operator.jl:299-392,
// recon_HOOp.jl:52-88).  A batch groups such operators so that each
// direction of every slice runs in ONE persistent tensor-core launch (work
// items of all slices split evenly over the SMs, hoe_tc.cu), and the
// per-slice CGNR solves run in lockstep inside one CUDA graph (hoe_cg.cu).
// Members that use the plain FP32 engine are applied one after another.
#include "hoe_internal.cuh"

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>

namespace {

bool valid_batch(const hoe_batch *b) { return b && b->magic == HOE_BATCH_MAGIC; }
bool valid_op(const hoe_handle *h) { return h && h->magic == HOE_MAGIC; }

int bfail(hoe_batch *b, int code, const char *fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  if (b) b->err = buf;
  hoe::record_error(buf);
  return code;
}

int bcuda(hoe_batch *b, cudaError_t e, const char *what) {
  cudaGetLastError();
  if (e == cudaErrorMemoryAllocation) return bfail(b, HOE_ERR_OOM, "%s: out of device memory", what);
  return bfail(b, HOE_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

int usable(hoe_batch *b) {
  if (!valid_batch(b)) return bfail(nullptr, HOE_ERR_ARG, "invalid batch");
  for (size_t i = 0; i < b->hs.size(); ++i)
    if (!valid_op(b->hs[i]) || b->hs[i]->closed)
      return bfail(b, HOE_ERR_CLOSED, "member operator %zu is closed", i);
  return HOE_OK;
}

struct DeviceGuard {
  int prev = -1;
  explicit DeviceGuard(int d) {
    cudaGetDevice(&prev);
    if (prev != d) cudaSetDevice(d);
  }
  ~DeviceGuard() {
    if (prev >= 0) cudaSetDevice(prev);
  }
};

int64_t member_launches(const hoe_batch *b) {
  int64_t s = 0;
  for (auto *h : b->hs) s += h->launches;
  return s;
}

template <typename T>
bool all_set(T *const *v, size_t n) {
  if (!v) return false;
  for (size_t i = 0; i < n; ++i)
    if (!v[i]) return false;
  return true;
}

}  // namespace

extern "C" {

int hoe_batch_create(hoe_batch **out, hoe_handle *const *ops, int32_t n) {
  if (!out) return bfail(nullptr, HOE_ERR_ARG, "output pointer must not be NULL");
  *out = nullptr;
  if (!ops || n < 1) return bfail(nullptr, HOE_ERR_ARG, "a batch needs at least one operator");
  bool allTc = true;
  for (int i = 0; i < n; ++i) {
    if (!valid_op(ops[i])) return bfail(nullptr, HOE_ERR_ARG, "member %d is not an operator", i);
    if (ops[i]->closed) return bfail(nullptr, HOE_ERR_CLOSED, "member %d is closed", i);
    if (ops[i]->device != ops[0]->device)
      return bfail(nullptr, HOE_ERR_ARG, "members must share one device (member %d)", i);
    for (int j = 0; j < i; ++j)
      if (ops[j] == ops[i]) return bfail(nullptr, HOE_ERR_ARG, "member %d repeats member %d", i, j);
    allTc = allTc && ops[i]->engine == HOE_ENGINE_TC_BF16X3 && ops[i]->tc.ready &&
            ops[i]->t.nCha == ops[0]->t.nCha;
  }
  auto *b = new hoe_batch();
  b->device = ops[0]->device;
  b->hs.assign(ops, ops + n);
  if (allTc) {
    DeviceGuard guard(b->device);
    std::string why;
    b->tcplan = hoe::tc_batch_plan(b->hs.data(), n, &why);
    if (!b->tcplan) {
      delete b;
      return bfail(nullptr, HOE_ERR_UNSUPPORTED, "batched tensor-core plan: %s", why.c_str());
    }
  }
  *out = b;
  return HOE_OK;
}

void hoe_batch_free(hoe_batch *b) {
  if (!valid_batch(b)) return;
  DeviceGuard guard(b->device);
  hoe::cg_graph_release(b->graph);
  hoe::tc_batch_plan_free(b->tcplan);
  b->magic = 0;
  delete b;
}

const char *hoe_batch_last_error(const hoe_batch *b) {
  if (!valid_batch(b)) return hoe_last_error(nullptr);
  return b->err.c_str();
}

int hoe_batch_get_info(const hoe_batch *b, hoe_batch_info *o) {
  if (!valid_batch(b) || !o) return bfail(nullptr, HOE_ERR_ARG, "invalid batch or output");
  o->n = (int32_t)b->hs.size();
  o->contraction_launches = b->tcplan ? hoe::tc_batch_launches(b->tcplan) : (int32_t)b->hs.size();
  o->launches = b->launches;
  return HOE_OK;
}

int hoe_batch_forward(hoe_batch *b, const void *const *x, void *const *y, void *stream) {
  int rc = usable(b);
  if (rc) return rc;
  const size_t n = b->hs.size();
  if (!all_set(x, n) || !all_set(y, n)) return bfail(b, HOE_ERR_ARG, "x and y need one device pointer per member");
  DeviceGuard guard(b->device);
  cudaStream_t st = (cudaStream_t)stream;
  const int64_t l0 = member_launches(b);
  cudaError_t e = cudaSuccess;
  if (b->tcplan) {
    e = hoe::tc_batch_forward(b->tcplan, (const float2 *const *)x, (float2 *const *)y, st);
  } else {
    for (size_t i = 0; i < n && e == cudaSuccess; ++i)
      e = hoe::apply_forward(b->hs[i], (const float2 *)x[i], (float2 *)y[i], st);
  }
  b->launches += member_launches(b) - l0;
  if (e == cudaSuccess) e = cudaGetLastError();
  return e == cudaSuccess ? HOE_OK : bcuda(b, e, "hoe_batch_forward");
}

int hoe_batch_adjoint(hoe_batch *b, const void *const *y, void *const *x, void *stream) {
  int rc = usable(b);
  if (rc) return rc;
  const size_t n = b->hs.size();
  if (!all_set(x, n) || !all_set(y, n)) return bfail(b, HOE_ERR_ARG, "x and y need one device pointer per member");
  DeviceGuard guard(b->device);
  cudaStream_t st = (cudaStream_t)stream;
  const int64_t l0 = member_launches(b);
  cudaError_t e = cudaSuccess;
  if (b->tcplan) {
    e = hoe::tc_batch_adjoint(b->tcplan, (const float2 *const *)y, nullptr, (float2 *const *)x, st);
  } else {
    for (size_t i = 0; i < n && e == cudaSuccess; ++i)
      e = hoe::apply_adjoint_weighted(b->hs[i], (const float2 *)y[i], nullptr, (float2 *)x[i], st);
  }
  b->launches += member_launches(b) - l0;
  if (e == cudaSuccess) e = cudaGetLastError();
  return e == cudaSuccess ? HOE_OK : bcuda(b, e, "hoe_batch_adjoint");
}

int hoe_batch_normal(hoe_batch *b, const float *const *D, const void *const *x, void *const *out, void *stream) {
  int rc = usable(b);
  if (rc) return rc;
  const size_t n = b->hs.size();
  if (!all_set(x, n) || !all_set(out, n))
    return bfail(b, HOE_ERR_ARG, "x and out need one device pointer per member");
  DeviceGuard guard(b->device);
  cudaStream_t st = (cudaStream_t)stream;
  const int64_t l0 = member_launches(b);
  cudaError_t e = cudaSuccess;
  if (b->tcplan) {
    e = hoe::tc_batch_normal(b->tcplan, D, (const float2 *const *)x, (float2 *const *)out, st);
  } else {
    for (size_t i = 0; i < n && e == cudaSuccess; ++i)
      e = hoe::apply_normal(b->hs[i], D ? D[i] : nullptr, (const float2 *)x[i], (float2 *)out[i], st);
  }
  b->launches += member_launches(b) - l0;
  if (e == cudaSuccess) e = cudaGetLastError();
  return e == cudaSuccess ? HOE_OK : bcuda(b, e, "hoe_batch_normal");
}

int hoe_batch_recon(hoe_batch *b, const void *const *data, const void *const *weights, void *const *x,
                    const hoe_cg_params *p, hoe_cg_stats *stats, void *stream) {
  int rc = usable(b);
  if (rc) return rc;
  const size_t n = b->hs.size();
  if (!all_set(data, n) || !all_set(x, n))
    return bfail(b, HOE_ERR_ARG, "data and x need one device pointer per member");
  if (!p) return bfail(b, HOE_ERR_ARG, "solver parameters must not be NULL");
  if (p->iterations < 0) return bfail(b, HOE_ERR_ARG, "iterations must be >= 0 (got %d)", p->iterations);
  if (!(p->rel_tol >= 0.0) || !std::isfinite(p->rel_tol)) return bfail(b, HOE_ERR_ARG, "rel_tol must be finite and >= 0");
  if (!(p->lambda >= 0.0) || !std::isfinite(p->lambda)) return bfail(b, HOE_ERR_ARG, "lambda must be finite and >= 0");
  DeviceGuard guard(b->device);
  cudaStream_t st = (cudaStream_t)stream;
  hoe::CgRequest r;
  r.iterations = p->iterations;
  r.use_graph = p->use_graph != 0;
  r.rel_tol = p->rel_tol;
  r.lambda = p->lambda;
  std::vector<const float2 *> w(n, nullptr);
  if (weights)
    for (size_t i = 0; i < n; ++i) w[i] = (const float2 *)weights[i];
  cudaError_t e = hoe::cg_batch_solve(b, (const float2 *const *)data, w.data(), (float2 *const *)x, r, st);
  if (e == cudaSuccess) e = cudaGetLastError();
  if (e != cudaSuccess) return bcuda(b, e, "hoe_batch_recon");
  if (stats) {
    for (size_t i = 0; i < n; ++i) {
      hoe::CgScalars S{};
      e = hoe::cg_read_stats(b->hs[i], st, &S);
      if (e != cudaSuccess) return bcuda(b, e, "hoe_batch_recon: reading the solver state");
      stats[i].iterations = S.iters;
      stats[i].status = S.status[r.iterations & 1];
      stats[i].residual0 = std::sqrt(S.zz0);
      stats[i].residual = std::sqrt(S.zz[r.iterations & 1]);
    }
  }
  return HOE_OK;
}

int hoe_batch_check(hoe_batch *b, void *stream) {
  int rc = usable(b);
  if (rc) return rc;
  DeviceGuard guard(b->device);
  cudaError_t e = cudaStreamSynchronize((cudaStream_t)stream);
  if (e != cudaSuccess) return bcuda(b, e, "hoe_batch_check");
  int *word = hoe::tc_batch_error_word(b->tcplan);
  if (word) {
    int v = 0;
    e = cudaMemcpy(&v, word, sizeof(int), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return bcuda(b, e, "hoe_batch_check");
    if (v != 0) {
      cudaMemset(word, 0, sizeof(int));
      return bfail(b, HOE_ERR_TIMEOUT, "a bounded device wait ran out (batched tensor-core pipeline)");
    }
  }
  for (auto *h : b->hs) {
    rc = hoe_check(h, stream);
    if (rc) return bfail(b, rc, "%s", hoe_last_error(h));
  }
  return HOE_OK;
}

}  // extern "C"
