// C ABI of libhoexplicit.so: handle lifetime, model preparation on the
// device, and dispatch of forward / adjoint / normal / derivative / backward.
//
// Mirrors the resident single-GPU operator of the reference
// (src/EncodingOperator/Explicit/explicit_gpu_operator.jl): the handle owns
// the model arrays and scratch space (ExplicitGPUState, :3-29), applications
// take caller-owned device vectors, `close` is idempotent and later use is an
// error (:40-44, :435-446).
#include <cuda_runtime.h>
#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <numeric>
#include <string>
#include <vector>

#include "hoe_internal.cuh"

#define HOE_VERSION_STRING "hoexplicit 0.1.0 (sm_103a)"

namespace {

thread_local std::string g_err;  // failures without a usable handle

int fail(hoe_handle *h, int code, const char *fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  if (h) h->err = buf;
  g_err = buf;
  return code;
}

int cuda_fail(hoe_handle *h, cudaError_t e, const char *what) {
  int code = (e == cudaErrorMemoryAllocation) ? HOE_ERR_OOM : HOE_ERR_CUDA;
  return fail(h, code, "%s: %s", what, cudaGetErrorString(e));
}

// Restores the caller's current device on scope exit.
struct DeviceGuard {
  int prev = -1;
  bool ok = true;
  explicit DeviceGuard(int dev) {
    if (cudaGetDevice(&prev) != cudaSuccess) prev = -1;
    if (prev != dev) ok = cudaSetDevice(dev) == cudaSuccess;
  }
  ~DeviceGuard() {
    int cur = -1;
    if (prev >= 0 && cudaGetDevice(&cur) == cudaSuccess && cur != prev) cudaSetDevice(prev);
  }
};

// Host-side allocation-failure injection for tests of the cleanup path:
// HOE_INJECT_ALLOC_FAIL=n makes the n-th device allocation of hoe_create fail.
struct Allocator {
  hoe_handle *h;
  int count = 0;
  int failAt = -1;
  explicit Allocator(hoe_handle *hh) : h(hh) {
    const char *e = getenv("HOE_INJECT_ALLOC_FAIL");
    if (e && *e) failAt = atoi(e);
  }
  template <class T>
  cudaError_t alloc(T **p, size_t elems) {
    ++count;
    if (failAt > 0 && count == failAt) return cudaErrorMemoryAllocation;
    size_t bytes = std::max<size_t>(elems, 1) * sizeof(T);
    cudaError_t e = cudaMalloc((void **)p, bytes);
    if (e == cudaSuccess) h->bytes += (int64_t)bytes;
    return e;
  }
};

template <class T>
void dfree(T *&p) {
  if (p) cudaFree(p);
  p = nullptr;
}

void release_events(hoe_handle *h) {
  for (auto &e : h->ev) {
    if (e) cudaEventDestroy(e);
    e = nullptr;
  }
  h->timing = 0;
}

void release_device(hoe_handle *h) {
  release_events(h);
  hoe::cg_release(h);
  hoe::tc_backward_release(h);
  hoe::tc_release(h);
  auto &t = h->t;
  dfree(t.dbeta); dfree(t.kappa); dfree(t.Atab); dfree(t.Btab); dfree(t.csm);
  dfree(t.dbHi); dfree(t.dbLo); dfree(t.kpHi); dfree(t.kpLo);
  dfree(t.perm);  dfree(t.unmasked);  dfree(t.bfraw); dfree(t.kdot); dfree(t.times);
  dfree(t.beta64); dfree(t.betabar); dfree(t.gambar); dfree(t.kap64); dfree(t.times64);
  dfree(t.bal); dfree(t.Vr);
  auto &s = h->s;
  dfree(s.Z); dfree(s.Yt); dfree(s.part); dfree(s.gpart); dfree(s.dred);
  h->bytes = 0;
}

inline uint64_t spread2(uint64_t v) {  // 32 bits -> even bit positions
  v &= 0xffffffffull;
  v = (v | (v << 16)) & 0x0000ffff0000ffffull;
  v = (v | (v << 8)) & 0x00ff00ff00ff00ffull;
  v = (v | (v << 4)) & 0x0f0f0f0f0f0f0f0full;
  v = (v | (v << 2)) & 0x3333333333333333ull;
  v = (v | (v << 1)) & 0x5555555555555555ull;
  return v;
}
inline uint64_t spread3(uint64_t v) {  // 21 bits -> every third bit
  v &= 0x1fffffull;
  v = (v | (v << 32)) & 0x1f00000000ffffull;
  v = (v | (v << 16)) & 0x1f0000ff0000ffull;
  v = (v | (v << 8)) & 0x100f00f00f00f00full;
  v = (v | (v << 4)) & 0x10c30c30c30c30c3ull;
  v = (v | (v << 2)) & 0x1249249249249249ull;
  return v;
}

// FP64 table kernels: the range-reduced anchor phases.
__global__ void k_table_A(const double *__restrict__ betabar,  // [nVt][R]
                          const double *__restrict__ kap64,    // [nSamPad][R]
                          float *__restrict__ A, int R, int nVt, int nSamPad, int nSam) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (int64_t)nVt * nSamPad) return;
  int vt = (int)(i / nSamPad), s = (int)(i % nSamPad);
  double a = 0.0;
  if (s < nSam)
    for (int l = 0; l < R; ++l) a = fma(betabar[(int64_t)vt * R + l], kap64[(int64_t)s * R + l], a);
  A[i] = (float)(a - rint(a));
}

__global__ void k_table_B(const double *__restrict__ beta64,    // [nVoxPad][R]
                          const double *__restrict__ gammabar,  // [nSt][R]
                          const int *__restrict__ perm, float *__restrict__ B, int R, int nSt,
                          int nVoxPad) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (int64_t)nSt * nVoxPad) return;
  int st = (int)(i / nVoxPad), p = (int)(i % nVoxPad);
  double b = 0.0;
  if (perm[p] >= 0)
    for (int l = 0; l < R; ++l) b = fma(beta64[(int64_t)p * R + l], gammabar[(int64_t)st * R + l], b);
  B[i] = (float)(b - rint(b));
}

bool valid_handle(const hoe_handle *h) { return h && h->magic == HOE_MAGIC; }

int check_usable(hoe_handle *h) {
  if (!valid_handle(h)) return fail(nullptr, HOE_ERR_ARG, "invalid handle");
  if (h->closed) return fail(h, HOE_ERR_CLOSED, "operator is closed");
  return HOE_OK;
}

int finish(hoe_handle *h, cudaError_t e, const char *what) {
  if (e == cudaSuccess) e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(h, e, what);
  return HOE_OK;
}

}  // namespace

namespace hoe {
void record_error(const char *msg) { g_err = msg; }
}  // namespace hoe

extern "C" {

const char *hoe_version(void) { return HOE_VERSION_STRING; }
int hoe_abi_version(void) { return HOE_ABI_VERSION; }

const char *hoe_last_error(const hoe_handle *h) {
  if (valid_handle(h) && !h->err.empty()) return h->err.c_str();
  return g_err.c_str();
}

int hoe_is_closed(const hoe_handle *h) { return valid_handle(h) ? h->closed : 1; }

}  // extern "C"

namespace {

// Host-side plan of an operator: tiling, anchors and the tables uploaded by
// hoe_create.  Built without touching the device (also used by hoe_plan).
struct Plan {
  hoe::Tables t;                                   // sizes (device pointers unused)
  std::vector<int> order, perm, unmasked;
  std::vector<double> beta64, gam64, betabar, gambar, kap64, bal, Vr;
  std::vector<float> dbeta, kappa, bfraw, kdot, times_f;
  std::vector<float> dbHi, dbLo, kpHi, kpLo;   // TF32 hi/lo, UMMA K-major tiles
  std::vector<float2> csm;
};

// Round to the nearest TF32 value (10 explicit mantissa bits, ties to even).
float tf32_round(float f) {
  uint32_t b;
  memcpy(&b, &f, 4);
  if ((b & 0x7f800000u) != 0x7f800000u) {
    b += 0x00000fffu + ((b >> 13) & 1u);
    b &= 0xffffe000u;
  }
  memcpy(&f, &b, 4);
  return f;
}

// Index of element (row, k) in a K-major no-swizzle TF32 table with KP columns:
// [row/8][k/4][row%8][k%4].
inline size_t tf32_index(size_t row, int k, int KP) {
  return ((row / 8) * (KP / 4) + (size_t)(k / 4)) * 32 + (row % 8) * 4 + (k % 4);
}

void split_tf32(const std::vector<double> &v, int n, int rank, int KP, size_t nPad,
                std::vector<float> &hi, std::vector<float> &lo, double scale = 1.0) {
  hi.assign(nPad * KP, 0.f);
  lo.assign(nPad * KP, 0.f);
  for (int i = 0; i < n; ++i)
    for (int k = 0; k < rank; ++k) {
      double x = scale * v[(size_t)i * rank + k];
      float h = tf32_round((float)x);
      float l = tf32_round((float)(x - (double)h));
      size_t o = tf32_index((size_t)i, k, KP);
      hi[o] = h;
      lo[o] = l;
    }
}

int make_plan(const hoe_desc *d, Plan &P) {
  if (!d) return fail(nullptr, HOE_ERR_ARG, "descriptor must not be NULL");
  if (d->abi_version != HOE_ABI_VERSION)
    return fail(nullptr, HOE_ERR_ARG, "descriptor ABI version %d, library %d", d->abi_version,
                HOE_ABI_VERSION);
  if (d->nTerm != 9 && d->nTerm != 16)
    return fail(nullptr, HOE_ERR_ARG, "kspha requires 9 or 16 terms, got %d", d->nTerm);
  if (d->has_concomitant != 0 && d->has_concomitant != 1)
    return fail(nullptr, HOE_ERR_ARG, "has_concomitant must be 0 or 1");
  if (d->nX <= 0 || d->nY <= 0 || d->nZ <= 0)
    return fail(nullptr, HOE_ERR_DIM, "grid sizes must be positive");
  int64_t nFull = (int64_t)d->nX * d->nY * d->nZ;
  if (nFull > (1ll << 30)) return fail(nullptr, HOE_ERR_DIM, "grid too large");
  if (d->nVox <= 0) return fail(nullptr, HOE_ERR_ARG, "mask must contain voxels");
  if (d->nVox > nFull) return fail(nullptr, HOE_ERR_DIM, "mask and grid");
  if (d->nSam <= 0 || d->nCha <= 0)
    return fail(nullptr, HOE_ERR_ARG, "samples and coils must be positive");
  if ((int64_t)d->nSam * d->nCha > (1ll << 31) - 1)
    return fail(nullptr, HOE_ERR_DIM, "nSam*nCha too large");
  if (d->engine != HOE_ENGINE_FP32_SIMT && d->engine != HOE_ENGINE_TC_BF16X3 && d->engine != HOE_ENGINE_AUTO)
    return fail(nullptr, HOE_ERR_ARG, "unknown engine %d", d->engine);
  if (!d->mask_idx || !d->bf || !d->kspha || !d->times)
    return fail(nullptr, HOE_ERR_ARG, "mask_idx, bf, kspha and times are required");
  if (!d->csm && d->nCha != 1)
    return fail(nullptr, HOE_ERR_ARG, "csm may be omitted only for one coil");
  for (int m = 0; m < d->nVox; ++m) {
    if (d->mask_idx[m] < 0 || d->mask_idx[m] >= nFull)
      return fail(nullptr, HOE_ERR_DIM, "mask index %d out of range", m);
    if (m > 0 && d->mask_idx[m] <= d->mask_idx[m - 1])
      return fail(nullptr, HOE_ERR_ARG, "mask indices must be strictly ascending");
  }
  if (d->tc_plan < 0 || d->tc_plan >= 5)
    return fail(nullptr, HOE_ERR_ARG, "tc_plan must be in 0..4");
  if (d->tc_plan > 0 && d->nCha > 16)
    return fail(nullptr, HOE_ERR_ARG, "tensor-core plans 1-4 serve up to 16 coils");
  if (d->reserved != 0) return fail(nullptr, HOE_ERR_ARG, "reserved must be 0");

  auto &t = P.t;
  t.nX = d->nX; t.nY = d->nY; t.nZ = d->nZ; t.nFull = (int)nFull;
  t.nSam = d->nSam; t.nCha = d->nCha; t.nTerm = d->nTerm;
  t.R0 = d->nTerm + 4 * d->has_concomitant;
  t.R = t.R0 + 1;
  t.nVox = d->nVox;
  t.nSt = (t.nSam + t.ST - 1) / t.ST;
  t.nVt = (t.nVox + t.VT - 1) / t.VT;
  t.nSamPad = t.nSt * t.ST;
  t.nVoxPad = t.nVt * t.VT;
  t.nChaPad = t.nCha <= 4 ? 4 : (t.nCha <= 8 ? 8 : (t.nCha + 15) / 16 * 16);
  t.hasKdot = d->kspha_dt != nullptr;
  const int R = t.R, R0 = t.R0;
  const int nVox = t.nVox, nSam = t.nSam;

  // ---- voxel order: Morton order of grid indices, chunks of VT voxels ----
  auto &order = P.order;
  order.assign(nVox, 0);
  {
    std::vector<uint64_t> code(nVox);
    for (int m = 0; m < nVox; ++m) {
      int64_t lin = d->mask_idx[m];
      uint64_t i = lin % t.nX, j = (lin / t.nX) % t.nY, k = lin / ((int64_t)t.nX * t.nY);
      code[m] = (t.nZ == 1) ? (spread2(i) | (spread2(j) << 1))
                            : (spread3(i) | (spread3(j) << 1) | (spread3(k) << 2));
    }
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(),
                     [&](int a, int b) { return code[a] < code[b]; });
  }

  // ---- beta / gamma in FP64, tile anchors (component midrange) ----
  auto &beta64 = P.beta64, &gam64 = P.gam64;
  auto &perm = P.perm;
  beta64.assign((size_t)t.nVoxPad * R, 0.0);
  gam64.assign((size_t)t.nSamPad * R, 0.0);
  perm.assign(t.nVoxPad, -1);
  {
    // grid points outside the mask: the adjoint writes zeros there
    std::vector<char> in(t.nFull, 0);
    for (int m = 0; m < nVox; ++m) in[d->mask_idx[m]] = 1;
    P.unmasked.clear();
    for (int g = 0; g < t.nFull; ++g)
      if (!in[g]) P.unmasked.push_back(g);
    t.nUnmasked = (int)P.unmasked.size();
  }
  for (int p = 0; p < nVox; ++p) {
    int m = order[p];
    perm[p] = d->mask_idx[m];
    for (int l = 0; l < R0; ++l) beta64[(size_t)p * R + l] = d->bf[(size_t)m + (size_t)l * nVox];
    beta64[(size_t)p * R + R0] = d->fieldmap ? d->fieldmap[m] : 0.0;
  }
  for (int s = 0; s < nSam; ++s) {
    for (int l = 0; l < R0; ++l) gam64[(size_t)s * R + l] = d->kspha[(size_t)l + (size_t)s * R0];
    gam64[(size_t)s * R + R0] = d->times[s];
  }
  for (size_t i = 0; i < beta64.size(); ++i)
    if (!std::isfinite(beta64[i])) return fail(nullptr, HOE_ERR_ARG, "bf/fieldmap must be finite");
  for (size_t i = 0; i < gam64.size(); ++i)
    if (!std::isfinite(gam64[i])) return fail(nullptr, HOE_ERR_ARG, "kspha/times must be finite");

  // ---- tile anchors ----
  // voxel tiles: the basis of the voxel nearest the tile's bounding-box centre
  // (grid index space) for the basis components, the midrange for the fieldmap
  auto &betabar = P.betabar, &gambar = P.gambar;
  betabar.assign((size_t)t.nVt * R, 0.0);
  gambar.assign((size_t)t.nSt * R, 0.0);
  for (int vt = 0; vt < t.nVt; ++vt) {
    int p0 = vt * t.VT, p1 = std::min(nVox, p0 + t.VT);
    int64_t lo[3] = {INT64_MAX, INT64_MAX, INT64_MAX}, hi[3] = {INT64_MIN, INT64_MIN, INT64_MIN};
    auto ijk = [&](int p, int64_t *c) {
      int64_t lin = perm[p];
      c[0] = lin % t.nX; c[1] = (lin / t.nX) % t.nY; c[2] = lin / ((int64_t)t.nX * t.nY);
    };
    for (int p = p0; p < p1; ++p) {
      int64_t c[3];
      ijk(p, c);
      for (int a = 0; a < 3; ++a) { lo[a] = std::min(lo[a], c[a]); hi[a] = std::max(hi[a], c[a]); }
    }
    int best = p0;
    double bestd = INFINITY;
    for (int p = p0; p < p1; ++p) {
      int64_t c[3];
      ijk(p, c);
      double dd = 0;
      for (int a = 0; a < 3; ++a) { double e = 2.0 * c[a] - (double)(lo[a] + hi[a]); dd += e * e; }
      if (dd < bestd) { bestd = dd; best = p; }
    }
    for (int l = 0; l < R0; ++l) betabar[(size_t)vt * R + l] = beta64[(size_t)best * R + l];
    double flo = INFINITY, fhi = -INFINITY;
    for (int p = p0; p < p1; ++p) { double v = beta64[(size_t)p * R + R0]; flo = std::min(flo, v); fhi = std::max(fhi, v); }
    betabar[(size_t)vt * R + R0] = 0.5 * (flo + fhi);
  }
  // sample tiles: component midrange
  for (int st = 0; st < t.nSt; ++st) {
    int s0 = st * t.ST, s1 = std::min(nSam, s0 + t.ST);
    for (int l = 0; l < R; ++l) {
      double lo = INFINITY, hi = -INFINITY;
      for (int s = s0; s < s1; ++s) { double v = gam64[(size_t)s * R + l]; lo = std::min(lo, v); hi = std::max(hi, v); }
      gambar[(size_t)st * R + l] = 0.5 * (lo + hi);
    }
  }

  // ---- residual vectors in FP64, balanced per component ----
  std::vector<double> db64((size_t)nVox * R);
  auto &kap64 = P.kap64;
  kap64.assign((size_t)t.nSamPad * R, 0.0);
  for (int p = 0; p < nVox; ++p)
    for (int l = 0; l < R; ++l)
      db64[(size_t)p * R + l] = beta64[(size_t)p * R + l] - betabar[(size_t)(p / t.VT) * R + l];
  for (int s = 0; s < nSam; ++s)
    for (int l = 0; l < R; ++l)
      kap64[(size_t)s * R + l] = gam64[(size_t)s * R + l] - gambar[(size_t)(s / t.ST) * R + l];
  auto &bal = P.bal;
  bal.assign(R, 1.0);
  for (int l = 0; l < R; ++l) {
    double a = 0, b = 0;
    for (int p = 0; p < nVox; ++p) a = std::max(a, std::fabs(db64[(size_t)p * R + l]));
    for (int s = 0; s < nSam; ++s) b = std::max(b, std::fabs(kap64[(size_t)s * R + l]));
    if (a > 0 && b > 0) bal[l] = std::sqrt(b / a);
  }
  // ---- reduced basis: Householder QR of the balanced dbeta, Jacobi SVD of R ----
  auto &Vr = P.Vr;  // [R][r] right singular vectors kept
  int rank = 0;
  {
    std::vector<double> A((size_t)nVox * R);  // column-major nVox x R
    for (int p = 0; p < nVox; ++p)
      for (int l = 0; l < R; ++l) A[(size_t)p + (size_t)l * nVox] = db64[(size_t)p * R + l] * bal[l];
    const int kmax = std::min(R, nVox);
    std::vector<double> v(nVox);
    for (int j = 0; j < kmax; ++j) {
      double *cj = &A[(size_t)j * nVox];
      double nrm = 0;
      for (int i = j; i < nVox; ++i) nrm += cj[i] * cj[i];
      nrm = std::sqrt(nrm);
      if (nrm == 0) continue;
      double alpha = cj[j] >= 0 ? -nrm : nrm;
      double vn = 0;
      for (int i = j; i < nVox; ++i) { v[i] = cj[i]; }
      v[j] -= alpha;
      for (int i = j; i < nVox; ++i) vn += v[i] * v[i];
      if (vn == 0) continue;
      for (int k = j + 1; k < R; ++k) {
        double *ck = &A[(size_t)k * nVox];
        double d = 0;
        for (int i = j; i < nVox; ++i) d += v[i] * ck[i];
        double tau = 2.0 * d / vn;
        for (int i = j; i < nVox; ++i) ck[i] -= tau * v[i];
      }
      cj[j] = alpha;
    }
    std::vector<double> W((size_t)R * R, 0.0), V((size_t)R * R, 0.0);  // row-major R x R
    for (int i = 0; i < kmax; ++i)
      for (int k = i; k < R; ++k) W[(size_t)i * R + k] = A[(size_t)i + (size_t)k * nVox];
    for (int i = 0; i < R; ++i) V[(size_t)i * R + i] = 1.0;
    for (int sweep = 0; sweep < 80; ++sweep) {
      double off = 0;
      for (int pp = 0; pp < R - 1; ++pp)
        for (int qq = pp + 1; qq < R; ++qq) {
          double al = 0, be = 0, ga = 0;
          for (int i = 0; i < R; ++i) {
            double wp = W[(size_t)i * R + pp], wq = W[(size_t)i * R + qq];
            al += wp * wp; be += wq * wq; ga += wp * wq;
          }
          if (ga == 0 || std::fabs(ga) <= 1e-15 * std::sqrt(al * be)) continue;
          off = std::max(off, std::fabs(ga) / std::sqrt(al * be));
          double zeta = (be - al) / (2 * ga);
          double tt = (zeta >= 0 ? 1.0 : -1.0) / (std::fabs(zeta) + std::sqrt(1 + zeta * zeta));
          double c = 1 / std::sqrt(1 + tt * tt), sn = c * tt;
          for (int i = 0; i < R; ++i) {
            double wp = W[(size_t)i * R + pp], wq = W[(size_t)i * R + qq];
            W[(size_t)i * R + pp] = c * wp - sn * wq;
            W[(size_t)i * R + qq] = sn * wp + c * wq;
            double vp = V[(size_t)i * R + pp], vq = V[(size_t)i * R + qq];
            V[(size_t)i * R + pp] = c * vp - sn * vq;
            V[(size_t)i * R + qq] = sn * vp + c * vq;
          }
        }
      if (off < 1e-15) break;
    }
    std::vector<std::pair<double, int>> sig(R);
    for (int k = 0; k < R; ++k) {
      double n2 = 0;
      for (int i = 0; i < R; ++i) n2 += W[(size_t)i * R + k] * W[(size_t)i * R + k];
      sig[k] = {std::sqrt(n2), k};
    }
    std::sort(sig.begin(), sig.end(), [](auto a, auto b) { return a.first > b.first; });
    double kmaxn = 0;
    for (int s = 0; s < nSam; ++s) {
      double n2 = 0;
      for (int l = 0; l < R; ++l) { double e = kap64[(size_t)s * R + l] / bal[l]; n2 += e * e; }
      kmaxn = std::max(kmaxn, std::sqrt(n2));
    }
    // keep every direction whose largest possible contribution exceeds 1e-9 cycles
    std::vector<int> keep;
    for (int k = 0; k < R; ++k)
      if (sig[k].first * kmaxn >= 1e-9 || keep.empty()) keep.push_back(sig[k].second);
    rank = (int)keep.size();
    Vr.assign((size_t)R * rank, 0.0);
    for (int l = 0; l < R; ++l)
      for (int k = 0; k < rank; ++k) Vr[(size_t)l * rank + k] = V[(size_t)l * R + keep[k]];
  }
  t.rank = rank;
  t.Rp = rank <= 8 ? 8 : (rank <= 12 ? 12 : (rank <= 16 ? 16 : 24));
  const int Rp = t.Rp;

  auto &dbeta = P.dbeta, &kappa = P.kappa;
  dbeta.assign((size_t)t.nVoxPad * Rp, 0.f);
  kappa.assign((size_t)t.nSamPad * Rp, 0.f);
  std::vector<double> dbr((size_t)nVox * rank), kpr((size_t)nSam * rank);
  for (int p = 0; p < nVox; ++p)
    for (int k = 0; k < rank; ++k) {
      double acc = 0;
      for (int l = 0; l < R; ++l) acc += db64[(size_t)p * R + l] * bal[l] * Vr[(size_t)l * rank + k];
      dbr[(size_t)p * rank + k] = acc;
      dbeta[(size_t)p * Rp + k] = (float)acc;
    }
  for (int s = 0; s < nSam; ++s)
    for (int k = 0; k < rank; ++k) {
      double acc = 0;
      for (int l = 0; l < R; ++l) acc += kap64[(size_t)s * R + l] / bal[l] * Vr[(size_t)l * rank + k];
      kpr[(size_t)s * rank + k] = acc;
      kappa[(size_t)s * Rp + k] = (float)acc;
    }
  t.KP = rank <= 8 ? 8 : (rank <= 16 ? 16 : 24);
  split_tf32(dbr, nVox, rank, t.KP, t.nVoxPad, P.dbHi, P.dbLo);
  // the tensor-core residual phase is formed in radians: 2*pi on the sample side
  split_tf32(kpr, nSam, rank, t.KP, t.nSamPad, P.kpHi, P.kpLo, 2.0 * M_PI);
  // worst-case residual magnitude over tile pairs (reported)
  {
    std::vector<double> dmx((size_t)t.nVt * rank, 0.0), kmx((size_t)t.nSt * rank, 0.0);
    for (int p = 0; p < nVox; ++p)
      for (int k = 0; k < rank; ++k) {
        double &m = dmx[(size_t)(p / t.VT) * rank + k];
        m = std::max(m, std::fabs(dbr[(size_t)p * rank + k]));
      }
    for (int s = 0; s < nSam; ++s)
      for (int k = 0; k < rank; ++k) {
        double &m = kmx[(size_t)(s / t.ST) * rank + k];
        m = std::max(m, std::fabs(kpr[(size_t)s * rank + k]));
      }
    double bound = 0.0;
    for (int vt = 0; vt < t.nVt; ++vt)
      for (int st = 0; st < t.nSt; ++st) {
        double b = 0.0;
        for (int k = 0; k < rank; ++k) b += dmx[(size_t)vt * rank + k] * kmx[(size_t)st * rank + k];
        bound = std::max(bound, b);
      }
    t.residBound = bound;
  }

  auto &bfraw = P.bfraw, &kdot = P.kdot, &times_f = P.times_f;
  bfraw.assign((size_t)t.nVoxPad * hoe::kRF, 0.f);
  kdot.assign((size_t)t.nSamPad * hoe::kRF, 0.f);
  times_f.assign(t.nSamPad, 0.f);
  for (int p = 0; p < nVox; ++p)
    for (int l = 0; l < R; ++l) bfraw[(size_t)p * hoe::kRF + l] = (float)beta64[(size_t)p * R + l];
  for (int s = 0; s < nSam; ++s) {
    if (d->kspha_dt)
      for (int l = 0; l < t.nTerm; ++l)
        kdot[(size_t)s * hoe::kRF + l] = (float)d->kspha_dt[(size_t)l + (size_t)s * t.nTerm];
    times_f[s] = (float)d->times[s];
  }
  auto &csm = P.csm;
  csm.assign((size_t)t.nVoxPad * t.nChaPad, make_float2(0.f, 0.f));
  for (int p = 0; p < nVox; ++p) {
    int m = order[p];
    for (int c = 0; c < t.nCha; ++c) {
      float2 v = make_float2(1.f, 0.f);
      if (d->csm) {
        size_t o = 2 * ((size_t)m + (size_t)c * nVox);
        v = make_float2((float)d->csm[o], (float)d->csm[o + 1]);
      }
      csm[(size_t)p * t.nChaPad + c] = v;
    }
  }

  return HOE_OK;
}

}  // namespace

extern "C" {

int hoe_create(hoe_handle **out, const hoe_desc *d) {
  if (!out) return fail(nullptr, HOE_ERR_ARG, "out must not be NULL");
  *out = nullptr;
  Plan P;
  int prc = make_plan(d, P);
  if (prc != HOE_OK) return prc;

  int ndev = 0;
  cudaError_t ce = cudaGetDeviceCount(&ndev);
  if (ce != cudaSuccess || ndev == 0) return fail(nullptr, HOE_ERR_CUDA, "no CUDA device");
  int dev = d->device;
  if (dev < 0) cudaGetDevice(&dev);
  if (dev < 0 || dev >= ndev) return fail(nullptr, HOE_ERR_ARG, "invalid visible GPU ID");

  hoe_handle *h = new hoe_handle();
  h->device = dev;
  DeviceGuard guard(dev);
  if (!guard.ok) {
    delete h;
    return fail(nullptr, HOE_ERR_CUDA, "cannot select device %d", dev);
  }
  cudaDeviceGetAttribute(&h->numSMs, cudaDevAttrMultiProcessorCount, dev);
  if (h->numSMs <= 0) h->numSMs = 148;

  auto &t = h->t;
  t = P.t;
  const int nSam = t.nSam;
  auto &dbeta = P.dbeta, &kappa = P.kappa, &bfraw = P.bfraw, &kdot = P.kdot, &times_f = P.times_f;
  auto &beta64 = P.beta64, &kap64 = P.kap64, &betabar = P.betabar, &gambar = P.gambar;
  auto &csm = P.csm;
  auto &perm = P.perm;

  // ---- split-K choice for the SIMT engine ----
  {
    int target = 4 * h->numSMs;
    int nCC = (t.nChaPad + 15) / 16;
    int sf = std::max(1, std::min(t.nVt, (target + t.nSt * nCC - 1) / (t.nSt * nCC)));
    int tps = (t.nVt + sf - 1) / sf;
    h->splitF = (t.nVt + tps - 1) / tps;
    int sa = std::max(1, std::min(t.nSt, (target + t.nVt * nCC - 1) / (t.nVt * nCC)));
    tps = (t.nSt + sa - 1) / sa;
    h->splitA = (t.nSt + tps - 1) / tps;
    h->tcPlan = d->tc_plan;
    if (d->split_hint > 0) {
      h->splitF = std::min(d->split_hint, t.nVt);
      h->splitA = std::min(d->split_hint, t.nSt);
    }
  }

  // ---- device allocations ----
  Allocator al(h);
  cudaError_t e = cudaSuccess;
  auto A = [&](cudaError_t r) { if (e == cudaSuccess) e = r; };
  A(al.alloc(&t.dbeta, dbeta.size()));
  A(al.alloc(&t.kappa, kappa.size()));
  A(al.alloc(&t.dbHi, P.dbHi.size()));
  A(al.alloc(&t.dbLo, P.dbLo.size()));
  A(al.alloc(&t.kpHi, P.kpHi.size()));
  A(al.alloc(&t.kpLo, P.kpLo.size()));
  A(al.alloc(&t.Atab, (size_t)t.nVt * t.nSamPad));
  A(al.alloc(&t.Btab, (size_t)t.nSt * t.nVoxPad));
  A(al.alloc(&t.csm, csm.size()));
  A(al.alloc(&t.perm, perm.size()));
  A(al.alloc(&t.unmasked, std::max<size_t>(P.unmasked.size(), 1)));
  A(al.alloc(&t.bfraw, bfraw.size()));
  A(al.alloc(&t.kdot, kdot.size()));
  A(al.alloc(&t.times, times_f.size()));
  A(al.alloc(&h->s.Z, (size_t)t.nVoxPad * t.nChaPad));
  A(al.alloc(&h->s.Yt, (size_t)t.nSamPad * t.nChaPad));
  h->s.partElems = std::max((size_t)h->splitF * t.nSamPad, (size_t)h->splitA * t.nVoxPad) * t.nChaPad;
  A(al.alloc(&h->s.part, h->s.partElems));
  A(al.alloc(&t.beta64, beta64.size()));
  A(al.alloc(&t.betabar, betabar.size()));
  A(al.alloc(&t.gambar, gambar.size()));
  A(al.alloc(&t.kap64, kap64.size()));
  A(al.alloc(&t.times64, (size_t)t.nSamPad));
  A(al.alloc(&t.bal, P.bal.size()));
  A(al.alloc(&t.Vr, std::max<size_t>(P.Vr.size(), 1)));
  if (e != cudaSuccess) {
    release_device(h);
    delete h;
    return cuda_fail(nullptr, e, "hoe_create: device allocation");
  }
  std::vector<double> times64(t.nSamPad, 0.0);
  for (int s = 0; s < nSam; ++s) times64[s] = d->times[s];
  auto H2D = [&](void *dst, const void *src, size_t bytes) { A(cudaMemcpy(dst, src, bytes, cudaMemcpyHostToDevice)); };
  if (e == cudaSuccess) {
    H2D(t.dbeta, dbeta.data(), dbeta.size() * sizeof(float));
    H2D(t.kappa, kappa.data(), kappa.size() * sizeof(float));
    H2D(t.dbHi, P.dbHi.data(), P.dbHi.size() * sizeof(float));
    H2D(t.dbLo, P.dbLo.data(), P.dbLo.size() * sizeof(float));
    H2D(t.kpHi, P.kpHi.data(), P.kpHi.size() * sizeof(float));
    H2D(t.kpLo, P.kpLo.data(), P.kpLo.size() * sizeof(float));
    H2D(t.csm, csm.data(), csm.size() * sizeof(float2));
    H2D(t.perm, perm.data(), perm.size() * sizeof(int));
    if (!P.unmasked.empty()) H2D(t.unmasked, P.unmasked.data(), P.unmasked.size() * sizeof(int));
    H2D(t.bfraw, bfraw.data(), bfraw.size() * sizeof(float));
    H2D(t.kdot, kdot.data(), kdot.size() * sizeof(float));
    H2D(t.times, times_f.data(), times_f.size() * sizeof(float));
    H2D(t.beta64, beta64.data(), beta64.size() * sizeof(double));
    H2D(t.kap64, kap64.data(), kap64.size() * sizeof(double));
    H2D(t.betabar, betabar.data(), betabar.size() * sizeof(double));
    H2D(t.gambar, gambar.data(), gambar.size() * sizeof(double));
    H2D(t.times64, times64.data(), times64.size() * sizeof(double));
    H2D(t.bal, P.bal.data(), P.bal.size() * sizeof(double));
    if (!P.Vr.empty()) H2D(t.Vr, P.Vr.data(), P.Vr.size() * sizeof(double));
  }
  if (e == cudaSuccess) {
    A(hoe::build_anchor_tables(h, 0));
    A(cudaDeviceSynchronize());
  }
  if (e != cudaSuccess) {
    release_device(h);
    delete h;
    return cuda_fail(nullptr, e, "hoe_create: model upload");
  }
  h->engine = d->engine;
  if (h->engine == HOE_ENGINE_AUTO)
    h->engine = hoe::tc_supported(h, nullptr) ? HOE_ENGINE_TC_BF16X3 : HOE_ENGINE_FP32_SIMT;
  if (h->engine == HOE_ENGINE_TC_BF16X3) {
    std::string why;
    if (!hoe::tc_supported(h, &why)) {
      release_device(h);
      delete h;
      return fail(nullptr, HOE_ERR_UNSUPPORTED, "tensor-core engine unavailable: %s", why.c_str());
    }
    cudaError_t te = hoe::tc_prepare(h);
    if (te != cudaSuccess) {
      release_device(h);
      delete h;
      return cuda_fail(nullptr, te, "hoe_create: tensor-core operands");
    }
  }
  *out = h;
  return HOE_OK;
}

int hoe_plan(const hoe_desc *d, hoe_info *o) {
  if (!o) return fail(nullptr, HOE_ERR_ARG, "output must not be NULL");
  Plan P;
  int rc = make_plan(d, P);
  if (rc != HOE_OK) return rc;
  const auto &t = P.t;
  memset(o, 0, sizeof(*o));
  o->nSam = t.nSam; o->nCha = t.nCha; o->nVox = t.nVox; o->nTermEff = t.R0; o->nFull = t.nFull;
  o->engine = d->engine;
  o->tile_samples = t.ST; o->tile_voxels = t.VT;
  o->n_sample_tiles = t.nSt; o->n_voxel_tiles = t.nVt;
  o->residual_rank = t.rank; o->residual_width = t.Rp;
  o->residual_phase_bound = t.residBound;
  o->tc_plan = d->tc_plan;
  o->tc_plans = d->nCha <= 16 ? 5 : 1;
  return HOE_OK;
}

int hoe_close(hoe_handle *h) {
  if (!valid_handle(h)) return fail(nullptr, HOE_ERR_ARG, "invalid handle");
  if (h->closed) return HOE_OK;
  DeviceGuard guard(h->device);
  cudaDeviceSynchronize();
  release_device(h);
  h->closed = 1;
  return HOE_OK;
}

void hoe_free(hoe_handle *h) {
  if (!valid_handle(h)) return;
  hoe_close(h);
  h->magic = 0;
  delete h;
}

int hoe_get_info(const hoe_handle *h, hoe_info *o) {
  if (!valid_handle(h) || !o) return fail(nullptr, HOE_ERR_ARG, "invalid handle or output");
  const auto &t = h->t;
  o->nSam = t.nSam; o->nCha = t.nCha; o->nVox = t.nVox; o->nTermEff = t.R0; o->nFull = t.nFull;
  o->engine = h->engine;
  o->tile_samples = t.ST; o->tile_voxels = t.VT;
  o->n_sample_tiles = t.nSt; o->n_voxel_tiles = t.nVt;
  o->split_forward = h->splitF; o->split_adjoint = h->splitA;
  o->residual_rank = t.rank; o->residual_width = t.Rp;
  o->residual_phase_bound = t.residBound;
  o->device_bytes = h->bytes + (int64_t)h->tc.bytes;
  o->tc_plan = h->tc.ready ? hoe::tc_get_plan(h) : h->tcPlan;
  o->tc_plans = t.nCha <= 16 ? 5 : 1;
  return HOE_OK;
}

int hoe_set_engine(hoe_handle *h, int32_t engine) {
  int rc = check_usable(h);
  if (rc) return rc;
  if (engine == HOE_ENGINE_AUTO)
    engine = hoe::tc_supported(h, nullptr) ? HOE_ENGINE_TC_BF16X3 : HOE_ENGINE_FP32_SIMT;
  if (engine == HOE_ENGINE_FP32_SIMT) { h->engine = engine; return HOE_OK; }
  if (engine != HOE_ENGINE_TC_BF16X3) return fail(h, HOE_ERR_ARG, "unknown engine %d", engine);
  std::string why;
  if (!hoe::tc_supported(h, &why))
    return fail(h, HOE_ERR_UNSUPPORTED, "tensor-core engine unavailable: %s", why.c_str());
  DeviceGuard guard(h->device);
  if (!h->tc.ready) {
    cudaError_t e = hoe::tc_prepare(h);
    if (e != cudaSuccess) return cuda_fail(h, e, "tensor-core operands");
  }
  h->engine = engine;
  return HOE_OK;
}

int hoe_set_timing(hoe_handle *h, int32_t enable) {
  int rc = check_usable(h);
  if (rc) return rc;
  DeviceGuard guard(h->device);
  if (enable && !h->ev[0]) {
    for (auto &e : h->ev) {
      cudaError_t ce = cudaEventCreate(&e);
      if (ce != cudaSuccess) { release_events(h); return cuda_fail(h, ce, "hoe_set_timing"); }
    }
  }
  h->timing = enable ? 1 : 0;
  return HOE_OK;
}

int hoe_get_timings(hoe_handle *h, hoe_timings *o) {
  int rc = check_usable(h);
  if (rc) return rc;
  if (!o) return fail(h, HOE_ERR_ARG, "output must not be NULL");
  memset(o, 0, sizeof(*o));
  o->launches = h->launches;
  if (!h->ev[0]) return HOE_OK;
  DeviceGuard guard(h->device);
  auto span = [&](int a, int b, float *out) {
    if (cudaEventQuery(h->ev[b]) == cudaErrorNotReady) cudaEventSynchronize(h->ev[b]);
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, h->ev[a], h->ev[b]) == cudaSuccess) *out = ms;
    cudaGetLastError();  // events never recorded report an error; not a failure here
  };
  span(hoe::EV_FK0, hoe::EV_FK1, &o->forward_kernel_ms);
  span(hoe::EV_AK0, hoe::EV_AK1, &o->adjoint_kernel_ms);
  span(hoe::EV_F0, hoe::EV_F1, &o->forward_total_ms);
  span(hoe::EV_A0, hoe::EV_A1, &o->adjoint_total_ms);
  return HOE_OK;
}

int hoe_check(hoe_handle *h, void *stream) {
  int rc = check_usable(h);
  if (rc) return rc;
  DeviceGuard guard(h->device);
  cudaError_t e = cudaStreamSynchronize((cudaStream_t)stream);
  if (e != cudaSuccess) return cuda_fail(h, e, "hoe_check");
  int *word = hoe::tc_error_word(h);
  if (word) {
    int v = 0;
    e = cudaMemcpy(&v, word, sizeof(int), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_fail(h, e, "hoe_check");
    if (v != 0) {
      cudaMemset(word, 0, sizeof(int));
      return fail(h, HOE_ERR_TIMEOUT, "a bounded device wait ran out (tensor-core pipeline)");
    }
  }
  return HOE_OK;
}

int hoe_coil_gram(const void *A, int32_t complex128, int64_t nObs, int32_t nCoil, int32_t center, double *G,
                  void *stream) {
  if (!A || !G) return fail(nullptr, HOE_ERR_ARG, "A must be a device pointer and G a host pointer");
  if (nObs < 1 || nCoil < 1 || nCoil > 128) return fail(nullptr, HOE_ERR_ARG, "need nObs >= 1 and 1 <= nCoil <= 128");
  std::vector<std::complex<double>> g;
  cudaError_t e = hoe::coil_gram(A, complex128 != 0, nObs, nCoil, center != 0, g, (cudaStream_t)stream);
  if (e != cudaSuccess) return cuda_fail(nullptr, e, "hoe_coil_gram");
  for (int i = 0; i < nCoil; ++i)
    for (int j = 0; j < nCoil; ++j) {
      const std::complex<double> v = g[(size_t)i * nCoil + j];
      G[2 * ((size_t)j * nCoil + i)] = v.real();
      G[2 * ((size_t)j * nCoil + i) + 1] = v.imag();
    }
  return HOE_OK;
}

int hoe_coil_fit(const void *A, int32_t complex128, int64_t nObs, int32_t nCoil, int32_t nVirtual,
                 double energyThreshold, const double *noiseCov, double scale, double *matrix, double *sv,
                 int32_t *rank, double *retained, void *stream) {
  if (!A || !matrix || !sv || !rank || !retained)
    return fail(nullptr, HOE_ERR_ARG, "A must be a device pointer; matrix, sv, rank and retained host pointers");
  std::string why;
  int r = 0;
  int rc = hoe::coil_fit(A, complex128 != 0, nObs, nCoil, nVirtual, energyThreshold, noiseCov, scale, matrix, sv, &r,
                         retained, &why, (cudaStream_t)stream);
  if (rc != HOE_OK) return fail(nullptr, rc, "%s", why.c_str());
  *rank = r;
  return HOE_OK;
}

int hoe_coil_apply(const void *a, int64_t n, int32_t nCoil, const void *M, int32_t nVirt, void *out, void *stream) {
  if (!a || !M || !out) return fail(nullptr, HOE_ERR_ARG, "a, M and out must be device pointers");
  if (n < 1 || nCoil < 1 || nCoil > 128 || nVirt < 1 || nVirt > nCoil)
    return fail(nullptr, HOE_ERR_ARG, "need n >= 1, 1 <= nCoil <= 128 and 1 <= nVirt <= nCoil");
  cudaError_t e = hoe::coil_apply((const float2 *)a, n, nCoil, (const float2 *)M, nVirt, (float2 *)out,
                                  (cudaStream_t)stream);
  return finish(nullptr, e, "hoe_coil_apply");
}

int hoe_autotune(hoe_handle *h, int32_t reps, hoe_tune_result *o, void *stream) {
  int rc = check_usable(h);
  if (rc) return rc;
  if (!o) return fail(h, HOE_ERR_ARG, "output must not be NULL");
  if (reps < 1) return fail(h, HOE_ERR_ARG, "reps must be >= 1");
  memset(o, 0, sizeof(*o));
  DeviceGuard guard(h->device);
  cudaStream_t st = (cudaStream_t)stream;
  const auto &t = h->t;
  float2 *x = nullptr, *y = nullptr, *xo = nullptr, *yo = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  cudaError_t e = cudaMalloc(&x, (size_t)t.nFull * sizeof(float2));
  if (e == cudaSuccess) e = cudaMalloc(&xo, (size_t)t.nFull * sizeof(float2));
  if (e == cudaSuccess) e = cudaMalloc(&y, (size_t)t.nSam * t.nCha * sizeof(float2));
  if (e == cudaSuccess) e = cudaMalloc(&yo, (size_t)t.nSam * t.nCha * sizeof(float2));
  if (e == cudaSuccess) e = cudaMemsetAsync(x, 0, (size_t)t.nFull * sizeof(float2), st);
  if (e == cudaSuccess) e = cudaMemsetAsync(y, 0, (size_t)t.nSam * t.nCha * sizeof(float2), st);
  if (e == cudaSuccess) e = cudaEventCreate(&e0);
  if (e == cudaSuccess) e = cudaEventCreate(&e1);
  const int savedTiming = h->timing;
  h->timing = 0;
  const int defF = h->splitF, defA = h->splitA, defEngine = h->engine;
  struct Cand { int engine, sf, sa, plan; };
  std::vector<Cand> cands;
  for (int div : {4, 2, 1}) {
    Cand c{HOE_ENGINE_FP32_SIMT, std::max(1, defF / div), std::max(1, defA / div), -1};
    bool dup = false;
    for (auto &k : cands) dup = dup || (k.sf == c.sf && k.sa == c.sa);
    if (!dup) cands.push_back(c);
  }
  std::string why;
  int defPlan = 0;
  if (hoe::tc_supported(h, &why)) {
    if (!h->tc.ready && e == cudaSuccess) {
      cudaError_t te = hoe::tc_prepare(h);
      if (te != cudaSuccess) cudaGetLastError();
    }
    if (h->tc.ready) {
      defPlan = hoe::tc_get_plan(h);
      for (int pl = 0; pl < hoe::tc_plan_count(h); ++pl) cands.push_back({HOE_ENGINE_TC_BF16X3, 0, 0, pl});
    }
  }
  float best = INFINITY;
  Cand bestC{defEngine, defF, defA, defPlan};
  float bestTc = INFINITY;
  int bestPlan = defPlan;
  for (size_t i = 0; i < cands.size() && e == cudaSuccess && i < 8; ++i) {
    const Cand &c = cands[i];
    h->engine = c.engine;
    if (c.engine == HOE_ENGINE_FP32_SIMT) { h->splitF = c.sf; h->splitA = c.sa; }
    else {
      h->splitF = defF; h->splitA = defA;
      if (hoe::tc_set_plan(h, c.plan) != cudaSuccess) {   // plan unavailable on this device
        cudaGetLastError();
        continue;
      }
    }
    auto run = [&]() {
      cudaError_t r = hoe::apply_forward(h, x, yo, st);
      if (r == cudaSuccess) r = hoe::apply_adjoint_weighted(h, y, nullptr, xo, st);
      return r;
    };
    e = run();  // warm-up
    if (e == cudaSuccess) e = cudaEventRecord(e0, st);
    for (int r = 0; r < reps && e == cudaSuccess; ++r) e = run();
    if (e == cudaSuccess) e = cudaEventRecord(e1, st);
    if (e == cudaSuccess) e = cudaEventSynchronize(e1);
    float ms = 0.f;
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
    ms /= (float)reps;
    const int k = o->candidates;
    o->cand_engine[k] = c.engine;
    o->cand_split[k] = c.engine == HOE_ENGINE_FP32_SIMT ? c.sf : 0;
    o->cand_plan[k] = c.plan;
    o->cand_ms[k] = ms;
    o->candidates = k + 1;
    if (e == cudaSuccess && ms < best) { best = ms; bestC = {c.engine, h->splitF, h->splitA, c.plan}; }
    if (e == cudaSuccess && c.engine == HOE_ENGINE_TC_BF16X3 && ms < bestTc) { bestTc = ms; bestPlan = c.plan; }
  }
  for (int k = o->candidates; k < 8; ++k) o->cand_plan[k] = -1;
  h->engine = bestC.engine;
  h->splitF = bestC.sf;
  h->splitA = bestC.sa;
  if (h->tc.ready) {
    // the fastest tensor-core plan stays selected, also when the FP32 engine won
    cudaError_t pe = hoe::tc_set_plan(h, bestPlan);
    if (pe != cudaSuccess && e == cudaSuccess) e = pe;
    h->tcPlan = bestPlan;
  }
  h->timing = savedTiming;
  o->engine = h->engine;
  o->split_forward = h->splitF;
  o->split_adjoint = h->splitA;
  o->tc_plan = h->tc.ready ? hoe::tc_get_plan(h) : h->tcPlan;
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  cudaFree(x); cudaFree(xo); cudaFree(y); cudaFree(yo);
  return finish(h, e, "hoe_autotune");
}

int hoe_forward(hoe_handle *h, const void *x, void *y, void *stream) {
  int rc = check_usable(h);
  if (rc) return rc;
  if (!x || !y) return fail(h, HOE_ERR_ARG, "x and y must be device pointers");
  DeviceGuard guard(h->device);
  cudaStream_t st = (cudaStream_t)stream;
  hoe::trace(h, hoe::EV_F0, st);
  cudaError_t e = hoe::apply_forward(h, (const float2 *)x, (float2 *)y, st);
  hoe::trace(h, hoe::EV_F1, st);
  return finish(h, e, "hoe_forward");
}

int hoe_adjoint(hoe_handle *h, const void *y, void *x, void *stream) {
  int rc = check_usable(h);
  if (rc) return rc;
  if (!x || !y) return fail(h, HOE_ERR_ARG, "x and y must be device pointers");
  DeviceGuard guard(h->device);
  cudaStream_t st = (cudaStream_t)stream;
  hoe::trace(h, hoe::EV_A0, st);
  cudaError_t e = hoe::apply_adjoint_weighted(h, (const float2 *)y, nullptr, (float2 *)x, st);
  hoe::trace(h, hoe::EV_A1, st);
  return finish(h, e, "hoe_adjoint");
}

int hoe_normal(hoe_handle *h, const float *D, const void *x, void *out, void *stream) {
  int rc = check_usable(h);
  if (rc) return rc;
  if (!x || !out) return fail(h, HOE_ERR_ARG, "x and out must be device pointers");
  DeviceGuard guard(h->device);
  cudaError_t e = hoe::apply_normal(h, D, (const float2 *)x, (float2 *)out, (cudaStream_t)stream);
  return finish(h, e, "hoe_normal");
}

int hoe_recon(hoe_handle *h, const void *data, const void *weights, void *x, const hoe_cg_params *p,
              hoe_cg_stats *stats, void *stream) {
  int rc = check_usable(h);
  if (rc) return rc;
  if (!data || !x) return fail(h, HOE_ERR_ARG, "data and x must be device pointers");
  if (!p) return fail(h, HOE_ERR_ARG, "solver parameters must not be NULL");
  if (p->iterations < 0) return fail(h, HOE_ERR_ARG, "iterations must be >= 0 (got %d)", p->iterations);
  if (!(p->rel_tol >= 0.0) || !std::isfinite(p->rel_tol))
    return fail(h, HOE_ERR_ARG, "rel_tol must be finite and >= 0");
  if (!(p->lambda >= 0.0) || !std::isfinite(p->lambda))
    return fail(h, HOE_ERR_ARG, "lambda must be finite and >= 0");
  DeviceGuard guard(h->device);
  cudaStream_t st = (cudaStream_t)stream;
  hoe::CgRequest r;
  r.iterations = p->iterations;
  r.use_graph = p->use_graph != 0;
  r.rel_tol = p->rel_tol;
  r.lambda = p->lambda;
  cudaError_t e = hoe::cg_solve(h, (const float2 *)data, (const float2 *)weights, (float2 *)x, r, st);
  if (e == cudaSuccess) e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(h, e, "hoe_recon");
  if (stats) {
    hoe::CgScalars S{};
    e = hoe::cg_read_stats(h, st, &S);
    if (e != cudaSuccess) return cuda_fail(h, e, "hoe_recon: reading the solver state");
    stats->iterations = S.iters;
    const int status = S.status[r.iterations & 1];
    stats->status = status;
    stats->residual0 = std::sqrt(S.zz0);
    stats->residual = std::sqrt(S.zz[r.iterations & 1]);
  }
  return HOE_OK;
}

int hoe_set_kspha(hoe_handle *h, const double *kspha, const double *kspha_dt, void *stream) {
  int rc = check_usable(h);
  if (rc) return rc;
  if (!kspha) return fail(h, HOE_ERR_ARG, "kspha must be a device pointer");
  DeviceGuard guard(h->device);
  cudaError_t e = hoe::replan_samples(h, kspha, h->t.R0, kspha_dt, h->t.nTerm, nullptr, (cudaStream_t)stream);
  return finish(h, e, "hoe_set_kspha");
}

int hoe_kdot_stencil(const double *traj, int64_t nField, int32_t nTerm, double dt, double *out, void *stream) {
  if (!traj || !out) return fail(nullptr, HOE_ERR_ARG, "traj and out must be device pointers");
  if (nField < 1 || nTerm < 1) return fail(nullptr, HOE_ERR_ARG, "nField and nTerm must be positive");
  if (!(dt > 0.0) || !std::isfinite(dt)) return fail(nullptr, HOE_ERR_ARG, "dt must be finite and positive");
  cudaError_t e = hoe::kdot_stencil(traj, nField, nTerm, dt, out, (cudaStream_t)stream);
  return finish(nullptr, e, "hoe_kdot_stencil");
}

int hoe_sfu_rate(double *lanes_per_clock_per_sm, void *stream) {
  if (!lanes_per_clock_per_sm) return fail(nullptr, HOE_ERR_ARG, "lanes_per_clock_per_sm must not be NULL");
  cudaError_t e = hoe::sfu_rate(lanes_per_clock_per_sm, (cudaStream_t)stream);
  return finish(nullptr, e, "hoe_sfu_rate");
}

int hoe_interp_traj_time(const double *traj, int64_t nField, int32_t nTerm, double dt, double delTime,
                         const double *datatime, int64_t nData, double *out, int32_t layout, void *stream) {
  if (!traj || !datatime || !out) return fail(nullptr, HOE_ERR_ARG, "traj, datatime and out must be device pointers");
  if (nField < 2 || nTerm < 1 || nData < 1)
    return fail(nullptr, HOE_ERR_ARG, "need nField >= 2, nTerm >= 1 and nData >= 1");
  if (!(dt > 0.0) || !std::isfinite(dt) || !std::isfinite(delTime))
    return fail(nullptr, HOE_ERR_ARG, "dt must be finite and positive, delTime finite");
  if (layout != 0 && layout != 1) return fail(nullptr, HOE_ERR_ARG, "layout must be 0 or 1");
  cudaError_t e = hoe::interp_akima(traj, nField, nTerm, dt, nullptr, delTime, datatime, nData, out, layout, nTerm,
                                    nullptr, (cudaStream_t)stream);
  return finish(nullptr, e, "hoe_interp_traj_time");
}

int hoe_find_delay(hoe_handle *h, const hoe_delay_params *p, const void *data, const void *weights,
                   const double *traj, int64_t nField, void *x, hoe_delay_result *out, void *stream) {
  int rc = check_usable(h);
  if (rc) return rc;
  if (!p || !out) return fail(h, HOE_ERR_ARG, "params and out must not be NULL");
  if (!data || !traj) return fail(h, HOE_ERR_ARG, "data and traj must be device pointers");
  if (h->t.R0 != h->t.nTerm)
    return fail(h, HOE_ERR_ARG, "delay estimation needs an operator without concomitant terms");
  if (nField < 2) return fail(h, HOE_ERR_ARG, "need at least two coefficient samples");
  if (!(p->dt > 0.0) || !std::isfinite(p->dt)) return fail(h, HOE_ERR_ARG, "dt must be finite and positive");
  if (!(p->dtau_min > 0.0) || !std::isfinite(p->dtau_min))
    return fail(h, HOE_ERR_ARG, "dtau_min must be finite and positive");
  if (!(p->jump_fact >= 1.0) || !std::isfinite(p->jump_fact)) return fail(h, HOE_ERR_ARG, "jump_fact must be >= 1");
  if (!(p->lambda >= 0.0) || !std::isfinite(p->lambda)) return fail(h, HOE_ERR_ARG, "lambda must be finite and >= 0");
  if (!std::isfinite(p->start_time)) return fail(h, HOE_ERR_ARG, "start_time must be finite");
  if (p->iter_max < 0 || p->max_outer < 1) return fail(h, HOE_ERR_ARG, "iter_max >= 0 and max_outer >= 1 required");
  DeviceGuard guard(h->device);
  memset(out, 0, sizeof(*out));
  cudaError_t e = hoe::find_delay(h, h, 1, nullptr, *p, (const float2 *)data, (const float2 *)weights, traj, nField,
                                  (float2 *)x, out, (cudaStream_t)stream);
  return finish(h, e, "hoe_find_delay");
}

int hoe_find_delay_multishot(hoe_handle *h, hoe_handle *h_resid, const hoe_delay_params *p, int32_t nShot,
                             const double *start_times, const void *data, const void *weights, const double *traj,
                             int64_t nField, void *x, hoe_delay_result *out, void *stream) {
  int rc = check_usable(h);
  if (rc) return rc;
  hoe_handle *hr = h_resid ? h_resid : h;
  if (hr != h && (rc = check_usable(hr)) != 0) return rc;
  if (!p || !out || !start_times) return fail(h, HOE_ERR_ARG, "params, start_times and out must not be NULL");
  if (!data || !traj) return fail(h, HOE_ERR_ARG, "data and traj must be device pointers");
  if (nShot < 1) return fail(h, HOE_ERR_ARG, "nShot must be positive");
  if (h->t.nSam % nShot != 0) return fail(h, HOE_ERR_DIM, "the operator's samples must split evenly into nShot shots");
  if (h->t.R0 != h->t.nTerm || hr->t.R0 != hr->t.nTerm)
    return fail(h, HOE_ERR_ARG, "delay estimation needs operators without concomitant terms");
  if (hr != h && (hr->device != h->device || hr->t.nSam != h->t.nSam || hr->t.nCha != h->t.nCha ||
                  hr->t.nTerm != h->t.nTerm || hr->t.nFull != h->t.nFull || hr->t.nVox != h->t.nVox))
    return fail(h, HOE_ERR_DIM, "h_resid must have the operator's device, samples, coils, terms and voxels");
  if (nField < 2) return fail(h, HOE_ERR_ARG, "need at least two coefficient samples");
  if (!(p->dt > 0.0) || !std::isfinite(p->dt)) return fail(h, HOE_ERR_ARG, "dt must be finite and positive");
  if (!(p->dtau_min > 0.0) || !std::isfinite(p->dtau_min))
    return fail(h, HOE_ERR_ARG, "dtau_min must be finite and positive");
  if (!(p->jump_fact >= 1.0) || !std::isfinite(p->jump_fact)) return fail(h, HOE_ERR_ARG, "jump_fact must be >= 1");
  if (!(p->lambda >= 0.0) || !std::isfinite(p->lambda)) return fail(h, HOE_ERR_ARG, "lambda must be finite and >= 0");
  for (int s = 0; s < nShot; ++s)
    if (!std::isfinite(start_times[s])) return fail(h, HOE_ERR_ARG, "start_times must be finite");
  if (p->iter_max < 0 || p->max_outer < 1) return fail(h, HOE_ERR_ARG, "iter_max >= 0 and max_outer >= 1 required");
  DeviceGuard guard(h->device);
  memset(out, 0, sizeof(*out));
  cudaError_t e = hoe::find_delay(h, hr, nShot, start_times, *p, (const float2 *)data, (const float2 *)weights, traj,
                                  nField, (float2 *)x, out, (cudaStream_t)stream);
  return finish(h, e, "hoe_find_delay_multishot");
}

}  // extern "C"

namespace hoe {

cudaError_t build_anchor_tables(const hoe_handle *h, cudaStream_t st) {
  const auto &t = h->t;
  int64_t nA = (int64_t)t.nVt * t.nSamPad, nB = (int64_t)t.nSt * t.nVoxPad;
  k_table_A<<<(unsigned)((nA + 255) / 256), 256, 0, st>>>(t.betabar, t.kap64, t.Atab, t.R, t.nVt, t.nSamPad,
                                                          t.nSam);
  k_table_B<<<(unsigned)((nB + 255) / 256), 256, 0, st>>>(t.beta64, t.gambar, t.perm, t.Btab, t.R, t.nSt,
                                                          t.nVoxPad);
  h->launches += 2;
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = tc_anchor_tables(h, st);
  return e;
}

cudaError_t apply_forward(hoe_handle *h, const float2 *x, float2 *y, cudaStream_t st) {
  if (h->engine == HOE_ENGINE_TC_BF16X3) return tc_forward(h, x, y, st);
  cudaError_t e = prep_Z(h, x, st);
  if (e == cudaSuccess) e = simt_forward(h, nullptr, y, nullptr, FWD_TO_Y, st);
  return e;
}

cudaError_t apply_derivative(hoe_handle *h, const float2 *x, float2 *y, cudaStream_t st) {
  if (h->engine == HOE_ENGINE_TC_BF16X3 && tc_derivative_supported(h)) return tc_derivative(h, x, y, st);
  cudaError_t e = prep_Z(h, x, st);
  if (e == cudaSuccess) e = simt_forward(h, nullptr, y, nullptr, FWD_DERIV_TO_Y, st);
  return e;
}

cudaError_t apply_normal(hoe_handle *h, const float *D, const float2 *x, float2 *out, cudaStream_t st) {
  if (h->engine == HOE_ENGINE_TC_BF16X3) return tc_normal(h, D, x, out, st);
  cudaError_t e = prep_Z(h, x, st);
  if (e == cudaSuccess) e = simt_forward(h, nullptr, nullptr, D, FWD_TO_YT_WEIGHTED, st);
  if (e == cudaSuccess) e = simt_adjoint_from_Yt(h, out, st);
  return e;
}

cudaError_t apply_adjoint_weighted(hoe_handle *h, const float2 *y, const float *D, float2 *x,
                                   cudaStream_t st) {
  if (h->engine == HOE_ENGINE_TC_BF16X3) return tc_adjoint(h, y, D, x, st);
  cudaError_t e = prep_Yt(h, y, D, st);
  if (e == cudaSuccess) e = simt_adjoint_from_Yt(h, x, st);
  return e;
}

}  // namespace hoe

extern "C" {

int hoe_derivative(hoe_handle *h, const void *x, void *y, void *stream) {
  int rc = check_usable(h);
  if (rc) return rc;
  if (!h->t.hasKdot) return fail(h, HOE_ERR_ARG, "operator was created without kspha_dt");
  if (!x || !y) return fail(h, HOE_ERR_ARG, "x and y must be device pointers");
  DeviceGuard guard(h->device);
  cudaStream_t st = (cudaStream_t)stream;
  const cudaError_t e = hoe::apply_derivative(h, (const float2 *)x, (float2 *)y, st);
  return finish(h, e, "hoe_derivative");
}

int hoe_backward(hoe_handle *h, const void *x, const void *r, float *dk, float *ddf, double *dt0,
                 int32_t flags, void *stream) {
  int rc = check_usable(h);
  if (rc) return rc;
  if (!x || !r) return fail(h, HOE_ERR_ARG, "x and r must be device pointers");
  if ((flags & HOE_GRAD_T0_COEF) && !h->t.hasKdot)
    return fail(h, HOE_ERR_ARG, "the coefficient part of dL/dt0 needs kspha_dt");
  if ((flags & HOE_GRAD_KSPHA) && !dk) return fail(h, HOE_ERR_ARG, "dk must be given");
  if ((flags & HOE_GRAD_FIELDMAP) && !ddf) return fail(h, HOE_ERR_ARG, "ddf must be given");
  if ((flags & (HOE_GRAD_T0_B0 | HOE_GRAD_T0_COEF)) && !dt0) return fail(h, HOE_ERR_ARG, "dt0 must be given");
  DeviceGuard guard(h->device);
  cudaStream_t st = (cudaStream_t)stream;
  cudaError_t e = cudaSuccess;
  if (h->engine == HOE_ENGINE_TC_BF16X3 && hoe::tc_backward_supported(h)) {
    e = hoe::tc_backward(h, (const float2 *)x, (const float2 *)r, dk, ddf, dt0, flags, st);
  } else if (h->t.nChaPad > 16) {
    return fail(h, HOE_ERR_UNSUPPORTED,
                "hoe_backward: the tensor-core backward covers up to 32 coils (residual width <= 16 above 16 "
                "coils), the FP32 backward up to 16 coils");
  } else {
    e = hoe::prep_Z(h, (const float2 *)x, st);
    if (e == cudaSuccess)
      e = hoe::simt_backward(h, (const float2 *)x, (const float2 *)r, dk, ddf, dt0, flags, st);
  }
  return finish(h, e, "hoe_backward");
}

}  // extern "C"
