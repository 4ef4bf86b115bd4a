// hoe_sync.cu — delay synchronisation and trajectory preprocessing on the device.
//
//   k̇ stencil        FindDelay.jl:179-180   conv(kspha, [1/8 1/4 0 -1/4 -1/8]')[3:end-2,:]/dt
//   InterpTrajTime   InterpTraj.jl:18-40    sample j at (j-1)*dt - delTime, Akima per column,
//                                           zero outside the shifted interval
//   sample re-plan   the operator rebuilds of FindDelay.jl:190-193, done on the device: the
//                    voxel side (basis, fieldmap, coil maps, reduced residual basis) is kept,
//                    the sample-tile anchors, residual vectors, TF32 tables and anchor-phase
//                    tables are recomputed from the new coefficients
//   FindDelay        FindDelay.jl:139-214   weighted CGNR image update, then
//                                           Δτ = J·Re(y2 \ y1), y1 = data − E x, y2 = B x
//
// Akima's interpolant (1970): slopes of the knot intervals, extended past both
// ends by linear extrapolation, knot tangents weighted by the slope
// differences on either side; cubic Hermite between knots.  The reference
// calls Interpolations.jl (AkimaMonotonicInterpolation) for this method.
#include "hoe_internal.cuh"

#include <cmath>
#include <vector>

namespace hoe {
namespace {

constexpr int kRmax = 32;
constexpr int kThreads = 256;
constexpr int kDotBlocks = 304;

__device__ __forceinline__ float tf32_round_dev(float f) {
  uint32_t b = __float_as_uint(f);
  if ((b & 0x7f800000u) != 0x7f800000u) {
    b += 0x00000fffu + ((b >> 13) & 1u);
    b &= 0xffffe000u;
  }
  return __uint_as_float(b);
}

__device__ __forceinline__ size_t tf32_index_dev(size_t row, int k, int KP) {
  return ((row / 8) * (KP / 4) + (size_t)(k / 4)) * 32 + (row % 8) * 4 + (k % 4);
}

// One block per sample tile, one thread per sample.
__global__ void __launch_bounds__(kTileS)
k_replan_samples(const double *__restrict__ kspha, int ldk, const double *__restrict__ kdot, int ldd,
                 const double *__restrict__ termMask, const double *__restrict__ times64,
                 const double *__restrict__ bal, const double *__restrict__ Vr, int R0, int R, int rank, int Rp,
                 int KP, int nTerm, int nSam, double *__restrict__ gambar, double *__restrict__ kap64,
                 float *__restrict__ kappa, float *__restrict__ kpHi, float *__restrict__ kpLo,
                 float *__restrict__ kdotT) {
  __shared__ double sLo[kTileS / 32], sHi[kTileS / 32];
  __shared__ double gb[kRmax];
  const int st = blockIdx.x, s = st * kTileS + threadIdx.x;
  const bool real = s < nSam;
  const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
  auto value = [&](int l) -> double {
    if (!real) return 0.0;
    if (l < R0) return kspha[(size_t)s * ldk + l] * (termMask ? termMask[l] : 1.0);
    return times64[s];
  };
  // component midrange over the tile's samples
  for (int l = 0; l < R; ++l) {
    const double v = value(l);
    double lo = real ? v : INFINITY, hi = real ? v : -INFINITY;
    for (int o = 16; o > 0; o >>= 1) {
      lo = fmin(lo, __shfl_down_sync(0xffffffffu, lo, o));
      hi = fmax(hi, __shfl_down_sync(0xffffffffu, hi, o));
    }
    if (lane == 0) { sLo[warp] = lo; sHi[warp] = hi; }
    __syncthreads();
    if (threadIdx.x == 0) {
      double a = sLo[0], b = sHi[0];
      for (int w = 1; w < kTileS / 32; ++w) { a = fmin(a, sLo[w]); b = fmax(b, sHi[w]); }
      gb[l] = 0.5 * (a + b);
    }
    __syncthreads();
  }
  if (threadIdx.x < R) gambar[(size_t)st * R + threadIdx.x] = gb[threadIdx.x];
  double kap[kRmax];
#pragma unroll 1
  for (int l = 0; l < R; ++l) {
    kap[l] = real ? value(l) - gb[l] : 0.0;
    kap64[(size_t)s * R + l] = kap[l];
  }
#pragma unroll 1
  for (int k = 0; k < rank; ++k) {
    double acc = 0.0;
    for (int l = 0; l < R; ++l) acc += kap[l] / bal[l] * Vr[(size_t)l * rank + k];
    kappa[(size_t)s * Rp + k] = (float)acc;
    // the tensor-core tables hold the sample side in radians
    const double accr = 6.283185307179586476925 * acc;
    const float h = tf32_round_dev((float)accr);
    const float lo = tf32_round_dev((float)(accr - (double)h));
    const size_t o = tf32_index_dev((size_t)s, k, KP);
    kpHi[o] = h;
    kpLo[o] = lo;
  }
  if (kdot)
    for (int l = 0; l < kRF; ++l)
      kdotT[(size_t)s * kRF + l] = (real && l < nTerm) ? (float)kdot[(size_t)s * ldd + l] : 0.f;
}

// out[:, l] = conv(traj[:, l], [1/8 1/4 0 -1/4 -1/8])[3:end-2] / dt, traj column-major (n x nTerm).
__global__ void k_kdot_stencil(const double *__restrict__ traj, int64_t n, int nTerm, double invDt,
                               double *__restrict__ out) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n * nTerm) return;
  const int64_t l = i / n, j = i % n;
  const double *y = traj + l * n;
  auto at = [&](int64_t q) { return (q >= 0 && q < n) ? y[q] : 0.0; };
  out[i] = (0.125 * at(j + 2) + 0.25 * at(j + 1) - 0.25 * at(j - 1) - 0.125 * at(j - 2)) * invDt;
}

// Akima slope of knot interval i (knots uniformly dt apart), extended past
// both ends by linear extrapolation.
__device__ double akima_slope(const double *y, int64_t n, double invDt, int64_t i) {
  auto m = [&](int64_t q) { return (y[q + 1] - y[q]) * invDt; };
  if (i >= 0 && i <= n - 2) return m(i);
  if (n == 2) return m(0);
  if (i == -1) return 2.0 * m(0) - m(1);
  if (i == -2) return 2.0 * (2.0 * m(0) - m(1)) - m(0);
  const double mn1 = 2.0 * m(n - 2) - m(n - 3);  // slope index n-1
  if (i == n - 1) return mn1;
  return 2.0 * mn1 - m(n - 2);                   // slope index n
}

__device__ double akima_tangent(const double *y, int64_t n, double invDt, int64_t i) {
  if (n == 2) return (y[1] - y[0]) * invDt;
  const double m2 = akima_slope(y, n, invDt, i - 2), m1 = akima_slope(y, n, invDt, i - 1);
  const double m0 = akima_slope(y, n, invDt, i), p1 = akima_slope(y, n, invDt, i + 1);
  const double w1 = fabs(p1 - m0), w2 = fabs(m1 - m2);
  return (w1 + w2 > 0.0) ? (w1 * m1 + w2 * m0) / (w1 + w2) : 0.5 * (m1 + m0);
}

// out = InterpTrajTime(traj, dt, delTime, datatime): layout 0 writes
// out[s + l*nData] (the reference's (nData, nTerm)), layout 1 writes
// out[l + s*ldo] (the operator's kspha, one sample's terms contiguous).
// delTime is *delTimeDev when given (read on the device), else delTimeHost.
__global__ void k_akima_eval(const double *__restrict__ traj, int64_t n, int nTerm, double dt,
                             const double *__restrict__ delTimeDev, double delTimeHost,
                             const double *__restrict__ datatime, int64_t nData, double *__restrict__ out,
                             int layout, int ldo, const double *__restrict__ termMask) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nData * nTerm) return;
  const int64_t s = i % nData;
  const int l = (int)(i / nData);
  const double del = (delTimeDev ? *delTimeDev : 0.0) + delTimeHost;   // device state plus a fixed offset
  const double *y = traj + (int64_t)l * n;
  const double t = datatime[s];
  const double x0 = -del, xl = (double)(n - 1) * dt - del;
  double v = 0.0;
  if (n >= 2 && t >= x0 && t <= xl) {
    const double invDt = 1.0 / dt;
    int64_t j = (int64_t)floor((t - x0) * invDt);
    j = j < 0 ? 0 : (j > n - 2 ? n - 2 : j);
    const double xj = (double)j * dt - del;
    const double u = (t - xj) * invDt;
    const double tj = akima_tangent(y, n, invDt, j), tj1 = akima_tangent(y, n, invDt, j + 1);
    const double h00 = (1.0 + 2.0 * u) * (1.0 - u) * (1.0 - u), h10 = u * (1.0 - u) * (1.0 - u);
    const double h01 = u * u * (3.0 - 2.0 * u), h11 = u * u * (u - 1.0);
    v = h00 * y[j] + h10 * dt * tj + h01 * y[j + 1] + h11 * dt * tj1;
  }
  if (termMask) v *= termMask[l];
  if (layout == 0) out[s + (int64_t)l * nData] = v;
  else out[(int64_t)l + s * ldo] = v;
}

// ---------------------------------------------------------------- FindDelay
struct DelayState {
  double tau, dtau, dtauPrev, J, delTime, result, num, den;
  int nIter, done, status, pad;
};
enum { DELAY_RUNNING = 0, DELAY_CONVERGED = 1, DELAY_DEGENERATE = 2 };

__device__ double block_sum256(double v) {
  __shared__ double sh[kThreads / 32];
  __shared__ double total;
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x < 32) {
    double r = threadIdx.x < kThreads / 32 ? sh[threadIdx.x] : 0.0;
    for (int o = 16; o > 0; o >>= 1) r += __shfl_down_sync(0xffffffffu, r, o);
    if (threadIdx.x == 0) total = r;
  }
  __syncthreads();
  double r = total;
  __syncthreads();
  return r;
}

// partials of Re(y2ᴴ y1) with y1 = data − yf, y2 = yd, and of ‖y2‖²
__global__ void __launch_bounds__(kThreads) k_delay_dots(const float2 *__restrict__ data,
                                                         const float2 *__restrict__ yf,
                                                         const float2 *__restrict__ yd, int64_t n,
                                                         const DelayState *S, double *__restrict__ part) {
  double a = 0.0, b = 0.0;
  if (!S->done)
    for (int64_t i = (int64_t)blockIdx.x * kThreads + threadIdx.x; i < n; i += (int64_t)gridDim.x * kThreads) {
      const float2 d = data[i], f = yf[i], g = yd[i];
      const double r1 = (double)d.x - f.x, i1 = (double)d.y - f.y;
      a += (double)g.x * r1 + (double)g.y * i1;
      b += (double)g.x * g.x + (double)g.y * g.y;
    }
  const double sa = block_sum256(a), sb = block_sum256(b);
  if (threadIdx.x == 0) {
    part[blockIdx.x] = sa;
    part[kDotBlocks + blockIdx.x] = sb;
  }
}

__device__ __forceinline__ int sgn(double v) { return (v > 0.0) - (v < 0.0); }

// The scalar update of FindDelay.jl:201-211.
__global__ void __launch_bounds__(kThreads) k_delay_update(const double *__restrict__ part, int G, DelayState *S,
                                                           double startTime, double dtauMin) {
  double a = 0.0, b = 0.0;
  for (int i = threadIdx.x; i < G; i += kThreads) { a += part[i]; b += part[kDotBlocks + i]; }
  const double num = block_sum256(a), den = block_sum256(b);
  if (threadIdx.x != 0 || S->done) return;
  S->num = num;
  S->den = den;
  if (!(den > 0.0) || !isfinite(num / den)) {
    S->status = DELAY_DEGENERATE;
    S->done = 1;
    return;
  }
  const double dtau = S->J * (num / den);
  S->tau += dtau;
  if (S->nIter > 1 && sgn(S->dtauPrev) != sgn(dtau)) S->J = fmax(1.0, S->J / 2.0);
  S->dtauPrev = dtau;
  S->dtau = dtau;
  S->nIter += 1;
  S->result = S->tau - dtau / S->J * (S->J - 1.0);
  S->delTime = startTime + S->tau;
  if (!(fabs(dtau) > dtauMin)) {
    S->status = DELAY_CONVERGED;
    S->done = 1;
  }
}

}  // namespace

cudaError_t replan_samples(hoe_handle *h, const double *kspha, int ldk, const double *kdot, int ldd,
                           const double *termMask, cudaStream_t st) {
  auto &t = h->t;
  k_replan_samples<<<t.nSt, kTileS, 0, st>>>(kspha, ldk, kdot, ldd, termMask, t.times64, t.bal, t.Vr, t.R0, t.R,
                                             t.rank, t.Rp, t.KP, t.nTerm, t.nSam, t.gambar, t.kap64, t.kappa,
                                             t.kpHi, t.kpLo, t.kdot);
  h->launches += 1;
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = build_anchor_tables(h, st);
  if (e == cudaSuccess && kdot) t.hasKdot = 1;
  return e;
}

cudaError_t kdot_stencil(const double *traj, int64_t n, int nTerm, double dt, double *out, cudaStream_t st) {
  const int64_t N = n * nTerm;
  k_kdot_stencil<<<(unsigned)((N + 255) / 256), 256, 0, st>>>(traj, n, nTerm, 1.0 / dt, out);
  return cudaGetLastError();
}

cudaError_t interp_akima(const double *traj, int64_t n, int nTerm, double dt, const double *delTimeDev,
                         double delTimeHost, const double *datatime, int64_t nData, double *out, int layout,
                         int ldo, const double *termMask, cudaStream_t st) {
  const int64_t N = nData * nTerm;
  k_akima_eval<<<(unsigned)((N + 255) / 256), 256, 0, st>>>(traj, n, nTerm, dt, delTimeDev, delTimeHost,
                                                            datatime, nData, out, layout, ldo, termMask);
  return cudaGetLastError();
}

// FindDelay on the device.  The operator h (no concomitant terms, times =
// the ADC times) is re-planned in place at every outer iteration.
//
// nShot > 1 (FindDelay_multishot.jl:65-158): h holds all shots' samples
// shot-major (sample j of shot s at s*nSPI + j, nSPI = nSam / nShot) and traj
// one coefficient series per shot, [nField x nTerm] column-major, shots
// consecutive.  Shot s is interpolated at delay tau + startTimes[s] (host
// array) with its own k-dot stencil; q.start_time is not used.  The image
// update uses h; the residual and derivative products use hr (h, or an
// operator with the same model on other ADC times: the reference builds its
// per-shot operators on the concatenated time vector, so every shot gets the
// first shot's times).  nShot == 1 is FindDelay.jl:139-214 with q.start_time.
cudaError_t find_delay(hoe_handle *h, hoe_handle *hr, int nShot, const double *startTimes,
                       const hoe_delay_params &q, const float2 *data, const float2 *weights,
                       const double *traj, int64_t nField, float2 *xOut, hoe_delay_result *res, cudaStream_t st) {
  auto &t = h->t;
  const int nTerm = t.nTerm;
  const int64_t nD = (int64_t)t.nSam * t.nCha;
  const bool multi = startTimes != nullptr;
  const int nSPI = t.nSam / nShot;
  const int64_t trajStride = nField * nTerm;
  // delTime state: start + tau for one shot, tau (plus each shot's start
  // time, passed per launch) for several
  const double base = multi ? 0.0 : q.start_time;
  // scratch
  size_t bytes = 0;
  auto add = [&](size_t b) { size_t o = bytes; bytes += (b + 255) & ~(size_t)255; return o; };
  const size_t oKd = add((size_t)nShot * nField * nTerm * sizeof(double));
  const size_t oKs = add((size_t)t.nSam * nTerm * sizeof(double));
  const size_t oKdt = add((size_t)t.nSam * nTerm * sizeof(double));
  const size_t oYf = add((size_t)nD * sizeof(float2));
  const size_t oYd = add((size_t)nD * sizeof(float2));
  const size_t oX = add((size_t)t.nFull * sizeof(float2));
  const size_t oP = add(2 * kDotBlocks * sizeof(double));
  const size_t oS = add(sizeof(DelayState));
  const size_t oM = add(kRmax * sizeof(double));
  char *buf = nullptr;
  cudaError_t e = cudaMalloc(&buf, bytes);
  if (e != cudaSuccess) return e;
  double *kd = (double *)(buf + oKd), *ks = (double *)(buf + oKs), *kdt = (double *)(buf + oKdt);
  float2 *yf = (float2 *)(buf + oYf), *yd = (float2 *)(buf + oYd);
  float2 *x = xOut ? xOut : (float2 *)(buf + oX);
  double *part = (double *)(buf + oP), *mask = (double *)(buf + oM);
  DelayState *S = (DelayState *)(buf + oS);
  DelayState S0{};
  S0.tau = 0.0;
  S0.dtau = INFINITY;
  S0.dtauPrev = INFINITY;
  S0.J = q.jump_fact;
  S0.delTime = base;
  S0.result = 0.0;
  S0.nIter = 1;
  std::vector<double> hm(kRmax, 1.0);
  for (int l = 0; l < nTerm; ++l) hm[l] = q.term_mask ? q.term_mask[l] : 1.0;
  cudaGraphExec_t exec = nullptr;
  cudaStream_t cap = nullptr;
  const int G = (int)std::min<int64_t>(kDotBlocks, std::max<int64_t>(1, (nD + kThreads - 1) / kThreads));
  CgRequest r;
  r.iterations = q.iter_max;
  r.use_graph = 0;
  r.rel_tol = 0.0;
  r.lambda = q.lambda;
  const int savedTiming = h->timing;
  auto cleanup = [&]() {
    h->timing = savedTiming;
    if (exec) cudaGraphExecDestroy(exec);
    if (cap) cudaStreamDestroy(cap);
    cudaFree(buf);
  };
  e = cudaMemcpyAsync(S, &S0, sizeof(S0), cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(mask, hm.data(), kRmax * sizeof(double), cudaMemcpyHostToDevice, st);
  for (int s = 0; s < nShot && e == cudaSuccess; ++s)
    e = kdot_stencil(traj + s * trajStride, nField, nTerm, q.dt, kd + s * trajStride, st);
  if (e == cudaSuccess) e = cg_prepare(h);
  // the replan below supplies kspha_dt, so the tensor-core derivative runs
  // in the captured iteration: its buffers are allocated before the capture
  if (e == cudaSuccess && hr->engine == HOE_ENGINE_TC_BF16X3 && hr->tc.ready) e = tc_derivative_prepare(hr);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);  // host staging above must be consumed
  if (e != cudaSuccess) { cleanup(); return e; }

  // one outer iteration, captured once and replayed
  auto enqueue = [&](cudaStream_t s) -> cudaError_t {
    cudaError_t err = cudaSuccess;
    for (int sh = 0; sh < nShot && err == cudaSuccess; ++sh) {
      const double off = multi ? startTimes[sh] : 0.0;
      const int64_t o = (int64_t)sh * nSPI;
      err = interp_akima(traj + sh * trajStride, nField, nTerm, q.dt, &S->delTime, off, t.times64 + o, nSPI,
                         ks + o * nTerm, 1, nTerm, nullptr, s);
      if (err == cudaSuccess)
        err = interp_akima(kd + sh * trajStride, nField, nTerm, q.dt, &S->delTime, off, t.times64 + o, nSPI,
                           kdt + o * nTerm, 1, nTerm, nullptr, s);
      h->launches += 2;
    }
    if (err == cudaSuccess) err = replan_samples(h, ks, nTerm, kdt, nTerm, mask, s);
    if (err == cudaSuccess && hr != h) err = replan_samples(hr, ks, nTerm, kdt, nTerm, mask, s);
    if (err == cudaSuccess) err = cg_enqueue(h, data, weights, x, r, s);
    if (err == cudaSuccess) err = apply_forward(hr, x, yf, s);
    if (err == cudaSuccess) err = apply_derivative(hr, x, yd, s);
    if (err == cudaSuccess) {
      k_delay_dots<<<G, kThreads, 0, s>>>(data, yf, yd, nD, S, part);
      k_delay_update<<<1, kThreads, 0, s>>>(part, G, S, base, q.dtau_min);
      h->launches += 2;
      err = cudaGetLastError();
    }
    return err;
  };
  h->timing = 0;
  const int savedTimingR = hr->timing;
  hr->timing = 0;
  e = cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking);
  if (e == cudaSuccess) {
    const int64_t l0 = h->launches, lr0 = hr->launches;
    e = cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal);
    cudaError_t eq = e == cudaSuccess ? enqueue(cap) : e;
    cudaGraph_t g = nullptr;
    if (e == cudaSuccess) e = cudaStreamEndCapture(cap, &g);
    const int64_t per = h->launches - l0 + (hr != h ? hr->launches - lr0 : 0);
    h->launches = l0;
    if (hr != h) hr->launches = lr0;
    if (eq != cudaSuccess) e = eq;
    if (e == cudaSuccess) e = cudaGraphInstantiate(&exec, g, 0);
    if (g) cudaGraphDestroy(g);
    DelayState Sh{};
    int outer = 0;
    while (e == cudaSuccess) {
      e = cudaGraphLaunch(exec, st);
      if (e != cudaSuccess) break;
      h->launches += per;
      ++outer;
      e = cudaMemcpyAsync(&Sh, S, sizeof(Sh), cudaMemcpyDeviceToHost, st);
      if (e == cudaSuccess) e = cudaStreamSynchronize(st);
      if (e != cudaSuccess || Sh.done || outer >= q.max_outer) break;
    }
    if (e == cudaSuccess) {
      res->tau = Sh.result;
      res->tau_last = Sh.tau;
      res->dtau = Sh.dtau;
      res->jump = Sh.J;
      res->iterations = Sh.nIter - 1;
      res->status = Sh.done ? (Sh.status == DELAY_CONVERGED ? 0 : 2) : 1;
    }
  }
  cudaGetLastError();
  hr->timing = savedTimingR;
  cleanup();
  return e;
}

}  // namespace hoe
