// hoe_coils.cu — SVD coil compression (src/Recon/CoilCompression.jl:150-353).
//
// The reference copies the calibration matrix A (observations x coils) to
// the CPU and takes svd(A*W), W the optional noise-whitening matrix.  Here the
// O(nObs * nCoil^2) part, the Gram matrix A^H A, is accumulated on the GPU in
// FP64 (column-centred for noise-covariance estimation); the nCoil-sized
// algebra runs on the host in FP64:
//   * W = sqrt(s) * inv(U), Psi = U^H U the Cholesky factorisation of the
//     noise covariance (CoilCompression.jl:150-183);
//   * the eigen-decomposition of the Hermitian W^H (A^H A) W by cyclic complex
//     Jacobi rotations: its eigenvalues are the squared singular values of A*W
//     and its eigenvectors the right singular vectors;
//   * rank by count or by the cumulative-energy threshold, compression matrix
//     W * V[:, 1:rank] (CoilCompression.jl:239-275).
// Applying the transform (CoilCompression.jl:289-301) is a small complex GEMM
// per observation, done on the GPU.
#include "hoe_internal.cuh"

#include <algorithm>
#include <cmath>
#include <complex>
#include <vector>

namespace hoe {
namespace {

using cd = std::complex<double>;
constexpr int kGramThreads = 256;
constexpr int kMaxCoils = 128;

template <class C>
__device__ __forceinline__ double2 load_c(const C *p, int64_t i);
template <>
__device__ __forceinline__ double2 load_c<float2>(const float2 *p, int64_t i) {
  float2 v = p[i];
  return make_double2(v.x, v.y);
}
template <>
__device__ __forceinline__ double2 load_c<double2>(const double2 *p, int64_t i) {
  return p[i];
}

// Column sums of A (nObs x nCoil, column-major) in FP64, one block per column.
template <class C>
__global__ void k_col_sums(const C *__restrict__ A, int64_t nObs, double2 *__restrict__ sums) {
  __shared__ double sre[kGramThreads], sim[kGramThreads];
  const int c = blockIdx.x;
  double re = 0.0, im = 0.0;
  for (int64_t i = threadIdx.x; i < nObs; i += kGramThreads) {
    double2 v = load_c(A, i + c * nObs);
    re += v.x;
    im += v.y;
  }
  sre[threadIdx.x] = re;
  sim[threadIdx.x] = im;
  __syncthreads();
  for (int o = kGramThreads / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) { sre[threadIdx.x] += sre[threadIdx.x + o]; sim[threadIdx.x] += sim[threadIdx.x + o]; }
    __syncthreads();
  }
  if (threadIdx.x == 0) sums[c] = make_double2(sre[0], sim[0]);
}

// Block partials of G = (A - 1 m^T)^H (A - 1 m^T) over row chunks: block b
// takes rows [b*rows, (b+1)*rows) and writes its upper-triangle partial; the
// pairs (i <= j) are taken in chunks of kPairsPerPass, a thread owning
// kPairsPerThread of them, and rows are staged kRowBatch at a time.
constexpr int kPairsPerThread = 8;
constexpr int kPairsPerPass = kPairsPerThread * kGramThreads;
constexpr int kRowBatch = 16;   // kRowBatch * kMaxCoils * 16 B = 32 KB of shared memory

template <class C>
__global__ void __launch_bounds__(kGramThreads) k_gram_partial(const C *__restrict__ A, int64_t nObs, int nCoil,
                                                               int64_t rows, const double2 *__restrict__ mean,
                                                               double2 *__restrict__ part) {
  extern __shared__ double2 srow[];  // [kRowBatch][nCoil]
  const int64_t r0 = (int64_t)blockIdx.x * rows, r1 = min(nObs, r0 + rows);
  const int nPairs = nCoil * (nCoil + 1) / 2;
  for (int pc = 0; pc < nPairs; pc += kPairsPerPass) {
    double2 acc[kPairsPerThread];
    int pi[kPairsPerThread], pj[kPairsPerThread];
#pragma unroll
    for (int k = 0; k < kPairsPerThread; ++k) {
      acc[k] = make_double2(0.0, 0.0);
      int rem = pc + threadIdx.x + k * kGramThreads, i = 0;
      if (rem < nPairs)
        while (rem >= nCoil - i) { rem -= nCoil - i; ++i; }
      pi[k] = i;
      pj[k] = i + rem;
    }
    for (int64_t base = r0; base < r1; base += kRowBatch) {
      const int nr = (int)min((int64_t)kRowBatch, r1 - base);
      __syncthreads();
      for (int e = threadIdx.x; e < kRowBatch * nCoil; e += kGramThreads) {
        const int rr = e % kRowBatch, c = e / kRowBatch;
        double2 v = make_double2(0.0, 0.0);
        if (rr < nr) {
          v = load_c(A, base + rr + (int64_t)c * nObs);
          if (mean) { v.x -= mean[c].x; v.y -= mean[c].y; }
        }
        srow[rr * nCoil + c] = v;
      }
      __syncthreads();
#pragma unroll
      for (int k = 0; k < kPairsPerThread; ++k) {
        if (pc + threadIdx.x + k * kGramThreads >= nPairs) break;
        double re = acc[k].x, im = acc[k].y;
        for (int rr = 0; rr < nr; ++rr) {
          const double2 a = srow[rr * nCoil + pi[k]], b = srow[rr * nCoil + pj[k]];
          re += a.x * b.x + a.y * b.y;   // conj(a) * b
          im += a.x * b.y - a.y * b.x;
        }
        acc[k] = make_double2(re, im);
      }
    }
#pragma unroll
    for (int k = 0; k < kPairsPerThread; ++k) {
      const int pidx = pc + threadIdx.x + k * kGramThreads;
      if (pidx < nPairs) part[(size_t)blockIdx.x * nPairs + pidx] = acc[k];
    }
  }
}

// Fixed-order sum of the block partials.
__global__ void k_gram_reduce(const double2 *__restrict__ part, int nBlocks, int nPairs, double2 *__restrict__ out) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= nPairs) return;
  double re = 0.0, im = 0.0;
  for (int b = 0; b < nBlocks; ++b) {
    const double2 v = part[(size_t)b * nPairs + p];
    re += v.x;
    im += v.y;
  }
  out[p] = make_double2(re, im);
}

// out[r + k*n] = sum_c a[r + c*n] * M[c + k*nCoil] (complex64, column-major);
// block (x, k) stages column k of M.
__global__ void k_cc_apply(const float2 *__restrict__ a, int64_t n, int nCoil, const float2 *__restrict__ M,
                           float2 *__restrict__ out) {
  __shared__ float2 sM[kMaxCoils];
  const int k = blockIdx.y;
  for (int c = threadIdx.x; c < nCoil; c += blockDim.x) sM[c] = M[c + (int64_t)k * nCoil];
  __syncthreads();
  const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= n) return;
  float re = 0.f, im = 0.f;
  for (int c = 0; c < nCoil; ++c) {
    const float2 v = a[r + (int64_t)c * n], m = sM[c];
    re = fmaf(v.x, m.x, fmaf(-v.y, m.y, re));
    im = fmaf(v.x, m.y, fmaf(v.y, m.x, im));
  }
  out[r + (int64_t)k * n] = make_float2(re, im);
}

// Cyclic complex Jacobi for a Hermitian matrix H (n x n, row-major): on
// return H's diagonal holds the eigenvalues and V (row-major, V[i*n+k] =
// component i of eigenvector k) the orthonormal eigenvectors.  Each rotation
// first turns H[p][q] real with a phase on column q, then applies the real
// Jacobi rotation that zeroes it.
void hermitian_jacobi(std::vector<cd> &H, std::vector<cd> &V, int n) {
  V.assign((size_t)n * n, cd(0.0, 0.0));
  for (int i = 0; i < n; ++i) V[(size_t)i * n + i] = 1.0;
  double fro = 0.0;
  for (const cd &h : H) fro += std::norm(h);
  fro = std::sqrt(fro);
  for (int sweep = 0; sweep < 100; ++sweep) {
    double off = 0.0;
    for (int p = 0; p < n; ++p)
      for (int q = p + 1; q < n; ++q) off = std::max(off, std::abs(H[(size_t)p * n + q]));
    if (off <= 1e-15 * fro || fro == 0.0) break;
    for (int p = 0; p < n - 1; ++p)
      for (int q = p + 1; q < n; ++q) {
        const cd a = H[(size_t)p * n + q];
        const double aa = std::abs(a);
        if (aa <= 1e-300 || aa <= 1e-17 * fro) continue;
        const cd e = std::conj(a) / aa;  // a * e = |a|
        const double app = H[(size_t)p * n + p].real(), aqq = H[(size_t)q * n + q].real();
        const double theta = (aqq - app) / (2.0 * aa);
        const double t = (theta >= 0 ? 1.0 : -1.0) / (std::fabs(theta) + std::sqrt(theta * theta + 1.0));
        const double c = 1.0 / std::sqrt(t * t + 1.0), s = t * c;
        // J = diag(1, e) * [[c, s], [-s, c]] on (p, q): H <- J^H H J, V <- V J
        for (int k = 0; k < n; ++k) {
          const cd hp = H[(size_t)k * n + p], hq = H[(size_t)k * n + q];
          H[(size_t)k * n + p] = c * hp - s * e * hq;
          H[(size_t)k * n + q] = s * hp + c * e * hq;
          const cd vp = V[(size_t)k * n + p], vq = V[(size_t)k * n + q];
          V[(size_t)k * n + p] = c * vp - s * e * vq;
          V[(size_t)k * n + q] = s * vp + c * e * vq;
        }
        for (int k = 0; k < n; ++k) {
          const cd hp = H[(size_t)p * n + k], hq = H[(size_t)q * n + k];
          H[(size_t)p * n + k] = c * hp - s * std::conj(e) * hq;
          H[(size_t)q * n + k] = s * hp + c * std::conj(e) * hq;
        }
        H[(size_t)p * n + q] = 0.0;
        H[(size_t)q * n + p] = 0.0;
        H[(size_t)p * n + p] = H[(size_t)p * n + p].real();
        H[(size_t)q * n + q] = H[(size_t)q * n + q].real();
      }
  }
}

}  // namespace

// G (nCoil x nCoil, row-major, complex128 host) = (A - 1 m^T)^H (A - 1 m^T),
// m the column means when center, else 0.
cudaError_t coil_gram(const void *A, int doubleInput, int64_t nObs, int nCoil, int center, std::vector<cd> &G,
                      cudaStream_t st) {
  const int nPairs = nCoil * (nCoil + 1) / 2;
  const int64_t rows = std::max<int64_t>(256, (nObs + 303) / 304);
  const int nBlocks = (int)((nObs + rows - 1) / rows);
  double2 *buf = nullptr;
  const size_t elems = (size_t)nBlocks * nPairs + nPairs + nCoil;
  cudaError_t e = cudaMalloc(&buf, elems * sizeof(double2));
  if (e != cudaSuccess) return e;
  double2 *part = buf, *out = buf + (size_t)nBlocks * nPairs, *sums = out + nPairs;
  double2 *mean = nullptr;
  const size_t smem = (size_t)kRowBatch * nCoil * sizeof(double2);
  if (center) {
    if (doubleInput) k_col_sums<double2><<<nCoil, kGramThreads, 0, st>>>((const double2 *)A, nObs, sums);
    else k_col_sums<float2><<<nCoil, kGramThreads, 0, st>>>((const float2 *)A, nObs, sums);
    mean = sums;
  }
  std::vector<double2> h(nPairs + nCoil);
  e = cudaGetLastError();
  if (e == cudaSuccess && center) {
    // column means on the host (nCoil values), back to the device
    std::vector<double2> s(nCoil);
    e = cudaMemcpyAsync(s.data(), sums, nCoil * sizeof(double2), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    for (auto &v : s) { v.x /= (double)nObs; v.y /= (double)nObs; }
    if (e == cudaSuccess) e = cudaMemcpyAsync(sums, s.data(), nCoil * sizeof(double2), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  }
  if (e == cudaSuccess) {
    if (doubleInput)
      k_gram_partial<double2><<<nBlocks, kGramThreads, smem, st>>>((const double2 *)A, nObs, nCoil, rows, mean, part);
    else
      k_gram_partial<float2><<<nBlocks, kGramThreads, smem, st>>>((const float2 *)A, nObs, nCoil, rows, mean, part);
    k_gram_reduce<<<(nPairs + 255) / 256, 256, 0, st>>>(part, nBlocks, nPairs, out);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpyAsync(h.data(), out, nPairs * sizeof(double2), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  cudaFree(buf);
  if (e != cudaSuccess) return e;
  G.assign((size_t)nCoil * nCoil, cd(0.0, 0.0));
  int pidx = 0;
  for (int i = 0; i < nCoil; ++i)
    for (int j = i; j < nCoil; ++j, ++pidx) {
      const cd v(h[pidx].x, h[pidx].y);
      G[(size_t)i * nCoil + j] = v;
      G[(size_t)j * nCoil + i] = std::conj(v);
    }
  for (int i = 0; i < nCoil; ++i) G[(size_t)i * nCoil + i] = G[(size_t)i * nCoil + i].real();
  return cudaSuccess;
}

// Fit (CoilCompression.jl:239-275).  Returns 0 or an HOE_ERR_* code with why.
int coil_fit(const void *A, int doubleInput, int64_t nObs, int nCoil, int nVirtual, double energyThreshold,
             const double *noiseCov, double scale, double *matrixOut, double *svOut, int *rankOut,
             double *retainedOut, std::string *why, cudaStream_t st) {
  if (nCoil < 1 || nCoil > kMaxCoils) { *why = "nCoil must be between 1 and 128"; return HOE_ERR_ARG; }
  if (nObs < 1) { *why = "calibration data must contain observations"; return HOE_ERR_ARG; }
  if ((nVirtual > 0) == (energyThreshold > 0)) {
    *why = "specify exactly one of n_virtual_coils and energy_threshold";
    return HOE_ERR_ARG;
  }
  if (!(std::isfinite(scale) && scale > 0.0)) { *why = "prewhitening_scale_factor must be finite and positive"; return HOE_ERR_ARG; }
  const int n = nCoil;
  // whitening W = sqrt(s) * inv(U), Psi = U^H U (U upper triangular)
  std::vector<cd> W((size_t)n * n, cd(0.0, 0.0));
  if (!noiseCov) {
    if (scale != 1.0) { *why = "prewhitening_scale_factor requires noise_covariance"; return HOE_ERR_ARG; }
    for (int i = 0; i < n; ++i) W[(size_t)i * n + i] = 1.0;
  } else {
    std::vector<cd> P((size_t)n * n);
    double nrm = 0.0;
    for (int i = 0; i < n * n; ++i) {
      P[i] = cd(noiseCov[2 * i], noiseCov[2 * i + 1]);  // column-major input: P[i] = Psi(i % n, i / n)
      if (!std::isfinite(P[i].real()) || !std::isfinite(P[i].imag())) { *why = "noise_covariance must contain only finite values"; return HOE_ERR_ARG; }
      nrm += std::norm(P[i]);
    }
    nrm = std::max(std::sqrt(nrm), 2.220446049250313e-16);
    // Hermitian check (rtol sqrt(eps), atol eps * norm), then symmetrise
    double diff = 0.0;
    for (int r = 0; r < n; ++r)
      for (int c = 0; c < n; ++c) diff += std::norm(P[(size_t)c * n + r] - std::conj(P[(size_t)r * n + c]));
    if (std::sqrt(diff) > 1.4901161193847656e-08 * nrm + 2.220446049250313e-16 * nrm) {
      *why = "noise_covariance must be Hermitian";
      return HOE_ERR_ARG;
    }
    std::vector<cd> Psi((size_t)n * n);  // row-major
    for (int r = 0; r < n; ++r)
      for (int c = 0; c < n; ++c)
        Psi[(size_t)r * n + c] = 0.5 * (P[(size_t)c * n + r] + std::conj(P[(size_t)r * n + c]));
    // Cholesky Psi = U^H U
    std::vector<cd> U((size_t)n * n, cd(0.0, 0.0));
    for (int j = 0; j < n; ++j) {
      cd d = Psi[(size_t)j * n + j];
      for (int k = 0; k < j; ++k) d -= std::conj(U[(size_t)k * n + j]) * U[(size_t)k * n + j];
      if (!(d.real() > 0.0) || !std::isfinite(d.real())) {
        *why = "noise_covariance must be positive definite; use more noise samples or regularize it explicitly";
        return HOE_ERR_ARG;
      }
      const double ujj = std::sqrt(d.real());
      U[(size_t)j * n + j] = ujj;
      for (int c = j + 1; c < n; ++c) {
        cd v = Psi[(size_t)j * n + c];
        for (int k = 0; k < j; ++k) v -= std::conj(U[(size_t)k * n + j]) * U[(size_t)k * n + c];
        U[(size_t)j * n + c] = v / ujj;
      }
    }
    // W = sqrt(s) * U^{-1} (back substitution per column)
    const double rs = std::sqrt(scale);
    for (int c = 0; c < n; ++c)
      for (int r = n - 1; r >= 0; --r) {
        cd v = (r == c) ? cd(1.0, 0.0) : cd(0.0, 0.0);
        for (int k = r + 1; k < n; ++k) v -= U[(size_t)r * n + k] * W[(size_t)k * n + c];
        W[(size_t)r * n + c] = v / U[(size_t)r * n + r];
      }
    for (auto &w : W) w *= rs;
  }
  std::vector<cd> G;
  cudaError_t e = coil_gram(A, doubleInput, nObs, n, 0, G, st);
  if (e != cudaSuccess) { *why = cudaGetErrorString(e); return HOE_ERR_CUDA; }
  for (const cd &g : G)
    if (!std::isfinite(g.real()) || !std::isfinite(g.imag())) { *why = "calibration_data must contain only finite values"; return HOE_ERR_ARG; }
  // H = W^H G W
  std::vector<cd> T((size_t)n * n, cd(0.0, 0.0)), H((size_t)n * n, cd(0.0, 0.0));
  for (int r = 0; r < n; ++r)
    for (int c = 0; c < n; ++c) {
      cd v(0.0, 0.0);
      for (int k = 0; k < n; ++k) v += G[(size_t)r * n + k] * W[(size_t)k * n + c];
      T[(size_t)r * n + c] = v;
    }
  for (int r = 0; r < n; ++r)
    for (int c = 0; c < n; ++c) {
      cd v(0.0, 0.0);
      for (int k = 0; k < n; ++k) v += std::conj(W[(size_t)k * n + r]) * T[(size_t)k * n + c];
      H[(size_t)r * n + c] = v;
    }
  std::vector<cd> V;
  hermitian_jacobi(H, V, n);
  std::vector<int> order(n);
  for (int i = 0; i < n; ++i) order[i] = i;
  std::stable_sort(order.begin(), order.end(),
                   [&](int a, int b) { return H[(size_t)a * n + a].real() > H[(size_t)b * n + b].real(); });
  const int maxRank = (int)std::min<int64_t>(nObs, n);
  double energy = 0.0;
  std::vector<double> sv(n, 0.0);
  for (int i = 0; i < n; ++i) {
    const double lam = std::max(0.0, H[(size_t)order[i] * n + order[i]].real());
    sv[i] = i < maxRank ? std::sqrt(lam) : 0.0;
  }
  for (int i = 0; i < maxRank; ++i) energy += sv[i] * sv[i];
  if (!(energy > 0.0)) { *why = "calibration_data must have nonzero signal energy"; return HOE_ERR_ARG; }
  int rank;
  if (nVirtual > 0) {
    if (nVirtual > maxRank) { *why = "n_virtual_coils must be between 1 and min(nObservation, nCoil)"; return HOE_ERR_ARG; }
    rank = nVirtual;
  } else {
    if (!(std::isfinite(energyThreshold) && energyThreshold > 0.0 && energyThreshold <= 1.0)) {
      *why = "energy_threshold must be finite and in (0, 1]";
      return HOE_ERR_ARG;
    }
    rank = maxRank;
    double cum = 0.0;
    for (int i = 0; i < maxRank; ++i) {
      cum += sv[i] * sv[i];
      if (cum >= energyThreshold * energy) { rank = i + 1; break; }
    }
  }
  double kept = 0.0;
  for (int i = 0; i < rank; ++i) kept += sv[i] * sv[i];
  // compression matrix W * V[:, order[0:rank]], column-major complex128
  for (int k = 0; k < rank; ++k)
    for (int r = 0; r < n; ++r) {
      cd v(0.0, 0.0);
      for (int j = 0; j < n; ++j) v += W[(size_t)r * n + j] * V[(size_t)j * n + order[k]];
      matrixOut[2 * ((size_t)k * n + r)] = v.real();
      matrixOut[2 * ((size_t)k * n + r) + 1] = v.imag();
    }
  for (int i = 0; i < maxRank; ++i) svOut[i] = sv[i];
  *rankOut = rank;
  *retainedOut = kept / energy;
  return HOE_OK;
}

cudaError_t coil_apply(const float2 *a, int64_t n, int nCoil, const float2 *M, int nVirt, float2 *out,
                       cudaStream_t st) {
  dim3 grid((unsigned)((n + 255) / 256), (unsigned)nVirt);
  k_cc_apply<<<grid, 256, 0, st>>>(a, n, nCoil, M, out);
  return cudaGetLastError();
}

}  // namespace hoe
