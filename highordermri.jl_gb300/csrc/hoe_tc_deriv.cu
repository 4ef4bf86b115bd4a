// Instances of the tensor-core contraction for the derivative product
// (kspha_dt mode, array_operator.jl:187-235) in one pass, up to 16 coils:
//   (B x)[s,c] = (1/sqrt(nVox)) sum_v 2 pi i F[s,v] e^{i2pi phi[s,v]} Z[v,c],
//   F[s,v] = sum_l kdot[l,s] bf[v,l]
// The phase warps form F with packed FP32x2 FMAs from the stage's basis tile
// and the row's kdot, and scale the phase tile by 2 pi i F before the BF16
// split; the rest is the forward kernel (hoe_tc_kernel.cuh).
//
// F is formed in a reduced basis: with the basis columns normalised by D,
// bf D = U S V^T, and bf = (bf D V_r)(V_r^T D^-1) when r columns of V carry
// the whole range.  So F[s,v] = sum_{k < r} kd'[s,k] bf'[v,k] with
// bf' = bf D V_r and kd' = V_r^T D^-1 kdot.  On a 2-D slice the 16 solid harmonics span only the 10
// monomials of degree <= 3 in x and y (the z factors are constant), so r = 10
// and the phase warps do 10 instead of 16 multiply-adds per pair.  The
// voxel-side table is built on the host once per operator (tc_deriv_basis);
// kd' per call by k_tc_deriv_kdot, because hoe_set_kspha may replace kdot.
#include <cmath>
#include <vector>

#include "hoe_tc_kernel.cuh"

namespace hoe {
namespace {

// kd1[s][k] = 2 pi sum_{l < nTerm} M[l][k] kdot[s][l] for k < KF, with
// M = D^-1 V_r (zero beyond the reduced rank): the sample side of the reduced
// factor.
__global__ void k_tc_deriv_kdot(const float *__restrict__ kdot, const float *__restrict__ M, int nSamPad,
                                int nTerm, float *__restrict__ kd1) {
  const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= (int64_t)nSamPad * KF) return;
  const int s = (int)(j / KF), k = (int)(j % KF);
  float acc = 0.f;
  for (int l = 0; l < nTerm; ++l) acc = fmaf(M[l * KF + k], kdot[(int64_t)s * kRF + l], acc);
  kd1[j] = 6.28318530717958647692f * acc;
}

// Eigen-decomposition of a symmetric n x n matrix a (row-major, destroyed) by
// cyclic Jacobi rotations: eigenvalues in w, eigenvectors in the columns of v.
void jacobi_eigen(std::vector<double> &a, int n, std::vector<double> &w, std::vector<double> &v) {
  v.assign((size_t)n * n, 0.0);
  for (int i = 0; i < n; ++i) v[(size_t)i * n + i] = 1.0;
  for (int sweep = 0; sweep < 60; ++sweep) {
    double off = 0.0, tot = 0.0;
    for (int i = 0; i < n; ++i)
      for (int j = 0; j < n; ++j) {
        const double x = a[(size_t)i * n + j] * a[(size_t)i * n + j];
        tot += x;
        if (i != j) off += x;
      }
    if (off <= 1e-30 * tot || off == 0.0) break;
    for (int p = 0; p < n - 1; ++p)
      for (int q = p + 1; q < n; ++q) {
        const double apq = a[(size_t)p * n + q];
        if (apq == 0.0) continue;
        const double app = a[(size_t)p * n + p], aqq = a[(size_t)q * n + q];
        const double theta = (aqq - app) / (2.0 * apq);
        const double t = (theta >= 0 ? 1.0 : -1.0) / (std::fabs(theta) + std::sqrt(theta * theta + 1.0));
        const double c = 1.0 / std::sqrt(t * t + 1.0), sn = t * c;
        for (int k = 0; k < n; ++k) {   // columns p, q
          const double akp = a[(size_t)k * n + p], akq = a[(size_t)k * n + q];
          a[(size_t)k * n + p] = c * akp - sn * akq;
          a[(size_t)k * n + q] = sn * akp + c * akq;
        }
        for (int k = 0; k < n; ++k) {   // rows p, q
          const double apk = a[(size_t)p * n + k], aqk = a[(size_t)q * n + k];
          a[(size_t)p * n + k] = c * apk - sn * aqk;
          a[(size_t)q * n + k] = sn * apk + c * aqk;
        }
        for (int k = 0; k < n; ++k) {
          const double vkp = v[(size_t)k * n + p], vkq = v[(size_t)k * n + q];
          v[(size_t)k * n + p] = c * vkp - sn * vkq;
          v[(size_t)k * n + q] = sn * vkp + c * vkq;
        }
      }
  }
  w.resize(n);
  for (int i = 0; i < n; ++i) w[i] = a[(size_t)i * n + i];
}

}  // namespace

// The reduced basis of the derivative factor, once per operator: the voxel
// table bfT[chunk][k][v] = sum_l bf[v][l] (D V_r)[l][k] for k < kfd, the rank r
// rounded up to 6, 10 or 16 (uploaded; zero rows from r), and the
// sample-side matrix D^-1 V_r (uploaded to Mdev, KF x KF), with D the column
// normalisation and V_r the eigenvectors of the normalised Gram matrix whose
// eigenvalues exceed 1e-9 of the largest.  Returns r in *rank and the kernel
// instance's term count in *kfd.
cudaError_t tc_deriv_basis(const hoe_handle *h, float *bfT, float *Mdev, int *rank, int *kfd) {
  const auto &t = h->t;
  const int n = t.nTerm;
  std::vector<float> bf((size_t)t.nVoxPad * kRF);
  cudaError_t e = cudaMemcpy(bf.data(), t.bfraw, bf.size() * sizeof(float), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return e;
  std::vector<double> g((size_t)n * n, 0.0);
  for (int v = 0; v < t.nVoxPad; ++v)
    for (int i = 0; i < n; ++i) {
      const double bi = bf[(size_t)v * kRF + i];
      if (bi == 0.0) continue;
      for (int j = 0; j < n; ++j) g[(size_t)i * n + j] += bi * (double)bf[(size_t)v * kRF + j];
    }
  std::vector<double> d(n);
  for (int i = 0; i < n; ++i) d[i] = g[(size_t)i * n + i] > 0.0 ? 1.0 / std::sqrt(g[(size_t)i * n + i]) : 0.0;
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) g[(size_t)i * n + j] *= d[i] * d[j];
  std::vector<double> w, vec;
  jacobi_eigen(g, n, w, vec);
  std::vector<int> order(n);
  for (int i = 0; i < n; ++i) order[i] = i;
  std::sort(order.begin(), order.end(), [&](int a, int b) { return w[a] > w[b]; });
  const double wmax = n > 0 ? w[order[0]] : 0.0;
  int r = 0;
  while (r < n && w[order[r]] > 1e-9 * wmax) ++r;
  std::vector<float> M((size_t)KF * KF, 0.f);   // D^-1 V_r, sample side
  std::vector<double> Md((size_t)n * KF, 0.0);  // D V_r, voxel side
  for (int k = 0; k < r; ++k)
    for (int l = 0; l < n; ++l) {
      const double vlk = vec[(size_t)l * n + order[k]];
      Md[(size_t)l * KF + k] = d[l] * vlk;
      // a zero basis column (d = 0) contributes nothing on either side
      M[(size_t)l * KF + k] = d[l] > 0.0 ? (float)(vlk / d[l]) : 0.f;
    }
  // terms of the kernel instance: the rank rounded up to 6, 10 or 16 (zero
  // rows), the ranks of 2-D slices with 9 or 16 terms and of 3-D volumes
  const int kf = r <= 6 ? 6 : (r <= 10 ? 10 : 16);
  std::vector<float> tab((size_t)t.nVoxPad * kf, 0.f);
  for (int v = 0; v < t.nVoxPad; ++v) {
    const int ch = v / TV, vl = v % TV;
    for (int k = 0; k < r; ++k) {
      double acc = 0.0;
      for (int l = 0; l < n; ++l) acc += (double)bf[(size_t)v * kRF + l] * Md[(size_t)l * KF + k];
      tab[((size_t)ch * kf + k) * TV + vl] = (float)acc;
    }
  }
  e = cudaMemcpy(bfT, tab.data(), tab.size() * sizeof(float), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(Mdev, M.data(), M.size() * sizeof(float), cudaMemcpyHostToDevice);
  *rank = r;
  *kfd = kf;
  return e;
}

cudaError_t tc_deriv_kdot(const hoe_handle *h, const float *Mdev, float *kd1, cudaStream_t st) {
  const auto &t = h->t;
  const int64_t n = (int64_t)t.nSamPad * KF;
  k_tc_deriv_kdot<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(t.kdot, Mdev, t.nSamPad, t.nTerm, kd1);
  h->launches += 1;
  return cudaGetLastError();
}

cudaError_t tc_launch_deriv(const hoe_handle *h, const TcParams<1> &p, int KP, int N, int KFD, int G,
                            cudaStream_t st) {
#define HOE_DERIV_KFD(KPV)                                                       \
  return KFD == 6 ? launch_deriv_nk<KPV, 6>(h, p, N, G, st)                      \
       : KFD == 10 ? launch_deriv_nk<KPV, 10>(h, p, N, G, st)                    \
                   : launch_deriv_nk<KPV, 16>(h, p, N, G, st)
  switch (KP) {
    case 8: HOE_DERIV_KFD(8);
    case 16: HOE_DERIV_KFD(16);
    default: HOE_DERIV_KFD(24);
  }
#undef HOE_DERIV_KFD
}

int tc_configure_deriv(int KP, int N, int KFD) {
#define HOE_DERIV_KFD(KPV)                                                       \
  return KFD == 6 ? configure_deriv_nk<KPV, 6>(N)                                \
       : KFD == 10 ? configure_deriv_nk<KPV, 10>(N) : configure_deriv_nk<KPV, 16>(N)
  switch (KP) {
    case 8: HOE_DERIV_KFD(8);
    case 16: HOE_DERIV_KFD(16);
    default: HOE_DERIV_KFD(24);
  }
#undef HOE_DERIV_KFD
}

}  // namespace hoe
