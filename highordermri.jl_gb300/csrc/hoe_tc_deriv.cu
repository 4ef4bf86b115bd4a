// Instances of the tensor-core contraction for the derivative product
// (kspha_dt mode, array_operator.jl:187-235) in one pass, up to 16 coils:
//   (B x)[s,c] = (1/sqrt(nVox)) sum_v 2 pi i F[s,v] e^{i2pi phi[s,v]} Z[v,c],
//   F[s,v] = sum_l kdot[l,s] bf[v,l]
// The phase warps form F with packed FP32x2 FMAs from the stage's basis tile
// and the row's kdot, and scale the phase tile by 2 pi i F before the BF16
// split; the rest is the forward kernel (hoe_tc_kernel.cuh).  The tables come
// from k_tc_deriv_tables.
#include "hoe_tc_kernel.cuh"

namespace hoe {
namespace {

// bfT[chunk][l][v] = bf[chunk*TV + v][l] (tile order, l < nTerm, else 0) and
// kd1[s][l] = 2 pi kdot[l][s] (l < nTerm, else 0).  Either table is skipped
// when its output is NULL.
__global__ void k_tc_deriv_tables(const float *__restrict__ bfraw, const float *__restrict__ kdot, int nVoxPad,
                                  int nSamPad, int nTerm, float *__restrict__ bfT, float *__restrict__ kd1) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t nB = bfT ? (int64_t)nVoxPad * KF : 0;
  if (i < nB) {
    const int ch = (int)(i / (KF * TV)), r = (int)(i % (KF * TV)), l = r / TV, v = r % TV;
    bfT[i] = l < nTerm ? bfraw[((int64_t)ch * TV + v) * kRF + l] : 0.f;
    return;
  }
  const int64_t j = i - nB;
  if (!kd1 || j >= (int64_t)nSamPad * KF) return;
  const int s = (int)(j / KF), l = (int)(j % KF);
  constexpr float kTwoPiF = 6.28318530717958647692f;
  kd1[j] = l < nTerm ? kTwoPiF * kdot[(int64_t)s * kRF + l] : 0.f;
}

}  // namespace

cudaError_t tc_deriv_tables(const hoe_handle *h, float *bfT, float *kd1, cudaStream_t st) {
  const auto &t = h->t;
  const int64_t n = (bfT ? (int64_t)t.nVoxPad * KF : 0) + (kd1 ? (int64_t)t.nSamPad * KF : 0);
  if (n == 0) return cudaSuccess;
  k_tc_deriv_tables<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(t.bfraw, t.kdot, t.nVoxPad, t.nSamPad, t.nTerm,
                                                                 bfT, kd1);
  h->launches += 1;
  return cudaGetLastError();
}

cudaError_t tc_launch_deriv(const hoe_handle *h, const TcParams<1> &p, int KP, int N, int G, cudaStream_t st) {
  switch (KP) {
    case 8: return launch_deriv_n<8>(h, p, N, G, st);
    case 16: return launch_deriv_n<16>(h, p, N, G, st);
    default: return launch_deriv_n<24>(h, p, N, G, st);
  }
}

int tc_configure_deriv(int KP, int N) {
  switch (KP) {
    case 8: return configure_deriv_n<8>(N);
    case 16: return configure_deriv_n<16>(N);
    default: return configure_deriv_n<24>(N);
  }
}

}  // namespace hoe
