// Tensor-core engine (tcgen05).  Placeholder until the UMMA kernels land:
// reports itself unavailable so that hoe_create/hoe_set_engine fail loudly.
#include "hoe_internal.cuh"

namespace hoe {

bool tc_supported(const hoe_handle *, std::string *why) {
  if (why) *why = "tensor-core kernels not built";
  return false;
}
cudaError_t tc_prepare(hoe_handle *) { return cudaErrorNotSupported; }
void tc_release(hoe_handle *h) { h->tc = TcState(); }
cudaError_t tc_forward(const hoe_handle *, const float2 *, float2 *, const float *, int, cudaStream_t) {
  return cudaErrorNotSupported;
}
cudaError_t tc_adjoint_from_Yt(const hoe_handle *, float2 *, cudaStream_t) {
  return cudaErrorNotSupported;
}

}  // namespace hoe
