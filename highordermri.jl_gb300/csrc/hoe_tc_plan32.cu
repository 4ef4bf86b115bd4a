// Execution plans 1-4 of the tensor-core contraction at coil width N = 32
// (9 to 16 coils), the candidates that hoe_autotune times besides the
// default plan (hoe_tc_kernel.cuh, TcPlan).  A translation unit of their own
// so that the build compiles them in parallel with the default instances.
#include "hoe_tc_kernel.cuh"

namespace hoe {

cudaError_t tc_launch_plan32(const hoe_handle *h, const TcParams<1> &p, int KP, int plan, int G, cudaStream_t st) {
  switch (KP) {
    case 8: return launch_plan_nk<32, 8>(h, p, plan, G, st);
    case 16: return launch_plan_nk<32, 16>(h, p, plan, G, st);
    default: return launch_plan_nk<32, 24>(h, p, plan, G, st);
  }
}

int tc_configure_plan32(int KP, int plan) {
  switch (KP) {
    case 8: return configure_plan_nk<32, 8>(plan);
    case 16: return configure_plan_nk<32, 16>(plan);
    default: return configure_plan_nk<32, 24>(plan);
  }
}

}  // namespace hoe
