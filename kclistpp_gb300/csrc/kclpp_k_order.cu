// kclpp_k_order.cu -- instantiates the MODE_ORDER clique kernels (one translation
// unit per mode so that the library builds in parallel).
#include "kclpp_kernels.cuh"

namespace kclpp {
cudaError_t launch_order(int k, const TierLaunch &t, dev::PassArgs a, cudaStream_t st) {
  return launch_mode<dev::MODE_ORDER>(k, t, a, st);
}
}  // namespace kclpp
