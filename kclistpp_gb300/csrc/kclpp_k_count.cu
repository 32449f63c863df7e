// kclpp_k_count.cu -- instantiates the MODE_COUNT clique kernels (one translation
// unit per mode so that the library builds in parallel).
#include "kclpp_kernels.cuh"

namespace kclpp {
cudaError_t launch_count(int k, const TierLaunch &t, dev::PassArgs a, cudaStream_t st) {
  return launch_mode<dev::MODE_COUNT>(k, t, a, st);
}
}  // namespace kclpp
