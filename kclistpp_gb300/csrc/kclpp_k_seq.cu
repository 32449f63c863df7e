// kclpp_k_seq.cu -- instantiates the MODE_SEQ clique kernels (one translation
// unit per mode so that the library builds in parallel).
#include "kclpp_kernels.cuh"

namespace kclpp {
cudaError_t launch_seq(int k, const TierLaunch &t, dev::PassArgs a, cudaStream_t st) {
  return launch_mode<dev::MODE_SEQ>(k, t, a, st);
}
}  // namespace kclpp
