// Sweep kernels for volumes on cluster plans (one thread-block cluster owns
// the whole cross-section; neighbour rows travel through distributed shared
// memory).
#include "fg_pass.cuh"

namespace fgi {
int launch_pass_cluster(const PassArgs &a, const LaunchCfg &c, int M, int mode, bool wt, cudaStream_t s) {
  return launch_cross<2, true>(a, c, M, mode, wt, s);
}
}  // namespace fgi
