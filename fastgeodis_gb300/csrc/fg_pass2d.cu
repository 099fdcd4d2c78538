// Sweep kernels for 2D images (one-dimensional cross-section, 3-cell stencil).
#include "fg_pass.cuh"

namespace fgi {
int launch_pass_cross1(const PassArgs &a, const LaunchCfg &c, int M, int mode, bool wt, cudaStream_t s) {
  return launch_cross<1>(a, c, M, mode, wt, s);
}
}  // namespace fgi
