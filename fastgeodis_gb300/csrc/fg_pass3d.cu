// Sweep kernels for volumes (two-dimensional cross-section, 9-cell stencil).
#include "fg_pass.cuh"

namespace fgi {
int launch_pass_cross2(const PassArgs &a, const LaunchCfg &c, int M, int mode, bool wt, cudaStream_t s) {
  return launch_cross<2>(a, c, M, mode, wt, s);
}
}  // namespace fgi
