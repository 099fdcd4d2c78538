// Volume passes on cluster plans: one thread-block cluster owns the whole
// cross-section and neighbour rows travel through distributed shared memory.
// Runs per thread 0: the pass kernel's body (one run per thread, up to 1024
// threads); 2: the cluster sweep kernel (fg_sweep3d_cluster.cu).
#include "fg_pass.cuh"

namespace fgi {
int launch_pass_cluster(const PassArgs &a, const LaunchCfg &c, int M, int mode, bool wt, cudaStream_t s) {
  if (c.rpt != 0) return launch_sweep_cluster(a, c, M, mode, wt, s);
  return launch_cross<2, true>(a, c, M, mode, wt, s);
}
}  // namespace fgi
