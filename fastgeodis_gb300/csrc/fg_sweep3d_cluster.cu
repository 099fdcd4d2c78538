// The cluster sweep kernel's variants (fg_cluster.cuh): volume passes that
// read at most one image channel, 2 runs of 4 cells per thread.
#include "fg_cluster.cuh"

namespace fgi {
namespace {

template <int CT, int M, int MODE, bool WT, int RPT>
int launch_sweep(const PassArgs &a, const LaunchCfg &c, cudaStream_t s) {
  static unsigned long long configured = 0;  // bit per device (set under the engine's launch lock)
  if (c.threads > kThreads) return set_error(FG_ERR_UNSUPPORTED, "a cluster sweep CTA has at most 512 threads");
  return launch_one_cluster((const void *)fg_sweep_cluster_kernel<CT, M, MODE, WT, RPT>, configured, a, c, s);
}

template <int CT, int M, int MODE, bool WT>
int launch_rpt(const PassArgs &a, const LaunchCfg &c, cudaStream_t s) {
  if (c.rpt == 2) return launch_sweep<CT, M, MODE, WT, 2>(a, c, s);
  return set_error(FG_ERR_UNSUPPORTED, "a cluster sweep thread owns 2 runs");
}

// one image channel (or none read): images with more channels take the pass
// kernel's cluster path (their channel rows would not fit the registers)
template <int M, bool WT>
int launch_sweep_mode(const PassArgs &a, const LaunchCfg &c, int mode, cudaStream_t s) {
  if (mode == MODE_EUCLID) return launch_rpt<1, M, MODE_EUCLID, WT>(a, c, s);
  if (a.C != 1) return set_error(FG_ERR_UNSUPPORTED, "the cluster sweep kernel reads one image channel");
  if (mode == MODE_GEO) return launch_rpt<1, M, MODE_GEO, WT>(a, c, s);
  return launch_rpt<1, M, MODE_GENERAL, WT>(a, c, s);
}

}  // namespace

int launch_sweep_cluster(const PassArgs &a, const LaunchCfg &c, int M, int mode, bool wt, cudaStream_t s) {
  if (M == 1) return wt ? launch_sweep_mode<1, true>(a, c, mode, s) : launch_sweep_mode<1, false>(a, c, mode, s);
  if (M == 2) return wt ? launch_sweep_mode<2, true>(a, c, mode, s) : launch_sweep_mode<2, false>(a, c, mode, s);
  return set_error(FG_ERR_UNSUPPORTED, "a pass updates one or two distance maps");
}

}  // namespace fgi
