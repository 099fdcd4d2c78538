// The cluster sweep kernel's variants (fg_cluster.cuh): volume passes that
// read at most one image channel, 2 runs of 4 cells per thread.
#include "fg_cluster.cuh"

namespace fgi {
namespace {

template <int CT, int M, int MODE, int RPT>
int launch_sweep(const PassArgs &a, const LaunchCfg &c, cudaStream_t s) {
  static unsigned long long configured = 0;  // bit per device (set under the engine's launch lock)
  if (c.threads > kThreads) return set_error(FG_ERR_UNSUPPORTED, "a cluster sweep CTA has at most 512 threads");
  return launch_one_cluster((const void *)fg_sweep_cluster_kernel<CT, M, MODE, RPT>, configured, a, c, s);
}

template <int CT, int M, int MODE>
int launch_rpt(const PassArgs &a, const LaunchCfg &c, cudaStream_t s) {
  if (c.rpt == 2) return launch_sweep<CT, M, MODE, 2>(a, c, s);
  return set_error(FG_ERR_UNSUPPORTED, "a cluster sweep thread owns 2 runs");
}

// one image channel (or none read): images with more channels take the pass
// kernel's cluster path (their channel rows would not fit the registers)
template <int M>
int launch_sweep_mode(const PassArgs &a, const LaunchCfg &c, int mode, cudaStream_t s) {
  if (mode == MODE_EUCLID) return launch_rpt<1, M, MODE_EUCLID>(a, c, s);
  if (a.C != 1) return set_error(FG_ERR_UNSUPPORTED, "the cluster sweep kernel reads one image channel");
  if (mode == MODE_GEO) return launch_rpt<1, M, MODE_GEO>(a, c, s);
  return launch_rpt<1, M, MODE_GENERAL>(a, c, s);
}

}  // namespace

// How many clusters of `size` CTAs (threads, smem each) of the cluster sweep
// kernel the current device co-schedules (cudaOccupancyMaxActiveClusters).
int cluster_capacity(int size, int threads, size_t smem, int *out) {
  const void *fn = (const void *)fg_sweep_cluster_kernel<1, 1, MODE_GENERAL, 2>;
  cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024);
  if (e == cudaSuccess) e = cudaFuncSetAttribute(fn, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
  if (e != cudaSuccess) return set_error(FG_ERR_CUDA, cudaGetErrorString(e));
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(size);
  cfg.blockDim = dim3(threads);
  cfg.dynamicSmemBytes = smem;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = size;
  at[0].val.clusterDim.y = 1;
  at[0].val.clusterDim.z = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  int n = 0;
  e = cudaOccupancyMaxActiveClusters(&n, fn, &cfg);
  if (e != cudaSuccess) {
    (void)cudaGetLastError();
    return set_error(FG_ERR_CUDA, cudaGetErrorString(e));
  }
  *out = n;
  return FG_OK;
}

// A cluster plan changes layout as an in-place pass followed by a transpose
// (the engine's pass generator): no variant here writes transposed.
int launch_sweep_cluster(const PassArgs &a, const LaunchCfg &c, int M, int mode, bool wt, cudaStream_t s) {
  if (wt) return set_error(FG_ERR_UNSUPPORTED, "cluster plans do not write transposed");
  if (M == 1) return launch_sweep_mode<1>(a, c, mode, s);
  if (M == 2) return launch_sweep_mode<2>(a, c, mode, s);
  return set_error(FG_ERR_UNSUPPORTED, "a pass updates one or two distance maps");
}

}  // namespace fgi
