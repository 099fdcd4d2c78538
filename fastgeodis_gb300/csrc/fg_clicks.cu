// Click rasterisation: the soft mask of an interactive request, written on
// the device in one pass.
//
// Interactive segmentation turns user clicks into a soft mask that is 0 at
// the seeds and 1 elsewhere (the reference's callers build it on the host;
// its benchmark and demos set a disk or ball of zeros around each seed).  A
// request's mask is written here directly from the click list: every voxel
// tests its squared distance to each click against radius^2 in integer
// arithmetic, so the result is exact and independent of the order of the
// clicks.  One write of 4 bytes per voxel, no reads.

#include <cuda_runtime.h>

#include <algorithm>
#include <string>

#include "fg_common.cuh"

namespace fgi {
namespace {

constexpr int kMaxClicks = 64;

struct ClickList {
  int n;
  int r2;  // radius squared
  int z[kMaxClicks], y[kMaxClicks], x[kMaxClicks];
};

__global__ void fg_click_mask_kernel(float *mask, int D, int H, int W, const ClickList cl) {
  const long long P = (long long)D * H * W;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < P; i += (long long)gridDim.x * blockDim.x) {
    const int w = (int)(i % W);
    const long long q = i / W;
    const int h = (int)(q % H), d = (int)(q / H);
    bool seed = false;
    for (int k = 0; k < cl.n; k++) {
      const long long dz = d - cl.z[k], dy = h - cl.y[k], dx = w - cl.x[k];
      seed = seed || (dz * dz + dy * dy + dx * dx <= cl.r2);
    }
    mask[i] = seed ? 0.0f : 1.0f;
  }
}

}  // namespace
}  // namespace fgi

extern "C" FG_API int fg_click_mask(float *mask, int D, int H, int W, const int *clicks, int n_clicks, int radius,
                                    void *stream) {
  using namespace fgi;
  if (D < 1 || H < 1 || W < 1 || n_clicks < 0 || radius < 0 || (n_clicks > 0 && !clicks) || !mask)
    return set_error(FG_ERR_INVALID_ARGUMENT, "click mask: bad arguments");
  if (n_clicks > kMaxClicks)
    return set_error(FG_ERR_UNSUPPORTED, "click mask: at most 64 clicks per call");
  if ((long long)radius * radius > (1LL << 30)) return set_error(FG_ERR_INVALID_ARGUMENT, "click mask: radius too large");
  ClickList cl{};
  cl.n = n_clicks;
  cl.r2 = radius * radius;
  for (int k = 0; k < n_clicks; k++) {
    cl.z[k] = clicks[3 * k];
    cl.y[k] = clicks[3 * k + 1];
    cl.x[k] = clicks[3 * k + 2];
  }
  const long long P = (long long)D * H * W;
  const int grid = (int)std::min<long long>((P + 255) / 256, 152LL * 16);
  fg_click_mask_kernel<<<grid, 256, 0, static_cast<cudaStream_t>(stream)>>>(mask, D, H, W, cl);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return set_error(FG_ERR_CUDA, cudaGetErrorString(e));
  return FG_OK;
}
