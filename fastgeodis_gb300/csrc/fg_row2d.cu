// Whole 2D transforms of small images (both sides up to FG_ONE_LAUNCH_SIDE)
// in one launch of one CTA, one thread per cell of a row (fg_row2d.cuh).

#include <math.h>

#include <algorithm>
#include <type_traits>

#include "fg_row2d.cuh"

namespace fgi {
namespace {

// One image's whole transform: initial distances and transpose, `iterations`
// x 4 passes (along H forward / backward writing [W][H], along W forward /
// backward writing [H][W]), and the signed difference.
template <int C, int M, int MODE>
__global__ void __launch_bounds__(512, 1)
    fg_row2d_kernel(const fg_batch2d_item it, int iterations, int S, float r2, int *status) {
  extern __shared__ __align__(16) float sm[];
  __shared__ PassArgs s_args;
  const int H = it.H, W = it.W;
  const long long Pn = (long long)H * W;
  if (Pn <= 0) return;
  batch_prologue(it, 0, M, MODE != MODE_EUCLID, sm);  // the Euclidean passes read no image
  __threadfence();
  __syncthreads();
  for (int iter = 0; iter < iterations; iter++) {
    for (int k = 0; k < 4; k++) {
      const int L = k >= 2 ? W : H;
      const bool wt = k & 1;
      if (L <= 1 && !wt) continue;
      if (threadIdx.x == 0) batch_pass_args(it, M, 0, k, S, 2, r2, status, &s_args);
      __syncthreads();
      if (wt)
        row_pass<C, M, MODE, true>(s_args, sm);
      else
        row_pass<C, M, MODE, false>(s_args, sm);
      __threadfence();
      __syncthreads();
    }
  }
  if (M == 2) {
    float *out = it.out;
    const float *d2 = it.d2;
    for (long long p = threadIdx.x; p < Pn; p += blockDim.x) out[p] = __fsub_rn(out[p], d2[p]);
  }
}

}  // namespace

int launch_image_one(const fg_batch2d_item &it, bool is_signed, int iterations, int *status, cudaStream_t s) {
  const int ext = std::max(it.H, it.W);
  if (it.C < 1 || it.C > kMaxChannels || ext > kOneLaunchSide)
    return set_error(FG_ERR_UNSUPPORTED, "one-launch image transform: 1 to 4 channels, sides up to 512");
  const int M = is_signed ? 2 : 1;
  const int NT = std::max(32, (ext + 31) / 32 * 32);
  const int S = 8;  // rows per write-back
  const size_t smem = std::max(row_smem(it.C, M, ext, S), (size_t)(NT / 32) * 32 * 33 * 4);
  if (smem > kBatchSmemLimit) return set_error(FG_ERR_UNSUPPORTED, "one-launch image transform: shared memory");
  const float r2 = (float)sqrt(2.0);  // fastgeodis_cpu.cpp:67
  auto launch = [&](auto fn) -> int {
    cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return set_error(FG_ERR_CUDA, cudaGetErrorString(e));
    fn<<<1, NT, smem, s>>>(it, std::max(iterations, 0), S, r2, status);
    e = cudaGetLastError();
    return e == cudaSuccess ? FG_OK : set_error(FG_ERR_CUDA, cudaGetErrorString(e));
  };
  const int mode = it.l_grad == 0.0f ? MODE_EUCLID : (it.l_eucl == 0.0f && it.l_grad == 1.0f ? MODE_GEO : MODE_GENERAL);
  if (mode == MODE_EUCLID)
    return is_signed ? launch(fg_row2d_kernel<1, 2, MODE_EUCLID>) : launch(fg_row2d_kernel<1, 1, MODE_EUCLID>);
  auto by_c = [&](auto md) -> int {
    constexpr int MD = decltype(md)::value;
    switch (it.C) {
      case 1: return is_signed ? launch(fg_row2d_kernel<1, 2, MD>) : launch(fg_row2d_kernel<1, 1, MD>);
      case 2: return is_signed ? launch(fg_row2d_kernel<2, 2, MD>) : launch(fg_row2d_kernel<2, 1, MD>);
      case 3: return is_signed ? launch(fg_row2d_kernel<3, 2, MD>) : launch(fg_row2d_kernel<3, 1, MD>);
      default: return is_signed ? launch(fg_row2d_kernel<4, 2, MD>) : launch(fg_row2d_kernel<4, 1, MD>);
    }
  };
  return mode == MODE_GEO ? by_c(std::integral_constant<int, MODE_GEO>{})
                          : by_c(std::integral_constant<int, MODE_GENERAL>{});
}

}  // namespace fgi
