// Tiled images of a batched 2D transform.
//
// In the persistent batched launch (fg_batch.cu) one CTA sweeps a whole
// image, so the batch lasts at least as long as its longest image's chain of
// 2 * iterations * (H + W) row steps over rows of up to 2048 cells.  The few
// images whose one-CTA job would set that time run instead in this
// cooperative launch, beside the batched one (another stream of the same
// graph): the k CTAs of an image each own a strip of every row, with S-cell
// halos whose exact values are handed over through L2 every S steps (the
// exchange words of the per-call tile plans, pass_body's MULTI form), and
// meet at a bounded per-image barrier between passes.  The cooperative
// launch keeps an image's CTAs co-resident, so every wait ends (and each is
// bounded: FG_ERR_TIMEOUT in the status word if one does not).  Results are
// bit-identical to the one-CTA job and to the per-call path: the same
// arithmetic per cell, in the same order.

#include <math.h>

#include <algorithm>

#include "fg_batch.cuh"
#include "fg_wait.cuh"

namespace fgi {
namespace {

constexpr int kMaxTiledImages = 32;
constexpr int kMaxTilesPerImage = 16;

struct TiledTable {
  int n;
  int start[kMaxTiledImages + 1];  // CTAs [start[i], start[i + 1]) run image i
};

// The b-th call of the k CTAs of one image returns once all k have made it.
__device__ __forceinline__ void group_sync(unsigned *bar, unsigned target, int *status) {
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    atomicAdd(bar, 1u);
    wait_count(bar, target, status, kSpinLimit);
  }
  __syncthreads();
}

// strip width of a row of N2 cells over k CTAs: a multiple of 4 (runs of 4
// cells never straddle strips), at least the halo S
__host__ __device__ inline int tiled_width(int N2, int k, int S) {
  const int T2 = ((N2 + k - 1) / k + 3) & ~3;
  return T2 < S ? S : T2;
}

template <int CT, int M>
__device__ __forceinline__ void tiled_pass(bool wt, const PassArgs &a, int tile, float *sm) {
  if (wt)
    pass_body<1, CT, M, MODE_GENERAL, true, false, true>(a, tile, sm);
  else
    pass_body<1, CT, M, MODE_GENERAL, false, false, true>(a, tile, sm);
}

template <int CT>
__global__ void __launch_bounds__(kThreads, 1)
    fg_batch2d_tiled_kernel(const fg_batch2d_item *items, TiledTable tab, int iterations, size_t smem, float r2,
                            unsigned *bars, unsigned long long *xch, long long xch_words, int *status) {
  extern __shared__ __align__(16) float sm[];
  __shared__ PassArgs s_args;
  int i = 0;
  while (i + 1 < tab.n && (int)blockIdx.x >= tab.start[i + 1]) i++;
  const int ti = (int)blockIdx.x - tab.start[i], k = tab.start[i + 1] - tab.start[i];
  const fg_batch2d_item &it = items[i];
  const int H = it.H, W = it.W;
  const long long P = (long long)H * W;
  if (P <= 0) return;  // every CTA of this image returns here
  if (it.C != CT) {      // a launch holds images of one channel count
    if (threadIdx.x == 0) atomicCAS(status, 0, FG_ERR_INVALID_ARGUMENT);
    return;
  }
  const int M = (it.flags & FG_BATCH_SIGNED) ? 2 : 1;
  unsigned *bar = bars + i;
  unsigned long long *xw = xch + (long long)i * xch_words;
  unsigned nsync = 0;
  // this CTA's share of the transpose, the initial distances and the
  // clearing of the image's exchange words
  batch_prologue(it, 0, M, true, sm, ti, k);
  for (long long q = threadIdx.x + (long long)ti * blockDim.x; q < xch_words; q += (long long)blockDim.x * k)
    xw[q] = 0ull;
  group_sync(bar, ++nsync * k, status);
  int pi = 0;
  for (int iter = 0; iter < iterations; iter++) {
    for (int kk = 0; kk < 4; kk++) {
      const int L = kk >= 2 ? W : H;
      const bool wt = kk & 1;
      if (L <= 1 && !wt) continue;
      const int N2 = kk >= 2 ? H : W;
      // hand-off period (= flush steps) and staging depth within the launch's
      // shared memory, fitted at this pass's region with the longest halo
      int S = 8, depth = 2;
      tiled_job_fit(it.C, M, tiled_width(N2, k, 32) + 64, smem, &S, &depth);
      const int T2 = tiled_width(N2, k, S), tiles = (N2 + T2 - 1) / T2;
      if (threadIdx.x == 0) {
        batch_pass_args(it, M, 0, kk, S, depth, r2, status, &s_args);
        const int K2 = tiles > 1 ? S : 0, R2 = T2 + 2 * K2;
        s_args.T2 = T2, s_args.K2 = K2, s_args.tiles2 = tiles;
        s_args.B2 = ((R2 + 3) & ~3) + 8;
        s_args.rowf = ring_pitch(s_args.B2);
        s_args.vec = s_args.vec && (K2 % 4 == 0);
        s_args.xch = xw;
        s_args.epoch_base = (unsigned)(pi + 1) << 12;  // chunks of this pass: base + 1 ... base + L / S
      }
      __syncthreads();
      if (ti < tiles) {
        if (M == 2)
          tiled_pass<CT, 2>(wt, s_args, ti, sm);
        else
          tiled_pass<CT, 1>(wt, s_args, ti, sm);
      }
      group_sync(bar, ++nsync * k, status);
      pi++;
    }
  }
  if (M == 2) {
    float *out = it.out;
    const float *d2 = it.d2;
    for (long long p = threadIdx.x + (long long)ti * blockDim.x; p < P; p += (long long)blockDim.x * k)
      out[p] = __fsub_rn(__ldcg(out + p), __ldcg(d2 + p));
  }
}

size_t tiled_bars_bytes(int n) { return ((size_t)n * 4 + 255) / 256 * 256; }
long long tiled_xch_words(int max_extent) { return 2LL * kMaxMaps * max_extent; }

}  // namespace
}  // namespace fgi

extern "C" FG_API size_t fg_batch2d_tiled_scratch_bytes(int n, int max_extent) {
  if (n < 0 || max_extent < 1) return 0;
  return fgi::tiled_bars_bytes(n) + (size_t)n * fgi::tiled_xch_words(max_extent) * 8;
}

extern "C" FG_API int fg_batch_geodesic2d_tiled(const fg_batch2d_item *items, const int *tiles, int n, int C,
                                                int max_extent, int iterations, void *scratch, size_t scratch_bytes,
                                                int *status, void *stream) {
  using namespace fgi;
  if (n < 0 || n > kMaxTiledImages)
    return set_error(FG_ERR_INVALID_ARGUMENT, "tiled batch: 0 to 32 images per launch");
  if (n == 0) return FG_OK;
  if (!items || !tiles || !scratch || !status)
    return set_error(FG_ERR_INVALID_ARGUMENT, "tiled batch: null descriptor, tile, scratch or status pointer");
  if (C < 1 || C > kMaxChannels) return set_error(FG_ERR_UNSUPPORTED, "tiled batch: images need 1 to 4 channels");
  if (max_extent < 1 || max_extent > 4 * kThreads)
    return set_error(FG_ERR_UNSUPPORTED, "tiled batch: image sides up to 2048 are supported");
  if (scratch_bytes < fg_batch2d_tiled_scratch_bytes(n, max_extent))
    return set_error(FG_ERR_WORKSPACE, "tiled batch: scratch smaller than fg_batch2d_tiled_scratch_bytes");
  TiledTable tab{};
  tab.n = n;
  int kmin = kMaxTilesPerImage;
  for (int i = 0; i < n; i++) {
    if (tiles[i] < 2 || tiles[i] > kMaxTilesPerImage)
      return set_error(FG_ERR_INVALID_ARGUMENT, "tiled batch: 2 to 16 CTAs per image");
    tab.start[i + 1] = tab.start[i] + tiles[i];
    kmin = std::min(kmin, tiles[i]);
  }
  const int grid = tab.start[n];
  // the widest region of any pass at the longest halo (32), for both map counts
  const int R2 = tiled_width(max_extent, kmin, 32) + 64;
  size_t smem = kBatchTransposeSmem;
  for (int M = 1; M <= 2; M++) {
    int S = 0, depth = 0;
    if (!tiled_job_fit(C, M, R2, kBatchSmemLimit, &S, &depth))
      return set_error(FG_ERR_UNSUPPORTED, "tiled batch: shared memory plan too large");
    smem = std::max(smem, batch_job_smem(C, M, R2, S, depth));
  }
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  unsigned *bars = static_cast<unsigned *>(scratch);
  unsigned long long *xch =
      reinterpret_cast<unsigned long long *>(static_cast<char *>(scratch) + tiled_bars_bytes(n));
  long long xw = tiled_xch_words(max_extent);
  cudaError_t e = cudaMemsetAsync(bars, 0, (size_t)n * 4, s);
  if (e != cudaSuccess) return set_error(FG_ERR_CUDA, cudaGetErrorString(e));
  int its = std::max(iterations, 0);
  const float r2 = (float)sqrt(2.0);  // fastgeodis_cpu.cpp:67
  auto launch = [&](auto fn) -> int {
    cudaError_t e2 = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e2 != cudaSuccess) return set_error(FG_ERR_CUDA, cudaGetErrorString(e2));
    int dev = 0, per_sm = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    e2 = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, kThreads, smem);
    if (e2 != cudaSuccess) return set_error(FG_ERR_CUDA, cudaGetErrorString(e2));
    if (grid > per_sm * sms) return set_error(FG_ERR_UNSUPPORTED, "tiled batch: more CTAs than the GPU holds at once");
    void *args[] = {const_cast<fg_batch2d_item **>(&items), &tab, &its, &smem, const_cast<float *>(&r2),
                    &bars, &xch, &xw, &status};
    e2 = cudaLaunchCooperativeKernel((const void *)fn, dim3(grid), dim3(kThreads), args, smem, s);
    return e2 == cudaSuccess ? FG_OK : set_error(FG_ERR_CUDA, cudaGetErrorString(e2));
  };
  switch (C) {
    case 1: return launch(fg_batch2d_tiled_kernel<1>);
    case 2: return launch(fg_batch2d_tiled_kernel<2>);
    case 3: return launch(fg_batch2d_tiled_kernel<3>);
    default: return launch(fg_batch2d_tiled_kernel<4>);
  }
}
