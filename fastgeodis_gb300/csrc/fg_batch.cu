// Batched 2D transforms: many images of uneven size, channel count and form
// (plain or signed) in one persistent launch.
//
// Each CTA repeatedly claims the next job from a work queue (an atomic
// counter; the caller orders the jobs largest first) and runs it by itself
// (pass_body, one tile covering the whole cross-section, no halo exchange).
// A job is one descriptor: a plain image (initial distances, image transpose,
// `iterations` x 4 passes), a signed image with both distance maps in one
// CTA (they share the image reads), or one half of a signed image split over
// two consecutive descriptors (half the latency).  The first half transposes
// the image and computes D(mask); the second computes D(1 - mask) and reads
// the transposed image after the first half has published it (a bounded wait
// on a per-pair word: the first half was claimed earlier by a running CTA and
// waits for nothing); whichever half finishes second writes the difference.
// No other CTA waits for another, so any number of jobs and any grid size is
// safe, and the launch can be captured in a CUDA graph (memset of the
// counters + one kernel).
//
// Every job runs the pass body compiled for its image's channel count (1 to
// 4), so a mixed batch costs what its images cost alone; with the count a
// run-time value the general body spilled registers beside the others in
// this kernel.  Each image's arithmetic is exactly that of the per-call path:
// results are bit-identical, alone, in a batch, split or not.

#include <math.h>

#include <algorithm>

#include "fg_batch.cuh"
#include "fg_wait.cuh"

namespace fgi {
namespace {

// One job: the passes of M maps from map `first` of one image.  `pair` is the
// split pair's word (ready +1 by the first half, +2 by each half when done).
template <int CT, int M>
__device__ __forceinline__ void batch_item(const fg_batch2d_item &it, int first, bool split, unsigned *pair,
                                           int iterations, size_t smem, float r2, int *status, float *sm,
                                           PassArgs &s_args, int &s_flag) {
  const int H = it.H, W = it.W;
  const long long P = (long long)H * W;
  if (P <= 0) return;
  int S = 4, depth = 2;  // the launch sized `smem` for every job variant
  batch_job_fit(it.C, M, max(H, W), smem, &S, &depth);
  batch_prologue(it, first, M, first == 0, sm);
  __threadfence();
  __syncthreads();
  if (split && first == 0 && threadIdx.x == 0) {
    __threadfence();
    atomicAdd(pair, 1u);  // the transposed image is published
  }
  bool need_t = split && first == 1;
  for (int iter = 0; iter < iterations; iter++) {
    for (int k = 0; k < 4; k++) {
      const int L = k >= 2 ? W : H;
      const bool wt = k & 1;
      if (L <= 1 && !wt) continue;
      if (need_t && k >= 2) {
        if (threadIdx.x == 0) wait_count(pair, 1u, status, kSpinLimit);
        __syncthreads();
        need_t = false;
      }
      if (threadIdx.x == 0) batch_pass_args(it, M, first, k, S, depth, r2, status, &s_args);
      __syncthreads();
      if (wt)
        pass_body<1, CT, M, MODE_GENERAL, true, false, false>(s_args, 0, sm);
      else
        pass_body<1, CT, M, MODE_GENERAL, false, false, false>(s_args, 0, sm);
      __threadfence();
      __syncthreads();
    }
  }
  float *out = it.out;  // in registers: the stores below could alias the descriptor
  const float *d2 = it.d2;
  if (M == 2) {
    for (long long p = threadIdx.x; p < P; p += blockDim.x) out[p] = __fsub_rn(out[p], d2[p]);
  }
  if (split) {
    // the second half to finish subtracts (the other's stores were fenced
    // before its count; read them from L2)
    if (threadIdx.x == 0) {
      __threadfence();
      s_flag = atomicAdd(pair, 2u) == 3u;
      __threadfence();
    }
    __syncthreads();
    if (s_flag) {
      for (long long p = threadIdx.x; p < P; p += blockDim.x) out[p] = __fsub_rn(__ldcg(out + p), __ldcg(d2 + p));
    }
  }
}

// the job's channel variant
template <int M>
__device__ __forceinline__ void batch_item_ct(const fg_batch2d_item &it, int first, bool split, unsigned *pair,
                                              int iterations, size_t smem, float r2, int *status, float *sm,
                                              PassArgs &s_args, int &s_flag) {
  switch (batch_ct(it.C)) {
    case 1: batch_item<1, M>(it, first, split, pair, iterations, smem, r2, status, sm, s_args, s_flag); break;
    case 2: batch_item<2, M>(it, first, split, pair, iterations, smem, r2, status, sm, s_args, s_flag); break;
    case 3: batch_item<3, M>(it, first, split, pair, iterations, smem, r2, status, sm, s_args, s_flag); break;
    default: batch_item<4, M>(it, first, split, pair, iterations, smem, r2, status, sm, s_args, s_flag); break;
  }
}

__device__ __forceinline__ bool same_image(const fg_batch2d_item &a, const fg_batch2d_item &b) {
  return a.image == b.image && a.mask == b.mask && a.out == b.out && a.image_t == b.image_t && a.d2 == b.d2 &&
         a.t1 == b.t1 && a.t2 == b.t2 && a.C == b.C && a.H == b.H && a.W == b.W && a.v == b.v &&
         a.l_grad == b.l_grad && a.l_eucl == b.l_eucl;
}

// Job j of the queue.  A split half whose partner descriptor is missing or
// differs records FG_ERR_INVALID_ARGUMENT and runs nothing.
__device__ void batch_job(const fg_batch2d_item *items, int n, int j, int all_signed, int iterations, size_t smem,
                          float r2, unsigned *pairs, int *status, float *sm, PassArgs &s_args, int &s_flag) {
  const fg_batch2d_item &it = items[j];  // read where used: a copy would stay live across the passes
  const int sgn = all_signed ? FG_BATCH_SIGNED : 0;
  const int f = it.flags | sgn;
  const bool is_signed = (f & FG_BATCH_SIGNED) != 0;
  const bool split = is_signed && (f & FG_BATCH_SPLIT) != 0;
  const int first = split && (f & FG_BATCH_SECOND) ? 1 : 0;
  if (split) {
    const int jo = first ? j - 1 : j + 1;
    bool ok = jo >= 0 && jo < n;
    if (ok) {
      const fg_batch2d_item &o = items[jo];
      const int fo = o.flags | sgn;
      ok = same_image(it, o) && (fo & FG_BATCH_SIGNED) && (fo & FG_BATCH_SPLIT) &&
           ((fo & FG_BATCH_SECOND) != 0) == (first == 0);
    }
    if (!ok) {
      if (threadIdx.x == 0) atomicCAS(status, 0, FG_ERR_INVALID_ARGUMENT);
      return;
    }
  }
  if (is_signed && !split)
    batch_item_ct<2>(it, 0, false, nullptr, iterations, smem, r2, status, sm, s_args, s_flag);
  else
    batch_item_ct<1>(it, first, split, pairs + (j - first), iterations, smem, r2, status, sm, s_args, s_flag);
}

__global__ void __launch_bounds__(kThreads, 1)
    fg_batch2d_kernel(const fg_batch2d_item *items, int n, int all_signed, int iterations, size_t smem, float r2,
                      int *counter, int *status) {
  extern __shared__ __align__(16) float sm[];
  __shared__ int s_job, s_flag;
  __shared__ PassArgs s_args;
  unsigned *pairs = reinterpret_cast<unsigned *>(counter + 1);
  for (;;) {
    if (threadIdx.x == 0) s_job = atomicAdd(counter, 1);
    __syncthreads();
    const int j = s_job;
    if (j >= n) break;
    batch_job(items, n, j, all_signed, iterations, smem, r2, pairs, status, sm, s_args, s_flag);
    __syncthreads();
  }
}

// Dynamic shared memory of a launch whose jobs have up to max_C channels,
// sides up to max_extent and 1 to `maps` distance maps: the most any job
// variant takes at the first (S, depth) of batch_job_fit that fits the
// limit.  0 if some variant fits none.
size_t batch_plan(int max_C, int max_extent, int maps) {
  size_t need = kBatchTransposeSmem;
  for (int C = 1; C <= max_C; C++) {
    for (int M = 1; M <= maps; M++) {
      int S = 0, depth = 0;
      if (!batch_job_fit(C, M, max_extent, kBatchSmemLimit, &S, &depth)) return 0;
      need = std::max(need, batch_job_smem(C, M, max_extent, S, depth));
    }
  }
  return need;
}

}  // namespace
}  // namespace fgi

extern "C" FG_API size_t fg_batch2d_smem_bytes(int max_C, int max_extent, int is_signed) {
  if (max_C < 1 || max_C > fgi::kMaxChannels || max_extent < 1) return 0;
  (void)is_signed;  // a launch sizes for plain, split and two-map signed jobs alike
  return fgi::batch_plan(max_C, max_extent, 2);
}

extern "C" FG_API int fg_batch_geodesic2d(const fg_batch2d_item *items, int n, int max_C, int max_extent,
                                          int is_signed, int iterations, int *counter, int *status, int max_ctas,
                                          void *stream) {
  using namespace fgi;
  if (n < 0 || (n > 0 && (!items || !counter || !status)))
    return set_error(FG_ERR_INVALID_ARGUMENT, "batch: null descriptor, counter or status pointer");
  if (max_C < 1 || max_C > kMaxChannels)
    return set_error(FG_ERR_UNSUPPORTED, "batch: images need 1 to 4 channels");
  if (max_extent > 4 * kThreads)
    return set_error(FG_ERR_UNSUPPORTED, "batch: image sides up to 2048 are supported (one CTA sweeps a whole row)");
  if (n == 0) return FG_OK;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  cudaError_t e = cudaMemsetAsync(counter, 0, sizeof(int) * (1 + (size_t)n), s);  // queue and pair words
  if (e != cudaSuccess) return set_error(FG_ERR_CUDA, cudaGetErrorString(e));
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const size_t smem = batch_plan(max_C, std::max(max_extent, 1), 2);
  if (smem == 0)
    return set_error(FG_ERR_UNSUPPORTED, "batch: shared memory plan too large");
  const int grid = std::max(1, std::min(n, max_ctas > 0 ? std::min(max_ctas, sms) : sms));
  const float r2 = (float)sqrt(2.0);  // fastgeodis_cpu.cpp:67
  auto fn = fg_batch2d_kernel;
  e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return set_error(FG_ERR_CUDA, cudaGetErrorString(e));
  fn<<<grid, kThreads, smem, s>>>(items, n, is_signed ? 1 : 0, std::max(iterations, 0), smem, r2, counter, status);
  e = cudaGetLastError();
  if (e != cudaSuccess) return set_error(FG_ERR_CUDA, cudaGetErrorString(e));
  return FG_OK;
}
