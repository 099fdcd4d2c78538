// A batch of volume transforms in one persistent launch (fg_batch3d.cuh).
//
// The launch holds as many thread-block clusters as the device co-schedules;
// each cluster loops: its first CTA claims the next job of the queue (one
// atomic add), waits (bounded) until the job's predecessor in its volume's
// chain has finished, and hands the job to the cluster's CTAs through its
// shared memory (read by the others over distributed shared memory between
// two cluster barriers).  The CTAs run the job -- a pass on the cluster sweep
// body (fg_cluster.cuh, 2 runs of 4 cells per thread), or a prologue /
// epilogue shared out over the cluster -- then make their global writes
// visible (fence, cluster barrier) and the first CTA advances the volume's
// progress counter (release).
//
// The queue is ordered by position in the chains (every volume's prologue,
// then every volume's first pass, ...), so a claimed job's predecessor was
// claimed earlier by a running cluster; every wait ends.  A wait that runs
// out records FG_ERR_TIMEOUT and the volume's chain continues (its results are
// void), so one lost job cannot stall the rest for long.
#include <algorithm>

#include "fg_batch3d.cuh"
#include "fg_cluster.cuh"

namespace fgi {
namespace {

__device__ __forceinline__ unsigned cl_nranks() {
  unsigned r;
  asm volatile("mov.u32 %0, %%cluster_nctarank;\n" : "=r"(r));
  return r;
}
__device__ __forceinline__ int ld_cluster_s32(unsigned a) {
  int v;
  asm volatile("ld.shared::cluster.s32 %0, [%1];\n" : "=r"(v) : "r"(a) : "memory");
  return v;
}
__device__ __forceinline__ void red_release_add(unsigned *p, unsigned v) {
  asm volatile("red.release.gpu.global.add.u32 [%0], %1;\n" ::"l"(p), "r"(v) : "memory");
}

// dst[c][r] = src[r][c] for a rows x cols matrix, shared out over the
// cluster's CTAs: each warp moves one 32 x 32 tile at a time through its own
// padded shared tile (32 independent row loads in flight per lane, full
// 128-byte lines read and written, no block barrier).
__device__ void transpose_tiles(const float *src, float *dst, long long rows, int cols, float *sm, unsigned rank,
                                unsigned G) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  float(*tile)[33] = reinterpret_cast<float(*)[33]>(sm + warp * 32 * 33);
  const long long tc = (cols + 31) / 32, ntiles = ((rows + 31) / 32) * tc;
  for (long long k = (long long)rank * nwarps + warp; k < ntiles; k += (long long)G * nwarps) {
    const long long r0 = (k / tc) * 32;
    const int c0 = (int)(k % tc) * 32;
    const int c = c0 + lane;
    // all 32 row loads of the lane in flight before the first store
    float v[32];
#pragma unroll
    for (int y = 0; y < 32; y++) {
      const long long r = r0 + y;
      v[y] = (r < rows && c < cols) ? __ldg(src + r * cols + c) : 0.0f;
    }
#pragma unroll
    for (int y = 0; y < 32; y++) tile[y][lane] = v[y];
    __syncwarp();
    const long long r = r0 + lane;
#pragma unroll
    for (int y = 0; y < 32; y++) {
      const int cc = c0 + y;
      if (r < rows && cc < cols) dst[(long long)cc * rows + r] = tile[lane][y];
    }
    __syncwarp();
  }
}

// Initial distances (v*M, and v*(1-M) for the signed form's second map) and
// the transposed image copy [C][W][D][H], shared out over the cluster's CTAs.
__device__ void run_prologue(const Batch3dJob &jb, float *sm, unsigned rank, unsigned G) {
  const int tid = threadIdx.x, NT = blockDim.x;
  const long long P = (long long)jb.D * jb.H * jb.W;
  const float v = jb.v;
  for (long long i = (long long)rank * NT + tid; i < P; i += (long long)G * NT) {
    const float m = jb.mask[i];
    jb.out[i] = __fmul_rn(v, m);
    if (jb.is_signed) jb.d2[i] = __fmul_rn(v, __fsub_rn(1.0f, m));
  }
  if (!jb.image_t) return;
  // each channel [(D H)][W] -> [W][(D H)]
  for (int c = 0; c < jb.C; c++)
    transpose_tiles(jb.image + c * P, jb.image_t + c * P, (long long)jb.D * jb.H, jb.W, sm, rank, G);
}

// D(M) - D(1 - M) of the signed form.
__device__ void run_epilogue(const Batch3dJob &jb, unsigned rank, unsigned G) {
  const int tid = threadIdx.x, NT = blockDim.x;
  const long long P = (long long)jb.D * jb.H * jb.W;
  for (long long i = (long long)rank * NT + tid; i < P; i += (long long)G * NT)
    jb.out[i] = __fsub_rn(jb.out[i], jb.d2[i]);
}

// MODE: the batch's arithmetic mode when every pass shares it, else
// MODE_GENERAL, whose candidate expression gives the other modes' bits too
// (l_grad = 0 adds +0, l_eucl = 0 adds +0 and l_grad = 1 multiplies by 1).
// No pass writes transposed (layout changes are transpose jobs).
template <int M, int MODE>
__device__ void run_pass(const Batch3dJob &jb, float *sm, unsigned rank) {
  // the pass's arguments in shared memory: the step loop reads them there
  // (a kernel parameter would sit in the constant bank; a job's do not)
  __shared__ PassArgs s_args;
  {
    const int *src = reinterpret_cast<const int *>(&jb.a);
    int *dst = reinterpret_cast<int *>(&s_args);
    for (int i = threadIdx.x; i < (int)(sizeof(PassArgs) / 4); i += blockDim.x) dst[i] = src[i];
    __syncthreads();
  }
  const PassArgs &a = s_args;
  if ((int)rank >= a.tiles1) {
    // no strip of this cross-section: take part in the body's two cluster barriers only
    cl_sync();
    cl_sync();
    return;
  }
  cluster_body<1, M, MODE, 2>(a, sm);
}

template <int M, int MODE>
__global__ void __maxnreg__(128) fg_batch3d_kernel(const Batch3dJob *jobs, int njobs, unsigned *counters,
                                                        int *status) {
  extern __shared__ __align__(16) float sm[];
  __shared__ int s_claim[2];  // job index and whether its predecessor finished in time
  const unsigned rank = cl_rank(), G = cl_nranks();
  const int tid = threadIdx.x;
  for (;;) {
    if (rank == 0 && tid == 0) {
      const int j = (int)atomicAdd(&counters[0], 1u);
      int ok = 1;
      if (j < njobs) {
        const Batch3dJob &jb = jobs[j];
        if (jb.seq > 0 && !wait_count(&counters[1 + jb.vol], (unsigned)jb.seq, status, kSpinLimit)) ok = 0;
      }
      s_claim[0] = j;
      s_claim[1] = ok;
    }
    __syncwarp();  // the cluster barrier is .aligned: warp 0 converges after its first thread's wait
    cl_sync();
    const unsigned a0 = cl_map(smem_u32(s_claim), 0);
    const int j = ld_cluster_s32(a0);
    const int ok = ld_cluster_s32(a0 + 4);
    cl_sync();  // every CTA has its copy before the first CTA claims again
    if (j >= njobs) break;
    const Batch3dJob &jb = jobs[j];
    if (ok) {
      // the predecessor's writes (other clusters) are visible to every thread
      // of this CTA: each acquires the counter the first CTA saw advance
      if (jb.seq > 0) (void)ld_acquire_u32(&counters[1 + jb.vol]);
      __syncthreads();
      if (jb.kind == JOB3_PASS) run_pass<M, MODE>(jb, sm, rank);
      else if (jb.kind == JOB3_PROLOGUE) run_prologue(jb, sm, rank, G);
      else if (jb.kind == JOB3_TRANSPOSE) transpose_tiles(jb.tsrc, jb.tdst, jb.trows, jb.tcols, sm, rank, G);
      else run_epilogue(jb, rank, G);
    }
    __threadfence();
    cl_sync();
    if (rank == 0 && tid == 0) red_release_add(&counters[1 + jb.vol], 1u);
  }
}

const void *kernel_of(int M, int mode) {
  if (M == 1)
    return mode == MODE_EUCLID ? (const void *)fg_batch3d_kernel<1, MODE_EUCLID>
           : mode == MODE_GEO  ? (const void *)fg_batch3d_kernel<1, MODE_GEO>
                               : (const void *)fg_batch3d_kernel<1, MODE_GENERAL>;
  return mode == MODE_EUCLID ? (const void *)fg_batch3d_kernel<2, MODE_EUCLID>
         : mode == MODE_GEO  ? (const void *)fg_batch3d_kernel<2, MODE_GEO>
                             : (const void *)fg_batch3d_kernel<2, MODE_GENERAL>;
}

cudaLaunchConfig_t config(int G, int threads, size_t smem, cudaStream_t s, cudaLaunchAttribute *at) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(G);
  cfg.blockDim = dim3(threads);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = G;
  at[0].val.clusterDim.y = 1;
  at[0].val.clusterDim.z = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  return cfg;
}

int set_attributes(const void *fn) {
  // dynamic shared memory up to the planner's budget (227 KB less 1 KB: the
  // kernel's static shared memory, the claim and the pass arguments, fits)
  cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024 - 1024);
  if (e == cudaSuccess) e = cudaFuncSetAttribute(fn, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
  if (e != cudaSuccess) return set_error(FG_ERR_CUDA, cudaGetErrorString(e));
  return FG_OK;
}

}  // namespace

int batch3d_capacity(int M, int mode, int G, int threads, size_t smem, int *clusters) {
  if (M < 1 || M > 2 || mode < 0 || mode > 2 || G < 1 || G > kMaxCluster || threads < 32 || threads > kThreads)
    return set_error(FG_ERR_INVALID_ARGUMENT, "batch3d: bad launch shape");
  const void *fn = kernel_of(M, mode);
  int rc = set_attributes(fn);
  if (rc != FG_OK) return rc;
  cudaLaunchAttribute at[1];
  cudaLaunchConfig_t cfg = config(G, threads, smem, nullptr, at);
  int n = 0;
  const cudaError_t e = cudaOccupancyMaxActiveClusters(&n, fn, &cfg);
  if (e != cudaSuccess) {
    (void)cudaGetLastError();
    return set_error(FG_ERR_CUDA, cudaGetErrorString(e));
  }
  *clusters = n;
  return FG_OK;
}

int launch_batch3d(const Batch3dJob *jobs, int njobs, int nvol, int M, int mode, int G, int threads, size_t smem,
                   unsigned *counters, int *status, cudaStream_t s) {
  int clusters = 0;
  int rc = batch3d_capacity(M, mode, G, threads, smem, &clusters);
  if (rc != FG_OK) return rc;
  if (clusters < 1) return set_error(FG_ERR_UNSUPPORTED, "batch3d: the device cannot co-schedule this cluster shape");
  cudaError_t e = cudaMemsetAsync(counters, 0, sizeof(unsigned) * (size_t)(nvol + 1), s);
  if (e != cudaSuccess) return set_error(FG_ERR_CUDA, cudaGetErrorString(e));
  if (njobs == 0) return FG_OK;
  cudaLaunchAttribute at[1];
  cudaLaunchConfig_t cfg = config(G, threads, smem, s, at);
  cfg.gridDim = dim3((unsigned)(G * std::min(clusters, std::max(1, njobs))));
  void *args[] = {const_cast<Batch3dJob **>(&jobs), &njobs, &counters, &status};
  e = cudaLaunchKernelExC(&cfg, kernel_of(M, mode), args);
  if (e != cudaSuccess) return set_error(FG_ERR_CUDA, cudaGetErrorString(e));
  return FG_OK;
}

}  // namespace fgi
