// Whole 2D transforms of small images (both sides up to FG_ONE_LAUNCH_SIDE)
// in one launch of one CTA, one thread per cell of a row.
//
// The pass body of the tile and batched kernels gives each thread a run of 4
// cells (float4 staging, 3D cross-sections up to 4096 cells per CTA); a
// 512-cell row then occupies 128 threads, and the row's step is one chain of
// 4 warps with every latency exposed.  Here each thread owns one cell: 16
// warps share a 512-cell step, each with a quarter of the instructions, and
// the previous row's neighbours are conflict-free scalar shared-memory reads.
// The arithmetic is the pass body's (candidates (D + le*ld) + lg*|dI| in the
// same order, fminf folds of a set whose minimum does not depend on the
// order): results are bit-identical to every other path.
//
// Per pass (fastgeodis_cpu.cpp:78-118 for the order of passes and the
// 3-neighbour stencil): step t reads the previous row's distances and image
// values from shared rings and its own old distance and image values from
// registers, loaded through L2 during step t-1, and keeps its new distance
// in a ring of S rows; every S steps the ring goes back to global memory, in
// place as whole rows or, for the passes that change the layout, transposed
// (S consecutive positions of a cell are contiguous there).  Measured on a
// 512x512 transform: a store per step and cp.async staging each cost about
// a tenth of a microsecond per step.

#include <math.h>

#include <algorithm>
#include <type_traits>

#include "fg_batch.cuh"

namespace fgi {
namespace {

// shared memory of the row body: S distance rows per map, 2 image rows per
// channel
__host__ __device__ inline size_t row_smem(int C, int M, int N, int S) {
  return ((size_t)S * M * N + (size_t)2 * C * N) * 4;
}

// One pass.  MODE as the pass kernels choose it (select_mode): EUCLID
// (lamb 0: D + le*ld, no image), GEO (lamb 1: D + sum |dI|) or GENERAL, each
// bit-identical to the general candidate for its lamb.
template <int C, int M, int MODE, bool WT>
__device__ __forceinline__ void row_pass(const PassArgs &ar, float *sm) {
  constexpr int CI = MODE == MODE_EUCLID ? 0 : C;  // image channels read
  const PassArgs a = ar;
  const int tid = threadIdx.x, NT = blockDim.x, lane = tid & 31, warp = tid >> 5, nwarps = NT >> 5;
  const int N = a.N2, L = a.L, S = a.S, lgS = __ffs(S) - 1;
  const bool on = tid < N, has_l = on && tid > 0, has_r = tid + 1 < N;
  float *drow = sm;                // [S][M][N] distance rows of the current chunk
  float *irow = drow + S * M * N;  // [2][CI][N] image rows of the last 2 steps
  // offsets fit 32 bits: the engine rejects images of 2^31 or more elements
  const int rstep = a.dir > 0 ? a.s_str : -a.s_str;
  int roff = (a.dir > 0 ? 0 : (L - 1) * a.s_str) + tid;  // read offset of the next step to load
  float e[M][3], lg[M];
#pragma unroll
  for (int m = 0; m < M; m++) {
    lg[m] = a.lg[m];
#pragma unroll
    for (int n = 0; n < 3; n++) e[m][n] = a.e[m][n];
  }
  // own old distances and image values of the next two steps, loaded
  // (through L2) while the current steps compute: two register sets, the
  // loop unrolled by two so each set stays in registers
  float nd[2][M], ni[2][CI > 0 ? CI : 1];
  auto load = [&](int set) {
#pragma unroll
    for (int m = 0; m < M; m++) nd[set][m] = __ldcg(a.dsrc[m] + roff);
#pragma unroll
    for (int c = 0; c < CI; c++) ni[set][c] = __ldcg(a.img + c * a.img_cs + roff);
    roff += rstep;
  };
  if (on) load(0);
  if (on && L > 1) load(1);
  auto step = [&](int t, int set) {
    float best[M], ic[CI > 0 ? CI : 1];
#pragma unroll
    for (int m = 0; m < M; m++) best[m] = nd[set][m];
#pragma unroll
    for (int c = 0; c < CI; c++) ic[c] = ni[set][c];
    if (on && t + 2 < L) load(set);
    if (on) {
      if (t > 0) {
        const float *dp = drow + ((t - 1) & (S - 1)) * (M * N) + tid;
        const float *ip = irow + ((t - 1) & 1) * (CI * N) + tid;
        // neighbour o (-1, 0, +1) of the previous row
        auto cand = [&](int o) {
          float l1 = 0.0f, d = 0.0f;
          if (MODE != MODE_EUCLID) {
            if (C == 1) {
              d = __fsub_rn(ic[0], ip[o]);
              l1 = fabsf(d);
            } else {
#pragma unroll
              for (int c = 0; c < CI; c++) l1 = __fadd_rn(l1, fabsf(__fsub_rn(ic[c], ip[c * N + o])));
            }
          }
#pragma unroll
          for (int m = 0; m < M; m++) {
            const float dq = dp[m * N + o];
            float v;
            if (MODE == MODE_EUCLID)
              v = __fadd_rn(dq, e[m][o + 1]);
            else if (MODE == MODE_GEO)
              v = __fadd_rn(dq, l1);
            else if (C == 1)  // the reference's l_grad * |d| equals |l_grad * d| bit for bit
              v = __fadd_rn(__fadd_rn(dq, e[m][o + 1]), fabsf(__fmul_rn(lg[m], d)));
            else
              v = __fadd_rn(__fadd_rn(dq, e[m][o + 1]), __fmul_rn(lg[m], l1));
            best[m] = fminf(best[m], v);
          }
        };
        cand(0);
        if (has_l) cand(-1);
        if (has_r) cand(1);
      }
      float *dc = drow + (t & (S - 1)) * (M * N) + tid;
#pragma unroll
      for (int m = 0; m < M; m++) dc[m * N] = best[m];
      float *icw = irow + (t & 1) * (CI * N) + tid;
#pragma unroll
      for (int c = 0; c < CI; c++) icw[c * N] = ic[c];
    }
    __syncthreads();
    if (((t + 1) & (S - 1)) == 0 || t == L - 1) {
      // the chunk's rows t0 .. t back to global memory
      const int t0 = t & ~(S - 1), Sn = t - t0 + 1;
      if (WT) {
        // transposed: cell x of step s at s + x * wst2; lanes take S
        // consecutive steps of 32 / S cells
        const int cpw = 32 / S, j = lane & (S - 1);
        if (j < Sn) {
          const int so = a.dir > 0 ? t0 + j : L - 1 - t0 - j;
          const float *src = drow + j * M * N;
          for (int x = warp * cpw + (lane >> lgS); x < N; x += nwarps * cpw) {
#pragma unroll
            for (int m = 0; m < M; m++) a.ddst[m][so + x * a.wst2] = src[m * N + x];
          }
        }
      } else if (on) {
        // in place, whole rows
        for (int j = 0; j < Sn; j++) {
          const int ro = (a.dir > 0 ? t0 + j : L - 1 - t0 - j) * a.s_str + tid;
#pragma unroll
          for (int m = 0; m < M; m++) a.ddst[m][ro] = drow[j * M * N + m * N + tid];
        }
      }
      __syncthreads();
    }
  };
  for (int t = 0; t < L; t += 2) {
    step(t, 0);
    if (t + 1 < L) step(t + 1, 1);
  }
}

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
