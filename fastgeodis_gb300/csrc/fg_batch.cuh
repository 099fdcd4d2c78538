// One 2D image's transform run by one CTA: the pieces shared by the batched
// kernel, the one-launch single-image kernel (fg_batch.cu) and the
// differentiable forward (fg_grad2d.cu).
//
// An image's distance maps live in the descriptor's buffers: map 0 in `out`
// (read layout [H][W]) and `t1` (transposed [W][H]); map 1, the signed form's
// D(1 - mask), in `d2` and `t2`.  A job computes one map (`first` = 0 or 1)
// or both (M = 2); passes along W read the transposed image `image_t`.
#pragma once

#include <math.h>

#include "fg_pass.cuh"

namespace fgi {

constexpr size_t kBatchSmemLimit = 227 * 1024;

// channel template of an image with C channels: the pass body compiled for
// exactly that count (the general body, with the count a run-time value,
// takes more registers and spills beside the others in one kernel)
__host__ __device__ constexpr int batch_ct(int C) { return C; }

// prefetch depth of a job variant when its shared memory allows it
__host__ __device__ constexpr int batch_natural_depth(int C, int M) {
  return pass_depth(pass_nch(batch_ct(C), MODE_GENERAL), M);
}

// shared memory of one image pass body: rows of an image side `ext`, S
// distance rows per map for the transposed flush, 2 image rows per channel,
// `depth` steps of own inputs in flight, the own-cell table
__host__ __device__ inline size_t batch_job_smem(int C, int M, int ext, int S, int depth) {
  const int rowf = ring_pitch(((ext + 3) & ~3) + 8);  // one row: 4-cell apron, runs of 4, apron
  return (size_t)(S * M + 2 * C) * rowf * 4 + (size_t)depth * (M + C) * kThreads * 16 + (size_t)ext * 8 + 64;
}

// the image transpose of the prologue: one 32x33 tile per warp
constexpr size_t kBatchTransposeSmem = (size_t)(kThreads / 32) * 32 * 33 * 4;

// Flush steps S and prefetch depth of a job within `smem` bytes, in order of
// preference: S = 8 at the natural depth, 4 at the natural depth, 4 at depth
// 2, 2 at depth 2.  False if none fits.
__host__ __device__ inline bool batch_job_fit(int C, int M, int ext, size_t smem, int *S, int *depth) {
  const int nat = batch_natural_depth(C, M);
  const int Ss[4] = {8, 4, 4, 2}, Ds[4] = {nat, nat, 2, 2};
  for (int i = 0; i < 4; i++) {
    if (batch_job_smem(C, M, ext, Ss[i], Ds[i]) <= smem) {
      *S = Ss[i];
      *depth = Ds[i];
      return true;
    }
  }
  return false;
}

// The same for a strip of a tiled image, whose S is also its hand-off period
// (halos of S cells): the longest period first, S = 32 down to 8 at the
// natural depth, then as batch_job_fit.  A row's halo is only its two ends, so
// a longer period costs little redundant work and saves hand-offs.
__host__ __device__ inline bool tiled_job_fit(int C, int M, int ext, size_t smem, int *S, int *depth) {
  const int nat = batch_natural_depth(C, M);
  const int Ss[3] = {32, 16, 8};
  for (int i = 0; i < 3; i++) {
    if (batch_job_smem(C, M, ext, Ss[i], nat) <= smem) {
      *S = Ss[i];
      *depth = nat;
      return true;
    }
  }
  return batch_job_fit(C, M, ext, smem, S, depth);
}

// Transposed image copy (unless `transpose` is false) and the initial
// distances of the job's maps: v*M for map 0, v*(1-M) for map 1.  A CTA that
// is part `part` of `parts` CTAs sharing one image does that share.
__device__ inline void batch_prologue(const fg_batch2d_item &it, int first, int M, bool transpose, float *sm,
                                      int part = 0, int parts = 1) {
  const int tid = threadIdx.x, NT = blockDim.x, lane = tid & 31, warp = tid >> 5, nwarps = NT >> 5;
  // the descriptor's fields in registers: the stores below could alias a
  // descriptor in global memory and would make every iteration reload them
  const int C = it.C, H = it.H, W = it.W;
  const float v = it.v;
  const float *image = it.image, *mask = it.mask;
  float *image_t = it.image_t, *out = it.out, *d2 = it.d2;
  const long long P = (long long)H * W;
  if (transpose) {
    // image [C][H][W] -> [C][W][H], 32x32 tiles through shared memory, one per warp
    float *tb = sm + warp * 32 * 33;
    const int th = (H + 31) / 32, tw = (W + 31) / 32;
    for (int job = warp + part * nwarps; job < C * th * tw; job += nwarps * parts) {
      const int c = job / (th * tw), r = job - c * th * tw, h0 = (r / tw) * 32, w0 = (r % tw) * 32;
      const float *src = image + c * P;
      float *dst = image_t + c * P;
      for (int y = 0; y < 32; y++) {
        int h = h0 + y, w = w0 + lane;
        if (h < H && w < W) tb[y * 33 + lane] = src[(long long)h * W + w];
      }
      __syncwarp();
      for (int y = 0; y < 32; y++) {
        int w = w0 + y, h = h0 + lane;
        if (h < H && w < W) dst[(long long)w * H + h] = tb[lane * 33 + y];
      }
      __syncwarp();
    }
  }
  const bool m0 = first == 0, m1 = first == 1 || M == 2;
  for (long long i = tid + (long long)part * NT; i < P; i += (long long)NT * parts) {
    const float m = mask[i];
    if (m0) out[i] = __fmul_rn(v, m);
    if (m1) d2[i] = __fmul_rn(v, __fsub_rn(1.0f, m));
  }
}

// arguments of pass `k` (0: along H forward, 1: along H backward writing
// [W][H], 2: along W forward, 3: along W backward writing [H][W]) over the
// job's M maps starting at map `first`
__device__ inline void batch_pass_args(const fg_batch2d_item &it, int M, int first, int k, int S, int depth,
                                       float r2, int *status, PassArgs *pa) {
  PassArgs a;
  const int H = it.H, W = it.W;
  const bool alongW = k >= 2, back = (k & 1) != 0;
  const long long P = (long long)H * W;
  a.img = alongW ? it.image_t : it.image;
  a.img_cs = P;
  a.C = it.C;
  float *r[2] = {it.out, it.d2}, *t[2] = {it.t1, it.t2};
  const float ld[3] = {r2, 1.0f, r2};
  bool vec = (H % 4 == 0) && (W % 4 == 0) && ((reinterpret_cast<uintptr_t>(a.img) & 15) == 0);
  for (int m = 0; m < kMaxMaps; m++) {
    const int mm = (m < M ? m : 0) + first;
    a.dsrc[m] = alongW ? t[mm] : r[mm];
    a.ddst[m] = (k == 1) ? t[mm] : ((k == 3) ? r[mm] : const_cast<float *>(a.dsrc[m]));
    a.lg[m] = it.l_grad;
    for (int n = 0; n < 9; n++) a.e[m][n] = n < 3 ? __fmul_rn(it.l_eucl, ld[n]) : 0.0f;
    vec = vec && ((reinterpret_cast<uintptr_t>(r[mm]) & 15) == 0) &&
          ((reinterpret_cast<uintptr_t>(t[mm]) & 15) == 0);
  }
  a.L = alongW ? W : H;
  a.dir = back ? -1 : 1;
  a.s_str = alongW ? H : W;
  a.st1 = 0;
  const int N2 = alongW ? H : W;
  if (k == 1) {
    a.ws_str = 1, a.wst1 = 0, a.wst2 = H;
  } else if (k == 3) {
    a.ws_str = 1, a.wst1 = 0, a.wst2 = W;
  } else {
    a.ws_str = a.s_str, a.wst1 = 0, a.wst2 = 1;
  }
  a.N1 = 1;
  a.N2 = N2;
  a.T1 = 1, a.T2 = N2, a.K1 = 0, a.K2 = 0, a.tiles1 = 1, a.tiles2 = 1;
  a.S = S;
  a.B2 = ((N2 + 3) & ~3) + 8;
  a.rowf = ring_pitch(a.B2);
  a.vec = vec ? 1 : 0;
  a.xch = nullptr;  // one tile per image: no halo exchange
  a.epoch_base = 0;
  a.status = status;
  a.tape = nullptr;
  a.P = depth;
  a.t_begin = 0, a.t_end = 0;
  *pa = a;
}

}  // namespace fgi
