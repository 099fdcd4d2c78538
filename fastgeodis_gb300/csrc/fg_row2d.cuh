// The row body: one pass of a 2D transform by one CTA with one thread per
// cell of a row (rows up to the CTA's size, 512 cells), shared by the
// one-launch small-image kernel (fg_row2d.cu) and the differentiable forward
// (fg_grad2d.cu).
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
// registers, loaded through L2 two steps ahead, and keeps its new distance
// in a ring of S rows; every S steps the ring goes back to global memory, in
// place as whole rows or, for the passes that change the layout, transposed
// (S consecutive positions of a cell are contiguous there).  Measured on a
// 512x512 transform: a store per step and cp.async staging each cost about
// a tenth of a microsecond per step.
#pragma once

#include "fg_batch.cuh"

namespace fgi {

// shared memory of the row body: S distance rows per map, 2 image rows per
// channel, with a tape S rows of one byte per cell
__host__ __device__ inline size_t row_smem(int C, int M, int N, int S, bool tape = false) {
  return ((size_t)S * M * N + (size_t)2 * C * N) * 4 + (tape ? ((size_t)S * N + 3) / 4 * 4 : 0);
}

// One pass.  MODE as the pass kernels choose it (select_mode): EUCLID
// (lamb 0: D + le*ld, no image), GEO (lamb 1: D + sum |dI|) or GENERAL, each
// bit-identical to the general candidate for its lamb.  TAPE (one map):
// also record which candidate won, as the tile body does -- candidates in
// the order of the reference's stencil, a later one only when strictly
// smaller, 1 + its index (0: the cell's own value) -- one byte per cell in
// the read layout at a.tape.
template <int C, int M, int MODE, bool WT, bool TAPE = false>
__device__ __forceinline__ void row_pass(const PassArgs &ar, float *sm) {
  constexpr int CI = MODE == MODE_EUCLID ? 0 : C;  // image channels read
  const PassArgs a = ar;
  const int tid = threadIdx.x, NT = blockDim.x, lane = tid & 31, warp = tid >> 5, nwarps = NT >> 5;
  const int N = a.N2, L = a.L, S = a.S, lgS = __ffs(S) - 1;
  const bool on = tid < N, has_l = on && tid > 0, has_r = tid + 1 < N;
  float *drow = sm;                // [S][M][N] distance rows of the current chunk
  float *irow = drow + S * M * N;  // [2][CI][N] image rows of the last 2 steps
  unsigned char *trow = reinterpret_cast<unsigned char *>(irow + 2 * CI * N);  // TAPE: [S][N]
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
  // own old distances and image values of the next PF steps, loaded
  // (through L2) while the current steps compute: PF register sets, the
  // loop unrolled by PF so each set stays in registers
  constexpr int PF = 2;  // 4 was measured no faster (and spills beside the tape)
  float nd[PF][M], ni[PF][CI > 0 ? CI : 1];
  auto load = [&](int set) {
#pragma unroll
    for (int m = 0; m < M; m++) nd[set][m] = __ldcg(a.dsrc[m] + roff);
#pragma unroll
    for (int c = 0; c < CI; c++) ni[set][c] = __ldcg(a.img + c * a.img_cs + roff);
    roff += rstep;
  };
#pragma unroll
  for (int k = 0; k < PF; k++)
    if (on && k < L) load(k);
  auto step = [&](int t, int set) {
    float best[M], ic[CI > 0 ? CI : 1];
#pragma unroll
    for (int m = 0; m < M; m++) best[m] = nd[set][m];
#pragma unroll
    for (int c = 0; c < CI; c++) ic[c] = ni[set][c];
    if (on && t + PF < L) load(set);
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
            else if (C == 1)  // the reference's l_grad * |d| (any sign of l_grad)
              v = __fadd_rn(__fadd_rn(dq, e[m][o + 1]), __fmul_rn(lg[m], fabsf(d)));
            else
              v = __fadd_rn(__fadd_rn(dq, e[m][o + 1]), __fmul_rn(lg[m], l1));
            best[m] = fminf(best[m], v);
          }
        };
        if (TAPE) {
          // map 0 alone: the three candidates computed independently, then
          // strict comparisons in stencil order (a later candidate wins only
          // when smaller; the value is the set's minimum either way)
          const float qn = __int_as_float(0x7fffffff);
          float v[3];
#pragma unroll
          for (int o = -1; o <= 1; o++) {
            const float keep = best[0];
            best[0] = __int_as_float(0x7f800000);
            cand(o);
            v[o + 1] = best[0];
            best[0] = keep;
          }
          if (!has_l) v[0] = qn;
          if (!has_r) v[2] = qn;
          unsigned code = kTapeSelf;
          float b = best[0];
#pragma unroll
          for (int o = 0; o < 3; o++) {
            if (v[o] < b) b = v[o], code = 1 + o;
          }
          best[0] = b;
          trow[(t & (S - 1)) * N + tid] = (unsigned char)code;
        } else {
          cand(0);
          if (has_l) cand(-1);
          if (has_r) cand(1);
        }
      } else if (TAPE) {
        trow[tid] = (unsigned char)kTapeSelf;  // step 0 has no candidates
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
      if (TAPE && on && a.tape) {
        // the tape in the read layout, whole rows
        for (int j = 0; j < Sn; j++)
          a.tape[(a.dir > 0 ? t0 + j : L - 1 - t0 - j) * a.s_str + tid] = trow[j * N + tid];
      }
      __syncthreads();
    }
  };
  for (int t = 0; t < L; t += PF) {
#pragma unroll
    for (int k = 0; k < PF; k++)
      if (t + k < L) step(t + k, k);
  }
}

}  // namespace fgi
