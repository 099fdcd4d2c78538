// Warp tiles: one pass of a 2D transform over rows of up to kWarpTileMaxRow
// cells in one CTA, each warp running its own strip of the row with no
// block-wide barrier between steps.
//
//   D[t][x] = min(D[t][x], min_{k in -1,0,1} D[t-1][x+k] + l_eucl*ld[k] + l_grad*L1(I[t][x], I[t-1][x+k]))
//   (reference: FastGeodis/fastgeodis_cpu.cpp:53-162)
//
// A warp owns T2 cells of the row and covers them with halos of K cells on
// each side: kWarpCells = 128 region cells, 4 consecutive cells per lane
// (T2 = 128 - 2K; a row of at most 128 cells is one warp with no halo).  A
// lane keeps its 4 cells of the previous row in registers and takes the
// neighbouring lanes' edge cells with shuffles, so a step is a chain of two
// shuffles, the candidates and the minimum, with no shared memory and no
// barrier.  Every K steps the warps hand over: each lane stores its own cells
// of the chunk's last row into a shared row (two parities), one barrier, and
// each halo cell takes its owner's value.  Cells within j of a region's outer
// end are stale at chunk step j, but an own cell (at least K from it) never
// reads one before the next hand-off.  Own old distances and image values
// are loaded through L2 PF steps ahead into registers (16-byte loads where
// the row allows); own cells are written in place each step (a pass that
// changes layout runs in place and a transpose follows).  One image channel
// (or none: l_grad == 0), one or two maps.  Arithmetic as every other path:
// the same candidate expression in the reference's operation order.
#include "fg_pass.cuh"

namespace fgi {
namespace {

constexpr unsigned kFull = 0xffffffffu;

template <int M, int MODE, int PF>
__global__ void __launch_bounds__(kWarpTileMaxThreads, 1) fg_warp_tile_kernel(const PassArgs a) {
  extern __shared__ __align__(16) float sm[];  // [2 parities][M][N2]: own cells at hand-offs
  constexpr bool IMG = MODE != MODE_EUCLID;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int L = a.L, S = a.S, lgS = __ffs(S) - 1, N2 = a.N2, T2 = a.T2, K = a.K2;
  const int g0 = w * T2 - K + 4 * lane;  // this lane's first cell of the row
  const int o0 = w * T2, o1 = min(o0 + T2, N2);
  const float qnan = __int_as_float(0x7fffffff);
  bool valid[4], own[4];
#pragma unroll
  for (int i = 0; i < 4; i++) {
    const int g = g0 + i;
    valid[i] = g >= 0 && g < N2;
    own[i] = valid[i] && g >= o0 && g < o1;
  }
  const bool all_valid = valid[0] && valid[1] && valid[2] && valid[3];
  const bool all_own = own[0] && own[1] && own[2] && own[3];
  const bool vec = a.vec != 0;
  float e[M][3], lg[M];
#pragma unroll
  for (int m = 0; m < M; m++) {
    lg[m] = a.lg[m];
#pragma unroll
    for (int n = 0; n < 3; n++) e[m][n] = a.e[m][n];
  }

  // own inputs of the next PF steps: old distances and image values
  float nd[PF][M][4], ni[PF][4];
  const long long rstep = a.dir > 0 ? a.s_str : -a.s_str;
  long long roff = (a.dir > 0 ? 0 : (long long)(L - 1) * a.s_str) + g0;  // next step to load
  auto load = [&](int set) {
    if (vec && all_valid) {
#pragma unroll
      for (int m = 0; m < M; m++) {
        const float4 v = __ldcg(reinterpret_cast<const float4 *>(a.dsrc[m] + roff));
        nd[set][m][0] = v.x, nd[set][m][1] = v.y, nd[set][m][2] = v.z, nd[set][m][3] = v.w;
      }
      if (IMG) {
        const float4 v = __ldcg(reinterpret_cast<const float4 *>(a.img + roff));
        ni[set][0] = v.x, ni[set][1] = v.y, ni[set][2] = v.z, ni[set][3] = v.w;
      }
    } else {
#pragma unroll
      for (int i = 0; i < 4; i++) {
#pragma unroll
        for (int m = 0; m < M; m++) nd[set][m][i] = valid[i] ? __ldcg(a.dsrc[m] + roff + i) : qnan;
        ni[set][i] = IMG && valid[i] ? __ldcg(a.img + roff + i) : 0.0f;
      }
    }
    roff += rstep;
  };
#pragma unroll
  for (int k = 0; k < PF; k++)
    if (k < L) load(k);

  float pd[M][4], pi[4], pil = 0.0f, pir = 0.0f;  // the previous row: this lane's cells, image edges
  const long long wstep = a.dir > 0 ? a.ws_str : -a.ws_str;
  long long woff = (a.dir > 0 ? 0 : (long long)(L - 1) * a.ws_str) + g0;
  auto step = [&](int t, int set) {
    float od[M][4], ci[4], nw[M][4];
#pragma unroll
    for (int i = 0; i < 4; i++) {
      ci[i] = ni[set][i];
#pragma unroll
      for (int m = 0; m < M; m++) od[m][i] = nd[set][m][i];
    }
    if (t + PF < L) load(set);
    if (t == 0) {
#pragma unroll
      for (int m = 0; m < M; m++)
#pragma unroll
        for (int i = 0; i < 4; i++) nw[m][i] = valid[i] ? od[m][i] : qnan;
    } else {
      if (K > 0 && (t & (S - 1)) == 0) {
        // the halo cells of the previous row from their owners (stored
        // before the barrier at the end of the previous step)
        const float *src = sm + ((t >> lgS) & 1) * M * N2;
#pragma unroll
        for (int i = 0; i < 4; i++)
          if (valid[i] && !own[i]) {
#pragma unroll
            for (int m = 0; m < M; m++) pd[m][i] = src[m * N2 + g0 + i];
          }
      }
#pragma unroll
      for (int m = 0; m < M; m++) {
        // the previous row at cells g0-1 .. g0+4: the neighbour lanes' edge
        // cells (outside the warp's region: missing, NaN)
        float x[6];
        x[0] = __shfl_up_sync(kFull, pd[m][3], 1);
        x[5] = __shfl_down_sync(kFull, pd[m][0], 1);
        if (lane == 0) x[0] = qnan;
        if (lane == 31) x[5] = qnan;
#pragma unroll
        for (int i = 0; i < 4; i++) x[i + 1] = pd[m][i];
        const float xi[6] = {pil, pi[0], pi[1], pi[2], pi[3], pir};
#pragma unroll
        for (int i = 0; i < 4; i++) {
          float best = od[m][i];
#pragma unroll
          for (int o = -1; o <= 1; o++) {
            const float dq = x[i + 1 + o];
            float v;
            if (MODE == MODE_EUCLID) {
              v = __fadd_rn(dq, e[m][o + 1]);
            } else {
              const float d = __fsub_rn(ci[i], xi[i + 1 + o]);
              if (MODE == MODE_GEO)
                v = __fadd_rn(dq, fabsf(d));
              else  // the reference's l_grad * |d| (any sign of l_grad)
                v = __fadd_rn(__fadd_rn(dq, e[m][o + 1]), __fmul_rn(lg[m], fabsf(d)));
            }
            best = fminf(best, v);  // a NaN neighbour (missing) never wins
          }
          nw[m][i] = valid[i] ? best : qnan;
        }
      }
      // own cells in place
      if (vec && all_own) {
#pragma unroll
        for (int m = 0; m < M; m++)
          *reinterpret_cast<float4 *>(a.ddst[m] + woff) = make_float4(nw[m][0], nw[m][1], nw[m][2], nw[m][3]);
      } else {
#pragma unroll
        for (int i = 0; i < 4; i++)
          if (own[i]) {
#pragma unroll
            for (int m = 0; m < M; m++) a.ddst[m][woff + i] = nw[m][i];
          }
      }
    }
    woff += wstep;
    // this row becomes the previous one; the image edges move with it
#pragma unroll
    for (int i = 0; i < 4; i++) {
      pi[i] = ci[i];
#pragma unroll
      for (int m = 0; m < M; m++) pd[m][i] = nw[m][i];
    }
    if (IMG) {
      pil = __shfl_up_sync(kFull, ci[3], 1);
      pir = __shfl_down_sync(kFull, ci[0], 1);
    }
    if (K > 0 && ((t + 1) & (S - 1)) == 0 && t + 1 < L) {
      // last step of a chunk: own cells for the neighbour warps' halos
      float *dst = sm + (((t + 1) >> lgS) & 1) * M * N2;
#pragma unroll
      for (int i = 0; i < 4; i++)
        if (own[i]) {
#pragma unroll
          for (int m = 0; m < M; m++) dst[m * N2 + g0 + i] = pd[m][i];
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

template <int M, int MODE>
int launch_wt(const PassArgs &a, const LaunchCfg &c, cudaStream_t s) {
  constexpr int PF = M == 1 ? 8 : 4;  // steps of own inputs ahead: 8 covers an L2 round trip at ~0.05 us a step
  void *args[] = {const_cast<PassArgs *>(&a)};
  const cudaError_t e =
      cudaLaunchKernel((const void *)fg_warp_tile_kernel<M, MODE, PF>, dim3(1), dim3(c.threads), args, c.smem, s);
  if (e != cudaSuccess) return set_error(FG_ERR_CUDA, cudaGetErrorString(e));
  return FG_OK;
}

template <int M>
int launch_wt_mode(const PassArgs &a, const LaunchCfg &c, int mode, cudaStream_t s) {
  if (mode == MODE_EUCLID) return launch_wt<M, MODE_EUCLID>(a, c, s);
  if (a.C != 1) return set_error(FG_ERR_UNSUPPORTED, "warp tiles read one image channel");
  if (mode == MODE_GEO) return launch_wt<M, MODE_GEO>(a, c, s);
  return launch_wt<M, MODE_GENERAL>(a, c, s);
}

}  // namespace

// Shared memory of a warp-tile pass: two rows per map for the hand-off
// (none with one warp).
size_t warp_tile_smem(int M, int N2, int K) { return K > 0 ? (size_t)2 * M * N2 * 4 : 0; }

int launch_warp_tiles(const PassArgs &a, const LaunchCfg &c, int M, int mode, bool wt, cudaStream_t s) {
  if (wt) return set_error(FG_ERR_UNSUPPORTED, "warp tiles write in place (a transpose moves the map)");
  const int K = a.K2, T2 = a.T2;
  const bool shape_ok = K == 0 ? (a.N2 <= kWarpCells && T2 >= a.N2 && c.threads == 32)
                               : (K == a.S && T2 == kWarpCells - 2 * K && c.threads == 32 * ((a.N2 + T2 - 1) / T2));
  if (!shape_ok || c.threads > kWarpTileMaxThreads || a.N2 > kWarpTileMaxRow)
    return set_error(FG_ERR_UNSUPPORTED, "warp tiles: 128-cell regions, T2 = 128 - 2K, K = S, one warp per tile");
  if (M == 1) return launch_wt_mode<1>(a, c, mode, s);
  if (M == 2) return launch_wt_mode<2>(a, c, mode, s);
  return set_error(FG_ERR_UNSUPPORTED, "a pass updates one or two distance maps");
}

}  // namespace fgi
