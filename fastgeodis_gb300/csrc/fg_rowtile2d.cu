// Row tiles: one pass of a 2D transform whose rows are split into tiles of
// T2 cells, one CTA per tile and one thread per cell of the tile and its
// halos of S cells (the row body's layout, fg_row2d.cuh, on a strip of the
// row instead of all of it).
//
//   D[t][x] = min(D[t][x], min_{k in -1,0,1} D[t-1][x+k] + l_eucl*ld[k] + l_grad*L1(I[t][x], I[t-1][x+k]))
//   (reference: FastGeodis/fastgeodis_cpu.cpp:53-162)
//
// A strip runs S steps on its own and hands over at the end of every chunk
// of S steps: its own cells go to 64-bit exchange words (value | chunk epoch
// << 32, the tile kernel's words, fg_pass.cuh), and at the start of the next
// chunk each halo cell of the previous row takes its owner's word (bounded
// waits: FG_ERR_TIMEOUT).  A row's halo is only its two ends, so a long
// period is cheap: cells within j of a halo's outer end are stale at chunk
// step j, but an own cell (at least S from it) never reads one before the
// next hand-off, so every cell computes every step (a plan of one tile,
// for rows of up to 32 cells, has no halos and no hand-off).  Each thread keeps its
// cell's old distance and image values 4-8 steps ahead in registers; the
// previous row's distances and image values are shared-memory rows with a
// NaN apron (cells outside the image never win a min).  Each step's own
// cells are written in place (measured: holding a chunk's rows and writing
// them at its end cost 7-13%, the burst of stores stalling the next step);
// a pass that changes layout runs in place and a tiled transpose then moves
// the map (5-7% faster than writing the chunk's rows transposed from shared
// memory at its end).
// Arithmetic as every other path: the same candidate expression in the
// reference's operation order.
//
// Cluster form (CLU, 2 to 16 tiles, halos no wider than a tile): the CTAs are
// one thread-block cluster and the hand-off goes through distributed shared
// memory instead: at a chunk's end each own cell within S of a tile boundary
// is stored with st.async into the neighbour's receive rows (two parities,
// one per side), completing on the neighbour's mbarrier of that parity; at
// the next chunk's start the halo threads wait on it (bounded) and copy the
// received row into the ring.  A neighbour cannot be two hand-offs ahead (it
// needs this CTA's row of the hand-off between), so two parities suffice.
#include "fg_pass.cuh"
#include "fg_wait.cuh"

namespace fgi {
namespace {

__device__ __forceinline__ void st_word_rt(unsigned long long *p, unsigned long long v) {
  asm volatile("st.relaxed.gpu.global.b64 [%0], %1;\n" ::"l"(p), "l"(v) : "memory");
}

template <int C, int M, int MODE, bool CLU>
__global__ void __launch_bounds__(512, 1) fg_row_tile_kernel(const PassArgs a) {
  extern __shared__ __align__(16) float sm[];
  constexpr int CI = MODE == MODE_EUCLID ? 0 : C;  // image channels read
  const int tid = threadIdx.x;
  const int L = a.L, S = a.S, lgS = __ffs(S) - 1, N2 = a.N2;
  const int ti = blockIdx.x, T2 = a.T2, K = a.K2;
  const int R = T2 + 2 * K, RP = a.rowf;  // region cells, floats per shared row (apron + R + apron)
  constexpr int SR = 2;  // distance rows kept: a step reads one while it writes the other
  const int g2 = ti * T2 - K + tid;       // this thread's cell of the row
  const bool valid = tid < R && g2 >= 0 && g2 < N2;
  const bool own = valid && tid >= K && tid < K + T2;
  const bool halo = valid && !own;
  const float qnan = __int_as_float(0x7fffffff);
  float *drow = sm;                  // [SR][M][RP], cell x of the region at index x + 1
  float *irow = drow + SR * M * RP;  // [2][CI][RP]
  for (int i = tid; i < (SR * M + 2 * CI) * RP; i += blockDim.x) sm[i] = qnan;
  const int rstep = a.dir > 0 ? (int)a.s_str : -(int)a.s_str;
  const int wstep = a.dir > 0 ? (int)a.ws_str : -(int)a.ws_str;
  int roff = (a.dir > 0 ? 0 : (L - 1) * (int)a.s_str) + g2;  // read offset of the next step to load
  int woff = (a.dir > 0 ? 0 : (L - 1) * (int)a.ws_str) + g2 * (int)a.wst2;
  float e[M][3], lg[M];
#pragma unroll
  for (int m = 0; m < M; m++) {
    lg[m] = a.lg[m];
#pragma unroll
    for (int n = 0; n < 3; n++) e[m][n] = a.e[m][n];
  }
  // exchange words of this cell: [2 parities][kMaxMaps][N2]
  unsigned long long *const xw = a.xch + g2;
  const long long xpar = (long long)kMaxMaps * N2;
  // cluster form: receive rows [2 parities][2 sides][M][K] after the rings,
  // then two mbarriers (one per parity)
  float *const rbuf = irow + 2 * CI * RP;
  const int nq = (L + S - 1) / S - 1;  // hand-offs of the pass
  const int xo = tid - K;              // this thread's cell within the tile (own cells: 0 .. T2-1)
  unsigned cbar = 0, rbl = 0, rbr = 0, barl = 0, barr = 0, cl_bytes = 0;
  bool pushl = false, pushr = false, dead = false;
  if (CLU) {
    const int tiles = a.tiles2;
    const unsigned rb = smem_u32(rbuf);
    cbar = rb + 4u * (unsigned)(4 * M * K);
    const int nl = ti > 0 ? K : 0, nr = ti < tiles - 1 ? min(K, N2 - (ti + 1) * T2) : 0;
    cl_bytes = (unsigned)((nl + nr) * M * 4);
    // own cells within K of a boundary go to that neighbour's halo of this side
    pushl = own && ti > 0 && xo < K;
    pushr = own && ti < tiles - 1 && xo >= T2 - K;
    if (pushl) rbl = cl_map(rb, (unsigned)(ti - 1)), barl = cl_map(cbar, (unsigned)(ti - 1));
    if (pushr) rbr = cl_map(rb, (unsigned)(ti + 1)), barr = cl_map(cbar, (unsigned)(ti + 1));
    if (tid == 0) {
      mbar_init(cbar, 1);
      mbar_init(cbar + 8, 1);
      mbar_fence_init();
      if (nq >= 1) mbar_expect(cbar, cl_bytes);      // hand-off 0
      if (nq >= 2) mbar_expect(cbar + 8, cl_bytes);  // hand-off 1
    }
  }
  __syncthreads();
  if (CLU) cl_sync();  // rings filled and mbarriers armed in every CTA before the first store

  // steps of own inputs held in registers, loaded through L2 ahead of their
  // use: deep enough to cover DRAM latency for images beyond L2 (on 4096^2
  // and 8192^2 images, 2 -> 4 -> 8 steps took 12.8 -> 10.0 -> 8.5 ms and
  // 27.0 -> 20.7 -> 17.4 ms), 4 where 8 would spill (4 channels, two maps)
  constexpr int PF = CI + M <= 4 ? 8 : 4;
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
    if (valid && k < L) load(k);

  auto step = [&](int t, int set) {
    float best[M], ic[CI > 0 ? CI : 1];
#pragma unroll
    for (int m = 0; m < M; m++) best[m] = nd[set][m];
#pragma unroll
    for (int c = 0; c < CI; c++) ic[c] = ni[set][c];
    if (valid && t + PF < L) load(set);
    if (CLU && t > 0 && (t & (S - 1)) == 0) {
      // the halo's previous row from the neighbours' stores of hand-off q
      const int q = (t >> lgS) - 1;
      const unsigned bar = cbar + (unsigned)(q & 1) * 8u;
      if ((halo || tid == 0) && !dead) {
        if (!wait_phase(bar, (unsigned)(q >> 1) & 1u, a.status, kClusterSpinLimit)) dead = true;  // results void
        if (tid == 0 && !dead && q + 2 < nq) mbar_expect(bar, cl_bytes);  // the same parity's next hand-off
      }
      if (halo) {
        const float *src = rbuf + (q & 1) * 2 * M * K + (tid < K ? tid : M * K + tid - K - T2);
#pragma unroll
        for (int m = 0; m < M; m++) drow[((t - 1) & (SR - 1)) * M * RP + m * RP + tid + 1] = src[m * K];
      }
      __syncthreads();
    } else if (t > 0 && (t & (S - 1)) == 0) {
      // the halo's previous row from the owners' words of the chunk just ended
      if (halo) {
        const unsigned want = a.epoch_base + (unsigned)(t >> lgS);
        const unsigned long long *w = xw + (long long)((t >> lgS) & 1) * xpar;
        unsigned long long wd[M];
#pragma unroll
        for (int m = 0; m < M; m++) wd[m] = ld_word(w + (long long)m * N2);
#pragma unroll
        for (int m = 0; m < M; m++) {
          wd[m] = wait_word(w + (long long)m * N2, want, wd[m], a.status, kSpinLimit);
          drow[((t - 1) & (SR - 1)) * M * RP + m * RP + tid + 1] = __uint_as_float((unsigned)wd[m]);
        }
      }
      __syncthreads();
    }
    if (valid) {
      if (t > 0) {
        const float *dp = drow + ((t - 1) & (SR - 1)) * M * RP + tid + 1;
        const float *ip = irow + ((t - 1) & 1) * CI * RP + tid + 1;
#pragma unroll
        for (int o = -1; o <= 1; o++) {
          float l1 = 0.0f, d = 0.0f;
          if (MODE != MODE_EUCLID) {
            if (C == 1) {
              d = __fsub_rn(ic[0], ip[o]);
              l1 = fabsf(d);
            } else {
#pragma unroll
              for (int c = 0; c < CI; c++) l1 = __fadd_rn(l1, fabsf(__fsub_rn(ic[c], ip[c * RP + o])));
            }
          }
#pragma unroll
          for (int m = 0; m < M; m++) {
            const float dq = dp[m * RP + o];
            float v;
            if (MODE == MODE_EUCLID)
              v = __fadd_rn(dq, e[m][o + 1]);
            else if (MODE == MODE_GEO)
              v = __fadd_rn(dq, l1);
            else if (C == 1)  // the reference's l_grad * |d| (any sign of l_grad)
              v = __fadd_rn(__fadd_rn(dq, e[m][o + 1]), __fmul_rn(lg[m], fabsf(d)));
            else
              v = __fadd_rn(__fadd_rn(dq, e[m][o + 1]), __fmul_rn(lg[m], l1));
            best[m] = fminf(best[m], v);  // a NaN neighbour (outside the image) never wins
          }
        }
      }
      float *dc = drow + (t & (SR - 1)) * M * RP + tid + 1;
#pragma unroll
      for (int m = 0; m < M; m++) dc[m * RP] = best[m];
      float *icw = irow + (t & 1) * CI * RP + tid + 1;
#pragma unroll
      for (int c = 0; c < CI; c++) icw[c * RP] = ic[c];
      if (own) {
        if (t > 0) {
#pragma unroll
          for (int m = 0; m < M; m++) a.ddst[m][woff] = best[m];
        }
        if (CLU && ((t + 1) & (S - 1)) == 0 && t + 1 < L) {
          // last step of a chunk: this cell into the neighbours' receive rows
          const int q = ((t + 1) >> lgS) - 1;
          const unsigned po = (unsigned)((q & 1) * 2 * M * K), bo = (unsigned)(q & 1) * 8u;
          if (pushl) {  // the left neighbour's right halo, cell xo
#pragma unroll
            for (int m = 0; m < M; m++) st_async1(rbl + 4u * (po + (unsigned)(M * K + m * K + xo)), best[m], barl + bo);
          }
          if (pushr) {  // the right neighbour's left halo, cell xo - (T2 - K)
#pragma unroll
            for (int m = 0; m < M; m++)
              st_async1(rbr + 4u * (po + (unsigned)(m * K + xo - (T2 - K))), best[m], barr + bo);
          }
        } else if (((t + 1) & (S - 1)) == 0 && t + 1 < L && a.tiles2 > 1) {
          // last step of a chunk: publish this cell for the neighbours' halos
          const unsigned long long ep = (unsigned long long)(a.epoch_base + (unsigned)((t + 1) >> lgS)) << 32;
          unsigned long long *w = xw + (long long)(((t + 1) >> lgS) & 1) * xpar;
#pragma unroll
          for (int m = 0; m < M; m++) st_word_rt(w + (long long)m * N2, ep | __float_as_uint(best[m]));
        }
      }
    }
    woff += wstep;
    __syncthreads();
  };
  for (int t = 0; t < L; t += PF) {
#pragma unroll
    for (int k = 0; k < PF; k++)
      if (t + k < L) step(t + k, k);
  }
  if (CLU) {
    cl_sync();  // no CTA leaves while a neighbour may still store into its shared memory
    if (tid == 0) {
      mbar_inval(cbar);
      mbar_inval(cbar + 8);
    }
  }
}

template <int C, int M, int MODE>
int launch_rt(const PassArgs &a, const LaunchCfg &c, bool clu, cudaStream_t s) {
  if (clu) {
    static unsigned long long configured_cl = 0;  // bit per device (set under the engine's launch lock)
    return launch_one_cluster((const void *)fg_row_tile_kernel<C, M, MODE, true>, configured_cl, a, c, s);
  }
  void (*fn)(const PassArgs) = fg_row_tile_kernel<C, M, MODE, false>;
  static unsigned long long configured = 0;  // bit per device (set under the engine's launch lock)
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return set_error(FG_ERR_CUDA, cudaGetErrorString(e));
  if (dev < 64 && !(configured & (1ull << dev))) {
    e = cudaFuncSetAttribute((const void *)fn, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024);
    if (e != cudaSuccess) return set_error(FG_ERR_CUDA, cudaGetErrorString(e));
    configured |= 1ull << dev;
  }
  void *args[] = {const_cast<PassArgs *>(&a)};
  if (c.tiles > 1)
    e = cudaLaunchCooperativeKernel((const void *)fn, dim3(c.tiles), dim3(c.threads), args, c.smem, s);
  else
    e = cudaLaunchKernel((const void *)fn, dim3(1), dim3(c.threads), args, c.smem, s);
  if (e != cudaSuccess) return set_error(FG_ERR_CUDA, cudaGetErrorString(e));
  return FG_OK;
}

template <int M, int MODE>
int launch_rt_c(const PassArgs &a, const LaunchCfg &c, bool clu, cudaStream_t s) {
  switch (a.C) {
    case 1: return launch_rt<1, M, MODE>(a, c, clu, s);
    case 2: return launch_rt<2, M, MODE>(a, c, clu, s);
    case 3: return launch_rt<3, M, MODE>(a, c, clu, s);
    case 4: return launch_rt<4, M, MODE>(a, c, clu, s);
    default: return set_error(FG_ERR_UNSUPPORTED, "row tiles read 1 to 4 image channels");
  }
}

template <int M>
int launch_rt_mode(const PassArgs &a, const LaunchCfg &c, int mode, bool clu, cudaStream_t s) {
  if (mode == MODE_EUCLID) return launch_rt<1, M, MODE_EUCLID>(a, c, clu, s);
  if (mode == MODE_GEO) return launch_rt_c<M, MODE_GEO>(a, c, clu, s);
  return launch_rt_c<M, MODE_GENERAL>(a, c, clu, s);
}

}  // namespace

size_t row_tile_smem(int cimg, int M, int R, int S, bool clu) {
  // two rows of distances and of image values; the cluster form adds its
  // receive rows (2 parities, 2 sides, K = S cells per map) and two mbarriers
  const size_t rings = (size_t)(2 * M + 2 * cimg) * ring_pitch(R + 2) * 4;
  return rings + (clu ? (size_t)(4 * M * S + 4) * 4 : 0);
}

int launch_row_tiles(const PassArgs &a, const LaunchCfg &c, int M, int mode, bool wt, bool clu, cudaStream_t s) {
  if (wt) return set_error(FG_ERR_UNSUPPORTED, "row tiles write in place (a transpose moves the map)");
  if (c.threads > 512 || c.threads < a.T2 + 2 * a.K2)
    return set_error(FG_ERR_UNSUPPORTED, "row tiles: one thread per cell of a tile and its halos, at most 512");
  if (clu && (c.tiles != a.tiles2 || c.tiles < 2 || c.tiles > kMaxCluster || a.K2 != a.S || a.K2 > a.T2))
    return set_error(FG_ERR_UNSUPPORTED, "row tiles in a cluster: 2 to 16 tiles, halos of S cells at most a tile wide");
  if (M == 1) return launch_rt_mode<1>(a, c, mode, clu, s);
  if (M == 2) return launch_rt_mode<2>(a, c, mode, clu, s);
  return set_error(FG_ERR_UNSUPPORTED, "a pass updates one or two distance maps");
}

}  // namespace fgi
