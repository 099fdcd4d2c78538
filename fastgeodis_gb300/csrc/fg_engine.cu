// fastgeodis_gb300 engine: raster-scan generalised geodesic distance on GB300.
//
// One directional sweep ("pass") of the raster scan updates every cell of a
// step from the three (2D) or nine (3D) cells of the previous step:
//     D[t][x] = min(D[t][x], min_n D[t-1][x+n] + l_eucl*ld[n] + l_grad*L1(I[t][x], I[t-1][x+n]))
// (reference: FastGeodis/fastgeodis_cpu.cpp:53-162, :203-340;
//  FastGeodis/fastgeodis_cuda.cu:131-202, :407-493).
//
// Work decomposition (this build's own design, not the reference's):
//   * The cross-section of the swept axis is cut into tiles; one CTA owns one
//     tile for the whole pass and walks all steps.  Grid = tiles, launched
//     cooperatively so that every CTA is resident.
//   * A CTA computes its tile plus a halo of K cells on each side.  The halo
//     lets it run S <= K steps on its own; every S steps it takes the exact
//     boundary row from its neighbours (published through per-tile progress
//     flags with release/acquire) and continues.  Halo cells that have
//     drifted are never written back, so results are exact.
//   * Steps are staged through shared memory in chunks of S positions, in a
//     ring of three buffers filled by cp.async one chunk ahead; the swept
//     axis may be the contiguous one (columns of a 2D image, W of a volume),
//     in which case every cell's S positions form one 32-byte segment.
//   * No transposes: each axis is addressed in place with its own strides.
//   * Arithmetic is float32 with round-to-nearest on every operation, in the
//     reference CPU order ((D + l_eucl*ld) + l_grad*L1); no FMA contraction.
//     The step-length table is computed on the host with IEEE sqrt.
//   * Cells outside the image hold NaN in shared memory; fminf ignores NaN
//     candidates, which is the reference's "skip out-of-bounds neighbour".
//
// The C ABI at the bottom (declared in include/fastgeodis_gb300.h) composes
// passes into the plain, signed and GSF transforms of the reference.

#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <math.h>

#include <algorithm>
#include <atomic>
#include <map>
#include <mutex>
#include <string>
#include <tuple>
#include <vector>

#include "../../include/fastgeodis_gb300.h"

namespace {

constexpr int kThreads = 512;       // threads per CTA
constexpr int kMaxMaps = 4;         // distance maps swept together (shared image)
constexpr int kMaxRegion = kThreads * 4;  // region cells (one run of 4 cells per thread)
constexpr int kMaxTiles = 2048;     // progress flags in a workspace
constexpr size_t kSmemBudget = 227 * 1024 - 2048;
constexpr size_t kWsHeader = 256;   // status word and spare
constexpr size_t kWsFlags = kMaxTiles * sizeof(unsigned);
constexpr unsigned kSpinLimit = 1u << 24;  // ~1-2 s of polling before FG_ERR_TIMEOUT

struct PassArgs {
  const float *img;      // channel 0 of the image
  long long img_cs;      // elements between image channels
  int C;                 // image channels
  int M;                 // distance maps swept in this launch
  float *dist[kMaxMaps]; // channel-0 plane of each map (same layout as the image)
  float lg[kMaxMaps];    // l_grad per map
  float e[kMaxMaps][9];  // l_eucl * ld[n] per map and neighbour
  int L;                 // steps along the swept axis
  long long s_str;       // element stride of one step
  int dir;               // +1 forward, -1 backward
  int N1, N2;            // cross-section extents (N1 = 1 for 2D)
  long long st1, st2;    // cross-section strides
  int T1, T2, K1, K2;    // own tile extents and halo widths
  int tiles1, tiles2;
  int S;                 // chunk depth (positions per chunk), divides 32
  int stepc;             // swept axis is the contiguous one
  int B2, NCP;           // buffer row width (with apron) and floats per position
  int NB;                // ring buffers (chunks); NB - 2 chunks are prefetched ahead
  unsigned *flags;
  unsigned flag_base;
  int *status;
};

__device__ __forceinline__ void cp_async4(float *dst, const float *src) {
  unsigned d = (unsigned)__cvta_generic_to_shared(dst);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
// wait until at most `pending` of this thread's cp.async groups are in flight
__device__ __forceinline__ void cp_async_wait(int pending) {
  switch (pending) {
    case 0: asm volatile("cp.async.wait_group 0;\n" ::: "memory"); break;
    case 1: asm volatile("cp.async.wait_group 1;\n" ::: "memory"); break;
    case 2: asm volatile("cp.async.wait_group 2;\n" ::: "memory"); break;
    case 3: asm volatile("cp.async.wait_group 3;\n" ::: "memory"); break;
    default: asm volatile("cp.async.wait_group 4;\n" ::: "memory"); break;
  }
}

__device__ __forceinline__ unsigned ld_acquire(const unsigned *p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];\n" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_release(unsigned *p, unsigned v) {
  asm volatile("st.release.gpu.global.u32 [%0], %1;\n" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ int ld_status(const int *p) {
  int v;
  asm volatile("ld.relaxed.gpu.global.s32 %0, [%1];\n" : "=r"(v) : "l"(p) : "memory");
  return v;
}

constexpr unsigned kOwnBit = 1u << 30;
constexpr unsigned kCellMask = kOwnBit - 1;

// Arithmetic of one candidate.  GENERAL is the reference expression
// (D + l_eucl*ld) + l_grad*L1.  EUCLID (l_grad == 0) and GEO (l_eucl == 0,
// l_grad == 1) drop a term that is exactly +0 or exactly a factor of 1 for
// finite inputs, so they return the same bits with less work.
enum Mode { MODE_GENERAL = 0, MODE_EUCLID = 1, MODE_GEO = 2 };

// One directional pass over one tile per CTA.  CROSS = 1 (2D image, 3-cell
// stencil) or 2 (volume, 9-cell stencil).  ONECH = single image channel.
// M = distance maps updated together (they share the image).
//
// Shared-memory buffer of one position: rows of B2 floats (B2 a multiple of
// 4); region cell (r1, r2) lives at (r1 + A1) * B2 + 4 + r2, so every run of 4
// cells starting at a multiple of 4 is 16-byte aligned.  Everything that is
// not an in-image region cell holds NaN.
template <int CROSS, bool ONECH, int M, int MODE>
__global__ void __launch_bounds__(kThreads, 1) fg_pass_kernel(const PassArgs a) {
  extern __shared__ __align__(16) float sm[];
  constexpr int A1 = CROSS == 2 ? 1 : 0;  // apron rows above the region
  constexpr bool USE_IMG = MODE != MODE_EUCLID;
  const int NT = blockDim.x;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int nwarps = NT >> 5;

  const int tile = blockIdx.x;
  const int ti1 = tile / a.tiles2, ti2 = tile - ti1 * a.tiles2;
  const int C = a.C, S = a.S, L = a.L;
  const int CI = USE_IMG ? C : 0;  // image arrays staged
  const int A = CI + M;            // arrays per position
  const int R1 = CROSS == 2 ? a.T1 + 2 * a.K1 : 1;
  const int R2 = a.T2 + 2 * a.K2;
  const int B2 = a.B2, NCP = a.NCP;
  const int rs1 = CROSS == 2 ? ti1 * a.T1 - a.K1 : 0;
  const int rs2 = ti2 * a.T2 - a.K2;
  const int l1lo = max(0, -rs1), l1hi = min(R1, a.N1 - rs1);
  const int l2lo = max(0, -rs2), l2hi = min(R2, a.N2 - rs2);
  const int LR1 = l1hi - l1lo, LR2 = l2hi - l2lo;
  const int o1lo = CROSS == 2 ? a.K1 : 0;
  const int o1hi = CROSS == 2 ? a.K1 + min(a.T1, a.N1 - ti1 * a.T1) : 1;
  const int o2lo = a.K2, o2hi = a.K2 + min(a.T2, a.N2 - ti2 * a.T2);
  const int O1 = o1hi - o1lo, O2 = o2hi - o2lo;
  const int nload = LR1 * LR2, nown = O1 * O2;
  const int astride = S * NCP;              // floats between arrays of one buffer
  const int slot = A * astride;             // floats in one ring buffer
  const int NB = a.NB, PD = NB - 2;

  float *ring = sm;
  int2 *ltab = reinterpret_cast<int2 *>(sm + NB * slot);
  int2 *otab = ltab + nload;

  // --- set-up: NaN everywhere, cell tables, this thread's run ---
  const float qnan = __int_as_float(0x7fffffff);
  for (int i = tid; i < NB * slot; i += NT) ring[i] = qnan;
  for (int i = tid; i < nload; i += NT) {
    int l1 = l1lo + i / LR2, l2 = l2lo + i % LR2;
    int cell = (l1 + A1) * B2 + 4 + l2;
    bool own = l1 >= o1lo && l1 < o1hi && l2 >= o2lo && l2 < o2hi;
    long long g = (long long)(rs1 + l1) * a.st1 + (long long)(rs2 + l2) * a.st2;
    ltab[i] = make_int2((int)(cell | (own ? kOwnBit : 0u)), (int)g);
  }
  for (int i = tid; i < nown; i += NT) {
    int o1 = o1lo + i / O2, o2 = o2lo + i % O2;
    long long g = (long long)(rs1 + o1) * a.st1 + (long long)(rs2 + o2) * a.st2;
    otab[i] = make_int2((o1 + A1) * B2 + 4 + o2, (int)g);
  }
  const int rpr = (R2 + 3) >> 2;  // runs per region row
  int cb = -1;                    // first buffer cell of this thread's run
  unsigned valid = 0;             // which of its 4 cells are in-image region cells
  if (tid < R1 * rpr) {
    int r1 = tid / rpr, u = tid - (tid / rpr) * rpr;
    cb = (r1 + A1) * B2 + 4 + 4 * u;
    int g1 = rs1 + r1;
    for (int i = 0; i < 4; i++) {
      int r2 = 4 * u + i, g2 = rs2 + r2;
      if (r2 < R2 && g1 >= 0 && g1 < a.N1 && g2 >= 0 && g2 < a.N2) valid |= 1u << i;
    }
    if (!valid) cb = -1;
  }
  // neighbour tiles whose progress this CTA waits on
  int nbr = -1;
  if (tid < 8) {
    int d1, d2;
    if (CROSS == 2) {
      int k = tid < 4 ? tid : tid + 1;
      d1 = k / 3 - 1;
      d2 = k % 3 - 1;
    } else {
      d1 = 0;
      d2 = tid == 0 ? -1 : 1;
    }
    int n1 = ti1 + d1, n2 = ti2 + d2;
    bool ok = (CROSS == 2 || tid < 2) && n1 >= 0 && n1 < a.tiles1 && n2 >= 0 && n2 < a.tiles2;
    if (ok) nbr = n1 * a.tiles2 + n2;
  }
  const bool has_nb = a.tiles1 * a.tiles2 > 1;
  __syncthreads();

  auto pos = [&](int t) -> long long { return a.dir > 0 ? (long long)t : (long long)(L - 1 - t); };
  auto arr_src = [&](int ai) -> const float * { return ai < CI ? a.img + (long long)ai * a.img_cs : a.dist[ai - CI]; };
  auto buf = [&](int q, int ai, int j) -> float * { return ring + q * slot + ai * astride + j * NCP; };

  auto load_chunk = [&](int n, int q) {
    const int t0 = n * S, Sn = min(S, L - t0);
    if (!a.stepc) {
      for (int ai = 0; ai < A; ai++) {
        const float *gb = arr_src(ai);
        for (int j = 0; j < Sn; j++) {
          const float *gj = gb + pos(t0 + j) * a.s_str + (long long)rs2 * a.st2;
          float *dj = buf(q, ai, j) + A1 * B2 + 4;
          if (LR1 >= nwarps) {
            for (int l1 = l1lo + warp; l1 < l1hi; l1 += nwarps) {
              const float *g = gj + (long long)(rs1 + l1) * a.st1;
              float *d = dj + l1 * B2;
              for (int l2 = l2lo + lane; l2 < l2hi; l2 += 32) cp_async4(d + l2, g + l2);
            }
          } else {
            for (int l1 = l1lo; l1 < l1hi; l1++) {
              const float *g = gj + (long long)(rs1 + l1) * a.st1;
              float *d = dj + l1 * B2;
              for (int l2 = l2lo + tid; l2 < l2hi; l2 += NT) cp_async4(d + l2, g + l2);
            }
          }
        }
      }
    } else {
      const int cpw = 32 / S, j = lane % S;
      if (j < Sn) {
        const long long soff = pos(t0 + j) * a.s_str;
        for (int ai = 0; ai < A; ai++) {
          const float *gb = arr_src(ai) + soff;
          float *d = buf(q, ai, j);
          for (int i = warp * cpw + lane / S; i < nload; i += nwarps * cpw) {
            int2 e = ltab[i];
            cp_async4(d + (e.x & kCellMask), gb + e.y);
          }
        }
      }
    }
  };

  auto writeback = [&](int n, int q) {
    const int t0 = n * S, Sn = min(S, L - t0);
    if (!a.stepc) {
      for (int m = 0; m < M; m++) {
        for (int j = 0; j < Sn; j++) {
          float *gj = a.dist[m] + pos(t0 + j) * a.s_str + (long long)rs2 * a.st2;
          const float *sj = buf(q, CI + m, j) + A1 * B2 + 4;
          if (O1 >= nwarps) {
            for (int o1 = o1lo + warp; o1 < o1hi; o1 += nwarps) {
              float *g = gj + (long long)(rs1 + o1) * a.st1;
              const float *s = sj + o1 * B2;
              for (int o2 = o2lo + lane; o2 < o2hi; o2 += 32) g[o2] = s[o2];
            }
          } else {
            for (int o1 = o1lo; o1 < o1hi; o1++) {
              float *g = gj + (long long)(rs1 + o1) * a.st1;
              const float *s = sj + o1 * B2;
              for (int o2 = o2lo + tid; o2 < o2hi; o2 += NT) g[o2] = s[o2];
            }
          }
        }
      }
    } else {
      const int cpw = 32 / S, j = lane % S;
      if (j < Sn) {
        const long long soff = pos(t0 + j) * a.s_str;
        for (int m = 0; m < M; m++) {
          float *g = a.dist[m] + soff;
          const float *s = buf(q, CI + m, j);
          for (int i = warp * cpw + lane / S; i < nown; i += nwarps * cpw) {
            int2 e = otab[i];
            g[e.y] = s[e.x];
          }
        }
      }
    }
  };

  // exact boundary row from the neighbours: halo cells of step t (buffer q, position j)
  auto refresh = [&](int t, int q, int j) {
    const long long soff = pos(t) * a.s_str;
    for (int i = tid; i < nload; i += NT) {
      int2 e = ltab[i];
      if (e.x & kOwnBit) continue;
      int cell = e.x & kCellMask;
#pragma unroll
      for (int m = 0; m < M; m++) buf(q, CI + m, j)[cell] = __ldcg(a.dist[m] + soff + e.y);
    }
  };

  auto wait_neighbours = [&](unsigned target) {
    if (nbr >= 0) {
      unsigned spins = 0;
      while ((int)(ld_acquire(a.flags + nbr) - target) < 0) {
        if (++spins > kSpinLimit || ld_status(a.status) != 0) {
          atomicCAS(a.status, 0, FG_ERR_TIMEOUT);
          break;
        }
        __nanosleep(32);
      }
      __threadfence();
    }
    __syncthreads();
  };

  // One step for this thread's run of 4 cells.  cur/prv point at array 0 of
  // the current and previous positions.
  auto compute_step = [&](const float *cur, const float *prv) {
    if (cb < 0) return;
    float best[M][4];
#pragma unroll
    for (int m = 0; m < M; m++) {
      float4 v = *reinterpret_cast<const float4 *>(cur + (CI + m) * astride + cb);
      best[m][0] = v.x, best[m][1] = v.y, best[m][2] = v.z, best[m][3] = v.w;
    }
    float ic[4] = {0.f, 0.f, 0.f, 0.f};
    if (USE_IMG && ONECH) {
      float4 v = *reinterpret_cast<const float4 *>(cur + cb);
      ic[0] = v.x, ic[1] = v.y, ic[2] = v.z, ic[3] = v.w;
    }
#pragma unroll
    for (int r = 0; r < (CROSS == 2 ? 3 : 1); r++) {
      const int d1 = CROSS == 2 ? r - 1 : 0;
      const float *pr = prv + cb + d1 * B2;
      float ip[6];
      if (USE_IMG && ONECH) {
        float4 v = *reinterpret_cast<const float4 *>(pr);
        ip[0] = pr[-1], ip[1] = v.x, ip[2] = v.y, ip[3] = v.z, ip[4] = v.w, ip[5] = pr[4];
      }
      float dp[M][6];
#pragma unroll
      for (int m = 0; m < M; m++) {
        const float *q = pr + (CI + m) * astride;
        float4 v = *reinterpret_cast<const float4 *>(q);
        dp[m][0] = q[-1], dp[m][1] = v.x, dp[m][2] = v.y, dp[m][3] = v.z, dp[m][4] = v.w, dp[m][5] = q[4];
      }
#pragma unroll
      for (int d2 = -1; d2 <= 1; d2++) {
        const int n = CROSS == 2 ? (d1 + 1) * 3 + (d2 + 1) : d2 + 1;
#pragma unroll
        for (int i = 0; i < 4; i++) {
          float l1 = 0.0f;
          if (USE_IMG) {
            if (ONECH) {
              l1 = fabsf(__fsub_rn(ic[i], ip[i + 1 + d2]));
            } else {
              for (int c = 0; c < C; c++)
                l1 = __fadd_rn(l1, fabsf(__fsub_rn(cur[c * astride + cb + i], pr[c * astride + i + d2])));
            }
          }
#pragma unroll
          for (int m = 0; m < M; m++) {
            float cand;
            if (MODE == MODE_GENERAL)
              cand = __fadd_rn(__fadd_rn(dp[m][i + 1 + d2], a.e[m][n]), __fmul_rn(a.lg[m], l1));
            else if (MODE == MODE_EUCLID)
              cand = __fadd_rn(dp[m][i + 1 + d2], a.e[m][n]);
            else
              cand = __fadd_rn(dp[m][i + 1 + d2], l1);
            best[m][i] = fminf(best[m][i], cand);
          }
        }
      }
    }
#pragma unroll
    for (int m = 0; m < M; m++) {
      float *o = const_cast<float *>(cur) + (CI + m) * astride + cb;
      float4 v;
      // cells outside the image or the region keep their NaN
      v.x = (valid & 1u) ? best[m][0] : o[0];
      v.y = (valid & 2u) ? best[m][1] : o[1];
      v.z = (valid & 4u) ? best[m][2] : o[2];
      v.w = (valid & 8u) ? best[m][3] : o[3];
      *reinterpret_cast<float4 *>(o) = v;
    }
  };

  // --- main loop over chunks: PD chunks of cp.async in flight ---
  const int nch = (L + S - 1) / S;
  for (int c = 0; c < PD; c++) {
    if (c < nch) load_chunk(c, c);
    cp_async_commit();
  }
  for (int n = 0; n < nch; n++) {
    const int q = n % NB, qp = (n + NB - 1) % NB;
    if (n + PD < nch) load_chunk(n + PD, (n + PD) % NB);
    cp_async_commit();
    if (n > 0 && has_nb) {
      wait_neighbours(a.flag_base + (unsigned)n);
      refresh(n * S - 1, qp, S - 1);
    }
    cp_async_wait(PD);
    __syncthreads();
    const int Sn = min(S, L - n * S);
    for (int j = (n == 0 ? 1 : 0); j < Sn; j++) {
      compute_step(buf(q, 0, j), j > 0 ? buf(q, 0, j - 1) : buf(qp, 0, S - 1));
      __syncthreads();
    }
    writeback(n, q);
    if (has_nb) {
      __syncthreads();
      if (tid == 0) {
        __threadfence();
        st_release(a.flags + tile, a.flag_base + (unsigned)n + 1u);
      }
    }
  }
}

// ---------------------------------------------------------------------------
// elementwise kernels: initial distances and signed / GSF combinations
// ---------------------------------------------------------------------------

enum InitOp { INIT_VM = 0, INIT_V1M = 1 };

// dst = v*src or v*(1-src) over n elements
__global__ void fg_init_kernel(float *dst, const float *src, long long n, float v, int op) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    float m = src[i];
    dst[i] = op == INIT_VM ? __fmul_rn(v, m) : __fmul_rn(v, __fsub_rn(1.0f, m));
  }
}

// Mask channels 1.. are never swept: every transform leaves them at v*mask.
// Writes the final value of the chosen operation for those elements.
__global__ void fg_unswept_kernel(float *out, const float *mask, long long n, float v, float theta, int op) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    float m = mask[i];
    float r;
    if (op == FG_OP_PLAIN) {
      r = __fmul_rn(v, m);
    } else {
      // signed(x) on an unswept channel: v*x - v*(1-x)
      float ds = __fsub_rn(__fmul_rn(v, m), __fmul_rn(v, __fsub_rn(1.0f, m)));
      if (op == FG_OP_SIGNED) {
        r = ds;
      } else {
        float md = ds > theta ? 1.0f : 0.0f, me = ds > -theta ? 1.0f : 0.0f;
        float am = __fsub_rn(1.0f, md);
        float s1 = __fsub_rn(__fmul_rn(v, am), __fmul_rn(v, __fsub_rn(1.0f, am)));
        float s2 = __fsub_rn(__fmul_rn(v, me), __fmul_rn(v, __fsub_rn(1.0f, me)));
        r = __fadd_rn(-s1, s2);
      }
    }
    out[i] = r;
  }
}

// out = a - b
__global__ void fg_sub_kernel(float *out, const float *x, const float *y, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    out[i] = __fsub_rn(x[i], y[i]);
}

// GSF stage two initial maps from Ds = d0 - d1 (FastGeodis/fastgeodis.cpp:321-327):
// Md = Ds > theta, Me = Ds > -theta;
// ma = v*(1-Md), mb = v*(1-(1-Md)), mc = v*Me, me = v*(1-Me)
__global__ void fg_gsf_mid_kernel(const float *d0, const float *d1, float *ma, float *mb, float *mc, float *me,
                                  long long n, float v, float theta) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    float ds = __fsub_rn(d0[i], d1[i]);
    float md = ds > theta ? 1.0f : 0.0f, mE = ds > -theta ? 1.0f : 0.0f;
    float am = __fsub_rn(1.0f, md);
    ma[i] = __fmul_rn(v, am);
    mb[i] = __fmul_rn(v, __fsub_rn(1.0f, am));
    mc[i] = __fmul_rn(v, mE);
    me[i] = __fmul_rn(v, __fsub_rn(1.0f, mE));
  }
}

// GSF result: -(A - B) + (C - E)   (FastGeodis/fastgeodis.cpp:326-329)
__global__ void fg_gsf_final_kernel(float *out, const float *da, const float *db, const float *dc, const float *de,
                                    long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    float s1 = __fsub_rn(da[i], db[i]);
    float s2 = __fsub_rn(dc[i], de[i]);
    out[i] = __fadd_rn(-s1, s2);
  }
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------

thread_local std::string g_err;

int fail(int code, const std::string &msg) {
  g_err = msg;
  return code;
}

#define FG_CUDA(call)                                                                         \
  do {                                                                                        \
    cudaError_t e_ = (call);                                                                  \
    if (e_ != cudaSuccess) return fail(FG_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)

struct DeviceInfo {
  int sms = 0;
  bool ok = false;
};

DeviceInfo device_info() {
  static std::mutex mu;
  static std::map<int, DeviceInfo> cache;
  int dev = 0;
  cudaGetDevice(&dev);
  std::lock_guard<std::mutex> g(mu);
  auto it = cache.find(dev);
  if (it != cache.end()) return it->second;
  DeviceInfo d;
  if (cudaDeviceGetAttribute(&d.sms, cudaDevAttrMultiProcessorCount, dev) == cudaSuccess) d.ok = true;
  cache[dev] = d;
  return d;
}

struct Plan {
  int T1, T2, K1, K2, tiles1, tiles2, S, B2, NCP, NB, NT;
  size_t smem;
};

size_t plan_smem(int cross, int A, int S, int NB, int T1, int T2, int K1, int K2, bool stepc, int *B2o, int *NCPo) {
  int R1 = cross == 2 ? T1 + 2 * K1 : 1, R2 = T2 + 2 * K2;
  int B1 = cross == 2 ? R1 + 2 : 1, B2 = ((R2 + 3) & ~3) + 8;  // 4-cell left apron, runs of 4, right apron
  int ncp = B1 * B2;
  if (stepc) {
    while (ncp % 32 != 4) ncp += 4;  // conflict-free transposing stage writes
  }
  *B2o = B2;
  *NCPo = ncp;
  return (size_t)NB * A * S * ncp * 4 + (size_t)2 * R1 * R2 * 8 + 64;
}

// Deepest ring (2 + up to 4 chunks in flight) that fits the shared-memory budget.
int pick_nb(int cross, int A, int S, int T1, int T2, int K1, int K2, bool stepc, size_t *smem, int *B2, int *NCP) {
  for (int nb = 6; nb >= 3; nb--) {
    size_t sm = plan_smem(cross, A, S, nb, T1, T2, K1, K2, stepc, B2, NCP);
    if (sm <= kSmemBudget) {
      *smem = sm;
      return nb;
    }
  }
  return 0;
}

std::atomic<int> g_tune_region{kMaxRegion};  // largest per-CTA region (cells) the planner may use
std::atomic<int> g_tune_tiles{0};            // cap on tiles per pass (0: the SM count)

// Cost model of one step of a pass, in SM cycles: the slower of the step's
// dependency chain and its issue time (about one cycle per 4-cell run at the
// observed issue rate), plus the per-chunk overhead and, when tiles exchange
// halos, the flag hand-off, both spread over the S steps of a chunk.
constexpr double kStepLatency = 150.0, kCyclesPerRun = 0.8, kChunkOverhead = 400.0, kHandoff = 2000.0;

double plan_cost(int runs, int S, bool multi, int nb) {
  double c = std::max(kStepLatency, kCyclesPerRun * runs) + kChunkOverhead / S + (multi ? kHandoff / S : 0.0);
  if (nb < 4) c += 300.0 / S;  // shallow prefetch exposes load latency
  return c;
}

// Choose tiles for a pass: the cheapest per-step plan such that all tiles are
// co-resident (one CTA per SM), the halo stays inside the neighbour tile and
// the ring fits in shared memory.
bool make_plan(int cross, int N1, int N2, int A, bool stepc, int max_tiles, Plan *out) {
  static std::mutex mu;
  static std::map<std::tuple<int, int, int, int, bool, int, int>, Plan> cache;
  const int max_region = g_tune_region.load();
  if (g_tune_tiles.load() > 0) max_tiles = std::min(max_tiles, g_tune_tiles.load());
  auto key = std::make_tuple(cross, N1, N2, A, stepc, max_tiles, max_region);
  {
    std::lock_guard<std::mutex> g(mu);
    auto it = cache.find(key);
    if (it != cache.end()) {
      *out = it->second;
      return true;
    }
  }
  bool found = false;
  Plan best{};
  double best_cost = 0.0;
  auto consider = [&](int S, int T1, int T2, int t1, int t2) {
    int K1 = (cross == 2 && t1 > 1) ? S : 0, K2 = t2 > 1 ? S : 0;
    if ((t1 > 1 && T1 < K1) || (t2 > 1 && T2 < K2)) return;
    int R1 = cross == 2 ? T1 + 2 * K1 : 1, R2 = T2 + 2 * K2;
    if ((long long)R1 * R2 > max_region) return;
    int runs = R1 * ((R2 + 3) / 4);
    if (runs > kThreads) return;
    int B2, NCP;
    size_t sm;
    int nb = pick_nb(cross, A, S, T1, T2, K1, K2, stepc, &sm, &B2, &NCP);
    if (nb == 0) return;
    double cost = plan_cost(runs, S, t1 * t2 > 1, nb);
    if (!found || cost < best_cost - 1e-9) {
      int nt = std::max(32, std::min(kThreads, (runs + 31) / 32 * 32));
      best = Plan{T1, T2, K1, K2, t1, t2, S, B2, NCP, nb, nt, sm};
      best_cost = cost;
      found = true;
    }
  };
  for (int S : {16, 8, 4, 2, 1}) {
    if (cross == 1) {
      for (int tiles2 = 1; tiles2 <= max_tiles; tiles2++) {
        int T2 = (N2 + tiles2 - 1) / tiles2;
        if (tiles2 > 1) T2 = (T2 + 3) & ~3;
        int t2 = (N2 + T2 - 1) / T2;
        if (t2 != tiles2 && tiles2 > 1) continue;
        consider(S, 1, T2, 1, t2);
        if (T2 <= 4) break;
      }
    } else {
      for (int T2 = std::min(N2, 4);; T2 = std::min(N2, T2 + 4)) {
        int t2 = (N2 + T2 - 1) / T2;
        for (int T1 = 1; T1 <= N1; T1++) {
          int t1 = (N1 + T1 - 1) / T1;
          if ((long long)t1 * t2 > max_tiles) continue;
          consider(S, T1, T2, t1, t2);
          break;  // larger T1 only grows the region
        }
        if (T2 >= N2) break;
      }
    }
  }
  if (found) {
    std::lock_guard<std::mutex> g(mu);
    cache[key] = best;
    *out = best;
    static const bool debug = getenv("FASTGEODIS_GB300_DEBUG_PLAN") != nullptr;
    if (debug)
      fprintf(stderr,
              "[fg plan] cross=%d N=%dx%d arrays=%d stepc=%d -> T=%dx%d K=%d,%d tiles=%dx%d S=%d NB=%d NT=%d smem=%zu "
              "cost=%.0f\n",
              cross, N1, N2, A, (int)stepc, best.T1, best.T2, best.K1, best.K2, best.tiles1, best.tiles2, best.S,
              best.NB, best.NT, best.smem, best_cost);
  }
  return found;
}

struct Workspace {
  int *status;
  unsigned *flags;
  float *maps;      // extra distance maps
  size_t map_stride;  // floats between maps
};

size_t map_bytes(long long P) { return ((size_t)P * 4 + 255) & ~(size_t)255; }

int extra_maps(int op) { return op == FG_OP_PLAIN ? 0 : (op == FG_OP_SIGNED ? 1 : 4); }

size_t workspace_bytes(int op, long long P) { return kWsHeader + kWsFlags + extra_maps(op) * map_bytes(P); }

int bind_workspace(void *ws, size_t bytes, int op, long long P, Workspace *w) {
  if (ws == nullptr) return fail(FG_ERR_WORKSPACE, "workspace pointer is null");
  if ((reinterpret_cast<uintptr_t>(ws) & 255) != 0) return fail(FG_ERR_WORKSPACE, "workspace must be 256-byte aligned");
  size_t need = workspace_bytes(op, P);
  if (bytes < need)
    return fail(FG_ERR_WORKSPACE, "workspace too small: need " + std::to_string(need) + " bytes, got " + std::to_string(bytes));
  char *base = static_cast<char *>(ws);
  w->status = reinterpret_cast<int *>(base);
  w->flags = reinterpret_cast<unsigned *>(base + kWsHeader);
  w->maps = reinterpret_cast<float *>(base + kWsHeader + kWsFlags);
  w->map_stride = map_bytes(P) / 4;
  return FG_OK;
}

// Geometry of one transform: 2D (D == 1 and is3d false) or 3D.
struct Geometry {
  bool is3d;
  int C, D, H, W;
  long long P;  // voxels per channel
  float spacing_sq[3];
};

struct MapSet {
  int M;
  float *dist[kMaxMaps];
  float lg[kMaxMaps];
  float le[kMaxMaps];
};

// Optional timing of pass launches with CUDA events on the launching stream
// (fg_profile_begin / fg_profile_end).
struct ProfileState {
  std::mutex mu;
  bool on = false;
  std::vector<std::pair<cudaEvent_t, cudaEvent_t>> ev;
  std::vector<long long> vp;  // voxel-passes of each recorded launch
};
ProfileState &profile() {
  static ProfileState p;
  return p;
}

template <int CROSS, bool ONECH, int M, int MODE>
int launch_pass_t(const PassArgs &a, const Plan &p, cudaStream_t s) {
  auto fn = fg_pass_kernel<CROSS, ONECH, M, MODE>;
  static std::mutex mu;
  static unsigned long long configured = 0;  // bit per device
  int dev = 0;
  FG_CUDA(cudaGetDevice(&dev));
  {
    std::lock_guard<std::mutex> g(mu);
    if (dev < 64 && !(configured & (1ull << dev))) {
      FG_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmemBudget));
      configured |= 1ull << dev;
    }
  }
  int ntiles = p.tiles1 * p.tiles2;
  void *args[] = {const_cast<PassArgs *>(&a)};
  ProfileState &ps = profile();
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  {
    std::lock_guard<std::mutex> g(ps.mu);
    if (ps.on) {
      FG_CUDA(cudaEventCreate(&e0));
      FG_CUDA(cudaEventCreate(&e1));
      FG_CUDA(cudaEventRecord(e0, s));
    }
  }
  if (ntiles > 1) {
    FG_CUDA(cudaLaunchCooperativeKernel((const void *)fn, dim3(ntiles), dim3(p.NT), args, p.smem, s));
  } else {
    FG_CUDA(cudaLaunchKernel((const void *)fn, dim3(1), dim3(p.NT), args, p.smem, s));
  }
  if (e0) {
    FG_CUDA(cudaEventRecord(e1, s));
    std::lock_guard<std::mutex> g(ps.mu);
    ps.ev.emplace_back(e0, e1);
    ps.vp.push_back((long long)a.L * a.N1 * a.N2 * M);
  }
  return FG_OK;
}

template <int CROSS, int M>
int launch_pass_mode(const PassArgs &a, const Plan &p, int mode, cudaStream_t s) {
  const bool one = a.C == 1;
  if (mode == MODE_EUCLID) return launch_pass_t<CROSS, true, M, MODE_EUCLID>(a, p, s);  // image unused
  if (mode == MODE_GEO)
    return one ? launch_pass_t<CROSS, true, M, MODE_GEO>(a, p, s) : launch_pass_t<CROSS, false, M, MODE_GEO>(a, p, s);
  return one ? launch_pass_t<CROSS, true, M, MODE_GENERAL>(a, p, s)
             : launch_pass_t<CROSS, false, M, MODE_GENERAL>(a, p, s);
}

template <int CROSS>
int launch_pass_m(const PassArgs &a, const Plan &p, int mode, cudaStream_t s) {
  switch (a.M) {
    case 1: return launch_pass_mode<CROSS, 1>(a, p, mode, s);
    case 2: return launch_pass_mode<CROSS, 2>(a, p, mode, s);
    case 4: return launch_pass_mode<CROSS, 4>(a, p, mode, s);
  }
  return fail(FG_ERR_UNSUPPORTED, "map count must be 1, 2 or 4");
}

int launch_pass(const PassArgs &a, const Plan &p, int cross, int mode, cudaStream_t s) {
  if (cross == 2) return launch_pass_m<2>(a, p, mode, s);
  return launch_pass_m<1>(a, p, mode, s);
}

// The cheapest exact arithmetic for the weights of a launch (all maps share
// the mode): l_grad == 0 drops the image term, (l_eucl, l_grad) == (0, 1)
// drops the step-length term and the multiplication.
int select_mode(const MapSet &ms) {
  bool euclid = true, geo = true;
  for (int m = 0; m < ms.M; m++) {
    euclid = euclid && ms.lg[m] == 0.0f;
    geo = geo && ms.le[m] == 0.0f && ms.lg[m] == 1.0f;
  }
  return euclid ? MODE_EUCLID : (geo ? MODE_GEO : MODE_GENERAL);
}

// Axis description inside one transform.
struct Axis {
  int L;
  long long s_str;
  int N1, N2;
  long long st1, st2;
  bool stepc;
  float ld[9];  // step lengths indexed by this build's neighbour numbering
};

void axes_for(const Geometry &g, Axis *ax, int *nax) {
  if (!g.is3d) {
    const float r2 = (float)sqrt(2.0);  // fastgeodis_cpu.cpp:67
    float ld2[9] = {r2, 1.0f, r2, 0, 0, 0, 0, 0, 0};
    ax[0] = Axis{g.H, g.W, 1, g.W, 0, 1, false, {}};  // along H, cross-section a row
    ax[1] = Axis{g.W, 1, 1, g.H, 0, g.W, true, {}};   // along W, cross-section a column
    memcpy(ax[0].ld, ld2, sizeof ld2);
    memcpy(ax[1].ld, ld2, sizeof ld2);
    *nax = 2;
    return;
  }
  const float *s = g.spacing_sq;
  // reference step-length table (fastgeodis_cpu.cpp:220-231): sp permuted per axis,
  // index 3*i+j with i the offset along the reference's dim 3 and j along dim 4.
  auto table = [](float s0, float s1, float s2, float out[9]) {
    for (int i = 0; i < 3; i++)
      for (int j = 0; j < 3; j++) {
        float v = s0;
        v += (float)abs(i - 1) * s1;
        v += (float)abs(j - 1) * s2;
        out[i * 3 + j] = sqrtf(v);
      }
  };
  long long HW = (long long)g.H * g.W;
  float t[9];
  // along D: cross (h, w); reference dims (H, W) -> same numbering
  ax[0] = Axis{g.D, HW, g.H, g.W, g.W, 1, false, {}};
  table(s[0], s[1], s[2], ax[0].ld);
  // along H: cross (d, w); reference transposes to [H, D, W] -> same numbering
  ax[1] = Axis{g.H, g.W, g.D, g.W, HW, 1, false, {}};
  table(s[1], s[0], s[2], ax[1].ld);
  // along W: cross (d, h); reference transposes to [W, H, D]: its i runs over h
  // (this build's second cross index) and its j over d (the first)
  ax[2] = Axis{g.W, 1, g.D, g.H, HW, g.W, true, {}};
  table(s[2], s[1], s[0], t);
  for (int d1 = 0; d1 < 3; d1++)
    for (int d2 = 0; d2 < 3; d2++) ax[2].ld[d1 * 3 + d2] = t[d2 * 3 + d1];
  *nax = 3;
}

// Runs `iterations` of the full pass sequence on the maps in `ms`.
int run_transform(const Geometry &g, const float *img, const MapSet &ms, int iterations, Workspace &w,
                  unsigned *launch_counter, cudaStream_t s) {
  if (g.P == 0 || iterations <= 0) return FG_OK;
  DeviceInfo di = device_info();
  if (!di.ok) return fail(FG_ERR_CUDA, "cannot query the current CUDA device");
  Axis ax[3];
  int nax = 0;
  axes_for(g, ax, &nax);
  const int cross = g.is3d ? 2 : 1;
  const int mode = select_mode(ms);
  const int staged = (mode == MODE_EUCLID ? 0 : g.C) + ms.M;  // arrays staged per position
  Plan plans[3];
  for (int k = 0; k < nax; k++) {
    if (!make_plan(cross, ax[k].N1, ax[k].N2, staged, ax[k].stepc, std::min(di.sms, kMaxTiles), &plans[k]))
      return fail(FG_ERR_UNSUPPORTED, "cross-section " + std::to_string(ax[k].N1) + "x" + std::to_string(ax[k].N2) +
                                          " with " + std::to_string(g.C) + " channels exceeds the planner's limits");
  }
  for (int it = 0; it < iterations; it++) {
    for (int k = 0; k < nax; k++) {
      if (ax[k].L <= 1) continue;
      for (int dir : {1, -1}) {
        if (*launch_counter >= 0xFFFFu) {  // progress values would wrap: start a fresh flag epoch
          FG_CUDA(cudaMemsetAsync(w.flags, 0, kWsFlags, s));
          *launch_counter = 0;
        }
        PassArgs a{};
        a.img = img;
        a.img_cs = g.P;
        a.C = g.C;
        a.M = ms.M;
        for (int m = 0; m < ms.M; m++) {
          a.dist[m] = ms.dist[m];
          a.lg[m] = ms.lg[m];
          for (int n = 0; n < 9; n++) a.e[m][n] = ms.le[m] * ax[k].ld[n];
        }
        a.L = ax[k].L;
        a.s_str = ax[k].s_str;
        a.dir = dir;
        a.N1 = ax[k].N1;
        a.N2 = ax[k].N2;
        a.st1 = ax[k].st1;
        a.st2 = ax[k].st2;
        const Plan &p = plans[k];
        a.T1 = p.T1;
        a.T2 = p.T2;
        a.K1 = p.K1;
        a.K2 = p.K2;
        a.tiles1 = p.tiles1;
        a.tiles2 = p.tiles2;
        a.S = p.S;
        a.stepc = ax[k].stepc ? 1 : 0;
        a.B2 = p.B2;
        a.NCP = p.NCP;
        a.NB = p.NB;
        a.flags = w.flags;
        a.flag_base = (*launch_counter) << 16;
        a.status = w.status;
        (*launch_counter)++;
        int rc = launch_pass(a, p, cross, mode, s);
        if (rc != FG_OK) return rc;
      }
    }
  }
  return FG_OK;
}

dim3 ew_grid(long long n) {
  long long b = (n + 255) / 256;
  return dim3((unsigned)std::min<long long>(std::max<long long>(b, 1), 152 * 16));
}

int check_common(const float *image, int C, int D, int H, int W, const float *mask, int Cm, const float *out) {
  if (C < 1 || Cm < 1) return fail(FG_ERR_INVALID_ARGUMENT, "channel counts must be at least 1");
  if (D < 0 || H < 0 || W < 0) return fail(FG_ERR_INVALID_ARGUMENT, "negative extent");
  long long P = (long long)D * H * W;
  if (P > 0 && (!image || !mask || !out)) return fail(FG_ERR_INVALID_ARGUMENT, "null tensor pointer");
  if (P * std::max(C, Cm) >= (1LL << 31)) return fail(FG_ERR_UNSUPPORTED, "tensors of 2^31 or more elements are not supported");
  return FG_OK;
}

// Common driver for plain / signed / GSF in 2D and 3D.
int run_op(int op, const Geometry &g, const float *image, const float *mask, int Cm, float *out, float v, float lg,
           float le, float theta, int iterations, void *ws, size_t ws_bytes, void *stream) {
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  int rc = check_common(image, g.C, g.D, g.H, g.W, mask, Cm, out);
  if (rc != FG_OK) return rc;
  if (g.P == 0) return FG_OK;
  Workspace w;
  rc = bind_workspace(ws, ws_bytes, op, g.P, &w);
  if (rc != FG_OK) return rc;
  FG_CUDA(cudaMemsetAsync(w.flags, 0, kWsFlags, s));
  unsigned counter = 0;
  const long long P = g.P;
  // unswept mask channels
  if (Cm > 1) {
    long long n = (long long)(Cm - 1) * P;
    fg_unswept_kernel<<<ew_grid(n), 256, 0, s>>>(out + P, mask + P, n, v, theta, op);
    FG_CUDA(cudaGetLastError());
  }
  if (op == FG_OP_PLAIN) {
    fg_init_kernel<<<ew_grid(P), 256, 0, s>>>(out, mask, P, v, INIT_VM);
    FG_CUDA(cudaGetLastError());
    MapSet ms{1, {out}, {lg}, {le}};
    return run_transform(g, image, ms, iterations, w, &counter, s);
  }
  float *m1 = w.maps;
  if (op == FG_OP_SIGNED) {
    fg_init_kernel<<<ew_grid(P), 256, 0, s>>>(out, mask, P, v, INIT_VM);
    fg_init_kernel<<<ew_grid(P), 256, 0, s>>>(m1, mask, P, v, INIT_V1M);
    FG_CUDA(cudaGetLastError());
    MapSet ms{2, {out, m1}, {lg, lg}, {le, le}};
    rc = run_transform(g, image, ms, iterations, w, &counter, s);
    if (rc != FG_OK) return rc;
    fg_sub_kernel<<<ew_grid(P), 256, 0, s>>>(out, out, m1, P);
    FG_CUDA(cudaGetLastError());
    return FG_OK;
  }
  // GSF: stage one is signed(mask) into (m0, m1); stage two sweeps four maps.
  float *m0 = w.maps, *mB = w.maps + w.map_stride, *mC = w.maps + 2 * w.map_stride, *mE = w.maps + 3 * w.map_stride;
  float *mA = out;
  fg_init_kernel<<<ew_grid(P), 256, 0, s>>>(m0, mask, P, v, INIT_VM);
  fg_init_kernel<<<ew_grid(P), 256, 0, s>>>(mB, mask, P, v, INIT_V1M);
  FG_CUDA(cudaGetLastError());
  {
    MapSet ms{2, {m0, mB}, {lg, lg}, {le, le}};
    rc = run_transform(g, image, ms, iterations, w, &counter, s);
    if (rc != FG_OK) return rc;
  }
  // Ds = m0 - mB; Md/Me thresholds; four initial maps (m0 is free afterwards, reuse it for C)
  fg_gsf_mid_kernel<<<ew_grid(P), 256, 0, s>>>(m0, mB, mA, mB, mC, mE, P, v, theta);
  FG_CUDA(cudaGetLastError());
  {
    MapSet ms{4, {mA, mB, mC, mE}, {lg, lg, lg, lg}, {le, le, le, le}};
    rc = run_transform(g, image, ms, iterations, w, &counter, s);
    if (rc != FG_OK) return rc;
  }
  fg_gsf_final_kernel<<<ew_grid(P), 256, 0, s>>>(out, mA, mB, mC, mE, P);
  FG_CUDA(cudaGetLastError());
  (void)m0;
  return FG_OK;
}

Geometry geom2d(int C, int H, int W) { return Geometry{false, C, 1, H, W, (long long)H * W, {1, 1, 1}}; }

int geom3d(int C, int D, int H, int W, const float *spacing, Geometry *g) {
  if (!spacing) return fail(FG_ERR_INVALID_ARGUMENT, "spacing pointer is null");
  *g = Geometry{true, C, D, H, W, (long long)D * H * W, {}};
  for (int i = 0; i < 3; i++) g->spacing_sq[i] = spacing[i] * spacing[i];  // fastgeodis_cuda.cu:602
  return FG_OK;
}

}  // namespace

extern "C" {

int fg_abi_version(void) { return FG_ABI_VERSION; }

const char *fg_last_error(void) { return g_err.c_str(); }

int fg_profile_begin(void) {
  ProfileState &ps = profile();
  std::lock_guard<std::mutex> g(ps.mu);
  for (auto &e : ps.ev) {
    cudaEventDestroy(e.first);
    cudaEventDestroy(e.second);
  }
  ps.ev.clear();
  ps.vp.clear();
  ps.on = true;
  return FG_OK;
}

int fg_profile_end(double *pass_ms, int *pass_launches, double *voxel_passes) {
  ProfileState &ps = profile();
  std::lock_guard<std::mutex> g(ps.mu);
  ps.on = false;
  double total = 0.0, vps = 0.0;
  int rc = FG_OK;
  for (size_t i = 0; i < ps.ev.size(); i++) {
    float ms = 0.0f;
    if (cudaEventSynchronize(ps.ev[i].second) != cudaSuccess ||
        cudaEventElapsedTime(&ms, ps.ev[i].first, ps.ev[i].second) != cudaSuccess)
      rc = fail(FG_ERR_CUDA, "event timing failed");
    total += ms;
    vps += (double)ps.vp[i];
    cudaEventDestroy(ps.ev[i].first);
    cudaEventDestroy(ps.ev[i].second);
  }
  if (pass_ms) *pass_ms = total;
  if (pass_launches) *pass_launches = (int)ps.ev.size();
  if (voxel_passes) *voxel_passes = vps;
  ps.ev.clear();
  ps.vp.clear();
  return rc;
}

int fg_set_tuning(int max_region_cells, int max_tiles) {
  if (max_region_cells < 0 || max_region_cells > kMaxRegion || max_tiles < 0 || max_tiles > kMaxTiles)
    return fail(FG_ERR_INVALID_ARGUMENT, "tuning values out of range");
  g_tune_region.store(max_region_cells == 0 ? kMaxRegion : max_region_cells);
  g_tune_tiles.store(max_tiles);
  return FG_OK;
}

size_t fg_workspace_bytes(int op, int C, int D, int H, int W) {
  (void)C;
  if (op < FG_OP_PLAIN || op > FG_OP_GSF || D < 0 || H < 0 || W < 0) return 0;
  return workspace_bytes(op, (long long)D * H * W);
}

int fg_workspace_status(void *workspace, void *stream) {
  if (!workspace) return fail(FG_ERR_WORKSPACE, "workspace pointer is null");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  int st = 0;
  FG_CUDA(cudaMemcpyAsync(&st, workspace, sizeof(int), cudaMemcpyDeviceToHost, s));
  FG_CUDA(cudaStreamSynchronize(s));
  if (st != 0) {
    FG_CUDA(cudaMemsetAsync(workspace, 0, sizeof(int), s));
    FG_CUDA(cudaStreamSynchronize(s));
    return fail(st, "a kernel reported error code " + std::to_string(st) + " (bounded wait expired)");
  }
  return FG_OK;
}

int fg_generalised_geodesic2d(const float *image, int C, int H, int W, const float *mask, int Cm, float *out, float v,
                              float l_grad, float l_eucl, int iterations, void *workspace, size_t workspace_bytes,
                              void *stream) {
  return run_op(FG_OP_PLAIN, geom2d(C, H, W), image, mask, Cm, out, v, l_grad, l_eucl, 0.0f, iterations, workspace,
                workspace_bytes, stream);
}

int fg_generalised_geodesic3d(const float *image, int C, int D, int H, int W, const float *mask, int Cm,
                              const float *spacing, float *out, float v, float l_grad, float l_eucl, int iterations,
                              void *workspace, size_t workspace_bytes, void *stream) {
  Geometry g;
  int rc = geom3d(C, D, H, W, spacing, &g);
  if (rc != FG_OK) return rc;
  return run_op(FG_OP_PLAIN, g, image, mask, Cm, out, v, l_grad, l_eucl, 0.0f, iterations, workspace, workspace_bytes,
                stream);
}

int fg_signed_generalised_geodesic2d(const float *image, int C, int H, int W, const float *mask, int Cm, float *out,
                                     float v, float l_grad, float l_eucl, int iterations, void *workspace,
                                     size_t workspace_bytes, void *stream) {
  return run_op(FG_OP_SIGNED, geom2d(C, H, W), image, mask, Cm, out, v, l_grad, l_eucl, 0.0f, iterations, workspace,
                workspace_bytes, stream);
}

int fg_signed_generalised_geodesic3d(const float *image, int C, int D, int H, int W, const float *mask, int Cm,
                                     const float *spacing, float *out, float v, float l_grad, float l_eucl,
                                     int iterations, void *workspace, size_t workspace_bytes, void *stream) {
  Geometry g;
  int rc = geom3d(C, D, H, W, spacing, &g);
  if (rc != FG_OK) return rc;
  return run_op(FG_OP_SIGNED, g, image, mask, Cm, out, v, l_grad, l_eucl, 0.0f, iterations, workspace,
                workspace_bytes, stream);
}

int fg_GSF2d(const float *image, int C, int H, int W, const float *mask, int Cm, float theta, float v, float lambda,
             int iterations, float *out, void *workspace, size_t workspace_bytes, void *stream) {
  const float le = 1.0f - lambda;  // float arithmetic, FastGeodis/fastgeodis.cpp:321
  return run_op(FG_OP_GSF, geom2d(C, H, W), image, mask, Cm, out, v, lambda, le, theta, iterations, workspace,
                workspace_bytes, stream);
}

int fg_GSF3d(const float *image, int C, int D, int H, int W, const float *mask, int Cm, float theta,
             const float *spacing, float v, float lambda, int iterations, float *out, void *workspace,
             size_t workspace_bytes, void *stream) {
  Geometry g;
  int rc = geom3d(C, D, H, W, spacing, &g);
  if (rc != FG_OK) return rc;
  const float le = 1.0f - lambda;
  return run_op(FG_OP_GSF, g, image, mask, Cm, out, v, lambda, le, theta, iterations, workspace, workspace_bytes,
                stream);
}

}  // extern "C"
