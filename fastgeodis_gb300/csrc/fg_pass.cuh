// The sweep kernel: one directional pass of the raster scan over one tile of
// the cross-section per CTA.
//
//   D[t][x] = min(D[t][x], min_n D[t-1][x+n] + l_eucl*ld[n] + l_grad*L1(I[t][x], I[t-1][x+n]))
//   (reference: FastGeodis/fastgeodis_cpu.cpp:53-162 and :203-340)
//
// Design:
//   * A CTA owns a tile of the cross-section plus a halo of K cells per side
//     and walks every step of the pass.  Each thread owns a run of 4
//     consecutive cells along the innermost cross dimension.
//   * A thread's own inputs of a step (old distance and image values) are
//     loaded straight into registers P steps ahead (16-byte loads where the
//     layout allows).  Shared memory only holds the rows its neighbours read:
//     the previous step's distances and image values.  One barrier per step.
//   * With several tiles, the halo lets a CTA run S <= K steps on its own.
//     At the last step of every chunk of S steps a CTA publishes its own
//     cells as 64-bit exchange words (value and chunk epoch in one atomic
//     access); at the start of the next chunk it replaces its halo cells of
//     that row by the words of its neighbours, re-polling (bounded) only words
//     that do not yet carry the wanted epoch.  One L2 round trip per hand-off,
//     no fences, no flags.  Halo cells are never written back.
//   * Cluster plans (volumes, CL = true): one thread-block cluster owns the
//     whole cross-section as strips of whole rows and the strips exchange
//     their boundary rows every step through distributed shared memory (see
//     pass_body); fg_cluster.cuh holds the cluster sweep kernel, which runs
//     the same plans with two runs per thread.
//   * Layout: the swept axis is never the contiguous one in the read layout.
//     The pass that hands over to a sweep along the contiguous axis writes
//     its result transposed (step innermost), through an S-row shared ring
//     flushed as S-element segments.
//   * Arithmetic: float32, every operation rounded on its own, in the
//     reference CPU order; fminf ignores NaN, so cells outside the image
//     (held as NaN) never contribute a candidate, as in the reference.
#pragma once

#include <map>
#include <mutex>
#include <tuple>

#include "fg_common.cuh"
#include "fg_wait.cuh"

namespace fgi {

__device__ __forceinline__ void st_word(unsigned long long *p, unsigned long long v) {
  asm volatile("st.relaxed.gpu.global.b64 [%0], %1;\n" ::"l"(p), "l"(v) : "memory");
}
// Global loads pinned where they are written (asm volatile), so that the
// prefetch of step t+P is issued at step t and not moved next to its use.
__device__ __forceinline__ float4 ldg4_pinned(const float *p) {
  float4 v;
  asm volatile("ld.global.v4.f32 {%0, %1, %2, %3}, [%4];\n" : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w) : "l"(p));
  return v;
}
__device__ __forceinline__ float4 ldg4_nc_pinned(const float *p) {
  float4 v;
  asm volatile("ld.global.nc.v4.f32 {%0, %1, %2, %3}, [%4];\n" : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w) : "l"(p));
  return v;
}
__device__ __forceinline__ float ldg_pinned(const float *p) {
  float v;
  asm volatile("ld.global.f32 %0, [%1];\n" : "=f"(v) : "l"(p));
  return v;
}
__device__ __forceinline__ float ldg_nc_pinned(const float *p) {
  float v;
  asm volatile("ld.global.nc.f32 %0, [%1];\n" : "=f"(v) : "l"(p));
  return v;
}

// --- thread-block cluster primitives (cluster plans) ---
__device__ __forceinline__ unsigned cl_rank() {
  unsigned r;
  asm volatile("mov.u32 %0, %%cluster_ctarank;\n" : "=r"(r));
  return r;
}
__device__ __forceinline__ unsigned smem_u32(const void *p) { return (unsigned)__cvta_generic_to_shared(p); }
// address of the same shared-memory offset in CTA `rank` of the cluster
__device__ __forceinline__ unsigned cl_map(unsigned a, unsigned rank) {
  unsigned r;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;\n" : "=r"(r) : "r"(a), "r"(rank));
  return r;
}
__device__ __forceinline__ void cl_sync() {
  asm volatile("barrier.cluster.arrive.release.aligned;\nbarrier.cluster.wait.acquire.aligned;\n" ::: "memory");
}
__device__ __forceinline__ void mbar_init(unsigned a, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(a), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_fence_init() { asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory"); }
__device__ __forceinline__ void mbar_inval(unsigned a) {
  asm volatile("mbarrier.inval.shared::cta.b64 [%0];\n" ::"r"(a) : "memory");
}
// one arrival that also expects `tx` bytes of asynchronous stores in this phase
__device__ __forceinline__ void mbar_expect(unsigned a, unsigned tx) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(a), "r"(tx) : "memory");
}
// stores into another CTA's shared memory that complete on its mbarrier `bar`
__device__ __forceinline__ void st_async4(unsigned a, const float4 &v, unsigned bar) {
  asm volatile("st.async.shared::cluster.mbarrier::complete_tx::bytes.v4.b32 [%0], {%1, %2, %3, %4}, [%5];\n" ::"r"(a),
               "r"(__float_as_uint(v.x)), "r"(__float_as_uint(v.y)), "r"(__float_as_uint(v.z)),
               "r"(__float_as_uint(v.w)), "r"(bar)
               : "memory");
}
__device__ __forceinline__ void st_async1(unsigned a, float v, unsigned bar) {
  asm volatile("st.async.shared::cluster.mbarrier::complete_tx::bytes.b32 [%0], %1, [%2];\n" ::"r"(a),
               "r"(__float_as_uint(v)), "r"(bar)
               : "memory");
}
constexpr unsigned kClusterSpinLimit = 1u << 16;  // failed mbarrier polls of one step before FG_ERR_TIMEOUT

__device__ __forceinline__ float f4get(const float4 &v, int i) {
  return i == 0 ? v.x : (i == 1 ? v.y : (i == 2 ? v.z : v.w));
}
__device__ __forceinline__ void f4set(float4 &v, int i, float x) {
  if (i == 0) v.x = x;
  else if (i == 1) v.y = x;
  else if (i == 2) v.z = x;
  else v.w = x;
}

// min of three (PTX min.f32 with three inputs, sm_100+): NaN inputs are
// ignored as by fminf, and the minimum of a set does not depend on the order
// it is taken in, so folding candidates three at a time gives fminf's bits.
__device__ __forceinline__ float fmin3(float a, float b, float c) {
  float r;
  asm("min.f32 %0, %1, %2, %3;\n" : "=f"(r) : "f"(a), "f"(b), "f"(c));
  return r;
}

// Cone of a chunk.  After a hand-off every cell of the last row is exact;
// at chunk step j (0 <= j < S) only cells whose distance to the region's
// halo boundary exceeds j are ever read again before the next hand-off (own
// cells are at distance >= K = S).  Distance of run q (4 cells along cross
// dimension 2), capped at S; -1 for a run outside the region.
__device__ __forceinline__ int run_cone_dist(int q, int rpr, int R1, int R2, int K1, int K2, int S) {
  const int r1 = q / rpr, u = q - r1 * rpr;
  if (r1 >= R1) return -1;
  const int d1 = K1 > 0 ? min(r1, R1 - 1 - r1) : S;
  int d = -1;
#pragma unroll
  for (int i = 0; i < 4; i++) {
    const int r2 = 4 * u + i;
    if (r2 < R2) d = max(d, min(d1, K2 > 0 ? min(r2, R2 - 1 - r2) : S));
  }
  return min(d, S);
}

// Stable counting sort of the CTA's threads by key (0 .. nkeys-1): returns
// this thread's position.  `scratch` holds nwarps * nkeys ints.  Ends with a
// barrier after its last shared-memory read.
__device__ __forceinline__ int cta_sort_position(int key, int nkeys, int *scratch) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  unsigned mine = 0;
  for (int b = 0; b < nkeys; b++) {
    const unsigned bal = __ballot_sync(0xffffffffu, key == b);
    if (key == b) mine = bal;
    if (lane == 0) scratch[warp * nkeys + b] = __popc(bal);
  }
  __syncthreads();
  int pos = __popc(mine & ((1u << lane) - 1u));
  for (int w = 0; w < nwarps; w++) {
    for (int b = 0; b < key; b++) pos += scratch[w * nkeys + b];
    if (w < warp) pos += scratch[w * nkeys + key];
  }
  __syncthreads();
  return pos;
}

// channels staged per step and the prefetch depth (steps) of a kernel variant;
// ct < 0 (kWideChannels): more than kMaxChannels channels, none staged
__host__ __device__ constexpr int pass_nch(int ct, int mode) {
  return mode == MODE_EUCLID || ct < 0 ? 0 : (ct == 0 ? kMaxChannels : ct);
}
__host__ __device__ constexpr int pass_depth(int nch, int m) { return (nch + m <= 4) ? 4 : 2; }

__device__ __forceinline__ void cp_async16(void *dst, const void *src) {
  unsigned d = (unsigned)__cvta_generic_to_shared(dst);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async4(void *dst, const void *src) {
  unsigned d = (unsigned)__cvta_generic_to_shared(dst);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

// The body of one pass over tile `tile`, shared by the per-pass kernel and the
// batched kernel.  `ar` may live in parameter or shared memory; it is copied
// into registers first so the step loop never reloads its fields.
// MULTI = false compiles a single-tile body (no halo exchange, no cone): the
// batched kernels, whose CTA always owns a whole image.
//
// CT: image channels staged through shared memory, 1 .. 4 (0: any count up
// to 4), or kWideChannels for images of more than 4 channels.  A wide pass
// stages no image values (its shared memory does not grow with the channel
// count, so every cross-section still tiles): at each step a thread reads its
// own cells' and the previous row's image values through L1 (the neighbour
// rows of consecutive steps overlap, so they hit) and sums the L1 distances
// of its 3 x 3 (2D: 3) candidates x 4 cells in registers, channel 0 first --
// the reference's summation order (fastgeodis_cpu.cpp:96-104,
// fastgeodis_cuda.cu:170-177).  Coordinates outside the image are clamped
// to it: such a neighbour's distance is NaN in the rings, so its candidate is
// NaN whatever its L1 sum, and the minimum ignores it, as with staged values.
// Tile plans only (no cluster plans, no batch or tape variants).
//
// CL = true: a cluster plan.  The CTAs of one thread-block cluster own strips
// of whole rows of the cross-section (tiles1 = cluster size, tiles2 = 1, no
// halo; `tile` is the CTA's rank).  After every step but the last, a strip's
// first and last rows (distances and image values, with their edge slots) go
// straight into the apron rows of the neighbour strips' rings with st.async,
// which completes on the receiver's mbarrier of that step's parity.  The
// receiver arms that mbarrier with the bytes it expects, and its apron
// readers wait on it before the next step.  A sender cannot run more than one
// step ahead of a receiver's reads (it needs the receiver's rows of the step
// before), so rings of two steps suffice and no hand-off goes through L2.
template <int CROSS, int CT, int M, int MODE, bool WT, bool TAPE = false, bool MULTI = true, bool CL = false>
__device__ __forceinline__ void pass_body(const PassArgs &ar, const int tile, float *sm) {
  const PassArgs a = ar;
  constexpr bool USE_IMG = MODE != MODE_EUCLID;
  constexpr bool WIDE = CT < 0 && USE_IMG;  // image read through L1, not staged
  static_assert(!(CT < 0 && (CL || TAPE || !MULTI)), "wide images run on tile plans only");
  constexpr int NCH = pass_nch(CT, MODE);
  constexpr int NCHR = NCH > 0 ? NCH : 1;
  const int P = a.P;                     // steps of own inputs in flight (power of 2)
  constexpr int A1 = CROSS == 2 ? 1 : 0; // apron row above the region
  constexpr int NR = CROSS == 2 ? 3 : 1; // stencil rows

  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int NT = blockDim.x, nwarps = NT >> 5;
  const int C = USE_IMG && !WIDE ? (CT == 0 ? a.C : CT) : 0;  // channels staged in shared memory
  const int CW = WIDE ? a.C : 0;                                // channels read through L1
  const int L = a.L, S = a.S, lgS = __ffs(S) - 1;  // S is a power of two
  const int tb = a.t_begin, te = a.t_end > 0 ? a.t_end : L;  // steps of this launch
  const int SR = WT ? S : 2;                        // distance rows kept in shared memory
  const int ti1 = tile / a.tiles2, ti2 = tile - ti1 * a.tiles2;
  const int R1 = CROSS == 2 ? a.T1 + 2 * a.K1 : 1, R2 = a.T2 + 2 * a.K2;
  const int B2 = a.B2, rowf = a.rowf;
  const int rs1 = CROSS == 2 ? ti1 * a.T1 - a.K1 : 0, rs2 = ti2 * a.T2 - a.K2;
  const int o1lo = CROSS == 2 ? a.K1 : 0;
  const int o1hi = CROSS == 2 ? a.K1 + min(a.T1, a.N1 - ti1 * a.T1) : 1;
  const int o2lo = a.K2, o2hi = a.K2 + min(a.T2, a.N2 - ti2 * a.T2);
  const float qnan = __int_as_float(0x7fffffff);

  const int rpr = (R2 + 3) >> 2;                               // runs per region row
  const int edgef = pass_edge_floats(CROSS, R1, R2);
  const int AR = M + C;                                        // arrays staged per step
  float *dring = sm;                                           // [SR][M][rowf] distances, last SR steps
  float *iring = dring + SR * M * rowf;                        // [2][C][rowf] image values, last 2 steps
  float *dedge = iring + 2 * C * rowf;                         // [SR][M][edgef] run edges of dring
  float *iedge = dedge + SR * M * edgef;                       // [2][C][edgef] run edges of iring
  float4 *oring = reinterpret_cast<float4 *>(iedge + 2 * C * edgef);  // [P][AR][NT] own inputs in flight
  int2 *otab = reinterpret_cast<int2 *>(oring + P * AR * NT);  // own cells (transposed flush)

  // --- set-up ---
  const bool has_nb = MULTI && !CL && a.tiles1 * a.tiles2 > 1;
  // run of this thread: with neighbours, runs ordered innermost first, so
  // the runs outside a step's cone are whole trailing warps
  int qrun = tid, cdist = S;
  if (has_nb) {
    int *scr = reinterpret_cast<int *>(sm);  // nwarps * (S + 2) counters, then NT positions
    int *perm = scr + nwarps * (S + 2);
    const int key = S - run_cone_dist(tid, rpr, R1, R2, a.K1, a.K2, S);  // 0 .. S + 1
    perm[cta_sort_position(key, S + 2, scr)] = tid;
    __syncthreads();
    qrun = perm[tid];
    cdist = run_cone_dist(qrun, rpr, R1, R2, a.K1, a.K2, S);
    __syncthreads();
  }
  for (int i = tid; i < (SR * M + 2 * C) * (rowf + edgef) + P * AR * NT * 4; i += NT) sm[i] = qnan;
  int nown = 0;
  if (WT) {
    const int O1 = o1hi - o1lo, O2 = o2hi - o2lo;
    nown = O1 * O2;
    for (int i = tid; i < nown; i += NT) {
      int o1 = o1lo + i / O2, o2 = o2lo + i % O2;
      long long g = (long long)(rs1 + o1) * a.wst1 + (long long)(rs2 + o2) * a.wst2;
      otab[i] = make_int2((o1 + A1) * B2 + 4 + o2, (int)g);
    }
  }
  const int r1 = qrun / rpr, u = qrun - (qrun / rpr) * rpr;
  const int g1 = rs1 + r1, g20 = rs2 + 4 * u;
  const int cb = (r1 + A1) * B2 + 4 + 4 * u;
  // this run's float2 in an edge array; it writes its first cell into the left
  // run's slot (e0 - 1) and its last into the right run's (e0 + 2)
  const int EP2 = (rpr + 2) * 2;  // floats per edge row
  const int e0 = (r1 + A1) * EP2 + (u + 1) * 2;
  constexpr bool EDGES = CROSS == 2;  // edge arrays (pass_edge_floats)
  auto put_edges = [&](float *edge, const float4 &v) {
    if (EDGES) {
      edge[e0 - 1] = v.x;
      edge[e0 + 2] = v.w;
    }
  };
  unsigned valid = 0, own = 0;
  if (r1 < R1) {
#pragma unroll
    for (int i = 0; i < 4; i++) {
      int r2 = 4 * u + i, g2 = g20 + i;
      bool in = r2 < R2 && g1 >= 0 && g1 < a.N1 && g2 >= 0 && g2 < a.N2;
      if (in) valid |= 1u << i;
      if (in && r1 >= o1lo && r1 < o1hi && r2 >= o2lo && r2 < o2hi) own |= 1u << i;
    }
  }
  const bool active = valid != 0;
  const bool full = valid == 0xFu && a.vec;
  const unsigned halo = valid & ~own;
  // exchange words of this thread's run (cell (g1, g20) of the cross-section), parity 0, map 0
  const long long xplane = (long long)a.N1 * a.N2;
  unsigned long long *const xrun = has_nb ? a.xch + (long long)g1 * a.N2 + g20 : nullptr;

  // cluster plan: two mbarriers after the own-cell table; every neighbour
  // strip sends its boundary row each step, 24 bytes per run and array
  unsigned cbar = 0, cl_bytes = 0, cl_sm[2] = {0, 0};
  bool cl_push[2] = {false, false}, cl_waits = false, cl_dead = false;
  if (CL) {
    const int rank = tile, nr = a.tiles1;
    cbar = smem_u32(otab + (WT ? R1 * R2 : 0));
    cl_bytes = (unsigned)(((rank > 0 ? 1 : 0) + (rank < nr - 1 ? 1 : 0)) * rpr * 24 * (M + C));
    cl_push[0] = active && r1 == 0 && rank > 0;           // first row -> the upper strip's lower apron
    cl_push[1] = active && r1 == R1 - 1 && rank < nr - 1; // last row -> the lower strip's upper apron
    if (cl_push[0]) cl_sm[0] = cl_map(smem_u32(sm), rank - 1);
    if (cl_push[1]) cl_sm[1] = cl_map(smem_u32(sm), rank + 1);
    cl_waits = tid == 0 || (active && (r1 == 0 || r1 == R1 - 1));  // apron readers, and the arming thread
    if (tid == 0) {
      mbar_init(cbar, 1);
      mbar_init(cbar + 8, 1);
      mbar_fence_init();
      if (L >= 2) mbar_expect(cbar, cl_bytes);      // step 0
      if (L >= 3) mbar_expect(cbar + 8, cl_bytes);  // step 1
    }
    cl_sync();  // rings filled and mbarriers armed in every CTA before the first push
  } else {
    __syncthreads();
  }

  // running offsets: read layout of the next step to prefetch, write layout of the current step
  const long long rstep = a.dir > 0 ? a.s_str : -a.s_str;
  const long long wstep = a.dir > 0 ? a.ws_str : -a.ws_str;
  const long long r0 = (a.dir > 0 ? 0 : (long long)(L - 1) * a.s_str) + (long long)g1 * a.st1 + g20;
  const long long w0 = (a.dir > 0 ? 0 : (long long)(L - 1) * a.ws_str) + (long long)g1 * a.wst1 + (long long)g20 * a.wst2;
  long long rnext = r0 + (long long)tb * rstep;  // read offset of the next step to stage
  long long rcur = rnext;                         // read offset of the current step
  long long wcur = w0 + (long long)tb * wstep;    // write offset of the current step

  // stage the own inputs of step `step` into ring slot `slot` (one commit group per step)
  // A run outside a step's cone still needs its image values at a chunk's
  // last step: the next chunk's first step reads the whole previous row of
  // the image (the exchange supplies only the distances).
  auto stage = [&](int slot, int step) {
    const int js = step & (S - 1);
    const bool sd = active && cdist > js;           // distances and image
    if (sd || (active && js == S - 1)) {            // image
      float4 *dst = oring + slot * AR * NT + tid;
      if (full) {
#pragma unroll
        for (int m = 0; m < M; m++)
          if (sd) cp_async16(dst + m * NT, a.dsrc[m] + rnext);
#pragma unroll
        for (int c = 0; c < NCH; c++)
          if (c < C) cp_async16(dst + (M + c) * NT, a.img + c * a.img_cs + rnext);
      } else {
#pragma unroll
        for (int i = 0; i < 4; i++) {
          if (valid & (1u << i)) {
#pragma unroll
            for (int m = 0; m < M; m++)
              if (sd) cp_async4(reinterpret_cast<float *>(dst + m * NT) + i, a.dsrc[m] + rnext + i);
#pragma unroll
            for (int c = 0; c < NCH; c++)
              if (c < C) cp_async4(reinterpret_cast<float *>(dst + (M + c) * NT) + i, a.img + c * a.img_cs + rnext + i);
          }
        }
      }
    }
    cp_async_commit();
    rnext += rstep;
  };

  for (int k = 0; k < P; k++) {
    if (tb + k < te) stage((tb + k) & (P - 1), tb + k);
    else cp_async_commit();
  }

  for (int t = tb; t < te; t++) {
    const int slot = t & (P - 1);
    if (CL && t > 0 && cl_waits) {
      // the neighbour strips' rows of step t-1 have landed in the apron rows
      const unsigned bar = cbar + ((t - 1) & 1) * 8, par = ((t - 1) >> 1) & 1;
      if (!cl_dead && !wait_phase(bar, par, a.status, kClusterSpinLimit))
        cl_dead = true;  // results are void; later steps no longer wait
      if (tid == 0 && !cl_dead && t + 1 <= L - 2) mbar_expect(bar, cl_bytes);  // the same parity's next step
    }
    // exact halo values of the previous row from the neighbour tiles; the
    // first step of a chunk launch takes the whole previous row (own cells
    // too) from the words the launch before published, and its image values
    if (has_nb && t > 0 && (t & (S - 1)) == 0) {
      const unsigned need = t == tb ? valid : halo;
      if (need) {
        const unsigned want = a.epoch_base + (unsigned)(t >> lgS);
        const unsigned long long *xw = xrun + (long long)((t >> lgS) & 1) * kMaxMaps * xplane;
        float *pr = dring + ((t - 1) & (SR - 1)) * M * rowf + cb;
        unsigned long long wd[M][4];
#pragma unroll
        for (int m = 0; m < M; m++)
#pragma unroll
          for (int i = 0; i < 4; i++)
            if (need & (1u << i)) wd[m][i] = ld_word(xw + m * xplane + i);  // all in flight at once
#pragma unroll
        for (int m = 0; m < M; m++)
#pragma unroll
          for (int i = 0; i < 4; i++)
            if (need & (1u << i)) {
              wd[m][i] = wait_word(xw + m * xplane + i, want, wd[m][i], a.status, kSpinLimit);
              const float hv = __uint_as_float((unsigned)wd[m][i]);
              pr[m * rowf + i] = hv;
              // a run's first and last cells also live in its neighbours' edge slots
              float *pe = dedge + ((t - 1) & (SR - 1)) * M * edgef + m * edgef;
              if (EDGES && i == 0) pe[e0 - 1] = hv;
              if (EDGES && i == 3) pe[e0 + 2] = hv;
            }
      }
      if (t == tb && NCH > 0 && active) {
        float *ic = iring + ((t - 1) & 1) * C * rowf + cb;
        float *ice = iedge + ((t - 1) & 1) * C * edgef;
#pragma unroll
        for (int c = 0; c < NCH; c++)
          if (c < C) {
            float4 v = make_float4(qnan, qnan, qnan, qnan);
#pragma unroll
            for (int i = 0; i < 4; i++)
              if (valid & (1u << i)) f4set(v, i, __ldg(a.img + c * a.img_cs + (rcur - rstep) + i));
            *reinterpret_cast<float4 *>(ic + c * rowf) = v;
            put_edges(ice + c * edgef, v);
          }
      }
      __syncthreads();
    }
    // this thread's inputs of step t have landed (P - 1 younger groups may still be in flight)
    if (P == 8) cp_async_wait<7>();
    else if (P == 4) cp_async_wait<3>();
    else cp_async_wait<1>();
    const int jstep = t & (S - 1);  // step within the chunk
    if (active && cdist > jstep) {  // in this step's cone
      const float4 *mine = oring + slot * AR * NT + tid;
      float4 dold[M], icur[NCHR];
#pragma unroll
      for (int m = 0; m < M; m++) dold[m] = mine[m * NT];
#pragma unroll
      for (int c = 0; c < NCH; c++)
        if (c < C) icur[c] = mine[(M + c) * NT];  // the ring holds M + C arrays
      float4 out[M];
      if (t == 0) {
#pragma unroll
        for (int m = 0; m < M; m++) out[m] = dold[m];
      } else {
        const float *dp0 = dring + ((t - 1) & (SR - 1)) * M * rowf;
        const float *ip0 = iring + ((t - 1) & 1) * C * rowf;
        const float *de0 = dedge + ((t - 1) & (SR - 1)) * M * edgef + e0;
        const float *ie0 = iedge + ((t - 1) & 1) * C * edgef + e0;
        // running minimum per map and cell, folded three values per min: the
        // old value and 9 candidates (3D) in 4 three-way mins and one two-way
        // min; an even-numbered candidate waits in pend for the next one
        float best[M][4], pend[M][4];
        unsigned code[4] = {kTapeSelf, kTapeSelf, kTapeSelf, kTapeSelf};  // TAPE: argmin of map 0
        // wide images: columns g20 - 1 .. g20 + 4 clamped to the image
        int colo[6];
        if (WIDE) {
#pragma unroll
          for (int j = 0; j < 6; j++) colo[j] = min(max(g20 - 1 + j, 0), a.N2 - 1) - g20;
        }
#pragma unroll
        for (int m = 0; m < M; m++)
#pragma unroll
          for (int i = 0; i < 4; i++) best[m][i] = f4get(dold[m], i);
#pragma unroll
        for (int r = 0; r < NR; r++) {
          const int d1 = CROSS == 2 ? r - 1 : 0;
          const int pc = cb + d1 * B2;
          float ip[NCHR][6];
#pragma unroll
          for (int c = 0; c < NCH; c++) {
            if (c < C) {
              const float *q = ip0 + c * rowf + pc;
              const float4 v = *reinterpret_cast<const float4 *>(q);
              const float2 ev = EDGES ? *reinterpret_cast<const float2 *>(ie0 + c * edgef + d1 * EP2)
                                      : make_float2(q[-1], q[4]);
              ip[c][0] = ev.x, ip[c][1] = v.x, ip[c][2] = v.y, ip[c][3] = v.z, ip[c][4] = v.w, ip[c][5] = ev.y;
            }
          }
          // wide images: this row's L1 sums (3 columns x 4 cells), channel by
          // channel in order, from the image in global memory
          float l1w[3][4];
          if (WIDE) {
            const int g = CROSS == 2 ? min(max(g1 + d1, 0), a.N1 - 1) : g1;  // previous step's row d1, clamped
            const long long ro = rcur - rstep + (long long)(g - g1) * a.st1;
#pragma unroll
            for (int j = 0; j < 3; j++)
#pragma unroll
              for (int i = 0; i < 4; i++) l1w[j][i] = 0.0f;
            for (int c = 0; c < CW; c++) {
              const float *ic = a.img + c * a.img_cs;
              float own[4], nb[6];
#pragma unroll
              for (int i = 0; i < 4; i++) own[i] = __ldg(ic + rcur + colo[i + 1]);
#pragma unroll
              for (int j = 0; j < 6; j++) nb[j] = __ldg(ic + ro + colo[j]);
#pragma unroll
              for (int j = 0; j < 3; j++)
#pragma unroll
                for (int i = 0; i < 4; i++) l1w[j][i] = __fadd_rn(l1w[j][i], fabsf(__fsub_rn(own[i], nb[i + j])));
            }
          }
          float dp[M][6];
#pragma unroll
          for (int m = 0; m < M; m++) {
            const float *q = dp0 + m * rowf + pc;
            const float4 v = *reinterpret_cast<const float4 *>(q);
            const float2 ev = EDGES ? *reinterpret_cast<const float2 *>(de0 + m * edgef + d1 * EP2)
                                    : make_float2(q[-1], q[4]);
            dp[m][0] = ev.x, dp[m][1] = v.x, dp[m][2] = v.y, dp[m][3] = v.z, dp[m][4] = v.w, dp[m][5] = ev.y;
          }
#pragma unroll
          for (int d2 = -1; d2 <= 1; d2++) {
            const int n = CROSS == 2 ? (d1 + 1) * 3 + (d2 + 1) : d2 + 1;
            const int k = r * 3 + (d2 + 1);  // candidate number 0 .. 3 * NR - 1
#pragma unroll
            for (int i = 0; i < 4; i++) {
              // one image channel: d = I(x) - I(y), the image term l_grad * |d|
              // as the reference forms it (any sign of l_grad)
              float d = 0.0f, l1 = 0.0f;
              if (WIDE) {
                l1 = l1w[d2 + 1][i];
              } else if (USE_IMG) {
                if (CT == 1) {
                  d = __fsub_rn(f4get(icur[0], i), ip[0][i + 1 + d2]);
                  l1 = fabsf(d);
                } else {
#pragma unroll
                  for (int c = 0; c < NCH; c++)
                    if (c < C) l1 = __fadd_rn(l1, fabsf(__fsub_rn(f4get(icur[c], i), ip[c][i + 1 + d2])));
                }
              }
#pragma unroll
              for (int m = 0; m < M; m++) {
                float cand;
                if (MODE == MODE_GENERAL && CT == 1)
                  cand = __fadd_rn(__fadd_rn(dp[m][i + 1 + d2], a.e[m][n]), __fmul_rn(a.lg[m], fabsf(d)));
                else if (MODE == MODE_GENERAL)
                  cand = __fadd_rn(__fadd_rn(dp[m][i + 1 + d2], a.e[m][n]), __fmul_rn(a.lg[m], l1));
                else if (MODE == MODE_EUCLID)
                  cand = __fadd_rn(dp[m][i + 1 + d2], a.e[m][n]);
                else
                  cand = __fadd_rn(dp[m][i + 1 + d2], l1);
                if (TAPE && m == 0) {
                  // same value as fminf for the non-NaN current distance of an in-image cell
                  if (cand < best[m][i]) best[m][i] = cand, code[i] = 1 + n;
                } else if (k == 3 * NR - 1) {
                  best[m][i] = fminf(best[m][i], cand);  // the last candidate
                } else if (k & 1) {
                  best[m][i] = fmin3(best[m][i], pend[m][i], cand);
                } else {
                  pend[m][i] = cand;  // waits for the next candidate
                }
              }
            }
          }
        }
        if (TAPE && own) {
          unsigned char *tp = a.tape + rcur;  // the tape has the read layout, one byte per cell
          if (own == 0xFu && a.vec) {
            *reinterpret_cast<unsigned *>(tp) = code[0] | (code[1] << 8) | (code[2] << 16) | (code[3] << 24);
          } else {
#pragma unroll
            for (int i = 0; i < 4; i++)
              if (own & (1u << i)) tp[i] = (unsigned char)code[i];
          }
        }
#pragma unroll
        for (int m = 0; m < M; m++) {
          // cells outside the image or the region stay NaN
          out[m].x = (valid & 1u) ? best[m][0] : qnan;
          out[m].y = (valid & 2u) ? best[m][1] : qnan;
          out[m].z = (valid & 4u) ? best[m][2] : qnan;
          out[m].w = (valid & 8u) ? best[m][3] : qnan;
        }
      }
      if (has_nb && own && ((t + 1) & (S - 1)) == 0 && t + 1 < L) {
        // last step of a chunk: publish the own cells for the neighbours' halos
        const unsigned long long ep = (unsigned long long)(a.epoch_base + (unsigned)((t + 1) >> lgS)) << 32;
        unsigned long long *xw = xrun + (long long)(((t + 1) >> lgS) & 1) * kMaxMaps * xplane;
#pragma unroll
        for (int m = 0; m < M; m++)
#pragma unroll
          for (int i = 0; i < 4; i++)
            if (own & (1u << i)) st_word(xw + m * xplane + i, ep | __float_as_uint(f4get(out[m], i)));
      }
      if (CL && t + 1 < L && (cl_push[0] || cl_push[1])) {
        // this strip's boundary row of step t into the neighbours' apron rows
        const unsigned bar = cbar + (t & 1) * 8;
#pragma unroll
        for (int side = 0; side < 2; side++) {
          if (!cl_push[side]) continue;
          const int row = side == 0 ? R1 + 1 : 0;  // the receiver's apron row
          const unsigned rsm = cl_sm[side], rbar = rsm + (bar - smem_u32(sm));
          const unsigned lsm = smem_u32(sm);
          const int pe = row * EP2 + (u + 1) * 2;
#pragma unroll
          for (int m = 0; m < M; m++) {
            const unsigned d = rsm + (smem_u32(dring + (t & (SR - 1)) * M * rowf + m * rowf + row * B2 + 4 + 4 * u) - lsm);
            const unsigned e = rsm + (smem_u32(dedge + (t & (SR - 1)) * M * edgef + m * edgef + pe) - lsm);
            st_async4(d, out[m], rbar);
            st_async1(e - 4, out[m].x, rbar);
            st_async1(e + 8, out[m].w, rbar);
          }
#pragma unroll
          for (int c = 0; c < NCH; c++)
            if (c < C) {
              const unsigned d = rsm + (smem_u32(iring + (t & 1) * C * rowf + c * rowf + row * B2 + 4 + 4 * u) - lsm);
              const unsigned e = rsm + (smem_u32(iedge + (t & 1) * C * edgef + c * edgef + pe) - lsm);
              st_async4(d, icur[c], rbar);
              st_async1(e - 4, icur[c].x, rbar);
              st_async1(e + 8, icur[c].w, rbar);
            }
        }
      }
      float *dc = dring + (t & (SR - 1)) * M * rowf + cb;
      float *dce = dedge + (t & (SR - 1)) * M * edgef;
#pragma unroll
      for (int m = 0; m < M; m++) {
        *reinterpret_cast<float4 *>(dc + m * rowf) = out[m];
        put_edges(dce + m * edgef, out[m]);
      }
      float *ic = iring + (t & 1) * C * rowf + cb;
      float *ice = iedge + (t & 1) * C * edgef;
#pragma unroll
      for (int c = 0; c < NCH; c++)
        if (c < C) {
          *reinterpret_cast<float4 *>(ic + c * rowf) = icur[c];
          put_edges(ice + c * edgef, icur[c]);
        }
      if (!WT && t > 0 && own) {
#pragma unroll
        for (int m = 0; m < M; m++) {
          if (own == 0xFu && a.vec) {
            *reinterpret_cast<float4 *>(a.ddst[m] + wcur) = out[m];
          } else {
#pragma unroll
            for (int i = 0; i < 4; i++)
              if (own & (1u << i)) a.ddst[m][wcur + i * a.wst2] = f4get(out[m], i);
          }
        }
      }
    } else if (active && jstep == S - 1) {
      // outside the cone at a chunk's last step: pass the image values on
      const float4 *mine = oring + slot * AR * NT + tid;
      float *ic = iring + (t & 1) * C * rowf + cb;
      float *ice = iedge + (t & 1) * C * edgef;
#pragma unroll
      for (int c = 0; c < NCH; c++)
        if (c < C) {
          const float4 v = mine[(M + c) * NT];
          *reinterpret_cast<float4 *>(ic + c * rowf) = v;
          put_edges(ice + c * edgef, v);
        }
    }
    // the slot's values are consumed (they are in registers): refill it with step t+P
    if (t + P < te) stage(slot, t + P);
    else cp_async_commit();
    wcur += wstep;
    rcur += rstep;
    __syncthreads();
    const bool chunk_end = ((t + 1) & (S - 1)) == 0 || t == L - 1;
    if (WT && chunk_end) {
      // transposed write-back of the chunk's own cells: S consecutive
      // positions of one cell are contiguous in the write layout
      const int t0 = t & ~(S - 1), Sn = t - t0 + 1;
      const int cpw = 32 / S, j = lane & (S - 1);
      if (j < Sn) {
        const long long so = (a.dir > 0 ? (long long)(t0 + j) : (long long)(L - 1 - t0 - j)) * a.ws_str;
        const float *src = dring + j * M * rowf;
#pragma unroll
        for (int m = 0; m < M; m++)
          for (int i = warp * cpw + (lane >> lgS); i < nown; i += nwarps * cpw) {
            int2 e = otab[i];
            a.ddst[m][so + e.y] = src[m * rowf + e.x];
          }
      }
      __syncthreads();
    }
  }
  cp_async_wait<0>();
  if (CL) cl_sync();  // no CTA leaves while a neighbour may still address its shared memory
}

// Register budget: 128 (CTAs up to 512 threads), or 64 for the lean kernel
// of a lean-capable variant (pass_lean: no spills at 64; CTAs up to 1024
// threads, or two CTAs of up to 512 threads per SM).
template <int CROSS, int CT, int M, int MODE, bool WT, bool LEAN>
__global__ void __maxnreg__((LEAN ? 64 : 128)) fg_pass_kernel(const PassArgs a) {
  extern __shared__ __align__(16) float sm[];
  pass_body<CROSS, CT, M, MODE, WT>(a, blockIdx.x, sm);
}

// The same pass on a cluster plan: one cluster of tiles1 CTAs, one strip each.
template <int CROSS, int CT, int M, int MODE, bool WT, bool LEAN>
__global__ void __maxnreg__((LEAN ? 64 : 128)) fg_pass_cluster_kernel(const PassArgs a) {
  extern __shared__ __align__(16) float sm[];
  pass_body<CROSS, CT, M, MODE, WT, false, true, true>(a, (int)cl_rank(), sm);
}

// Whether one cluster of this launch configuration can be co-scheduled on
// the device (cached per kernel, cluster size, CTA size and shared memory).
inline bool cluster_fits(const void *fn, const cudaLaunchConfig_t &cfg, int dev) {
  static std::mutex mu;
  static std::map<std::tuple<const void *, unsigned, unsigned, size_t, int>, bool> cache;
  const auto key = std::make_tuple(fn, cfg.gridDim.x, cfg.blockDim.x, cfg.dynamicSmemBytes, dev);
  std::lock_guard<std::mutex> g(mu);
  auto it = cache.find(key);
  if (it != cache.end()) return it->second;
  int n = 0;
  const cudaError_t e = cudaOccupancyMaxActiveClusters(&n, fn, &cfg);
  if (e != cudaSuccess) (void)cudaGetLastError();
  const bool ok = e == cudaSuccess && n > 0;
  cache[key] = ok;
  return ok;
}

// One cluster of c.tiles CTAs running `fn` (cudaLaunchKernelEx with a cluster
// dimension).  `configured`: per-device bits of the caller's kernel whose
// attributes are set (under the engine's launch lock).
inline int launch_one_cluster(const void *fn, unsigned long long &configured, const PassArgs &a, const LaunchCfg &c,
                              cudaStream_t s) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return set_error(FG_ERR_CUDA, cudaGetErrorString(e));
  if (dev < 64 && !(configured & (1ull << dev))) {
    e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(fn, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
    if (e != cudaSuccess) return set_error(FG_ERR_CUDA, cudaGetErrorString(e));
    configured |= 1ull << dev;
  }
  if (c.tiles < 2 || c.tiles > kMaxCluster) return set_error(FG_ERR_UNSUPPORTED, "a cluster plan has 2 to 16 CTAs");
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(c.tiles);
  cfg.blockDim = dim3(c.threads);
  cfg.dynamicSmemBytes = c.smem;
  cfg.stream = s;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = c.tiles;
  at[0].val.clusterDim.y = 1;
  at[0].val.clusterDim.z = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  if (!cluster_fits(fn, cfg, dev)) return set_error(FG_ERR_UNSUPPORTED, "the device cannot co-schedule this cluster plan");
  void *args[] = {const_cast<PassArgs *>(&a)};
  e = cudaLaunchKernelExC(&cfg, fn, args);
  if (e != cudaSuccess) return set_error(FG_ERR_CUDA, cudaGetErrorString(e));
  return FG_OK;
}

// Launch of one variant.  CLU: the cluster plan (one cluster of c.tiles CTAs);
// otherwise a cooperative launch of c.tiles CTAs, or an ordinary one for a
// chunk of a chunked plan.
template <int CROSS, int CT, int M, int MODE, bool WT, bool LEAN, bool CLU>
int launch_variant(const PassArgs &a, const LaunchCfg &c, cudaStream_t s) {
  void (*fn)(const PassArgs);
  if constexpr (CLU) fn = fg_pass_cluster_kernel<CROSS, CT, M, MODE, WT, LEAN>;
  else fn = fg_pass_kernel<CROSS, CT, M, MODE, WT, LEAN>;
  static unsigned long long configured = 0;  // bit per device (set under the engine's launch lock)
  if constexpr (CLU) return launch_one_cluster((const void *)fn, configured, a, c, s);
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return set_error(FG_ERR_CUDA, cudaGetErrorString(e));
  if (dev < 64 && !(configured & (1ull << dev))) {
    e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024);
    if (e != cudaSuccess) return set_error(FG_ERR_CUDA, cudaGetErrorString(e));
    configured |= 1ull << dev;
  }
  void *args[] = {const_cast<PassArgs *>(&a)};
  if (c.tiles > 1 && !c.chunked)
    e = cudaLaunchCooperativeKernel((const void *)fn, dim3(c.tiles), dim3(c.threads), args, c.smem, s);
  else  // one tile, or a chunk launch (its CTAs never wait on one another)
    e = cudaLaunchKernel((const void *)fn, dim3(c.tiles), dim3(c.threads), args, c.smem, s);
  if (e != cudaSuccess) return set_error(FG_ERR_CUDA, cudaGetErrorString(e));
  return FG_OK;
}

template <int CROSS, int CT, int M, int MODE, bool WT, bool CLU>
int launch_regs(const PassArgs &a, const LaunchCfg &c, cudaStream_t s) {
  if constexpr (pass_lean(CROSS, CT <= 0 ? kMaxChannels : CT, M)) {  // CT = 0: up to 4 channels; < 0: more
    if (c.lean) return launch_variant<CROSS, CT, M, MODE, WT, true, CLU>(a, c, s);
  }
  if (c.threads > kThreads) return set_error(FG_ERR_UNSUPPORTED, "a 128-register sweep CTA has at most 512 threads");
  return launch_variant<CROSS, CT, M, MODE, WT, false, CLU>(a, c, s);
}

template <int CROSS, int M, bool WT, bool CLU>
int launch_mode(const PassArgs &a, const LaunchCfg &c, int mode, cudaStream_t s) {
  const bool one = a.C == 1;
  if (mode == MODE_EUCLID) return launch_regs<CROSS, 1, M, MODE_EUCLID, WT, CLU>(a, c, s);
  if (a.C > kMaxChannels) {
    if constexpr (CLU) {
      return set_error(FG_ERR_UNSUPPORTED, "images with more than 4 channels run on tile plans");
    } else {
      return mode == MODE_GEO ? launch_regs<CROSS, kWideChannels, M, MODE_GEO, WT, false>(a, c, s)
                              : launch_regs<CROSS, kWideChannels, M, MODE_GENERAL, WT, false>(a, c, s);
    }
  }
  if (mode == MODE_GEO)
    return one ? launch_regs<CROSS, 1, M, MODE_GEO, WT, CLU>(a, c, s) : launch_regs<CROSS, 0, M, MODE_GEO, WT, CLU>(a, c, s);
  return one ? launch_regs<CROSS, 1, M, MODE_GENERAL, WT, CLU>(a, c, s)
             : launch_regs<CROSS, 0, M, MODE_GENERAL, WT, CLU>(a, c, s);
}

template <int CROSS, bool CLU = false>
int launch_cross(const PassArgs &a, const LaunchCfg &c, int M, int mode, bool wt, cudaStream_t s) {
  if constexpr (CLU) {
    // a cluster plan changes layout as an in-place pass and a transpose (the engine's pass generator)
    if (wt) return set_error(FG_ERR_UNSUPPORTED, "cluster plans do not write transposed");
    if (M == 1) return launch_mode<CROSS, 1, false, CLU>(a, c, mode, s);
    if (M == 2) return launch_mode<CROSS, 2, false, CLU>(a, c, mode, s);
    return set_error(FG_ERR_UNSUPPORTED, "a pass updates one or two distance maps");
  }
  if (M == 1)
    return wt ? launch_mode<CROSS, 1, true, CLU>(a, c, mode, s) : launch_mode<CROSS, 1, false, CLU>(a, c, mode, s);
  if (M == 2)
    return wt ? launch_mode<CROSS, 2, true, CLU>(a, c, mode, s) : launch_mode<CROSS, 2, false, CLU>(a, c, mode, s);
  return set_error(FG_ERR_UNSUPPORTED, "a pass updates one or two distance maps");
}

}  // namespace fgi
