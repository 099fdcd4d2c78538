// The cluster sweep kernel: one directional pass of a volume sweep on a
// cluster plan, with RPT runs of 4 cells per thread.
//
//   D[t][x] = min(D[t][x], min_n D[t-1][x+n] + l_eucl*ld[n] + l_grad*L1(I[t][x], I[t-1][x+n]))
//   (reference: FastGeodis/fastgeodis_cpu.cpp:203-340)
//
// Design:
//   * One thread-block cluster of G <= 16 CTAs owns the whole cross-section;
//     CTA `rank` owns the strip of T1 whole rows starting at rank * T1 (T1 a
//     multiple of RPT).  No halo, no hand-off through global memory.
//   * A thread owns the same 4-cell run u of RPT (2) consecutive rows.  The
//     previous step's rows it reads (rows rf-1 .. rf+RPT of the shared ring)
//     pass through a sliding window of three rows, so RPT runs load RPT + 2
//     rows instead of 3 * RPT, and the per-step overhead (waits, staging,
//     barrier, offsets) is paid once per RPT runs.  With at most 512 threads
//     per CTA every variant keeps its state in registers (128 per thread).
//   * After every step but the last, a strip's first and last rows (distances
//     and image values, with their edge slots) go straight into the apron
//     rows of the neighbour strips' rings with st.async, completing on the
//     receiver's mbarrier of that step's parity; the receiver arms it with the
//     bytes it expects, and only the threads whose window reads an apron row
//     wait on it.  A sender cannot be more than one step ahead of a
//     receiver's reads (it needs the receiver's rows of the step before), so
//     rings of two steps suffice.
//   * Own inputs (old distances, image values) are staged P steps ahead with
//     per-thread cp.async; results are written in place (a pass that changes
//     layout is followed by a transpose of the map); the arithmetic is the
//     pass kernel's, operation by operation.
#pragma once

#include "fg_pass.cuh"

namespace fgi {

template <int CT, int M, int MODE, int RPT>
__device__ __forceinline__ void cluster_body(const PassArgs &a, float *sm) {
  constexpr bool USE_IMG = MODE != MODE_EUCLID;
  constexpr int NCH = pass_nch(CT, MODE);
  constexpr int NCHR = NCH > 0 ? NCH : 1;
  const int tid = threadIdx.x, NT = blockDim.x;
  const int C = USE_IMG ? (CT == 0 ? a.C : CT) : 0;
  const int P = a.P, L = a.L;  // P: a power of two
  constexpr int SR = 2;        // distance rows kept per map
  const int rank = (int)cl_rank(), G = a.tiles1;
  const int T1 = a.T1, N2 = a.N2;
  const ClusterLayout ly = cluster_layout(C, M, T1, N2, NT, RPT, P);
  const int rpr = ly.rpr, B2 = ly.B2, rowf = ly.rowf, edgef = ly.edgef, EP2 = (rpr + 2) * 2;
  float *const dring = sm + ly.dring;
  float *const iring = sm + ly.iring;
  float *const dedge = sm + ly.dedge;
  float *const iedge = sm + ly.iedge;
  float4 *const oring = reinterpret_cast<float4 *>(sm + ly.oring);  // [P][M + C][RPT][NT]
  const unsigned lsm = smem_u32(sm), cbar = lsm + ly.bar;
  const int row0 = rank * T1, nrows = max(0, min(T1, a.N1 - row0));
  const int AR = M + C, NTR = NT * RPT;
  const float qnan = __int_as_float(0x7fffffff);

  // this thread: run u (cells 4u .. 4u+3) of strip rows rf .. rf + RPT - 1
  const int u = tid % rpr, rb = tid / rpr, rf = rb * RPT;
  unsigned vmask = 0;  // bit 4k + i: cell i of run k is in the image
#pragma unroll
  for (int k = 0; k < RPT; k++)
#pragma unroll
    for (int i = 0; i < 4; i++)
      if (rf + k < nrows && 4 * u + i < N2) vmask |= 1u << (4 * k + i);
  const bool active = vmask != 0;
  const bool vec = a.vec != 0;

  // --- set-up: rings NaN (cells outside the image never win a min) ---
  for (int i = tid; i < ly.bar / 4; i += NT) sm[i] = qnan;
  // neighbour strips: bytes this CTA receives per step, and where this thread sends
  const unsigned cl_bytes = (unsigned)(((rank > 0 ? 1 : 0) + (rank < G - 1 ? 1 : 0)) * rpr * 24 * AR);
  const int k_dn = T1 - 1 - rf;  // the run of this thread on the strip's last row, if any
  const bool push_up = active && rf == 0 && rank > 0;
  const bool push_dn = rank < G - 1 && k_dn >= 0 && k_dn < RPT && ((vmask >> (4 * k_dn)) & 0xFu) != 0;
  const unsigned rsm_up = push_up ? cl_map(lsm, rank - 1) : 0u;
  const unsigned rsm_dn = push_dn ? cl_map(lsm, rank + 1) : 0u;
  // a strip with no neighbour (one strip) never waits: its mbarriers stay unused
  const bool waits = G > 1 && (tid == 0 || (active && (rf == 0 || rf + RPT >= T1)));  // the window reads an apron row
  bool dead = false;
  if (tid == 0) {
    mbar_init(cbar, 1);
    mbar_init(cbar + 8, 1);
    mbar_fence_init();
    if (G > 1 && L >= 2) mbar_expect(cbar, cl_bytes);      // step 0
    if (G > 1 && L >= 3) mbar_expect(cbar + 8, cl_bytes);  // step 1
  }
  cl_sync();  // rings filled and mbarriers armed in every CTA before the first push

  // offsets (elements) of run 0 of this thread; run k adds k rows
  const int kst = (int)a.st1, kwst = (int)a.wst1;
  const int rstep = a.dir > 0 ? (int)a.s_str : -(int)a.s_str;
  const int wstep = a.dir > 0 ? (int)a.ws_str : -(int)a.ws_str;
  const int gr = row0 + rf;
  int rnext = (a.dir > 0 ? 0 : (L - 1) * (int)a.s_str) + gr * kst + 4 * u;  // next step to stage
  int wcur = (a.dir > 0 ? 0 : (L - 1) * (int)a.ws_str) + gr * kwst + 4 * u * (int)a.wst2;

  auto stage = [&](int slot) {
    if (active) {
      float4 *dst = oring + slot * AR * NTR + tid;
#pragma unroll
      for (int k = 0; k < RPT; k++) {
        const unsigned vk = (vmask >> (4 * k)) & 0xFu;
        const int o = rnext + k * kst;
        if (vk == 0xFu && vec) {
#pragma unroll
          for (int m = 0; m < M; m++) cp_async16(dst + (m * RPT + k) * NT, a.dsrc[m] + o);
#pragma unroll
          for (int c = 0; c < NCH; c++)
            if (c < C) cp_async16(dst + ((M + c) * RPT + k) * NT, a.img + c * a.img_cs + o);
        } else if (vk) {
#pragma unroll
          for (int i = 0; i < 4; i++)
            if (vk & (1u << i)) {
#pragma unroll
              for (int m = 0; m < M; m++)
                cp_async4(reinterpret_cast<float *>(dst + (m * RPT + k) * NT) + i, a.dsrc[m] + o + i);
#pragma unroll
              for (int c = 0; c < NCH; c++)
                if (c < C)
                  cp_async4(reinterpret_cast<float *>(dst + ((M + c) * RPT + k) * NT) + i,
                            a.img + c * a.img_cs + o + i);
            }
        }
      }
    }
    cp_async_commit();
    rnext += rstep;
  };
  for (int k = 0; k < P; k++) {
    if (k < L) stage(k);
    else cp_async_commit();
  }

  // one run's row of step t into a neighbour strip's apron row `srow` (st.async)
  auto push = [&](unsigned rsm, int srow, int t, const float4 *out, const float4 *ic) {
    const unsigned bar = rsm + (cbar - lsm) + (t & 1) * 8;
    const int pc = srow * B2 + 4 + 4 * u, pe = srow * EP2 + (u + 1) * 2;
    const int ds = ly.dring + (t & (SR - 1)) * M * rowf, des = ly.dedge + (t & (SR - 1)) * M * edgef;
    const int is = ly.iring + (t & 1) * C * rowf, ies = ly.iedge + (t & 1) * C * edgef;
#pragma unroll
    for (int m = 0; m < M; m++) {
      st_async4(rsm + 4u * (unsigned)(ds + m * rowf + pc), out[m], bar);
      st_async1(rsm + 4u * (unsigned)(des + m * edgef + pe - 1), out[m].x, bar);
      st_async1(rsm + 4u * (unsigned)(des + m * edgef + pe + 2), out[m].w, bar);
    }
#pragma unroll
    for (int c = 0; c < NCH; c++)
      if (c < C) {
        st_async4(rsm + 4u * (unsigned)(is + c * rowf + pc), ic[c], bar);
        st_async1(rsm + 4u * (unsigned)(ies + c * edgef + pe - 1), ic[c].x, bar);
        st_async1(rsm + 4u * (unsigned)(ies + c * edgef + pe + 2), ic[c].w, bar);
      }
  };

  for (int t = 0; t < L; t++) {
    const int slot = t & (P - 1);
    if (t > 0 && waits && !dead) {
      // the neighbour strips' rows of step t-1 have landed in the apron rows
      const unsigned bar = cbar + ((t - 1) & 1) * 8, par = ((t - 1) >> 1) & 1;
      if (!wait_phase(bar, par, a.status, kClusterSpinLimit)) dead = true;  // results are void; later steps no longer wait
      if (tid == 0 && !dead && t + 1 <= L - 2) mbar_expect(bar, cl_bytes);  // the same parity's next step
    }
    // this thread's inputs of step t have landed (P - 1 younger groups may still be in flight)
    if (P == 8) cp_async_wait<7>();
    else if (P == 4) cp_async_wait<3>();
    else cp_async_wait<1>();
    if (active) {
      const float4 *mine = oring + slot * AR * NTR + tid;
      float *const dc = dring + (t & (SR - 1)) * M * rowf;
      float *const dce = dedge + (t & (SR - 1)) * M * edgef;
      float *const ic0 = iring + (t & 1) * C * rowf;
      float *const ice = iedge + (t & 1) * C * edgef;
      const float *const dp0 = dring + ((t - 1) & (SR - 1)) * M * rowf;
      const float *const ip0 = iring + ((t - 1) & 1) * C * rowf;
      const float *const de0 = dedge + ((t - 1) & (SR - 1)) * M * edgef;
      const float *const ie0 = iedge + ((t - 1) & 1) * C * edgef;
      // window of the previous step's rows: slot (j % 3) holds strip row rf - 1 + j
      float wd[3][M][6], wi[3][NCHR][6];
      auto load_row = [&](int j, int lr) {  // lr: strip row -1 .. T1
        const int pc = (lr + 1) * B2 + 4 + 4 * u, pe = (lr + 1) * EP2 + (u + 1) * 2;
#pragma unroll
        for (int m = 0; m < M; m++) {
          const float4 v = *reinterpret_cast<const float4 *>(dp0 + m * rowf + pc);
          const float2 e = *reinterpret_cast<const float2 *>(de0 + m * edgef + pe);
          wd[j][m][0] = e.x, wd[j][m][1] = v.x, wd[j][m][2] = v.y, wd[j][m][3] = v.z, wd[j][m][4] = v.w,
          wd[j][m][5] = e.y;
        }
#pragma unroll
        for (int c = 0; c < NCH; c++)
          if (c < C) {
            const float4 v = *reinterpret_cast<const float4 *>(ip0 + c * rowf + pc);
            const float2 e = *reinterpret_cast<const float2 *>(ie0 + c * edgef + pe);
            wi[j][c][0] = e.x, wi[j][c][1] = v.x, wi[j][c][2] = v.y, wi[j][c][3] = v.z, wi[j][c][4] = v.w,
            wi[j][c][5] = e.y;
          }
      };
      if (t > 0) {
        load_row(0, rf - 1);
        load_row(1, rf);
      }
#pragma unroll
      for (int k = 0; k < RPT; k++) {
        const unsigned vk = (vmask >> (4 * k)) & 0xFu;
        if (vk == 0) break;  // rows past the image's end: so are the later runs
        if (t > 0) load_row((k + 2) % 3, rf + k + 1);
        float4 dold[M], ic[NCHR], out[M];
#pragma unroll
        for (int m = 0; m < M; m++) dold[m] = mine[(m * RPT + k) * NT];
#pragma unroll
        for (int c = 0; c < NCH; c++)
          if (c < C) ic[c] = mine[((M + c) * RPT + k) * NT];
        if (t == 0) {
#pragma unroll
          for (int m = 0; m < M; m++) out[m] = dold[m];
        } else {
          // running minimum per map and cell: the old value and 9 candidates
          // in four three-way mins and one two-way min
          float best[M][4], pend[M][4];
#pragma unroll
          for (int m = 0; m < M; m++)
#pragma unroll
            for (int i = 0; i < 4; i++) best[m][i] = f4get(dold[m], i);
#pragma unroll
          for (int r = 0; r < 3; r++) {
            const int j = (k + r) % 3;  // window slot of strip row rf + k + r - 1
#pragma unroll
            for (int d2 = -1; d2 <= 1; d2++) {
              const int n = r * 3 + (d2 + 1);  // neighbour number (d1 = r - 1)
#pragma unroll
              for (int i = 0; i < 4; i++) {
                // one image channel: d = I(x) - I(y), the image term l_grad * |d| as
                // the reference forms it (any sign of l_grad)
                float d = 0.0f, l1 = 0.0f;
                if (USE_IMG) {
                  if (CT == 1) {
                    d = __fsub_rn(f4get(ic[0], i), wi[j][0][i + 1 + d2]);
                    l1 = fabsf(d);
                  } else {
#pragma unroll
                    for (int c = 0; c < NCH; c++)
                      if (c < C) l1 = __fadd_rn(l1, fabsf(__fsub_rn(f4get(ic[c], i), wi[j][c][i + 1 + d2])));
                  }
                }
#pragma unroll
                for (int m = 0; m < M; m++) {
                  float cand;
                  if (MODE == MODE_GENERAL && CT == 1)
                    cand = __fadd_rn(__fadd_rn(wd[j][m][i + 1 + d2], a.e[m][n]), __fmul_rn(a.lg[m], fabsf(d)));
                  else if (MODE == MODE_GENERAL)
                    cand = __fadd_rn(__fadd_rn(wd[j][m][i + 1 + d2], a.e[m][n]), __fmul_rn(a.lg[m], l1));
                  else if (MODE == MODE_EUCLID)
                    cand = __fadd_rn(wd[j][m][i + 1 + d2], a.e[m][n]);
                  else
                    cand = __fadd_rn(wd[j][m][i + 1 + d2], l1);
                  if (n == 8) best[m][i] = fminf(best[m][i], cand);  // the last candidate
                  else if (n & 1) best[m][i] = fmin3(best[m][i], pend[m][i], cand);
                  else pend[m][i] = cand;                             // waits for the next candidate
                }
              }
            }
          }
#pragma unroll
          for (int m = 0; m < M; m++) out[m] = make_float4(best[m][0], best[m][1], best[m][2], best[m][3]);
          if (vk != 0xFu) {
#pragma unroll
            for (int m = 0; m < M; m++) {
              out[m].x = (vk & 1u) ? best[m][0] : qnan;  // cells outside the image stay NaN
              out[m].y = (vk & 2u) ? best[m][1] : qnan;
              out[m].z = (vk & 4u) ? best[m][2] : qnan;
              out[m].w = (vk & 8u) ? best[m][3] : qnan;
            }
          }
        }
        // this run's row of step t into the ring, then to the neighbour strips
        const int lr = rf + k;
        const int pc = (lr + 1) * B2 + 4 + 4 * u, pe = (lr + 1) * EP2 + (u + 1) * 2;
#pragma unroll
        for (int m = 0; m < M; m++) {
          *reinterpret_cast<float4 *>(dc + m * rowf + pc) = out[m];
          dce[m * edgef + pe - 1] = out[m].x;
          dce[m * edgef + pe + 2] = out[m].w;
        }
#pragma unroll
        for (int c = 0; c < NCH; c++)
          if (c < C) {
            *reinterpret_cast<float4 *>(ic0 + c * rowf + pc) = ic[c];
            ice[c * edgef + pe - 1] = ic[c].x;
            ice[c * edgef + pe + 2] = ic[c].w;
          }
        if (t + 1 < L) {
          if (k == 0 && push_up) push(rsm_up, T1 + 1, t, out, ic);  // the upper strip's lower apron
          if (k == k_dn && push_dn) push(rsm_dn, 0, t, out, ic);     // the lower strip's upper apron
        }
        if (t > 0) {
          const int w = wcur + k * kwst;
#pragma unroll
          for (int m = 0; m < M; m++) {
            if (vk == 0xFu && vec) {
              *reinterpret_cast<float4 *>(a.ddst[m] + w) = out[m];
            } else {
#pragma unroll
              for (int i = 0; i < 4; i++)
                if (vk & (1u << i)) a.ddst[m][w + i * (int)a.wst2] = f4get(out[m], i);
            }
          }
        }
      }
    }
    // the slot's values are consumed (they are in registers): refill it with step t+P
    if (t + P < L) stage(slot);
    else cp_async_commit();
    wcur += wstep;
    __syncthreads();
  }
  cp_async_wait<0>();
  cl_sync();  // no CTA leaves while a neighbour may still address its shared memory
  // the mbarriers' memory may serve other data next (a kernel running several
  // passes in turn): invalidate them first, as an mbarrier object requires
  if (tid == 0) {
    mbar_inval(cbar);
    mbar_inval(cbar + 8);
  }
}

template <int CT, int M, int MODE, int RPT>
__global__ void __launch_bounds__(512) fg_sweep_cluster_kernel(const PassArgs a) {
  extern __shared__ __align__(16) float sm[];
  cluster_body<CT, M, MODE, RPT>(a, sm);
}

}  // namespace fgi
