// The differentiable 2D transform: a forward that records, for every cell of
// every pass, which candidate won (the argmin tape), and the adjoint that walks
// the passes in reverse and routes dLoss/dD along the recorded predecessors to
// the image and the soft mask.  One CTA runs one image at a time from a work
// queue, like the batched transform (fg_batch.cu).

#include <math.h>

#include <algorithm>
#include <type_traits>

#include "fg_row2d.cuh"

namespace fgi {
namespace {
// shared memory of the forward with S steps per transposed flush: one map,
// the channel body of max_C (1, or the general one)
size_t grad_fwd_smem(int max_C, int max_extent, int S) {
  const int depth = pass_depth(pass_nch(max_C == 1 ? 1 : 0, MODE_GENERAL), 1);
  return std::max(batch_job_smem(max_C, 1, max_extent, S, depth), kBatchTransposeSmem);
}
int grad_flush_steps(int max_C, int max_extent) {
  return grad_fwd_smem(max_C, max_extent, 8) <= kBatchSmemLimit ? 8 : 4;
}
}  // namespace
}  // namespace fgi


// ---------------------------------------------------------------------------
// differentiable 2D transform: forward with argmin tape, adjoint kernel
// ---------------------------------------------------------------------------

namespace fgi {
namespace {

__device__ fg_batch2d_item as_batch_item(const fg_grad2d_item &g) {
  fg_batch2d_item b;
  b.image = g.image, b.mask = g.mask, b.out = g.out, b.image_t = g.image_t;
  b.d2 = nullptr, b.t1 = g.t1, b.t2 = nullptr;
  b.C = g.C, b.H = g.H, b.W = g.W, b.flags = 0;
  b.v = g.v, b.l_grad = g.l_grad, b.l_eucl = g.l_eucl, b.reserved1 = 0.0f;
  return b;
}

// tape_pass < 0: record the tape of every pass at (iteration * 4 + pass) * H * W.
// tape_pass >= 0: run the passes up to that one (numbered iteration * 4 + k)
// and record only its tape, at the start of the item's tape buffer (the
// memory-saving mode's recomputation).
template <int CT>
__global__ void __launch_bounds__(kThreads, 1)
    fg_grad2d_forward_kernel(const fg_grad2d_item *items, int n, int iterations, int tape_pass, int S, float r2,
                             int *counter, int *status) {
  extern __shared__ __align__(16) float sm[];
  __shared__ int s_item;
  __shared__ PassArgs s_args;
  for (;;) {
    if (threadIdx.x == 0) s_item = atomicAdd(counter, 1);
    __syncthreads();
    const int i = s_item;
    if (i >= n) break;
    const fg_grad2d_item g = items[i];
    const fg_batch2d_item it = as_batch_item(g);
    const long long P = (long long)it.H * it.W;
    if (P > 0) {
      batch_prologue(it, 0, 1, true, sm);
      __threadfence();
      __syncthreads();
      const int npass = tape_pass >= 0 ? tape_pass + 1 : 4 * iterations;
      for (int pi = 0; pi < npass; pi++) {
        const int k = pi & 3;
        const int L = k >= 2 ? it.W : it.H;
        const bool wt = k & 1;
        if (L <= 1 && !wt) continue;
        const bool rec = tape_pass < 0 || pi == tape_pass;
        if (threadIdx.x == 0) {
          batch_pass_args(it, 1, 0, k, S, pass_depth(pass_nch(CT, MODE_GENERAL), 1), r2, status, &s_args);
          s_args.tape = rec ? g.tape + (tape_pass < 0 ? (long long)pi * P : 0) : nullptr;
        }
        __syncthreads();
        // the tape-recording body gives the same distances as the plain one
        if (rec) {
          if (wt)
            pass_body<1, CT, 1, MODE_GENERAL, true, true, false>(s_args, 0, sm);
          else
            pass_body<1, CT, 1, MODE_GENERAL, false, true, false>(s_args, 0, sm);
        } else {
          if (wt)
            pass_body<1, CT, 1, MODE_GENERAL, true, false, false>(s_args, 0, sm);
          else
            pass_body<1, CT, 1, MODE_GENERAL, false, false, false>(s_args, 0, sm);
        }
        __threadfence();
        __syncthreads();
      }
    }
    __syncthreads();
  }
}

// The forward of images up to 512 per side: the row body (one thread per
// cell of a row, fg_row2d.cuh), compiled per channel count, the same
// distances and the same tape as fg_grad2d_forward_kernel.
template <bool REC, bool WT>
__device__ __forceinline__ void grad_row_pass(int C, const PassArgs &a, float *sm) {
  switch (C) {
    case 1: row_pass<1, 1, MODE_GENERAL, WT, REC>(a, sm); break;
    case 2: row_pass<2, 1, MODE_GENERAL, WT, REC>(a, sm); break;
    case 3: row_pass<3, 1, MODE_GENERAL, WT, REC>(a, sm); break;
    default: row_pass<4, 1, MODE_GENERAL, WT, REC>(a, sm); break;
  }
}

__global__ void __launch_bounds__(512, 1)
    fg_grad2d_forward_row_kernel(const fg_grad2d_item *items, int n, int iterations, int tape_pass, int S, float r2,
                                 int *counter, int *status) {
  extern __shared__ __align__(16) float sm[];
  __shared__ int s_item;
  __shared__ PassArgs s_args;
  for (;;) {
    if (threadIdx.x == 0) s_item = atomicAdd(counter, 1);
    __syncthreads();
    const int i = s_item;
    if (i >= n) break;
    const fg_grad2d_item g = items[i];
    const fg_batch2d_item it = as_batch_item(g);
    const long long P = (long long)it.H * it.W;
    if (P > 0) {
      batch_prologue(it, 0, 1, true, sm);
      __threadfence();
      __syncthreads();
      const int npass = tape_pass >= 0 ? tape_pass + 1 : 4 * iterations;
      for (int pi = 0; pi < npass; pi++) {
        const int k = pi & 3;
        const int L = k >= 2 ? it.W : it.H;
        const bool wt = k & 1;
        if (L <= 1 && !wt) continue;
        const bool rec = tape_pass < 0 || pi == tape_pass;
        if (threadIdx.x == 0) {
          batch_pass_args(it, 1, 0, k, S, 2, r2, status, &s_args);
          s_args.tape = rec ? g.tape + (tape_pass < 0 ? (long long)pi * P : 0) : nullptr;
        }
        __syncthreads();
        // every pass runs the recording body; a pass without a tape (the
        // memory-saving mode's earlier passes) skips only its write-back
        if (wt)
          grad_row_pass<true, true>(it.C, s_args, sm);
        else
          grad_row_pass<true, false>(it.C, s_args, sm);
        __threadfence();
        __syncthreads();
      }
    }
    __syncthreads();
  }
}

__device__ __forceinline__ float sgnf(float d) { return d > 0.0f ? 1.0f : (d < 0.0f ? -1.0f : 0.0f); }

// Adjoint of one pass of one image (one CTA).  The forward pass computed, for
// t = 1..L-1 and every cell x, D[t][x] = min(Dold[t][x], D[t-1][x+k] + cost_k);
// the tape holds which term won.  Walking t downwards, the gradient of a cell
// either stays with Dold (the pass input) or moves to the predecessor
// D[t-1][x+k] (and to the image through l_grad * |I - I'| of that step).
template <int NCH, int J>
__device__ void adjoint_pass(const fg_grad2d_item &g, int k, const unsigned char *tape, int C, float *sm) {
  const int tid = threadIdx.x, NT = blockDim.x;
  const int H = g.H, W = g.W;
  const long long P = (long long)H * W;
  const bool alongW = k >= 2;
  const int dir = (k & 1) ? -1 : 1;
  const int L = alongW ? W : H, N = alongW ? H : W;
  const long long s_str = alongW ? H : W;                      // read layout: step stride (cross stride 1)
  long long ws_str, wc;                                        // write layout
  if (k == 1) ws_str = 1, wc = H;
  else if (k == 3) ws_str = 1, wc = W;
  else ws_str = s_str, wc = 1;
  const float *Gout = (k == 0 || k == 3) ? g.g_r : g.g_t;
  float *Gin = alongW ? g.g_t : g.g_r;
  const float *I = alongW ? g.image_t : g.image;
  float *gI = alongW ? g.gi_t : g.g_image;
  const float lg = g.l_grad;
  // the gradient each cell of a row hands to the previous row and its tape
  // code, double-buffered by step parity (one barrier per step)
  float *gvb = sm;                                   // [2][N]
  int *cdb = reinterpret_cast<int *>(sm + 2 * N);    // [2][N]
  // J cells per thread, x = tid + j * NT: N <= J * NT (J is chosen from the
  // batch's widest image, so no thread carries empty cells)
  auto pos = [&](int t) -> long long { return dir > 0 ? (long long)t : (long long)(L - 1 - t); };
  // Per cell x = tid + j * NT: the step's inputs, loaded one step ahead so
  // that no global load sits on a step's critical path.  Image rows are kept
  // at x-1, x, x+1 (row s of the step and row sp before it); each step loads
  // one new row, the next step's sp.
  float go[J], gi[J][NCH], is_[J][NCH][3], isp[J][NCH][3];
  int cd[J];
  float go_n[J], gi_n[J][NCH], isp_n[J][NCH][3];
  int cd_n[J];
  auto load_row = [&](float (&dst)[J][NCH][3], long long r) {
#pragma unroll
    for (int j = 0; j < J; j++) {
      const int x = tid + j * NT;
#pragma unroll
      for (int c = 0; c < NCH; c++)
#pragma unroll
        for (int q = 0; q < 3; q++) {
          const int xx = x + q - 1;
          dst[j][c][q] = (c < C && x < N && xx >= 0 && xx < N) ? I[c * P + r * s_str + xx] : 0.0f;
        }
    }
  };
  auto load_step = [&](float (&go_)[J], int (&cd_)[J], float (&gi_)[J][NCH], int t) {
    const long long s = pos(t);
#pragma unroll
    for (int j = 0; j < J; j++) {
      const int x = tid + j * NT;
      go_[j] = x < N ? Gout[s * ws_str + x * wc] : 0.0f;
      cd_[j] = (x < N && t > 0) ? (int)tape[s * s_str + x] : 0;
#pragma unroll
      for (int c = 0; c < NCH; c++) gi_[j][c] = (c < C && x < N) ? gI[c * P + s * s_str + x] : 0.0f;
    }
  };
  float racc[J], gip[J][NCH];
#pragma unroll
  for (int j = 0; j < J; j++) {
    racc[j] = 0.0f;
#pragma unroll
    for (int c = 0; c < NCH; c++) gip[j][c] = 0.0f;
  }
  load_step(go, cd, gi, L - 1);
  load_row(is_, pos(L - 1));
  if (L > 1) load_row(isp, pos(L - 2));
  for (int t = L - 1; t >= 0; t--) {
    const long long s = pos(t);
    // the next step's inputs, in flight during this step
    if (t > 0) load_step(go_n, cd_n, gi_n, t - 1);
    if (t > 1) load_row(isp_n, pos(t - 2));
    float *gv = gvb + (t & 1) * N;
    int *cdr = cdb + (t & 1) * N;
#pragma unroll
    for (int j = 0; j < J; j++) {
      const int x = tid + j * NT;
      if (x >= N) continue;
      const float G = __fadd_rn(go[j], racc[j]);
      const int code = cd[j];
      float gself[NCH];
#pragma unroll
      for (int c = 0; c < NCH; c++) gself[c] = 0.0f;
      if (code == kTapeSelf) {
        Gin[s * s_str + x] = G;
        gv[x] = 0.0f;
      } else {
        Gin[s * s_str + x] = 0.0f;
#pragma unroll
        for (int c = 0; c < NCH; c++)
          if (c < C) {
            // the predecessor x + code - 2 of row sp
            const float ip = code == 1 ? isp[j][c][0] : (code == 2 ? isp[j][c][1] : isp[j][c][2]);
            const float d = __fsub_rn(is_[j][c][1], ip);
            gself[c] = __fmul_rn(__fmul_rn(G, lg), sgnf(d));
          }
        gv[x] = G;
      }
      cdr[x] = code;
#pragma unroll
      for (int c = 0; c < NCH; c++)
        if (c < C) gI[c * P + s * s_str + x] = __fadd_rn(gi[j][c], __fadd_rn(gself[c], gip[j][c]));
    }
    __syncthreads();
    if (t > 0) {
#pragma unroll
      for (int j = 0; j < J; j++) {
        const int xq = tid + j * NT;  // cell of row t-1
        racc[j] = 0.0f;
#pragma unroll
        for (int c = 0; c < NCH; c++) gip[j][c] = 0.0f;
        if (xq >= N) continue;
#pragma unroll
        for (int d = -1; d <= 1; d++) {
          const int x = xq - d;  // a cell of row t whose step came from xq
          if (x < 0 || x >= N || cdr[x] != d + 2) continue;
          const float gx = gv[x];
          racc[j] = __fadd_rn(racc[j], gx);
#pragma unroll
          for (int c = 0; c < NCH; c++)
            if (c < C) {
              const float dd = __fsub_rn(is_[j][c][1 - d], isp[j][c][1]);
              gip[j][c] = __fsub_rn(gip[j][c], __fmul_rn(__fmul_rn(gx, lg), sgnf(dd)));
            }
        }
      }
      // rows and inputs move down one step
#pragma unroll
      for (int j = 0; j < J; j++) {
        go[j] = go_n[j];
        cd[j] = cd_n[j];
#pragma unroll
        for (int c = 0; c < NCH; c++) {
          gi[j][c] = gi_n[j][c];
#pragma unroll
          for (int q = 0; q < 3; q++) is_[j][c][q] = isp[j][c][q], isp[j][c][q] = isp_n[j][c][q];
        }
      }
    }
  }
  __syncthreads();  // the next pass reuses the exchange rows
}

// Ring of the staged adjoint (adjoint_pass_ring): a step's image row is read
// again as the previous row of the next step, so a slot is refilled two
// steps after its own and the loads run kAdjRing - 2 steps ahead.
constexpr int kAdjRing = 8;
// floats of one ring slot: upstream gradients, image-gradient row, image row
// (C channels each where it applies) and the tape row as 4-byte words
__host__ __device__ inline int adj_slot_floats(int N, int C) { return N * (1 + 2 * C) + (N + 3) / 4; }

// The adjoint of one pass as adjoint_pass, with every global input of a step
// (upstream gradient and image-gradient rows, image row, tape row) staged
// into a shared ring by cp.async kAdjRing - 2 steps ahead; same arithmetic,
// same order, same bits.
template <int NCH, int J>
__device__ void adjoint_pass_ring(const fg_grad2d_item &g, int k, const unsigned char *tape, int C, float *sm) {
  const int tid = threadIdx.x, NT = blockDim.x;
  const int H = g.H, W = g.W;
  const long long P = (long long)H * W;
  const bool alongW = k >= 2;
  const int dir = (k & 1) ? -1 : 1;
  const int L = alongW ? W : H, N = alongW ? H : W;
  const long long s_str = alongW ? H : W;
  long long ws_str, wc;
  if (k == 1) ws_str = 1, wc = H;
  else if (k == 3) ws_str = 1, wc = W;
  else ws_str = s_str, wc = 1;
  const float *Gout = (k == 0 || k == 3) ? g.g_r : g.g_t;
  float *Gin = alongW ? g.g_t : g.g_r;
  const float *I = alongW ? g.image_t : g.image;
  float *gI = alongW ? g.gi_t : g.g_image;
  const float lg = g.l_grad;
  float *gvb = sm;                                   // [2][N] by step parity
  int *cdb = reinterpret_cast<int *>(sm + 2 * N);    // [2][N]
  float *ring = sm + 4 * N;                          // [kAdjRing][slot]
  const int SLOT = adj_slot_floats(N, C);
  // tape rows as 4-byte words where every row starts on one
  const bool tw = N % 4 == 0 && s_str % 4 == 0 && (reinterpret_cast<uintptr_t>(tape) & 3) == 0;
  auto pos = [&](int t) -> long long { return dir > 0 ? (long long)t : (long long)(L - 1 - t); };
  auto slot = [&](int t) -> float * { return ring + (t & (kAdjRing - 1)) * SLOT; };
  auto stage = [&](int u) {  // step u's inputs into its slot: one commit group, possibly empty
    if (u >= 0) {
      float *sl = slot(u);
      const long long s = pos(u);
      for (int x = tid; x < N; x += NT) {
        cp_async4(sl + x, Gout + s * ws_str + x * wc);
        for (int c = 0; c < C; c++) {
          cp_async4(sl + (1 + c) * N + x, gI + c * P + s * s_str + x);
          cp_async4(sl + (1 + C + c) * N + x, I + c * P + s * s_str + x);
        }
      }
      if (tw && u > 0)
        for (int w = tid; w < N / 4; w += NT) cp_async4(sl + (1 + 2 * C) * N + w, tape + s * s_str + 4 * w);
    }
    cp_async_commit();
  };
  float racc[J], gip[J][NCH];
#pragma unroll
  for (int j = 0; j < J; j++) {
    racc[j] = 0.0f;
#pragma unroll
    for (int c = 0; c < NCH; c++) gip[j][c] = 0.0f;
  }
  for (int u = L - 1; u >= L - (kAdjRing - 2); u--) stage(u);
  cp_async_wait<kAdjRing - 4>();  // steps L-1 and L-2 have landed
  __syncthreads();
  for (int t = L - 1; t >= 0; t--) {
    const long long s = pos(t);
    const float *sl = slot(t), *slp = slot(t - 1);
    float *gv = gvb + (t & 1) * N;
    int *cdr = cdb + (t & 1) * N;
#pragma unroll
    for (int j = 0; j < J; j++) {
      const int x = tid + j * NT;
      if (x >= N) continue;
      const float G = __fadd_rn(sl[x], racc[j]);
      const int code = t == 0 ? 0
                              : (tw ? (int)reinterpret_cast<const unsigned char *>(sl + (1 + 2 * C) * N)[x]
                                    : (int)tape[s * s_str + x]);
      float gself[NCH];
#pragma unroll
      for (int c = 0; c < NCH; c++) gself[c] = 0.0f;
      if (code == kTapeSelf) {
        Gin[s * s_str + x] = G;
        gv[x] = 0.0f;
      } else {
        Gin[s * s_str + x] = 0.0f;
        const int xp = x + code - 2;
#pragma unroll
        for (int c = 0; c < NCH; c++)
          if (c < C) {
            const float d = __fsub_rn(sl[(1 + C + c) * N + x], slp[(1 + C + c) * N + xp]);
            gself[c] = __fmul_rn(__fmul_rn(G, lg), sgnf(d));
          }
        gv[x] = G;
      }
      cdr[x] = code;
#pragma unroll
      for (int c = 0; c < NCH; c++)
        if (c < C) gI[c * P + s * s_str + x] = __fadd_rn(sl[(1 + c) * N + x], __fadd_rn(gself[c], gip[j][c]));
    }
    cp_async_wait<kAdjRing - 5>();  // step t-2 has landed (read after the barrier)
    __syncthreads();
    stage(t + 2 - kAdjRing);         // into the slot of step t+2, whose last reader (step t+1) is done
    if (t > 0) {
#pragma unroll
      for (int j = 0; j < J; j++) {
        const int xq = tid + j * NT;  // cell of row t-1
        racc[j] = 0.0f;
#pragma unroll
        for (int c = 0; c < NCH; c++) gip[j][c] = 0.0f;
        if (xq >= N) continue;
#pragma unroll
        for (int d = -1; d <= 1; d++) {
          const int x = xq - d;  // a cell of row t whose step came from xq
          if (x < 0 || x >= N || cdr[x] != d + 2) continue;
          const float gx = gv[x];
          racc[j] = __fadd_rn(racc[j], gx);
#pragma unroll
          for (int c = 0; c < NCH; c++)
            if (c < C) {
              const float dd = __fsub_rn(sl[(1 + C + c) * N + x], slp[(1 + C + c) * N + xq]);
              gip[j][c] = __fsub_rn(gip[j][c], __fmul_rn(__fmul_rn(gx, lg), sgnf(dd)));
            }
        }
      }
    }
  }
  cp_async_wait<0>();
  __syncthreads();  // the next pass reuses the ring and the exchange rows
}

// Adjoints of the passes pass_hi down to pass_lo (numbered iteration * 4 + k);
// the tape of pass pi is at (pi - tape_base) * H * W.  kGradInit: the gradient
// state starts from dLoss/dD; kGradFinal: dLoss/dmask and dLoss/dimage are
// written at the end.  One call with both flags over every pass is the whole
// backward; the memory-saving mode calls it once per pass.
constexpr int kGradInit = 1, kGradFinal = 2;

template <int NCH, int J, bool RING>
__global__ void __launch_bounds__(kThreads, 1)
    fg_grad2d_backward_kernel(const fg_grad2d_item *items, int n, int pass_hi, int pass_lo, int tape_base,
                              int flags, int *counter) {
  extern __shared__ __align__(16) float sm[];
  __shared__ int s_item;
  for (;;) {
    if (threadIdx.x == 0) s_item = atomicAdd(counter, 1);
    __syncthreads();
    const int i = s_item;
    if (i >= n) break;
    const fg_grad2d_item g = items[i];
    const int H = g.H, W = g.W, C = g.C;
    const long long P = (long long)H * W;
    if (P > 0) {
      if (flags & kGradInit) {
        for (long long p = threadIdx.x; p < P; p += blockDim.x) g.g_r[p] = g.g_out[p];
        for (long long p = threadIdx.x; p < C * P; p += blockDim.x) g.g_image[p] = 0.0f, g.gi_t[p] = 0.0f;
        __threadfence();
        __syncthreads();
      }
      for (int pi = pass_hi; pi >= pass_lo; pi--) {
        const int k = pi & 3;
        const int L = k >= 2 ? W : H;
        if (L <= 1 && !(k & 1)) continue;  // the forward skipped this pass
        if (RING)
          adjoint_pass_ring<NCH, J>(g, k, g.tape + (long long)(pi - tape_base) * P, C, sm);
        else
          adjoint_pass<NCH, J>(g, k, g.tape + (long long)(pi - tape_base) * P, C, sm);
        __threadfence();
        __syncthreads();
      }
      if (flags & kGradFinal) {
        // dLoss/dmask = v * dLoss/dD0 ; dLoss/dimage = its original-layout part + the transposed part
        for (long long p = threadIdx.x; p < P; p += blockDim.x) g.g_mask[p] = __fmul_rn(g.v, g.g_r[p]);
        for (long long q = threadIdx.x; q < C * P; q += blockDim.x) {
          const long long c = q / P, r = q - c * P, h = r / W, w = r - h * W;
          g.g_image[q] = __fadd_rn(g.g_image[q], g.gi_t[c * P + w * H + h]);
        }
      }
    }
    __syncthreads();
  }
}

}  // namespace
}  // namespace fgi

namespace fgi {
namespace {
int grad_forward(const fg_grad2d_item *items, int n, int max_C, int max_extent, int iterations, int tape_pass,
                 int *counter, int *status, void *stream) {
  if (n < 0 || (n > 0 && (!items || !counter || !status)))
    return set_error(FG_ERR_INVALID_ARGUMENT, "grad: null descriptor, counter or status pointer");
  if (max_C < 1 || max_C > kMaxChannels) return set_error(FG_ERR_UNSUPPORTED, "grad: images need 1 to 4 channels");
  if (max_extent > 4 * kThreads) return set_error(FG_ERR_UNSUPPORTED, "grad: image sides up to 2048 are supported");
  if (n == 0) return FG_OK;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  cudaError_t e = cudaMemsetAsync(counter, 0, sizeof(int), s);
  if (e != cudaSuccess) return set_error(FG_ERR_CUDA, cudaGetErrorString(e));
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int grid = std::max(1, std::min(n, sms));
  const float r2 = (float)sqrt(2.0);  // fastgeodis_cpu.cpp:67
  if (max_extent <= kOneLaunchSide) {
    // rows up to 512 cells: the row body, one thread per cell
    const int NT = std::max(32, (max_extent + 31) / 32 * 32), S = 8;
    const size_t smem = std::max(row_smem(max_C, 1, max_extent, S, true), (size_t)(NT / 32) * 32 * 33 * 4);
    auto fn = fg_grad2d_forward_row_kernel;
    cudaError_t e2 = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e2 != cudaSuccess) return set_error(FG_ERR_CUDA, cudaGetErrorString(e2));
    fn<<<grid, NT, smem, s>>>(items, n, std::max(iterations, 0), tape_pass, S, r2, counter, status);
    e2 = cudaGetLastError();
    return e2 == cudaSuccess ? FG_OK : set_error(FG_ERR_CUDA, cudaGetErrorString(e2));
  }
  const int S = grad_flush_steps(max_C, max_extent);
  const size_t smem = grad_fwd_smem(max_C, max_extent, S);
  if (smem > kBatchSmemLimit) return set_error(FG_ERR_UNSUPPORTED, "grad: shared memory plan too large");
  auto launch = [&](auto fn) -> int {
    cudaError_t e2 = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e2 != cudaSuccess) return set_error(FG_ERR_CUDA, cudaGetErrorString(e2));
    fn<<<grid, kThreads, smem, s>>>(items, n, std::max(iterations, 0), tape_pass, S, r2, counter, status);
    e2 = cudaGetLastError();
    return e2 == cudaSuccess ? FG_OK : set_error(FG_ERR_CUDA, cudaGetErrorString(e2));
  };
  return max_C == 1 ? launch(fg_grad2d_forward_kernel<1>) : launch(fg_grad2d_forward_kernel<0>);
}
}  // namespace
}  // namespace fgi

extern "C" FG_API int fg_grad_geodesic2d_forward(const fg_grad2d_item *items, int n, int max_C, int max_extent,
                                                 int iterations, int *counter, int *status, void *stream) {
  return fgi::grad_forward(items, n, max_C, max_extent, iterations, -1, counter, status, stream);
}

extern "C" FG_API int fg_grad_geodesic2d_forward_pass(const fg_grad2d_item *items, int n, int max_C, int max_extent,
                                                      int pass, int *counter, int *status, void *stream) {
  if (pass < 0) return fgi::set_error(FG_ERR_INVALID_ARGUMENT, "grad: negative pass index");
  return fgi::grad_forward(items, n, max_C, max_extent, pass / 4 + 1, pass, counter, status, stream);
}

namespace fgi {
namespace {
int grad_backward(const fg_grad2d_item *items, int n, int max_C, int max_extent, int pass_hi, int pass_lo,
                  int tape_base, int flags, int *counter, void *stream) {
  if (n < 0 || (n > 0 && (!items || !counter)))
    return set_error(FG_ERR_INVALID_ARGUMENT, "grad: null descriptor or counter pointer");
  if (max_C < 1 || max_C > kMaxChannels) return set_error(FG_ERR_UNSUPPORTED, "grad: images need 1 to 4 channels");
  if (max_extent > 4 * kThreads) return set_error(FG_ERR_UNSUPPORTED, "grad: image sides up to 2048 are supported");
  if (n == 0) return FG_OK;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  cudaError_t e = cudaMemsetAsync(counter, 0, sizeof(int), s);
  if (e != cudaSuccess) return set_error(FG_ERR_CUDA, cudaGetErrorString(e));
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  // adjoint_pass: gradient and code rows, two of each; the staged form adds its ring
  const size_t smem_reg = (size_t)4 * max_extent * 4 + 64;
  const size_t smem_ring = smem_reg + (size_t)kAdjRing * adj_slot_floats(max_extent, max_C) * 4;
  const bool ring = smem_ring <= kBatchSmemLimit;
  const size_t smem = ring ? smem_ring : smem_reg;
  const int grid = std::max(1, std::min(n, sms));
  auto launch = [&](auto fn) -> int {
    cudaError_t e2 = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e2 != cudaSuccess) return set_error(FG_ERR_CUDA, cudaGetErrorString(e2));
    fn<<<grid, kThreads, smem, s>>>(items, n, pass_hi, pass_lo, tape_base, flags, counter);
    e2 = cudaGetLastError();
    return e2 == cudaSuccess ? FG_OK : set_error(FG_ERR_CUDA, cudaGetErrorString(e2));
  };
  // cells per thread: the fewest that cover the widest image's rows and columns;
  // the staged adjoint where its ring fits shared memory
  auto by_j = [&](auto ring_tag) -> int {
    constexpr bool R = decltype(ring_tag)::value;
    if (max_extent <= kThreads)
      return max_C == 1 ? launch(fg_grad2d_backward_kernel<1, 1, R>) : launch(fg_grad2d_backward_kernel<kMaxChannels, 1, R>);
    if (max_extent <= 2 * kThreads)
      return max_C == 1 ? launch(fg_grad2d_backward_kernel<1, 2, R>) : launch(fg_grad2d_backward_kernel<kMaxChannels, 2, R>);
    return max_C == 1 ? launch(fg_grad2d_backward_kernel<1, 4, R>) : launch(fg_grad2d_backward_kernel<kMaxChannels, 4, R>);
  };
  return ring ? by_j(std::true_type{}) : by_j(std::false_type{});
}
}  // namespace
}  // namespace fgi

extern "C" FG_API int fg_grad_geodesic2d_backward(const fg_grad2d_item *items, int n, int max_C, int max_extent,
                                                  int iterations, int *counter, int *status, void *stream) {
  (void)status;
  return fgi::grad_backward(items, n, max_C, max_extent, 4 * std::max(iterations, 0) - 1, 0, 0,
                            fgi::kGradInit | fgi::kGradFinal, counter, stream);
}

extern "C" FG_API int fg_grad_geodesic2d_backward_pass(const fg_grad2d_item *items, int n, int max_C, int max_extent,
                                                       int pass, int first, int last, int *counter, void *stream) {
  if (pass < 0) return fgi::set_error(FG_ERR_INVALID_ARGUMENT, "grad: negative pass index");
  return fgi::grad_backward(items, n, max_C, max_extent, pass, pass, pass,
                            (first ? fgi::kGradInit : 0) | (last ? fgi::kGradFinal : 0), counter, stream);
}
