// Toivanen's raster scan on the GPU, as a wavefront.
//
// Reference: FastGeodis/geodis_toivanen.cpp (CPU only there; one thread).
// Each iteration is a forward pass that visits every cell in memory order
// (depth, rows, columns) and replaces it by the minimum of itself and the
// candidates (D[n] + l_eucl*ld[n]) + l_grad*L1 of its causal neighbours n,
// then a backward pass in reverse order with the mirrored neighbour set
// (2D :40-146, 3D :166-329).  A cell reads neighbours that the sequential
// order has already updated in this pass and, in 3D, four cells of the next
// plane that it has not (they keep the previous pass's values).
//
// Wavefront: give cell (z, h, w) the wave t = 4z + 2h + w (2D: z = 0).  Every
// neighbour the sequential order updates first has a smaller wave (offsets
// change t by -7 .. -1) and each next-plane neighbour a larger one (+1 .. +3),
// so sweeping the waves in order, the cells of a wave in parallel and a
// barrier between waves, every cell reads exactly the values the sequential
// scan reads: the results are the reference's bits.  The backward pass is the
// same schedule on the mirrored coordinates.
//
// Each distance map is swept by its own group of CTAs (signed and GSF run
// their maps side by side).  A small image's waves fit one CTA, whose barrier
// orders them.  A volume's waves hold thousands of cells, so its group spans up
// to one CTA per SM (cooperative launch, all resident) and the waves are
// ordered by a grid barrier of the group: an arrive counter in the workspace
// header, polled with acquire loads under a bound (FG_ERR_TIMEOUT in the
// status word if it ever expires).  Distances are read and written through L2
// (.cg): another SM's L1 may hold a line from an earlier wave.

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>

#include "fg_common.cuh"
#include "fg_wait.cuh"

namespace fgi {
namespace {

constexpr int kToivMaps = 4;

struct ToivArgs {
  const float *img;   // [C][D][H][W]
  long long img_cs;   // elements between channels
  int C;
  float *dist[kToivMaps];  // one map per group of CTAs, [D][H][W] (channel 0 of the distance tensor)
  int D, H, W;             // D = 1 for images
  float lg, le;
  float ldf[13], ldb[13];  // step lengths of the forward and backward neighbours
  int iterations;
  int group;               // CTAs per map
  unsigned *bar;           // arrive counters, one per map (zero at launch)
  int *status;             // FG_ERR_TIMEOUT if a barrier wait expired
};

// Barrier of the `group` CTAs of one map: the n-th call returns once all of
// them have arrived n times.  Bounded: after kSpinLimit polls (or once another
// CTA has recorded a timeout) it records FG_ERR_TIMEOUT and returns.
__device__ __forceinline__ void toiv_group_sync(const ToivArgs &a, unsigned *bar, unsigned &arrivals) {
  __syncthreads();
  if (threadIdx.x == 0) {
    arrivals += (unsigned)a.group;
    __threadfence();  // this CTA's cell writes (ordered by the barrier above) before the arrival
    atomicAdd(bar, 1u);
    wait_count(bar, arrivals, a.status, kSpinLimit);
  }
  __syncthreads();
}

// Neighbour offsets (dz, dh, dw) in the reference's order:
// 2D forward / backward geodis_toivanen.cpp:56-57, 101-102;
// 3D forward / backward :182-184, :209-211.
template <bool IS3D, bool BWD>
__device__ __forceinline__ void toiv_offset(int j, int &dz, int &dh, int &dw) {
  if (!IS3D) {
    constexpr int fh[4] = {-1, -1, -1, 0}, fw[4] = {-1, 0, 1, -1};
    constexpr int bh[4] = {0, 1, 1, 1}, bw[4] = {1, -1, 0, 1};
    dz = 0;
    dh = BWD ? bh[j] : fh[j];
    dw = BWD ? bw[j] : fw[j];
  } else {
    constexpr int fz[13] = {-1, -1, -1, -1, -1, 0, 0, 0, 0, 1, 1, 1, 1};
    constexpr int fh[13] = {-1, -1, -1, 0, 0, -1, -1, -1, 0, -1, -1, -1, 0};
    constexpr int fw[13] = {-1, 0, 1, -1, 0, -1, 0, 1, -1, -1, 0, 1, -1};
    constexpr int bz[13] = {-1, -1, -1, -1, 0, 0, 0, 0, 1, 1, 1, 1, 1};
    constexpr int bh[13] = {0, 1, 1, 1, 0, 1, 1, 1, 0, 0, 1, 1, 1};
    constexpr int bw[13] = {1, -1, 0, 1, 1, -1, 0, 1, 0, 1, -1, 0, 1};
    dz = BWD ? bz[j] : fz[j];
    dh = BWD ? bh[j] : fh[j];
    dw = BWD ? bw[j] : fw[j];
  }
}

// GROUP: the map is swept by several CTAs, so distances go through L2 (.cg);
// one CTA reads its own writes through its SM's L1.
template <bool IS3D, bool BWD, bool GROUP>
__device__ __forceinline__ float toiv_ld(const float *p) {
  return GROUP ? __ldcg(p) : *p;
}

template <bool IS3D, bool BWD, bool GROUP>
__device__ __forceinline__ void toiv_cell(const ToivArgs &a, float *dm, int z, int h, int w) {
  constexpr int N = IS3D ? 13 : 4;
  const int H = a.H, W = a.W;
  const long long i = ((long long)z * H + h) * W + w;
  float nd = toiv_ld<IS3D, BWD, GROUP>(dm + i);
#pragma unroll
  for (int j = 0; j < N; j++) {
    int dz, dh, dw;
    toiv_offset<IS3D, BWD>(j, dz, dh, dw);
    const int zi = z + dz, hi = h + dh, wi = w + dw;
    if (zi < 0 || zi >= a.D || hi < 0 || hi >= H || wi < 0 || wi >= W) continue;
    const long long q = ((long long)zi * H + hi) * W + wi;
    float l1;
    if (a.C == 1) {
      l1 = fabsf(__fsub_rn(__ldg(a.img + i), __ldg(a.img + q)));  // geodis_toivanen.cpp:35-38
    } else {
      l1 = 0.0f;
      for (int c = 0; c < a.C; c++)
        l1 = __fadd_rn(l1, fabsf(__fsub_rn(__ldg(a.img + c * a.img_cs + i), __ldg(a.img + c * a.img_cs + q))));
    }
    const float ld = BWD ? a.ldb[j] : a.ldf[j];
    const float cur = __fadd_rn(__fadd_rn(toiv_ld<IS3D, BWD, GROUP>(dm + q), __fmul_rn(a.le, ld)), __fmul_rn(a.lg, l1));
    nd = cur < nd ? cur : nd;  // std::min(new_dist, cur_dist)
  }
  if (GROUP)
    __stcg(dm + i, nd);
  else
    dm[i] = nd;
}

// One pass: waves t = 0 .. T-1 of the (mirrored, if BWD) coordinates.
template <bool IS3D, bool BWD, bool GROUP>
__device__ __forceinline__ void toiv_pass(const ToivArgs &a, float *dm, int rank, unsigned *bar, unsigned &arrivals) {
  const int D = a.D, H = a.H, W = a.W;
  const int T = 4 * (D - 1) + 2 * (H - 1) + (W - 1) + 1;
  const int wb = min(H, (W - 1) / 2 + 1);  // cells of one wave in one plane, at most
  for (int t = 0; t < T; t++) {
    const int x = t - 2 * (H - 1) - (W - 1);
    const int zlo = x > 0 ? (x + 3) / 4 : 0, zhi = min(D - 1, t / 4);
    const int n = (zhi - zlo + 1) * wb;
    for (int k = rank * blockDim.x + threadIdx.x; k < n; k += a.group * blockDim.x) {
      const int zm = zlo + k / wb, j = k - (k / wb) * wb;
      const int rem = t - 4 * zm;
      const int y = rem - (W - 1);
      const int hm = (y > 0 ? (y + 1) / 2 : 0) + j;
      if (hm > min(H - 1, rem / 2)) continue;
      const int wm = rem - 2 * hm;  // 0 <= wm < W by the bounds on hm
      if (BWD)
        toiv_cell<IS3D, true, GROUP>(a, dm, D - 1 - zm, H - 1 - hm, W - 1 - wm);
      else
        toiv_cell<IS3D, false, GROUP>(a, dm, zm, hm, wm);
    }
    if (GROUP)
      toiv_group_sync(a, bar, arrivals);  // the wave's writes are visible to the next wave
    else
      __syncthreads();
  }
}

template <bool IS3D, bool GROUP>
__global__ void __launch_bounds__(1024, 1) fg_toivanen_kernel(const ToivArgs a) {
  const int map = blockIdx.x / a.group, rank = blockIdx.x - map * a.group;
  float *dm = a.dist[map];
  unsigned *bar = GROUP ? a.bar + map : nullptr;  // counters exist for grouped launches only
  unsigned arrivals = 0;
  for (int it = 0; it < a.iterations; it++) {
    toiv_pass<IS3D, false, GROUP>(a, dm, rank, bar, arrivals);
    toiv_pass<IS3D, true, GROUP>(a, dm, rank, bar, arrivals);
  }
}

// Images of at most 1024 rows: one thread per row.  Row h computes its cell
// w = t - 2h at wave t (mirrored coordinates in the backward pass, whose
// neighbour set is the mirror of the forward one).  The three neighbours in
// the row above and the left neighbour come from 4-slot shared rings of the
// rows' latest values (at wave t row h-1 writes slot (w+2) & 3 while row h
// reads slots w-1 .. w+1 of it), so a wave needs no global reads of fresh
// values; a row's own old distance and image values are loaded 4 cells ahead
// into registers.  CT: 1 for one image channel, 0 for 2-4 channels.
constexpr int kRowAhead = 4;

// VEC (rows a multiple of 4 cells, 16-byte aligned maps and image): a
// thread's own cells are read and written four at a time (one float4 per 4
// waves) instead of one scalar access per wave; across a warp every access
// is a different row, so each warp instruction is 32 separate requests and
// their number, not their bytes, bounds a wave.
template <int CT, bool VEC>
__global__ void __launch_bounds__(1024, 1) fg_toivanen_rows_kernel(const ToivArgs a) {
  extern __shared__ float rings[];
  constexpr int NCH = CT == 1 ? 1 : 4;
  constexpr int WIN = VEC ? 8 : kRowAhead;  // own cells held ahead (VEC: this group of 4 and the next)
  const int C = CT == 1 ? 1 : a.C;
  const int H = a.H, W = a.W;
  float *dm = a.dist[blockIdx.x];
  // the latest 4 distances and image values of each row, [4][H] and
  // [C][4][H]: a warp's threads (consecutive rows) read consecutive words
  float *rd = rings;
  float *ri = rings + 4 * H;
  const int hm = threadIdx.x;  // this thread's row, in the pass's (mirrored) coordinates
  const bool row = hm < H;
  const int T = 2 * (H - 1) + W;
  for (int it = 0; it < a.iterations; it++) {
    for (int dir = 0; dir < 2; dir++) {
      const bool bwd = dir == 1;
      const int h = bwd ? H - 1 - hm : hm;  // the row in memory
      auto at = [&](int wm) { return (long long)h * W + (bwd ? W - 1 - wm : wm); };
      // cells wm .. wm + 3 as a float4 in pass order (the memory order reversed backwards)
      auto ld4 = [&](const float *base, int wm, float *out) {
        const float4 v = *reinterpret_cast<const float4 *>(base + (bwd ? at(wm + 3) : at(wm)));
        if (bwd) out[0] = v.w, out[1] = v.z, out[2] = v.y, out[3] = v.x;
        else out[0] = v.x, out[1] = v.y, out[2] = v.z, out[3] = v.w;
      };
      // own old values of cells wm .. wm + WIN - 1, loaded ahead
      float dpf[WIN], ipf[WIN][NCH], wbuf[4];
      if (VEC) {
        if (row) {
          ld4(dm, 0, dpf);
#pragma unroll
          for (int c = 0; c < NCH; c++)
            if (c < C) {
              float t4[4];
              ld4(a.img + c * a.img_cs, 0, t4);
#pragma unroll
              for (int k = 0; k < 4; k++) ipf[k][c] = t4[k];
            }
        }
      } else {
#pragma unroll
        for (int k = 0; k < kRowAhead; k++) {
          if (row && k < W) {
            dpf[k] = dm[at(k)];
#pragma unroll
            for (int c = 0; c < NCH; c++)
              if (c < C) ipf[k][c] = __ldg(a.img + c * a.img_cs + at(k));
          }
        }
      }
      // step lengths by relative position: above-left, above, above-right, left
      const float r2 = a.ldf[0], one = a.ldf[1];
      for (int t = 0; t < T; t++) {
        const int wm = t - 2 * hm;
        if (row && wm >= 0 && wm < W) {
          if (VEC && (wm & 3) == 0 && wm + 4 < W) {
            // the next group of 4 behind this one
            float t4[4];
            ld4(dm, wm + 4, t4);
#pragma unroll
            for (int k = 0; k < 4; k++) dpf[4 + k] = t4[k];
#pragma unroll
            for (int c = 0; c < NCH; c++)
              if (c < C) {
                ld4(a.img + c * a.img_cs, wm + 4, t4);
#pragma unroll
                for (int k = 0; k < 4; k++) ipf[4 + k][c] = t4[k];
              }
          }
          const float dold = dpf[0];
          float icur[NCH];
#pragma unroll
          for (int c = 0; c < NCH; c++)
            if (c < C) icur[c] = ipf[0][c];
          // next cell ahead
#pragma unroll
          for (int k = 0; k < WIN - 1; k++) {
            dpf[k] = dpf[k + 1];
#pragma unroll
            for (int c = 0; c < NCH; c++) ipf[k][c] = ipf[k + 1][c];
          }
          if (!VEC && wm + kRowAhead < W) {
            dpf[kRowAhead - 1] = dm[at(wm + kRowAhead)];
#pragma unroll
            for (int c = 0; c < NCH; c++)
              if (c < C) ipf[kRowAhead - 1][c] = __ldg(a.img + c * a.img_cs + at(wm + kRowAhead));
          }
          float nd = dold;
          // candidates: (row above, wm-1 / wm / wm+1) and (this row, wm-1)
#pragma unroll
          for (int j = 0; j < 4; j++) {
            const int r = j < 3 ? hm - 1 : hm, x = j < 3 ? wm - 1 + j : wm - 1;
            if (r < 0 || x < 0 || x >= W) continue;
            float l1;
            if (CT == 1) {
              l1 = fabsf(__fsub_rn(icur[0], ri[(x & 3) * H + r]));
            } else {
              l1 = 0.0f;
#pragma unroll
              for (int c = 0; c < NCH; c++)
                if (c < C) l1 = __fadd_rn(l1, fabsf(__fsub_rn(icur[c], ri[(c * 4 + (x & 3)) * H + r])));
            }
            const float ld = (j == 0 || j == 2) ? r2 : one;
            const float cur = __fadd_rn(__fadd_rn(rd[(x & 3) * H + r], __fmul_rn(a.le, ld)), __fmul_rn(a.lg, l1));
            nd = cur < nd ? cur : nd;  // std::min(new_dist, cur_dist)
          }
          rd[(wm & 3) * H + hm] = nd;
#pragma unroll
          for (int c = 0; c < NCH; c++)
            if (c < C) ri[(c * 4 + (wm & 3)) * H + hm] = icur[c];
          if (VEC) {
            // results of cells wm - 3 .. wm, written as one float4 when a group ends
            wbuf[0] = wbuf[1], wbuf[1] = wbuf[2], wbuf[2] = wbuf[3], wbuf[3] = nd;
            if ((wm & 3) == 3) {
              const float4 v = bwd ? make_float4(wbuf[3], wbuf[2], wbuf[1], wbuf[0])
                                   : make_float4(wbuf[0], wbuf[1], wbuf[2], wbuf[3]);
              *reinterpret_cast<float4 *>(dm + (bwd ? at(wm) : at(wm - 3))) = v;
            }
          } else {
            dm[at(wm)] = nd;
          }
        }
        __syncthreads();
      }
    }
  }
}

int device_sms() {
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
    return 1;
  return std::max(1, sms);
}

}  // namespace

int launch_toivanen(const float *img, int C, int D, int H, int W, const float *spacing_sq, float *const *maps,
                    int nmaps, float lg, float le, int iterations, unsigned *bar, int *status, cudaStream_t s) {
  if (nmaps < 1 || nmaps > kToivMaps) return set_error(FG_ERR_INVALID_ARGUMENT, "toivanen: 1 to 4 maps per launch");
  if (iterations <= 0) return FG_OK;
  ToivArgs a{};
  a.img = img;
  a.img_cs = (long long)D * H * W;
  a.C = C;
  for (int m = 0; m < nmaps; m++) a.dist[m] = maps[m];
  a.D = D, a.H = H, a.W = W;
  a.lg = lg, a.le = le;
  a.iterations = iterations;
  const bool is3d = spacing_sq != nullptr;
  if (!is3d) {
    const float r2 = sqrtf(2.0f);  // geodis_toivanen.cpp:59, :104
    const float f[4] = {r2, 1.0f, r2, 1.0f}, b[4] = {1.0f, r2, 1.0f, r2};
    for (int j = 0; j < 4; j++) a.ldf[j] = f[j], a.ldb[j] = b[j];
  } else {
    // geodis_toivanen.cpp:186-207, :213-234: sqrt of the summed squared spacings
    // of the axes a neighbour moves along, summed in axis order
    const int fz[13] = {-1, -1, -1, -1, -1, 0, 0, 0, 0, 1, 1, 1, 1};
    const int fh[13] = {-1, -1, -1, 0, 0, -1, -1, -1, 0, -1, -1, -1, 0};
    const int fw[13] = {-1, 0, 1, -1, 0, -1, 0, 1, -1, -1, 0, 1, -1};
    const int bz[13] = {-1, -1, -1, -1, 0, 0, 0, 0, 1, 1, 1, 1, 1};
    const int bh[13] = {0, 1, 1, 1, 0, 1, 1, 1, 0, 0, 1, 1, 1};
    const int bw[13] = {1, -1, 0, 1, 1, -1, 0, 1, 0, 1, -1, 0, 1};
    for (int j = 0; j < 13; j++) {
      float vf = 0.0f, vb = 0.0f;
      if (fz[j]) vf += spacing_sq[0];
      if (fh[j]) vf += spacing_sq[1];
      if (fw[j]) vf += spacing_sq[2];
      if (bz[j]) vb += spacing_sq[0];
      if (bh[j]) vb += spacing_sq[1];
      if (bw[j]) vb += spacing_sq[2];
      a.ldf[j] = sqrtf(vf);
      a.ldb[j] = sqrtf(vb);
    }
  }
  if (!is3d && H <= 1024 && C <= 4) {  // images: one thread per row
    const int threads = std::max(32, (H + 31) / 32 * 32);
    const size_t smem = (size_t)4 * H * (1 + C) * sizeof(float);
    // own cells four at a time where every row starts on 16 bytes
    bool vec = W % 4 == 0 && (reinterpret_cast<uintptr_t>(img) & 15) == 0;
    for (int m = 0; m < nmaps; m++) vec = vec && (reinterpret_cast<uintptr_t>(maps[m]) & 15) == 0;
    auto launch = [&](auto fn) -> cudaError_t {
      cudaError_t e2 = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      if (e2 == cudaSuccess) fn<<<nmaps, threads, smem, s>>>(a);
      return e2;
    };
    cudaError_t e;
    // (several channels keep the scalar form: their 8-cell window of image
    // values spills at the 64 registers of a 1024-thread CTA)
    if (C == 1)
      e = vec ? launch(fg_toivanen_rows_kernel<1, true>) : launch(fg_toivanen_rows_kernel<1, false>);
    else
      e = launch(fg_toivanen_rows_kernel<0, false>);
    if (e == cudaSuccess) e = cudaGetLastError();
    if (e != cudaSuccess) return set_error(FG_ERR_CUDA, cudaGetErrorString(e));
    return FG_OK;
  }
  // threads: the most cells one wave can hold, in whole warps; beyond 4096
  // cells a group of 256-thread CTAs, at most one per SM for each map
  const long long wb = std::min(H, (W - 1) / 2 + 1);
  const long long planes = std::min<long long>(D, (2LL * (H - 1) + (W - 1)) / 4 + 1);
  const long long cells = wb * planes;
  int threads, group = 1;
  if (cells <= 4096) {
    threads = (int)std::max<long long>(32, std::min<long long>(1024, (cells + 31) / 32 * 32));
  } else {
    threads = 256;
    group = (int)std::max<long long>(1, std::min<long long>(device_sms() / nmaps, (cells + 255) / 256));
  }
  a.group = group;
  a.bar = bar;
  a.status = status;
  cudaError_t e = cudaSuccess;
  if (group > 1) {
    if (!bar || !status) return set_error(FG_ERR_INVALID_ARGUMENT, "toivanen: barrier counters missing");
    e = cudaMemsetAsync(bar, 0, kToivMaps * sizeof(unsigned), s);
    if (e != cudaSuccess) return set_error(FG_ERR_CUDA, cudaGetErrorString(e));
    void *args[] = {&a};
    const void *fn =
        is3d ? (const void *)fg_toivanen_kernel<true, true> : (const void *)fg_toivanen_kernel<false, true>;
    e = cudaLaunchCooperativeKernel(fn, dim3(nmaps * group), dim3(threads), args, 0, s);
  } else if (is3d) {
    fg_toivanen_kernel<true, false><<<nmaps, threads, 0, s>>>(a);
  } else {
    fg_toivanen_kernel<false, false><<<nmaps, threads, 0, s>>>(a);
  }
  if (e == cudaSuccess) e = cudaGetLastError();
  if (e != cudaSuccess) return set_error(FG_ERR_CUDA, cudaGetErrorString(e));
  return FG_OK;
}

}  // namespace fgi
