// fastgeodis_gb300 engine: host side and elementwise kernels.
//
// Composes sweep passes (fg_pass.cuh) into the reference's transforms:
//   plain  D(mask)                           FastGeodis/fastgeodis_cuda.cu:278-318, :587-656
//   signed D(mask) - D(1 - mask)             FastGeodis/fastgeodis.cpp:241-258
//   GSF    -signed(1 - Md) + signed(Me)      FastGeodis/fastgeodis.cpp:319-343
// with the reference's pass order: per iteration, 2D: H forward/backward,
// then W forward/backward; 3D: D, H, W pairs (fastgeodis_cpu.cpp:164-201,
// :342-407).
//
// Layouts.  Every pass walks a layout whose innermost dimension is a
// cross-section dimension.  Passes along the last (contiguous) axis W use a
// transposed copy: 2D [W][H], 3D [W][D][H].  The image is transposed once per
// call; distance maps change layout inside the passes that border the W
// passes (H backward writes the transposed layout, W backward writes the
// original one back), so the layout changes cost no extra memory traffic.
//
// Tiles.  A pass cuts its cross-section into tiles, one CTA each, launched
// cooperatively (all resident).  The planner picks tile extents, halo and
// chunk length from a small cost model of one step.

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

#include "fg_batch3d.cuh"
#include "fg_common.cuh"

namespace fgi {

thread_local std::string g_err;

int set_error(int code, const char *msg) {
  g_err = msg;
  return code;
}

}  // namespace fgi

namespace {

using namespace fgi;

constexpr size_t kSmemBudget = 227 * 1024 - 1024;
constexpr size_t kWsHeader = 256;  // status word and spare

int fail(int code, const std::string &msg) { return set_error(code, msg.c_str()); }

#define FG_CUDA(call)                                                                                      \
  do {                                                                                                     \
    cudaError_t e_ = (call);                                                                               \
    if (e_ != cudaSuccess) return fail(FG_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_));   \
  } while (0)

// ---------------------------------------------------------------------------
// elementwise kernels: initial distances, transposes, signed / GSF combinations
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

// out = x - y
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

// Image to the layout of the W passes: src [C][D][H][W] -> dst [C][W][D][H]
// (D == 1 for 2D images).  32x32 tiles through shared memory.
__global__ void fg_transpose_kernel(const float *src, float *dst, int D, int H, int W) {
  __shared__ float tile[32][33];
  const int cd = blockIdx.z;  // channel * D + d
  const int c = cd / D, d = cd - c * D;
  const long long P = (long long)D * H * W;
  const float *s = src + c * P + (long long)d * H * W;
  float *o = dst + c * P + (long long)d * H;
  const int w0 = blockIdx.x * 32, h0 = blockIdx.y * 32;
  for (int y = threadIdx.y; y < 32; y += blockDim.y) {
    int h = h0 + y, w = w0 + threadIdx.x;
    if (h < H && w < W) tile[y][threadIdx.x] = s[(long long)h * W + w];
  }
  __syncthreads();
  for (int y = threadIdx.y; y < 32; y += blockDim.y) {
    int w = w0 + y, h = h0 + threadIdx.x;
    if (h < H && w < W) o[(long long)w * D * H + h] = tile[threadIdx.x][y];
  }
}

// A row-major rows x cols matrix to its transpose (dst[c][r] = src[r][c]):
// a map between the original layout [D][H][W] = [(D H)][W] and the layout of
// the W passes [W][D][H] = [W][(D H)] (2D: [H][W] and [W][H]).  32x32 tiles
// through shared memory, full 128-byte lines read and written; one block per
// tile on a 1D grid (rows / 32 may exceed a grid's y extent).
__global__ void fg_transpose2d_kernel(const float *__restrict__ src, float *__restrict__ dst, long long rows,
                                      int cols) {
  __shared__ float tile[32][33];
  const long long tc = (cols + 31) / 32;
  const long long b = blockIdx.x;
  const long long r0 = (b / tc) * 32;
  const int c0 = (int)(b % tc) * 32;
  for (int y = threadIdx.y; y < 32; y += blockDim.y) {
    const long long r = r0 + y;
    const int c = c0 + threadIdx.x;
    if (r < rows && c < cols) tile[y][threadIdx.x] = src[r * cols + c];
  }
  __syncthreads();
  for (int y = threadIdx.y; y < 32; y += blockDim.y) {
    const int c = c0 + y;
    const long long r = r0 + threadIdx.x;
    if (r < rows && c < cols) dst[(long long)c * rows + r] = tile[threadIdx.x][y];
  }
}

dim3 ew_grid(long long n) {
  long long b = (n + 255) / 256;
  return dim3((unsigned)std::min<long long>(std::max<long long>(b, 1), 152 * 16));
}

// ---------------------------------------------------------------------------
// planner
// ---------------------------------------------------------------------------

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
  int T1, T2, K1, K2, tiles1, tiles2, S, NT, B2, rowf, P;
  size_t smem;
  bool lean;     // 64-register kernel
  bool cluster;  // one thread-block cluster of tiles1 strips of whole rows (fg_pass3d_cluster.cu)
  int rpt;       // cluster plans: runs per thread of the cluster sweep kernel (0: the pass kernel)
  bool chunked = false;  // one ordinary launch per chunk of S steps, any number of tiles
  bool rowtile = false;  // 2D: the row-tile kernel (fg_rowtile2d.cu), one thread per cell of a tile and its halos
  bool rowcl = false;    // row tiles of one thread-block cluster, handing over through distributed shared memory
};

std::atomic<int> g_tune_region{kMaxRegion};  // largest per-CTA region (cells) the planner may use
std::atomic<int> g_tune_tiles{0};            // cap on tiles per pass (0: the SM count)

// Cost model of one step of a pass in SM cycles, fitted to single-tile and
// multi-tile step times measured on GB300 (256^3 and 64^2 x 256 sweeps): a
// fixed dependency chain, issue time per 4-cell run of the step's cone
// (averaged over a chunk, whole warps), and the neighbour hand-off of a
// multi-tile plan (an L2 round trip, longer with more tiles) spread over the
// S steps of a chunk.
constexpr double kStepBase = 620.0, kCyclesPerRunGeneral = 2.4, kCyclesPerRunEuclid = 1.3;
constexpr double kHandoffBase = 2000.0, kHandoffPerTile = 8.0;
// Chunked plans: a launch's start-up (launch latency, prefetch and the
// previous row's exchange words) in the same cycles, and the shared memory of an SM.
constexpr double kChunkLaunch = 12000.0;
constexpr size_t kSmemPerSm = 228 * 1024;

// Runs computed per step, averaged over the S steps of a chunk and rounded up
// to whole warps: the kernel orders runs innermost first and skips, at chunk
// step j, the runs whose cone distance is <= j (run_cone_dist in the kernel).
double cone_avg_runs(int cross, int R1, int R2, int K1, int K2, int S) {
  const int rpr = (R2 + 3) / 4, nruns = R1 * rpr;
  int count[33] = {0};  // runs by cone distance 0 .. S (S <= 32)
  for (int q = 0; q < nruns; q++) {
    const int r1 = q / rpr, u = q % rpr;
    const int d1 = (cross == 2 && K1 > 0) ? std::min(r1, R1 - 1 - r1) : S;
    int d = -1;
    for (int i = 0; i < 4; i++) {
      const int r2 = 4 * u + i;
      if (r2 < R2) d = std::max(d, std::min(d1, K2 > 0 ? std::min(r2, R2 - 1 - r2) : S));
    }
    count[std::min(d, S)]++;
  }
  double sum = 0.0;
  int active = nruns;  // runs with distance > j
  for (int j = 0; j < S; j++) {
    active -= count[j];
    sum += (double)((active + 31) / 32 * 32);
  }
  return sum / S;
}

// Whether an image of H x W takes the one-launch path (launch_image_one):
// small enough, and no plan pinned or planner limit set for its passes (so
// that fg_plan_override and fg_set_tuning still reach the pass kernel).
bool one_launch_image(int H, int W);

// Plan overrides set by the autotuner (fg_plan_override): (cross-section
// shape, mode key) -> (S, T1, T2, flags); flags: FG_PLAN_LEAN, FG_PLAN_CLUSTER,
// FG_PLAN_RUNS2.  Mode key 0 applies to every arithmetic mode, 1 + mode to
// that mode only (and wins over key 0).
std::mutex g_override_mu;
std::map<std::tuple<int, int, int, int>, std::tuple<int, int, int, int>> g_overrides;

bool has_override(int cross, int N1, int N2) {  // under g_override_mu
  for (int k = 0; k <= 3; k++)
    if (g_overrides.find(std::make_tuple(cross, N1, N2, k)) != g_overrides.end()) return true;
  return false;
}

// A cluster plan for a volume pass: ceil(N1 / T1) strips of T1 whole rows,
// one CTA each, 2 to 16 CTAs in one cluster.  Its passes write in place (a
// pass that changes layout is followed by a transpose: the pass generator
// splits it), so `wt` and S play no part; the staging depth is the largest
// that fits one CTA per SM.  rpt = 2: the cluster sweep kernel, 2 vertically
// adjacent runs per thread (T1 rounded up to an even number, at most 512
// threads, at most one image channel read); rpt = 0: the pass kernel, one
// run per thread.
bool cluster_plan(int N1, int N2, int C, int M, int mode, bool wt, int S, int T1, int rpt, bool want_lean, Plan *out) {
  (void)wt;
  (void)S;
  const int cimg = mode == MODE_EUCLID ? 0 : C;
  if (rpt != 0 && (cimg > 1 || rpt != 2)) return false;
  if (cimg > kMaxChannels) return false;  // wide images run on tile plans
  const int step = std::max(rpt, 1);
  T1 = std::max(1, std::min(T1, N1));
  T1 = (T1 + step - 1) / step * step;
  const int G = (N1 + T1 - 1) / T1;
  if (G < 2 || G > kMaxCluster) return false;
  const int rpr = (N2 + 3) / 4;
  const int nt = std::max(32, ((T1 + step - 1) / step * rpr + 31) / 32 * 32);
  if (nt > (rpt ? kThreads : pass_max_threads(2, cimg, M))) return false;
  const bool lean = rpt == 0 && (nt > kThreads || (want_lean && pass_lean(2, cimg, M)));
  const int nch = mode == MODE_EUCLID ? 0 : (C == 1 ? 1 : kMaxChannels);
  for (int depth = max_pass_depth(nch, M); depth >= 2; depth /= 2) {
    int B2, rowf, nown;
    size_t sm;
    if (rpt) {
      const ClusterLayout ly = cluster_layout(cimg, M, T1, N2, nt, rpt, depth);
      sm = (size_t)ly.bytes;
      B2 = ly.B2;
      rowf = ly.rowf;
    } else {
      sm = pass_smem_bytes(2, C, M, mode, false, 2, T1, N2, &B2, &rowf, &nown, depth);
    }
    if (sm <= kSmemBudget) {
      *out = Plan{T1, N2, 0, 0, G, 1, 8, nt, B2, rowf, depth, sm, lean, true, rpt};
      return true;
    }
  }
  return false;
}
std::atomic<unsigned> g_plan_epoch{0};  // bumped when overrides change: older cache entries are stale

// Measured on GB300 (iterations 2, lamb 1, through the public call): one
// CTA in one launch 0.28 / 0.55 / 0.87 / 1.23 ms at 128 / 256 / 384 / 512
// per side, per-pass launches on 32-cell row tiles 0.27 / 0.47 / 0.68 / 0.88
// (global hand-offs, layout changes written by the passes); with clustered
// row tiles the one launch still won on 64^2 (0.158 against 0.170 ms), 96^2
// (0.215 / 0.217) and 64 x 200 (0.261 / 0.269), and lost on 120 x 300 (0.425
// / 0.396), 64 x 512 (0.522 / 0.478) and 100 x 512 (0.664 / 0.528).
bool one_launch_image(int H, int W) {
  if (std::max(H, W) > kOneLaunchSide || (long long)H * W >= kOneLaunchCells || g_tune_region.load() < kMaxRegion ||
      g_tune_tiles.load() > 0)
    return false;
  std::lock_guard<std::mutex> g(g_override_mu);
  return !has_override(1, 1, W) && !has_override(1, 1, H);
}

bool make_plan(int cross, int N1, int N2, int C, int M, int mode, bool wt, int max_tiles, Plan *out) {
  static std::mutex mu;
  static std::map<std::tuple<int, int, int, int, int, int, bool, int, int, unsigned>, Plan> cache;
  const int max_region = g_tune_region.load();
  if (g_tune_tiles.load() > 0) max_tiles = std::min(max_tiles, g_tune_tiles.load());
  auto key = std::make_tuple(cross, N1, N2, C, M, mode, wt, max_tiles, max_region, g_plan_epoch.load());
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
  const int max_threads = pass_max_threads(cross, mode == MODE_EUCLID ? 0 : C, M);
  const bool lean_capable = pass_lean(cross, mode == MODE_EUCLID ? 0 : C, M);
  // returns 1 if the plan is valid, 0 if not, -1 if it is too large (so is every larger T1)
  auto consider = [&](int S, int T1, int T2, int t1, int t2, bool want_lean, bool chunked = false) -> int {
    const bool multi = t1 * t2 > 1;
    int K1 = (cross == 2 && t1 > 1) ? S : 0, K2 = t2 > 1 ? S : 0;
    if ((t1 > 1 && T1 < K1) || (t2 > 1 && T2 < K2)) return 0;
    if (t2 > 1 && T2 % 4) return 0;  // runs of 4 must not straddle tiles
    int R1 = cross == 2 ? T1 + 2 * K1 : 1, R2 = T2 + 2 * K2;
    if ((long long)R1 * R2 > std::min(max_region, 4 * max_threads)) return -1;
    int runs = R1 * ((R2 + 3) / 4);
    if (runs > max_threads) return -1;
    int B2, rowf, nown;
    // image channels staged per step (wide images: none, they are read through L1)
    const int nch = mode == MODE_EUCLID || C > kMaxChannels ? 0 : (C == 1 ? 1 : kMaxChannels);
    // deepest staging that still leaves room for a second CTA on the SM (then
    // concurrent transforms on other streams share its issue slots)
    int depth = max_pass_depth(nch, M);
    size_t sm = pass_smem_bytes(cross, C, M, mode, wt, S, R1, R2, &B2, &rowf, &nown, depth);
    while (depth > 2 && sm > kSmemBudget / 2) {
      depth /= 2;
      sm = pass_smem_bytes(cross, C, M, mode, wt, S, R1, R2, &B2, &rowf, &nown, depth);
    }
    (void)nown;
    if (sm > kSmemBudget) return -1;
    // a 2D step has 3 candidates per cell instead of 9
    const double per_run = (mode == MODE_EUCLID ? kCyclesPerRunEuclid
                                                : (kCyclesPerRunGeneral + 0.8 * (C - 1)) * (M == 2 ? 1.8 : 1.0)) /
                           (cross == 2 ? 1.0 : 3.0);
    const double avg_runs = multi ? cone_avg_runs(cross, R1, R2, K1, K2, S) : (double)((runs + 31) / 32 * 32);
    double cost = kStepBase + per_run * avg_runs + (multi ? (kHandoffBase + kHandoffPerTile * t1 * t2) / S : 0.0);
    const int nt = std::max(32, std::min(max_threads, (runs + 31) / 32 * 32));
    const bool lean = nt > kThreads || (want_lean && lean_capable);
    if (lean) cost += 0.13 * per_run * avg_runs;  // the 64-register kernel's extra instructions
    // one CTA per SM (shared memory or registers): no room for a concurrent transform
    if (sm > kSmemBudget / 2 || nt > kThreads) cost *= 1.05;
    if (chunked) {
      // tiles run in waves of the CTAs the SMs hold at once (max_tiles is the
      // SM count here); each launch's start-up is spread over its S steps
      const int per_sm = (int)std::max<size_t>(1, std::min<size_t>(kSmemPerSm / (sm + 1024), 2048 / nt));
      const long long slots = (long long)max_tiles * per_sm, tiles = (long long)t1 * t2;
      const long long waves = (tiles + slots - 1) / slots;
      const double conc = (double)std::min<long long>(per_sm, (tiles + max_tiles - 1) / max_tiles);
      cost = (double)waves * std::max(kStepBase, conc * per_run * avg_runs * (lean ? 1.13 : 1.0)) + kChunkLaunch / S;
    }
    if (!found || cost < best_cost - 1e-9) {
      best = Plan{T1, T2, K1, K2, t1, t2, S, nt, B2, rowf, depth, sm, lean, false, 0, chunked && multi};
      best_cost = cost;
      found = true;
    }
    return 1;
  };
  int ovS = 0, ovT1 = 0, ovT2 = 0, ovLean = 0;
  {
    std::lock_guard<std::mutex> g(g_override_mu);
    auto it = g_overrides.find(std::make_tuple(cross, N1, N2, 1 + mode));
    if (it == g_overrides.end()) it = g_overrides.find(std::make_tuple(cross, N1, N2, 0));
    if (it != g_overrides.end()) std::tie(ovS, ovT1, ovT2, ovLean) = it->second;
  }
  // a 2D tile plan on the row-tile kernel: one thread per cell of the tile and
  // its halos (at most 512), images of 1 to 4 channels read
  auto to_row_tiles = [&](Plan &p, bool clu) {
    const int R = p.T2 + 2 * p.K2;
    if (cross != 1 || p.chunked || C > kMaxChannels || R > 512) return false;  // one tile: no halos, no hand-off
    p.rowtile = true;
    p.rowcl = clu && p.tiles2 <= kMaxCluster && p.K2 == p.S && p.K2 <= p.T2;
    p.NT = (R + 31) / 32 * 32;
    p.rowf = ring_pitch(R + 2);
    p.smem = row_tile_smem(C, M, R, p.S, p.rowcl);
    p.lean = false;
    return true;
  };
  if (ovS > 0 && (ovLean & FG_PLAN_CLUSTER) && cross == 2) {
    Plan cp;
    const int rpt = (ovLean & FG_PLAN_RUNS2) ? 2 : 0;
    if (cluster_plan(N1, N2, C, M, mode, wt, ovS, ovT1, rpt, (ovLean & FG_PLAN_LEAN) != 0, &cp)) {
      best = cp;
      found = true;
    }
  } else if (ovS > 0) {
    const int T1 = cross == 2 ? std::min(ovT1, N1) : 1, T2 = std::min(ovT2, N2);
    const int t1 = (N1 + T1 - 1) / T1, t2 = (N2 + T2 - 1) / T2;
    const bool chunked = (ovLean & FG_PLAN_CHUNKED) != 0;
    if (chunked || (long long)t1 * t2 <= max_tiles) consider(ovS, T1, T2, t1, t2, (ovLean & FG_PLAN_LEAN) != 0, chunked);
    if (found && (ovLean & FG_PLAN_ROWS)) to_row_tiles(best, (ovLean & FG_PLAN_CLUSTER) != 0);
  }
  // 2D passes of 1 to 4 image channels run on row tiles: one thread per cell
  // and a hand-off every 32 steps (halos of 32 cells: a row's halo is only
  // its two ends).  Measured on GB300 (images of 64 x 512 to 8192^2, lamb 0.5
  // and 1): S = 32 was the fastest period (11-20% ahead of S = 8 on the pass
  // kernel's tiles) and the row-tile kernel with narrow tiles the fastest
  // form (4096^2: 18.3 ms on the cost model's plan, 13.0 on the pass
  // kernel's 128-cell tiles, 7.85 on 32-cell row tiles); on rows of 16 to 256
  // cells (3000 steps, iterations 2) the pass kernel's plan took 4.0-4.8 ms
  // and row tiles 2.1-2.4.
  //   * Rows of up to 32 cells: one tile of the whole row (no hand-off).
  //   * Up to 1024 cells: one thread-block cluster of at most 16 tiles (32
  //     cells up to 512, else 64) handing over through distributed shared
  //     memory: 5-7% faster than the same tiles handing over through global
  //     memory (512^2: 0.877 -> 0.826 ms plain, 1.015 -> 0.946 signed;
  //     1024^2: 1.710 ms on 32 tiles of 32 -> 1.638 on 16 tiles of 64).
  //   * Longer rows: the narrowest of 32, 64 or 128 cells that the SMs hold,
  //     handing over through global memory (2048^2 on a cluster of 16 tiles
  //     of 128 took 3.458 ms against 3.356 on 64 tiles of 32).
  // Images of more than 4 channels take the pass kernel (on 128-cell tiles
  // for rows of more than 512 cells).
  if (!found && cross == 1 && N2 <= 32) {
    consider(32, 1, N2, 1, 1, false);
    if (found && !to_row_tiles(best, false)) found = false;
  }
  if (!found && cross == 1 && N2 > 32 && N2 <= 2 * 32 * kMaxCluster) {
    const int T2 = N2 <= 32 * kMaxCluster ? 32 : 64, t2 = (N2 + T2 - 1) / T2;
    if (t2 <= max_tiles) {
      consider(32, 1, T2, 1, t2, false);
      if (found && !(to_row_tiles(best, true) && best.rowcl)) found = false;
    }
  }
  if (!found && cross == 1 && N2 > 32 && (C <= kMaxChannels || N2 > 512)) {
    for (int T2 : {32, 64, 128}) {
      if ((N2 + T2 - 1) / T2 > max_tiles) continue;
      consider(32, 1, T2, 1, (N2 + T2 - 1) / T2, false);
      if (found && !to_row_tiles(best, false) && T2 < 128) found = false;  // narrow tiles only as row tiles
      if (found) break;
    }
  }
  for (int S : {8, 4, 2, 1}) {
    if (found) break;  // an override that fits wins
    if (cross == 1) {
      for (int tiles2 = 1; tiles2 <= max_tiles; tiles2++) {
        int T2 = (N2 + tiles2 - 1) / tiles2;
        if (tiles2 > 1) T2 = (T2 + 3) & ~3;
        int t2 = (N2 + T2 - 1) / T2;
        if (tiles2 > 1 && t2 != tiles2) continue;
        consider(S, 1, T2, 1, t2, false);
        if (T2 <= 4) break;
      }
    } else {
      for (int T2 = std::min(N2, 4);; T2 = std::min(N2, T2 + 4)) {
        int t2 = (N2 + T2 - 1) / T2;
        for (int T1 = 1; T1 <= N1; T1++) {
          int t1 = (N1 + T1 - 1) / T1;
          if ((long long)t1 * t2 > max_tiles) continue;
          if (consider(S, T1, T2, t1, t2, false) != 0) break;  // larger T1 only grows the region
        }
        if (T2 >= N2) break;
      }
    }
  }
  // No plan whose tiles are all resident at once (a cross-section larger than
  // the SMs' regions): a chunked plan, one ordinary launch per chunk of S
  // steps over as many tiles as it takes.  Volumes: for each tile width, the
  // tallest tile that fits, evened out over the cross-section; rows: the
  // longest tile, evened out.
  const bool need_chunks = !found;
  const int lim = std::min(max_region, 4 * max_threads);
  for (int S : {8, 4, 2}) {
    if (!need_chunks) break;
    if (cross == 1) {
      int T2 = std::min(lim, 4 * max_threads) - 2 * S;
      T2 &= ~3;
      if (T2 < S || T2 >= N2) continue;
      const int t2 = (N2 + T2 - 1) / T2;
      T2 = (((N2 + t2 - 1) / t2) + 3) & ~3;
      consider(S, 1, T2, 1, (N2 + T2 - 1) / T2, false, true);
      continue;
    }
    for (int T2 = std::min(N2, 4);; T2 = std::min(N2, T2 + 4)) {
      const int t2 = (N2 + T2 - 1) / T2, K2 = t2 > 1 ? S : 0, R2 = T2 + 2 * K2;
      const int R1max = std::min(lim / R2, max_threads / ((R2 + 3) / 4));
      int T1 = N1;
      if (R1max < N1) {
        const int T1max = R1max - 2 * S;
        T1 = T1max >= S ? (N1 + (N1 + T1max - 1) / T1max - 1) / ((N1 + T1max - 1) / T1max) : 0;
      }
      if (T1 > 0 && (long long)((N1 + T1 - 1) / T1) * t2 > 1) consider(S, T1, T2, (N1 + T1 - 1) / T1, t2, false, true);
      if (T2 >= N2) break;
    }
  }
  if (found) {
    std::lock_guard<std::mutex> g(mu);
    cache[key] = best;
    *out = best;
    static const bool debug = getenv("FASTGEODIS_GB300_DEBUG_PLAN") != nullptr;
    if (debug)
      fprintf(stderr,
              "[fg plan] cross=%d N=%dx%d C=%d M=%d mode=%d wt=%d -> T=%dx%d K=%d,%d tiles=%dx%d S=%d NT=%d "
              "P=%d smem=%zu lean=%d cluster=%d chunked=%d cost=%.0f\n",
              cross, N1, N2, C, M, mode, (int)wt, best.T1, best.T2, best.K1, best.K2, best.tiles1, best.tiles2,
              best.S, best.NT, best.P, best.smem, (int)best.lean, (int)best.cluster, (int)best.chunked, best_cost);
  }
  return found;
}

// ---------------------------------------------------------------------------
// workspace
// ---------------------------------------------------------------------------

struct Workspace {
  int *status;
  unsigned long long *xch;  // halo exchange words (PassArgs::xch)
  size_t xch_bytes;
  unsigned long long *xch2;  // GSF: the words of its second map group, swept beside the first
  char *base;
  size_t map_stride;  // floats between maps
};

size_t map_bytes(long long P) { return ((size_t)P * 4 + 255) & ~(size_t)255; }

// Largest pass cross-section of a transform.  With D == 1 the sweep along D
// has one step and no tiles, so a 2D image and a one-slice volume both need
// max(H, W).
long long max_cross_cells(int D, int H, int W) {
  if (D <= 1) return std::max(H, W);
  return std::max({(long long)H * W, (long long)D * W, (long long)D * H});
}

// exchange words: 2 parities x kMaxMaps maps x the largest cross-section
size_t xch_bytes(int D, int H, int W) {
  return ((size_t)2 * kMaxMaps * max_cross_cells(D, H, W) * 8 + 255) & ~(size_t)255;
}

// extra maps in the original layout (beyond `out`), maps in the transposed
// layout, and the transposed image copy
int extra_maps(int op) { return op == FG_OP_PLAIN ? 0 : (op == FG_OP_SIGNED ? 1 : 4); }
int t_maps(int op) { return op == FG_OP_PLAIN ? 1 : (op == FG_OP_SIGNED ? 2 : 4); }

// exchange-word regions: GSF sweeps its four second-stage maps as two groups
// of two at once, each with its own words
int xch_regions(int op) { return op == FG_OP_GSF ? 2 : 1; }

size_t workspace_bytes(int op, int C, int D, int H, int W) {
  const long long P = (long long)D * H * W;
  return kWsHeader + xch_regions(op) * xch_bytes(D, H, W) + (size_t)(extra_maps(op) + t_maps(op)) * map_bytes(P) +
         map_bytes(P * C);
}

int bind_workspace(void *ws, size_t bytes, int op, int C, int D, int H, int W, Workspace *w) {
  if (ws == nullptr) return fail(FG_ERR_WORKSPACE, "workspace pointer is null");
  if ((reinterpret_cast<uintptr_t>(ws) & 255) != 0) return fail(FG_ERR_WORKSPACE, "workspace must be 256-byte aligned");
  const long long P = (long long)D * H * W;
  size_t need = workspace_bytes(op, C, D, H, W);
  if (bytes < need)
    return fail(FG_ERR_WORKSPACE, "workspace too small: need " + std::to_string(need) + " bytes, got " + std::to_string(bytes));
  char *base = static_cast<char *>(ws);
  w->status = reinterpret_cast<int *>(base);
  w->xch = reinterpret_cast<unsigned long long *>(base + kWsHeader);
  w->xch_bytes = xch_bytes(D, H, W);
  w->xch2 = xch_regions(op) > 1 ? reinterpret_cast<unsigned long long *>(base + kWsHeader + w->xch_bytes) : nullptr;
  w->base = base + kWsHeader + xch_regions(op) * w->xch_bytes;
  w->map_stride = map_bytes(P) / 4;
  return FG_OK;
}

// ---------------------------------------------------------------------------
// transforms
// ---------------------------------------------------------------------------

struct Geometry {
  bool is3d;
  int C, D, H, W;
  long long P;  // voxels per channel
  float spacing_sq[3];
};

// Maps swept together: original-layout plane and transposed-layout buffer of each.
struct MapSet {
  int M;
  float *r[4];
  float *t[4];
  float lg, le;
};

// Optional timing of pass launches with CUDA events on the launching stream
// (fg_profile_begin / fg_profile_end).
struct ProfileState {
  std::mutex mu;
  bool on = false;
  std::vector<std::pair<cudaEvent_t, cudaEvent_t>> ev;
  std::vector<long long> vp;  // cells x maps updated by each recorded launch
  std::vector<int> steps;     // pass length of each recorded launch
  std::vector<float> last_ms; // per-launch times of the last closed window
  std::vector<int> last_steps;
  int aux = 0, last_aux = 0;  // kernel launches besides one per pass (chunks after the first, map transposes)
};
ProfileState &profile() {
  static ProfileState p;
  return p;
}

std::mutex g_launch_mu;  // serialises the per-device function attribute set-up

void count_aux_launches(int n) {
  ProfileState &ps = profile();
  std::lock_guard<std::mutex> g(ps.mu);
  if (ps.on) ps.aux += n;
}

// Runs `launch` on stream s, bracketed by timing events while profiling is on;
// vp: cells x maps the launch updates, steps: its sequential steps.
template <typename Launch>
int profiled_launch(cudaStream_t s, long long vp, int steps, Launch launch) {
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
  int rc;
  {
    std::lock_guard<std::mutex> g(g_launch_mu);
    rc = launch();
  }
  if (rc != FG_OK) return rc;
  if (e0) {
    FG_CUDA(cudaEventRecord(e1, s));
    std::lock_guard<std::mutex> g(ps.mu);
    ps.ev.emplace_back(e0, e1);
    ps.vp.push_back(vp);
    ps.steps.push_back(steps);
  }
  return FG_OK;
}

int launch_pass(const PassArgs &a, const Plan &p, int cross, int M, int mode, bool wt, cudaStream_t s) {
  LaunchCfg c{p.tiles1 * p.tiles2, p.NT, p.smem, p.lean, p.rpt, p.chunked};
  return profiled_launch(s, (long long)a.L * a.N1 * a.N2 * M, a.L, [&] {
    if (p.cluster) return launch_pass_cluster(a, c, M, mode, wt, s);
    if (p.rowtile) return launch_row_tiles(a, c, M, mode, wt, p.rowcl, s);
    if (!p.chunked)
      return cross == 2 ? launch_pass_cross2(a, c, M, mode, wt, s) : launch_pass_cross1(a, c, M, mode, wt, s);
    // one ordinary launch per chunk of S steps, in stream order
    count_aux_launches((a.L + p.S - 1) / p.S - 1);
    for (int t0 = 0; t0 < a.L; t0 += p.S) {
      PassArgs b = a;
      b.t_begin = t0;
      b.t_end = std::min(a.L, t0 + p.S);
      const int rc = cross == 2 ? launch_pass_cross2(b, c, M, mode, wt, s) : launch_pass_cross1(b, c, M, mode, wt, s);
      if (rc != FG_OK) return rc;
    }
    return FG_OK;
  });
}

// The cheapest exact arithmetic for the weights: l_grad == 0 drops the image
// term, (l_eucl, l_grad) == (0, 1) drops the step-length term and the product.
int select_mode(float lg, float le) {
  if (lg == 0.0f) return MODE_EUCLID;
  if (le == 0.0f && lg == 1.0f) return MODE_GEO;
  return MODE_GENERAL;
}

// Reference step-length table of a 3D pass (fastgeodis_cpu.cpp:220-231):
// squared spacings permuted for the swept axis; index 3*i+j, i the offset
// along the reference's tensor dim 3 and j along dim 4.
void table3(float s0, float s1, float s2, float out[9]) {
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) {
      float v = s0;
      v += (float)abs(i - 1) * s1;
      v += (float)abs(j - 1) * s2;
      out[i * 3 + j] = sqrtf(v);
    }
}

// One axis of a transform in the layout its passes read.
struct Axis {
  int L;
  long long s_str, st1;  // read strides (cross 2 has stride 1)
  int N1, N2;
  bool transposed;       // reads the [W]-major layout
  float ld[9];           // step lengths in the engine's neighbour numbering (n = 3*(d1+1) + (d2+1))
};

void axes_for(const Geometry &g, Axis *ax, int *nax) {
  if (!g.is3d) {
    const float r2 = (float)sqrt(2.0);  // fastgeodis_cpu.cpp:67
    ax[0] = Axis{g.H, g.W, 0, 1, g.W, false, {r2, 1.0f, r2}};  // along H over [H][W]
    ax[1] = Axis{g.W, g.H, 0, 1, g.H, true, {r2, 1.0f, r2}};   // along W over [W][H]
    *nax = 2;
    return;
  }
  const float *s = g.spacing_sq;
  const long long HW = (long long)g.H * g.W, DH = (long long)g.D * g.H;
  // along D over [D][H][W]: cross (h, w), the reference's dims (H, W)
  ax[0] = Axis{g.D, HW, g.W, g.H, g.W, false, {}};
  table3(s[0], s[1], s[2], ax[0].ld);
  // along H over [D][H][W]: cross (d, w); the reference transposes to [H, D, W]
  ax[1] = Axis{g.H, g.W, HW, g.D, g.W, false, {}};
  table3(s[1], s[0], s[2], ax[1].ld);
  // along W over [W][D][H]: cross (d, h); the reference transposes to [W, H, D],
  // whose i runs over h (the engine's cross 2) and j over d (cross 1)
  ax[2] = Axis{g.W, DH, g.H, g.D, g.H, true, {}};
  float t[9];
  table3(s[2], s[1], s[0], t);
  for (int d1 = 0; d1 < 3; d1++)
    for (int d2 = 0; d2 < 3; d2++) ax[2].ld[d1 * 3 + d2] = t[d2 * 3 + d1];
  *nax = 3;
}

// The pass sequence of `iterations` iterations on the maps of `ms`, whose
// original-layout planes hold the initial distances (img_r / img_t: the image
// in the original and the transposed layout), in launch order: for each pass
// and group of at most kMaxMaps maps, `plan_fn(cross, N1, N2, Cimg, M, mode,
// wt, &plan)` picks the plan and `emit(args, plan, cross, M, mode, wt)` gets
// the pass's arguments (all but the halo exchange fields).  Returns the first
// non-FG_OK code of either.
//
// A pass that changes layout on a cluster plan (a strip of whole rows per
// SM, thousands of own cells) would write S-element segments of every own
// cell at each flush, one memory transaction each: measured, that doubles
// the pass; on row tiles the transposed flush at chunk ends cost 5-7% of a
// 2D transform.  (Volume tile plans keep their own flush: splitting them
// too took the 128 x 256^2 three-transform step from 6.3 to 6.6 ms and
// 256^3 from 14.3 to 14.6 ms.)  With `emit_t` such a pass writes in place and
// `emit_t(src, dst, rows, cols)` then transposes each map (a rows x cols
// matrix) into the other layout at full-line width.  Without it (nullptr)
// every pass writes its own layout change (row tiles then refuse the pass).
template <typename PlanFn, typename Emit, typename EmitT>
int for_each_pass(const Geometry &g, const float *img_r, const float *img_t, const MapSet &ms, int iterations,
                  PlanFn plan_fn, Emit emit, EmitT *emit_t) {
  if (g.P == 0 || iterations <= 0) return FG_OK;
  Axis ax[3];
  int nax = 0;
  axes_for(g, ax, &nax);
  const int cross = g.is3d ? 2 : 1;
  const int mode = select_mode(ms.lg, ms.le);
  const int Cimg = mode == MODE_EUCLID ? 0 : g.C;  // any count: above kMaxChannels the wide pass variant
  const long long HW = (long long)g.H * g.W, DH = (long long)g.D * g.H;
  for (int it = 0; it < iterations; it++) {
    for (int k = 0; k < nax; k++) {
      const Axis &A = ax[k];
      for (int dir : {1, -1}) {
        // the pass that hands over to the W passes writes transposed, and the
        // last W pass writes back; a pass of one step only moves data
        const bool to_t = (k == nax - 2) && dir < 0;
        const bool to_r = A.transposed && dir < 0;
        const bool wt = to_t || to_r;
        if (A.L <= 1 && !wt) continue;
        for (int m0 = 0; m0 < ms.M; m0 += kMaxMaps) {
          const int M = std::min(kMaxMaps, ms.M - m0);
          Plan p;
          int rc = plan_fn(cross, A.N1, A.N2, Cimg, M, mode, wt, &p);
          if (rc != FG_OK) return rc;
          const bool split = wt && emit_t != nullptr && (p.cluster || p.rowtile);  // in place, then a transpose
          if (split) {
            rc = plan_fn(cross, A.N1, A.N2, Cimg, M, mode, false, &p);
            if (rc != FG_OK) return rc;
          }
          const bool pwt = wt && !split;  // this launch changes layout itself
          PassArgs a{};
          a.img = A.transposed ? img_t : img_r;
          a.img_cs = g.P;
          a.C = g.C;
          for (int m = 0; m < M; m++) {
            float *rbuf = ms.r[m0 + m], *tbuf = ms.t[m0 + m];
            a.dsrc[m] = A.transposed ? tbuf : rbuf;
            a.ddst[m] = pwt ? (to_t ? tbuf : rbuf) : const_cast<float *>(a.dsrc[m]);
            a.lg[m] = ms.lg;
            for (int n = 0; n < 9; n++) a.e[m][n] = ms.le * A.ld[n];
          }
          a.L = A.L;
          a.dir = dir;
          a.s_str = A.s_str;
          a.st1 = A.st1;
          a.N1 = A.N1;
          a.N2 = A.N2;
          if (!pwt) {
            a.ws_str = A.s_str;
            a.wst1 = A.st1;
            a.wst2 = 1;
          } else if (to_t) {  // write [W][H] / [W][D][H]: element (step, c1, c2 = w)
            a.ws_str = 1;
            a.wst1 = g.is3d ? g.H : 0;
            a.wst2 = g.is3d ? DH : g.H;
          } else if (to_r) {  // write [H][W] / [D][H][W]: element (step = w, c1 = d, c2 = h)
            a.ws_str = 1;
            a.wst1 = g.is3d ? HW : 0;
            a.wst2 = g.W;
          } else {
            a.ws_str = A.s_str;
            a.wst1 = A.st1;
            a.wst2 = 1;
          }
          a.T1 = p.T1;
          a.T2 = p.T2;
          a.K1 = p.K1;
          a.K2 = p.K2;
          a.tiles1 = p.tiles1;
          a.tiles2 = p.tiles2;
          a.S = p.S;
          a.B2 = p.B2;
          a.rowf = p.rowf;
          bool vec = A.N2 % 4 == 0 && p.T2 % 4 == 0 && p.K2 % 4 == 0 && A.s_str % 4 == 0 && A.st1 % 4 == 0 &&
                     g.P % 4 == 0 && (reinterpret_cast<uintptr_t>(a.img) & 15) == 0;
          for (int m = 0; m < M; m++)
            vec = vec && (reinterpret_cast<uintptr_t>(a.dsrc[m]) & 15) == 0 &&
                  (reinterpret_cast<uintptr_t>(a.ddst[m]) & 15) == 0;
          a.vec = vec ? 1 : 0;
          a.P = p.P;
          a.wt = pwt ? 1 : 0;
          rc = emit(a, p, cross, M, mode, pwt);
          if (rc != FG_OK) return rc;
          if (split) {
            // [(D H)][W] -> [W][(D H)] after the pass that hands over to the W
            // passes, back after the last W pass (2D: [H][W] and [W][H])
            const long long DHr = g.is3d ? DH : g.H;
            for (int m = 0; m < M; m++) {
              rc = to_t ? (*emit_t)(ms.r[m0 + m], ms.t[m0 + m], DHr, g.W)
                        : (*emit_t)(ms.t[m0 + m], ms.r[m0 + m], (long long)g.W, DHr);
              if (rc != FG_OK) return rc;
            }
          }
        }
      }
    }
  }
  return FG_OK;
}

// Runs `iterations` of the full pass sequence on the maps of `ms`, one launch
// per pass on the planner's tiles (or a pinned plan).
int run_transform(const Geometry &g, const float *img_r, const float *img_t, const MapSet &ms, int iterations,
                  Workspace &w, unsigned *launch_counter, cudaStream_t s) {
  if (g.P == 0 || iterations <= 0) return FG_OK;
  DeviceInfo di = device_info();
  if (!di.ok) return fail(FG_ERR_CUDA, "cannot query the current CUDA device");
  auto plan_fn = [&](int cross, int N1, int N2, int Cimg, int M, int mode, bool wt, Plan *p) {
    if (!make_plan(cross, N1, N2, Cimg, M, mode, wt, std::min(di.sms, kMaxTiles), p))
      return fail(FG_ERR_UNSUPPORTED, "no tiling for a cross-section of " + std::to_string(N1) + "x" +
                                          std::to_string(N2));
    return FG_OK;
  };
  auto emit = [&](PassArgs &a, const Plan &p, int cross, int M, int mode, bool wt) {
    // chunk epochs of this pass: base + 1 ... base + L/S; a pass of 65536 or
    // more chunks takes as many counter values as its epochs need, so no two
    // passes of the call share an epoch
    const unsigned slots = (unsigned)(((long long)a.L + a.S - 1) / a.S / 65536) + 1;
    if (*launch_counter + slots > 0xFFFFu) {  // epochs would repeat: clear the exchange words
      FG_CUDA(cudaMemsetAsync(w.xch, 0, w.xch_bytes, s));
      *launch_counter = 0;
    }
    a.xch = w.xch;
    a.epoch_base = (*launch_counter) << 16;
    a.status = w.status;
    *launch_counter += slots;
    return launch_pass(a, p, cross, M, mode, wt, s);
  };
  auto emit_t = [&](const float *src, float *dst, long long rows, long long cols) {
    const long long tiles = ((rows + 31) / 32) * ((cols + 31) / 32);
    fg_transpose2d_kernel<<<dim3((unsigned)tiles), dim3(32, 8), 0, s>>>(src, dst, rows, (int)cols);
    FG_CUDA(cudaGetLastError());
    count_aux_launches(1);
    return FG_OK;
  };
  return for_each_pass(g, img_r, img_t, ms, iterations, plan_fn, emit, &emit_t);
}

int check_common(const float *image, int C, int D, int H, int W, const float *mask, int Cm, const float *out) {
  if (C < 1 || Cm < 1) return fail(FG_ERR_INVALID_ARGUMENT, "channel counts must be at least 1");
  if (D < 0 || H < 0 || W < 0) return fail(FG_ERR_INVALID_ARGUMENT, "negative extent");
  long long P = (long long)D * H * W;
  if (P > 0 && (!image || !mask || !out)) return fail(FG_ERR_INVALID_ARGUMENT, "null tensor pointer");
  if (P * std::max(C, Cm) >= (1LL << 31)) return fail(FG_ERR_UNSUPPORTED, "tensors of 2^31 or more elements are not supported");
  return FG_OK;
}

// Common driver for plain / signed / GSF in 2D and 3D, by the raster scan of
// fastgeodis_cpu.cpp (toivanen = false) or Toivanen's scan of
// geodis_toivanen.cpp (toivanen = true); the compositions are the same
// (FastGeodis/fastgeodis.cpp:241-258, 319-343 and :260-277, 345-369).
// A side stream of the calling host thread for work that runs beside the
// caller's stream `s` (same device and priority, non-blocking; created once
// per thread), or nullptr while `s` is being captured into a graph (the work
// then stays on `s`) or if none can be made.
cudaStream_t side_stream(cudaStream_t s) {
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(s, &cs) != cudaSuccess || cs != cudaStreamCaptureStatusNone) {
    (void)cudaGetLastError();
    return nullptr;
  }
  int dev = 0, prio = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || cudaStreamGetPriority(s, &prio) != cudaSuccess) {
    (void)cudaGetLastError();
    return nullptr;
  }
  thread_local std::map<std::pair<int, int>, cudaStream_t> streams;
  cudaStream_t &st = streams[std::make_pair(dev, prio)];
  if (st == nullptr && cudaStreamCreateWithPriority(&st, cudaStreamNonBlocking, prio) != cudaSuccess) {
    (void)cudaGetLastError();
    st = nullptr;
  }
  return st;
}

int run_op(int op, const Geometry &g, const float *image, const float *mask, int Cm, float *out, float v, float lg,
           float le, float theta, int iterations, void *ws, size_t ws_bytes, void *stream, bool toivanen = false) {
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  int rc = check_common(image, g.C, g.D, g.H, g.W, mask, Cm, out);
  if (rc != FG_OK) return rc;
  if (g.P == 0) return FG_OK;
  Workspace w;
  rc = bind_workspace(ws, ws_bytes, op, g.C, g.is3d ? g.D : 1, g.H, g.W, &w);
  if (rc != FG_OK) return rc;
  const long long P = g.P;
  const size_t ms_ = w.map_stride;
  float *maps = reinterpret_cast<float *>(w.base);
  float *xr[4] = {maps, maps + ms_, maps + 2 * ms_, maps + 3 * ms_};  // extra original-layout maps
  float *tb = maps + extra_maps(op) * ms_;
  float *xt[4] = {tb, tb + ms_, tb + 2 * ms_, tb + 3 * ms_};          // transposed-layout maps
  float *img_t = tb + t_maps(op) * ms_;
  // epoch 0 is never wanted; earlier calls' words must not match this call's epochs
  if (!toivanen) FG_CUDA(cudaMemsetAsync(w.xch, 0, w.xch_bytes, s));
  if (!toivanen && w.xch2) FG_CUDA(cudaMemsetAsync(w.xch2, 0, w.xch_bytes, s));
  unsigned counter = 0;
  // Toivanen's group barriers: 4 counters in the spare bytes of the header
  unsigned *toiv_bar = reinterpret_cast<unsigned *>(reinterpret_cast<char *>(w.status) + 64);
  auto sweep = [&](const MapSet &ms) {
    if (toivanen) {
      // one launch runs every iteration: 2 passes of D*H*W cells per map, in
      // 4(D-1) + 2(H-1) + W waves each
      const int D = g.is3d ? g.D : 1;
      const long long waves = 4LL * (D - 1) + 2LL * (g.H - 1) + g.W;
      return profiled_launch(s, 2LL * iterations * g.P * ms.M, (int)(2 * iterations * waves), [&] {
        return launch_toivanen(image, g.C, D, g.H, g.W, g.is3d ? g.spacing_sq : nullptr, ms.r, ms.M, ms.lg, ms.le,
                               iterations, toiv_bar, w.status, s);
      });
    }
    return run_transform(g, image, img_t, ms, iterations, w, &counter, s);
  };
  if (Cm > 1) {
    long long n = (long long)(Cm - 1) * P;
    fg_unswept_kernel<<<ew_grid(n), 256, 0, s>>>(out + P, mask + P, n, v, theta, op);
    FG_CUDA(cudaGetLastError());
  }
  if (!g.is3d && !toivanen && op != FG_OP_GSF && g.C <= kMaxChannels && one_launch_image(g.H, g.W)) {
    // small images: the whole transform in one launch (its CTA runs the passes
    // back to back), with the workspace's buffers as scratch
    fg_batch2d_item it{};
    it.image = image, it.mask = mask, it.out = out, it.image_t = img_t;
    it.t1 = xt[0];
    it.d2 = op == FG_OP_SIGNED ? xr[0] : nullptr;
    it.t2 = op == FG_OP_SIGNED ? xt[1] : nullptr;
    it.C = g.C, it.H = g.H, it.W = g.W;
    it.v = v, it.l_grad = lg, it.l_eucl = le;
    const int M = op == FG_OP_SIGNED ? 2 : 1;
    return profiled_launch(s, 4LL * std::max(iterations, 0) * P * M, 2 * std::max(iterations, 0) * (g.H + g.W),
                           [&] { return launch_image_one(it, op == FG_OP_SIGNED, iterations, w.status, s); });
  }
  if (iterations > 0 && !toivanen) {
    dim3 tg((g.W + 31) / 32, (g.H + 31) / 32, g.C * g.D);
    fg_transpose_kernel<<<tg, dim3(32, 8), 0, s>>>(image, img_t, g.D, g.H, g.W);
    FG_CUDA(cudaGetLastError());
  }
  if (op == FG_OP_PLAIN) {
    fg_init_kernel<<<ew_grid(P), 256, 0, s>>>(out, mask, P, v, INIT_VM);
    FG_CUDA(cudaGetLastError());
    MapSet ms{1, {out}, {xt[0]}, lg, le};
    return sweep(ms);
  }
  if (op == FG_OP_SIGNED) {
    fg_init_kernel<<<ew_grid(P), 256, 0, s>>>(out, mask, P, v, INIT_VM);
    fg_init_kernel<<<ew_grid(P), 256, 0, s>>>(xr[0], mask, P, v, INIT_V1M);
    FG_CUDA(cudaGetLastError());
    MapSet ms{2, {out, xr[0]}, {xt[0], xt[1]}, lg, le};
    rc = sweep(ms);
    if (rc != FG_OK) return rc;
    fg_sub_kernel<<<ew_grid(P), 256, 0, s>>>(out, out, xr[0], P);
    FG_CUDA(cudaGetLastError());
    return FG_OK;
  }
  // GSF: stage one is signed(mask) into (xr0, xr1); stage two sweeps four maps.
  fg_init_kernel<<<ew_grid(P), 256, 0, s>>>(xr[0], mask, P, v, INIT_VM);
  fg_init_kernel<<<ew_grid(P), 256, 0, s>>>(xr[1], mask, P, v, INIT_V1M);
  FG_CUDA(cudaGetLastError());
  {
    MapSet ms{2, {xr[0], xr[1]}, {xt[0], xt[1]}, lg, le};
    rc = sweep(ms);
    if (rc != FG_OK) return rc;
  }
  // Ds = xr0 - xr1; the four initial maps go to out, xr1, xr2, xr3
  fg_gsf_mid_kernel<<<ew_grid(P), 256, 0, s>>>(xr[0], xr[1], out, xr[1], xr[2], xr[3], P, v, theta);
  FG_CUDA(cudaGetLastError());
  cudaStream_t side = toivanen ? nullptr : side_stream(s);
  if (side) {
    // the two signed transforms of stage two at once: maps (out, xr1) on the
    // caller's stream, (xr2, xr3) on a side stream with their own exchange
    // words (a pass of a 2D image or a volume slab fills few SMs)
    MapSet ma{2, {out, xr[1]}, {xt[0], xt[1]}, lg, le};
    MapSet mb{2, {xr[2], xr[3]}, {xt[2], xt[3]}, lg, le};
    Workspace w2 = w;
    w2.xch = w.xch2;
    unsigned counter2 = 0;
    cudaEvent_t fork = nullptr, join = nullptr;
    FG_CUDA(cudaEventCreateWithFlags(&fork, cudaEventDisableTiming));
    if (cudaEventCreateWithFlags(&join, cudaEventDisableTiming) != cudaSuccess) {
      cudaEventDestroy(fork);
      return fail(FG_ERR_CUDA, cudaGetErrorString(cudaGetLastError()));
    }
    cudaError_t e = cudaEventRecord(fork, s);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(side, fork, 0);
    if (e == cudaSuccess) {
      rc = run_transform(g, image, img_t, ma, iterations, w, &counter, s);
      const int rc2 = run_transform(g, image, img_t, mb, iterations, w2, &counter2, side);
      if (rc == FG_OK) rc = rc2;
      e = cudaEventRecord(join, side);  // the caller's stream waits for the side stream's work either way
      if (e == cudaSuccess) e = cudaStreamWaitEvent(s, join, 0);
    }
    cudaEventDestroy(fork);
    cudaEventDestroy(join);
    if (e != cudaSuccess) return fail(FG_ERR_CUDA, cudaGetErrorString(e));
    if (rc != FG_OK) return rc;
  } else {
    MapSet ms{4, {out, xr[1], xr[2], xr[3]}, {xt[0], xt[1], xt[2], xt[3]}, lg, le};
    rc = sweep(ms);
    if (rc != FG_OK) return rc;
  }
  fg_gsf_final_kernel<<<ew_grid(P), 256, 0, s>>>(out, out, xr[1], xr[2], xr[3], P);
  FG_CUDA(cudaGetLastError());
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

namespace fgi {

size_t pass_smem_bytes(int cross, int C, int M, int mode, bool wt, int S, int R1, int R2, int *B2o, int *rowfo,
                       int *nown_max, int depth) {
  const int ci = mode == MODE_EUCLID || C > kMaxChannels ? 0 : C;  // image arrays staged (wide: none)
  const int B1 = cross == 2 ? R1 + 2 : 1, B2 = ((R2 + 3) & ~3) + 8;
  const int rowf = ring_pitch(B1 * B2);
  const int SR = wt ? S : 2;
  const int nt = std::max(32, (R1 * ((R2 + 3) / 4) + 31) / 32 * 32);
  *B2o = B2;
  *rowfo = rowf;
  *nown_max = R1 * R2;
  return (size_t)(SR * M + 2 * ci) * (rowf + pass_edge_floats(cross, R1, R2)) * 4 + (size_t)depth * (M + ci) * nt * 16 +
         (wt ? (size_t)R1 * R2 * 8 : 0) + 64;
}

}  // namespace fgi

extern "C" {

int fg_abi_version(void) { return FG_ABI_VERSION; }

const char *fg_last_error(void) { return fgi::g_err.c_str(); }

int fg_profile_begin(void) {
  ProfileState &ps = profile();
  std::lock_guard<std::mutex> g(ps.mu);
  for (auto &e : ps.ev) {
    cudaEventDestroy(e.first);
    cudaEventDestroy(e.second);
  }
  ps.ev.clear();
  ps.vp.clear();
  ps.steps.clear();
  ps.aux = 0;
  ps.on = true;
  return FG_OK;
}

int fg_profile_end(double *pass_ms, int *pass_launches, double *voxel_passes) {
  ProfileState &ps = profile();
  std::lock_guard<std::mutex> g(ps.mu);
  ps.on = false;
  double total = 0.0, vps = 0.0;
  int rc = FG_OK;
  ps.last_ms.clear();
  ps.last_steps = ps.steps;
  for (size_t i = 0; i < ps.ev.size(); i++) {
    float ms = 0.0f;
    if (cudaEventSynchronize(ps.ev[i].second) != cudaSuccess ||
        cudaEventElapsedTime(&ms, ps.ev[i].first, ps.ev[i].second) != cudaSuccess)
      rc = fail(FG_ERR_CUDA, "event timing failed");
    total += ms;
    ps.last_ms.push_back(ms);
    vps += (double)ps.vp[i];
    cudaEventDestroy(ps.ev[i].first);
    cudaEventDestroy(ps.ev[i].second);
  }
  if (pass_ms) *pass_ms = total;
  if (pass_launches) *pass_launches = (int)ps.ev.size();
  if (voxel_passes) *voxel_passes = vps;
  ps.ev.clear();
  ps.vp.clear();
  ps.steps.clear();
  ps.last_aux = ps.aux;
  ps.aux = 0;
  return rc;
}

int fg_profile_aux_launches(int *n) {
  if (!n) return fail(FG_ERR_INVALID_ARGUMENT, "profile query: null output");
  ProfileState &ps = profile();
  std::lock_guard<std::mutex> g(ps.mu);
  *n = ps.last_aux;
  return FG_OK;
}

int fg_profile_launch_times(float *ms, int *steps, int cap, int *n) {
  ProfileState &ps = profile();
  std::lock_guard<std::mutex> g(ps.mu);
  const int k = (int)ps.last_ms.size();
  for (int i = 0; i < k && i < cap; i++) {
    if (ms) ms[i] = ps.last_ms[i];
    if (steps) steps[i] = ps.last_steps[i];
  }
  if (n) *n = k;
  return FG_OK;
}

int fg_plan_override(int cross, int N1, int N2, int S, int T1, int T2, int lean) {
  if (cross < 1 || cross > 2 || N1 < 1 || N2 < 1) return fail(FG_ERR_INVALID_ARGUMENT, "plan override: bad shape");
  const int mkey = (lean & FG_PLAN_MODE_MASK) >> 4;  // 0: every mode, 1 + mode: that mode only
  lean &= ~FG_PLAN_MODE_MASK;
  std::lock_guard<std::mutex> g(g_override_mu);
  auto key = std::make_tuple(cross, N1, N2, mkey);
  if (S == 0) {
    g_overrides.erase(key);
  } else {
    if (S < 1 || S > 32 || (S & (S - 1)))
      return fail(FG_ERR_INVALID_ARGUMENT, "plan override: S must be a power of two up to 32");
    if (T1 < 1 || T2 < 1 || (T2 < N2 && T2 % 4)) return fail(FG_ERR_INVALID_ARGUMENT, "plan override: bad tile extents");
    const int all = FG_PLAN_LEAN | FG_PLAN_CLUSTER | FG_PLAN_RUNS2 | FG_PLAN_CHUNKED | FG_PLAN_ROWS;
    if (lean < 0 || (lean & ~all)) return fail(FG_ERR_INVALID_ARGUMENT, "plan override: bad flags");
    if ((lean & FG_PLAN_CHUNKED) && (lean & FG_PLAN_CLUSTER))
      return fail(FG_ERR_INVALID_ARGUMENT, "plan override: a chunked plan is a tile plan");
    if ((lean & FG_PLAN_ROWS) && (cross != 1 || (lean & (FG_PLAN_CHUNKED | FG_PLAN_RUNS2))))
      return fail(FG_ERR_INVALID_ARGUMENT, "plan override: row tiles are 2D tile plans");
    if ((lean & FG_PLAN_RUNS2) && !(lean & FG_PLAN_CLUSTER))
      return fail(FG_ERR_INVALID_ARGUMENT, "plan override: runs per thread apply to cluster plans");
    if ((lean & FG_PLAN_CLUSTER) && !(lean & FG_PLAN_ROWS) && (cross != 2 || S < 2))
      return fail(FG_ERR_INVALID_ARGUMENT, "plan override: cluster plans are for volume passes, with S >= 2");
    g_overrides[key] = std::make_tuple(S, T1, T2, lean);
  }
  g_plan_epoch.fetch_add(1);
  return FG_OK;
}

int fg_plan_describe(int cross, int N1, int N2, int C, int maps, int mode, int transposed_write, int sms,
                     int *plan) {
  if (cross < 1 || cross > 2 || N1 < 1 || N2 < 1 || C < 0 || maps < 1 || maps > kMaxMaps || mode < 0 || mode > 2 ||
      sms < 1 || !plan)
    return fail(FG_ERR_INVALID_ARGUMENT, "plan query: bad arguments");
  Plan p;
  const int c = mode == MODE_EUCLID ? 0 : C;
  if (!make_plan(cross, N1, N2, c, maps, mode, transposed_write != 0, std::min(sms, kMaxTiles), &p))
    return fail(FG_ERR_UNSUPPORTED, "no tiling for this cross-section");
  const int v[11] = {p.S,  p.T1, p.T2, p.K1, p.K2, p.tiles1, p.tiles2, p.NT, p.P, (int)p.smem,
                     (p.lean ? FG_PLAN_LEAN : 0) | (p.cluster ? FG_PLAN_CLUSTER : 0) |
                         (p.rpt == 2 ? FG_PLAN_RUNS2 : 0) | (p.chunked ? FG_PLAN_CHUNKED : 0) |
                         (p.rowtile ? FG_PLAN_ROWS : 0) | (p.rowcl ? FG_PLAN_CLUSTER : 0)};
  for (int i = 0; i < 11; i++) plan[i] = v[i];
  return FG_OK;
}

int fg_cluster_capacity(int cluster_size, int threads, size_t smem, int *clusters) {
  if (cluster_size < 1 || cluster_size > kMaxCluster || threads < 32 || threads > kThreads || !clusters)
    return fail(FG_ERR_INVALID_ARGUMENT, "cluster capacity: bad arguments");
  return cluster_capacity(cluster_size, threads, smem, clusters);
}

int fg_set_tuning(int max_region_cells, int max_tiles) {
  if (max_region_cells < 0 || max_region_cells > kMaxRegion || max_tiles < 0 || max_tiles > kMaxTiles)
    return fail(FG_ERR_INVALID_ARGUMENT, "tuning values out of range");
  g_tune_region.store(max_region_cells == 0 ? kMaxRegion : max_region_cells);
  g_tune_tiles.store(max_tiles);
  return FG_OK;
}

size_t fg_workspace_bytes(int op, int C, int D, int H, int W) {
  if (op < FG_OP_PLAIN || op > FG_OP_GSF || C < 1 || D < 0 || H < 0 || W < 0) return 0;
  return workspace_bytes(op, C, D, H, W);
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

// Toivanen's raster scan (FastGeodis/fastgeodis.cpp:148-177, 260-277, 345-369;
// CPU only in the reference): same arguments as the raster entries above.
int fg_generalised_geodesic2d_toivanen(const float *image, int C, int H, int W, const float *mask, int Cm, float *out,
                                       float v, float l_grad, float l_eucl, int iterations, void *workspace,
                                       size_t workspace_bytes, void *stream) {
  return run_op(FG_OP_PLAIN, geom2d(C, H, W), image, mask, Cm, out, v, l_grad, l_eucl, 0.0f, iterations, workspace,
                workspace_bytes, stream, true);
}

int fg_generalised_geodesic3d_toivanen(const float *image, int C, int D, int H, int W, const float *mask, int Cm,
                                       const float *spacing, float *out, float v, float l_grad, float l_eucl,
                                       int iterations, void *workspace, size_t workspace_bytes, void *stream) {
  Geometry g;
  int rc = geom3d(C, D, H, W, spacing, &g);
  if (rc != FG_OK) return rc;
  return run_op(FG_OP_PLAIN, g, image, mask, Cm, out, v, l_grad, l_eucl, 0.0f, iterations, workspace, workspace_bytes,
                stream, true);
}

int fg_signed_generalised_geodesic2d_toivanen(const float *image, int C, int H, int W, const float *mask, int Cm,
                                              float *out, float v, float l_grad, float l_eucl, int iterations,
                                              void *workspace, size_t workspace_bytes, void *stream) {
  return run_op(FG_OP_SIGNED, geom2d(C, H, W), image, mask, Cm, out, v, l_grad, l_eucl, 0.0f, iterations, workspace,
                workspace_bytes, stream, true);
}

int fg_signed_generalised_geodesic3d_toivanen(const float *image, int C, int D, int H, int W, const float *mask,
                                              int Cm, const float *spacing, float *out, float v, float l_grad,
                                              float l_eucl, int iterations, void *workspace, size_t workspace_bytes,
                                              void *stream) {
  Geometry g;
  int rc = geom3d(C, D, H, W, spacing, &g);
  if (rc != FG_OK) return rc;
  return run_op(FG_OP_SIGNED, g, image, mask, Cm, out, v, l_grad, l_eucl, 0.0f, iterations, workspace,
                workspace_bytes, stream, true);
}

int fg_GSF2d_toivanen(const float *image, int C, int H, int W, const float *mask, int Cm, float theta, float v,
                      float lambda, int iterations, float *out, void *workspace, size_t workspace_bytes,
                      void *stream) {
  const float le = 1.0f - lambda;  // float arithmetic, FastGeodis/fastgeodis.cpp:347
  return run_op(FG_OP_GSF, geom2d(C, H, W), image, mask, Cm, out, v, lambda, le, theta, iterations, workspace,
                workspace_bytes, stream, true);
}

int fg_GSF3d_toivanen(const float *image, int C, int D, int H, int W, const float *mask, int Cm, float theta,
                      const float *spacing, float v, float lambda, int iterations, float *out, void *workspace,
                      size_t workspace_bytes, void *stream) {
  Geometry g;
  int rc = geom3d(C, D, H, W, spacing, &g);
  if (rc != FG_OK) return rc;
  const float le = 1.0f - lambda;
  return run_op(FG_OP_GSF, g, image, mask, Cm, out, v, lambda, le, theta, iterations, workspace, workspace_bytes,
                stream, true);
}

}  // extern "C"

extern "C" {

// ---------------------------------------------------------------------------
// a batch of volumes in one persistent launch (fg_batch3d.cu)
// ---------------------------------------------------------------------------

size_t fg_batch3d_job_bytes(void) { return sizeof(fgi::Batch3dJob); }

int fg_batch3d_plan(const fg_batch3d_item *items, int n, int iterations, int cluster_size, int *status, void *jobs,
                    size_t jobs_bytes, int *info) {
  using namespace fgi;
  if (n < 0 || iterations < 0 || cluster_size < 1 || cluster_size > kMaxCluster || !info || (n > 0 && !items))
    return fail(FG_ERR_INVALID_ARGUMENT, "batch3d plan: bad arguments");
  const int G = cluster_size;
  const bool sg = n > 0 && (items[0].flags & FG_BATCH_SIGNED);
  const int M = sg ? 2 : 1;
  // the launch's arithmetic: the mode every volume shares, else the general
  // expression (exact for all of them)
  int lmode = -1;
  for (int v = 0; v < n; v++) {
    const fg_batch3d_item &it = items[v];
    if (((it.flags & FG_BATCH_SIGNED) != 0) != sg)
      return fail(FG_ERR_INVALID_ARGUMENT, "batch3d plan: every volume must be plain, or every volume signed");
    if (it.C < 1 || it.D < 1 || it.H < 1 || it.W < 1)
      return fail(FG_ERR_INVALID_ARGUMENT, "batch3d plan: volumes need at least one channel and one cell");
    if (!it.image || !it.mask || !it.out || !it.image_t || !it.t1 || (sg && (!it.d2 || !it.t2)))
      return fail(FG_ERR_INVALID_ARGUMENT, "batch3d plan: null buffer");
    const int mode = select_mode(it.l_grad, it.l_eucl);
    if (mode != MODE_EUCLID && it.C != 1)
      return fail(FG_ERR_UNSUPPORTED, "batch3d plan: volumes read at most one image channel");
    if ((long long)it.D * it.H * it.W * std::max(it.C, 1) >= (1LL << 31))
      return fail(FG_ERR_UNSUPPORTED, "batch3d plan: tensors of 2^31 or more elements are not supported");
    lmode = lmode < 0 ? mode : (lmode == mode ? mode : MODE_GENERAL);
  }
  if (lmode < 0) lmode = MODE_GENERAL;
  const int cimg = lmode == MODE_EUCLID ? 0 : 1;  // image channels the launch's body stages
  std::vector<Batch3dJob> out;
  int threads = 32;
  for (int v = 0; v < n; v++) {
    const fg_batch3d_item &it = items[v];
    Geometry g;
    int rc = geom3d(it.C, it.D, it.H, it.W, it.spacing, &g);
    if (rc != FG_OK) return rc;
    MapSet ms{M, {it.out, it.d2, nullptr, nullptr}, {it.t1, it.t2, nullptr, nullptr}, it.l_grad, it.l_eucl};
    int seq = 0;
    Batch3dJob pro{};
    pro.kind = JOB3_PROLOGUE;
    pro.vol = v;
    pro.seq = seq++;
    pro.image = it.image;
    pro.image_t = cimg ? it.image_t : nullptr;
    pro.mask = it.mask;
    pro.out = it.out;
    pro.d2 = sg ? it.d2 : nullptr;
    pro.C = it.C, pro.D = it.D, pro.H = it.H, pro.W = it.W;
    pro.v = it.v;
    pro.is_signed = sg ? 1 : 0;
    out.push_back(pro);
    auto plan_fn = [&](int, int N1, int N2, int, int, int, bool, Plan *p) {
      int T1 = (N1 + G - 1) / G;
      T1 = (T1 + 1) & ~1;  // two runs per thread: whole row pairs
      const int rpr = (N2 + 3) / 4;
      const int nt = std::max(32, ((T1 / 2) * rpr + 31) / 32 * 32);
      if (nt > kThreads)
        return fail(FG_ERR_UNSUPPORTED, "batch3d plan: a cross-section of " + std::to_string(N1) + "x" +
                                            std::to_string(N2) + " does not fit a cluster of " + std::to_string(G) +
                                            " CTAs");
      const int B2 = 4 * rpr + 8;
      *p = Plan{T1, N2, 0, 0, (N1 + T1 - 1) / T1, 1, 8, nt, B2, ring_pitch((T1 + 2) * B2), 8, 0, false, true, 2};
      threads = std::max(threads, nt);
      return FG_OK;
    };
    auto emit = [&](PassArgs &a, const Plan &, int, int, int mode, bool wt) {
      Batch3dJob j{};
      a.xch = nullptr;
      a.epoch_base = 0;
      a.status = status;
      j.a = a;
      j.kind = JOB3_PASS;
      j.mode = mode;
      j.wt = wt ? 1 : 0;
      j.vol = v;
      j.seq = seq++;
      out.push_back(j);
      return FG_OK;
    };
    auto emit_t = [&](const float *src, float *dst, long long rows, long long cols) {
      Batch3dJob j{};
      j.kind = JOB3_TRANSPOSE;
      j.vol = v;
      j.seq = seq++;
      j.tsrc = src;
      j.tdst = dst;
      j.trows = rows;
      j.tcols = (int)cols;
      out.push_back(j);
      return FG_OK;
    };
    rc = for_each_pass(g, it.image, it.image_t, ms, iterations, plan_fn, emit, &emit_t);
    if (rc != FG_OK) return rc;
    if (sg) {
      Batch3dJob epi = pro;
      epi.kind = JOB3_EPILOGUE;
      epi.seq = seq++;
      out.push_back(epi);
    }
  }
  // staging depth of each pass for the launch's CTA size (no pass writes
  // transposed: the layout changes are transpose jobs)
  size_t smem = (size_t)(threads / 32) * 32 * 33 * 4;  // a transpose tile per warp
  for (Batch3dJob &j : out) {
    if (j.kind != JOB3_PASS) continue;
    if (j.wt) return fail(FG_ERR_UNSUPPORTED, "batch3d plan: a pass writes transposed");
    PassArgs &a = j.a;
    bool fit = false;
    for (int P = 8; P >= 2 && !fit; P /= 2) {
      const ClusterLayout ly = cluster_layout(cimg, M, a.T1, a.N2, threads, 2, P);
      if ((size_t)ly.bytes <= kSmemBudget) {
        a.S = 8;
        a.P = P;
        smem = std::max(smem, (size_t)ly.bytes);
        fit = true;
      }
    }
    if (!fit) return fail(FG_ERR_UNSUPPORTED, "batch3d plan: a pass's rings do not fit the shared memory");
  }
  // queue order: by position in the chains, larger volumes first at each position
  std::stable_sort(out.begin(), out.end(), [&](const Batch3dJob &x, const Batch3dJob &y) {
    if (x.seq != y.seq) return x.seq < y.seq;
    const long long cx = (long long)items[x.vol].D * items[x.vol].H * items[x.vol].W;
    const long long cy = (long long)items[y.vol].D * items[y.vol].H * items[y.vol].W;
    if (cx != cy) return cx > cy;
    return x.vol < y.vol;
  });
  static const bool debug = getenv("FASTGEODIS_GB300_DEBUG_PLAN") != nullptr;
  if (debug)
    for (const Batch3dJob &j : out)
      fprintf(stderr, "[fg batch3d] kind=%d vol=%d seq=%d mode=%d wt=%d L=%d dir=%d N=%dx%d T1=%d tiles1=%d S=%d P=%d "
                      "s_str=%lld st1=%lld ws=%lld,%lld,%lld vec=%d transpose=%lldx%d\n",
              j.kind, j.vol, j.seq, j.mode, j.wt, j.a.L, j.a.dir, j.a.N1, j.a.N2, j.a.T1, j.a.tiles1, j.a.S, j.a.P,
              j.a.s_str, j.a.st1, j.a.ws_str, j.a.wst1, j.a.wst2, j.a.vec, j.trows, j.tcols);
  info[0] = (int)out.size();
  info[1] = threads;
  info[2] = (int)smem;
  info[3] = M;
  info[4] = lmode;
  if (out.size() * sizeof(Batch3dJob) > jobs_bytes || (!jobs && !out.empty()))
    return fail(FG_ERR_WORKSPACE, "batch3d plan: the job buffer holds " + std::to_string(jobs_bytes) +
                                      " bytes, the batch needs " + std::to_string(out.size() * sizeof(Batch3dJob)));
  if (!out.empty()) memcpy(jobs, out.data(), out.size() * sizeof(Batch3dJob));
  return FG_OK;
}

int fg_batch3d_launch(const void *jobs, int njobs, int n, int maps, int mode, int cluster_size, int threads,
                      size_t smem, unsigned *counters, int *status, void *stream) {
  if (njobs < 0 || n < 0 || (njobs > 0 && (!jobs || !counters || !status)))
    return fail(FG_ERR_INVALID_ARGUMENT, "batch3d launch: bad arguments");
  if (smem > kSmemBudget) return fail(FG_ERR_INVALID_ARGUMENT, "batch3d launch: shared memory too large");
  if (njobs == 0) return FG_OK;
  std::lock_guard<std::mutex> g(g_launch_mu);
  return fgi::launch_batch3d(static_cast<const fgi::Batch3dJob *>(jobs), njobs, n, maps, mode, cluster_size, threads,
                             smem, counters, status, static_cast<cudaStream_t>(stream));
}

int fg_batch3d_capacity(int maps, int mode, int cluster_size, int threads, size_t smem, int *clusters) {
  if (!clusters) return fail(FG_ERR_INVALID_ARGUMENT, "batch3d capacity: null output");
  std::lock_guard<std::mutex> g(g_launch_mu);
  return fgi::batch3d_capacity(maps, mode, cluster_size, threads, smem, clusters);
}

}  // extern "C"
