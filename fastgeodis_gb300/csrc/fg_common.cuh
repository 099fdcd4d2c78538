// Shared declarations of the engine's translation units.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/fastgeodis_gb300.h"

namespace fgi {

constexpr int kThreads = 512;            // largest CTA of a 128-register variant; one thread per run of 4 cells
constexpr int kThreadsLean = 1024;       // largest CTA of a 64-register ("lean") variant
constexpr int kMaxRegion = kThreadsLean * 4; // cells of one CTA's region (tile + halo), any plan

// Lean-capable variants: volume sweeps with at most one staged image channel
// and one distance map.  Besides the 128-register kernel they have a
// 64-register one (fg_pass_kernel<..., LEAN = true>), whose CTAs may have
// 1024 threads, or share an SM two at a time up to 512 threads; it executes
// about 30% more instructions (register pressure), so plans use it only for
// regions above 512 runs or when the autotuner measures it faster.  `cimg`
// is the number of image channels the pass reads (0 when l_grad == 0).
__host__ __device__ constexpr bool pass_lean(int cross, int cimg, int maps) {
  return cross == 2 && cimg <= 1 && maps == 1;
}
__host__ __device__ constexpr int pass_max_threads(int cross, int cimg, int maps) {
  return pass_lean(cross, cimg, maps) ? kThreadsLean : kThreads;
}
constexpr int kMaxMaps = 2;              // distance maps updated by one launch (they share the image)
constexpr int kMaxChannels = 4;          // image channels held in registers
constexpr int kWideChannels = -1;        // channel template argument of passes over more than kMaxChannels channels
constexpr int kMaxTiles = 2048;          // tiles of one pass (all co-resident)
constexpr int kMaxCluster = 16;          // CTAs of a cluster plan (non-portable cluster size)
constexpr unsigned kSpinLimit = 1u << 23; // polls of one halo word (each an L2 round trip, ~0.3-1 us) before FG_ERR_TIMEOUT

// Arithmetic of one candidate.  GENERAL is the reference expression
// (D + l_eucl*ld) + l_grad*L1.  EUCLID (l_grad == 0) and GEO (l_eucl == 0 and
// l_grad == 1) drop a term that is exactly +0 or a factor that is exactly 1
// for finite inputs, so they return the same bits with less work.
enum Mode { MODE_GENERAL = 0, MODE_EUCLID = 1, MODE_GEO = 2 };

// One directional pass ("sweep") over a layout whose innermost dimension is
// cross-section dimension 2 (stride 1).  Cross-section dimension 1 exists
// for volumes only (CROSS == 2).  The distance maps are read in that layout
// and written either in place or, for the pass that changes layout, in a
// layout whose innermost dimension is the swept one ("transposed write").
struct PassArgs {
  const float *img;               // image in the read layout, channel 0
  long long img_cs;               // elements between image channels
  int C;                          // image channels
  const float *dsrc[kMaxMaps];    // distance maps, read layout
  float *ddst[kMaxMaps];          // distance maps, write layout
  float lg[kMaxMaps];             // l_grad per map
  float e[kMaxMaps][9];           // l_eucl * ld[n] per map and neighbour n = 3*(d1+1) + (d2+1)
  int L, dir;                     // steps; +1 forward, -1 backward
  long long s_str, st1;           // read layout strides of a step and of cross dimension 1
  long long ws_str, wst1, wst2;   // write layout strides (step, cross 1, cross 2)
  int N1, N2;                     // cross-section extents
  int T1, T2, K1, K2;             // tile extents and halo widths
  int tiles1, tiles2;
  int S;                          // steps per chunk: halo hand-off and transposed-flush period
  int B2;                         // floats per buffer row (4-cell left apron, runs of 4, right apron)
  int rowf;                       // floats per ring row (ring_pitch: 4 mod 32)
  int vec;                        // runs may use 16-byte global loads and stores
  int P;                          // steps of own inputs staged ahead (2, 4 or 8)
  int wt;                         // the pass writes transposed (read by kernels that take it at run time)
  // Steps [t_begin, t_end) of the pass run in this launch (t_end == 0: all L).
  // A chunked plan runs one chunk of S steps per ordinary launch (t_begin a
  // multiple of S), for cross-sections whose tiles cannot all be resident at
  // once: its CTAs start from the previous row's exchange words, which the
  // launch before published, so no CTA waits on another.
  int t_begin, t_end;
  // Halo exchange between tiles: 64-bit words [2 parities][kMaxMaps][N1*N2],
  // each a cell's distance bits (low half) and the epoch of the chunk whose
  // last row it holds (high half).  One aligned 64-bit access carries both,
  // so a reader that sees the epoch it wants also sees the value.  Chunk c
  // (steps [c*S, (c+1)*S)) publishes epoch epoch_base + c + 1 at parity (c+1) & 1.
  unsigned long long *xch;
  unsigned epoch_base;
  int *status;                    // FG_ERR_TIMEOUT if a bounded wait expired
  unsigned char *tape;            // argmin tape of this pass, read layout, 1 byte per cell (TAPE variants)
};

// Argmin tape codes: 0 = the cell kept its old distance, 1 + n = it took the
// candidate of neighbour n (n = 3*(d1+1) + (d2+1); 2D: n = d2+1).
constexpr unsigned char kTapeSelf = 0;

struct LaunchCfg {
  int tiles;
  int threads;
  size_t smem;
  bool lean;  // the 64-register kernel (required above 512 threads)
  int rpt;    // cluster sweep kernel: 4-cell runs per thread (0: the pass kernel)
  bool chunked = false;  // an ordinary launch of any number of tiles (t_begin / t_end), not a cooperative one
};

// Pitch of the shared rings' rows: at least `floats`, a multiple of 4 (float4
// access) and 4 mod 32, so that consecutive rows start 4 banks apart and the
// transposed flush (one cell read from S consecutive rows) is conflict-free.
__host__ __device__ constexpr int ring_pitch(int floats) {
  return ((floats + 3) & ~3) + (36 - (((floats + 3) & ~3) % 32)) % 32;
}

// Floats of one edge array of a ring row set (volume sweeps only): for every
// row position (apron rows included) and run of 4 cells, the boundary cells of
// the neighbouring runs as a float2 (left neighbour's last cell, right
// neighbour's first).  A thread then reads its 6-cell neighbourhood of a row
// as one float4 and one float2, without bank conflicts.  Row sweeps (2D) read
// one row per step and keep long rings (up to 2048 cells x S rows), so they
// read the two edge cells directly and have no edge arrays.
__host__ __device__ constexpr int pass_edge_floats(int cross, int R1, int R2) {
  return cross == 2 ? ring_pitch((R1 + 2) * (((R2 + 3) / 4) + 2) * 2) : 0;
}

// Shared memory of a cluster sweep CTA (fg_cluster.cuh), a strip of T1 rows
// of N2 cells: offsets in floats, except `bar` (bytes).  Rows are stored
// with an apron row above and below (the neighbour strips' boundary rows)
// and a 4-cell apron left and right, as in the pass kernel.
struct ClusterLayout {
  int rpr, B2, rowf, edgef;               // runs per row, floats per ring row, ring and edge-array pitches
  int dring, iring, dedge, iedge, oring;  // distances [2][M], image [2][C], their edge arrays, staging [P][M+C][RPT][NT]
  int bar;                                // two mbarriers (bytes)
  int bytes;
};
__host__ __device__ inline ClusterLayout cluster_layout(int C, int M, int T1, int N2, int NT, int RPT, int P) {
  ClusterLayout l;
  l.rpr = (N2 + 3) / 4;
  l.B2 = 4 * l.rpr + 8;
  l.rowf = ring_pitch((T1 + 2) * l.B2);
  l.edgef = ring_pitch((T1 + 2) * (l.rpr + 2) * 2);
  l.dring = 0;
  l.iring = 2 * M * l.rowf;
  l.dedge = l.iring + 2 * C * l.rowf;
  l.iedge = l.dedge + 2 * M * l.edgef;
  l.oring = l.iedge + 2 * C * l.edgef;  // every pitch is a multiple of 4 floats: 16-byte aligned
  l.bar = (l.oring + P * (M + C) * RPT * NT * 4) * 4;
  l.bytes = l.bar + 16;
  return l;
}

// Shared-memory bytes of a pass kernel for a region of R1 x R2 cells.
size_t pass_smem_bytes(int cross, int C, int M, int mode, bool wt, int S, int R1, int R2, int *B2, int *rowf,
                       int *nown_max, int depth);
// largest staging depth a variant supports (registers hold none of it: it is shared memory)
constexpr int max_pass_depth(int nch, int m) { return (nch + m <= 4) ? 8 : 2; }

// Launchers (one translation unit per cross-section rank).
int launch_pass_cross1(const PassArgs &a, const LaunchCfg &c, int M, int mode, bool wt, cudaStream_t s);
int launch_pass_cross2(const PassArgs &a, const LaunchCfg &c, int M, int mode, bool wt, cudaStream_t s);
// Volume passes on a cluster plan (fg_pass3d_cluster.cu): c.tiles CTAs in one
// cluster; c.rpt = 2 selects the cluster sweep kernel (2 runs per thread).
int launch_pass_cluster(const PassArgs &a, const LaunchCfg &c, int M, int mode, bool wt, cudaStream_t s);
int launch_sweep_cluster(const PassArgs &a, const LaunchCfg &c, int M, int mode, bool wt, cudaStream_t s);
int cluster_capacity(int size, int threads, size_t smem, int *out);
// 2D passes on row tiles (fg_rowtile2d.cu): c.tiles CTAs of a cooperative
// launch, one thread per cell of a tile of a.T2 cells and its halos of a.K2 =
// a.S cells; row_tile_smem: its shared memory for `cimg` image channels read.
// clu: the tiles are one thread-block cluster and hand over through
// distributed shared memory (2 to 16 tiles, halos of S <= T2 cells).  Row
// tiles write in place (wt is refused: a transpose follows such a pass).
int launch_row_tiles(const PassArgs &a, const LaunchCfg &c, int M, int mode, bool wt, bool clu, cudaStream_t s);
size_t row_tile_smem(int cimg, int M, int R, int S, bool clu);

// A whole 2D transform (plain, or signed) of one image with both sides up to
// kOneLaunchSide by one CTA in one launch (fg_row2d.cu, one thread per cell
// of a row): initial distances, the image transpose, every pass and the
// signed difference.
int launch_image_one(const fg_batch2d_item &it, bool is_signed, int iterations, int *status, cudaStream_t s);
constexpr int kOneLaunchSide = FG_ONE_LAUNCH_SIDE;  // the one-CTA kernel's largest side
// the per-call path's one-CTA launch: images of fewer cells than this
constexpr long long kOneLaunchCells = FG_ONE_LAUNCH_CELLS;

// Toivanen's raster scan (fg_toivanen.cu): `nmaps` (1-4) distance maps swept
// in place; spacing_sq = nullptr for images.  bar: 4 counters (16 bytes) of
// scratch the launch clears, status: the workspace status word.
int launch_toivanen(const float *img, int C, int D, int H, int W, const float *spacing_sq, float *const *maps,
                    int nmaps, float lg, float le, int iterations, unsigned *bar, int *status, cudaStream_t s);

// Host error reporting shared by the units.
int set_error(int code, const char *msg);

}  // namespace fgi
