/*
 * fastgeodis_gb300 -- C ABI of the GB300 generalised geodesic distance engine.
 *
 * Every entry point takes plain device pointers, sizes and a CUDA stream
 * (passed as void*, a cudaStream_t), launches on that stream and returns
 * without synchronising.  Tensors are float32, contiguous, in the reference's
 * layout without the batch dimension (which the reference requires to be 1):
 *   image  [C][H][W]      or [C][D][H][W]
 *   mask   [Cm][H][W]     or [Cm][D][H][W]
 *   out    [Cm][H][W]     or [Cm][D][H][W]   (allocated by the caller)
 * As in the reference, every mask channel is scaled by v and only channel 0
 * is swept.  Inputs are never modified.
 *
 * Arithmetic follows the reference's CPU path operation by operation, in
 * float32 without contraction, so results are bit-identical to it.
 *
 * Scratch: each call needs a caller-provided device workspace of at least
 * fg_workspace_bytes(...) bytes (256-byte aligned).  The library allocates
 * no device memory.  A workspace may be reused by calls that are ordered on
 * one stream; calls that may run concurrently need separate workspaces.
 *
 * Return value: FG_OK or an FG_ERR_* code; fg_last_error() gives a message
 * (thread-local).  Kernels never trap: a bounded wait that expires records
 * FG_ERR_TIMEOUT in the workspace, readable with fg_workspace_status().
 */
#ifndef FASTGEODIS_GB300_H
#define FASTGEODIS_GB300_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(__GNUC__)
#define FG_API __attribute__((visibility("default")))
#else
#define FG_API
#endif

#define FG_ABI_VERSION 1

#define FG_OK 0
#define FG_ERR_INVALID_ARGUMENT 1 /* shape, size or pointer problem (the reference's std::invalid_argument) */
#define FG_ERR_CUDA 2             /* a CUDA runtime call failed */
#define FG_ERR_WORKSPACE 3        /* workspace missing or too small */
#define FG_ERR_TIMEOUT 4          /* a bounded inter-CTA wait expired (recorded on the device) */
#define FG_ERR_UNSUPPORTED 5      /* a size or form the engine does not handle */

/* Operation codes for fg_workspace_bytes. */
#define FG_OP_PLAIN 0
#define FG_OP_SIGNED 1
#define FG_OP_GSF 2

FG_API int fg_abi_version(void);
FG_API const char *fg_last_error(void);

/* Bytes of workspace needed by one call of the given operation on a volume
 * of D*H*W voxels (D = 1 for 2D) with C image channels. */
FG_API size_t fg_workspace_bytes(int op, int C, int D, int H, int W);

/* Planner limits (no counterpart in the reference, which has no planner):
 * the largest cross-section region, in cells, one CTA may own, and the most
 * tiles one pass may use.  0 restores the default.  Results do not depend on
 * these values; they exist to tune and to exercise multi-tile plans. */
FG_API int fg_set_tuning(int max_region_cells, int max_tiles);

/* Plan flags (fg_plan_override's `lean` argument, fg_plan_describe's last field). */
#define FG_PLAN_LEAN 1    /* the 64-register kernel */
#define FG_PLAN_CLUSTER 2 /* a cluster plan: one thread-block cluster owns the cross-section (with
                           * FG_PLAN_ROWS: row tiles forming one cluster) */
#define FG_PLAN_RUNS2 4   /* cluster plan on the cluster sweep kernel, 2 runs of 4 cells per thread */
#define FG_PLAN_CHUNKED 8 /* a tile plan run as one ordinary launch per chunk of S steps */
#define FG_PLAN_ROWS 64   /* a 2D tile plan on the row-tile kernel: one thread per cell of a tile and its halos */
/* fg_plan_override only: the plan applies to passes of arithmetic mode m
 * alone (0: general, 1: l_grad == 0, 2: l_eucl == 0 and l_grad == 1), and
 * wins over a plan without this flag; without it a plan applies to every
 * mode. */
#define FG_PLAN_MODE(m) (((m) + 1) << 4)
#define FG_PLAN_MODE_MASK 0x30

/* Plan override (no counterpart in the reference): for passes whose
 * cross-section is N1 x N2 (cross = 1 for 2D images, N1 = 1; cross = 2 for
 * volumes), use tiles of T1 x T2 cells with S steps per halo hand-off
 * (S a power of two up to 32, halo S).  Flag FG_PLAN_LEAN asks for the 64-register
 * kernel where the variant has one (volumes, one image channel or none, one
 * map: two CTAs of up to 512 threads per SM); without it the planner decides
 * (the 128-register kernel up to 512 threads).  Flag FG_PLAN_CLUSTER (volumes
 * only, S >= 2) asks for a cluster plan instead: ceil(N1 / T1) CTAs (2 to
 * 16) of one thread-block cluster each own T1 whole rows, and exchange their
 * boundary rows every step through distributed shared memory, with no halo
 * and no hand-off through global memory; T2 is ignored, and so is S (a
 * pass that changes layout runs in place on a cluster plan and a tiled
 * transpose then moves the map).  With FG_PLAN_RUNS2 (and at most one image
 * channel read) the strips run on the cluster sweep kernel, each thread
 * owning 2 vertically adjacent runs (T1 is rounded up to an even number), at
 * most 512 threads per CTA.  With FG_PLAN_CHUNKED a tile plan runs as one
 * ordinary launch per chunk of S steps instead of one cooperative launch, so
 * its tiles need not all be resident at once: each launch's CTAs start from
 * the previous row that the launch before published.  The planner takes a
 * chunked plan by itself only for cross-sections whose tiles cannot all be
 * resident (volumes with slices beyond about 600 thousand cells).  With
 * FG_PLAN_ROWS (2D only) a tile plan of 1 to 4 image channels and at most
 * 512 cells per tile and halos runs on the row-tile kernel, one thread per
 * cell; adding FG_PLAN_CLUSTER makes its tiles one thread-block cluster that
 * hands the halos over through distributed shared memory (2 to 16 tiles;
 * otherwise the hand-off goes through global memory as without the flag).
 * The planner takes row tiles for every 2D pass of 1 to 4 image channels:
 * one tile for rows of up to 32 cells, a cluster of up to 16 tiles for rows
 * of up to 1024 cells, tiles of 32 to 128 cells handing over through global
 * memory beyond.
 * FG_PLAN_MODE(m) restricts the plan to passes
 * of one arithmetic mode (several transforms of one shape with different
 * weights, e.g. the lambdas of one image, may then get different plans).
 * S = 0 removes the override of that mode key.  Used by the
 * autotuner (fastgeodis_gb300.tune); results do not depend on it.  A plan
 * that does not fit the device falls back to the planner's choice, and a
 * cluster plan that the device cannot co-schedule fails with
 * FG_ERR_UNSUPPORTED at launch. */
FG_API int fg_plan_override(int cross, int N1, int N2, int S, int T1, int T2, int lean);

/* How many clusters of `cluster_size` CTAs (2-16) of `threads` threads and
 * `smem` bytes of dynamic shared memory each the current device runs at once
 * (cudaOccupancyMaxActiveClusters for the cluster sweep kernel): the
 * concurrency of cluster plans (no counterpart in the reference). */
FG_API int fg_cluster_capacity(int cluster_size, int threads, size_t smem, int *clusters);

/* The plan the engine uses for one pass (no counterpart in the reference):
 * cross-section rank `cross` (1: a 2D row, 2: a 3D plane) of N1 x N2 cells,
 * C image channels, `maps` distance maps (1 or 2), arithmetic mode (0
 * general, 1 l_grad == 0, 2 l_eucl == 0 and l_grad == 1), transposed write
 * or not, on a GPU of `sms` SMs.  Writes 11 ints to `plan`: S, T1, T2, K1,
 * K2, tiles1, tiles2, threads, staging depth, shared-memory bytes, flags
 * (FG_PLAN_LEAN, FG_PLAN_CLUSTER, FG_PLAN_RUNS2, FG_PLAN_CHUNKED,
 * FG_PLAN_ROWS).  Needs
 * no GPU; honours fg_set_tuning and fg_plan_override. */
FG_API int fg_plan_describe(int cross, int N1, int N2, int C, int maps, int mode, int transposed_write, int sms,
                            int *plan);

/* Event timing of the sweep kernels (no counterpart in the reference):
 * between fg_profile_begin() and fg_profile_end(), every pass launch is
 * bracketed by CUDA events on its stream.  fg_profile_end synchronises those
 * events and returns the summed kernel time in ms, the number of launches and
 * the voxel-passes (cells x maps updated) they performed.  Not for use inside
 * CUDA graph capture. */
FG_API int fg_profile_begin(void);
FG_API int fg_profile_end(double *pass_ms, int *pass_launches, double *voxel_passes);
/* Per-launch times of the window closed by the last fg_profile_end, in launch
 * order: up to `cap` entries of ms and of steps swept (the pass length);
 * *n receives the number recorded. */
FG_API int fg_profile_launch_times(float *ms, int *steps, int cap, int *n);
/* Kernel launches of the window closed by the last fg_profile_end besides
 * one per pass: the launches after the first of a chunked pass, and the map
 * transposes that follow a layout-changing pass on a cluster plan. */
FG_API int fg_profile_aux_launches(int *n);

/* Reads (and clears) the device status word of a workspace after
 * synchronising `stream`: FG_OK, or FG_ERR_TIMEOUT if a kernel gave up. */
FG_API int fg_workspace_status(void *workspace, void *stream);

/* Self-test of failure detection (no counterpart in the reference): runs the
 * engine's bounded wait routine on something that never happens -- kind 0
 * an exchange word nobody publishes, kind 1 an mbarrier phase whose bytes
 * never arrive, kind 2 a group counter that never reaches its target -- with
 * a limit well under a second.  The kernel records FG_ERR_TIMEOUT in the
 * workspace status word (read it with fg_workspace_status) and returns; the
 * context stays usable.  Uses the first 256 bytes of the workspace. */
FG_API int fg_selftest_wait(int kind, void *workspace, size_t workspace_bytes, void *stream);

/* Images of fewer than FG_ONE_LAUNCH_CELLS cells, with sides of at most
 * FG_ONE_LAUNCH_SIDE, run their whole plain or signed transform in one
 * launch (one CTA: initial distances, transpose, every pass); the others, and
 * any image whose passes have a pinned plan (fg_plan_override) or planner
 * limits (fg_set_tuning), run one launch per pass on the planned tiles: row
 * tiles (FG_PLAN_ROWS) for 1 to 4 image channels, which measured faster than
 * the one-CTA launch from 128 x 128 and 64 x 512 up (512 x 512: 0.79 against
 * 1.23 ms, iterations 2; 64 x 64: 0.17 against 0.16). */
#define FG_ONE_LAUNCH_SIDE 512
#define FG_ONE_LAUNCH_CELLS 16384

/* Replaces FastGeodis.generalised_geodesic2d
 * (reference: FastGeodis/__init__.py:37-65 -> FastGeodis/fastgeodis.cpp:44-90
 *  -> FastGeodis/fastgeodis_cuda.cu:278-318).
 * l_grad = lamb, l_eucl = 1 - lamb, both already narrowed to float. */
FG_API int fg_generalised_geodesic2d(const float *image, int C, int H, int W,
                              const float *mask, int Cm, float *out, float v,
                              float l_grad, float l_eucl, int iterations,
                              void *workspace, size_t workspace_bytes,
                              void *stream);

/* Replaces FastGeodis.generalised_geodesic3d
 * (reference: FastGeodis/__init__.py:68-98 -> FastGeodis/fastgeodis.cpp:92-146
 *  -> FastGeodis/fastgeodis_cuda.cu:587-656).  spacing: 3 floats (host). */
FG_API int fg_generalised_geodesic3d(const float *image, int C, int D, int H, int W,
                              const float *mask, int Cm, const float *spacing,
                              float *out, float v, float l_grad, float l_eucl,
                              int iterations, void *workspace,
                              size_t workspace_bytes, void *stream);

/* Replaces FastGeodis.signed_generalised_geodesic2d: D(mask) - D(1 - mask)
 * (reference: FastGeodis/__init__.py:101-130 -> FastGeodis/fastgeodis.cpp:241-249). */
FG_API int fg_signed_generalised_geodesic2d(const float *image, int C, int H, int W,
                                     const float *mask, int Cm, float *out,
                                     float v, float l_grad, float l_eucl,
                                     int iterations, void *workspace,
                                     size_t workspace_bytes, void *stream);

/* Replaces FastGeodis.signed_generalised_geodesic3d
 * (reference: FastGeodis/__init__.py:133-162 -> FastGeodis/fastgeodis.cpp:251-258). */
FG_API int fg_signed_generalised_geodesic3d(const float *image, int C, int D, int H,
                                     int W, const float *mask, int Cm,
                                     const float *spacing, float *out, float v,
                                     float l_grad, float l_eucl, int iterations,
                                     void *workspace, size_t workspace_bytes,
                                     void *stream);

/* Replaces FastGeodis.GSF2d (reference: FastGeodis/__init__.py:526-553 ->
 * FastGeodis/fastgeodis.cpp:319-330).  lambda as float; 1 - lambda is formed
 * in float inside, as the reference does.  The two signed transforms of the
 * second stage run at once: the second on a side stream of the calling host
 * thread (same device and priority), forked from and joined back to `stream`
 * with events, so the call stays ordered on `stream` as usual; while `stream`
 * is being captured into a CUDA graph both run on it.  The same holds for
 * fg_GSF3d. */
FG_API int fg_GSF2d(const float *image, int C, int H, int W, const float *mask,
             int Cm, float theta, float v, float lambda, int iterations,
             float *out, void *workspace, size_t workspace_bytes, void *stream);

/* Replaces FastGeodis.GSF3d (reference: FastGeodis/__init__.py:556-585 ->
 * FastGeodis/fastgeodis.cpp:332-343). */
FG_API int fg_GSF3d(const float *image, int C, int D, int H, int W, const float *mask,
             int Cm, float theta, const float *spacing, float v, float lambda,
             int iterations, float *out, void *workspace,
             size_t workspace_bytes, void *stream);

/* Toivanen's raster scan: replace FastGeodisCpp.generalised_geodesic2d/3d_toivanen,
 * signed_generalised_geodesic2d/3d_toivanen and GSF2d/3d_toivanen
 * (reference: FastGeodis/__init__.py:165-308, 587-656 -> FastGeodis/fastgeodis.cpp
 *  :148-177, 260-277, 345-369 -> FastGeodis/geodis_toivanen.cpp:40-348, CPU only
 *  there).  Same arguments, workspace and status rules as the raster entries
 * above; any channel count.  Results equal the reference's CPU output bit for
 * bit: the sequential scan runs as a wavefront, one CTA per distance map. */
FG_API int fg_generalised_geodesic2d_toivanen(const float *image, int C, int H, int W, const float *mask, int Cm,
                                              float *out, float v, float l_grad, float l_eucl, int iterations,
                                              void *workspace, size_t workspace_bytes, void *stream);
FG_API int fg_generalised_geodesic3d_toivanen(const float *image, int C, int D, int H, int W, const float *mask,
                                              int Cm, const float *spacing, float *out, float v, float l_grad,
                                              float l_eucl, int iterations, void *workspace, size_t workspace_bytes,
                                              void *stream);
FG_API int fg_signed_generalised_geodesic2d_toivanen(const float *image, int C, int H, int W, const float *mask,
                                                     int Cm, float *out, float v, float l_grad, float l_eucl,
                                                     int iterations, void *workspace, size_t workspace_bytes,
                                                     void *stream);
FG_API int fg_signed_generalised_geodesic3d_toivanen(const float *image, int C, int D, int H, int W,
                                                     const float *mask, int Cm, const float *spacing, float *out,
                                                     float v, float l_grad, float l_eucl, int iterations,
                                                     void *workspace, size_t workspace_bytes, void *stream);
FG_API int fg_GSF2d_toivanen(const float *image, int C, int H, int W, const float *mask, int Cm, float theta,
                             float v, float lambda, int iterations, float *out, void *workspace,
                             size_t workspace_bytes, void *stream);
FG_API int fg_GSF3d_toivanen(const float *image, int C, int D, int H, int W, const float *mask, int Cm,
                             float theta, const float *spacing, float v, float lambda, int iterations, float *out,
                             void *workspace, size_t workspace_bytes, void *stream);

/* One job of a batched 2D transform (see fg_batch_geodesic2d).  All
 * pointers are device pointers; float32, contiguous.  The scratch buffers
 * belong to the caller and must not overlap between images. */
typedef struct fg_batch2d_item {
  const float *image; /* [C][H][W] */
  const float *mask;  /* [H][W] soft mask (one channel) */
  float *out;         /* [H][W] result: D(mask), or D(mask) - D(1 - mask) when signed */
  float *image_t;     /* scratch [C][W][H] */
  float *d2;          /* scratch [H][W] (signed only) */
  float *t1;          /* scratch [W][H] */
  float *t2;          /* scratch [W][H] (signed only) */
  int C, H, W, flags; /* flags: FG_BATCH_* */
  float v, l_grad, l_eucl, reserved1;
} fg_batch2d_item;

/* fg_batch2d_item.flags.  FG_BATCH_SPLIT runs a signed image as two jobs on
 * two CTAs: the descriptor computes D(mask) and the next one, an identical
 * copy with FG_BATCH_SECOND added, D(1 - mask); the job that finishes second
 * writes the difference.  Without it both maps run in one CTA. */
#define FG_BATCH_SIGNED 1 /* signed transform D(mask) - D(1 - mask) */
#define FG_BATCH_SPLIT 2  /* signed, as two jobs */
#define FG_BATCH_SECOND 4 /* the second descriptor of a split signed image */

/* Batched generalised_geodesic2d / signed_generalised_geodesic2d over n
 * jobs -- images of any sizes up to 2048 per side and 1-4 channels, plain or
 * signed, a signed image in one descriptor or split over two -- in one
 * persistent launch: each CTA takes the next job from a work queue and runs
 * it whole (no counterpart in the reference, which takes one image per call;
 * per image the results are bit-identical to fg_generalised_geodesic2d /
 * fg_signed_generalised_geodesic2d, split or not).
 * `items`: device array of n descriptors, ideally ordered largest first (the
 * two of a split image adjacent, the first first); max_C / max_extent: the
 * largest channel count and side among them; is_signed: nonzero makes every
 * descriptor signed (FG_BATCH_SIGNED implied), zero follows their flags;
 * `counter`: device scratch of 1 + n ints (the work queue and one word per
 * split image, cleared by the call); `status`: device int where
 * FG_ERR_TIMEOUT or FG_ERR_INVALID_ARGUMENT (a split half without its
 * partner) is recorded; max_ctas: CTAs of the persistent launch at most (0:
 * one per SM).  Capturable in a CUDA graph.  fg_batch2d_smem_bytes: the
 * launch's dynamic shared memory (is_signed is ignored). */
FG_API size_t fg_batch2d_smem_bytes(int max_C, int max_extent, int is_signed);
FG_API int fg_batch_geodesic2d(const fg_batch2d_item *items, int n, int max_C, int max_extent,
                               int is_signed, int iterations, int *counter, int *status,
                               int max_ctas, void *stream);

/* Tiled images beside a batch: images whose one-CTA job would set the
 * batch's time run in this cooperative launch (on another stream), the rows
 * of items[i] split over tiles[i] CTAs (2-16, a host array) that hand their
 * strips' edges over through L2 every few steps and meet between passes; up
 * to 32 images, all of C channels, plain or FG_BATCH_SIGNED (one descriptor
 * each, never split).  `scratch`: device memory of
 * fg_batch2d_tiled_scratch_bytes(n, max_extent) bytes; `status` as in
 * fg_batch_geodesic2d.  Bit-identical to the one-CTA job.  The launch needs
 * sum(tiles) CTAs resident at once: give the batch beside it max_ctas =
 * SMs - sum(tiles). */
FG_API size_t fg_batch2d_tiled_scratch_bytes(int n, int max_extent);
FG_API int fg_batch_geodesic2d_tiled(const fg_batch2d_item *items, const int *tiles, int n, int C, int max_extent,
                                     int iterations, void *scratch, size_t scratch_bytes, int *status,
                                     void *stream);

/* One volume of a batch run in one persistent launch (fg_batch3d_plan /
 * fg_batch3d_launch; no counterpart in the reference, which transforms one
 * volume per call).  Device pointers, float32, contiguous. */
typedef struct fg_batch3d_item {
  const float *image; /* [C][D][H][W] */
  const float *mask;  /* [D][H][W] soft mask (one channel) */
  float *out;         /* [D][H][W] result: D(mask), or D(mask) - D(1 - mask) when signed */
  float *image_t;     /* scratch [C][W][D][H] */
  float *t1;          /* scratch [W][D][H] */
  float *d2;          /* scratch [D][H][W] (signed only) */
  float *t2;          /* scratch [W][D][H] (signed only) */
  int C, D, H, W;
  int flags;          /* FG_BATCH_SIGNED, the same for every item of a batch */
  float v, l_grad, l_eucl;
  float spacing[3];   /* (z, y, x), as the drop-in's spacing */
  float reserved1;
} fg_batch3d_item;

/* Batched generalised_geodesic3d / signed_generalised_geodesic3d in ONE
 * persistent launch (no counterpart in the reference).  Every volume's
 * transform becomes a chain of jobs -- initial distances and the transposed
 * image copy, its passes in order, and for the signed form the difference --
 * in one queue; the launch holds as many thread-block clusters of
 * `cluster_size` CTAs (1-16) as the device co-schedules, and each cluster
 * runs one job at a time (a pass: the cross-section's rows split into strips
 * over the cluster, rows exchanged through distributed shared memory), a job
 * starting once its volume's previous job has finished.  Results are
 * bit-identical to fg_generalised_geodesic3d / fg_signed_generalised_geodesic3d.
 * Volumes read at most one image channel (C = 1, or l_grad = 0); a
 * cross-section must fit the cluster (at most 512 threads of 2 x 4 cells per
 * CTA).
 *
 * fg_batch3d_plan builds the job records on the host into `jobs` (host
 * memory, `jobs_bytes` bytes; fg_batch3d_job_bytes() each, at most
 * n * (2 + 10 * iterations) jobs: a prologue, six passes and a transpose of
 * each map before and after the passes along W per iteration, an epilogue)
 * and writes info[0] = jobs, info[1] =
 * threads per CTA, info[2] = shared-memory bytes per CTA, info[3] = maps per
 * pass, info[4] = arithmetic mode of the launch; `status` is the device word
 * a wait that runs out writes FG_ERR_TIMEOUT to.  FG_ERR_WORKSPACE when
 * `jobs_bytes` is too small (info[0] then holds the jobs needed).
 * fg_batch3d_launch runs the jobs after they were copied to device memory
 * (`jobs`), with `counters` device memory of (n + 1) 32-bit words that it
 * clears on `stream` first; capturable in a CUDA graph. */
FG_API size_t fg_batch3d_job_bytes(void);
FG_API int fg_batch3d_plan(const fg_batch3d_item *items, int n, int iterations, int cluster_size, int *status,
                           void *jobs, size_t jobs_bytes, int *info);
FG_API int fg_batch3d_launch(const void *jobs, int njobs, int n, int maps, int mode, int cluster_size, int threads,
                             size_t smem, unsigned *counters, int *status, void *stream);
/* How many clusters of that shape the launch co-schedules on the current device. */
FG_API int fg_batch3d_capacity(int maps, int mode, int cluster_size, int threads, size_t smem, int *clusters);

/* One image of a differentiable 2D transform (fg_grad_geodesic2d_forward /
 * _backward; no counterpart in the reference, which is not differentiable).
 * Device pointers, float32 unless noted, contiguous; scratch belongs to the
 * caller and is shared by the forward and the backward of one image. */
typedef struct fg_grad2d_item {
  const float *image;   /* [C][H][W] */
  const float *mask;    /* [H][W] soft mask */
  float *out;           /* forward output D [H][W] */
  float *image_t;       /* scratch [C][W][H] */
  float *t1;            /* scratch [W][H] */
  unsigned char *tape;  /* iterations * 4 * H * W bytes: argmin of every cell in every pass */
  const float *g_out;   /* backward input dLoss/dD [H][W] */
  float *g_image;       /* backward output dLoss/dimage [C][H][W] */
  float *g_mask;        /* backward output dLoss/dmask [H][W] */
  float *g_r;           /* scratch [H][W] */
  float *g_t;           /* scratch [W][H] */
  float *gi_t;          /* scratch [C][W][H] */
  int C, H, W, reserved0;
  float v, l_grad, l_eucl, reserved1;
} fg_grad2d_item;

/* Forward: D exactly as fg_generalised_geodesic2d, plus the argmin tape. */
FG_API int fg_grad_geodesic2d_forward(const fg_grad2d_item *items, int n, int max_C, int max_extent,
                                      int iterations, int *counter, int *status, void *stream);
/* Backward: routes dLoss/dD along the recorded argmins (the adjoint of every
 * pass, last pass first) to dLoss/dmask (= v * dLoss/dD0) and dLoss/dimage
 * (l_grad * sign(dI) of each step taken). */
FG_API int fg_grad_geodesic2d_backward(const fg_grad2d_item *items, int n, int max_C, int max_extent,
                                       int iterations, int *counter, int *status, void *stream);

/* Memory-saving form of the two calls above (no counterpart in the reference):
 * instead of every pass's tape (iterations * 4 * H * W bytes) an item's tape
 * buffer holds one pass (H * W bytes), and the passes are recomputed.  Passes
 * are numbered iteration * 4 + k (k: H forward, H backward, W forward, W
 * backward).  _forward_pass runs passes 0 .. pass from the initial distances
 * and records only that pass's tape; `out` receives the distances after it
 * (point it at scratch when recomputing, to keep the real output).
 * _backward_pass applies the adjoint of that one pass; first = 1 starts the
 * gradient state from g_out, last = 1 writes g_mask and g_image.  Calling
 * forward_pass(p) then backward_pass(p) for p from the last pass down to 0
 * gives the same gradients, bit for bit, as fg_grad_geodesic2d_backward. */
FG_API int fg_grad_geodesic2d_forward_pass(const fg_grad2d_item *items, int n, int max_C, int max_extent, int pass,
                                           int *counter, int *status, void *stream);
FG_API int fg_grad_geodesic2d_backward_pass(const fg_grad2d_item *items, int n, int max_C, int max_extent, int pass,
                                            int first, int last, int *counter, void *stream);

/* Soft mask of an interactive request from its clicks (no counterpart in the
 * reference, whose callers build masks on the host): writes mask[D][H][W]
 * (D = 1 for a 2D image) with 0.0 at every voxel within Euclidean distance
 * `radius` of a click and 1.0 elsewhere.  clicks: host array of n_clicks
 * (z, y, x) triples (z = 0 in 2D), at most 64; copied into the launch, so
 * the array may be reused as soon as the call returns.  Exact integer test,
 * one 4-byte write per voxel, on `stream`. */
FG_API int fg_click_mask(float *mask, int D, int H, int W, const int *clicks, int n_clicks, int radius, void *stream);

/* Allocation-free variant of fg_generalised_geodesic2d (no counterpart in
 * the reference).  For callers that cannot allocate device memory when they
 * need the transform -- code running inside a framework that owns the
 * allocator and forbids allocation during execution, or C callers without a
 * device allocator.  It takes no workspace: its scratch is a fixed 16 MiB
 * device array inside this library, held by every GPU that loads the library
 * until the process exits.  Limit: (C + 1) * H * W * 4 bytes plus
 * 32 * max(H, W) bytes plus about 1 KiB must fit in 16 MiB (for example C = 1 up to about 2 million pixels);
 * larger sizes return FG_ERR_UNSUPPORTED.  All calls share the array: calls
 * whose GPU work overlaps race and give wrong results, so order them on one
 * stream.  The array's address is looked up on the current device at every
 * call made outside a stream capture (so a context re-created by
 * cudaDeviceReset is followed); a call inside a capture reuses the last
 * lookup, so make one call on the device before capturing.  A bounded wait
 * that expires leaves FG_ERR_TIMEOUT in the array's status word until
 * fg_noalloc_status reads it.  Allocates nothing (no cudaMalloc /
 * cudaFree); results are bit-identical to fg_generalised_geodesic2d. */
FG_API int fg_generalised_geodesic2d_noalloc(const float *image, int C, int H, int W,
                                             const float *mask, int Cm, float *out, float v,
                                             float l_grad, float l_eucl, int iterations,
                                             void *stream);

/* Status of the allocation-free entry point's fixed scratch array (no
 * counterpart in the reference): synchronises `stream`, returns FG_OK or the
 * code a kernel of an earlier fg_generalised_geodesic2d_noalloc call left
 * there (FG_ERR_TIMEOUT), and clears it.  The word is not cleared by the
 * transform calls, so one check covers every call since the last one. */
FG_API int fg_noalloc_status(void *stream);

#ifdef __cplusplus
}
#endif

#endif /* FASTGEODIS_GB300_H */
