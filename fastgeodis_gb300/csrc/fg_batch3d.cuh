// A batch of volume transforms in one persistent launch: the job records the
// host builds (fg_engine.cu, fg_batch3d_plan) and the kernel runs
// (fg_batch3d.cu).
//
// A volume's transform is a chain of jobs: a prologue (initial distances and
// the transposed image copy), its passes in order (each a cluster-plan pass:
// the cluster's CTAs own strips of whole rows of the cross-section, rows
// exchanged through distributed shared memory), and for the signed form an
// epilogue (D(M) - D(1 - M)).  A pass that hands over to the passes along W,
// and the last of those, run in place and are followed by a transpose job
// ([(D H)][W] <-> [W][(D H)]).  Job k of a volume may start once its job
// k - 1 has finished (a per-volume progress counter).
#pragma once

#include "fg_common.cuh"

namespace fgi {

enum Batch3dJobKind { JOB3_PROLOGUE = 0, JOB3_PASS = 1, JOB3_EPILOGUE = 2, JOB3_TRANSPOSE = 3 };

struct Batch3dJob {
  PassArgs a;         // JOB3_PASS: the pass (tiles1 strips; rank >= tiles1 idles)
  int kind;           // Batch3dJobKind
  int mode, wt;       // JOB3_PASS: arithmetic mode, transposed write
  int vol, seq;       // volume and position of the job in the volume's chain
  // prologue / epilogue
  const float *image;  // [C][D][H][W]
  float *image_t;      // [C][W][D][H] (nullptr: no image pass reads it)
  const float *mask;   // [D][H][W]
  float *out, *d2;     // map 0 (= the output) and the signed form's map 1
  int C, D, H, W;
  float v;
  int is_signed;
  // transpose: tdst[c][r] = tsrc[r][c] for a trows x tcols matrix
  const float *tsrc;
  float *tdst;
  long long trows;
  int tcols;
};

// Launch of the persistent kernel for maps per pass M (1 plain, 2 signed)
// and arithmetic `mode` (every pass's, or MODE_GENERAL for a mixed batch):
// as many clusters of `G` CTAs of `threads` threads and `smem` bytes as the
// device co-schedules; counters[0] is the queue, counters[1 + v] volume v's
// progress (the launch clears them on `s` first).
int launch_batch3d(const Batch3dJob *jobs, int njobs, int nvol, int M, int mode, int G, int threads, size_t smem,
                   unsigned *counters, int *status, cudaStream_t s);
int batch3d_capacity(int M, int mode, int G, int threads, size_t smem, int *clusters);

}  // namespace fgi
