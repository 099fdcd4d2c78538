// Bounded waits shared by the kernels.  Every wait gives up after `limit`
// failed polls, or as soon as another CTA has recorded an error in the
// workspace status word, records FG_ERR_TIMEOUT there and returns: a kernel
// never traps and never spins without end, so a lost hand-off leaves the
// context usable and the host reads the error with fg_workspace_status().
#pragma once

#include "fg_common.cuh"

namespace fgi {

__device__ __forceinline__ int ld_status(const int *p) {
  int v;
  asm volatile("ld.relaxed.gpu.global.s32 %0, [%1];\n" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ unsigned long long ld_word(const unsigned long long *p) {
  unsigned long long v;
  asm volatile("ld.relaxed.gpu.global.b64 %0, [%1];\n" : "=l"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ unsigned ld_acquire_u32(const unsigned *p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];\n" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ bool mbar_try_wait(unsigned a, unsigned parity) {
  unsigned ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.acquire.cluster.shared::cta.b64 p, [%1], %2;\n"
      " selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(a), "r"(parity)
      : "memory");
  return ok != 0;
}

__device__ __forceinline__ void record_timeout(int *status) { atomicCAS(status, 0, FG_ERR_TIMEOUT); }

// The phase of parity `parity` of the mbarrier at shared address `bar` has
// completed.  False (FG_ERR_TIMEOUT recorded) if it did not in time.
__device__ __forceinline__ bool wait_phase(unsigned bar, unsigned parity, int *status, unsigned limit) {
  unsigned spins = 0;
  while (!mbar_try_wait(bar, parity)) {
    if (++spins > limit || ((spins & 255u) == 0 && ld_status(status) != 0)) {
      record_timeout(status);
      return false;
    }
  }
  return true;
}

// A 64-bit exchange word (value | epoch << 32) of epoch `want`; `w` is its
// first load, issued by the caller together with the others it needs.
__device__ __forceinline__ unsigned long long wait_word(const unsigned long long *p, unsigned want,
                                                        unsigned long long w, int *status, unsigned limit) {
  unsigned spins = 0;
  while ((unsigned)(w >> 32) != want) {
    if (++spins > limit || ((spins & 1023u) == 0 && ld_status(status) != 0)) {
      record_timeout(status);
      break;
    }
    w = ld_word(p);
  }
  return w;
}

// A counter (acquire loads) has reached `target`.
__device__ __forceinline__ bool wait_count(const unsigned *ctr, unsigned target, int *status, unsigned limit) {
  unsigned spins = 0;
  while (ld_acquire_u32(ctr) < target) {
    if (++spins > limit || ((spins & 1023u) == 0 && ld_status(status) != 0)) {
      record_timeout(status);
      return false;
    }
  }
  return true;
}

}  // namespace fgi
