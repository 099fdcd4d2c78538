// Self-test of the bounded waits (fg_wait.cuh): each kind waits for something
// that never happens, with the production wait routine and a short limit, so
// the kernel must record FG_ERR_TIMEOUT in the workspace status word and
// return.  Used by the tests of failure detection; it faults nothing.
#include "fg_wait.cuh"

namespace fgi {
namespace {

constexpr size_t kSelftestWord = 128;     // workspace header offset of the exchange word (8 bytes)
constexpr size_t kSelftestCounter = 136;  // and of the counter (4 bytes)

__global__ void fg_selftest_wait_kernel(int kind, const unsigned long long *word, const unsigned *counter,
                                        int *status, unsigned limit) {
  __shared__ __align__(8) unsigned long long bar;
  if (threadIdx.x != 0) return;
  if (kind == 0) {
    // an exchange word of epoch 1: the word is zero and nobody publishes it
    wait_word(word, 1u, ld_word(word), status, limit);
  } else if (kind == 1) {
    // an mbarrier phase that expects 16 bytes of asynchronous stores nobody sends
    const unsigned b = (unsigned)__cvta_generic_to_shared(&bar);
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(b) : "memory");
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], 16;\n" ::"r"(b) : "memory");
    wait_phase(b, 0u, status, limit);
  } else {
    // a group barrier counter that never reaches its target
    wait_count(counter, 1u, status, limit);
  }
}

}  // namespace
}  // namespace fgi

extern "C" int fg_selftest_wait(int kind, void *workspace, size_t workspace_bytes, void *stream) {
  using namespace fgi;
  if (kind < 0 || kind > 2) return set_error(FG_ERR_INVALID_ARGUMENT, "self-test kind is 0, 1 or 2");
  if (!workspace || workspace_bytes < 256 || (reinterpret_cast<uintptr_t>(workspace) & 255))
    return set_error(FG_ERR_WORKSPACE, "self-test needs a 256-byte aligned workspace of at least 256 bytes");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  char *base = static_cast<char *>(workspace);
  cudaError_t e = cudaMemsetAsync(base + kSelftestWord, 0, 16, s);
  if (e != cudaSuccess) return set_error(FG_ERR_CUDA, cudaGetErrorString(e));
  const unsigned limit = kind == 1 ? (1u << 14) : (1u << 16);  // well under a second
  fg_selftest_wait_kernel<<<1, 32, 0, s>>>(kind, reinterpret_cast<const unsigned long long *>(base + kSelftestWord),
                                          reinterpret_cast<const unsigned *>(base + kSelftestCounter),
                                          reinterpret_cast<int *>(base), limit);
  e = cudaGetLastError();
  if (e != cudaSuccess) return set_error(FG_ERR_CUDA, cudaGetErrorString(e));
  return FG_OK;
}
