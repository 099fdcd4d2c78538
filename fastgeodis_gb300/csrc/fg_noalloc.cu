// Allocation-free entry point: the plain 2D transform with its scratch held
// in a fixed device array of this library instead of a caller workspace.
//
// Some callers cannot allocate device memory at the point where they need a
// distance map: code running inside a host framework that owns the device
// allocator and forbids allocation while its work executes (plugin or
// operator callbacks, real-time loops that must not block on an allocator),
// or plain C callers that have no device allocator at all.  They pass their
// inputs and outputs and nothing else; the sweep kernels' scratch (halo
// exchange words, the transposed distance map and the transposed image copy) comes
// from `g_noalloc_scratch`, 16 MiB that every GPU loading the library holds
// until the process exits.
//
// Rules of use:
//   * Every call shares the one array and leaves its contents behind.  The
//     halo exchange words, which must start at zero, are cleared by each call
//     on its stream.  Calls whose GPU work overlaps (different streams, or
//     different host threads without ordering) race on the array and give
//     wrong results: order them on one stream.
//   * The array's first word is a status word.  A kernel whose bounded wait
//     expires writes FG_ERR_TIMEOUT there and stops; the word keeps that code
//     across later calls until fg_noalloc_status reads it (and clears it).
//     Check it after the calls whose results matter.
//   * The device address of the array is looked up on the device current at
//     the call (cudaGetSymbolAddress) whenever the call's stream is not being
//     captured, so a context re-created by cudaDeviceReset is followed.  A
//     call inside a stream capture reuses the address of the last uncaptured
//     call on that device, so make one call (or fg_noalloc_status) on the
//     device before capturing.
//   * Sizes whose scratch exceeds the array are refused with FG_ERR_UNSUPPORTED.
//   * Nothing here calls cudaMalloc, cudaFree or any other allocating routine.

#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include "fg_common.cuh"

namespace {

constexpr size_t kNoAllocScratchBytes = size_t(16) << 20;

__device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

std::mutex g_noalloc_mu;
void *g_noalloc_addr[64];  // device address of the array, per device ordinal (last uncaptured lookup)

// The array's device address on the current device.
int scratch_address(cudaStream_t s, void **ws) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return fgi::set_error(FG_ERR_CUDA, cudaGetErrorString(e));
  if (dev < 0 || dev >= 64) return fgi::set_error(FG_ERR_UNSUPPORTED, "device ordinal beyond 63");
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(s, &cap) != cudaSuccess) {
    (void)cudaGetLastError();
    cap = cudaStreamCaptureStatusActive;  // cannot tell: keep the cached address
  }
  std::lock_guard<std::mutex> g(g_noalloc_mu);
  if (cap == cudaStreamCaptureStatusNone || g_noalloc_addr[dev] == nullptr) {
    void *p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return fgi::set_error(FG_ERR_CUDA, cudaGetErrorString(e));
    g_noalloc_addr[dev] = p;
  }
  *ws = g_noalloc_addr[dev];
  return FG_OK;
}

}  // namespace

extern "C" FG_API int fg_generalised_geodesic2d_noalloc(const float *image, int C, int H, int W, const float *mask,
                                                        int Cm, float *out, float v, float l_grad, float l_eucl,
                                                        int iterations, void *stream) {
  const size_t need = fg_workspace_bytes(FG_OP_PLAIN, C, 1, H, W);
  if (need > kNoAllocScratchBytes) {
    std::string msg = "fg_generalised_geodesic2d_noalloc: this size needs " + std::to_string(need) +
                      " bytes of scratch; the fixed scratch array holds " + std::to_string(kNoAllocScratchBytes) +
                      " bytes ((C + 1) * H * W * 4 plus 32 * max(H, W) plus about 1 KiB must fit)";
    return fgi::set_error(FG_ERR_UNSUPPORTED, msg.c_str());
  }
  void *ws = nullptr;
  const int rc = scratch_address(static_cast<cudaStream_t>(stream), &ws);
  if (rc != FG_OK) return rc;
  // The status word is zero when the library loads and is cleared only by
  // fg_noalloc_status, so a timeout of an earlier call stays visible.
  return fg_generalised_geodesic2d(image, C, H, W, mask, Cm, out, v, l_grad, l_eucl, iterations, ws,
                                   kNoAllocScratchBytes, stream);
}

extern "C" FG_API int fg_noalloc_status(void *stream) {
  void *ws = nullptr;
  const int rc = scratch_address(static_cast<cudaStream_t>(stream), &ws);
  if (rc != FG_OK) return rc;
  return fg_workspace_status(ws, stream);
}
