// Scratch memory of hodlr3d_matvec_noalloc, the matvec entry point for
// callers that cannot allocate device memory while they run -- for example a
// caller working inside a fixed memory budget handed out up front, or one
// whose allocator must not be re-entered from the thread that computes.
//
// The scratch lives in one file-scope device array of kNoAllocScratchBytes
// (64 MiB).  Every GPU that loads this library holds it until the process
// exits.  Every call shares it and finds the previous call's contents there;
// the matvec writes each scratch value before it reads it, so nothing needs
// clearing, and calls that overlap on the GPU (two streams, or two handles at
// once) race on it.
//
// Host code cannot use the array's name as a device address (on the host it
// names a stand-in object), so the address is looked up here with
// cudaGetSymbolAddress, once per device, with that device current.  The first
// hodlr3d_matvec_noalloc call on a device performs that lookup; make the first
// call before any stream capture.
#include <cuda_runtime.h>

#include <mutex>

#include "noalloc.h"

namespace h3d {

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

namespace {
constexpr int kMaxDevices = 64;
std::mutex g_mu;
void* g_addr[kMaxDevices] = {};
}  // namespace

cudaError_t noalloc_scratch(int device, void** ptr) {
  if (device < 0 || device >= kMaxDevices) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lock(g_mu);
  if (!g_addr[device]) {
    int cur = -1;
    cudaError_t e = cudaGetDevice(&cur);
    if (e != cudaSuccess) return e;
    if (cur != device) return cudaErrorInvalidDevice;  // the caller makes `device` current
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return e;
    g_addr[device] = p;
  }
  *ptr = g_addr[device];
  return cudaSuccess;
}

}  // namespace h3d
