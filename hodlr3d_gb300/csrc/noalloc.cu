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
// cudaGetSymbolAddress, once per device and context, with that device
// current.  The first hodlr3d_matvec_noalloc call on a device performs that
// lookup; make the first call before any stream capture.  The address is
// cached together with the CUDA context it belongs to: after a
// cudaDeviceReset the next call finds another current context and looks the
// address up again.
#include <cuda.h>
#include <cuda_runtime.h>

#include <mutex>

#include "noalloc.h"

namespace h3d {

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

namespace {
constexpr int kMaxDevices = 64;
std::mutex g_mu;
struct Cached {
  CUcontext ctx;
  void* addr;
};
Cached g_cache[kMaxDevices] = {};

// the calling thread's current context (driver entry point, looked up once)
cudaError_t current_context(CUcontext* ctx) {
  using Fn = CUresult (*)(CUcontext*);
  static Fn get = nullptr;
  if (!get) {
    cudaDriverEntryPointQueryResult q;
    cudaError_t e = cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", (void**)&get, 12000,
                                                     cudaEnableDefault, &q);
    if (e != cudaSuccess) return e;
    if (!get || q != cudaDriverEntryPointSuccess) return cudaErrorNotSupported;
  }
  return get(ctx) == CUDA_SUCCESS ? cudaSuccess : cudaErrorDeviceUninitialized;
}
}  // namespace

cudaError_t noalloc_scratch(int device, void** ptr) {
  if (device < 0 || device >= kMaxDevices) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lock(g_mu);
  int cur = -1;
  cudaError_t e = cudaGetDevice(&cur);
  if (e != cudaSuccess) return e;
  if (cur != device) return cudaErrorInvalidDevice;  // the caller makes `device` current
  CUcontext ctx = nullptr;
  e = current_context(&ctx);
  if (e != cudaSuccess) return e;
  Cached& c = g_cache[device];
  if (!c.addr || !ctx || c.ctx != ctx) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return e;
    // the lookup makes the device's primary context current if none was
    e = current_context(&ctx);
    if (e != cudaSuccess) return e;
    c.addr = p;
    c.ctx = ctx;
  }
  *ptr = c.addr;
  return cudaSuccess;
}

}  // namespace h3d
