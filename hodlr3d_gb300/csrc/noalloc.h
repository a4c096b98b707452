// Scratch array of the no-allocation matvec entry point (noalloc.cu).
#pragma once
#include <cuda_runtime.h>
#include <stddef.h>

namespace h3d {

constexpr size_t kNoAllocScratchBytes = size_t(64) << 20;  // 64 MiB

// Device address of the scratch array on `device`, which must be current.
cudaError_t noalloc_scratch(int device, void** ptr);

}  // namespace h3d
