// Batched ACA launchers (aca.cu).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "common.cuh"

namespace h3d {

// Points in tree order, FP64.
struct PointsF64 {
  const double* x;
  const double* y;
  const double* z;
};

// One ACA task: the block K(rows [t0, t0+n), cols [s0, s0+m)) in tree order.
struct AcaTask {
  int32_t t0, n, s0, m;
  int32_t cap;      // rank capacity of the workspace
  int32_t pair;     // pair index
  int64_t ws_off;   // doubles: U (cap x n) then V (cap x m), column-major
  int64_t fl_off;   // bytes: used-row flags (n) then used-column flags (m)
  int64_t piv_off;  // ints: row pivots (cap) then column pivots (cap), local indices
};

enum AcaStatus { kAcaOk = 0, kAcaCapReached = 1, kAcaNonFinite = 2 };

size_t aca_shared_bytes(int cap_max);
// One warp per pair (pairs of at most 128 points a side): kAcaWarpsPerBlock
// warps per block, `grid` persistent blocks; same results as launch_aca.
constexpr int kAcaWarpsPerBlock = 4;
constexpr int kAcaWarpBlocksPerSm = 8;  // 32 pairs per SM at 64 registers
size_t aca_warp_shared_bytes(int cap_max);
cudaError_t launch_aca_warp(cudaStream_t s, int grid, const AcaTask* tasks, int ntasks, int* counter,
                            PointsF64 P, KernelDesc kd, double tol, double* ws, unsigned char* flags,
                            int32_t* piv, int32_t* out_rank, int32_t* out_status, int cap_max);
// One block of kAcaBlock threads per pair, `grid` persistent blocks.
constexpr int kAcaBlock = 256;
cudaError_t launch_aca(cudaStream_t s, int grid, const AcaTask* tasks, int ntasks, int* counter,
                       PointsF64 P, KernelDesc kd, double tol, double* ws, unsigned char* flags,
                       int32_t* piv, int32_t* out_rank, int32_t* out_status, int cap_max);
cudaError_t launch_aca_compact(cudaStream_t s, int ntasks, const AcaTask* tasks,
                               const int32_t* rank, const int64_t* dst_off, const double* ws,
                               double* out64);
// FP32 U of every pair from its FP64 U, or (lo) the remainders (see k_u32
// in aca.cu)
cudaError_t launch_u32(cudaStream_t s, int64_t npairs, const double* const* u64, float* const* u32,
                       const int32_t* nsize, const int32_t* us, const int32_t* rank, int lo);
// FP32 V of every pair from its FP64 V, or (lo) the remainders (see k_v32)
cudaError_t launch_v32(cudaStream_t s, int64_t npairs, const double* const* v64, float* const* v32,
                       const int32_t* msize, const int32_t* rank, int lo);

}  // namespace h3d
