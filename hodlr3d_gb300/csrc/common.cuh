// Shared device helpers of the hodlr3d_gb300 CUDA library (sm_103a).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace h3d {

constexpr int kMaxLevels = 10;      // keys of 3 * levels bits fit in 32 bits
constexpr int kCanonChunk = 8192;   // canonical reduction chunk (see warp_canonical_sum)

// ---------------------------------------------------------------------------
// Octree digit layout of the reference (assign_Center_Location,
// src/HODLR3DTree.cpp:1528-1553): child digit -> octant bits
//   0:(-,-,-) 1:(+,-,-) 2:(+,+,-) 3:(-,+,-) 4:(-,-,+) 5:(+,-,+) 6:(+,+,+) 7:(-,+,+)
// ---------------------------------------------------------------------------
__host__ __device__ inline int digit_x(int d) { return (0x66 >> d) & 1; }
__host__ __device__ inline int digit_y(int d) { return (0xCC >> d) & 1; }
__host__ __device__ inline int digit_z(int d) { return (0xF0 >> d) & 1; }
// octant bits -> digit; nibble (bx + 2 by + 4 bz) of 0x67542310
__host__ __device__ inline int digit_of(int bx, int by, int bz) {
  return (int)((0x67542310u >> (4 * (bx + 2 * by + 4 * bz))) & 0xFu);
}
// index of the first box of level j in the all-levels box numbering
__host__ __device__ inline int64_t level_base(int j) { return ((int64_t(1) << (3 * j)) - 1) / 7; }

// One-time settings that apply per device (kernel attributes such as the
// dynamic shared-memory limit) are tracked per device ordinal.
constexpr int kMaxDevices = 64;
inline int current_device() {
  int d = 0;
  if (cudaGetDevice(&d) != cudaSuccess || d < 0 || d >= kMaxDevices) d = 0;
  return d;
}

// ---------------------------------------------------------------------------
// Kernel entries.  `kind` is the reference's Qchoice (src/kernel.cpp:65-227);
// the diagonal is Kii for kind 16 and 0 otherwise (the dispatch of
// examples/testHODLR3Dsolve.cpp:32-75) unless an override is given.
// ---------------------------------------------------------------------------
struct KernelDesc {
  int kind;
  double kii;   // diagonal of kind 16
  double h3;    // 1/N scale of kind 16
  double diag;  // diagonal used by the device (resolved on the host)
};

// FP64 entry for i != j, evaluated with the same operations and rounding as
// the reference's C++ (no contraction into fused multiply-adds), so that the
// ACA sees bit-identical rows and columns for the algebraic kernels.
__device__ __forceinline__ double entry64_offdiag(const KernelDesc& kd, double dx, double dy,
                                                  double dz) {
  const double R2 = __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz));
  const double R = __dsqrt_rn(R2);
  switch (kd.kind) {
    case 0: return log(__dadd_rn(1.0, R));
    case 1: return exp(-R);
    case 2: return __ddiv_rn(1.0, __dadd_rn(1.0, __dmul_rn(R, R)));
    case 3: return __dadd_rn(1.0, __dmul_rn(R, R));
    case 4: return __ddiv_rn(1.0, __dsqrt_rn(__dadd_rn(__dmul_rn(R, R), 1.0)));
    case 5: return exp(-__dmul_rn(R, R));
    case 6: return __dsqrt_rn(__dadd_rn(__dmul_rn(R, R), 1.0));
    case 7: return __ddiv_rn(1.0, R);
    case 8: return __ddiv_rn(1.0, __dmul_rn(R2, R2));
    case 9: return log(R);
    case 10: return __dmul_rn(__dmul_rn(R, R), log(R));
    case 11: return j0(R);  // J_0(kappa R), kappa = 1
    case 12: return y0(R);  // Y_0(kappa R), kappa = 1
    case 13: return __ddiv_rn(cos(R), R);
    // K_{1/2}(R) / sqrt(R) = sqrt(pi / (2 R)) e^{-R} / sqrt(R) = sqrt(pi / 2) e^{-R} / R
    case 14: return __ddiv_rn(__dmul_rn(1.2533141373155002512, exp(-R)), R);
    case 15: return __ddiv_rn(exp(__dmul_rn(-50.0, R)), R);
    case 16: return __dmul_rn(kd.h3, __ddiv_rn(1.0, R));
  }
  return 0.0;
}

// FP32 entry from an FP32 displacement (mixed precision near field).
__device__ __forceinline__ float entry32_offdiag(const KernelDesc& kd, float dx, float dy,
                                                 float dz) {
  const float R2 = fmaf(dz, dz, fmaf(dy, dy, dx * dx));
  switch (kd.kind) {
    case 16: return (float)kd.h3 * rsqrtf(R2);
    case 7: return rsqrtf(R2);
    case 1: return __expf(-R2 * rsqrtf(R2));
    case 8: return 1.0f / (R2 * R2);
    case 2: return 1.0f / (1.0f + R2);
    case 3: return 1.0f + R2;
    case 4: return rsqrtf(R2 + 1.0f);
    case 5: return __expf(-R2);
    case 6: return sqrtf(R2 + 1.0f);
    default: break;
  }
  const float R = sqrtf(R2);
  switch (kd.kind) {
    case 0: return log1pf(R);
    case 9: return logf(R);
    case 10: return R2 * logf(R);
    case 11: return j0f(R);
    case 12: return y0f(R);
    case 13: return cosf(R) / R;
    case 14: return 1.25331414f * __expf(-R) / R;
    case 15: return expf(-50.0f * R) / R;
  }
  return 0.0f;
}

// ---------------------------------------------------------------------------
// TF32 forms of FP32 data for the tensor-core engine (a TF32 value is an FP32
// value whose 13 low mantissa bits are zero; the tensor core reads an FP32
// word as TF32 by ignoring those bits).
// ---------------------------------------------------------------------------
// x rounded to the nearest TF32 value (ties away from zero): half a TF32 ulp
// added to the magnitude bits, the low bits cleared.
__device__ __forceinline__ float tf32_rn(float x) {
  return __uint_as_float((__float_as_uint(x) + 0x1000u) & 0xFFFFE000u);
}
// x with the low bits cleared (rounded toward zero)
__device__ __forceinline__ float tf32_rz(float x) {
  return __uint_as_float(__float_as_uint(x) & 0xFFFFE000u);
}
// The "split-exact" FP32 form of x: v = hi + lo with hi = tf32_rz(v), the
// truncation of x, and lo = v - hi the remainder x - hi rounded to 11
// significant bits, so that both parts of v are TF32 and the tensor core
// reads hi straight from v.  |v - x| <= 2^-22 |x|.
__device__ __forceinline__ float tf32_split_value(double x) {
  const float hi = tf32_rz(__double2float_rz(x));
  const float lo = tf32_rn((float)(x - (double)hi));
  return hi + lo;
}

// ---------------------------------------------------------------------------
// Warp reductions
// ---------------------------------------------------------------------------
// The canonical reduction: each lane holds the sequential sum of its strided
// elements; the butterfly p[L] + p[L ^ o], o = 16..1, leaves the same value in
// every lane.  Its CPU restatement is the oracle's canonical_sum.
__device__ __forceinline__ double warp_butterfly_sum(double v) {
#pragma unroll
  for (int o = 16; o >= 1; o >>= 1) v = __dadd_rn(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}

// sum over i < n of a[i] * b[i] in the canonical order, by one warp
__device__ __forceinline__ double warp_canonical_dot(const double* __restrict__ a,
                                                     const double* __restrict__ b, int n,
                                                     int lane) {
  double total = 0.0;
  for (int c0 = 0; c0 < n; c0 += kCanonChunk) {
    const int c1 = min(n, c0 + kCanonChunk);
    double p = 0.0;
    for (int i = c0 + lane; i < c1; i += 32) p = __dadd_rn(p, __dmul_rn(a[i], b[i]));
    p = warp_butterfly_sum(p);
    total = c0 == 0 ? p : __dadd_rn(total, p);
  }
  return total;
}

// (|value|, index) maximum with ties to the lowest index (first maximum, as
// LowRank::maxAbsVector, src/ACA.cpp:10-23).  idx < 0 means "none".
__device__ __forceinline__ void argmax_merge(double& v, int& i, double v2, int i2) {
  if (i2 < 0) return;
  if (i < 0 || v2 > v || (v2 == v && i2 < i)) {
    v = v2;
    i = i2;
  }
}

__device__ __forceinline__ void warp_argmax(double& v, int& i) {
#pragma unroll
  for (int o = 16; o >= 1; o >>= 1) {
    const double v2 = __shfl_xor_sync(0xffffffffu, v, o);
    const int i2 = __shfl_xor_sync(0xffffffffu, i, o);
    argmax_merge(v, i, v2, i2);
  }
}

__device__ __forceinline__ float warp_sum_f(float v) {
#pragma unroll
  for (int o = 16; o >= 1; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

__device__ __forceinline__ double warp_sum_d(double v) {
#pragma unroll
  for (int o = 16; o >= 1; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

}  // namespace h3d
