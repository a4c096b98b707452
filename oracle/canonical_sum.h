/* TEST INFRASTRUCTURE.  The canonical FP64 reduction order of the CUDA
 * kernels (hodlr3d_gb300/csrc/common.cuh, warp_canonical_sum), restated for
 * the CPU oracle and the Eigen API shim so that norms and dot products --
 * and with them the stopping test of the ACA -- agree bit for bit.
 *
 * canonical_sum(f, n): the index range is cut into chunks of 8192; in a chunk,
 * lane L (0..31) adds f(i) for i = L, L+32, L+64, ... in increasing order,
 * starting from 0.0; the 32 lane sums are combined by the butterfly
 * p[L] = p[L] + p[L ^ o] for o = 16, 8, 4, 2, 1 (a warp's __shfl_xor
 * reduction) and the chunk sums are added in chunk order.  Products are
 * rounded before they are added (no fused multiply-add).
 */
#ifndef HODLR3D_CANONICAL_SUM_H
#define HODLR3D_CANONICAL_SUM_H
#define HODLR3D_CANON_CHUNK 8192
#define HODLR3D_CANON_LANES 32

#ifdef __cplusplus
template <class F>
static inline double hodlr3d_canonical_sum(F f, long n) {
  double total = 0.0;
  for (long c0 = 0; c0 < n; c0 += HODLR3D_CANON_CHUNK) {
    double p[HODLR3D_CANON_LANES];
    for (int L = 0; L < HODLR3D_CANON_LANES; ++L) p[L] = 0.0;
    const long c1 = c0 + HODLR3D_CANON_CHUNK < n ? c0 + HODLR3D_CANON_CHUNK : n;
    for (long i = c0; i < c1; ++i) p[i % HODLR3D_CANON_LANES] += f(i);
    for (int o = 16; o >= 1; o >>= 1) {
      double q[HODLR3D_CANON_LANES];
      for (int L = 0; L < HODLR3D_CANON_LANES; ++L) q[L] = p[L] + p[L ^ o];
      for (int L = 0; L < HODLR3D_CANON_LANES; ++L) p[L] = q[L];
    }
    total = c0 == 0 ? p[0] : total + p[0];
  }
  return total;
}
#endif
#endif
