// The FP64 form streamed: A x and A^T x, one right-hand side per pass, FP64
// factors grouped by box exactly like the FP32 copies of the few-column
// engine (matvec_gemv.cu: same element offsets, the same work lists and
// index tables), FP64 near-field blocks in the near-field layout, FP64 FMAs.
//
// On GB300 the FP64 pipe retires about 2 lane FMAs per clock per SM (~0.6 T
// FMA/s), so a product over the 7.7e9 factor entries of the 64^3 operator
// needs ~13 ms of FP64 arithmetic whatever the kernel; the 62 GB of FP64
// factors stream in ~9 ms.  The kernels therefore keep the FP64 pipe busy:
// 16-byte streaming loads (two entries), two FMAs each, many rows in flight
// per warp, FP64 sums throughout (no FP32 step anywhere).
//
// Reference: HODLR3D::MatVecProduct (src/HODLR3D.cpp:21-27) and its stages
// (src/HODLR3DTree.cpp:1647-1805): far field per interaction-list pair,
// V^T x then U t, near field over the leaf's neighbours and itself, sum
// over the levels, owner write in the original order.
#include "matvec.h"

namespace h3d {
namespace {

constexpr int THREADS = 256;
constexpr int WARPS = THREADS / 32;
constexpr int RW = 8;  // rows per warp in the per-leaf output kernels

__device__ __forceinline__ double2 ld2(const double* p, int64_t i) {
  return __ldcs(reinterpret_cast<const double2*>(p) + i);
}

__device__ __forceinline__ int level_of(int64_t box, int levels) {
  int j = 0;
  while (j < levels && level_base(j + 1) <= box) ++j;
  return j;
}

// Dot products of up to P G rows (row q at rowp + q ld, q < nrows, G = 32 /
// LW) of len2 16-byte groups with vec (2 len2 doubles, 16-byte aligned): LW
// lanes per row, P rows per lane; out(q, sum) is called once per row by its
// group's first lane.  Every lane of the warp takes part.
template <int LW, int P, class Out>
__device__ __forceinline__ void rows_dot(const double* __restrict__ rowp, int64_t ld, int nrows, int len2,
                                         const double* vec, Out&& out) {
  constexpr int G = 32 / LW;
  const int lane = threadIdx.x & 31, g = lane / LW, li = lane % LW;
  double acc[P];
#pragma unroll
  for (int q = 0; q < P; ++q) acc[q] = 0.0;
  for (int k2 = li; k2 < len2; k2 += LW) {
    const double2 x = reinterpret_cast<const double2*>(vec)[k2];
    double2 v[P];
#pragma unroll
    for (int q = 0; q < P; ++q) {
      const int row = q * G + g;
      v[q] = row < nrows ? ld2(rowp + (int64_t)row * ld, k2) : make_double2(0.0, 0.0);
    }
#pragma unroll
    for (int q = 0; q < P; ++q) {
      acc[q] = fma(v[q].x, x.x, acc[q]);
      acc[q] = fma(v[q].y, x.y, acc[q]);
    }
  }
#pragma unroll
  for (int o = LW / 2; o > 0; o >>= 1)
#pragma unroll
    for (int q = 0; q < P; ++q) acc[q] += __shfl_xor_sync(0xffffffffu, acc[q], o);
  if (li == 0) {
#pragma unroll
    for (int q = 0; q < P; ++q)
      if (q * G + g < nrows) out(q * G + g, acc[q]);
  }
}

// rows_dot over RB rows per warp pass, the lanes per row chosen from the row
// length (rows of at most 32 groups take fewer lanes, more rows at once)
template <int RB, class Out>
__device__ __forceinline__ void rows_dot_any(const double* __restrict__ rowp, int64_t ld, int nrows,
                                             int len2, const double* vec, Out&& out) {
  if (len2 > 16)
    rows_dot<32, RB>(rowp, ld, nrows, len2, vec, out);
  else if (len2 > 8)
    rows_dot<16, (RB / 2 > 0 ? RB / 2 : 1)>(rowp, ld, nrows, len2, vec, out);
  else if (len2 > 4)
    rows_dot<8, (RB / 4 > 0 ? RB / 4 : 1)>(rowp, ld, nrows, len2, vec, out);
  else
    rows_dot<4, (RB / 8 > 0 ? RB / 8 : 1)>(rowp, ld, nrows, len2, vec, out);
}

// x (original order, one column) -> tree order
__global__ void k64_gather(int64_t N, const double* __restrict__ X, const int32_t* __restrict__ perm,
                           double* __restrict__ xg) {
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t < N) xg[t] = X[perm[t]];
}

// nr rows of a V stack window (row stride m4, len2 groups) times xs, LW
// lanes per row, 4 rows per lane, the warps taking row blocks in turn; row R's
// sum goes to put(R, sum)
template <int LW, class Put>
__device__ __forceinline__ void vt_pass(const double* __restrict__ V, int64_t m4, int nr, int len2,
                                        const double* xs, Put&& put) {
  constexpr int P = 4, RB = P * (32 / LW);
  const int w = threadIdx.x >> 5;
  for (int b0 = w * RB; b0 < nr; b0 += WARPS * RB)
    rows_dot<LW, P>(V + (int64_t)b0 * m4, m4, min(RB, nr - b0), len2, xs,
                    [&](int q, double s) { put(b0 + q, s); });
}

// Forward far field, input side: item (a, ci, r0, nr): rows r0 .. r0 + nr of
// source box a's V stack over columns [ci CW, + CW) times x of those points;
// row R goes to its T row (vrow_t) or, for boxes wider than one chunk, to
// partial row R of chunk ci.
__global__ void __launch_bounds__(THREADS) k64_vt(GemvOp op, const double* __restrict__ v64,
                                                  const int4* __restrict__ items,
                                                  const double* __restrict__ xg, double* __restrict__ t,
                                                  double* __restrict__ part) {
  __shared__ __align__(16) double xs[kGemvCols];
  const int4 it = items[blockIdx.x];
  const int64_t a = it.x;
  const int ci = it.y, r0 = it.z, nr = it.w;
  const int d = op.levels;
  const int j = level_of(a, d);
  const int sh = 3 * (d - j);
  const int64_t ka = a - level_base(j);
  const int64_t box0 = op.leaf_off[ka << sh];
  const int64_t m = op.leaf_off[(ka + 1) << sh] - box0, m4 = (m + 3) & ~int64_t(3);
  const int64_t col0 = (int64_t)ci * kGemvCols;
  const int cl = (int)min((int64_t)kGemvCols, m4 - col0);
  for (int e = threadIdx.x; e < cl; e += THREADS) xs[e] = col0 + e < m ? xg[box0 + col0 + e] : 0.0;
  __syncthreads();
  const int rows_a = op.vbox_rows[a];
  const int64_t pofs = op.vpofs[a];
  const int32_t* vr = op.vrow_t + op.vrow0[a] + r0;
  const double* V = v64 + op.vbox_off[a] + (int64_t)r0 * m4 + col0;
  double* dst = pofs < 0 ? t : part + pofs + (int64_t)ci * rows_a + r0;
  const int len2 = cl / 2;
  auto put = [&](int R, double s) {
    if (pofs < 0)
      dst[vr[R]] = s;
    else
      dst[R] = s;
  };
  // lanes per row from the row length: about 8 groups (16 FMAs) per lane, so
  // that the FP64 additions of the lane reduction (log2 of the lanes) stay a
  // small share of the FP64 pipe's work (leaf-level stacks: 64 entries per row)
  if (len2 >= 256)
    vt_pass<32>(V, m4, nr, len2, xs, put);
  else if (len2 >= 128)
    vt_pass<16>(V, m4, nr, len2, xs, put);
  else if (len2 >= 64)
    vt_pass<8>(V, m4, nr, len2, xs, put);
  else if (len2 >= 32)
    vt_pass<4>(V, m4, nr, len2, xs, put);
  else
    vt_pass<2>(V, m4, nr, len2, xs, put);
}

// T rows of the source boxes wider than one chunk: sum of their chunk partials
__global__ void k64_tred(GemvOp op, const int32_t* __restrict__ boxes, const double* __restrict__ part,
                         double* __restrict__ t) {
  const int64_t a = boxes[blockIdx.x];
  const int d = op.levels;
  const int j = level_of(a, d);
  const int sh = 3 * (d - j);
  const int64_t ka = a - level_base(j);
  const int64_t m = op.leaf_off[(ka + 1) << sh] - op.leaf_off[ka << sh];
  const int nch = (int)((((m + 3) & ~int64_t(3)) + kGemvCols - 1) / kGemvCols);
  const int rows_a = op.vbox_rows[a];
  const double* p = part + op.vpofs[a];
  const int32_t* vr = op.vrow_t + op.vrow0[a];
  for (int R = threadIdx.x; R < rows_a; R += blockDim.x) {
    double s = 0.0;
    for (int ci = 0; ci < nch; ++ci) s += p[(int64_t)ci * rows_a + R];
    t[vr[R]] = s;
  }
}

// x of leaf k's neighbour leaves (slots 0..25, 26 = itself; absent ones
// skipped) in the column order of its near-field matrix, each zero padded to
// round4(ne).  The caller synchronises.
__device__ __forceinline__ void stage_near(const GemvOp& op, int64_t k, const double* xg, double* xn) {
  const int lane = threadIdx.x & 31;
  for (int sl = threadIdx.x >> 5; sl < 27; sl += WARPS) {
    const int64_t off = op.near_off[27 * k + sl];
    if (off < 0) continue;
    const int64_t col = off - op.near_base[k];
    const int64_t nn = sl < 26 ? (int64_t)op.nbr_leaf[k * 26 + sl] : k;
    const int64_t e0 = op.leaf_off[nn];
    const int ne = (int)(op.leaf_off[nn + 1] - e0), ne4 = (ne + 3) & ~3;
    for (int e = lane; e < ne4; e += 32) xn[col + e] = e < ne ? xg[e0 + e] : 0.0;
  }
}

// Near field of rows [i0, i0 + nrows) of leaf k into the warp's sums ya[q]
__device__ __forceinline__ void near_rows(const GemvOp& op, const double* knear64, int64_t k, int i0,
                                          int nrows, const double* xn, double* ya) {
  const int ld = op.near_ld[k];
  rows_dot_any<RW>(knear64 + op.near_base[k] + (int64_t)i0 * ld, ld, nrows, ld / 2, xn,
                   [&](int q, double s) { ya[q] += s; });
  __syncwarp();
}

// Forward output side, one block per leaf: the U rows of the d ancestor
// boxes times their T, then the near field; written once in the original
// order.
__global__ void __launch_bounds__(THREADS) k64_uy(GemvOp op, const double* __restrict__ u64,
                                                  const double* __restrict__ knear64,
                                                  const double* __restrict__ xg,
                                                  const double* __restrict__ t, double* __restrict__ y) {
  extern __shared__ __align__(16) unsigned char smem[];
  double* yacc = reinterpret_cast<double*>(smem);  // WARPS x RW
  double* xn = yacc + WARPS * RW;                  // 27 x max_leaf4
  const int64_t k = blockIdx.x;
  const int d = op.levels;
  const int64_t t0 = op.leaf_off[k];
  const int nk = (int)(op.leaf_off[k + 1] - t0);
  if (nk == 0) return;
  __shared__ int64_t lu[kMaxLevels + 1], lt[kMaxLevels + 1];
  __shared__ int lr[kMaxLevels + 1];
  if (threadIdx.x >= 1 && threadIdx.x <= d) {
    const int j = threadIdx.x, sh = 3 * (d - j);
    const int64_t kb = k >> sh, b = level_base(j) + kb;
    const int R = op.rbox[b];
    lr[j] = R;
    lu[j] = op.ubox_off[b] + (t0 - op.leaf_off[kb << sh]) * R;
    lt[j] = op.tbase[b];
  }
  stage_near(op, k, xg, xn);
  __syncthreads();
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  double* ya = yacc + w * RW;
  for (int i0 = w * RW; i0 < nk; i0 += WARPS * RW) {
    const int nrows = min(RW, nk - i0);
    if (lane < RW) ya[lane] = 0.0;
    __syncwarp();
    for (int j = 1; j <= d; ++j) {
      const int R = lr[j];
      if (R == 0) continue;
      rows_dot_any<RW>(u64 + lu[j] + (int64_t)i0 * R, R, nrows, R / 2, t + lt[j],
                       [&](int q, double s) { ya[q] += s; });
      __syncwarp();
    }
    near_rows(op, knear64, k, i0, nrows, xn, ya);
    if (lane < nrows) y[op.perm[t0 + i0 + lane]] = ya[lane];
    __syncwarp();
  }
}

// Transposed far field, output-box side: item (b, ci): T_b += U_b^T x over
// rows [ci CWT, + CWT) of target box b, lanes owning 16-byte column groups;
// T in the row order of the V stacks (or chunk partials).
__global__ void __launch_bounds__(THREADS) k64_ut(GemvOp op, const double* __restrict__ u64,
                                                  const int2* __restrict__ items,
                                                  const double* __restrict__ xg, double* __restrict__ tt,
                                                  double* __restrict__ part) {
  __shared__ double xs[kGemvRowsT];
  const int2 it = items[blockIdx.x];
  const int64_t b = it.x;
  const int ci = it.y;
  const int d = op.levels;
  const int j = level_of(b, d);
  const int sh = 3 * (d - j);
  const int64_t kb = b - level_base(j);
  const int64_t box0 = op.leaf_off[kb << sh];
  const int64_t n = op.leaf_off[(kb + 1) << sh] - box0;
  const int64_t i0 = (int64_t)ci * kGemvRowsT;
  const int nr = (int)min((int64_t)kGemvRowsT, n - i0);
  for (int e = threadIdx.x; e < nr; e += THREADS) xs[e] = xg[box0 + i0 + e];
  __syncthreads();
  const int R = op.rbox[b], len2 = R / 2;
  const int64_t pofs = op.upofs[b];
  const double* U = u64 + op.ubox_off[b] + i0 * R;
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  for (int k2b = w * 32; k2b < len2; k2b += WARPS * 32) {
    const int k2 = k2b + lane;
    const bool live = k2 < len2;
    double s0 = 0.0, s1 = 0.0;
    constexpr int UN = 8;
    int i = 0;
    for (; i + UN <= nr; i += UN) {
      double2 v[UN];
#pragma unroll
      for (int u = 0; u < UN; ++u) v[u] = live ? ld2(U, (int64_t)(i + u) * len2 + k2) : make_double2(0.0, 0.0);
#pragma unroll
      for (int u = 0; u < UN; ++u) {
        s0 = fma(v[u].x, xs[i + u], s0);
        s1 = fma(v[u].y, xs[i + u], s1);
      }
    }
    for (; i < nr; ++i) {
      const double2 v = live ? ld2(U, (int64_t)i * len2 + k2) : make_double2(0.0, 0.0);
      s0 = fma(v.x, xs[i], s0);
      s1 = fma(v.y, xs[i], s1);
    }
    if (!live) continue;
    if (pofs < 0) {
      const int32_t* tv = op.trow_v + op.tbase[b] + 2 * k2;
      if (tv[0] >= 0) tt[tv[0]] = s0;
      if (tv[1] >= 0) tt[tv[1]] = s1;
    } else {
      double* p = part + pofs + (int64_t)ci * R + 2 * k2;
      p[0] = s0;
      p[1] = s1;
    }
  }
}

__global__ void k64_tred_t(GemvOp op, const int32_t* __restrict__ boxes, const double* __restrict__ part,
                           double* __restrict__ tt) {
  const int64_t b = boxes[blockIdx.x];
  const int d = op.levels;
  const int j = level_of(b, d);
  const int sh = 3 * (d - j);
  const int64_t kb = b - level_base(j);
  const int64_t n = op.leaf_off[(kb + 1) << sh] - op.leaf_off[kb << sh];
  const int nch = (int)((n + kGemvRowsT - 1) / kGemvRowsT);
  const int R = op.rbox[b];
  const double* p = part + op.upofs[b];
  const int32_t* tv = op.trow_v + op.tbase[b];
  for (int k = threadIdx.x; k < R; k += blockDim.x) {
    const int32_t sv = tv[k];
    if (sv < 0) continue;
    double s = 0.0;
    for (int ci = 0; ci < nch; ++ci) s += p[(int64_t)ci * R + k];
    tt[sv] = s;
  }
}

// Transposed output side, one block per leaf: for every level the leaf's
// columns of the ancestor's V stack times the stack's T rows (warps split the
// rows, lanes own 16-byte column groups of the leaf's window), then the near
// field (the built-in kernels are symmetric, so the near blocks serve both
// directions); written once in the original order.
__global__ void __launch_bounds__(THREADS) k64_vy(GemvOp op, const double* __restrict__ v64,
                                                  const double* __restrict__ knear64,
                                                  const double* __restrict__ xg,
                                                  const double* __restrict__ tt, double* __restrict__ y) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int nep = op.max_leaf4 + 4;                // the leaf's window, 4-aligned start
  double* far = reinterpret_cast<double*>(smem);   // WARPS x nep
  double* yacc = far + WARPS * nep;                // WARPS x RW
  double* xn = yacc + WARPS * RW;                  // 27 x max_leaf4
  const int64_t k = blockIdx.x;
  const int d = op.levels;
  const int64_t t0 = op.leaf_off[k];
  const int nk = (int)(op.leaf_off[k + 1] - t0);
  if (nk == 0) return;
  __shared__ int64_t lv[kMaxLevels + 1], lm[kMaxLevels + 1], lt[kMaxLevels + 1];
  __shared__ int lrows[kMaxLevels + 1], llen[kMaxLevels + 1], lsh[kMaxLevels + 1];
  if (threadIdx.x >= 1 && threadIdx.x <= d) {
    const int j = threadIdx.x, sh = 3 * (d - j);
    const int64_t ka = k >> sh, a = level_base(j) + ka;
    const int64_t box0 = op.leaf_off[ka << sh];
    const int64_t c0 = t0 - box0, w0 = c0 & ~int64_t(3);
    lrows[j] = op.vbox_rows[a];
    lm[j] = (op.leaf_off[(ka + 1) << sh] - box0 + 3) & ~int64_t(3);
    llen[j] = (int)((((c0 + nk + 3) & ~int64_t(3)) - w0) / 2);
    lsh[j] = (int)(c0 - w0);
    lv[j] = op.vbox_off[a] + w0;
    lt[j] = op.vrow0[a];
  }
  for (int e = threadIdx.x; e < WARPS * nep; e += THREADS) far[e] = 0.0;
  stage_near(op, k, xg, xn);
  __syncthreads();
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  double* fw = far + (int64_t)w * nep;
  for (int j = 1; j <= d; ++j) {
    const int rows = lrows[j];
    if (rows == 0) continue;
    const int64_t m4 = lm[j];
    const int len2 = llen[j], shift = lsh[j];
    const double* V = v64 + lv[j];
    const double* T = tt + lt[j];
    for (int kw = 0; kw < len2; kw += 32) {
      const int k2 = kw + lane;
      const bool live = k2 < len2;
      double s0 = 0.0, s1 = 0.0;
      constexpr int UN = 4;
      int v = w;
      for (; v + (UN - 1) * WARPS < rows; v += UN * WARPS) {
        double2 f[UN];
        double tv[UN];
#pragma unroll
        for (int u = 0; u < UN; ++u) {
          const int64_t r = v + u * WARPS;
          f[u] = live ? ld2(V + r * m4, k2) : make_double2(0.0, 0.0);
          tv[u] = T[r];
        }
#pragma unroll
        for (int u = 0; u < UN; ++u) {
          s0 = fma(f[u].x, tv[u], s0);
          s1 = fma(f[u].y, tv[u], s1);
        }
      }
      for (; v < rows; v += WARPS) {
        const double2 f = live ? ld2(V + (int64_t)v * m4, k2) : make_double2(0.0, 0.0);
        const double tv = T[v];
        s0 = fma(f.x, tv, s0);
        s1 = fma(f.y, tv, s1);
      }
      if (live) {
        const int i = 2 * k2 - shift;  // leaf-local point of s0
        if (i >= 0 && i < nk) fw[i] += s0;
        if (i + 1 >= 0 && i + 1 < nk) fw[i + 1] += s1;
      }
    }
  }
  __syncthreads();
  double* ya = yacc + w * RW;
  for (int i0 = w * RW; i0 < nk; i0 += WARPS * RW) {
    const int nrows = min(RW, nk - i0);
    if (lane < RW) {
      double s = 0.0;
      if (lane < nrows)
        for (int u = 0; u < WARPS; ++u) s += far[(int64_t)u * nep + i0 + lane];
      ya[lane] = s;
    }
    __syncwarp();
    near_rows(op, knear64, k, i0, nrows, xn, ya);
    if (lane < nrows) y[op.perm[t0 + i0 + lane]] = ya[lane];
    __syncwarp();
  }
}

// FP64 near-field blocks in the near-field layout: the entry formula of the
// FP64 form from the tree-ordered FP64 points, the diagonal value on the
// leaf's own diagonal, zero in the padding columns
__global__ void k_near64(const int32_t* __restrict__ leaf_off, NearOp nr,
                         const int64_t* __restrict__ near_off, const int32_t* __restrict__ near_ld,
                         double* __restrict__ Knear) {
  const int64_t k = blockIdx.x;
  const int sl = blockIdx.y;
  const int64_t off = near_off[k * 27 + sl];
  if (off < 0) return;
  const int64_t nn = sl < 26 ? (int64_t)nr.nbr_leaf[k * 26 + sl] : k;
  const int64_t t0 = leaf_off[k], e0 = leaf_off[nn];
  const int nk = (int)(leaf_off[k + 1] - t0), ne = (int)(leaf_off[nn + 1] - e0);
  const int nep = (ne + 3) & ~3;
  const int64_t ld = near_ld[k];
  for (int e = threadIdx.x; e < nk * nep; e += blockDim.x) {
    const int i = e / nep, j = e - i * nep;
    double v = 0.0;
    if (j < ne) {
      const int64_t ti = t0 + i, ej = e0 + j;
      v = (nn == k && i == j) ? nr.kd.diag
                              : entry64_offdiag(nr.kd, __dsub_rn(nr.xs[ti], nr.xs[ej]),
                                                __dsub_rn(nr.ys[ti], nr.ys[ej]),
                                                __dsub_rn(nr.zs[ti], nr.zs[ej]));
    }
    Knear[off + (int64_t)i * ld + j] = v;
  }
}

// FP64 copies of the factors grouped by box: U of pair p (n x r, column-major)
// row-major with row stride us[p] at u[p], zeros up to round4(r); V of pair p
// (m x r) column-major with leading dimension round4(m) at v[p]
__global__ void k_group_u64(const double* const* __restrict__ u64, double* const* __restrict__ ug,
                            const int32_t* __restrict__ nsize, const int32_t* __restrict__ us,
                            const int32_t* __restrict__ rank) {
  const int64_t p = blockIdx.x;
  const int r = rank[p];
  if (r <= 0) return;
  const int rp = (r + 3) & ~3;
  const int64_t n = nsize[p], st = us[p];
  const double* src = u64[p];
  double* dst = ug[p];
  for (int64_t e = threadIdx.x; e < n * rp; e += blockDim.x) {
    const int64_t i = e / rp;
    const int l = (int)(e - i * rp);
    dst[i * st + l] = l < r ? src[(int64_t)l * n + i] : 0.0;
  }
}

__global__ void k_group_v64(const double* const* __restrict__ v64, double* const* __restrict__ vg,
                            const int32_t* __restrict__ msize, const int32_t* __restrict__ rank) {
  const int64_t p = blockIdx.x;
  const int r = rank[p];
  if (r <= 0) return;
  const int64_t m = msize[p], mp = (m + 3) & ~int64_t(3);
  const double* src = v64[p];
  double* dst = vg[p];
  for (int64_t e = threadIdx.x; e < mp * r; e += blockDim.x) {
    const int64_t l = e / mp, i = e - l * mp;
    dst[e] = i < m ? src[l * m + i] : 0.0;
  }
}

}  // namespace

size_t f64_smem_bytes(int max_leaf4) {
  // the transposed output kernel takes the most
  return sizeof(double) * ((size_t)WARPS * (max_leaf4 + 4) + WARPS * RW + 27 * (size_t)max_leaf4);
}

int launch_group_f64(cudaStream_t s, int64_t npairs, const double* const* u64, double* const* ug,
                     const int32_t* nsize, const int32_t* us, const double* const* v64,
                     double* const* vg, const int32_t* msize, const int32_t* rank) {
  if (npairs <= 0) return 0;
  k_group_u64<<<(unsigned)npairs, 256, 0, s>>>(u64, ug, nsize, us, rank);
  k_group_v64<<<(unsigned)npairs, 256, 0, s>>>(v64, vg, msize, rank);
  return 2;
}

int launch_near64(cudaStream_t s, int64_t nleaf, const int32_t* leaf_off, const NearOp& near,
                  const int64_t* near_off, const int32_t* near_ld, double* Knear64) {
  if (nleaf == 0) return 0;
  k_near64<<<dim3((unsigned)nleaf, 27), 256, 0, s>>>(leaf_off, near, near_off, near_ld, Knear64);
  return 1;
}

int launch_matvec_f64(cudaStream_t s, const GemvOp& op, const F64Buffers& B, const double* x,
                      double* y, bool trans, MatvecProfiler* prof) {
  static int attr_done[kMaxDevices] = {};
  const int dev = current_device();
  const size_t shv = f64_smem_bytes(op.max_leaf4);
  if ((int)shv > attr_done[dev]) {
    cudaFuncSetAttribute(k64_uy, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)shv);
    cudaFuncSetAttribute(k64_vy, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)shv);
    attr_done[dev] = (int)shv;
  }
  const size_t shu = sizeof(double) * ((size_t)WARPS * RW + 27 * (size_t)op.max_leaf4);
  int launches = 0;
  const int64_t N = op.N;
  if (prof) prof->begin(s);
  k64_gather<<<(unsigned)((N + 255) / 256), 256, 0, s>>>(N, x, op.perm, B.xg);
  ++launches;
  if (prof) prof->mark(s, "gather64");
  if (!trans) {
    if (B.n_vt_items > 0) {
      k64_vt<<<(unsigned)B.n_vt_items, THREADS, 0, s>>>(op, B.v64, B.vt_items, B.xg, B.t, B.p);
      ++launches;
      if (prof) prof->mark(s, "vt64");
    }
    if (B.n_vt_upper > 0) {
      k64_tred<<<(unsigned)B.n_vt_upper, 256, 0, s>>>(op, B.vt_upper, B.p, B.t);
      ++launches;
      if (prof) prof->mark(s, "tred64");
    }
    k64_uy<<<(unsigned)op.nleaf, THREADS, shu, s>>>(op, B.u64, B.knear64, B.xg, B.t, y);
    ++launches;
    if (prof) prof->mark(s, "uy64");
  } else {
    if (B.n_ut_items > 0) {
      k64_ut<<<(unsigned)B.n_ut_items, THREADS, 0, s>>>(op, B.u64, B.ut_items, B.xg, B.tt, B.pt);
      ++launches;
      if (prof) prof->mark(s, "ut64");
    }
    if (B.n_ut_upper > 0) {
      k64_tred_t<<<(unsigned)B.n_ut_upper, 256, 0, s>>>(op, B.ut_upper, B.pt, B.tt);
      ++launches;
      if (prof) prof->mark(s, "tred_t64");
    }
    k64_vy<<<(unsigned)op.nleaf, THREADS, shv, s>>>(op, B.v64, B.knear64, B.xg, B.tt, y);
    ++launches;
    if (prof) prof->mark(s, "vy64");
  }
  return launches;
}

}  // namespace h3d
