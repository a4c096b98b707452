// Mixed-precision product for 1, 2 or 4 right-hand sides on the CUDA cores:
// A X and A^T X streamed from the box-grouped FP32 factors.
//
// Reference: HODLR3D::MatVecProduct (src/HODLR3D.cpp:21-27) and the stages of
// src/HODLR3DTree.cpp:1647-1805 (far field V^T q then U T per interaction-list
// pair, near field over the leaf's neighbours and itself).
//
// With few right-hand sides the product is a set of matrix-vector products:
// every factor entry is used 1..4 times, so the FP32 factors (and the FP32
// near-field blocks) are read once, with 16-byte streaming loads, and the
// arithmetic is FP32 FMAs (FP64 on GB300 runs at a small fraction of the FP32
// rate).  Sums: FP32 within a row segment of at most 1024 columns (or a chunk
// of 256 rows, or 64 rows of a stack), FP64 across segments, chunks, levels
// and near blocks.
//
// Layouts (grouped by box, all levels numbered together):
//   U of target box b: row-major n_b x R_b at u32 + ubox_off[b], the pairs of
//     b side by side (each rank padded to a multiple of 4 with zero columns);
//   V of source box a: row-major (sum of ranks) x round4(m_a) at
//     v32 + vbox_off[a], one row per column of each V_p, pairs in the order of
//     a's reverse list (zero columns past m_a);
//   T = V^T X (forward): R_b x NR at row tbase[b], the same grouping as U;
//     vrow_t[v] maps row v of the V stacks (numbered over all boxes, box a's
//     from vrow0[a]) to its row of T, trow_v the other way (-1: padding);
//   T = U^T X (transposed): in the row order of the V stacks, so that each
//     stack meets its T rows contiguously;
//   X: N x NR FP32 in tree order; near blocks: nk x round4(ne) row-major.
// Stages:
//   forward   gather; vt (items: source box, 1024-column chunk, 2048 rows):
//             T rows or chunk partials; tred (boxes wider than one chunk);
//             uy (one block per leaf): far field U T of the d levels, near
//             field, written once in the original order.
//   transpose gather; ut (items: target box, 256-row chunk): T = U^T X or
//             chunk partials; tred_t; vy (one block per leaf): far field of
//             the leaf's columns of the d level stacks V T, near field (the
//             built-in kernels are symmetric, so the near blocks serve both).
#include "matvec.h"

#include <algorithm>

namespace h3d {
namespace {

constexpr int THREADS = 256;
constexpr int WARPS = THREADS / 32;
constexpr int ROWS = 8;  // rows per warp in the row-segment products

__device__ __forceinline__ int level_of(int64_t box, int levels) {
  int j = 0;
  while (j < levels && level_base(j + 1) <= box) ++j;
  return j;
}

// x[e][c]: 4 consecutive rows of an [row][NR] FP32 vector (16-byte aligned)
template <int NR>
__device__ __forceinline__ void load_rows4(const float* p, float (&x)[4][NR]) {
  const float4* q = reinterpret_cast<const float4*>(p);
  if constexpr (NR == 1) {
    const float4 a = q[0];
    x[0][0] = a.x; x[1][0] = a.y; x[2][0] = a.z; x[3][0] = a.w;
  } else if constexpr (NR == 2) {
    const float4 a = q[0], b = q[1];
    x[0][0] = a.x; x[0][1] = a.y; x[1][0] = a.z; x[1][1] = a.w;
    x[2][0] = b.x; x[2][1] = b.y; x[3][0] = b.z; x[3][1] = b.w;
  } else {
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      const float4 a = q[e];
      x[e][0] = a.x; x[e][1] = a.y; x[e][2] = a.z; x[e][3] = a.w;
    }
  }
}

template <int NR>
__device__ __forceinline__ void fma_row4(float (&acc)[NR], const float4 v, const float (&x)[4][NR]) {
#pragma unroll
  for (int c = 0; c < NR; ++c) {
    acc[c] = fmaf(v.x, x[0][c], acc[c]);
    acc[c] = fmaf(v.y, x[1][c], acc[c]);
    acc[c] = fmaf(v.z, x[2][c], acc[c]);
    acc[c] = fmaf(v.w, x[3][c], acc[c]);
  }
}

// Dot products of up to P (32 / LW) rows (row q at rowp + q ld, q < nrows) of
// len4 16-byte groups with the vector vec ([4 len4][NR], shared or global
// memory), LW lanes per row, P rows per lane; out(p, q, acc) is called once
// per row q by its group's first lane (p: the lane's row slot, q = p G + g).
// Every lane of the warp takes part (warp-uniform arguments).
template <int NR, int LW, int P = ROWS * LW / 32, class Out>
__device__ __forceinline__ void seg_rows(const float* __restrict__ rowp, int64_t ld, int nrows,
                                         int len4, const float* vec, Out&& out) {
  constexpr int G = 32 / LW;
  const int lane = threadIdx.x & 31, g = lane / LW, li = lane % LW;
  float acc[P][NR];
#pragma unroll
  for (int q = 0; q < P; ++q)
#pragma unroll
    for (int c = 0; c < NR; ++c) acc[q][c] = 0.f;
  for (int k4 = li; k4 < len4; k4 += LW) {
    float x[4][NR];
    load_rows4<NR>(vec + (int64_t)k4 * 4 * NR, x);
    float4 v[P];
#pragma unroll
    for (int q = 0; q < P; ++q) {
      const int row = q * G + g;
      v[q] = row < nrows ? __ldcs(reinterpret_cast<const float4*>(rowp + row * ld) + k4)
                         : make_float4(0.f, 0.f, 0.f, 0.f);
    }
#pragma unroll
    for (int q = 0; q < P; ++q) fma_row4<NR>(acc[q], v[q], x);
  }
#pragma unroll
  for (int o = LW / 2; o > 0; o >>= 1)
#pragma unroll
    for (int q = 0; q < P; ++q)
#pragma unroll
      for (int c = 0; c < NR; ++c) acc[q][c] += __shfl_xor_sync(0xffffffffu, acc[q][c], o);
  if (li == 0) {
#pragma unroll
    for (int q = 0; q < P; ++q)
      if (q * G + g < nrows) out(q, q * G + g, acc[q]);
  }
}

template <int NR, class Out>
__device__ __forceinline__ void seg_rows_any(const float* __restrict__ rowp, int64_t ld, int nrows,
                                             int len4, const float* vec, Out&& out) {
  if (len4 > 16)
    seg_rows<NR, 32>(rowp, ld, nrows, len4, vec, out);
  else if (len4 > 8)
    seg_rows<NR, 16>(rowp, ld, nrows, len4, vec, out);
  else if (len4 > 4)
    seg_rows<NR, 8>(rowp, ld, nrows, len4, vec, out);
  else
    seg_rows<NR, 4>(rowp, ld, nrows, len4, vec, out);
}

// ----------------------------------------------------------------------------
template <int NR>
__global__ void k_gather(int64_t N, int nrhs, const double* __restrict__ X, int64_t ldx,
                         const int32_t* __restrict__ perm, float* __restrict__ xg) {
  const int64_t o = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (o >= N * NR) return;
  const int64_t t = o / NR;
  const int c = (int)(o - t * NR);
  xg[o] = c < nrhs ? (float)X[c * ldx + perm[t]] : 0.f;
}

// nr rows of a V stack (row stride m4) times xs, 8 rows per lane and 8 G per
// warp pass; row R's sums go to dst[map[R] NR + c] (map null: dst[R NR + c]).
template <int NR, int LW>
__device__ __forceinline__ void vt_rows(const float* __restrict__ V, int64_t m4, int nr, int len4,
                                        const float* xs, float* __restrict__ dst,
                                        const int32_t* __restrict__ map) {
  constexpr int G = 32 / LW, RB = 8 * G;  // rows per warp pass
  const int w = threadIdx.x >> 5, g = (threadIdx.x & 31) / LW;
  for (int b0 = w * RB; b0 < nr; b0 += WARPS * RB) {
    // output rows of this lane's row slots, loaded ahead of the row data
    int orow[8];
#pragma unroll
    for (int p = 0; p < 8; ++p) {
      const int R = b0 + p * G + g;
      orow[p] = map && R < nr ? map[R] : R;
    }
    seg_rows<NR, LW, 8>(V + b0 * m4, m4, min(RB, nr - b0), len4, xs,
                        [&](int p, int, const float(&s)[NR]) {
                          float* o = dst + (int64_t)orow[p] * NR;
#pragma unroll
                          for (int c = 0; c < NR; ++c) o[c] = s[c];
                        });
  }
}

// Forward far field, input side: for item (a, ci, r0, nr), rows r0 .. r0+nr of
// source box a's V stack over columns [ci CW, + CW) times X of those points.
template <int NR>
__global__ void __launch_bounds__(THREADS) k_vt(GemvOp op, const int4* __restrict__ items,
                                                const float* __restrict__ xg, float* __restrict__ T,
                                                float* __restrict__ P) {
  __shared__ __align__(16) float xs[kGemvCols * NR];
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
  for (int e = threadIdx.x; e < cl * NR; e += THREADS) {
    const int col = e / NR;
    xs[e] = col0 + col < m ? xg[(box0 + col0) * NR + e] : 0.f;
  }
  __syncthreads();
  const int rows_a = op.vbox_rows[a];
  const int64_t pofs = op.vpofs[a];
  const int32_t* vr = op.vrow_t + op.vrow0[a];
  const float* V = op.v32 + op.vbox_off[a] + (int64_t)r0 * m4 + col0;
  // rows r0 + R of the item go to T row vr[R] or to partial row R of chunk ci
  float* dst = pofs < 0 ? T : P + (pofs + (int64_t)ci * rows_a + r0) * NR;
  const int32_t* map = pofs < 0 ? vr + r0 : nullptr;
  const int len4 = cl / 4;
  if (len4 > 16)
    vt_rows<NR, 32>(V, m4, nr, len4, xs, dst, map);
  else if (len4 > 8)
    vt_rows<NR, 16>(V, m4, nr, len4, xs, dst, map);
  else if (len4 > 4)
    vt_rows<NR, 8>(V, m4, nr, len4, xs, dst, map);
  else
    vt_rows<NR, 4>(V, m4, nr, len4, xs, dst, map);
}

// T rows of a source box wider than one chunk: FP64 sum of its chunk partials
template <int NR>
__global__ void k_tred(GemvOp op, const int32_t* __restrict__ boxes, const float* __restrict__ P,
                       float* __restrict__ T) {
  const int64_t a = boxes[blockIdx.x];
  const int d = op.levels;
  const int j = level_of(a, d);
  const int sh = 3 * (d - j);
  const int64_t ka = a - level_base(j);
  const int64_t m = op.leaf_off[(ka + 1) << sh] - op.leaf_off[ka << sh];
  const int nch = (int)((((m + 3) & ~int64_t(3)) + kGemvCols - 1) / kGemvCols);
  const int rows_a = op.vbox_rows[a];
  const float* src = P + op.vpofs[a] * NR;
  const int32_t* vr = op.vrow_t + op.vrow0[a];
  for (int o = threadIdx.x; o < rows_a * NR; o += blockDim.x) {
    double s = 0.0;
    for (int ci = 0; ci < nch; ++ci) s += (double)src[(int64_t)ci * rows_a * NR + o];
    const int R = o / NR;
    T[(int64_t)vr[R] * NR + (o - R * NR)] = (float)s;
  }
}

// The X of leaf k's neighbour leaves (slots 0..25, 26 = itself; absent ones
// skipped) in the column order of its near-field matrix: slot by slot, each
// zero padded to round4(ne) rows, xn[col][c].  The caller synchronises.
template <int NR>
__device__ __forceinline__ void stage_near_x(const GemvOp& op, int64_t k, const float* __restrict__ xg,
                                             float* xn) {
  const int lane = threadIdx.x & 31;
  for (int sl = threadIdx.x >> 5; sl < 27; sl += WARPS) {  // one slot per warp
    const int64_t off = op.near_off[27 * k + sl];
    if (off < 0) continue;
    const int64_t col = off - op.near_base[k];
    const int64_t nn = sl < 26 ? (int64_t)op.nbr_leaf[k * 26 + sl] : k;
    const int64_t e0 = op.leaf_off[nn];
    const int ne = (int)(op.leaf_off[nn + 1] - e0), ne4 = (ne + 3) & ~3;
    for (int e = lane; e < ne4 * NR; e += 32) xn[col * NR + e] = e < ne * NR ? xg[e0 * NR + e] : 0.f;
  }
}

// Near field of rows [i0, i0 + nrows) of leaf k (leaf-local): one segment of
// its near-field matrix, added to the warp's FP64 row sums ya[row][c].
template <int NR>
__device__ __forceinline__ void near_rows(const GemvOp& op, int64_t k, int i0, int nrows,
                                          const float* xn, double* ya) {
  const int ld = op.near_ld[k];
  seg_rows_any<NR>(op.knear + op.near_base[k] + (int64_t)i0 * ld, ld, nrows, ld / 4, xn,
                   [&](int, int q, const float(&s)[NR]) {
#pragma unroll
                     for (int c = 0; c < NR; ++c) ya[q * NR + c] += (double)s[c];
                   });
  __syncwarp();
}

// Forward output side, one block per leaf k: y = sum over the levels of
// U_b(rows) T_b + near field, FP64 across segments, written in the original
// order.
template <int NR>
__global__ void __launch_bounds__(THREADS) k_uy(GemvOp op, const float* __restrict__ xg,
                                                const float* __restrict__ T, int nrhs,
                                                double* __restrict__ Y, int64_t ldy) {
  extern __shared__ __align__(16) unsigned char smem[];
  double* yacc = reinterpret_cast<double*>(smem);                         // WARPS x ROWS x NR
  float* xn = reinterpret_cast<float*>(smem + sizeof(double) * WARPS * ROWS * NR);  // 27 max_leaf4 x NR
  const int64_t k = blockIdx.x;
  const int d = op.levels;
  const int64_t t0 = op.leaf_off[k];
  const int nk = (int)(op.leaf_off[k + 1] - t0);
  if (nk == 0) return;
  // per level: the U row of the leaf's first point, R_b, the T rows (times NR)
  __shared__ int64_t lu[kMaxLevels + 1], lt[kMaxLevels + 1];
  __shared__ int lr[kMaxLevels + 1];
  if (threadIdx.x >= 1 && threadIdx.x <= d) {
    const int j = threadIdx.x, sh = 3 * (d - j);
    const int64_t kb = k >> sh, b = level_base(j) + kb;
    const int R = op.rbox[b];
    lr[j] = R;
    lu[j] = op.ubox_off[b] + (t0 - op.leaf_off[kb << sh]) * R;
    lt[j] = op.tbase[b] * NR;
  }
  stage_near_x<NR>(op, k, xg, xn);
  __syncthreads();
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  double* ya = yacc + w * ROWS * NR;
  for (int i0 = w * ROWS; i0 < nk; i0 += WARPS * ROWS) {
    const int nrows = min(ROWS, nk - i0);
    for (int e = lane; e < ROWS * NR; e += 32) ya[e] = 0.0;
    __syncwarp();
    for (int j = 1; j <= d; ++j) {
      const int R = lr[j];
      if (R == 0) continue;
      const float* U = op.u32 + lu[j] + (int64_t)i0 * R;
      seg_rows_any<NR>(U, R, nrows, R / 4, T + lt[j], [&](int, int q, const float(&s)[NR]) {
#pragma unroll
        for (int c = 0; c < NR; ++c) ya[q * NR + c] += (double)s[c];
      });
      __syncwarp();
    }
    near_rows<NR>(op, k, i0, nrows, xn, ya);
    for (int e = lane; e < nrows * NR; e += 32) {
      const int q = e / NR, c = e - q * NR;
      if (c < nrhs) Y[c * ldy + op.perm[t0 + i0 + q]] = ya[e];
    }
    __syncwarp();
  }
}

// Transposed far field, output-box side: for item (b, ci), T_b += U_b^T X over
// rows [ci CWT, + CWT) of target box b (one 16-byte column group per lane,
// windows of 128 columns per warp).
template <int NR>
__global__ void __launch_bounds__(THREADS) k_ut(GemvOp op, const int2* __restrict__ items,
                                                const float* __restrict__ xg, float* __restrict__ T,
                                                float* __restrict__ P) {
  __shared__ __align__(16) float xs[kGemvRowsT * NR];
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
  for (int e = threadIdx.x; e < nr * NR; e += THREADS) xs[e] = xg[(box0 + i0) * NR + e];
  __syncthreads();
  const int R = op.rbox[b], len4 = R / 4;
  const int64_t pofs = op.upofs[b];
  const float* U = op.u32 + op.ubox_off[b] + i0 * R;
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  for (int k4b = w * 32; k4b < len4; k4b += WARPS * 32) {
    const int k4 = k4b + lane;
    const bool live = k4 < len4;
    float acc[4][NR];
#pragma unroll
    for (int e = 0; e < 4; ++e)
#pragma unroll
      for (int c = 0; c < NR; ++c) acc[e][c] = 0.f;
    const float4* col = reinterpret_cast<const float4*>(U) + k4;
    int i = 0;
    for (; i + 4 <= nr; i += 4) {
      float4 v[4];
#pragma unroll
      for (int u = 0; u < 4; ++u)
        v[u] = live ? __ldcs(col + (int64_t)(i + u) * len4) : make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
      for (int u = 0; u < 4; ++u)
#pragma unroll
        for (int c = 0; c < NR; ++c) {
          const float xv = xs[(i + u) * NR + c];
          acc[0][c] = fmaf(v[u].x, xv, acc[0][c]);
          acc[1][c] = fmaf(v[u].y, xv, acc[1][c]);
          acc[2][c] = fmaf(v[u].z, xv, acc[2][c]);
          acc[3][c] = fmaf(v[u].w, xv, acc[3][c]);
        }
    }
    for (; i < nr; ++i) {
      const float4 v = live ? __ldcs(col + (int64_t)i * len4) : make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
      for (int c = 0; c < NR; ++c) {
        const float xv = xs[i * NR + c];
        acc[0][c] = fmaf(v.x, xv, acc[0][c]);
        acc[1][c] = fmaf(v.y, xv, acc[1][c]);
        acc[2][c] = fmaf(v.z, xv, acc[2][c]);
        acc[3][c] = fmaf(v.w, xv, acc[3][c]);
      }
    }
    if (live && pofs < 0) {
      // rows of T in the order of the V stacks (padding rows dropped)
      const int32_t* tv = op.trow_v + op.tbase[b] + 4 * k4;
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        const int32_t sv = tv[e];
        if (sv >= 0)
#pragma unroll
          for (int c = 0; c < NR; ++c) T[(int64_t)sv * NR + c] = acc[e][c];
      }
    } else if (live) {
      float* dst = P + (pofs + (int64_t)ci * R + 4 * (int64_t)k4) * NR;
#pragma unroll
      for (int e = 0; e < 4; ++e)
#pragma unroll
        for (int c = 0; c < NR; ++c) dst[e * NR + c] = acc[e][c];
    }
  }
}

template <int NR>
__global__ void k_tred_t(GemvOp op, const int32_t* __restrict__ boxes, const float* __restrict__ P,
                         float* __restrict__ T) {
  const int64_t b = boxes[blockIdx.x];
  const int d = op.levels;
  const int j = level_of(b, d);
  const int sh = 3 * (d - j);
  const int64_t kb = b - level_base(j);
  const int64_t n = op.leaf_off[(kb + 1) << sh] - op.leaf_off[kb << sh];
  const int nch = (int)((n + kGemvRowsT - 1) / kGemvRowsT);
  const int R = op.rbox[b];
  const float* src = P + op.upofs[b] * NR;
  const int32_t* tv = op.trow_v + op.tbase[b];
  for (int o = threadIdx.x; o < R * NR; o += blockDim.x) {
    const int k = o / NR;
    const int32_t sv = tv[k];
    if (sv < 0) continue;
    double s = 0.0;
    for (int ci = 0; ci < nch; ++ci) s += (double)src[(int64_t)ci * R * NR + o];
    T[(int64_t)sv * NR + (o - k * NR)] = (float)s;
  }
}

// Transposed output side, one block per leaf k: for each level the leaf's
// columns of the V stack of its ancestor box times that stack's T rows (lanes
// own 16-byte column groups, rows split over lane groups and warps; FP32 over
// at most 64 rows, FP64 beyond), then the near field; written once.
template <int NR, int LW>
__device__ __forceinline__ void stack_cols(const float* __restrict__ V, int64_t m4, int rows,
                                           const float* __restrict__ Tv, int len4, int shift, int nk,
                                           double* fw) {
  constexpr int G = 32 / LW, U = 8;
  const int lane = threadIdx.x & 31, g = lane / LW, li = lane % LW, w = threadIdx.x >> 5;
  for (int kw = 0; kw < len4; kw += LW) {
    const int k4 = kw + li;
    const bool live = k4 < len4;
    double a64[4][NR];
#pragma unroll
    for (int e = 0; e < 4; ++e)
#pragma unroll
      for (int c = 0; c < NR; ++c) a64[e][c] = 0.0;
    const int stride = WARPS * G;
    for (int v0 = w * G + g; v0 < rows; v0 += 64 * stride) {
      float acc[4][NR];
#pragma unroll
      for (int e = 0; e < 4; ++e)
#pragma unroll
        for (int c = 0; c < NR; ++c) acc[e][c] = 0.f;
      const int vend = min(rows, v0 + 64 * stride);
      int v = v0;
      for (; v + (U - 1) * stride < vend; v += U * stride) {
        float4 f[U];
        float tv[U][NR];
#pragma unroll
        for (int u = 0; u < U; ++u) {
          f[u] = live ? __ldcs(reinterpret_cast<const float4*>(V + (int64_t)(v + u * stride) * m4) + k4)
                      : make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
          for (int c = 0; c < NR; ++c) tv[u][c] = Tv[(int64_t)(v + u * stride) * NR + c];
        }
#pragma unroll
        for (int u = 0; u < U; ++u)
#pragma unroll
          for (int c = 0; c < NR; ++c) {
            acc[0][c] = fmaf(f[u].x, tv[u][c], acc[0][c]);
            acc[1][c] = fmaf(f[u].y, tv[u][c], acc[1][c]);
            acc[2][c] = fmaf(f[u].z, tv[u][c], acc[2][c]);
            acc[3][c] = fmaf(f[u].w, tv[u][c], acc[3][c]);
          }
      }
      for (; v < vend; v += stride) {
        const float4 f = live ? __ldcs(reinterpret_cast<const float4*>(V + (int64_t)v * m4) + k4)
                              : make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
        for (int c = 0; c < NR; ++c) {
          const float tv = Tv[(int64_t)v * NR + c];
          acc[0][c] = fmaf(f.x, tv, acc[0][c]);
          acc[1][c] = fmaf(f.y, tv, acc[1][c]);
          acc[2][c] = fmaf(f.z, tv, acc[2][c]);
          acc[3][c] = fmaf(f.w, tv, acc[3][c]);
        }
      }
#pragma unroll
      for (int e = 0; e < 4; ++e)
#pragma unroll
        for (int c = 0; c < NR; ++c) a64[e][c] += (double)acc[e][c];
    }
    // the lane groups of the warp hold the same columns
#pragma unroll
    for (int o = 16; o >= LW; o >>= 1)
#pragma unroll
      for (int e = 0; e < 4; ++e)
#pragma unroll
        for (int c = 0; c < NR; ++c) a64[e][c] += __shfl_xor_sync(0xffffffffu, a64[e][c], o);
    if (g == 0 && live) {
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        const int i = 4 * k4 + e - shift;  // leaf-local point
        if (i >= 0 && i < nk)
#pragma unroll
          for (int c = 0; c < NR; ++c) fw[i * NR + c] += a64[e][c];
      }
    }
  }
}

template <int NR>
__global__ void __launch_bounds__(THREADS) k_vy(GemvOp op, const float* __restrict__ xg,
                                                const float* __restrict__ T, int nrhs,
                                                double* __restrict__ Y, int64_t ldy) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int nep = op.max_leaf4;
  double* yacc = reinterpret_cast<double*>(smem);                          // WARPS x ROWS x NR
  double* far = yacc + WARPS * ROWS * NR;                                  // WARPS x nep x NR
  float* xn = reinterpret_cast<float*>(far + (int64_t)WARPS * nep * NR);   // <= 27 nep x NR
  const int64_t k = blockIdx.x;
  const int d = op.levels;
  const int64_t t0 = op.leaf_off[k];
  const int nk = (int)(op.leaf_off[k + 1] - t0);
  if (nk == 0) return;
  // per level: the stack rows, the leaf's first column group of the stack,
  // its row length, the leaf's column window and the stack's T rows
  __shared__ int64_t lv[kMaxLevels + 1], lm[kMaxLevels + 1], lt[kMaxLevels + 1];
  __shared__ int lrows[kMaxLevels + 1], llen[kMaxLevels + 1], lsh[kMaxLevels + 1];
  if (threadIdx.x >= 1 && threadIdx.x <= d) {
    const int j = threadIdx.x, sh = 3 * (d - j);
    const int64_t ka = k >> sh, a = level_base(j) + ka;
    const int64_t box0 = op.leaf_off[ka << sh];
    const int64_t c0 = t0 - box0, w0 = c0 & ~int64_t(3);
    lrows[j] = op.vbox_rows[a];
    lm[j] = (op.leaf_off[(ka + 1) << sh] - box0 + 3) & ~int64_t(3);
    llen[j] = (int)((((c0 + nk + 3) & ~int64_t(3)) - w0) / 4);
    lsh[j] = (int)(c0 - w0);
    lv[j] = op.vbox_off[a] + w0;
    lt[j] = op.vrow0[a] * NR;
  }
  for (int e = threadIdx.x; e < WARPS * nep * NR; e += THREADS) far[e] = 0.0;
  stage_near_x<NR>(op, k, xg, xn);
  __syncthreads();
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  double* fw = far + (int64_t)w * nep * NR;
  for (int j = 1; j <= d; ++j) {
    const int rows = lrows[j];
    if (rows == 0) continue;
    const int64_t m4 = lm[j];
    const int len4 = llen[j];
    const float* V = op.v32 + lv[j];
    const float* Tv = T + lt[j];
    const int shift = lsh[j];
    if (len4 > 16)
      stack_cols<NR, 32>(V, m4, rows, Tv, len4, shift, nk, fw);
    else if (len4 > 8)
      stack_cols<NR, 16>(V, m4, rows, Tv, len4, shift, nk, fw);
    else if (len4 > 4)
      stack_cols<NR, 8>(V, m4, rows, Tv, len4, shift, nk, fw);
    else
      stack_cols<NR, 4>(V, m4, rows, Tv, len4, shift, nk, fw);
    __syncwarp();
  }
  __syncthreads();
  double* ya = yacc + w * ROWS * NR;
  for (int i0 = w * ROWS; i0 < nk; i0 += WARPS * ROWS) {
    const int nrows = min(ROWS, nk - i0);
    for (int e = lane; e < ROWS * NR; e += 32) {
      double s = 0.0;
      if (e < nrows * NR)
        for (int u = 0; u < WARPS; ++u) s += far[((int64_t)u * nep + i0) * NR + e];
      ya[e] = s;
    }
    __syncwarp();
    near_rows<NR>(op, k, i0, nrows, xn, ya);
    for (int e = lane; e < nrows * NR; e += 32) {
      const int q = e / NR, c = e - q * NR;
      if (c < nrhs) Y[c * ldy + op.perm[t0 + i0 + q]] = ya[e];
    }
    __syncwarp();
  }
}

template <int NR>
int run(cudaStream_t s, const GemvOp& op, const GemvBuffers& B, const double* X, int64_t ldx,
        double* Y, int64_t ldy, int nrhs, bool trans, MatvecProfiler* prof) {
  int launches = 0;
  const int64_t N = op.N;
  if (prof) prof->begin(s);
  k_gather<NR><<<(unsigned)((N * NR + 255) / 256), 256, 0, s>>>(N, nrhs, X, ldx, op.perm, B.xg);
  ++launches;
  if (prof) prof->mark(s, "gather");
  if (!trans) {
    if (B.n_vt_items > 0) {
      k_vt<NR><<<(unsigned)B.n_vt_items, THREADS, 0, s>>>(op, B.vt_items, B.xg, B.t, B.p);
      ++launches;
      if (prof) prof->mark(s, "vt");
    }
    if (B.n_vt_upper > 0) {
      k_tred<NR><<<(unsigned)B.n_vt_upper, 256, 0, s>>>(op, B.vt_upper, B.p, B.t);
      ++launches;
      if (prof) prof->mark(s, "tred");
    }
    const size_t shm = gemv_uy_smem(op.max_leaf4, NR);
    k_uy<NR><<<(unsigned)op.nleaf, THREADS, shm, s>>>(op, B.xg, B.t, nrhs, Y, ldy);
    ++launches;
    if (prof) prof->mark(s, "uy");
  } else {
    if (B.n_ut_items > 0) {
      k_ut<NR><<<(unsigned)B.n_ut_items, THREADS, 0, s>>>(op, B.ut_items, B.xg, B.tt, B.pt);
      ++launches;
      if (prof) prof->mark(s, "ut");
    }
    if (B.n_ut_upper > 0) {
      k_tred_t<NR><<<(unsigned)B.n_ut_upper, 256, 0, s>>>(op, B.ut_upper, B.pt, B.tt);
      ++launches;
      if (prof) prof->mark(s, "tred_t");
    }
    const size_t shm = gemv_vy_smem(op.max_leaf4, NR);
    k_vy<NR><<<(unsigned)op.nleaf, THREADS, shm, s>>>(op, B.xg, B.tt, nrhs, Y, ldy);
    ++launches;
    if (prof) prof->mark(s, "vy");
  }
  return launches;
}

template <int NR>
void set_attrs(int max_leaf4) {
  static int done = 0;  // largest shared-memory request set so far, per instantiation
  const int uy = (int)gemv_uy_smem(max_leaf4, NR), vy = (int)gemv_vy_smem(max_leaf4, NR);
  if (std::max(uy, vy) <= done) return;
  cudaFuncSetAttribute(k_uy<NR>, cudaFuncAttributeMaxDynamicSharedMemorySize, uy);
  cudaFuncSetAttribute(k_vy<NR>, cudaFuncAttributeMaxDynamicSharedMemorySize, vy);
  done = std::max(uy, vy);
}

}  // namespace

size_t gemv_uy_smem(int max_leaf4, int nr) {
  return sizeof(double) * WARPS * ROWS * nr + sizeof(float) * 27 * (size_t)max_leaf4 * nr;
}
size_t gemv_vy_smem(int max_leaf4, int nr) {
  return gemv_uy_smem(max_leaf4, nr) + sizeof(double) * WARPS * (size_t)max_leaf4 * nr;
}

int launch_matvec_gemv(cudaStream_t s, const GemvOp& op, const GemvBuffers& B, const double* X,
                       int64_t ldx, double* Y, int64_t ldy, int nrhs, bool trans,
                       MatvecProfiler* prof) {
  if (nrhs <= 1) {
    set_attrs<1>(op.max_leaf4);
    return run<1>(s, op, B, X, ldx, Y, ldy, nrhs, trans, prof);
  }
  if (nrhs <= 2) {
    set_attrs<2>(op.max_leaf4);
    return run<2>(s, op, B, X, ldx, Y, ldy, nrhs, trans, prof);
  }
  set_attrs<4>(op.max_leaf4);
  return run<4>(s, op, B, X, ldx, Y, ldy, nrhs, trans, prof);
}

}  // namespace h3d
