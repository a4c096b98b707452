// Few-column products on the CUDA cores (passes of 1, 2, 4 or, for the mixed
// transpose, 8 right-hand sides), A X and A^T X streamed from the
// box-grouped FP32 factors, in two arithmetics:
//   mixed  FP32 factors and near field, FP32 FMAs (DF = false);
//   fp64x  FP64-accurate: every FP64 entry a as the pair hi + lo of FP32
//          values (hi the mixed form's copy, lo = a - hi rounded, relative
//          error 2^-46), x as xh + xl, products hi xh made exact by an FMA
//          and summed with TwoSum (Knuth), the small terms hi xl + lo xh
//          and the rounding errors in a second FP32 sum (DF = true).  On
//          GB300 the FP32 pipes run ~60x the FP64 rate, so this streams at
//          the bandwidth of the 8 bytes per entry where FP64 FMAs could not.
//
// Reference: HODLR3D::MatVecProduct (src/HODLR3D.cpp:21-27) and the stages of
// src/HODLR3DTree.cpp:1647-1805 (far field V^T q then U T per interaction-list
// pair, near field over the leaf's neighbours and itself).
//
// Every factor entry is used once per column of the pass, so the factors and
// near-field blocks are read once per pass, with 16-byte streaming loads.  Sums: within a row segment of
// at most 1024 columns (or a chunk of 256 rows, or 64 rows of a stack) in the
// arithmetic above, FP64 across segments, chunks, levels and near blocks.
//
// Layouts (grouped by box, all levels numbered together):
//   U of target box b: row-major n_b x R_b at u32 + ubox_off[b], the pairs of
//     b side by side (each rank padded to a multiple of 4 with zero columns);
//   V of source box a: row-major (sum of ranks) x round4(m_a) at
//     v32 + vbox_off[a], one row per column of each V_p, pairs in the order of
//     a's reverse list (zero columns past m_a);
//   lo parts (fp64x): the same layouts at u32lo, v32lo, knearlo;
//   T = V^T X (forward): R_b x NR at row tbase[b], the same grouping as U;
//     vrow_t[v] maps row v of the V stacks (numbered over all boxes, box a's
//     from vrow0[a]) to its row of T, trow_v the other way (-1: padding);
//   T = U^T X (transposed): in the row order of the V stacks, so that each
//     stack meets its T rows contiguously;
//   X: N x NR FP32 in tree order; near field of leaf k: nk x near_ld[k]
//     row-major at knear + near_base[k] (its neighbours' blocks side by side).
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

// rows per warp in the output kernels (fewer for the fp64x form, whose
// accumulators and loads are twice as many, and for 8 columns)
template <int NR, bool DF>
__host__ __device__ constexpr int rows_per_warp() {
  return DF || NR == 8 ? 4 : 8;
}

__device__ __forceinline__ int level_of(int64_t box, int levels) {
  int j = 0;
  while (j < levels && level_base(j + 1) <= box) ++j;
  return j;
}

// s + c += v x, v = hi + lo, x = xh + xl (lo, xl only in the fp64x form)
template <bool DF>
__device__ __forceinline__ void mac(float& s, float& c, float v, float lo, float xh, float xl) {
  if constexpr (!DF) {
    s = fmaf(v, xh, s);
  } else {
    const float p = __fmul_rn(v, xh);
    const float e = fmaf(v, xh, -p);  // v xh = p + e exactly
    const float t = __fadd_rn(s, p);  // TwoSum: s + p = t + err exactly
    const float bb = __fsub_rn(t, s);
    const float err = __fadd_rn(__fsub_rn(s, __fsub_rn(t, bb)), __fsub_rn(p, bb));
    s = t;
    c = __fadd_rn(c, __fadd_rn(err, fmaf(v, xl, fmaf(lo, xh, e))));
  }
}

// (s, c) += (s2, c2)
template <bool DF>
__device__ __forceinline__ void merge(float& s, float& c, float s2, float c2) {
  if constexpr (!DF) {
    s += s2;
  } else {
    const float t = __fadd_rn(s, s2);
    const float bb = __fsub_rn(t, s);
    const float err = __fadd_rn(__fsub_rn(s, __fsub_rn(t, bb)), __fsub_rn(s2, bb));
    s = t;
    c = __fadd_rn(__fadd_rn(c, c2), err);
  }
}

template <bool DF>
__device__ __forceinline__ double value(float s, float c) {
  if constexpr (DF) return (double)s + (double)c;
  return (double)s;
}

// the FP32 pair of an FP64 value: hi = its rounding, lo = the remainder
__device__ __forceinline__ void split_pair(double v, float& hi, float& lo) {
  hi = (float)v;
  lo = (float)(v - (double)hi);
}

// (s, c) renormalised to hi + lo with hi = fl(s + c), in FP32 only (TwoSum):
// the few-column kernels keep FP64 instructions out of per-row work, GB300's
// FP64 pipe being ~1/60 of its FP32 rate
__device__ __forceinline__ void renorm(float s, float c, float& hi, float& lo) {
  const float t = __fadd_rn(s, c);
  const float bb = __fsub_rn(t, s);
  hi = t;
  lo = __fadd_rn(__fsub_rn(s, __fsub_rn(t, bb)), __fsub_rn(c, bb));
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
  } else if constexpr (NR == 4) {
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      const float4 a = q[e];
      x[e][0] = a.x; x[e][1] = a.y; x[e][2] = a.z; x[e][3] = a.w;
    }
  } else {
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      const float4 a = q[2 * e], b = q[2 * e + 1];
      x[e][0] = a.x; x[e][1] = a.y; x[e][2] = a.z; x[e][3] = a.w;
      x[e][4] = b.x; x[e][5] = b.y; x[e][6] = b.z; x[e][7] = b.w;
    }
  }
}

__device__ __forceinline__ float comp(const float4& v, int e) {
  return e == 0 ? v.x : e == 1 ? v.y : e == 2 ? v.z : v.w;
}

__device__ __forceinline__ float4 ld4(const float* p, int64_t i) {
  return __ldcs(reinterpret_cast<const float4*>(p) + i);
}

// Dot products of up to P G (G = 32 / LW) rows (row q at rowp + q ld, q < nrows) of
// len4 16-byte groups with the vector vec ([4 len4][NR], shared or global
// memory), LW lanes per row, P rows per lane; out(p, q, s, c) is called once
// per row q with its sums s[NR] + c[NR] (c: the mixed form passes s again, unused) by its
// group's first lane (p: the lane's row slot, q = p G + g).  fp64x: rowl, vecl
// hold the lo parts.  Every lane of the warp takes part (warp-uniform
// arguments).
template <int NR, bool DF, int LW, int P, bool COL_OUTER = false, class Out>
__device__ __forceinline__ void seg_rows(const float* __restrict__ rowp, const float* __restrict__ rowl,
                                         int64_t ld, int nrows, int len4, const float* vec,
                                         const float* vecl, Out&& out) {
  constexpr int G = 32 / LW;
  const int lane = threadIdx.x & 31, g = lane / LW, li = lane % LW;
  if constexpr (!DF) {
    // mixed form: one FP32 sum per row and column
    float acc[P][NR];
#pragma unroll
    for (int q = 0; q < P; ++q)
#pragma unroll
      for (int k = 0; k < NR; ++k) acc[q][k] = 0.f;
    for (int k4 = li; k4 < len4; k4 += LW) {
      float x[4][NR];
      load_rows4<NR>(vec + (int64_t)k4 * 4 * NR, x);
      float4 v[P];
#pragma unroll
      for (int q = 0; q < P; ++q) {
        const int row = q * G + g;
        v[q] = row < nrows ? ld4(rowp + row * ld, k4) : make_float4(0.f, 0.f, 0.f, 0.f);
      }
      // the same FMA sequence per row and column in either loop order (so the
      // results are identical); the order only steers the compiler's
      // scheduling, measured per kernel
      if constexpr (COL_OUTER) {
#pragma unroll
        for (int q = 0; q < P; ++q)
#pragma unroll
          for (int k = 0; k < NR; ++k) {
            acc[q][k] = fmaf(v[q].x, x[0][k], acc[q][k]);
            acc[q][k] = fmaf(v[q].y, x[1][k], acc[q][k]);
            acc[q][k] = fmaf(v[q].z, x[2][k], acc[q][k]);
            acc[q][k] = fmaf(v[q].w, x[3][k], acc[q][k]);
          }
      } else {
#pragma unroll
        for (int q = 0; q < P; ++q)
#pragma unroll
          for (int e = 0; e < 4; ++e)
#pragma unroll
            for (int k = 0; k < NR; ++k) acc[q][k] = fmaf(comp(v[q], e), x[e][k], acc[q][k]);
      }
    }
#pragma unroll
    for (int o = LW / 2; o > 0; o >>= 1)
#pragma unroll
      for (int q = 0; q < P; ++q)
#pragma unroll
        for (int k = 0; k < NR; ++k) acc[q][k] += __shfl_xor_sync(0xffffffffu, acc[q][k], o);
    if (li == 0) {
#pragma unroll
      for (int q = 0; q < P; ++q)
        if (q * G + g < nrows) out(q, q * G + g, acc[q], acc[q]);  // (the second sum is unused)
    }
  } else {
    // fp64x: the pair sums (s, c) of every row and column
    float s[P][NR], c[P][NR];
#pragma unroll
    for (int q = 0; q < P; ++q)
#pragma unroll
      for (int k = 0; k < NR; ++k) s[q][k] = c[q][k] = 0.f;
    for (int k4 = li; k4 < len4; k4 += LW) {
      float x[4][NR], xl[4][NR];
      load_rows4<NR>(vec + (int64_t)k4 * 4 * NR, x);
      load_rows4<NR>(vecl + (int64_t)k4 * 4 * NR, xl);
      float4 v[P], vl[P];
#pragma unroll
      for (int q = 0; q < P; ++q) {
        const int row = q * G + g;
        const bool ok = row < nrows;
        v[q] = ok ? ld4(rowp + row * ld, k4) : make_float4(0.f, 0.f, 0.f, 0.f);
        vl[q] = ok ? ld4(rowl + row * ld, k4) : make_float4(0.f, 0.f, 0.f, 0.f);
      }
      if constexpr (COL_OUTER) {
#pragma unroll
        for (int q = 0; q < P; ++q)
#pragma unroll
          for (int k = 0; k < NR; ++k)
#pragma unroll
            for (int e = 0; e < 4; ++e)
              mac<true>(s[q][k], c[q][k], comp(v[q], e), comp(vl[q], e), x[e][k], xl[e][k]);
      } else {
#pragma unroll
        for (int q = 0; q < P; ++q)
#pragma unroll
          for (int e = 0; e < 4; ++e)
#pragma unroll
            for (int k = 0; k < NR; ++k)
              mac<true>(s[q][k], c[q][k], comp(v[q], e), comp(vl[q], e), x[e][k], xl[e][k]);
      }
    }
#pragma unroll
    for (int o = LW / 2; o > 0; o >>= 1)
#pragma unroll
      for (int q = 0; q < P; ++q)
#pragma unroll
        for (int k = 0; k < NR; ++k) {
          const float s2 = __shfl_xor_sync(0xffffffffu, s[q][k], o);
          const float c2 = __shfl_xor_sync(0xffffffffu, c[q][k], o);
          merge<true>(s[q][k], c[q][k], s2, c2);
        }
    if (li == 0) {
#pragma unroll
      for (int q = 0; q < P; ++q)
        if (q * G + g < nrows) out(q, q * G + g, s[q], c[q]);
    }
  }
}

// seg_rows with the lanes per row chosen from the row length, RW rows per warp
template <int NR, bool DF, int RW, class Out>
__device__ __forceinline__ void seg_rows_any(const float* __restrict__ rowp, const float* __restrict__ rowl,
                                             int64_t ld, int nrows, int len4, const float* vec,
                                             const float* vecl, Out&& out) {
  if (len4 > 16)
    seg_rows<NR, DF, 32, RW>(rowp, rowl, ld, nrows, len4, vec, vecl, out);
  else if (len4 > 8)
    seg_rows<NR, DF, 16, RW / 2>(rowp, rowl, ld, nrows, len4, vec, vecl, out);
  else if (len4 > 4)
    seg_rows<NR, DF, 8, (RW / 4 > 0 ? RW / 4 : 1)>(rowp, rowl, ld, nrows, len4, vec, vecl, out);
  else
    seg_rows<NR, DF, 4, (RW / 8 > 0 ? RW / 8 : 1)>(rowp, rowl, ld, nrows, len4, vec, vecl, out);
}

// ----------------------------------------------------------------------------
// X in tree order, FP32 (and, fp64x, the lo parts in xl)
template <int NR, bool DF>
__global__ void k_gather(int64_t N, int nrhs, const double* __restrict__ X, int64_t ldx,
                         const int32_t* __restrict__ perm, float* __restrict__ xg,
                         float* __restrict__ xl) {
  const int64_t o = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (o >= N * NR) return;
  const int64_t t = o / NR;
  const int c = (int)(o - t * NR);
  const double v = c < nrhs ? X[c * ldx + perm[t]] : 0.0;
  if constexpr (DF) {
    split_pair(v, xg[o], xl[o]);
  } else {
    xg[o] = (float)v;
  }
}

// stores an output sum: FP32 (mixed) or its FP32 pair (fp64x)
template <bool DF>
__device__ __forceinline__ void put_t(float* th, float* tl, int64_t i, double v) {
  if constexpr (DF) {
    split_pair(v, th[i], tl[i]);
  } else {
    th[i] = (float)v;
  }
}

// Work buffers of one arithmetic: X, T (forward), T (transposed, V-stack
// order), chunk partials (FP32 for mixed, FP64 for fp64x)
struct Bufs {
  float* xg;
  float* xl;
  float* t;
  float* tl;
  float* tt;
  float* ttl;
  void* p;
  void* pt;
};

// nr rows of a V stack (row stride m4) times xs, P rows per lane and P G per
// warp pass; row R's sums go to T row map[R] of dst (fp64x: hi in dst, lo in
// dstl), or (map null) to partial row R of dst (fp64x: as FP32 pairs).
template <int NR, bool DF, int LW>
__device__ __forceinline__ void vt_rows(const float* __restrict__ V, const float* __restrict__ Vl,
                                        int64_t m4, int nr, int len4, const float* xs,
                                        const float* xsl, float* __restrict__ dst,
                                        float* __restrict__ dstl, const int32_t* __restrict__ map) {
  constexpr int P = DF || NR == 8 ? 4 : 8;
  constexpr int G = 32 / LW, RB = P * G;  // rows per warp pass
  const int w = threadIdx.x >> 5, g = (threadIdx.x & 31) / LW;
  for (int b0 = w * RB; b0 < nr; b0 += WARPS * RB) {
    // output rows of this lane's row slots, loaded ahead of the row data
    int orow[P];
#pragma unroll
    for (int p = 0; p < P; ++p) {
      const int R = b0 + p * G + g;
      orow[p] = map && R < nr ? map[R] : R;
    }
    seg_rows<NR, DF, LW, P, true>(V + b0 * m4, DF ? Vl + b0 * m4 : nullptr, m4, min(RB, nr - b0), len4, xs,
                            xsl, [&](int p, int, const float(&sv)[NR], const float(&cv)[NR]) {
                              if constexpr (!DF) {
                                float* o = dst + (int64_t)orow[p] * NR;
#pragma unroll
                                for (int k = 0; k < NR; ++k) o[k] = sv[k];
                              } else if (map) {
                                const int64_t o = (int64_t)orow[p] * NR;
#pragma unroll
                                for (int k = 0; k < NR; ++k) renorm(sv[k], cv[k], dst[o + k], dstl[o + k]);
                              } else {
                                float* o = dst + (int64_t)orow[p] * 2 * NR;  // FP32 pairs
#pragma unroll
                                for (int k = 0; k < NR; ++k) {
                                  o[2 * k] = sv[k];
                                  o[2 * k + 1] = cv[k];
                                }
                              }
                            });
  }
}

// Forward far field, input side: for item (a, ci, r0, nr), rows r0 .. r0+nr of
// source box a's V stack over columns [ci CW, + CW) times X of those points.
template <int NR, bool DF>
__global__ void __launch_bounds__(THREADS) k_vt(GemvOp op, const int4* __restrict__ items, Bufs B) {
  __shared__ __align__(16) float xs[kGemvCols * NR];
  __shared__ __align__(16) float xsl[DF ? kGemvCols * NR : 4];
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
    const bool in = col0 + e / NR < m;
    xs[e] = in ? B.xg[(box0 + col0) * NR + e] : 0.f;
    if constexpr (DF) xsl[e] = in ? B.xl[(box0 + col0) * NR + e] : 0.f;
  }
  __syncthreads();
  const int rows_a = op.vbox_rows[a];
  const int64_t pofs = op.vpofs[a];
  const int32_t* vr = op.vrow_t + op.vrow0[a];
  const int64_t vofs = op.vbox_off[a] + (int64_t)r0 * m4 + col0;
  const float* V = op.v32 + vofs;
  const float* Vl = DF ? op.v32lo + vofs : nullptr;
  // rows r0 + R of the item go to T row vr[R] or to partial row R of chunk ci
  const int32_t* map = pofs < 0 ? vr + r0 : nullptr;
  float* dst = map ? B.t
                   : static_cast<float*>(B.p) + (pofs + (int64_t)ci * rows_a + r0) * NR * (DF ? 2 : 1);
  float* dstl = map ? B.tl : nullptr;
  const int len4 = cl / 4;
  if (len4 > 16)
    vt_rows<NR, DF, 32>(V, Vl, m4, nr, len4, xs, xsl, dst, dstl, map);
  else if (len4 > 8)
    vt_rows<NR, DF, 16>(V, Vl, m4, nr, len4, xs, xsl, dst, dstl, map);
  else if (len4 > 4)
    vt_rows<NR, DF, 8>(V, Vl, m4, nr, len4, xs, xsl, dst, dstl, map);
  else
    vt_rows<NR, DF, 4>(V, Vl, m4, nr, len4, xs, xsl, dst, dstl, map);
}

// partial i (FP32, or in the fp64x form an FP32 pair) as FP64
template <bool DF>
__device__ __forceinline__ double partial(const void* p, int64_t i) {
  const float* f = static_cast<const float*>(p);
  if constexpr (DF) return (double)f[2 * i] + (double)f[2 * i + 1];
  return (double)f[i];
}

// T rows of a source box wider than one chunk: FP64 sum of its chunk partials
template <int NR, bool DF>
__global__ void k_tred(GemvOp op, const int32_t* __restrict__ boxes, Bufs B) {
  const int64_t a = boxes[blockIdx.x];
  const int d = op.levels;
  const int j = level_of(a, d);
  const int sh = 3 * (d - j);
  const int64_t ka = a - level_base(j);
  const int64_t m = op.leaf_off[(ka + 1) << sh] - op.leaf_off[ka << sh];
  const int nch = (int)((((m + 3) & ~int64_t(3)) + kGemvCols - 1) / kGemvCols);
  const int rows_a = op.vbox_rows[a];
  const int64_t base = op.vpofs[a] * NR;
  const int32_t* vr = op.vrow_t + op.vrow0[a];
  for (int o = threadIdx.x; o < rows_a * NR; o += blockDim.x) {
    double s = 0.0;
    for (int ci = 0; ci < nch; ++ci) s += partial<DF>(B.p, base + (int64_t)ci * rows_a * NR + o);
    const int R = o / NR;
    put_t<DF>(B.t, B.tl, (int64_t)vr[R] * NR + (o - R * NR), s);
  }
}

// The X of leaf k's neighbour leaves (slots 0..25, 26 = itself; absent ones
// skipped) in the column order of its near-field matrix: slot by slot, each
// zero padded to round4(ne) rows, xn[col][c] (and the lo parts in xnl).  The
// caller synchronises.
template <int NR, bool DF>
__device__ __forceinline__ void stage_near_x(const GemvOp& op, int64_t k, const Bufs& B, float* xn,
                                             float* xnl) {
  const int lane = threadIdx.x & 31;
  for (int sl = threadIdx.x >> 5; sl < 27; sl += WARPS) {  // one slot per warp
    const int64_t off = op.near_off[27 * k + sl];
    if (off < 0) continue;
    const int64_t col = off - op.near_base[k];
    const int64_t nn = sl < 26 ? (int64_t)op.nbr_leaf[k * 26 + sl] : k;
    const int64_t e0 = op.leaf_off[nn];
    const int ne = (int)(op.leaf_off[nn + 1] - e0), ne4 = (ne + 3) & ~3;
    for (int e = lane; e < ne4 * NR; e += 32) {
      const bool in = e < ne * NR;
      xn[col * NR + e] = in ? B.xg[e0 * NR + e] : 0.f;
      if constexpr (DF) xnl[col * NR + e] = in ? B.xl[e0 * NR + e] : 0.f;
    }
  }
}

// Near field of rows [i0, i0 + nrows) of leaf k (leaf-local): one segment of
// its near-field matrix, added to the warp's FP64 row sums ya[row][c].
template <int NR, bool DF>
__device__ __forceinline__ void near_rows(const GemvOp& op, int64_t k, int i0, int nrows,
                                          const float* xn, const float* xnl, double* ya) {
  constexpr int RW = rows_per_warp<NR, DF>();
  const int ld = op.near_ld[k];
  const int64_t o = op.near_base[k] + (int64_t)i0 * ld;
  seg_rows_any<NR, DF, RW>(op.knear + o, DF ? op.knearlo + o : nullptr, ld, nrows, ld / 4, xn, xnl,
                           [&](int, int q, const float(&sv)[NR], const float(&cv)[NR]) {
#pragma unroll
                             for (int c = 0; c < NR; ++c) ya[q * NR + c] += value<DF>(sv[c], cv[c]);
                           });
  __syncwarp();
}

// Forward output side, one block per leaf k: y = sum over the levels of
// U_b(rows) T_b + near field, FP64 across segments, written in the original
// order.
template <int NR, bool DF>
__global__ void __launch_bounds__(THREADS) k_uy(GemvOp op, Bufs B, int nrhs, double* __restrict__ Y,
                                                int64_t ldy) {
  constexpr int RW = rows_per_warp<NR, DF>();
  extern __shared__ __align__(16) unsigned char smem[];
  const int xn_floats = 27 * op.max_leaf4 * NR;
  double* yacc = reinterpret_cast<double*>(smem);  // WARPS x RW x NR
  float* xn = reinterpret_cast<float*>(smem + sizeof(double) * WARPS * RW * NR);
  float* xnl = xn + xn_floats;  // fp64x only
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
  stage_near_x<NR, DF>(op, k, B, xn, xnl);
  __syncthreads();
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  double* ya = yacc + w * RW * NR;
  for (int i0 = w * RW; i0 < nk; i0 += WARPS * RW) {
    const int nrows = min(RW, nk - i0);
    for (int e = lane; e < RW * NR; e += 32) ya[e] = 0.0;
    __syncwarp();
    for (int j = 1; j <= d; ++j) {
      const int R = lr[j];
      if (R == 0) continue;
      const int64_t uo = lu[j] + (int64_t)i0 * R;
      seg_rows_any<NR, DF, RW>(op.u32 + uo, DF ? op.u32lo + uo : nullptr, R, nrows, R / 4, B.t + lt[j],
                               DF ? B.tl + lt[j] : nullptr,
                               [&](int, int q, const float(&sv)[NR], const float(&cv)[NR]) {
#pragma unroll
                                 for (int c = 0; c < NR; ++c) ya[q * NR + c] += value<DF>(sv[c], cv[c]);
                               });
      __syncwarp();
    }
    near_rows<NR, DF>(op, k, i0, nrows, xn, xnl, ya);
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
template <int NR, bool DF>
__global__ void __launch_bounds__(THREADS) k_ut(GemvOp op, const int2* __restrict__ items, Bufs B) {
  __shared__ __align__(16) float xs[kGemvRowsT * NR];
  __shared__ __align__(16) float xsl[DF ? kGemvRowsT * NR : 4];
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
  for (int e = threadIdx.x; e < nr * NR; e += THREADS) {
    xs[e] = B.xg[(box0 + i0) * NR + e];
    if constexpr (DF) xsl[e] = B.xl[(box0 + i0) * NR + e];
  }
  __syncthreads();
  const int R = op.rbox[b], len4 = R / 4;
  const int64_t pofs = op.upofs[b];
  const int64_t uo = op.ubox_off[b] + i0 * R;
  const float* U = op.u32 + uo;
  const float* Ul = DF ? op.u32lo + uo : nullptr;
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  for (int k4b = w * 32; k4b < len4; k4b += WARPS * 32) {
    const int k4 = k4b + lane;
    const bool live = k4 < len4;
    float s[4][NR], c[4][NR];
#pragma unroll
    for (int e = 0; e < 4; ++e)
#pragma unroll
      for (int k = 0; k < NR; ++k) s[e][k] = c[e][k] = 0.f;
    constexpr int UN = 4;
    int i = 0;
    for (; i + UN <= nr; i += UN) {
      float4 v[UN], vl[UN];
#pragma unroll
      for (int u = 0; u < UN; ++u) {
        v[u] = live ? ld4(U, (int64_t)(i + u) * len4 + k4) : make_float4(0.f, 0.f, 0.f, 0.f);
        if constexpr (DF)
          vl[u] = live ? ld4(Ul, (int64_t)(i + u) * len4 + k4) : make_float4(0.f, 0.f, 0.f, 0.f);
      }
#pragma unroll
      for (int u = 0; u < UN; ++u)
#pragma unroll
        for (int k = 0; k < NR; ++k) {
          const float xh = xs[(i + u) * NR + k], xlo = DF ? xsl[(i + u) * NR + k] : 0.f;
#pragma unroll
          for (int e = 0; e < 4; ++e)
            mac<DF>(s[e][k], c[e][k], comp(v[u], e), DF ? comp(vl[u], e) : 0.f, xh, xlo);
        }
    }
    for (; i < nr; ++i) {
      const float4 v = live ? ld4(U, (int64_t)i * len4 + k4) : make_float4(0.f, 0.f, 0.f, 0.f);
      float4 vl = make_float4(0.f, 0.f, 0.f, 0.f);
      if constexpr (DF) vl = live ? ld4(Ul, (int64_t)i * len4 + k4) : vl;
#pragma unroll
      for (int k = 0; k < NR; ++k) {
        const float xh = xs[i * NR + k], xlo = DF ? xsl[i * NR + k] : 0.f;
#pragma unroll
        for (int e = 0; e < 4; ++e) mac<DF>(s[e][k], c[e][k], comp(v, e), comp(vl, e), xh, xlo);
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
          for (int k = 0; k < NR; ++k) {
            const int64_t o = (int64_t)sv * NR + k;
            if constexpr (DF)
              renorm(s[e][k], c[e][k], B.tt[o], B.ttl[o]);
            else
              B.tt[o] = s[e][k];
          }
      }
    } else if (live) {
      const int64_t o = (pofs + (int64_t)ci * R + 4 * (int64_t)k4) * NR;
#pragma unroll
      for (int e = 0; e < 4; ++e)
#pragma unroll
        for (int k = 0; k < NR; ++k) {
          float* pt = static_cast<float*>(B.pt);
          if constexpr (DF) {
            pt[2 * (o + e * NR + k)] = s[e][k];
            pt[2 * (o + e * NR + k) + 1] = c[e][k];
          } else {
            pt[o + e * NR + k] = s[e][k];
          }
        }
    }
  }
}

template <int NR, bool DF>
__global__ void k_tred_t(GemvOp op, const int32_t* __restrict__ boxes, Bufs B) {
  const int64_t b = boxes[blockIdx.x];
  const int d = op.levels;
  const int j = level_of(b, d);
  const int sh = 3 * (d - j);
  const int64_t kb = b - level_base(j);
  const int64_t n = op.leaf_off[(kb + 1) << sh] - op.leaf_off[kb << sh];
  const int nch = (int)((n + kGemvRowsT - 1) / kGemvRowsT);
  const int R = op.rbox[b];
  const int64_t base = op.upofs[b] * NR;
  const int32_t* tv = op.trow_v + op.tbase[b];
  for (int o = threadIdx.x; o < R * NR; o += blockDim.x) {
    const int k = o / NR;
    const int32_t sv = tv[k];
    if (sv < 0) continue;
    double s = 0.0;
    for (int ci = 0; ci < nch; ++ci) s += partial<DF>(B.pt, base + (int64_t)ci * R * NR + o);
    put_t<DF>(B.tt, B.ttl, (int64_t)sv * NR + (o - k * NR), s);
  }
}

// The leaf's columns [shift, shift + nk) of a V stack window (len4 column
// groups from V, row stride m4) times the stack's T rows Tv (contiguous),
// summed over the rows: lanes own 16-byte column groups, rows split over lane
// groups and warps; the arithmetic's sums over at most 64 rows, FP64 beyond;
// added to the warp's FP64 column sums fw[i][c].
template <int NR, bool DF, int LW>
__device__ __forceinline__ void stack_cols(const float* __restrict__ V, const float* __restrict__ Vl,
                                           int64_t m4, int rows, const float* __restrict__ Tv,
                                           const float* __restrict__ Tvl, int len4, int shift, int nk,
                                           double* fw) {
  // rows per lane summed in the arithmetic before an FP64 add: 64 (mixed),
  // 256 (fp64x, compensated)
  constexpr int G = 32 / LW, U = DF || NR == 8 ? 4 : 8, BLK = DF ? 256 : 64;
  const int lane = threadIdx.x & 31, g = lane / LW, li = lane % LW, w = threadIdx.x >> 5;
  for (int kw = 0; kw < len4; kw += LW) {
    const int k4 = kw + li;
    const bool live = k4 < len4;
    const int stride = WARPS * G;
    // every row block: the lane groups (which hold the same columns) are
    // merged, and the first group adds the block's sums to the warp's FP64
    // column sums; one summation order for every column count.  The groups
    // share the warp's row block starts, so every lane runs the same number
    // of blocks (the shuffles stay convergent).
    for (int vb = w * G; vb < rows; vb += BLK * stride) {
      const int v0 = vb + g;
      float s[4][NR], c[4][NR];
#pragma unroll
      for (int e = 0; e < 4; ++e)
#pragma unroll
        for (int k = 0; k < NR; ++k) s[e][k] = c[e][k] = 0.f;
      const int vend = min(rows, vb + BLK * stride);
      int v = v0;
      for (; v + (U - 1) * stride < vend; v += U * stride) {
        float4 f[U], fl[U];
        float tv[U][NR], tvl[U][NR];
#pragma unroll
        for (int u = 0; u < U; ++u) {
          const int64_t r = v + u * stride;
          f[u] = live ? ld4(V + r * m4, k4) : make_float4(0.f, 0.f, 0.f, 0.f);
          if constexpr (DF) fl[u] = live ? ld4(Vl + r * m4, k4) : make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
          for (int k = 0; k < NR; ++k) {
            tv[u][k] = Tv[r * NR + k];
            tvl[u][k] = DF ? Tvl[r * NR + k] : 0.f;
          }
        }
#pragma unroll
        for (int u = 0; u < U; ++u)
#pragma unroll
          for (int k = 0; k < NR; ++k)
#pragma unroll
            for (int e = 0; e < 4; ++e)
              mac<DF>(s[e][k], c[e][k], comp(f[u], e), DF ? comp(fl[u], e) : 0.f, tv[u][k], tvl[u][k]);
      }
      for (; v < vend; v += stride) {
        const float4 f = live ? ld4(V + (int64_t)v * m4, k4) : make_float4(0.f, 0.f, 0.f, 0.f);
        float4 fl = make_float4(0.f, 0.f, 0.f, 0.f);
        if constexpr (DF) fl = live ? ld4(Vl + (int64_t)v * m4, k4) : fl;
#pragma unroll
        for (int k = 0; k < NR; ++k) {
          const float th = Tv[(int64_t)v * NR + k], tl = DF ? Tvl[(int64_t)v * NR + k] : 0.f;
#pragma unroll
          for (int e = 0; e < 4; ++e) mac<DF>(s[e][k], c[e][k], comp(f, e), comp(fl, e), th, tl);
        }
      }
#pragma unroll
      for (int o = 16; o >= LW; o >>= 1)
#pragma unroll
        for (int e = 0; e < 4; ++e)
#pragma unroll
          for (int k = 0; k < NR; ++k) {
            const float s2 = __shfl_xor_sync(0xffffffffu, s[e][k], o);
            const float c2 = DF ? __shfl_xor_sync(0xffffffffu, c[e][k], o) : 0.f;
            merge<DF>(s[e][k], c[e][k], s2, c2);
          }
      if (g == 0 && live) {
#pragma unroll
        for (int e = 0; e < 4; ++e) {
          const int i = 4 * k4 + e - shift;  // leaf-local point
          if (i >= 0 && i < nk)
#pragma unroll
            for (int k = 0; k < NR; ++k) fw[i * NR + k] += value<DF>(s[e][k], c[e][k]);
        }
      }
    }
  }
}

template <int NR, bool DF>
__global__ void __launch_bounds__(THREADS) k_vy(GemvOp op, Bufs B, int nrhs, double* __restrict__ Y,
                                                int64_t ldy) {
  constexpr int RW = rows_per_warp<NR, DF>();
  extern __shared__ __align__(16) unsigned char smem[];
  const int nep = op.max_leaf4;
  double* yacc = reinterpret_cast<double*>(smem);                          // WARPS x RW x NR
  double* far = yacc + WARPS * RW * NR;                                    // WARPS x nep x NR
  float* xn = reinterpret_cast<float*>(far + (int64_t)WARPS * nep * NR);   // <= 27 nep x NR
  float* xnl = xn + 27 * nep * NR;                                         // fp64x only
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
  stage_near_x<NR, DF>(op, k, B, xn, xnl);
  __syncthreads();
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  double* fw = far + (int64_t)w * nep * NR;
  for (int j = 1; j <= d; ++j) {
    const int rows = lrows[j];
    if (rows == 0) continue;
    const int64_t m4 = lm[j];
    const int len4 = llen[j];
    const float* V = op.v32 + lv[j];
    const float* Vl = DF ? op.v32lo + lv[j] : nullptr;
    const float* Tv = B.tt + lt[j];
    const float* Tvl = DF ? B.ttl + lt[j] : nullptr;
    const int shift = lsh[j];
    if (len4 > 16)
      stack_cols<NR, DF, 32>(V, Vl, m4, rows, Tv, Tvl, len4, shift, nk, fw);
    else if (len4 > 8)
      stack_cols<NR, DF, 16>(V, Vl, m4, rows, Tv, Tvl, len4, shift, nk, fw);
    else if (len4 > 4)
      stack_cols<NR, DF, 8>(V, Vl, m4, rows, Tv, Tvl, len4, shift, nk, fw);
    else
      stack_cols<NR, DF, 4>(V, Vl, m4, rows, Tv, Tvl, len4, shift, nk, fw);
    __syncwarp();
  }
  __syncthreads();
  double* ya = yacc + w * RW * NR;
  for (int i0 = w * RW; i0 < nk; i0 += WARPS * RW) {
    const int nrows = min(RW, nk - i0);
    for (int e = lane; e < RW * NR; e += 32) {
      double s = 0.0;
      if (e < nrows * NR)
        for (int u = 0; u < WARPS; ++u) s += far[((int64_t)u * nep + i0) * NR + e];
      ya[e] = s;
    }
    __syncwarp();
    near_rows<NR, DF>(op, k, i0, nrows, xn, xnl, ya);
    for (int e = lane; e < nrows * NR; e += 32) {
      const int q = e / NR, c = e - q * NR;
      if (c < nrhs) Y[c * ldy + op.perm[t0 + i0 + q]] = ya[e];
    }
    __syncwarp();
  }
}

template <int NR, bool DF>
size_t uy_smem(int max_leaf4) {
  return sizeof(double) * WARPS * rows_per_warp<NR, DF>() * NR +
         sizeof(float) * (DF ? 2 : 1) * 27 * (size_t)max_leaf4 * NR;
}
template <int NR, bool DF>
size_t vy_smem(int max_leaf4) {
  return uy_smem<NR, DF>(max_leaf4) + sizeof(double) * WARPS * (size_t)max_leaf4 * NR;
}

template <int NR, bool DF>
int run(cudaStream_t s, const GemvOp& op, const GemvBuffers& G, const double* X, int64_t ldx,
        double* Y, int64_t ldy, int nrhs, bool trans, MatvecProfiler* prof) {
  // largest shared-memory request set so far, per instantiation and device
  static int attr_done[kMaxDevices] = {};
  const int dev = current_device();
  const size_t shu = uy_smem<NR, DF>(op.max_leaf4), shv = vy_smem<NR, DF>(op.max_leaf4);
  if ((int)shv > attr_done[dev]) {
    cudaFuncSetAttribute(k_uy<NR, DF>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)shu);
    cudaFuncSetAttribute(k_vy<NR, DF>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)shv);
    attr_done[dev] = (int)shv;
  }
  Bufs B{};
  B.xg = G.xg;
  B.t = G.t;
  B.tt = G.tt;
  if (DF) {
    B.xl = G.xl;
    B.tl = G.tl;
    B.ttl = G.ttl;
    B.p = G.pd;
    B.pt = G.ptd;
  } else {
    B.p = G.p;
    B.pt = G.pt;
  }
  int launches = 0;
  const int64_t N = op.N;
  if (prof) prof->begin(s);
  k_gather<NR, DF><<<(unsigned)((N * NR + 255) / 256), 256, 0, s>>>(N, nrhs, X, ldx, op.perm, B.xg, B.xl);
  ++launches;
  if (prof) prof->mark(s, "gather");
  if (!trans) {
    if (G.n_vt_items > 0) {
      k_vt<NR, DF><<<(unsigned)G.n_vt_items, THREADS, 0, s>>>(op, G.vt_items, B);
      ++launches;
      if (prof) prof->mark(s, "vt");
    }
    if (G.n_vt_upper > 0) {
      k_tred<NR, DF><<<(unsigned)G.n_vt_upper, 256, 0, s>>>(op, G.vt_upper, B);
      ++launches;
      if (prof) prof->mark(s, "tred");
    }
    k_uy<NR, DF><<<(unsigned)op.nleaf, THREADS, shu, s>>>(op, B, nrhs, Y, ldy);
    ++launches;
    if (prof) prof->mark(s, "uy");
  } else {
    if (G.n_ut_items > 0) {
      k_ut<NR, DF><<<(unsigned)G.n_ut_items, THREADS, 0, s>>>(op, G.ut_items, B);
      ++launches;
      if (prof) prof->mark(s, "ut");
    }
    if (G.n_ut_upper > 0) {
      k_tred_t<NR, DF><<<(unsigned)G.n_ut_upper, 256, 0, s>>>(op, G.ut_upper, B);
      ++launches;
      if (prof) prof->mark(s, "tred_t");
    }
    k_vy<NR, DF><<<(unsigned)op.nleaf, THREADS, shv, s>>>(op, B, nrhs, Y, ldy);
    ++launches;
    if (prof) prof->mark(s, "vy");
  }
  return launches;
}

template <bool DF>
int dispatch(cudaStream_t s, const GemvOp& op, const GemvBuffers& G, const double* X, int64_t ldx,
             double* Y, int64_t ldy, int nrhs, bool trans, MatvecProfiler* prof) {
  if (nrhs <= 1) return run<1, DF>(s, op, G, X, ldx, Y, ldy, nrhs, trans, prof);
  // mixed form: 2 or 3 columns in a zero-padded pass of 4 (measured at 64^3:
  // the 2-column V^T X takes 3.2 ms, the 4-column one 2.8)
  if (DF && nrhs <= 2) return run<2, true>(s, op, G, X, ldx, Y, ldy, nrhs, trans, prof);
  if (nrhs <= 4) return run<4, DF>(s, op, G, X, ldx, Y, ldy, nrhs, trans, prof);
  if constexpr (!DF) return run<8, false>(s, op, G, X, ldx, Y, ldy, nrhs, trans, prof);
  return 0;
}

}  // namespace

size_t gemv_smem_bytes(int max_leaf4, int nr, bool fp64x) {
  // the transposed output kernel takes the most
  if (fp64x) return vy_smem<4, true>(max_leaf4);
  return nr > 4 ? vy_smem<8, false>(max_leaf4) : vy_smem<4, false>(max_leaf4);
}

int launch_matvec_gemv(cudaStream_t s, const GemvOp& op, const GemvBuffers& B, const double* X,
                       int64_t ldx, double* Y, int64_t ldy, int nrhs, bool trans, bool fp64x,
                       MatvecProfiler* prof) {
  if (nrhs < 1 || nrhs > (fp64x ? 4 : 8)) return 0;
  return fp64x ? dispatch<true>(s, op, B, X, ldx, Y, ldy, nrhs, trans, prof)
               : dispatch<false>(s, op, B, X, ldx, Y, ldy, nrhs, trans, prof);
}

}  // namespace h3d
