// Fast matvec Y = A X (and Y = A^T X) over the uniform octree, 1..64 columns.
//
// Reference: HODLR3D::MatVecProduct (src/HODLR3D.cpp:21-27) = assignCharges,
// evaluateFarField, evaluate_NearField, collectPotential, reorder
// (src/HODLR3DTree.cpp:1647-1805).  The factors U, V of every pair are stored
// (the reference re-evaluates its CUR factors each call) and the near field
// is evaluated on the fly.  Every output row has a single owner block; no
// atomics anywhere.  Stages (d = leaf level, "slice" = box of level d - 1):
//   gather   X -> tree order, padded to NR columns
//   vtx      non-leaf pairs: partial V^T X over one slice of the input box
//   tred     pairs above level d - 1: T = sum of the slice partials (FP64)
//   ut       one block per (slice, row block): sum over levels < d of U T
//   leaf     one block per leaf: leaf-level pairs fused (T = V^T X in shared
//            memory, then U T), the near field (self and face/edge neighbour
//            leaves), the slice sum of `ut`; written once in the original order
// Precision: FT = double (FP64 form) or float (mixed form: FP32 products
// accumulated in FP32 within a pair or a near leaf, in FP64 across them).
// The transpose swaps U and V and targets and sources (the near field of the
// built-in kernels is symmetric and is reused).
#include "matvec.h"

#include <algorithm>

namespace h3d {

// ----------------------------------------------------------------------------
template <typename FT, int NR>
__global__ void k_gather_x(int64_t N, int nrhs, const double* __restrict__ X, int64_t ldx,
                           const int32_t* __restrict__ perm, FT* __restrict__ Xs) {
  const int64_t o = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (o >= N * NR) return;
  const int64_t t = o / NR;
  const int c = (int)(o - t * NR);
  Xs[o] = c < nrhs ? (FT)X[c * ldx + perm[t]] : (FT)0;
}

// column groups: G groups of CG consecutive right-hand sides per row
template <int NR>
struct Cols {
  static constexpr int G = NR >= 4 ? 4 : NR;
  static constexpr int CG = NR / G;
};

template <bool TRANS>
__device__ __forceinline__ int out_pair(const FarOp& op, int64_t q) {
  return TRANS ? op.rev[q] : (int)q;  // pairs whose output box owns list slot q
}
template <bool TRANS>
__device__ __forceinline__ int in_pair(const FarOp& op, int64_t q) {
  return TRANS ? (int)q : op.rev[q];  // pairs whose input box owns list slot q
}

// ----------------------------------------------------------------------------
// vtx: one block per work item (pair, slice of its input box).  Block of 64*G
// threads; thread (l, g) accumulates T[l][g*CG .. g*CG+CG) over 64-row tiles.
template <typename FT, int NR, bool TRANS>
__global__ void __launch_bounds__(256) k_vtx(FarOp op, const int32_t* __restrict__ items,
                                             const FT* __restrict__ Xs,
                                             FT* __restrict__ T, double* __restrict__ P) {
  using C = Cols<NR>;
  extern __shared__ __align__(16) unsigned char smem[];
  FT(*fs)[65] = reinterpret_cast<FT(*)[65]>(smem);
  FT(*xs)[NR] = reinterpret_cast<FT(*)[NR]>(smem + sizeof(FT) * 64 * 65);
  const int p = items[2 * blockIdx.x];
  const int slice = items[2 * blockIdx.x + 1];
  const int d = op.levels;
  const int j = op.pair_level[p];
  const int r = op.rank[p];
  const int64_t abox = (TRANS ? op.pair_tgt[p] : op.pair_src[p]) - level_base(j);
  const int sh = 3 * (d - j);
  const int64_t box0 = op.leaf_off[abox << sh];
  const int64_t ld = op.leaf_off[(abox + 1) << sh] - box0;
  const int64_t sb = (abox << (3 * (d - 1 - j))) + slice;  // slice box at level d - 1
  const int64_t s0 = op.leaf_off[sb << 3], s1 = op.leaf_off[(sb + 1) << 3];
  const FT* F = static_cast<const FT*>(TRANS ? op.ufac[p] : op.vfac[p]);
  const int tl = threadIdx.x & 63, g = threadIdx.x >> 6;
  const bool direct = (j == d - 1);
  for (int l0 = 0; l0 < r; l0 += 64) {
    FT acc[C::CG];
#pragma unroll
    for (int c = 0; c < C::CG; ++c) acc[c] = 0;
    for (int64_t i0 = s0; i0 < s1; i0 += 64) {
      const int ni = (int)min((int64_t)64, s1 - i0);
      __syncthreads();
      for (int e = threadIdx.x; e < 64 * 64; e += blockDim.x) {
        const int ll = e >> 6, ii = e & 63;
        fs[ll][ii] = (l0 + ll < r && ii < ni)
                         ? F[fac_idx<FT, TRANS>((i0 - box0) + ii, l0 + ll, r, ld, (sizeof(FT) == 4 ? (int64_t)op.ustride[p] : 0))]
                         : (FT)0;
      }
      for (int e = threadIdx.x; e < 64 * NR; e += blockDim.x) {
        const int ii = e / NR, c = e - ii * NR;
        xs[ii][c] = ii < ni ? Xs[(i0 + ii) * NR + c] : (FT)0;
      }
      __syncthreads();
      if (l0 + tl < r) {
#pragma unroll 4
        for (int ii = 0; ii < 64; ++ii) {
          const FT f = fs[tl][ii];
#pragma unroll
          for (int c = 0; c < C::CG; ++c) acc[c] += f * xs[ii][g * C::CG + c];
        }
      }
    }
    if (l0 + tl < r) {
      const int l = l0 + tl;
      if (direct) {
        FT* dst = T + op.tr_off[p] * NR + (int64_t)l * NR + g * C::CG;
#pragma unroll
        for (int c = 0; c < C::CG; ++c) dst[c] = acc[c];
      } else {
        double* dst = P + (op.part_off[p] + (int64_t)slice * r + l) * NR + g * C::CG;
#pragma unroll
        for (int c = 0; c < C::CG; ++c) dst[c] = (double)acc[c];
      }
    }
  }
}

// tred: T of the pairs above level d - 1 = sum of their slice partials, in
// slice order, in FP64.
template <typename FT, int NR>
__global__ void k_tred(FarOp op, const int32_t* __restrict__ pairs, const double* __restrict__ P,
                       FT* __restrict__ T) {
  const int p = pairs[blockIdx.x];
  const int r = op.rank[p];
  const int64_t ns = int64_t(1) << (3 * (op.levels - 1 - op.pair_level[p]));
  const double* src = P + op.part_off[p] * NR;
  FT* dst = T + op.tr_off[p] * NR;
  for (int o = threadIdx.x; o < r * NR; o += blockDim.x) {
    double acc = 0.0;
    for (int64_t s = 0; s < ns; ++s) acc += src[s * r * NR + o];
    dst[o] = (FT)acc;
  }
}

// ut: one block per (slice box, block of 64 rows): sum over the levels above
// the leaves of U_p[rows] T_p for the pairs whose output box contains the
// slice.  Writes FP64 partial sums Ynl[t][c].
template <typename FT, int NR, bool TRANS>
__global__ void __launch_bounds__(256) k_ut(FarOp op, const FT* __restrict__ T,
                                            double* __restrict__ Ynl) {
  using C = Cols<NR>;
  __shared__ FT ts[64][NR];
  const int d = op.levels;
  const int64_t sb = blockIdx.x;  // slice box at level d - 1
  const int64_t s0 = op.leaf_off[sb << 3], s1 = op.leaf_off[(sb + 1) << 3];
  const int tl = threadIdx.x & 63, g = threadIdx.x >> 6;
  for (int64_t rb = s0 + 64 * (int64_t)blockIdx.y; rb < s1; rb += 64 * (int64_t)gridDim.y) {
    const int64_t row = rb + tl;
    const bool live = row < s1;
    double acc[C::CG];
#pragma unroll
    for (int c = 0; c < C::CG; ++c) acc[c] = 0.0;
    for (int j = 1; j <= d - 1; ++j) {
      const int sh = 3 * (d - 1 - j);
      const int64_t a = sb >> sh;
      const int64_t gb = level_base(j) + a;
      const int64_t box0 = op.leaf_off[a << (sh + 3)];
      const int64_t ld = op.leaf_off[(a + 1) << (sh + 3)] - box0;
      for (int64_t q = op.il_ptr[gb]; q < op.il_ptr[gb + 1]; ++q) {
        const int p = out_pair<TRANS>(op, q);
        const int r = op.rank[p];
        const FT* F = static_cast<const FT*>(TRANS ? op.vfac[p] : op.ufac[p]);
        const FT* Tp = T + op.tr_off[p] * NR;
        FT part[C::CG];
#pragma unroll
        for (int c = 0; c < C::CG; ++c) part[c] = 0;
        for (int l0 = 0; l0 < r; l0 += 64) {
          const int nl = min(64, r - l0);
          __syncthreads();
          for (int e = threadIdx.x; e < nl * NR; e += blockDim.x) ts[e / NR][e % NR] = Tp[l0 * NR + e];
          __syncthreads();
          if (live) {
#pragma unroll 4
            for (int l = 0; l < nl; ++l) {
              const FT u = F[fac_idx<FT, !TRANS>(row - box0, l0 + l, r, ld, (sizeof(FT) == 4 ? (int64_t)op.ustride[p] : 0))];
#pragma unroll
              for (int c = 0; c < C::CG; ++c) part[c] += u * ts[l][g * C::CG + c];
            }
          }
        }
#pragma unroll
        for (int c = 0; c < C::CG; ++c) acc[c] += (double)part[c];
      }
    }
    if (live) {
#pragma unroll
      for (int c = 0; c < C::CG; ++c) Ynl[row * NR + g * C::CG + c] = acc[c];
    }
  }
}

// ----------------------------------------------------------------------------
template <typename FT>
struct NearPt;
template <>
struct NearPt<double> {
  double x, y, z;
};
template <>
struct NearPt<float> {
  float x, y, z;
};

__device__ __forceinline__ double near_kv(const KernelDesc& kd, const NearPt<double>& a,
                                          const NearPt<double>& b, const NearPt<double>&) {
  return entry64_offdiag(kd, __dsub_rn(a.x, b.x), __dsub_rn(a.y, b.y), __dsub_rn(a.z, b.z));
}
__device__ __forceinline__ float near_kv(const KernelDesc& kd, const NearPt<float>& a,
                                         const NearPt<float>& b, const NearPt<float>& dc) {
  return entry32_offdiag(kd, (a.x - b.x) + dc.x, (a.y - b.y) + dc.y, (a.z - b.z) + dc.z);
}

template <typename FT>
__device__ __forceinline__ NearPt<FT> load_pt(const NearOp& nr, int64_t t);
template <>
__device__ __forceinline__ NearPt<double> load_pt<double>(const NearOp& nr, int64_t t) {
  return {nr.xs[t], nr.ys[t], nr.zs[t]};
}
template <>
__device__ __forceinline__ NearPt<float> load_pt<float>(const NearOp& nr, int64_t t) {
  return {nr.xl[t], nr.yl[t], nr.zl[t]};
}

// leaf: one block per output leaf (64 * G threads, rows in tiles of 64).
template <typename FT, int NR, bool TRANS>
__global__ void __launch_bounds__(256) k_leaf(FarOp op, NearOp nr, const FT* __restrict__ Xs,
                                              const double* __restrict__ Ynl,
                                              const int32_t* __restrict__ perm, int nrhs,
                                              double* __restrict__ Y, int64_t ldy) {
  using C = Cols<NR>;
  extern __shared__ __align__(16) unsigned char smem[];
  FT(*fs)[65] = reinterpret_cast<FT(*)[65]>(smem);  // input-side factor tile
  FT(*xs)[NR] = reinterpret_cast<FT(*)[NR]>(smem + sizeof(FT) * 64 * 65);  // input rows
  FT(*ts)[NR] = reinterpret_cast<FT(*)[NR]>(smem + sizeof(FT) * (64 * 65 + 64 * NR));  // T
  NearPt<FT>* ps =
      reinterpret_cast<NearPt<FT>*>(smem + sizeof(FT) * (64 * 65 + 128 * NR));  // sources
  const int d = op.levels;
  const int64_t k = blockIdx.x;
  const int64_t t0 = op.leaf_off[k], t1 = op.leaf_off[k + 1];
  const int tl = threadIdx.x & 63, g = threadIdx.x >> 6;
  const int64_t lk = level_base(d) + k;
  for (int64_t rb = t0; rb < t1; rb += 64) {
    const int64_t row = rb + tl;
    const bool live = row < t1;
    double acc[C::CG];
#pragma unroll
    for (int c = 0; c < C::CG; ++c) acc[c] = (live && d >= 2) ? Ynl[row * NR + g * C::CG + c] : 0.0;
    // ---- leaf-level pairs, fused --------------------------------------
    for (int64_t q = op.il_ptr[lk]; q < op.il_ptr[lk + 1]; ++q) {
      const int p = out_pair<TRANS>(op, q);
      const int r = op.rank[p];
      if (r == 0) continue;
      const int64_t ibox = (TRANS ? op.pair_tgt[p] : op.pair_src[p]) - level_base(d);
      const int64_t i0 = op.leaf_off[ibox], ni = op.leaf_off[ibox + 1] - i0;
      const FT* Fin = static_cast<const FT*>(TRANS ? op.ufac[p] : op.vfac[p]);
      const FT* Fout = static_cast<const FT*>(TRANS ? op.vfac[p] : op.ufac[p]);
      FT part[C::CG];
#pragma unroll
      for (int c = 0; c < C::CG; ++c) part[c] = 0;
      for (int l0 = 0; l0 < r; l0 += 64) {
        const int nl = min(64, r - l0);
        // T[l0 .. l0+nl) = Fin^T X over the input leaf, 64 rows at a time
        FT tacc[C::CG];
#pragma unroll
        for (int c = 0; c < C::CG; ++c) tacc[c] = 0;
        for (int64_t a0 = 0; a0 < ni; a0 += 64) {
          const int na = (int)min((int64_t)64, ni - a0);
          __syncthreads();
          for (int e = threadIdx.x; e < 64 * 64; e += blockDim.x) {
            const int ll = e >> 6, ii = e & 63;
            fs[ll][ii] = (ll < nl && ii < na) ? Fin[fac_idx<FT, TRANS>(a0 + ii, l0 + ll, r, ni, (sizeof(FT) == 4 ? (int64_t)op.ustride[p] : 0))] : (FT)0;
          }
          for (int e = threadIdx.x; e < 64 * NR; e += blockDim.x) {
            const int ii = e / NR, c = e - ii * NR;
            xs[ii][c] = ii < na ? Xs[(i0 + a0 + ii) * NR + c] : (FT)0;
          }
          __syncthreads();
          if (tl < nl) {
#pragma unroll 4
            for (int ii = 0; ii < 64; ++ii) {
              const FT f = fs[tl][ii];
#pragma unroll
              for (int c = 0; c < C::CG; ++c) tacc[c] += f * xs[ii][g * C::CG + c];
            }
          }
        }
        __syncthreads();
        if (tl < nl) {
#pragma unroll
          for (int c = 0; c < C::CG; ++c) ts[tl][g * C::CG + c] = tacc[c];
        }
        __syncthreads();
        if (live) {
#pragma unroll 4
          for (int l = 0; l < nl; ++l) {
            const FT u = Fout[fac_idx<FT, !TRANS>(row - t0, l0 + l, r, t1 - t0, (sizeof(FT) == 4 ? (int64_t)op.ustride[p] : 0))];
#pragma unroll
            for (int c = 0; c < C::CG; ++c) part[c] += u * ts[l][g * C::CG + c];
          }
        }
      }
#pragma unroll
      for (int c = 0; c < C::CG; ++c) acc[c] += (double)part[c];
    }
    // ---- near field: neighbour slots 0..25, then the leaf itself -------
    const NearPt<FT> me = live ? load_pt<FT>(nr, row) : NearPt<FT>{0, 0, 0};
    for (int sl = 0; sl <= 26; ++sl) {
      const int64_t nn = sl < 26 ? nr.nbr_leaf[k * 26 + sl] : k;
      if (nn < 0) continue;
      const int64_t q0 = op.leaf_off[nn], q1 = op.leaf_off[nn + 1];
      NearPt<FT> dc{0, 0, 0};
      if (sizeof(FT) == 4) {
        dc.x = (FT)(nr.centre[3 * k] - nr.centre[3 * nn]);
        dc.y = (FT)(nr.centre[3 * k + 1] - nr.centre[3 * nn + 1]);
        dc.z = (FT)(nr.centre[3 * k + 2] - nr.centre[3 * nn + 2]);
      }
      FT part[C::CG];
#pragma unroll
      for (int c = 0; c < C::CG; ++c) part[c] = 0;
      for (int64_t e0 = q0; e0 < q1; e0 += 64) {
        const int ne = (int)min((int64_t)64, q1 - e0);
        __syncthreads();
        for (int e = threadIdx.x; e < ne; e += blockDim.x) ps[e] = load_pt<FT>(nr, e0 + e);
        for (int e = threadIdx.x; e < 64 * NR; e += blockDim.x) {
          const int ii = e / NR, c = e - ii * NR;
          xs[ii][c] = ii < ne ? Xs[(e0 + ii) * NR + c] : (FT)0;
        }
        __syncthreads();
        if (live) {
          for (int ii = 0; ii < ne; ++ii) {
            const FT kv = (e0 + ii == row) ? (FT)nr.kd.diag : near_kv(nr.kd, me, ps[ii], dc);
#pragma unroll
            for (int c = 0; c < C::CG; ++c) part[c] += kv * xs[ii][g * C::CG + c];
          }
        }
      }
#pragma unroll
      for (int c = 0; c < C::CG; ++c) acc[c] += (double)part[c];
    }
    if (live) {
      const int64_t orig = perm[row];
#pragma unroll
      for (int c = 0; c < C::CG; ++c) {
        const int cc = g * C::CG + c;
        if (cc < nrhs) Y[cc * ldy + orig] = acc[c];
      }
    }
  }
}

int padded_nrhs(int nrhs) {
  int nr = 1;
  while (nr < nrhs) nr <<= 1;
  return nr;
}

// ----------------------------------------------------------------------------
template <typename FT, int NR, bool TRANS>
static int run(cudaStream_t s, int64_t N, const int32_t* perm, const FarOp& far,
               const NearOp& near, const MatvecBuffers& B, const double* X, int64_t ldx,
               double* Y, int64_t ldy, int nrhs, MatvecProfiler* prof) {
  using C = Cols<NR>;
  FT* Xs = static_cast<FT*>(B.xsorted);
  FT* T = static_cast<FT*>(B.tbuf);
  const int bs = 256;
  int launches = 0;
  if (prof) prof->begin(s);
  k_gather_x<FT, NR><<<(unsigned)((N * NR + bs - 1) / bs), bs, 0, s>>>(N, nrhs, X, ldx, perm, Xs);
  ++launches;
  if (prof) prof->mark(s, "gather");
  const int threads = 64 * C::G;
  const size_t shm_vtx = sizeof(FT) * (64 * 65 + 64 * NR);
  const size_t shm_leaf = sizeof(FT) * (64 * 65 + 128 * NR) + sizeof(NearPt<FT>) * 64;
  static bool attr_set[kMaxDevices] = {};  // per instantiation and device
  const int dev = current_device();
  if (!attr_set[dev]) {
    cudaFuncSetAttribute(k_vtx<FT, NR, TRANS>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)shm_vtx);
    cudaFuncSetAttribute(k_leaf<FT, NR, TRANS>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)shm_leaf);
    attr_set[dev] = true;
  }
  if (far.levels >= 2) {
    if (B.n_items > 0) {
      k_vtx<FT, NR, TRANS><<<(unsigned)B.n_items, threads, shm_vtx, s>>>(far, B.items, Xs, T, B.pbuf);
      ++launches;
      if (prof) prof->mark(s, "vtx");
    }
    if (B.n_upper > 0) {
      k_tred<FT, NR><<<(unsigned)B.n_upper, 128, 0, s>>>(far, B.upper_pairs, B.pbuf, T);
      ++launches;
      if (prof) prof->mark(s, "tred");
    }
    const int64_t nslice = int64_t(1) << (3 * (far.levels - 1));
    const int rows_blocks = (B.max_slice + 63) / 64;
    k_ut<FT, NR, TRANS><<<dim3((unsigned)nslice, (unsigned)std::max(1, rows_blocks)), threads, 0, s>>>(
        far, T, B.ynl);
    ++launches;
    if (prof) prof->mark(s, "ut");
  }
  k_leaf<FT, NR, TRANS><<<(unsigned)far.nleaf, threads, shm_leaf, s>>>(far, near, Xs, B.ynl, perm,
                                                                      nrhs, Y, ldy);
  ++launches;
  if (prof) prof->mark(s, "leaf");
  return launches;
}

template <typename FT, bool TRANS>
static int dispatch_nr(cudaStream_t s, int64_t N, const int32_t* perm, const FarOp& far,
                       const NearOp& near, const MatvecBuffers& B, const double* X, int64_t ldx,
                       double* Y, int64_t ldy, int nrhs, MatvecProfiler* prof) {
  const int nr = padded_nrhs(nrhs);
#define H3D_NR(V)                                                                            \
  case V:                                                                                    \
    return run<FT, V, TRANS>(s, N, perm, far, near, B, X, ldx, Y, ldy, nrhs, prof);
  switch (nr) {
    H3D_NR(1)
    H3D_NR(2)
    H3D_NR(4)
    H3D_NR(8)
    H3D_NR(16)
    H3D_NR(32)
    H3D_NR(64)
  }
#undef H3D_NR
  return 0;
}

int launch_matvec(cudaStream_t s, int64_t N, const int32_t* perm, const FarOp& far,
                  const NearOp& near, const MatvecBuffers& B, const double* X, int64_t ldx,
                  double* Y, int64_t ldy, int nrhs, int precision, int trans,
                  MatvecProfiler* prof) {
  if (precision == 0)
    return trans ? dispatch_nr<double, true>(s, N, perm, far, near, B, X, ldx, Y, ldy, nrhs, prof)
                 : dispatch_nr<double, false>(s, N, perm, far, near, B, X, ldx, Y, ldy, nrhs, prof);
  return trans ? dispatch_nr<float, true>(s, N, perm, far, near, B, X, ldx, Y, ldy, nrhs, prof)
               : dispatch_nr<float, false>(s, N, perm, far, near, B, X, ldx, Y, ldy, nrhs, prof);
}

// ----------------------------------------------------------------------------
// y[r, c] = sum_j K(rows[r], j) x[j, c] in FP64 over the original points.
__global__ void k_dense_rows(int64_t N, const double* __restrict__ xyz, KernelDesc kd,
                             const int64_t* __restrict__ rows, const double* __restrict__ X,
                             int64_t ldx, double* __restrict__ Y, int64_t nrows, int nrhs) {
  __shared__ double red[32];
  const int64_t r = blockIdx.x;
  const int c = blockIdx.y;
  const int64_t i = rows[r];
  if (i < 0 || i >= N) {  // a row id outside the point set: NaN, nothing read
    if (threadIdx.x == 0) Y[c * nrows + r] = __longlong_as_double(0x7ff8000000000000LL);
    return;
  }
  const double xi = xyz[3 * i], yi = xyz[3 * i + 1], zi = xyz[3 * i + 2];
  double acc = 0.0;
  for (int64_t j = threadIdx.x; j < N; j += blockDim.x) {
    const double kv = (j == i) ? kd.diag
                               : entry64_offdiag(kd, xi - xyz[3 * j], yi - xyz[3 * j + 1],
                                                 zi - xyz[3 * j + 2]);
    acc += kv * X[c * ldx + j];
  }
  acc = warp_sum_d(acc);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x < 32) {
    double v = threadIdx.x < blockDim.x / 32 ? red[threadIdx.x] : 0.0;
    v = warp_sum_d(v);
    if (threadIdx.x == 0) Y[c * nrows + r] = v;
  }
}

// out[e] = K(rows[e], cols[e]) in FP64 over the original points (the FP64
// product's entry formula; the diagonal value where the ids are equal); an id
// outside [0, N) gives NaN.
__global__ void k_entries(int64_t N, const double* __restrict__ xyz, KernelDesc kd,
                          const int64_t* __restrict__ rc, int64_t n, double* __restrict__ out) {
  const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (e >= n) return;
  const int64_t i = rc[e], j = rc[n + e];
  if (i < 0 || i >= N || j < 0 || j >= N) {
    out[e] = __longlong_as_double(0x7ff8000000000000LL);
    return;
  }
  out[e] = i == j ? kd.diag
                  : entry64_offdiag(kd, xyz[3 * i] - xyz[3 * j], xyz[3 * i + 1] - xyz[3 * j + 1],
                                    xyz[3 * i + 2] - xyz[3 * j + 2]);
}

void launch_entries(cudaStream_t s, int64_t N, const double* xyz, KernelDesc kd, const int64_t* rc,
                    int64_t n, double* out) {
  if (n == 0) return;
  k_entries<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(N, xyz, kd, rc, n, out);
}

namespace {
// 32 x 32 tiles through shared memory (one padding column against bank conflicts)
__global__ void k_transpose(const double* __restrict__ in, int64_t rows, int64_t cols,
                            double* __restrict__ out) {
  __shared__ double tile[32][33];
  const int64_t r0 = (int64_t)blockIdx.y * 32, c0 = (int64_t)blockIdx.x * 32;
  for (int i = threadIdx.y; i < 32; i += blockDim.y) {
    const int64_t r = r0 + i, c = c0 + threadIdx.x;
    if (r < rows && c < cols) tile[i][threadIdx.x] = in[r * cols + c];
  }
  __syncthreads();
  for (int i = threadIdx.y; i < 32; i += blockDim.y) {
    const int64_t c = c0 + i, r = r0 + threadIdx.x;
    if (r < rows && c < cols) out[c * rows + r] = tile[threadIdx.x][i];
  }
}
}  // namespace

void launch_transpose(cudaStream_t s, const double* in, int64_t rows, int64_t cols, double* out) {
  const dim3 grid((unsigned)((cols + 31) / 32), (unsigned)((rows + 31) / 32));
  k_transpose<<<grid, dim3(32, 8), 0, s>>>(in, rows, cols, out);
}

void launch_dense_rows(cudaStream_t s, int64_t N, const double* xyz, KernelDesc kd,
                       const int64_t* rows, int64_t nrows, const double* X, int64_t ldx,
                       double* Y, int nrhs) {
  if (nrows == 0) return;
  dim3 grid((unsigned)nrows, (unsigned)nrhs);
  k_dense_rows<<<grid, 256, 0, s>>>(N, xyz, kd, rows, X, ldx, Y, nrows, nrhs);
}

}  // namespace h3d
