// Fast matvec y = A x (and y = A^T x) over the uniform octree.
//
// Reference: HODLR3D::MatVecProduct (src/HODLR3D.cpp:21-27) = assignCharges,
// evaluateFarField, evaluate_NearField, collectPotential, reorder
// (src/HODLR3DTree.cpp:1647-1805).  Here the factors are stored (U, V from
// the ACA) instead of re-evaluated, the near field is evaluated on the fly,
// and every output row has a single owner thread block (no atomics):
//   1. gather x into tree order,
//   2. per leaf: partial V^T x of every pair whose source box contains it,
//   3. per pair above the leaf level: sum of its leaf partials (fixed order),
//   4. per leaf: sum over levels of U (V^T x) restricted to its rows, plus
//      the near field (self and face/edge neighbour leaves), scattered back to
//      the original order.
// The transpose swaps the roles of U and V and of targets and sources; the
// near field of the built-in kernels is symmetric and is reused as is.
#include "matvec.h"

namespace h3d {

template <typename FT>
__global__ void k_gather_x(int64_t N, int nrhs, const double* __restrict__ X, int64_t ldx,
                           const int32_t* __restrict__ perm, FT* __restrict__ Xs) {
  const int64_t o = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (o >= N * nrhs) return;
  const int64_t t = o / nrhs;
  const int c = (int)(o - t * nrhs);
  Xs[o] = (FT)X[c * ldx + perm[t]];
}

// Partial products F^T x over the rows of one leaf for every pair whose
// "input box" (source box for A, target box for A^T) is an ancestor of the
// leaf.  One block per leaf, one warp per factor column.
template <typename FT, bool TRANS>
__global__ void __launch_bounds__(128) k_partial(FarOp op, const FT* __restrict__ Xs, int nrhs,
                                                 double* __restrict__ T, double* __restrict__ P) {
  extern __shared__ unsigned char smraw[];
  FT* xsh = reinterpret_cast<FT*>(smraw);
  const int64_t s = blockIdx.x;
  const int d = op.levels;
  const int l0 = op.leaf_off[s], len = op.leaf_off[s + 1] - l0;
  for (int i = threadIdx.x; i < len * nrhs; i += blockDim.x) xsh[i] = Xs[(int64_t)l0 * nrhs + i];
  __syncthreads();
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  for (int j = 1; j <= d; ++j) {
    const int sh = 3 * (d - j);
    const int64_t a = s >> sh;
    const int64_t gb = level_base(j) + a;
    const int64_t box0 = op.leaf_off[a << sh];
    const int64_t ld = op.leaf_off[(a + 1) << sh] - box0;
    const int64_t ro = l0 - box0;
    const int64_t chunk = s - (a << sh);
    for (int64_t q = op.il_ptr[gb]; q < op.il_ptr[gb + 1]; ++q) {
      const int p = TRANS ? (int)q : op.rev[q];
      const int r = op.rank[p];
      if (r == 0) continue;
      const FT* F = static_cast<const FT*>(TRANS ? op.ufac[p] : op.vfac[p]);
      double* out = (j == d) ? T + op.tr_off[p] * nrhs : P + (op.part_off[p] + chunk * r) * nrhs;
      for (int l = w; l < r; l += 4) {
        const FT* col = F + (int64_t)l * ld + ro;
        for (int c = 0; c < nrhs; ++c) {
          FT acc = 0;
          for (int i = lane; i < len; i += 32) acc += col[i] * xsh[i * nrhs + c];
#pragma unroll
          for (int o = 16; o >= 1; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
          if (lane == 0) out[l * nrhs + c] = (double)acc;
        }
      }
    }
  }
}

// T of every pair above the leaf level = sum of its leaf partials in leaf order.
__global__ void k_reduce_partials(FarOp op, const int32_t* __restrict__ nonleaf,
                                  const int32_t* __restrict__ pair_level, int nrhs,
                                  const double* __restrict__ P, double* __restrict__ T) {
  const int p = nonleaf[blockIdx.x];
  const int r = op.rank[p];
  const int64_t nch = int64_t(1) << (3 * (op.levels - pair_level[p]));
  const double* src = P + op.part_off[p] * nrhs;
  double* dst = T + op.tr_off[p] * nrhs;
  for (int o = threadIdx.x; o < r * nrhs; o += blockDim.x) {
    double acc = 0.0;
    for (int64_t c = 0; c < nch; ++c) acc += src[c * r * nrhs + o];
    dst[o] = acc;
  }
}

template <typename FT>
__device__ __forceinline__ FT near_entry(const NearOp& nr, int64_t t, int64_t e, float dcx,
                                         float dcy, float dcz);

template <>
__device__ __forceinline__ double near_entry<double>(const NearOp& nr, int64_t t, int64_t e, float,
                                                     float, float) {
  return entry64_offdiag(nr.kd, __dsub_rn(nr.xs[t], nr.xs[e]), __dsub_rn(nr.ys[t], nr.ys[e]),
                         __dsub_rn(nr.zs[t], nr.zs[e]));
}

template <>
__device__ __forceinline__ float near_entry<float>(const NearOp& nr, int64_t t, int64_t e,
                                                   float dcx, float dcy, float dcz) {
  return entry32_offdiag(nr.kd, (nr.xl[t] - nr.xl[e]) + dcx, (nr.yl[t] - nr.yl[e]) + dcy,
                         (nr.zl[t] - nr.zl[e]) + dcz);
}

// Output rows of one leaf: far field of every level through the pairs whose
// "output box" (target box for A, source box for A^T) contains the leaf, and
// the near field; written once, in the original order.
template <typename FT, bool TRANS>
__global__ void __launch_bounds__(128) k_apply(FarOp op, NearOp nr, const double* __restrict__ T,
                                               const FT* __restrict__ Xs, int nrhs,
                                               const int32_t* __restrict__ perm,
                                               double* __restrict__ Y, int64_t ldy) {
  const int64_t k = blockIdx.x;
  const int d = op.levels;
  const int64_t t0 = op.leaf_off[k];
  const int nk = op.leaf_off[k + 1] - (int)t0;
  for (int o = threadIdx.x; o < nk * nrhs; o += blockDim.x) {
    const int t = o / nrhs, c = o - t * nrhs;
    double acc = 0.0;
    for (int j = 1; j <= d; ++j) {
      const int sh = 3 * (d - j);
      const int64_t a = k >> sh;
      const int64_t gb = level_base(j) + a;
      const int64_t box0 = op.leaf_off[a << sh];
      const int64_t ld = op.leaf_off[(a + 1) << sh] - box0;
      const int64_t row = t0 - box0 + t;
      for (int64_t q = op.il_ptr[gb]; q < op.il_ptr[gb + 1]; ++q) {
        const int p = TRANS ? op.rev[q] : (int)q;
        const int r = op.rank[p];
        const FT* F = static_cast<const FT*>(TRANS ? op.vfac[p] : op.ufac[p]);
        const double* tp = T + op.tr_off[p] * nrhs + c;
        FT part = 0;
        for (int l = 0; l < r; ++l) part += F[(int64_t)l * ld + row] * (FT)tp[l * nrhs];
        acc += (double)part;
      }
    }
    // near field: neighbour slots 0..25 then the leaf itself (evaluate_NearField)
    const int64_t ti = t0 + t;
    for (int sl = 0; sl <= 26; ++sl) {
      const int64_t nn = sl < 26 ? nr.nbr_leaf[k * 26 + sl] : k;
      if (nn < 0) continue;
      const int64_t q0 = op.leaf_off[nn], q1 = op.leaf_off[nn + 1];
      float dcx = 0.f, dcy = 0.f, dcz = 0.f;
      if (sizeof(FT) == 4) {
        dcx = (float)(nr.centre[3 * k] - nr.centre[3 * nn]);
        dcy = (float)(nr.centre[3 * k + 1] - nr.centre[3 * nn + 1]);
        dcz = (float)(nr.centre[3 * k + 2] - nr.centre[3 * nn + 2]);
      }
      FT part = 0;
      for (int64_t e = q0; e < q1; ++e) {
        const FT kv = (e == ti) ? (FT)nr.kd.diag : near_entry<FT>(nr, ti, e, dcx, dcy, dcz);
        part += kv * Xs[e * nrhs + c];
      }
      acc += (double)part;
    }
    Y[c * ldy + perm[ti]] = acc;
  }
}

template <typename FT, bool TRANS>
static int run(cudaStream_t s, int64_t N, const int32_t* perm, const FarOp& far,
               const NearOp& near, const MatvecBuffers& B, const double* X, int64_t ldx,
               double* Y, int64_t ldy, int nrhs) {
  FT* Xs = static_cast<FT*>(B.xsorted);
  const int bs = 256;
  k_gather_x<FT><<<(unsigned)((N * nrhs + bs - 1) / bs), bs, 0, s>>>(N, nrhs, X, ldx, perm, Xs);
  const size_t shm = (size_t)B.max_leaf * nrhs * sizeof(FT);
  if (shm > 48 * 1024)
    cudaFuncSetAttribute(k_partial<FT, TRANS>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)shm);
  int launches = 1;
  if (far.levels >= 1) {
    k_partial<FT, TRANS><<<(unsigned)far.nleaf, 128, shm, s>>>(far, Xs, nrhs, B.tbuf, B.pbuf);
    ++launches;
    if (B.n_nonleaf > 0) {
      k_reduce_partials<<<(unsigned)B.n_nonleaf, 128, 0, s>>>(far, B.nonleaf_pairs, B.pair_level,
                                                              nrhs, B.pbuf, B.tbuf);
      ++launches;
    }
  }
  k_apply<FT, TRANS><<<(unsigned)far.nleaf, 128, 0, s>>>(far, near, B.tbuf, Xs, nrhs, perm, Y, ldy);
  return launches + 1;
}

int launch_matvec(cudaStream_t s, int64_t N, const int32_t* perm, const FarOp& far,
                  const NearOp& near, const MatvecBuffers& B, const double* X, int64_t ldx,
                  double* Y, int64_t ldy, int nrhs, int precision, int trans) {
  if (precision == 0)
    return trans ? run<double, true>(s, N, perm, far, near, B, X, ldx, Y, ldy, nrhs)
                 : run<double, false>(s, N, perm, far, near, B, X, ldx, Y, ldy, nrhs);
  return trans ? run<float, true>(s, N, perm, far, near, B, X, ldx, Y, ldy, nrhs)
               : run<float, false>(s, N, perm, far, near, B, X, ldx, Y, ldy, nrhs);
}

// y[r, c] = sum_j K(rows[r], j) x[j, c] in FP64 over the original points.
__global__ void k_dense_rows(int64_t N, const double* __restrict__ xyz, KernelDesc kd,
                             const int64_t* __restrict__ rows, const double* __restrict__ X,
                             int64_t ldx, double* __restrict__ Y, int64_t nrows, int nrhs) {
  __shared__ double red[32];
  const int64_t r = blockIdx.x;
  const int c = blockIdx.y;
  const int64_t i = rows[r];
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

void launch_dense_rows(cudaStream_t s, int64_t N, const double* xyz, KernelDesc kd,
                       const int64_t* rows, int64_t nrows, const double* X, int64_t ldx,
                       double* Y, int nrhs) {
  if (nrows == 0) return;
  dim3 grid((unsigned)nrows, (unsigned)nrhs);
  k_dense_rows<<<grid, 256, 0, s>>>(N, xyz, kd, rows, X, ldx, Y, nrows, nrhs);
}

}  // namespace h3d
