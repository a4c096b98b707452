// Batched partially pivoted ACA: one thread block per interaction-list pair,
// persistent blocks pulling pairs (largest first) from a work counter.
//
// Reference: LowRank::ACA_only_nodesCUR (src/ACA.cpp:127-238) driven by
// HODLR3DTree::getUVtTree / getUVtInstance (src/HODLR3DTree.cpp:1621-1645).
// The kept factors are the ACA's residual vectors: U = [u_1..u_r] (n x r) and
// V = [v_1..v_r] (m x r), column-major, so that K(box, source) ~ U V^T; the
// reference's CUR form Ac R^-1 L^-1 Ar is the same product (Ac R^-1 = U and
// L^-1 Ar = V^T with L(i,j) = U(row_i, j), R(j,i) = V(col_i, j)).
//
// Bit-exactness: kernel entries and residual rows/columns are evaluated with
// the reference's operation order and no fused multiply-adds; norms and dot
// products use the canonical reduction order; pivots are first maxima.  The
// CPU oracle reproduces the same ranks and pivots.
#include "aca.h"
#include "common.cuh"

namespace h3d {

struct AcaShared {
  double red_v[32];
  int red_i[32];
  int flag_bad;
  int ctl_break;
  int row_index, col_index, next_row;
  double nu, nv, normS;
};

template <int BS>
__device__ __forceinline__ void block_argmax(double v, int i, AcaShared& S, double& out_v,
                                             int& out_i) {
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  warp_argmax(v, i);
  if (lane == 0) {
    S.red_v[w] = v;
    S.red_i[w] = i;
  }
  __syncthreads();
  if (w == 0) {
    double vv = lane < BS / 32 ? S.red_v[lane] : 0.0;
    int ii = lane < BS / 32 ? S.red_i[lane] : -1;
    warp_argmax(vv, ii);
    if (lane == 0) {
      S.red_v[0] = vv;
      S.red_i[0] = ii;
    }
  }
  __syncthreads();
  out_v = S.red_v[0];
  out_i = S.red_i[0];
  __syncthreads();
}

// Residual row at `row` with r previous terms -> V[:, r]; returns the first
// maximum of |row| over unused columns.
template <int BS>
__device__ void row_pass(const AcaTask& T, const PointsF64& P, const KernelDesc& kd, int row,
                         int r, const double* __restrict__ ubuf, const double* __restrict__ U,
                         double* __restrict__ V, const unsigned char* __restrict__ used_c,
                         AcaShared& S, double& amax, int& aidx) {
  const double xi = P.x[T.t0 + row], yi = P.y[T.t0 + row], zi = P.z[T.t0 + row];
  double bv = 0.0;
  int bi = -1;
  bool bad = false;
  for (int s = threadIdx.x; s < T.m; s += BS) {
    const int q = T.s0 + s;
    double e = entry64_offdiag(kd, __dsub_rn(xi, P.x[q]), __dsub_rn(yi, P.y[q]),
                               __dsub_rn(zi, P.z[q]));
    for (int l = 0; l < r; ++l) e = __dsub_rn(e, __dmul_rn(ubuf[l], V[(size_t)l * T.m + s]));
    V[(size_t)r * T.m + s] = e;
    if (!isfinite(e)) bad = true;
    if (!used_c[s]) argmax_merge(bv, bi, fabs(e), s);
  }
  if (bad) S.flag_bad = 1;
  block_argmax<BS>(bv, bi, S, amax, aidx);
}

// Residual column at `col` with r previous terms, divided by the pivot ->
// U[:, r]; returns the first maximum of |column| over unused rows.
template <int BS>
__device__ void col_pass(const AcaTask& T, const PointsF64& P, const KernelDesc& kd, int col,
                         int r, double pivot, const double* __restrict__ vbuf,
                         double* __restrict__ U, const unsigned char* __restrict__ used_r,
                         AcaShared& S, double& amax, int& aidx) {
  const int qc = T.s0 + col;
  const double xj = P.x[qc], yj = P.y[qc], zj = P.z[qc];
  double bv = 0.0;
  int bi = -1;
  bool bad = false;
  for (int t = threadIdx.x; t < T.n; t += BS) {
    const int q = T.t0 + t;
    double e = entry64_offdiag(kd, __dsub_rn(P.x[q], xj), __dsub_rn(P.y[q], yj),
                               __dsub_rn(P.z[q], zj));
    for (int l = 0; l < r; ++l) e = __dsub_rn(e, __dmul_rn(vbuf[l], U[(size_t)l * T.n + t]));
    const double u = __ddiv_rn(e, pivot);
    U[(size_t)r * T.n + t] = u;
    if (!isfinite(u)) bad = true;
    if (!used_r[t]) argmax_merge(bv, bi, fabs(e), t);
  }
  if (bad) S.flag_bad = 1;
  block_argmax<BS>(bv, bi, S, amax, aidx);
}

// The larger pairs (the leaf pairs run in k_aca_warp, one warp each):
// 256-thread blocks, one per SM with all the registers they want (134,
// nothing spilled); held to 64 registers so that four fit, they spill and
// run slower: 5.8 s of ACA kernels at 64^3 against 6.8-7.0 s.
template <int BS>
__global__ void __launch_bounds__(BS, 1) k_aca(const AcaTask* __restrict__ tasks, int ntasks,
                                            int* __restrict__ counter, PointsF64 P, KernelDesc kd,
                                            double tol, double* __restrict__ ws,
                                            unsigned char* __restrict__ flags,
                                            int32_t* __restrict__ piv, int32_t* __restrict__ out_rank,
                                            int32_t* __restrict__ out_status) {
  extern __shared__ double dyn[];
  __shared__ AcaShared S;
  __shared__ int s_task;
  constexpr int NW = BS / 32;
  const int tid = threadIdx.x, w = tid >> 5, lane = tid & 31;
  for (;;) {
    if (tid == 0) s_task = atomicAdd(counter, 1);
    __syncthreads();
    const int ti = s_task;
    __syncthreads();
    if (ti >= ntasks) break;
    const AcaTask T = tasks[ti];
    double* ubuf = dyn;
    double* vbuf = dyn + T.cap;
    double* du = dyn + 2 * T.cap;
    double* dv = dyn + 3 * T.cap;
    double* U = ws + T.ws_off;
    double* V = U + (size_t)T.cap * T.n;
    unsigned char* used_r = flags + T.fl_off;
    unsigned char* used_c = used_r + T.n;
    int32_t* rows = piv + T.piv_off;
    int32_t* cols = rows + T.cap;
    const int mn = min(T.n, T.m);
    if (mn == 0 || T.cap == 0) {
      if (tid == 0) {
        out_rank[ti] = 0;
        out_status[ti] = mn == 0 ? 0 : 1;
      }
      continue;
    }
    for (int i = tid; i < T.n + T.m; i += BS) used_r[i] = 0;
    if (tid == 0) S.flag_bad = 0;
    __syncthreads();
    // first row with a maximum above 1e-16 (src/ACA.cpp:153-161)
    double amax;
    int aidx;
    int row_index = -1, col_index = -1;
    for (int l = 0; l < T.n; ++l) {
      row_pass<BS>(T, P, kd, l, 0, ubuf, U, V, used_c, S, amax, aidx);
      if (amax > 1e-16) {
        row_index = l;
        col_index = aidx;
        break;
      }
    }
    int status = 0;
    int r = 0;
    if (row_index >= 0) {
      const double pivot0 = V[col_index];
      if (tid == 0) used_r[row_index] = 1;
      __syncthreads();
      col_pass<BS>(T, P, kd, col_index, 0, pivot0, vbuf, U, used_r, S, amax, aidx);
      if (tid == 0) {
        rows[0] = row_index;
        cols[0] = col_index;
        used_c[col_index] = 1;
      }
      int next_row = aidx;
      r = 1;
      // norms of the first pair of vectors (loop test, src/ACA.cpp:178)
      if (w == 0) {
        const double s2 = warp_canonical_dot(U, U, T.n, lane);
        if (lane == 0) S.nu = sqrt(s2);
      }
      if (w == (NW > 1 ? 1 : 0)) {
        const double s2 = warp_canonical_dot(V, V, T.m, lane);
        if (lane == 0) S.nv = sqrt(s2);
      }
      if (tid == 0) S.normS = 0.0;
      __syncthreads();
      row_index = next_row;
      for (;;) {
        if (S.flag_bad) {
          status = 2;
          break;
        }
        if (!(__dmul_rn(S.nu, S.nv) > __dmul_rn(tol, S.normS) && r < mn)) break;
        if (r >= T.cap) {
          status = 1;
          break;
        }
        for (int l = tid; l < r; l += BS) ubuf[l] = U[(size_t)l * T.n + row_index];
        __syncthreads();
        row_pass<BS>(T, P, kd, row_index, r, ubuf, U, V, used_c, S, amax, aidx);
        col_index = aidx;
        const double pivot = V[(size_t)r * T.m + col_index];
        for (int l = tid; l < r; l += BS) vbuf[l] = V[(size_t)l * T.m + col_index];
        if (tid == 0) used_r[row_index] = 1;
        __syncthreads();
        col_pass<BS>(T, P, kd, col_index, r, pivot, vbuf, U, used_r, S, amax, aidx);
        next_row = aidx;
        const double* un = U + (size_t)r * T.n;
        const double* vn = V + (size_t)r * T.m;
        double nu2 = 0.0, nv2 = 0.0;
        if (w == 0) {
          nu2 = warp_canonical_dot(un, un, T.n, lane);
          if (lane == 0) {
            du[r] = nu2;
            S.nu = sqrt(nu2);
          }
        }
        if (w == (NW > 1 ? 1 : 0)) {
          nv2 = warp_canonical_dot(vn, vn, T.m, lane);
          if (lane == 0) {
            dv[r] = nv2;
            S.nv = sqrt(nv2);
          }
        }
        __syncthreads();
        if (S.flag_bad) {
          status = 2;
          break;
        }
        if (S.nu < 1e-16 || S.nv < 1e-16) break;  // src/ACA.cpp:199-203
        if (tid == 0) {
          rows[r] = row_index;
          cols[r] = col_index;
          used_c[col_index] = 1;
        }
        // dot products with every kept vector (src/ACA.cpp:212-214)
        for (int job = w; job < 2 * r; job += NW) {
          const int l = job >> 1;
          if (job & 1) {
            const double d = warp_canonical_dot(V + (size_t)l * T.m, vn, T.m, lane);
            if (lane == 0) dv[l] = d;
          } else {
            const double d = warp_canonical_dot(U + (size_t)l * T.n, un, T.n, lane);
            if (lane == 0) du[l] = d;
          }
        }
        ++r;
        __syncthreads();
        if (tid == 0) {
          const double p = __dmul_rn(S.nu, S.nv);
          double ns = __dadd_rn(__dmul_rn(S.normS, S.normS), __dmul_rn(p, p));
          for (int l = 0; l < r; ++l) ns = __dadd_rn(ns, __dmul_rn(2.0, fabs(__dmul_rn(du[l], dv[l]))));
          S.normS = __dsqrt_rn(ns);
        }
        __syncthreads();
        row_index = next_row;
      }
    } else if (S.flag_bad) {
      status = 2;
    }
    if (tid == 0) {
      out_rank[ti] = r;
      out_status[ti] = status;
    }
    __syncthreads();
  }
}

// One warp per pair (pairs of at most 128 points a side, the leaf level): the
// steps of k_aca with warp shuffles for every reduction and no block
// barrier, per-warp scratch (ubuf, vbuf, du, dv: cap_max doubles each) in
// shared memory, each warp pulling pairs from the work counter.  Every
// result is the same as k_aca's: the entries, residuals and quotients are the
// same operations; the argmax is a total order (|value| descending, ties to
// the lowest index) and the dot products canonical reductions, neither of
// which depends on how the work is split.
template <int WPB>
__global__ void __launch_bounds__(32 * WPB, kAcaWarpBlocksPerSm) k_aca_warp(const AcaTask* __restrict__ tasks, int ntasks,
                                                        int* __restrict__ counter, PointsF64 P,
                                                        KernelDesc kd, double tol, int cap_max,
                                                        double* __restrict__ ws,
                                                        unsigned char* __restrict__ flags,
                                                        int32_t* __restrict__ piv,
                                                        int32_t* __restrict__ out_rank,
                                                        int32_t* __restrict__ out_status) {
  extern __shared__ double dyn[];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  double* ubuf = dyn + (size_t)4 * cap_max * w;
  double* vbuf = ubuf + cap_max;
  double* du = vbuf + cap_max;
  double* dv = du + cap_max;
  for (;;) {
    int ti = 0;
    if (lane == 0) ti = atomicAdd(counter, 1);
    ti = __shfl_sync(0xffffffffu, ti, 0);
    if (ti >= ntasks) break;
    const AcaTask T = tasks[ti];
    double* U = ws + T.ws_off;
    double* V = U + (size_t)T.cap * T.n;
    unsigned char* used_r = flags + T.fl_off;
    unsigned char* used_c = used_r + T.n;
    int32_t* rows = piv + T.piv_off;
    int32_t* cols = rows + T.cap;
    const int mn = min(T.n, T.m);
    if (mn == 0 || T.cap == 0) {
      if (lane == 0) {
        out_rank[ti] = 0;
        out_status[ti] = mn == 0 ? 0 : 1;
      }
      continue;
    }
    for (int i = lane; i < T.n + T.m; i += 32) used_r[i] = 0;
    __syncwarp();
    bool bad = false;
    // residual row `row` with r terms -> V[:, r]; first max of |row| over
    // unused columns (all lanes get it)
    auto row_pass = [&](int row, int r, double& amax, int& aidx) {
      const double xi = P.x[T.t0 + row], yi = P.y[T.t0 + row], zi = P.z[T.t0 + row];
      double bv = 0.0;
      int bi = -1;
      bool b = false;
      for (int s = lane; s < T.m; s += 32) {
        const int q = T.s0 + s;
        double e = entry64_offdiag(kd, __dsub_rn(xi, P.x[q]), __dsub_rn(yi, P.y[q]), __dsub_rn(zi, P.z[q]));
        for (int l = 0; l < r; ++l) e = __dsub_rn(e, __dmul_rn(ubuf[l], V[(size_t)l * T.m + s]));
        V[(size_t)r * T.m + s] = e;
        if (!isfinite(e)) b = true;
        if (!used_c[s]) argmax_merge(bv, bi, fabs(e), s);
      }
      bad = bad || __any_sync(0xffffffffu, b);
      warp_argmax(bv, bi);
      amax = bv;
      aidx = bi;
      __syncwarp();
    };
    // residual column `col` with r terms, divided by the pivot -> U[:, r];
    // first max of |column| over unused rows
    auto col_pass = [&](int col, int r, double pivot, double& amax, int& aidx) {
      const int qc = T.s0 + col;
      const double xj = P.x[qc], yj = P.y[qc], zj = P.z[qc];
      double bv = 0.0;
      int bi = -1;
      bool b = false;
      for (int t = lane; t < T.n; t += 32) {
        const int q = T.t0 + t;
        double e = entry64_offdiag(kd, __dsub_rn(P.x[q], xj), __dsub_rn(P.y[q], yj), __dsub_rn(P.z[q], zj));
        for (int l = 0; l < r; ++l) e = __dsub_rn(e, __dmul_rn(vbuf[l], U[(size_t)l * T.n + t]));
        const double u = __ddiv_rn(e, pivot);
        U[(size_t)r * T.n + t] = u;
        if (!isfinite(u)) b = true;
        if (!used_r[t]) argmax_merge(bv, bi, fabs(e), t);
      }
      bad = bad || __any_sync(0xffffffffu, b);
      warp_argmax(bv, bi);
      amax = bv;
      aidx = bi;
      __syncwarp();
    };
    // first row with a maximum above 1e-16 (src/ACA.cpp:153-161)
    double amax;
    int aidx;
    int row_index = -1, col_index = -1;
    for (int l = 0; l < T.n; ++l) {
      row_pass(l, 0, amax, aidx);
      if (amax > 1e-16) {
        row_index = l;
        col_index = aidx;
        break;
      }
    }
    int status = 0;
    int r = 0;
    if (row_index >= 0) {
      const double pivot0 = V[col_index];
      if (lane == 0) used_r[row_index] = 1;
      __syncwarp();
      col_pass(col_index, 0, pivot0, amax, aidx);
      if (lane == 0) {
        rows[0] = row_index;
        cols[0] = col_index;
        used_c[col_index] = 1;
      }
      int next_row = aidx;
      r = 1;
      // norms of the first pair of vectors (loop test, src/ACA.cpp:178)
      double nu = sqrt(warp_canonical_dot(U, U, T.n, lane));
      double nv = sqrt(warp_canonical_dot(V, V, T.m, lane));
      double normS = 0.0;
      __syncwarp();
      row_index = next_row;
      for (;;) {
        if (bad) {
          status = 2;
          break;
        }
        if (!(__dmul_rn(nu, nv) > __dmul_rn(tol, normS) && r < mn)) break;
        if (r >= T.cap) {
          status = 1;
          break;
        }
        for (int l = lane; l < r; l += 32) ubuf[l] = U[(size_t)l * T.n + row_index];
        __syncwarp();
        row_pass(row_index, r, amax, aidx);
        col_index = aidx;
        const double pivot = V[(size_t)r * T.m + col_index];
        for (int l = lane; l < r; l += 32) vbuf[l] = V[(size_t)l * T.m + col_index];
        if (lane == 0) used_r[row_index] = 1;
        __syncwarp();
        col_pass(col_index, r, pivot, amax, aidx);
        next_row = aidx;
        const double* un = U + (size_t)r * T.n;
        const double* vn = V + (size_t)r * T.m;
        const double nu2 = warp_canonical_dot(un, un, T.n, lane);
        const double nv2 = warp_canonical_dot(vn, vn, T.m, lane);
        if (lane == 0) {
          du[r] = nu2;
          dv[r] = nv2;
        }
        nu = sqrt(nu2);
        nv = sqrt(nv2);
        if (bad) {
          status = 2;
          break;
        }
        if (nu < 1e-16 || nv < 1e-16) break;  // src/ACA.cpp:199-203
        if (lane == 0) {
          rows[r] = row_index;
          cols[r] = col_index;
          used_c[col_index] = 1;
        }
        // dot products with every kept vector (src/ACA.cpp:212-214)
        for (int l = 0; l < r; ++l) {
          const double a = warp_canonical_dot(U + (size_t)l * T.n, un, T.n, lane);
          const double c = warp_canonical_dot(V + (size_t)l * T.m, vn, T.m, lane);
          if (lane == 0) {
            du[l] = a;
            dv[l] = c;
          }
        }
        ++r;
        __syncwarp();
        double ns = 0.0;
        if (lane == 0) {
          const double p = __dmul_rn(nu, nv);
          ns = __dadd_rn(__dmul_rn(normS, normS), __dmul_rn(p, p));
          for (int l = 0; l < r; ++l) ns = __dadd_rn(ns, __dmul_rn(2.0, fabs(__dmul_rn(du[l], dv[l]))));
          ns = __dsqrt_rn(ns);
        }
        normS = __shfl_sync(0xffffffffu, ns, 0);
        row_index = next_row;
      }
    } else if (bad) {
      status = 2;
    }
    if (lane == 0) {
      out_rank[ti] = r;
      out_status[ti] = status;
    }
    __syncwarp();
  }
}

// Copies the first r columns of U and V of every task into the final FP64
// pool at dst_off: U (n x r) then V (m x r), column-major.  (The FP32 copies
// are written after the assembly, grouped by box: k_u32, k_v32.)
__global__ void k_aca_compact(const AcaTask* __restrict__ tasks, const int32_t* __restrict__ rank,
                              const int64_t* __restrict__ dst_off, const double* __restrict__ ws,
                              double* __restrict__ out64) {
  const AcaTask T = tasks[blockIdx.x];
  const int r = rank[blockIdx.x];
  const double* U = ws + T.ws_off;
  const double* V = U + (size_t)T.cap * T.n;
  const int64_t o = dst_off[blockIdx.x];
  const int64_t nu = (int64_t)r * T.n, nv = (int64_t)r * T.m;
  for (int64_t i = threadIdx.x; i < nu; i += blockDim.x) out64[o + i] = U[i];
  for (int64_t i = threadIdx.x; i < nv; i += blockDim.x) out64[o + nu + i] = V[i];
}

// FP32 U of every pair (split-exact form) from its FP64 U (n x r,
// column-major): row-major with row stride us[p] (the sum of the padded ranks
// of the pairs of its target box, whose U share the rows), its r columns
// followed by zeros up to round4(r), at u32[p]; one block per pair.  lo != 0:
// the remainders instead, FP64 value minus the split-exact value, rounded.
__global__ void k_u32(const double* const* __restrict__ u64, float* const* __restrict__ u32,
                      const int32_t* __restrict__ nsize, const int32_t* __restrict__ us,
                      const int32_t* __restrict__ rank, int lo) {
  const int64_t p = blockIdx.x;
  const int r = rank[p];
  if (r <= 0) return;
  const int rp = (r + 3) & ~3;
  const int64_t n = nsize[p], st = us[p];
  const double* src = u64[p];
  float* dst = u32[p];
  for (int64_t e = threadIdx.x; e < n * rp; e += blockDim.x) {
    const int64_t i = e / rp;
    const int l = (int)(e - i * rp);
    float v = 0.f;
    if (l < r) {
      const double a = src[(int64_t)l * n + i];
      v = lo ? (float)(a - (double)tf32_split_value(a)) : tf32_split_value(a);
    }
    dst[i * st + l] = v;
  }
}

// FP32 V of every pair (split-exact form) from its FP64 V (m x r,
// column-major): column-major with the leading dimension padded to
// mp = round4(m), padding zero, at v32[p]; one block per pair.  lo != 0: the
// remainders, as k_u32.
__global__ void k_v32(const double* const* __restrict__ v64, float* const* __restrict__ v32,
                      const int32_t* __restrict__ msize, const int32_t* __restrict__ rank, int lo) {
  const int64_t p = blockIdx.x;
  const int r = rank[p];
  if (r <= 0) return;
  const int64_t m = msize[p], mp = (m + 3) & ~int64_t(3);
  const double* src = v64[p];
  float* dst = v32[p];
  for (int64_t e = threadIdx.x; e < mp * r; e += blockDim.x) {
    const int64_t l = e / mp, i = e - l * mp;
    float v = 0.f;
    if (i < m) {
      const double a = src[l * m + i];
      v = lo ? (float)(a - (double)tf32_split_value(a)) : tf32_split_value(a);
    }
    dst[e] = v;
  }
}

size_t aca_shared_bytes(int cap_max) { return (size_t)4 * cap_max * sizeof(double); }

cudaError_t launch_aca(cudaStream_t s, int grid, const AcaTask* tasks, int ntasks, int* counter,
                       PointsF64 P, KernelDesc kd, double tol, double* ws, unsigned char* flags,
                       int32_t* piv, int32_t* out_rank, int32_t* out_status, int cap_max) {
  const size_t shm = aca_shared_bytes(cap_max);
  cudaError_t e = cudaFuncSetAttribute(k_aca<kAcaBlock>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)shm);
  if (e != cudaSuccess) return e;
  k_aca<kAcaBlock><<<grid, kAcaBlock, shm, s>>>(tasks, ntasks, counter, P, kd, tol, ws, flags, piv,
                                                out_rank, out_status);
  return cudaGetLastError();
}

size_t aca_warp_shared_bytes(int cap_max) { return (size_t)kAcaWarpsPerBlock * 4 * cap_max * sizeof(double); }

cudaError_t launch_aca_warp(cudaStream_t s, int grid, const AcaTask* tasks, int ntasks, int* counter,
                            PointsF64 P, KernelDesc kd, double tol, double* ws, unsigned char* flags,
                            int32_t* piv, int32_t* out_rank, int32_t* out_status, int cap_max) {
  const size_t shm = aca_warp_shared_bytes(cap_max);
  cudaError_t e = cudaFuncSetAttribute(k_aca_warp<kAcaWarpsPerBlock>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)shm);
  if (e != cudaSuccess) return e;
  k_aca_warp<kAcaWarpsPerBlock><<<grid, 32 * kAcaWarpsPerBlock, shm, s>>>(
      tasks, ntasks, counter, P, kd, tol, cap_max, ws, flags, piv, out_rank, out_status);
  return cudaGetLastError();
}

cudaError_t launch_aca_compact(cudaStream_t s, int ntasks, const AcaTask* tasks,
                               const int32_t* rank, const int64_t* dst_off, const double* ws,
                               double* out64) {
  k_aca_compact<<<ntasks, 256, 0, s>>>(tasks, rank, dst_off, ws, out64);
  return cudaGetLastError();
}

cudaError_t launch_u32(cudaStream_t s, int64_t npairs, const double* const* u64, float* const* u32,
                       const int32_t* nsize, const int32_t* us, const int32_t* rank, int lo) {
  if (npairs <= 0) return cudaSuccess;
  k_u32<<<(unsigned)npairs, 256, 0, s>>>(u64, u32, nsize, us, rank, lo);
  return cudaGetLastError();
}

cudaError_t launch_v32(cudaStream_t s, int64_t npairs, const double* const* v64, float* const* v32,
                       const int32_t* msize, const int32_t* rank, int lo) {
  if (npairs <= 0) return cudaSuccess;
  k_v32<<<(unsigned)npairs, 256, 0, s>>>(v64, v32, msize, rank, lo);
  return cudaGetLastError();
}

}  // namespace h3d
