// Device building blocks of the batched GMRES: fused modified Gram-Schmidt
// passes, deterministic two-stage reductions, Givens rotations on the device
// and the final update x += Q y.  All right-hand sides advance together; each
// column has its own Krylov space and Hessenberg matrix.
//
// Reference: classGMRES (src/gmres.cpp:5-94): arnoldi (MGS, :29-38),
// givensRotation / applyGivensRotation (:5-26), the residual estimate
// |beta(k+1)| / |b| (:80) and the final solve x = x + Q y (:91-93).
//
// Vectors are column-major, N x nrhs with leading dimension N.
#include "gmres.h"

namespace h3d {

constexpr int kRedBlock = 256;

// partial[b, c] = sum over the rows of block b of a[:, c] * b[:, c]; when
// `upd` is set first applies q[:, c] -= coef[c] * u[:, c] (the MGS update of
// the previous step) and takes the product with the updated q.
__global__ void __launch_bounds__(kRedBlock) k_mgs_pass(int64_t N, int nrhs, double* __restrict__ q,
                                                        const double* __restrict__ u,
                                                        const double* __restrict__ coef,
                                                        const double* __restrict__ w,
                                                        double* __restrict__ partial, int upd,
                                                        int self) {
  __shared__ double red[kRedBlock / 32];
  const int c = blockIdx.y;
  double* qc = q + (int64_t)c * N;
  const double* uc = u ? u + (int64_t)c * N : nullptr;
  const double* wc = w ? w + (int64_t)c * N : nullptr;
  const double h = upd ? coef[c] : 0.0;
  double acc = 0.0;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < N;
       t += (int64_t)gridDim.x * blockDim.x) {
    double v = qc[t];
    if (upd) {
      v = v - h * uc[t];
      qc[t] = v;
    }
    acc += v * (self ? v : wc[t]);
  }
  acc = warp_sum_d(acc);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x < 32) {
    double v = threadIdx.x < kRedBlock / 32 ? red[threadIdx.x] : 0.0;
    v = warp_sum_d(v);
    if (threadIdx.x == 0) partial[(int64_t)c * gridDim.x + blockIdx.x] = v;
  }
}

// out[c] = sum of the nblk partials of column c (fixed order); sqrt if asked.
__global__ void k_reduce_final(int nblk, int nrhs, const double* __restrict__ partial,
                               double* __restrict__ out, int take_sqrt) {
  const int c = blockIdx.x;
  __shared__ double red[32];
  double acc = 0.0;
  for (int b = threadIdx.x; b < nblk; b += blockDim.x) acc += partial[(int64_t)c * nblk + b];
  acc = warp_sum_d(acc);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x < 32) {
    double v = threadIdx.x < blockDim.x / 32 ? red[threadIdx.x] : 0.0;
    v = warp_sum_d(v);
    if (threadIdx.x == 0) out[c] = take_sqrt ? sqrt(v) : v;
  }
}

// y[:, c] = alpha[c]-scaled copy: y = x / s[c] (s == 0 gives 0)
__global__ void k_scale_copy(int64_t N, int nrhs, const double* __restrict__ x,
                             const double* __restrict__ s, double* __restrict__ y) {
  const int64_t o = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (o >= N * nrhs) return;
  const int c = (int)(o / N);
  const double d = s[c];
  y[o] = d != 0.0 ? x[o] / d : 0.0;
}

// y = a - b (elementwise, N * nrhs)
__global__ void k_sub(int64_t n, const double* __restrict__ a, const double* __restrict__ b,
                      double* __restrict__ y) {
  const int64_t o = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (o < n) y[o] = a[o] - b[o];
}

// y += x (elementwise)
__global__ void k_add(int64_t n, const double* __restrict__ x, double* __restrict__ y) {
  const int64_t o = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (o < n) y[o] += x[o];
}

// Column k of every Hessenberg matrix: rotate by the previous Givens
// rotations, form and apply the new one, update beta and the estimate.
// H is [nrhs][m][m + 1] (column-major per column c), hk holds the fresh
// coefficients h(0..k+1) of column k for every c ([nrhs][m + 1]).
__global__ void k_givens(int k, int m, int nrhs, const double* __restrict__ hk,
                         double* __restrict__ H, double* __restrict__ cs, double* __restrict__ sn,
                         double* __restrict__ beta, const double* __restrict__ bnorm,
                         double* __restrict__ err, int* __restrict__ breakdown) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= nrhs) return;
  double* h = H + ((int64_t)c * m + k) * (m + 1);
  const double* src = hk + (int64_t)c * (m + 1);
  for (int i = 0; i <= k + 1; ++i) h[i] = src[i];
  double* csc = cs + (int64_t)c * m;
  double* snc = sn + (int64_t)c * m;
  double* bc = beta + (int64_t)c * (m + 1);
  if (h[k + 1] == 0.0) breakdown[c] = 1;
  for (int i = 0; i < k; ++i) {
    const double tmp = csc[i] * h[i] + snc[i] * h[i + 1];
    h[i + 1] = -snc[i] * h[i] + csc[i] * h[i + 1];
    h[i] = tmp;
  }
  const double t = sqrt(h[k] * h[k] + h[k + 1] * h[k + 1]);
  const double ck = t != 0.0 ? h[k] / t : 1.0;
  const double sk = t != 0.0 ? h[k + 1] / t : 0.0;
  csc[k] = ck;
  snc[k] = sk;
  h[k] = ck * h[k] + sk * h[k + 1];
  h[k + 1] = 0.0;
  bc[k + 1] = -sk * bc[k];
  bc[k] = ck * bc[k];
  err[c] = fabs(bc[k + 1]) / bnorm[c];
}

// Solves R y = beta(0..kc) for each column (kc = kcol[c], R upper triangular
// from the rotated Hessenberg), one thread per column.
__global__ void k_solve_upper(int m, int nrhs, const double* __restrict__ H,
                              const double* __restrict__ beta, const int* __restrict__ kcol,
                              double* __restrict__ y) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= nrhs) return;
  const int n = kcol[c] + 1;
  const double* Hc = H + (int64_t)c * m * (m + 1);
  const double* bc = beta + (int64_t)c * (m + 1);
  double* yc = y + (int64_t)c * m;
  for (int i = m - 1; i >= n; --i) yc[i] = 0.0;
  for (int i = n - 1; i >= 0; --i) {
    double s = bc[i];
    for (int j = i + 1; j < n; ++j) s -= Hc[(int64_t)j * (m + 1) + i] * yc[j];
    const double dgl = Hc[(int64_t)i * (m + 1) + i];
    yc[i] = dgl != 0.0 ? s / dgl : 0.0;
  }
}

// x[:, c] += sum_l Q_l[:, c] y[c, l], l < nvec
__global__ void k_update_x(int64_t N, int nrhs, int nvec, int m, const double* __restrict__ Q,
                           const double* __restrict__ y, double* __restrict__ x, int64_t ldx) {
  const int64_t o = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (o >= N * nrhs) return;
  const int c = (int)(o / N);
  const int64_t t = o - (int64_t)c * N;
  double s = 0.0;
  for (int l = 0; l < nvec; ++l) s += Q[(int64_t)l * N * nrhs + o] * y[(int64_t)c * m + l];
  x[(int64_t)c * ldx + t] += s;
}

// copies between a column-major (ld) user array and a packed N x nrhs array
__global__ void k_pack(int64_t N, int nrhs, const double* __restrict__ a, int64_t lda,
                       double* __restrict__ b, int64_t ldb) {
  const int64_t o = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (o >= N * nrhs) return;
  const int c = (int)(o / N);
  const int64_t t = o - (int64_t)c * N;
  b[(int64_t)c * ldb + t] = a[(int64_t)c * lda + t];
}

static int nblocks_for(int64_t N) {
  int64_t b = (N + kRedBlock * 4 - 1) / (kRedBlock * 4);
  if (b > 1024) b = 1024;
  if (b < 1) b = 1;
  return (int)b;
}

int gmres_dot(cudaStream_t s, int64_t N, int nrhs, double* q, const double* u, const double* coef,
              const double* w, int upd, int self, double* partial, double* out, int take_sqrt) {
  const int nb = nblocks_for(N);
  k_mgs_pass<<<dim3(nb, nrhs), kRedBlock, 0, s>>>(N, nrhs, q, u, coef, w, partial, upd, self);
  k_reduce_final<<<nrhs, 256, 0, s>>>(nb, nrhs, partial, out, take_sqrt);
  return 2;
}

int gmres_scale_copy(cudaStream_t s, int64_t N, int nrhs, const double* x, const double* sc,
                     double* y) {
  const int64_t n = N * nrhs;
  k_scale_copy<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(N, nrhs, x, sc, y);
  return 1;
}

int gmres_sub(cudaStream_t s, int64_t n, const double* a, const double* b, double* y) {
  k_sub<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(n, a, b, y);
  return 1;
}

int gmres_add(cudaStream_t s, int64_t n, const double* x, double* y) {
  k_add<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(n, x, y);
  return 1;
}

int gmres_givens(cudaStream_t s, int k, int m, int nrhs, const double* hk, double* H, double* cs,
                 double* sn, double* beta, const double* bnorm, double* err, int* breakdown) {
  k_givens<<<(nrhs + 63) / 64, 64, 0, s>>>(k, m, nrhs, hk, H, cs, sn, beta, bnorm, err, breakdown);
  return 1;
}

int gmres_solve_update(cudaStream_t s, int64_t N, int nrhs, int m, const double* H,
                       const double* beta, const int* kcol, double* y, const double* Q, int nvec,
                       double* x, int64_t ldx) {
  k_solve_upper<<<(nrhs + 63) / 64, 64, 0, s>>>(m, nrhs, H, beta, kcol, y);
  const int64_t n = N * nrhs;
  k_update_x<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(N, nrhs, nvec, m, Q, y, x, ldx);
  return 2;
}

int gmres_pack(cudaStream_t s, int64_t N, int nrhs, const double* a, int64_t lda, double* b,
               int64_t ldb) {
  const int64_t n = N * nrhs;
  k_pack<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(N, nrhs, a, lda, b, ldb);
  return 1;
}

}  // namespace h3d
