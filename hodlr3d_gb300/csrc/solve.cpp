// Host side: GMRES cycles on the device vectors (classGMRES, src/gmres.cpp).
#include "host.h"

namespace hodlr3d_host {

// ---------------------------------------------------------------------------
// GMRES
// ---------------------------------------------------------------------------
// One GMRES(m) cycle from the current x (device, packed N x nrhs, ld = N) for
// right-hand side b (packed).  Returns the iterations done; err_out holds the
// final estimates per column.  Matvec precision `prec`.
int gmres_cycle(hodlr3d_t h, const double* b, double* x, int nrhs, int m, double tol, int prec,
                bool trans, bool x_is_zero, const std::vector<double>& bnorm_h, int* iters,
                std::vector<double>& err_out, std::vector<double>* hist, bool* breakdown_any) {
  cudaStream_t s = h->stream;
  const int64_t N = h->N;
  const int64_t vec = N * nrhs;
  H3D_CUDA(h->g_Q.ensure(sizeof(double) * vec * (m + 1)));
  H3D_CUDA(h->g_w.ensure(sizeof(double) * vec));
  H3D_CUDA(h->g_r.ensure(sizeof(double) * vec));
  H3D_CUDA(h->g_H.ensure(sizeof(double) * nrhs * m * (m + 1)));
  H3D_CUDA(h->g_cs.ensure(sizeof(double) * nrhs * m));
  H3D_CUDA(h->g_sn.ensure(sizeof(double) * nrhs * m));
  H3D_CUDA(h->g_beta.ensure(sizeof(double) * nrhs * (m + 1)));
  H3D_CUDA(h->g_hk.ensure(sizeof(double) * nrhs * (m + 1)));
  H3D_CUDA(h->g_bnorm.ensure(sizeof(double) * nrhs));
  H3D_CUDA(h->g_err.ensure(sizeof(double) * nrhs));
  H3D_CUDA(h->g_part.ensure(sizeof(double) * nrhs * 1024));
  H3D_CUDA(h->g_y.ensure(sizeof(double) * nrhs * m));
  H3D_CUDA(h->g_kcol.ensure(sizeof(int) * nrhs));
  H3D_CUDA(h->g_brk.ensure(sizeof(int) * nrhs));
  H3D_CUDA(h->g_scal.ensure(sizeof(double) * nrhs));
  H3D_CUDA(h->g_coef.ensure(sizeof(double) * nrhs));
  double* Q = h->g_Q.as<double>();
  double* w = h->g_w.as<double>();
  double* r = h->g_r.as<double>();
  double* hk = h->g_hk.as<double>();
  // r = b - A x
  if (x_is_zero) {
    H3D_CUDA(cudaMemcpyAsync(r, b, sizeof(double) * vec, cudaMemcpyDeviceToDevice, s));
  } else {
    H3D_TRY(matvec_device(h, x, w, nrhs, N, prec, s, trans));
    h->launches += h3d::gmres_sub(s, vec, b, w, r);
  }
  H3D_CUDA(cudaMemcpyAsync(h->g_bnorm.p, bnorm_h.data(), sizeof(double) * nrhs, cudaMemcpyHostToDevice, s));
  // beta(0) = |r|, Q0 = r / |r|
  h->launches += h3d::gmres_dot(s, N, nrhs, r, nullptr, nullptr, nullptr, 0, 1, h->g_part.as<double>(),
                                h->g_scal.as<double>(), 1);
  H3D_CUDA(cudaMemsetAsync(h->g_beta.p, 0, sizeof(double) * nrhs * (m + 1), s));
  H3D_CUDA(cudaMemsetAsync(h->g_H.p, 0, sizeof(double) * nrhs * m * (m + 1), s));
  H3D_CUDA(cudaMemsetAsync(h->g_brk.p, 0, sizeof(int) * nrhs, s));
  H3D_CUDA(cudaMemcpy2DAsync(h->g_beta.p, sizeof(double) * (m + 1), h->g_scal.p, sizeof(double),
                             sizeof(double), nrhs, cudaMemcpyDeviceToDevice, s));
  h->launches += h3d::gmres_scale_copy(s, N, nrhs, r, h->g_scal.as<double>(), Q);
  std::vector<double> rn(nrhs), err(nrhs);
  H3D_CUDA(cudaMemcpyAsync(rn.data(), h->g_scal.p, sizeof(double) * nrhs, cudaMemcpyDeviceToHost, s));
  H3D_CUDA(cudaStreamSynchronize(s));
  std::vector<int> kcol(nrhs, -1);
  std::vector<char> done(nrhs, 0);
  bool all_done = true;
  for (int c = 0; c < nrhs; ++c) {
    err[c] = rn[c] / bnorm_h[c];
    if (err[c] <= tol || rn[c] == 0.0) done[c] = 1;
    all_done = all_done && done[c];
  }
  int k = 0;
  for (; k < m && !all_done; ++k) {
    double* Qk = Q + (int64_t)k * vec;
    double* Qn = Q + (int64_t)(k + 1) * vec;
    H3D_TRY(matvec_device(h, Qk, Qn, nrhs, N, prec, s, trans));
    // modified Gram-Schmidt (arnoldi, src/gmres.cpp:29-38) as fused passes:
    // pass i applies q -= h_{i-1} Q_{i-1} and forms h_i = q . Q_i; the last
    // pass forms h_{k+1} = |q|.
    for (int i = 0; i <= k + 1; ++i) {
      const bool upd = i > 0;
      const bool last = i == k + 1;
      h->launches += h3d::gmres_dot(s, N, nrhs, Qn, upd ? Q + (int64_t)(i - 1) * vec : nullptr,
                                    upd ? h->g_coef.as<double>() : nullptr,
                                    last ? nullptr : Q + (int64_t)i * vec, upd ? 1 : 0, last ? 1 : 0,
                                    h->g_part.as<double>(), h->g_scal.as<double>(), last ? 1 : 0);
      H3D_CUDA(cudaMemcpy2DAsync(hk + i, sizeof(double) * (m + 1), h->g_scal.p, sizeof(double),
                                 sizeof(double), nrhs, cudaMemcpyDeviceToDevice, s));
      if (!last)
        H3D_CUDA(cudaMemcpyAsync(h->g_coef.p, h->g_scal.p, sizeof(double) * nrhs,
                                 cudaMemcpyDeviceToDevice, s));
    }
    // Q_{k+1} = q / h_{k+1}
    h->launches += h3d::gmres_scale_copy(s, N, nrhs, Qn, h->g_scal.as<double>(), Qn);
    h->launches += h3d::gmres_givens(s, k, m, nrhs, hk, h->g_H.as<double>(), h->g_cs.as<double>(),
                                     h->g_sn.as<double>(), h->g_beta.as<double>(),
                                     h->g_bnorm.as<double>(), h->g_err.as<double>(),
                                     h->g_brk.as<int>());
    H3D_CUDA(cudaMemcpyAsync(err.data(), h->g_err.p, sizeof(double) * nrhs, cudaMemcpyDeviceToHost, s));
    H3D_CUDA(cudaStreamSynchronize(s));
    if (hist) hist->push_back(err[0]);
    all_done = true;
    for (int c = 0; c < nrhs; ++c) {
      if (!done[c] && err[c] <= tol) {
        done[c] = 1;
        kcol[c] = k;
      }
      all_done = all_done && done[c];
    }
  }
  const int kdone = k;  // iterations performed
  for (int c = 0; c < nrhs; ++c)
    if (kcol[c] < 0) kcol[c] = kdone - 1;
  if (kdone > 0) {
    H3D_CUDA(cudaMemcpyAsync(h->g_kcol.p, kcol.data(), sizeof(int) * nrhs, cudaMemcpyHostToDevice, s));
    h->launches += h3d::gmres_solve_update(s, N, nrhs, m, h->g_H.as<double>(), h->g_beta.as<double>(),
                                           h->g_kcol.as<int>(), h->g_y.as<double>(), Q, kdone, x, N);
  }
  std::vector<int> brk(nrhs);
  H3D_CUDA(cudaMemcpyAsync(brk.data(), h->g_brk.p, sizeof(int) * nrhs, cudaMemcpyDeviceToHost, s));
  H3D_CUDA(cudaStreamSynchronize(s));
  *breakdown_any = false;
  for (int c = 0; c < nrhs; ++c) *breakdown_any = *breakdown_any || brk[c];
  err_out = err;
  *iters = kdone;
  return HODLR3D_OK;
}

}  // namespace hodlr3d_host
