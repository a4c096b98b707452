// The extern "C" entry points of include/hodlr3d.h.
#include "host.h"

using namespace hodlr3d_host;

// ===========================================================================
// C ABI
// ===========================================================================
extern "C" {

int hodlr3d_abi_version(void) { return HODLR3D_ABI_VERSION; }

const char* hodlr3d_last_error(void) { return g_last_error.c_str(); }

void hodlr3d_default_options(hodlr3d_options* opt) {
  if (!opt) return;
  opt->device = 0;
  opt->diag_override = NAN;
  opt->keep_fp32 = 1;
  opt->aca_workspace_bytes = 0;
  opt->rank_cap = 0;
}

int hodlr3d_create(const double* xyz, int64_t n, int nP1D, double L, int tol_pow, int kernel_id,
                   const hodlr3d_options* opt, hodlr3d_t* out) try {
  if (!out) return set_error(HODLR3D_ERR_INVALID_ARG, "null output handle");
  *out = nullptr;
  if (!xyz || n < 2) return set_error(HODLR3D_ERR_INVALID_ARG, "need at least 2 points");
  if (n > INT32_MAX / 2) return set_error(HODLR3D_ERR_INVALID_ARG, "too many points");
  if (nP1D < 1) return set_error(HODLR3D_ERR_INVALID_ARG, "nParticlesInLeafAlong1D must be >= 1");
  if (!(L > 0.0)) return set_error(HODLR3D_ERR_INVALID_ARG, "L must be positive");
  if (tol_pow < 0 || tol_pow > 30) return set_error(HODLR3D_ERR_INVALID_ARG, "TOL_POW out of range");
  if (!kernel_supported(kernel_id)) return set_error(HODLR3D_ERR_INVALID_ARG, "unknown Qchoice %d", kernel_id);
  for (int64_t i = 0; i < 3 * n; ++i)
    if (!std::isfinite(xyz[i])) return set_error(HODLR3D_ERR_NONFINITE, "non-finite coordinate");
  // depth as the reference computes it (src/HODLR3D.cpp:6-7)
  const double cubeRootN = std::pow(double(n), 1.0 / 3.0);
  const int levels = (int)std::ceil(3 * std::log(double(cubeRootN) / nP1D) / std::log(8));
  if (levels < 1) return set_error(HODLR3D_ERR_INVALID_ARG, "the tree would have %d levels (< 1)", levels);
  if (levels > h3d::kMaxLevels) return set_error(HODLR3D_ERR_INVALID_ARG, "the tree would have %d levels (> %d)", levels, h3d::kMaxLevels);
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0)
    return set_error(HODLR3D_ERR_NO_DEVICE, "no CUDA device");
  hodlr3d_handle* h = new hodlr3d_handle();
  if (opt) h->opt = *opt;
  else hodlr3d_default_options(&h->opt);
  h->device = h->opt.device;
  if (h->device < 0 || h->device >= ndev) {
    delete h;
    return set_error(HODLR3D_ERR_INVALID_ARG, "device %d out of range", h->opt.device);
  }
  cudaError_t e = cudaSetDevice(h->device);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&h->num_sms, cudaDevAttrMultiProcessorCount, h->device);
  if (e != cudaSuccess) {
    delete h;
    return set_error(HODLR3D_ERR_CUDA, "device setup: %s", cudaGetErrorString(e));
  }
  h->N = n;
  h->nP1D = nP1D;
  h->L = L;
  h->tol_pow = tol_pow;
  h->tol = std::pow(10, -1.0 * tol_pow);  // src/ACA.cpp:5
  h->levels = levels;
  h->kd.kind = kernel_id;
  if (kernel_id == 16) {
    h->kd.kii = quadrature_kii(n);
    h->kd.h3 = 1.0 / double(n);
  }
  h->kd.diag = std::isnan(h->opt.diag_override) ? (kernel_id == 16 ? h->kd.kii : 0.0)
                                                : h->opt.diag_override;
  const int st = build_tree(h, xyz);
  if (st != HODLR3D_OK) {
    delete h;
    return st;
  }
  *out = h;
  return HODLR3D_OK;
} catch (...) {
  return exception_status();
}

void hodlr3d_destroy(hodlr3d_t h) {
  if (!h) return;
  cudaSetDevice(h->device);
  if (h->stream) cudaStreamSynchronize(h->stream);
  delete h;
}

int hodlr3d_assemble(hodlr3d_t h) try {
  H3D_TRY(check_handle(h));
  return assemble(h);
} catch (...) {
  return exception_status();
}

int hodlr3d_save(hodlr3d_t h, const char* path) try {
  H3D_TRY(check_handle(h));
  if (!path) return set_error(HODLR3D_ERR_INVALID_ARG, "null path");
  return save_factors(h, path);
} catch (...) {
  return exception_status();
}

int hodlr3d_load(const char* path, const hodlr3d_options* opt, hodlr3d_t* out) try {
  if (!out) return set_error(HODLR3D_ERR_INVALID_ARG, "null output handle");
  *out = nullptr;
  if (!path) return set_error(HODLR3D_ERR_INVALID_ARG, "null path");
  return load_factors(path, opt, out);
} catch (...) {
  return exception_status();
}

int hodlr3d_matvec(hodlr3d_t h, const double* x, double* y, int nrhs, int64_t ld, int precision,
                   void* stream) try {
  H3D_TRY(check_handle(h));
  return matvec_device(h, x, y, nrhs, ld, precision, (cudaStream_t)stream, false);
} catch (...) {
  return exception_status();
}

int hodlr3d_matvec_transpose(hodlr3d_t h, const double* x, double* y, int nrhs, int64_t ld,
                             int precision, void* stream) try {
  H3D_TRY(check_handle(h));
  return matvec_device(h, x, y, nrhs, ld, precision, (cudaStream_t)stream, true);
} catch (...) {
  return exception_status();
}

int hodlr3d_matvec_noalloc(hodlr3d_t h, const double* x, double* y, int nrhs, int64_t ld,
                           int precision, void* stream) try {
  H3D_TRY(check_handle(h));
  if (!h->assembled) return set_error(HODLR3D_ERR_NOT_ASSEMBLED, "hodlr3d_assemble has not run");
  if (!x || !y) return set_error(HODLR3D_ERR_INVALID_ARG, "null vector");
  if (nrhs < 1 || nrhs > 64) return set_error(HODLR3D_ERR_INVALID_ARG, "nrhs must be in 1..64");
  if (ld < h->N) return set_error(HODLR3D_ERR_INVALID_ARG, "ld < n");
  if (precision != HODLR3D_FP64 && precision != HODLR3D_MIXED && precision != HODLR3D_FP64X)
    return set_error(HODLR3D_ERR_INVALID_ARG, "unknown precision %d", precision);
  if (precision == HODLR3D_MIXED && !h->opt.keep_fp32)
    return set_error(HODLR3D_ERR_INVALID_ARG, "mixed precision needs keep_fp32");
  if (precision == HODLR3D_FP64X) precision = HODLR3D_FP64;  // the CUDA-core kernels only
  // the work buffers of the product, carved from the fixed scratch array
  const int nr = h3d::padded_nrhs(nrhs);
  const size_t s_real = precision == HODLR3D_MIXED ? sizeof(float) : sizeof(double);
  auto up = [](size_t b) { return (b + 255) & ~size_t(255); };
  const size_t b_x = up(s_real * h->N * nr);
  const size_t b_t = up(s_real * std::max<int64_t>(h->sum_rank, 1) * nr);
  const size_t b_p = up(sizeof(double) * std::max<int64_t>(h->part_total, 1) * nr);
  const size_t b_y = up(sizeof(double) * h->N * nr);
  const size_t need = b_x + b_t + b_p + b_y;
  if (need > h3d::kNoAllocScratchBytes)
    return set_error(HODLR3D_ERR_INVALID_ARG,
                     "hodlr3d_matvec_noalloc needs %zu bytes of scratch for n = %lld and nrhs = %d; "
                     "its fixed scratch holds %zu bytes (use hodlr3d_matvec)",
                     need, (long long)h->N, nrhs, (size_t)h3d::kNoAllocScratchBytes);
  void* base = nullptr;
  H3D_CUDA(h3d::noalloc_scratch(h->device, &base));
  unsigned char* b8 = static_cast<unsigned char*>(base);
  const bool f32 = precision == HODLR3D_MIXED;
  const h3d::FarOp far = far_op(h, f32);
  const h3d::NearOp nrop = near_op(h);
  h3d::MatvecBuffers B{};
  B.xsorted = b8;
  B.tbuf = b8 + b_x;
  B.pbuf = reinterpret_cast<double*>(b8 + b_x + b_t);
  B.ynl = reinterpret_cast<double*>(b8 + b_x + b_t + b_p);
  B.items = h->items.as<int32_t>();
  B.n_items = h->n_items;
  B.upper_pairs = h->upper.as<int32_t>();
  B.n_upper = h->n_upper;
  B.max_slice = h->max_slice;
  h->launches += h3d::launch_matvec((cudaStream_t)stream, h->N, h->perm.as<int32_t>(), far, nrop, B,
                                    x, ld, y, ld, nrhs, precision, 0, nullptr);
  H3D_CUDA(cudaGetLastError());
  return HODLR3D_OK;
} catch (...) {
  return exception_status();
}

int hodlr3d_matvec_host(hodlr3d_t h, const double* x, double* y, int nrhs, int64_t ld,
                        int precision) try {
  H3D_TRY(check_handle(h));
  if (!x || !y) return set_error(HODLR3D_ERR_INVALID_ARG, "null vector");
  if (nrhs < 1 || nrhs > 64 || ld < h->N) return set_error(HODLR3D_ERR_INVALID_ARG, "bad nrhs or ld");
  // products still in flight on the caller's streams use the same work buffers
  H3D_CUDA(cudaDeviceSynchronize());
  const size_t bytes = sizeof(double) * h->N * nrhs;
  H3D_CUDA(h->stage_x.ensure(bytes));
  H3D_CUDA(h->stage_y.ensure(bytes));
  cudaStream_t s = h->stream;
  // the copy engines read and write the caller's (pageable) columns directly
  const size_t col = sizeof(double) * h->N, pitch = sizeof(double) * ld;
  H3D_CUDA(cudaMemcpy2DAsync(h->stage_x.p, col, x, pitch, col, nrhs, cudaMemcpyHostToDevice, s));
  H3D_TRY(matvec_device(h, h->stage_x.as<double>(), h->stage_y.as<double>(), nrhs, h->N, precision, s, false));
  H3D_CUDA(cudaMemcpy2DAsync(y, pitch, h->stage_y.p, col, col, nrhs, cudaMemcpyDeviceToHost, s));
  H3D_CUDA(cudaStreamSynchronize(s));
  return HODLR3D_OK;
} catch (...) {
  return exception_status();
}

int hodlr3d_matvec_host_rows(hodlr3d_t h, const double* x, double* y, int nrhs, int precision) try {
  H3D_TRY(check_handle(h));
  if (!x || !y) return set_error(HODLR3D_ERR_INVALID_ARG, "null vector");
  if (nrhs < 1 || nrhs > 64) return set_error(HODLR3D_ERR_INVALID_ARG, "bad nrhs");
  // products still in flight on the caller's streams use the same work buffers
  H3D_CUDA(cudaDeviceSynchronize());
  const size_t bytes = sizeof(double) * h->N * nrhs;
  H3D_CUDA(h->stage_x.ensure(bytes));
  H3D_CUDA(h->stage_y.ensure(bytes));
  H3D_CUDA(h->stage_t.ensure(bytes));
  cudaStream_t s = h->stream;
  H3D_CUDA(cudaMemcpyAsync(h->stage_t.p, x, bytes, cudaMemcpyHostToDevice, s));
  h3d::launch_transpose(s, h->stage_t.as<double>(), h->N, nrhs, h->stage_x.as<double>());
  H3D_TRY(matvec_device(h, h->stage_x.as<double>(), h->stage_y.as<double>(), nrhs, h->N, precision, s, false));
  h3d::launch_transpose(s, h->stage_y.as<double>(), nrhs, h->N, h->stage_t.as<double>());
  h->launches += 2;
  H3D_CUDA(cudaGetLastError());
  H3D_CUDA(cudaMemcpyAsync(y, h->stage_t.p, bytes, cudaMemcpyDeviceToHost, s));
  H3D_CUDA(cudaStreamSynchronize(s));
  return HODLR3D_OK;
} catch (...) {
  return exception_status();
}

int hodlr3d_dense_rows(hodlr3d_t h, const int64_t* rows, int64_t nrows, const double* x, double* y,
                       int nrhs, int64_t ldx, void* stream) try {
  H3D_TRY(check_handle(h));
  if (!rows || !x || !y || nrows < 0 || nrhs < 1 || ldx < h->N)
    return set_error(HODLR3D_ERR_INVALID_ARG, "bad arguments");
  // one block per (row, column): the grid's limits
  if (nrows > INT32_MAX || nrhs > 65535)
    return set_error(HODLR3D_ERR_INVALID_ARG, "nrows must be <= 2^31 - 1 and nrhs <= 65535");
  h3d::launch_dense_rows((cudaStream_t)stream, h->N, h->xyz.as<double>(), h->kd,
                         rows, nrows, x, ldx, y, nrhs);
  ++h->launches;
  H3D_CUDA(cudaGetLastError());
  return HODLR3D_OK;
} catch (...) {
  return exception_status();
}

int hodlr3d_quadrature_kii(int64_t n, double* kii) try {
  if (n < 1 || !kii) return set_error(HODLR3D_ERR_INVALID_ARG, "n must be >= 1 and kii non-null");
  *kii = quadrature_kii(n);
  return HODLR3D_OK;
} catch (...) {
  return exception_status();
}

int hodlr3d_entries(hodlr3d_t h, const int64_t* rows, const int64_t* cols, int64_t n,
                    double* out) try {
  H3D_TRY(check_handle(h));
  if (n < 0 || (n > 0 && (!rows || !cols || !out)))
    return set_error(HODLR3D_ERR_INVALID_ARG, "bad arguments");
  if (n == 0) return HODLR3D_OK;
  for (int64_t e = 0; e < n; ++e)
    if (rows[e] < 0 || rows[e] >= h->N || cols[e] < 0 || cols[e] >= h->N)
      return set_error(HODLR3D_ERR_INVALID_ARG, "entry %lld: ids (%lld, %lld) outside [0, %lld)",
                       (long long)e, (long long)rows[e], (long long)cols[e], (long long)h->N);
  DevBuf rc, v;
  H3D_CUDA(rc.ensure(sizeof(int64_t) * 2 * n));
  H3D_CUDA(v.ensure(sizeof(double) * n));
  cudaStream_t s = h->stream;
  H3D_CUDA(cudaMemcpyAsync(rc.p, rows, sizeof(int64_t) * n, cudaMemcpyHostToDevice, s));
  H3D_CUDA(cudaMemcpyAsync(rc.as<int64_t>() + n, cols, sizeof(int64_t) * n, cudaMemcpyHostToDevice, s));
  h3d::launch_entries(s, h->N, h->xyz.as<double>(), h->kd, rc.as<int64_t>(), n, v.as<double>());
  ++h->launches;
  H3D_CUDA(cudaGetLastError());
  H3D_CUDA(cudaMemcpyAsync(out, v.p, sizeof(double) * n, cudaMemcpyDeviceToHost, s));
  H3D_CUDA(cudaStreamSynchronize(s));
  return HODLR3D_OK;
} catch (...) {
  return exception_status();
}

int hodlr3d_gmres(hodlr3d_t h, const double* b, double* x, int nrhs, int64_t ld,
                  const hodlr3d_gmres_params* prm, hodlr3d_gmres_result* res, double* hist,
                  int hist_cap, int* n_hist, void* stream) try {
  H3D_TRY(check_handle(h));
  if (!h->assembled) return set_error(HODLR3D_ERR_NOT_ASSEMBLED, "hodlr3d_assemble has not run");
  if (!b || !x || !prm || nrhs < 1 || nrhs > 64 || ld < h->N || prm->maxit < 1 || !(prm->tol > 0))
    return set_error(HODLR3D_ERR_INVALID_ARG, "bad GMRES arguments");
  // inputs may still be in flight on the caller's stream, and products on
  // the caller's streams use the same work buffers
  H3D_CUDA(cudaStreamSynchronize((cudaStream_t)stream));
  H3D_CUDA(cudaDeviceSynchronize());
  cudaStream_t s = h->stream;
  const int64_t N = h->N;
  const int64_t vec = N * nrhs;
  H3D_CUDA(h->g_b.ensure(sizeof(double) * vec));
  H3D_CUDA(h->g_x.ensure(sizeof(double) * vec));
  H3D_CUDA(h->g_d.ensure(sizeof(double) * vec));
  h->launches += h3d::gmres_pack(s, N, nrhs, b, ld, h->g_b.as<double>(), N);
  H3D_CUDA(cudaMemsetAsync(h->g_x.p, 0, sizeof(double) * vec, s));
  H3D_CUDA(h->g_part.ensure(sizeof(double) * nrhs * 1024));
  H3D_CUDA(h->g_scal.ensure(sizeof(double) * nrhs));
  h->launches += h3d::gmres_dot(s, N, nrhs, h->g_b.as<double>(), nullptr, nullptr, nullptr, 0, 1,
                                h->g_part.as<double>(), h->g_scal.as<double>(), 1);
  std::vector<double> bnorm(nrhs);
  H3D_CUDA(cudaMemcpyAsync(bnorm.data(), h->g_scal.p, sizeof(double) * nrhs, cudaMemcpyDeviceToHost, s));
  H3D_CUDA(cudaStreamSynchronize(s));
  for (int c = 0; c < nrhs; ++c)
    if (bnorm[c] == 0.0) bnorm[c] = 1.0;  // b = 0: x = 0 is exact
  const bool trans = prm->transpose != 0;
  std::vector<double> history, err;
  std::vector<double>* hp = hist ? &history : nullptr;
  if (hp) hp->push_back(1.0);
  int total_it = 0, outer = 0;
  bool brk = false, converged = false;
  double final_err = 0.0;
  if (prm->precision == HODLR3D_FP64 || prm->precision == HODLR3D_FP64X) {
    const int m = prm->restart > 0 ? prm->restart : prm->maxit;
    bool first = true;
    while (total_it < prm->maxit) {
      int it = 0;
      const int mm = std::min(m, prm->maxit - total_it);
      H3D_TRY(gmres_cycle(h, h->g_b.as<double>(), h->g_x.as<double>(), nrhs, mm, prm->tol, prm->precision,
                          trans, first, bnorm, &it, err, hp, &brk));
      first = false;
      total_it += it;
      ++outer;
      final_err = *std::max_element(err.begin(), err.end());
      converged = final_err <= prm->tol;
      if (converged || prm->restart <= 0 || it == 0) break;
    }
  } else {
    // iterative refinement: FP64 residual, FP32-matvec inner GMRES(m) on the correction
    const int m = prm->restart > 0 ? prm->restart : 30;
    const int max_outer = prm->max_outer > 0 ? prm->max_outer : 20;
    const double itol = prm->inner_tol > 0 ? prm->inner_tol : 1e-5;
    double* r = h->g_d.as<double>();
    H3D_CUDA(cudaMemcpyAsync(r, h->g_b.p, sizeof(double) * vec, cudaMemcpyDeviceToDevice, s));
    DevBuf dx, wtmp;
    H3D_CUDA(dx.ensure(sizeof(double) * vec));
    H3D_CUDA(wtmp.ensure(sizeof(double) * vec));
    for (outer = 0; outer < max_outer && total_it < prm->maxit; ++outer) {
      // relative residual of the current x in FP64
      h->launches += h3d::gmres_dot(s, N, nrhs, r, nullptr, nullptr, nullptr, 0, 1,
                                    h->g_part.as<double>(), h->g_scal.as<double>(), 1);
      std::vector<double> rn(nrhs);
      H3D_CUDA(cudaMemcpyAsync(rn.data(), h->g_scal.p, sizeof(double) * nrhs, cudaMemcpyDeviceToHost, s));
      H3D_CUDA(cudaStreamSynchronize(s));
      final_err = 0.0;
      for (int c = 0; c < nrhs; ++c) final_err = std::max(final_err, rn[c] / bnorm[c]);
      if (hp && outer > 0) hp->push_back(final_err);
      if (final_err <= prm->tol) {
        converged = true;
        break;
      }
      // inner solve A d = r to relative accuracy itol (restarted until reached)
      H3D_CUDA(cudaMemsetAsync(dx.p, 0, sizeof(double) * vec, s));
      int inner_total = 0;
      bool first = true;
      while (inner_total < prm->maxit - total_it) {
        int it = 0;
        const int mm = std::min(m, prm->maxit - total_it - inner_total);
        H3D_TRY(gmres_cycle(h, r, dx.as<double>(), nrhs, mm, itol, HODLR3D_MIXED, trans, first, rn,
                            &it, err, nullptr, &brk));
        first = false;
        inner_total += it;
        if (*std::max_element(err.begin(), err.end()) <= itol || it == 0) break;
      }
      total_it += inner_total;
      h->launches += h3d::gmres_add(s, vec, dx.as<double>(), h->g_x.as<double>());
      // r = b - A x, the product FP64-accurate (FP32-pair arithmetic where the
      // few-column kernels take the tree, else FP64), the difference in FP64
      H3D_TRY(matvec_device(h, h->g_x.as<double>(), wtmp.as<double>(), nrhs, N, HODLR3D_FP64X, s, trans));
      h->launches += h3d::gmres_sub(s, vec, h->g_b.as<double>(), wtmp.as<double>(), r);
    }
    if (!converged) {
      h->launches += h3d::gmres_dot(s, N, nrhs, r, nullptr, nullptr, nullptr, 0, 1,
                                    h->g_part.as<double>(), h->g_scal.as<double>(), 1);
      std::vector<double> rn(nrhs);
      H3D_CUDA(cudaMemcpyAsync(rn.data(), h->g_scal.p, sizeof(double) * nrhs, cudaMemcpyDeviceToHost, s));
      H3D_CUDA(cudaStreamSynchronize(s));
      final_err = 0.0;
      for (int c = 0; c < nrhs; ++c) final_err = std::max(final_err, rn[c] / bnorm[c]);
      converged = final_err <= prm->tol;
    }
  }
  h->launches += h3d::gmres_pack(s, N, nrhs, h->g_x.as<double>(), N, x, ld);
  H3D_CUDA(cudaStreamSynchronize(s));
  if (res) {
    res->iterations = total_it;
    res->outer = outer;
    res->rel_residual = final_err;
    res->converged = converged ? 1 : 0;
  }
  if (hist && n_hist) {
    const int nh = std::min<int>(hist_cap, (int)history.size());
    for (int i = 0; i < nh; ++i) hist[i] = history[i];
    *n_hist = nh;
  }
  if (!converged) {
    if (brk) return set_error(HODLR3D_ERR_BREAKDOWN, "GMRES breakdown before the tolerance");
    return set_error(HODLR3D_ERR_NO_CONVERGENCE, "GMRES reached %d iterations at %.3e", total_it, final_err);
  }
  return HODLR3D_OK;
} catch (...) {
  return exception_status();
}

int hodlr3d_get_stats(hodlr3d_t h, hodlr3d_stats* s) try {
  if (!h || !s) return set_error(HODLR3D_ERR_INVALID_ARG, "null argument");
  std::memset(s, 0, sizeof(*s));
  s->n_points = h->N;
  s->levels = h->levels;
  s->n_pairs = h->npairs;
  s->max_rank = h->max_rank;
  s->sum_rank = h->sum_rank;
  s->factor_entries = h->factor_entries;
  s->u_entries = h->u_entries;
  s->v_entries = h->v_entries;
  s->factor_bytes_fp64 = h->factor_entries * 8;
  s->factor_bytes_fp32 = h->opt.keep_fp32 ? h->factor_entries * 4 : 0;
  s->tree_seconds = h->tree_seconds;
  s->assemble_seconds = h->assemble_seconds;
  s->aca_batches = h->aca_batches;
  s->aca_kernel_seconds = h->aca_kernel_seconds;
  s->finish_seconds = h->finish_seconds;
  // near blocks and the reference's memory count (findMemory, src/HODLR3DTree.cpp:1757-1778)
  const int d = h->levels;
  double mem = 0.0;
  int64_t nb = 0, ne = 0;
  std::vector<int32_t> nbl(26 * h->nleaf);
  if (cudaMemcpy(nbl.data(), h->nbr_leaf.p, sizeof(int32_t) * 26 * h->nleaf, cudaMemcpyDeviceToHost) != cudaSuccess)
    return set_error(HODLR3D_ERR_CUDA, "copy of the neighbour table failed");
  for (int64_t k = 0; k < h->nleaf; ++k) {
    const int64_t n = h->h_leaf_off[k + 1] - h->h_leaf_off[k];
    ++nb;
    ne += n * n;
    for (int sl = 0; sl < 26; ++sl) {
      const int32_t q = nbl[26 * k + sl];
      if (q < 0) continue;
      ++nb;
      ne += n * (int64_t)(h->h_leaf_off[q + 1] - h->h_leaf_off[q]);
    }
  }
  if (h->assembled) {
    for (int64_t p = 0; p < h->npairs; ++p) {
      const int j = h->h_pair_level[p];
      int64_t a0, a1, b0, b1;
      box_range(h, j, h->h_pair_tgt[p] - h3d::level_base(j), a0, a1);
      box_range(h, j, h->h_pair_src[p] - h3d::level_base(j), b0, b1);
      const double r = h->h_rank[p];
      mem += r * double(a1 - a0) + r * r + double(b1 - b0) * r;
    }
  }
  mem += (double)ne;
  (void)d;
  s->n_near_blocks = nb;
  s->near_entries = ne;
  s->memory_entries = mem;
  return HODLR3D_OK;
} catch (...) {
  return exception_status();
}

int hodlr3d_get_tree(hodlr3d_t h, int32_t* perm, int64_t* leaf_off) try {
  if (!h) return set_error(HODLR3D_ERR_INVALID_ARG, "null handle");
  if (perm) std::copy(h->h_perm.begin(), h->h_perm.end(), perm);
  if (leaf_off)
    for (int64_t k = 0; k <= h->nleaf; ++k) leaf_off[k] = h->h_leaf_off[k];
  return HODLR3D_OK;
} catch (...) {
  return exception_status();
}

int hodlr3d_get_neighbors(hodlr3d_t h, int level, int32_t* nbr) try {
  H3D_TRY(check_handle(h));
  if (!nbr || level < 0 || level > h->levels) return set_error(HODLR3D_ERR_INVALID_ARG, "bad level");
  const int64_t nb = int64_t(1) << (3 * level);
  H3D_CUDA(cudaMemcpy(nbr, h->nbr_all.as<int32_t>() + 26 * h3d::level_base(level),
                      sizeof(int32_t) * 26 * nb, cudaMemcpyDeviceToHost));
  return HODLR3D_OK;
} catch (...) {
  return exception_status();
}

int hodlr3d_get_pairs(hodlr3d_t h, int32_t* lts) try {
  if (!h || !lts) return set_error(HODLR3D_ERR_INVALID_ARG, "null argument");
  for (int64_t p = 0; p < h->npairs; ++p) {
    const int j = h->h_pair_level[p];
    lts[3 * p] = j;
    lts[3 * p + 1] = (int32_t)(h->h_pair_tgt[p] - h3d::level_base(j));
    lts[3 * p + 2] = (int32_t)(h->h_pair_src[p] - h3d::level_base(j));
  }
  return HODLR3D_OK;
} catch (...) {
  return exception_status();
}

int hodlr3d_get_ranks(hodlr3d_t h, int32_t* rank) try {
  if (!h || !rank) return set_error(HODLR3D_ERR_INVALID_ARG, "null argument");
  if (!h->assembled) return set_error(HODLR3D_ERR_NOT_ASSEMBLED, "not assembled");
  std::copy(h->h_rank.begin(), h->h_rank.end(), rank);
  return HODLR3D_OK;
} catch (...) {
  return exception_status();
}

int hodlr3d_get_pivots(hodlr3d_t h, int32_t* rows, int32_t* cols) try {
  if (!h || !rows || !cols) return set_error(HODLR3D_ERR_INVALID_ARG, "null argument");
  if (!h->assembled) return set_error(HODLR3D_ERR_NOT_ASSEMBLED, "not assembled");
  int64_t w = 0;
  for (int64_t p = 0; p < h->npairs; ++p) {
    const int j = h->h_pair_level[p];
    int64_t a0, a1, b0, b1;
    box_range(h, j, h->h_pair_tgt[p] - h3d::level_base(j), a0, a1);
    box_range(h, j, h->h_pair_src[p] - h3d::level_base(j), b0, b1);
    for (int r = 0; r < h->h_rank[p]; ++r) {
      rows[w] = h->h_perm[a0 + h->h_piv_rows[p][r]];
      cols[w] = h->h_perm[b0 + h->h_piv_cols[p][r]];
      ++w;
    }
  }
  return HODLR3D_OK;
} catch (...) {
  return exception_status();
}

int hodlr3d_get_pair_factors(hodlr3d_t h, int64_t pair, double* U, double* V) try {
  H3D_TRY(check_handle(h));
  if (!h->assembled) return set_error(HODLR3D_ERR_NOT_ASSEMBLED, "not assembled");
  if (pair < 0 || pair >= h->npairs) return set_error(HODLR3D_ERR_INVALID_ARG, "pair out of range");
  const int j = h->h_pair_level[pair];
  int64_t a0, a1, b0, b1;
  box_range(h, j, h->h_pair_tgt[pair] - h3d::level_base(j), a0, a1);
  box_range(h, j, h->h_pair_src[pair] - h3d::level_base(j), b0, b1);
  const int64_t r = h->h_rank[pair];
  if (U && r) H3D_CUDA(cudaMemcpy(U, h->h_u64[pair], sizeof(double) * r * (a1 - a0), cudaMemcpyDeviceToHost));
  if (V && r) H3D_CUDA(cudaMemcpy(V, h->h_v64[pair], sizeof(double) * r * (b1 - b0), cudaMemcpyDeviceToHost));
  return HODLR3D_OK;
} catch (...) {
  return exception_status();
}

int64_t hodlr3d_launch_count(hodlr3d_t h) { return h ? h->launches : 0; }

int hodlr3d_set_engine(hodlr3d_t h, int engine) try {
  if (!h || engine < 0 || engine > 3) return set_error(HODLR3D_ERR_INVALID_ARG, "engine must be 0, 1, 2 or 3");
  h->engine = engine;
  return HODLR3D_OK;
} catch (...) {
  return exception_status();
}

int hodlr3d_autotune(hodlr3d_t h, int reps, char* report, int cap) try {
  H3D_TRY(check_handle(h));
  if (reps < 0 || reps > 1000) return set_error(HODLR3D_ERR_INVALID_ARG, "reps must be in 0..1000");
  // products still in flight on the caller's streams use the same work buffers
  H3D_CUDA(cudaDeviceSynchronize());
  std::string rep;
  H3D_TRY(autotune(h, reps, rep));
  if (report && cap > 0) {
    const size_t n = std::min(rep.size(), (size_t)cap - 1);
    std::memcpy(report, rep.data(), n);
    report[n] = 0;
  }
  return HODLR3D_OK;
} catch (...) {
  return exception_status();
}

int hodlr3d_get_tuning(hodlr3d_t h, int32_t* choice) try {
  if (!h || !choice) return set_error(HODLR3D_ERR_INVALID_ARG, "null argument");
  for (int t = 0; t < 2; ++t)
    for (int n = 1; n <= 64; ++n) choice[64 * t + n - 1] = h->tuned[t][n];
  return HODLR3D_OK;
} catch (...) {
  return exception_status();
}

int hodlr3d_device_status(hodlr3d_t h) try {
  H3D_TRY(check_handle(h));
  H3D_CUDA(cudaDeviceSynchronize());
  int v = 0;
  if (h->dev_err.p) H3D_CUDA(cudaMemcpy(&v, h->dev_err.p, sizeof(int), cudaMemcpyDeviceToHost));
  if (v) H3D_CUDA(cudaMemset(h->dev_err.p, 0, sizeof(int)));  // reported once
  if (v == 2)
    return set_error(HODLR3D_ERR_CUDA, "a tensor-core block's operand table overflowed (results of that call are invalid)");
  if (v) return set_error(HODLR3D_ERR_CUDA, "a tensor-core wait gave up (results of that call are invalid)");
  return HODLR3D_OK;
} catch (...) {
  return exception_status();
}

int hodlr3d_test_drop_copy(hodlr3d_t h, int chunk) try {
  H3D_TRY(check_handle(h));
  if (chunk < -1) return set_error(HODLR3D_ERR_INVALID_ARG, "chunk %d < -1", chunk);
  H3D_CUDA(h3d::tc_set_drop_chunk(chunk));
  return HODLR3D_OK;
} catch (...) {
  return exception_status();
}

int hodlr3d_set_profiling(hodlr3d_t h, int enable) try {
  if (!h) return set_error(HODLR3D_ERR_INVALID_ARG, "null handle");
  h->profiling = enable != 0;
  h->prof.spans.clear();
  h->prof.used = 0;
  return HODLR3D_OK;
} catch (...) {
  return exception_status();
}

int hodlr3d_profile_report(hodlr3d_t h, char* buf, int cap) try {
  H3D_TRY(check_handle(h));
  if (!buf || cap <= 0) return set_error(HODLR3D_ERR_INVALID_ARG, "bad buffer");
  std::vector<std::string> names;
  std::vector<double> ms;
  std::vector<int> cnt;
  for (auto& sp : h->prof.spans) {
    H3D_CUDA(cudaEventSynchronize(sp.second.second));
    float t = 0.f;
    H3D_CUDA(cudaEventElapsedTime(&t, sp.second.first, sp.second.second));
    size_t i = 0;
    while (i < names.size() && names[i] != sp.first) ++i;
    if (i == names.size()) {
      names.push_back(sp.first);
      ms.push_back(0.0);
      cnt.push_back(0);
    }
    ms[i] += t;
    cnt[i] += 1;
  }
  std::string out;
  for (size_t i = 0; i < names.size(); ++i) {
    char line[128];
    snprintf(line, sizeof(line), "%s %d %.6f\n", names[i].c_str(), cnt[i], ms[i]);
    out += line;
  }
  h->prof.spans.clear();
  h->prof.used = 0;
  snprintf(buf, (size_t)cap, "%s", out.c_str());
  return HODLR3D_OK;
} catch (...) {
  return exception_status();
}

}  // extern "C"
