// Host side: error helpers, handle checks, the device tree build, the
// batched ACA orchestration and the tables built after it.
#include "host.h"

namespace hodlr3d_host {

thread_local std::string g_last_error;

int set_error(int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_last_error = buf;
  return code;
}

// The C entry points are function-try-blocks whose handler returns this: an
// exception (a host allocation that failed) becomes a status code instead of
// crossing the C ABI.
int exception_status() noexcept {
  try {
    throw;
  } catch (const std::bad_alloc&) {
    return set_error(HODLR3D_ERR_OUT_OF_MEMORY, "host allocation failed");
  } catch (const std::length_error&) {
    return set_error(HODLR3D_ERR_OUT_OF_MEMORY, "host allocation too large");
  } catch (const std::exception& e) {
    return set_error(HODLR3D_ERR_INVALID_ARG, "unexpected error: %s", e.what());
  } catch (...) {
    return set_error(HODLR3D_ERR_INVALID_ARG, "unexpected error");
  }
}


double now_s() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

// Gauss-Legendre nodes and weights on [-1, 1] by Newton iteration on the
// three-term Legendre recurrence (the classical "gauleg" method).
void gauss_legendre(int n, std::vector<double>& x, std::vector<double>& w) {
  x.assign(n, 0.0);
  w.assign(n, 0.0);
  for (int i = 0; i < (n + 1) / 2; ++i) {
    long double z = std::cos(3.1415926535897932384626L * (i + 0.75L) / (n + 0.5L));
    long double dp = 0.0L;
    for (int it = 0; it < 100; ++it) {
      long double p0 = 1.0L, p1 = 0.0L;
      for (int j = 1; j <= n; ++j) {
        const long double pm = p1;
        p1 = p0;
        p0 = ((2.0L * j - 1.0L) * z * p1 - (j - 1.0L) * pm) / j;
      }
      dp = n * (z * p0 - p1) / (z * z - 1.0L);
      const long double dz = p0 / dp;
      z -= dz;
      if (std::fabs((double)dz) < 1e-19) break;
    }
    x[i] = (double)(-z);
    x[n - 1 - i] = (double)z;
    const long double wi = 2.0L / ((1.0L - z * z) * dp * dp);
    w[i] = w[n - 1 - i] = (double)wi;
  }
}

// Diagonal of the second-kind integral operator (Qchoice 16): the integral of
// 1/(4 pi r) over the point's cell [-h/2, h/2]^3 (8 times the octant
// [0, h/2]^3, 16^3 Gauss-Legendre points) plus 1, h = 1 / cbrt(N)
// (include/kernel.hpp:43-61, src/Integral3D.cpp:9-43).
double quadrature_kii(int64_t N) {
  const double pi = 3.1415926535897932384;
  const double h = 1.0 / std::cbrt(double(N));
  std::vector<double> g, wg;
  gauss_legendre(16, g, wg);
  const double half = 0.5 * (h * 0.5), mid = 0.5 * (h * 0.5);
  double acc = 0.0;
  for (int i = 0; i < 16; ++i) {
    const double tx = half * g[i] + mid;
    for (int j = 0; j < 16; ++j) {
      const double ty = half * g[j] + mid;
      for (int k = 0; k < 16; ++k) {
        const double tz = half * g[k] + mid;
        const double f = 1.0 / ((4 * pi) * std::sqrt(tx * tx + ty * ty + tz * tz));
        acc += wg[i] * wg[j] * wg[k] * f;
      }
    }
  }
  acc *= (half * half * half);
  acc *= 8;
  return acc + 1.0;
}


int check_handle(hodlr3d_t h) {
  if (!h) return set_error(HODLR3D_ERR_INVALID_ARG, "null handle");
  cudaError_t e = cudaSetDevice(h->device);
  if (e != cudaSuccess) return set_error(HODLR3D_ERR_CUDA, "cudaSetDevice: %s", cudaGetErrorString(e));
  return HODLR3D_OK;
}

// every Qchoice of the reference (src/kernel.cpp:65-227) has a device form
bool kernel_supported(int k) { return k >= 0 && k <= 16; }

// ---------------------------------------------------------------------------
// tree
// ---------------------------------------------------------------------------
int build_tree(hodlr3d_t h, const double* xyz_host) {
  const double t_start = now_s();
  cudaStream_t s = h->stream;
  const int64_t N = h->N;
  const int d = h->levels;
  std::vector<double> radii(d + 1);
  radii[0] = h->L;
  for (int k = 1; k <= d; ++k) radii[k] = 0.5 * radii[k - 1];
  h->nleaf = int64_t(1) << (3 * d);
  h->nbox_all = h3d::level_base(d + 1);
  H3D_CUDA(h->xyz.ensure(sizeof(double) * 3 * N));
  H3D_CUDA(cudaMemcpyAsync(h->xyz.p, xyz_host, sizeof(double) * 3 * N, cudaMemcpyHostToDevice, s));
  DevBuf keys, keys_tmp, vals_tmp, counts;
  H3D_CUDA(keys.ensure(sizeof(uint32_t) * N));
  H3D_CUDA(keys_tmp.ensure(sizeof(uint32_t) * N));
  H3D_CUDA(vals_tmp.ensure(sizeof(int32_t) * N));
  H3D_CUDA(h->perm.ensure(sizeof(int32_t) * N));
  const int64_t ntiles = (N + 1023) / 1024;
  H3D_CUDA(counts.ensure(sizeof(int32_t) * 256 * ntiles));
  h3d::launch_leaf_keys(s, N, h->xyz.as<double>(), d, radii.data(), keys.as<uint32_t>(),
                        h->perm.as<int32_t>());
  int launches = 1;
  h3d::radix_sort_pairs(s, N, 3 * d, keys.as<uint32_t>(), h->perm.as<int32_t>(),
                        keys_tmp.as<uint32_t>(), vals_tmp.as<int32_t>(), counts.as<int32_t>(),
                        &launches);
  H3D_CUDA(h->leaf_off.ensure(sizeof(int32_t) * (h->nleaf + 1)));
  h3d::launch_leaf_offsets(s, N, keys.as<uint32_t>(), h->nleaf, h->leaf_off.as<int32_t>());
  H3D_CUDA(h->xs.ensure(8 * N));
  H3D_CUDA(h->ys.ensure(8 * N));
  H3D_CUDA(h->zs.ensure(8 * N));
  H3D_CUDA(h->xl.ensure(4 * N));
  H3D_CUDA(h->yl.ensure(4 * N));
  H3D_CUDA(h->zl.ensure(4 * N));
  H3D_CUDA(h->centre.ensure(sizeof(double) * 3 * h->nleaf));
  h3d::launch_gather_points(s, N, h->xyz.as<double>(), h->perm.as<int32_t>(), keys.as<uint32_t>(), d,
                            radii.data(), h->xs.as<double>(), h->ys.as<double>(),
                            h->zs.as<double>(), h->xl.as<float>(), h->yl.as<float>(),
                            h->zl.as<float>());
  h3d::launch_leaf_centres(s, h->nleaf, d, radii.data(), h->centre.as<double>());
  launches += 3;
  // neighbour slots and interaction lists, level by level: count, scan on the host, write
  H3D_CUDA(h->nbr_all.ensure(sizeof(int32_t) * 26 * h->nbox_all));
  H3D_CUDA(cudaMemsetAsync(h->nbr_all.p, 0xff, sizeof(int32_t) * 26 * h->nbox_all, s));
  DevBuf il_count;
  H3D_CUDA(il_count.ensure(sizeof(int32_t) * h->nbox_all));
  H3D_CUDA(cudaMemsetAsync(il_count.p, 0, sizeof(int32_t) * h->nbox_all, s));
  for (int j = 1; j <= d; ++j) {
    h3d::launch_box_lists(s, j, 0, nullptr, il_count.as<int32_t>(), nullptr, nullptr, nullptr);
    ++launches;
  }
  std::vector<int32_t> cnt(h->nbox_all);
  H3D_CUDA(cudaMemcpyAsync(cnt.data(), il_count.p, sizeof(int32_t) * h->nbox_all,
                           cudaMemcpyDeviceToHost, s));
  H3D_CUDA(cudaStreamSynchronize(s));
  h->h_il_ptr.assign(h->nbox_all + 1, 0);
  for (int64_t b = 0; b < h->nbox_all; ++b) h->h_il_ptr[b + 1] = h->h_il_ptr[b] + cnt[b];
  h->npairs = h->h_il_ptr[h->nbox_all];
  H3D_CUDA(h->il_ptr.ensure(sizeof(int64_t) * (h->nbox_all + 1)));
  H3D_CUDA(cudaMemcpyAsync(h->il_ptr.p, h->h_il_ptr.data(), sizeof(int64_t) * (h->nbox_all + 1),
                           cudaMemcpyHostToDevice, s));
  H3D_CUDA(h->pair_tgt.ensure(sizeof(int32_t) * std::max<int64_t>(1, h->npairs)));
  H3D_CUDA(h->pair_src.ensure(sizeof(int32_t) * std::max<int64_t>(1, h->npairs)));
  H3D_CUDA(h->rev.ensure(sizeof(int32_t) * std::max<int64_t>(1, h->npairs)));
  for (int j = 1; j <= d; ++j) {
    h3d::launch_box_lists(s, j, 1, h->nbr_all.as<int32_t>(), il_count.as<int32_t>(),
                          h->il_ptr.as<int64_t>(), h->pair_tgt.as<int32_t>(),
                          h->pair_src.as<int32_t>());
    ++launches;
  }
  DevBuf err;
  H3D_CUDA(err.ensure(sizeof(int32_t)));
  H3D_CUDA(cudaMemsetAsync(err.p, 0, sizeof(int32_t), s));
  h3d::launch_reverse_pairs(s, h->npairs, h->pair_tgt.as<int32_t>(), h->pair_src.as<int32_t>(),
                            h->il_ptr.as<int64_t>(), h->rev.as<int32_t>(), err.as<int32_t>());
  ++launches;
  // leaf neighbour table (a view of the leaf level of nbr_all, re-based to leaf ids)
  std::vector<int32_t> nb_leaf(26 * h->nleaf);
  H3D_CUDA(cudaMemcpyAsync(nb_leaf.data(),
                           h->nbr_all.as<int32_t>() + 26 * h3d::level_base(d),
                           sizeof(int32_t) * 26 * h->nleaf, cudaMemcpyDeviceToHost, s));
  h->h_perm.resize(N);
  h->h_leaf_off.resize(h->nleaf + 1);
  h->h_pair_tgt.resize(h->npairs);
  h->h_pair_src.resize(h->npairs);
  int32_t herr = 0;
  H3D_CUDA(cudaMemcpyAsync(h->h_perm.data(), h->perm.p, sizeof(int32_t) * N, cudaMemcpyDeviceToHost, s));
  H3D_CUDA(cudaMemcpyAsync(h->h_leaf_off.data(), h->leaf_off.p, sizeof(int32_t) * (h->nleaf + 1),
                           cudaMemcpyDeviceToHost, s));
  if (h->npairs) {
    H3D_CUDA(cudaMemcpyAsync(h->h_pair_tgt.data(), h->pair_tgt.p, sizeof(int32_t) * h->npairs,
                             cudaMemcpyDeviceToHost, s));
    H3D_CUDA(cudaMemcpyAsync(h->h_pair_src.data(), h->pair_src.p, sizeof(int32_t) * h->npairs,
                             cudaMemcpyDeviceToHost, s));
  }
  H3D_CUDA(cudaMemcpyAsync(&herr, err.p, sizeof(int32_t), cudaMemcpyDeviceToHost, s));
  H3D_CUDA(cudaStreamSynchronize(s));
  H3D_CUDA(cudaGetLastError());
  h->launches += launches;
  if (herr) return set_error(HODLR3D_ERR_CUDA, "interaction lists are not symmetric");
  H3D_CUDA(h->nbr_leaf.ensure(sizeof(int32_t) * 26 * h->nleaf));
  H3D_CUDA(cudaMemcpyAsync(h->nbr_leaf.p, nb_leaf.data(), sizeof(int32_t) * 26 * h->nleaf,
                           cudaMemcpyHostToDevice, s));
  h->h_pair_level.resize(h->npairs);
  for (int64_t p = 0; p < h->npairs; ++p) {
    int j = 0;
    while (h3d::level_base(j + 1) <= h->h_pair_tgt[p]) ++j;
    h->h_pair_level[p] = j;
  }
  h->max_leaf = 0;
  h->leaves_aligned = true;
  for (int64_t k = 0; k < h->nleaf; ++k) {
    const int nk = h->h_leaf_off[k + 1] - h->h_leaf_off[k];
    h->max_leaf = std::max(h->max_leaf, nk);
    if (nk % 4) h->leaves_aligned = false;
  }
  H3D_CUDA(cudaStreamSynchronize(s));
  h->tree_seconds = now_s() - t_start;
  return HODLR3D_OK;
}


// ---------------------------------------------------------------------------
// assembly
// ---------------------------------------------------------------------------
struct HostTask {
  int64_t pair;
  int32_t t0, n, s0, m;
  int32_t cap;
  bool leaf;
};

// FP32 copies of the factors (split-exact form), grouped by box:
// * U by target box: the pairs of box b (consecutive pair numbers) side by
//   side, U_p at columns [h_coff[p], + round4(r_p)) of one row-major
//   n_b x R_b matrix;
// * V by source box: the pairs whose source is box b (its reverse list) one
//   after the other, consecutive column-major round4(m_b) x r blocks, so that
//   they form one (sum of ranks) x round4(m_b) row-major matrix.
// Per-pair pointers keep working for the CUDA-core kernels (U row stride
// h_ustride[p]); the tensor-core kernels read one tensor map per box.
// Converted from the FP64 factors after the assembly.
int group_fp32(hodlr3d_t h) {
  const int64_t np = h->npairs;
  cudaStream_t s = h->stream;
  std::vector<int32_t> rev(std::max<int64_t>(np, 1));
  if (np)
    H3D_CUDA(cudaMemcpy(rev.data(), h->rev.p, sizeof(int32_t) * np, cudaMemcpyDeviceToHost));
  const int64_t nbox = (int64_t)h->h_il_ptr.size() - 1;
  h->h_vbox_off.assign(nbox + 1, 0);
  h->h_vbox_rows.assign(nbox, 0);
  h->h_ubox_off.assign(nbox + 1, 0);
  h->h_tbox_off.assign(nbox + 1, 0);
  h->h_rbox.assign(nbox, 0);
  h->h_ustride.assign(np, 0);
  h->h_coff.assign(np, 0);
  std::vector<int64_t> voff(np, 0);
  std::vector<int32_t> msize(np, 0), nsize(np, 0);
  int64_t vcur = 0, ucur = 0, tcur = 0;
  for (int64_t b = 0; b < nbox; ++b) {
    int j = 0;
    while (j < h->levels && h3d::level_base(j + 1) <= b) ++j;
    int64_t a0, a1;
    box_range(h, j, b - h3d::level_base(j), a0, a1);
    const int64_t m = a1 - a0, mp = (m + 3) & ~int64_t(3);
    h->h_vbox_off[b] = vcur;
    for (int64_t q = h->h_il_ptr[b]; q < h->h_il_ptr[b + 1]; ++q) {
      const int p = rev[q];
      voff[p] = vcur;
      msize[p] = (int32_t)m;
      vcur += (int64_t)h->h_rank[p] * mp;
      h->h_vbox_rows[b] += h->h_rank[p];
    }
    // the pairs with target b are the pair numbers il_ptr[b] .. il_ptr[b+1]
    int32_t R = 0;
    for (int64_t p = h->h_il_ptr[b]; p < h->h_il_ptr[b + 1]; ++p) {
      h->h_coff[p] = R;
      nsize[p] = (int32_t)m;
      R += (h->h_rank[p] + 3) & ~3;
    }
    h->h_rbox[b] = R;
    for (int64_t p = h->h_il_ptr[b]; p < h->h_il_ptr[b + 1]; ++p) h->h_ustride[p] = R;
    h->h_ubox_off[b] = ucur;
    ucur += m * R;
    h->h_tbox_off[b] = tcur;
    tcur += 32 * (int64_t)R;
  }
  h->h_vbox_off[nbox] = vcur;
  h->h_ubox_off[nbox] = ucur;
  h->h_tbox_off[nbox] = tcur;
  h->h_pair_m = msize;
  h->h_pair_n = nsize;
  h->lo_built = false;
  h->lo_unavailable = false;
  h->v32_pool = new DevBuf();
  h->pools.push_back(h->v32_pool);
  H3D_CUDA(h->v32_pool->ensure(sizeof(float) * std::max<int64_t>(vcur, 4)));
  h->u32_pool = new DevBuf();
  h->pools.push_back(h->u32_pool);
  H3D_CUDA(h->u32_pool->ensure(sizeof(float) * std::max<int64_t>(ucur, 4)));
  float* vbase = h->v32_pool->as<float>();
  float* ubase = h->u32_pool->as<float>();
  for (int64_t b = 0; b < nbox; ++b)
    for (int64_t p = h->h_il_ptr[b]; p < h->h_il_ptr[b + 1]; ++p)
      h->h_u32[p] = ubase + h->h_ubox_off[b] + h->h_coff[p];
  for (int64_t p = 0; p < np; ++p) h->h_v32[p] = vbase + voff[p];
  if (np) {
    DevBuf d64, d32, dm, dr, du64, du32, dn, dus;
    H3D_CUDA(d64.ensure(sizeof(void*) * np));
    H3D_CUDA(d32.ensure(sizeof(void*) * np));
    H3D_CUDA(dm.ensure(sizeof(int32_t) * np));
    H3D_CUDA(dr.ensure(sizeof(int32_t) * np));
    H3D_CUDA(du64.ensure(sizeof(void*) * np));
    H3D_CUDA(du32.ensure(sizeof(void*) * np));
    H3D_CUDA(dn.ensure(sizeof(int32_t) * np));
    H3D_CUDA(dus.ensure(sizeof(int32_t) * np));
    H3D_CUDA(cudaMemcpy(d64.p, h->h_v64.data(), sizeof(void*) * np, cudaMemcpyHostToDevice));
    H3D_CUDA(cudaMemcpy(d32.p, h->h_v32.data(), sizeof(void*) * np, cudaMemcpyHostToDevice));
    H3D_CUDA(cudaMemcpy(dm.p, msize.data(), sizeof(int32_t) * np, cudaMemcpyHostToDevice));
    H3D_CUDA(cudaMemcpy(dr.p, h->h_rank.data(), sizeof(int32_t) * np, cudaMemcpyHostToDevice));
    H3D_CUDA(cudaMemcpy(du64.p, h->h_u64.data(), sizeof(void*) * np, cudaMemcpyHostToDevice));
    H3D_CUDA(cudaMemcpy(du32.p, h->h_u32.data(), sizeof(void*) * np, cudaMemcpyHostToDevice));
    H3D_CUDA(cudaMemcpy(dn.p, nsize.data(), sizeof(int32_t) * np, cudaMemcpyHostToDevice));
    H3D_CUDA(cudaMemcpy(dus.p, h->h_ustride.data(), sizeof(int32_t) * np, cudaMemcpyHostToDevice));
    H3D_CUDA(h3d::launch_v32(s, np, d64.as<const double* const>(), d32.as<float* const>(),
                             dm.as<int32_t>(), dr.as<int32_t>(), 0));
    H3D_CUDA(h3d::launch_u32(s, np, du64.as<const double* const>(), du32.as<float* const>(),
                             dn.as<int32_t>(), dus.as<int32_t>(), dr.as<int32_t>(), 0));
    h->launches += 2;
    H3D_CUDA(cudaStreamSynchronize(s));
  }
  // device tables: U row strides; tensor-core T offsets per pair and per box
  std::vector<int64_t> toff(std::max<int64_t>(np, 1), 0);
  std::vector<int32_t> tld(std::max<int64_t>(np, 1), 0);
  for (int64_t b = 0; b < nbox; ++b)
    for (int64_t p = h->h_il_ptr[b]; p < h->h_il_ptr[b + 1]; ++p) {
      toff[p] = h->h_tbox_off[b] + h->h_coff[p];
      tld[p] = h->h_rbox[b];
    }
  const size_t npb = std::max<int64_t>(np, 1), nbb = std::max<int64_t>(nbox, 1);
  H3D_CUDA(h->ustride.ensure(sizeof(int32_t) * npb));
  H3D_CUDA(h->tc_toff.ensure(sizeof(int64_t) * npb));
  H3D_CUDA(h->tc_tld.ensure(sizeof(int32_t) * npb));
  H3D_CUDA(h->tc_tbox.ensure(sizeof(int64_t) * nbb));
  H3D_CUDA(h->tc_rbox.ensure(sizeof(int32_t) * nbb));
  if (np) {
    H3D_CUDA(cudaMemcpy(h->ustride.p, h->h_ustride.data(), sizeof(int32_t) * np, cudaMemcpyHostToDevice));
    H3D_CUDA(cudaMemcpy(h->tc_toff.p, toff.data(), sizeof(int64_t) * np, cudaMemcpyHostToDevice));
    H3D_CUDA(cudaMemcpy(h->tc_tld.p, tld.data(), sizeof(int32_t) * np, cudaMemcpyHostToDevice));
  }
  if (nbox) {
    H3D_CUDA(cudaMemcpy(h->tc_tbox.p, h->h_tbox_off.data(), sizeof(int64_t) * nbox, cudaMemcpyHostToDevice));
    H3D_CUDA(cudaMemcpy(h->tc_rbox.p, h->h_rbox.data(), sizeof(int32_t) * nbox, cudaMemcpyHostToDevice));
  }
  return HODLR3D_OK;
}

// The ACA batches of one pass: device buffers sized once for the largest
// batch and the batch in flight.
struct AcaLane {
  cudaStream_t s = nullptr;
  DevBuf d_tasks, d_ws, d_fl, d_pv, d_rank, d_status, d_counter, d_off;
  EventPair ev;
  std::vector<HostTask> batch;
  std::vector<h3d::AcaTask> tasks;
  int64_t pv = 0;
  bool small = false;
};

// workspace doubles, flag bytes and pivot entries of a batch
void batch_sizes(const std::vector<HostTask>& batch, int64_t& ws, int64_t& fl, int64_t& pv) {
  ws = fl = pv = 0;
  for (const HostTask& b : batch) {
    ws += (int64_t)b.cap * (b.n + b.m);
    fl += b.n + b.m;
    pv += 2 * (int64_t)b.cap;
  }
}

// Sizes the lane's buffers for the largest of its batches.
int aca_lane_reserve(AcaLane& L, const std::vector<std::vector<HostTask>>& batches) {
  int64_t nt = 1, ws = 1, fl = 1, pv = 1;
  for (const auto& b : batches) {
    int64_t w, f, p;
    batch_sizes(b, w, f, p);
    nt = std::max<int64_t>(nt, (int64_t)b.size());
    ws = std::max(ws, w);
    fl = std::max(fl, f);
    pv = std::max(pv, p);
  }
  H3D_CUDA(L.d_tasks.ensure(sizeof(h3d::AcaTask) * nt));
  H3D_CUDA(L.d_ws.ensure(sizeof(double) * ws));
  H3D_CUDA(L.d_fl.ensure(fl));
  H3D_CUDA(L.d_pv.ensure(sizeof(int32_t) * pv));
  H3D_CUDA(L.d_rank.ensure(sizeof(int32_t) * nt));
  H3D_CUDA(L.d_status.ensure(sizeof(int32_t) * nt));
  H3D_CUDA(L.d_counter.ensure(sizeof(int32_t)));
  H3D_CUDA(L.d_off.ensure(sizeof(int64_t) * nt));
  if (!L.ev.a) H3D_CUDA(cudaEventCreate(&L.ev.a));
  if (!L.ev.b) H3D_CUDA(cudaEventCreate(&L.ev.b));
  return HODLR3D_OK;
}

// Launches the ACA of a batch on the lane's stream (no host synchronisation).
int aca_launch(hodlr3d_t h, AcaLane& L, std::vector<HostTask>&& batch, bool small_kernel) {
  cudaStream_t s = L.s;
  L.batch = std::move(batch);
  L.small = small_kernel;
  const int nt = (int)L.batch.size();
  L.tasks.assign(nt, h3d::AcaTask{});
  int64_t ws = 0, fl = 0, pv = 0;
  int cap_max = 1;
  for (int i = 0; i < nt; ++i) {
    const HostTask& b = L.batch[i];
    h3d::AcaTask& t = L.tasks[i];
    t.t0 = b.t0;
    t.n = b.n;
    t.s0 = b.s0;
    t.m = b.m;
    t.cap = b.cap;
    t.pair = (int32_t)b.pair;
    t.ws_off = ws;
    t.fl_off = fl;
    t.piv_off = pv;
    ws += (int64_t)b.cap * (b.n + b.m);
    fl += b.n + b.m;
    pv += 2 * (int64_t)b.cap;
    cap_max = std::max(cap_max, b.cap);
  }
  L.pv = pv;
  H3D_CUDA(cudaMemcpyAsync(L.d_tasks.p, L.tasks.data(), sizeof(h3d::AcaTask) * nt, cudaMemcpyHostToDevice, s));
  H3D_CUDA(cudaMemsetAsync(L.d_counter.p, 0, sizeof(int32_t), s));
  h3d::PointsF64 P{h->xs.as<double>(), h->ys.as<double>(), h->zs.as<double>()};
  if (small_kernel) {
    // one warp per pair, no block barriers: 1.29 s for the 435,520 leaf
    // pairs at 64^3 against 1.35 s in 64-thread blocks (about half of the
    // FP64 floor of their operations either way)
    const int wpb = h3d::kAcaWarpsPerBlock;
    int per_sm = h3d::kAcaWarpBlocksPerSm;
    const size_t wshm = h3d::aca_warp_shared_bytes(cap_max);
    per_sm = std::max(1, std::min(per_sm, (int)((200 * 1024) / (wshm + 1024))));
    const int grid = std::max(1, std::min((nt + wpb - 1) / wpb, h->num_sms * per_sm));
    H3D_CUDA(cudaEventRecord(L.ev.a, s));
    H3D_CUDA(h3d::launch_aca_warp(s, grid, L.d_tasks.as<h3d::AcaTask>(), nt, L.d_counter.as<int>(), P,
                                  h->kd, h->tol, L.d_ws.as<double>(), L.d_fl.as<unsigned char>(),
                                  L.d_pv.as<int32_t>(), L.d_rank.as<int32_t>(), L.d_status.as<int32_t>(),
                                  cap_max));
    H3D_CUDA(cudaEventRecord(L.ev.b, s));
    ++h->launches;
    return HODLR3D_OK;
  }
  // the larger pairs: kAcaBlock-thread blocks, one per SM (k_aca's launch bounds)
  const size_t shm = h3d::aca_shared_bytes(cap_max);
  int per_sm = 1;
  if (shm > 0) {
    const int by_shm = (int)std::max<size_t>(1, (200 * 1024) / (shm + 2048));
    per_sm = std::max(1, std::min(per_sm, by_shm));
  }
  const int grid = std::max(1, std::min(nt, h->num_sms * per_sm));
  H3D_CUDA(cudaEventRecord(L.ev.a, s));
  H3D_CUDA(h3d::launch_aca(s, grid, L.d_tasks.as<h3d::AcaTask>(), nt, L.d_counter.as<int>(), P,
                           h->kd, h->tol, L.d_ws.as<double>(), L.d_fl.as<unsigned char>(),
                           L.d_pv.as<int32_t>(), L.d_rank.as<int32_t>(), L.d_status.as<int32_t>(),
                           cap_max));
  H3D_CUDA(cudaEventRecord(L.ev.b, s));
  ++h->launches;
  return HODLR3D_OK;
}

// Waits for the lane's batch: ranks and pivots to the host, finished tasks
// into an exact-size FP64 pool, capacity overflows into `retry` with twice
// the capacity.
int aca_finish(hodlr3d_t h, AcaLane& L, std::vector<HostTask>& retry) {
  cudaStream_t s = L.s;
  const std::vector<HostTask>& batch = L.batch;
  const int nt = (int)batch.size();
  std::vector<int32_t> rk(nt), st(nt), pvh(L.pv);
  H3D_CUDA(cudaMemcpyAsync(rk.data(), L.d_rank.p, sizeof(int32_t) * nt, cudaMemcpyDeviceToHost, s));
  H3D_CUDA(cudaMemcpyAsync(st.data(), L.d_status.p, sizeof(int32_t) * nt, cudaMemcpyDeviceToHost, s));
  if (L.pv) H3D_CUDA(cudaMemcpyAsync(pvh.data(), L.d_pv.p, sizeof(int32_t) * L.pv, cudaMemcpyDeviceToHost, s));
  H3D_CUDA(cudaStreamSynchronize(s));
  H3D_CUDA(cudaGetLastError());
  float aca_ms = 0.f;
  H3D_CUDA(cudaEventElapsedTime(&aca_ms, L.ev.a, L.ev.b));
  h->aca_kernel_seconds += 1e-3 * aca_ms;
  std::vector<int64_t> dst(nt, 0);
  int64_t total = 0;
  for (int i = 0; i < nt; ++i) {
    if (st[i] == h3d::kAcaNonFinite)
      return set_error(HODLR3D_ERR_NONFINITE,
                       "non-finite kernel entry in the ACA of pair %lld (coincident points?)",
                       (long long)batch[i].pair);
    if (st[i] == h3d::kAcaCapReached) {
      HostTask t = batch[i];
      t.cap = std::min(std::min(t.n, t.m), 2 * t.cap);
      retry.push_back(t);
      rk[i] = 0;
      continue;
    }
    dst[i] = total;
    total += (int64_t)rk[i] * (batch[i].n + batch[i].m);
  }
  DevBuf* pool64 = new DevBuf();
  h->pools.push_back(pool64);
  const int pool_id = (int)h->pools.size() - 1;
  H3D_CUDA(pool64->ensure(sizeof(double) * std::max<int64_t>(total, 1)));
  H3D_CUDA(cudaMemcpyAsync(L.d_off.p, dst.data(), sizeof(int64_t) * nt, cudaMemcpyHostToDevice, s));
  H3D_CUDA(cudaMemcpyAsync(L.d_rank.p, rk.data(), sizeof(int32_t) * nt, cudaMemcpyHostToDevice, s));
  H3D_CUDA(h3d::launch_aca_compact(s, nt, L.d_tasks.as<h3d::AcaTask>(), L.d_rank.as<int32_t>(),
                                   L.d_off.as<int64_t>(), L.d_ws.as<double>(), pool64->as<double>()));
  ++h->launches;
  for (int i = 0; i < nt; ++i) {
    if (st[i] == h3d::kAcaCapReached) continue;
    const int64_t p = batch[i].pair;
    const int r = rk[i];
    h->h_rank[p] = r;
    double* base64 = pool64->as<double>() + dst[i];
    h->h_fac_pool[p] = pool_id;
    h->h_fac_off[p] = dst[i];
    h->h_u64[p] = base64;
    h->h_v64[p] = base64 + (int64_t)r * batch[i].n;
    const int32_t* pr = pvh.data() + L.tasks[i].piv_off;
    h->h_piv_rows[p].assign(pr, pr + r);
    h->h_piv_cols[p].assign(pr + L.tasks[i].cap, pr + L.tasks[i].cap + r);
  }
  H3D_CUDA(cudaStreamSynchronize(s));
  ++h->aca_batches;
  return HODLR3D_OK;
}

// The batches of one pass, one after another on the handle's stream: those
// of the larger pairs (256-thread blocks, one per SM), then those of the leaf
// pairs (64-thread blocks).  Running the first leaf batch on a second stream
// beside the larger pairs' blocks (six per SM) did not shorten the assembly
// at 64^3 (4.51 s either way): the leaf batch at that occupancy became the
// longest, and both share the FP64 pipe.
int run_aca_batches(hodlr3d_t h, std::vector<std::vector<HostTask>>& big,
                    std::vector<std::vector<HostTask>>& small, std::vector<HostTask>& retry) {
  AcaLane L;
  L.s = h->stream;
  std::vector<std::vector<HostTask>> all;
  for (auto& b : big) all.push_back(std::move(b));
  const size_t nbig = all.size();
  for (auto& b : small) all.push_back(std::move(b));
  H3D_TRY(aca_lane_reserve(L, all));
  for (size_t k = 0; k < all.size(); ++k) {
    H3D_TRY(aca_launch(h, L, std::move(all[k]), k >= nbig));
    H3D_TRY(aca_finish(h, L, retry));
  }
  return HODLR3D_OK;
}

int finish_assembly(hodlr3d_t h, double t_start);

int assemble(hodlr3d_t h) {
  const double t_start = now_s();
  const int64_t np = h->npairs;
  h->h_rank.assign(np, 0);
  h->h_piv_rows.assign(np, {});
  h->h_piv_cols.assign(np, {});
  h->h_u64.assign(np, nullptr);
  h->h_v64.assign(np, nullptr);
  h->h_u32.assign(np, nullptr);
  h->h_v32.assign(np, nullptr);
  h->h_fac_pool.assign(np, -1);
  h->h_fac_off.assign(np, 0);
  for (DevBuf* b : h->pools) delete b;
  h->pools.clear();
  h->v32_pool = nullptr;
  h->u32_pool = nullptr;
  h->aca_batches = 0;
  h->aca_kernel_seconds = 0.0;
  // first rank capacity above leaf size, 128 (twice that for boxes of 2048
  // points and more): pairs that reach it run again with twice the capacity
  // (same ranks and pivots).  With the workspace below, at 64^3 (1/r, tol
  // 1e-10) 3 batches and 4.5 s; 256 for every pair above the leaves with an
  // 8 GiB workspace took 20 batches and 8.9-11.1 s (each batch waits for its
  // slowest pair); 96 costs more in repeated pairs than it saves.
  const int cap0 = h->opt.rank_cap > 0 ? h->opt.rank_cap : 128;
  std::vector<HostTask> todo;
  todo.reserve(np);
  for (int64_t p = 0; p < np; ++p) {
    const int j = h->h_pair_level[p];
    const int64_t kt = h->h_pair_tgt[p] - h3d::level_base(j);
    const int64_t ks = h->h_pair_src[p] - h3d::level_base(j);
    int64_t a0, a1, b0, b1;
    box_range(h, j, kt, a0, a1);
    box_range(h, j, ks, b0, b1);
    HostTask t;
    t.pair = p;
    t.t0 = (int32_t)a0;
    t.n = (int32_t)(a1 - a0);
    t.s0 = (int32_t)b0;
    t.m = (int32_t)(b1 - b0);
    t.leaf = j == h->levels;
    const int mn = std::min(t.n, t.m);
    // boxes of 2048 points and more start at twice the capacity: at 64^3 216
    // of the level-2 pairs (4096 points) pass rank 128, and run again as a
    // batch of their own that nothing overlaps (2.2 s of 6.0)
    t.cap = (t.leaf || mn <= cap0) ? mn : (mn >= 2048 ? std::min(mn, 2 * cap0) : cap0);
    todo.push_back(t);
  }
  size_t budget = h->opt.aca_workspace_bytes;
  if (!budget) {  // 64 GiB, or a quarter of the free device memory when less
    size_t free_b = 0, total_b = 0;
    H3D_CUDA(cudaMemGetInfo(&free_b, &total_b));
    budget = std::max<size_t>(size_t(1) << 30, std::min<size_t>(size_t(64) << 30, free_b / 4));
  }
  while (!todo.empty()) {
    // largest blocks first, in batches of at most `budget` bytes of workspace
    // each, those of the larger pairs and those of the leaf pairs apart
    std::stable_sort(todo.begin(), todo.end(), [](const HostTask& a, const HostTask& b) {
      return (int64_t)a.n * a.m > (int64_t)b.n * b.m;
    });
    std::vector<std::vector<HostTask>> big, small;
    size_t i = 0;
    while (i < todo.size()) {
      const bool is_small = std::max(todo[i].n, todo[i].m) <= 128;
      std::vector<HostTask> batch;
      size_t bytes = 0;
      while (i < todo.size()) {
        const HostTask& t = todo[i];
        if ((std::max(t.n, t.m) <= 128) != is_small) break;
        const size_t tb = sizeof(double) * (size_t)t.cap * (t.n + t.m) + (t.n + t.m) + 8 * t.cap + 64;
        if (!batch.empty() && bytes + tb > budget) break;
        batch.push_back(t);
        bytes += tb;
        ++i;
      }
      (is_small ? small : big).push_back(std::move(batch));
    }
    std::vector<HostTask> retry;
    H3D_TRY(run_aca_batches(h, big, small, retry));
    todo.swap(retry);
  }
  return finish_assembly(h, t_start);
}

// Everything after the factors exist (assembly or hodlr3d_load): the FP32
// copies, the matvec's per-pair tables and their device copies.
int finish_assembly(hodlr3d_t h, double t_start) {
  const double t_finish = now_s();
  const int64_t np = h->npairs;
  std::memset(h->tuned, 0, sizeof h->tuned);  // timings of another operator
  h->tc_split = 0;
  if (h->opt.keep_fp32) H3D_TRY(group_fp32(h));
  // per-pair tables for the matvec: T offsets, slice work items of the
  // non-leaf pairs, partial offsets of the pairs above level d - 1
  const int d = h->levels;
  std::vector<int64_t> tr(np), po(np, -1);
  std::vector<int32_t> items, upper;
  int64_t acc = 0, acc4 = 0, pacc = 0, fe = 0, ue = 0, ve = 0;
  h->max_rank = 0;
  for (int64_t p = 0; p < np; ++p) {
    tr[p] = acc;
    acc += h->h_rank[p];
    acc4 += (h->h_rank[p] + 3) & ~3;
    h->max_rank = std::max(h->max_rank, h->h_rank[p]);
    const int j = h->h_pair_level[p];
    const int64_t kt = h->h_pair_tgt[p] - h3d::level_base(j), ks = h->h_pair_src[p] - h3d::level_base(j);
    int64_t a0, a1, b0, b1;
    box_range(h, j, kt, a0, a1);
    box_range(h, j, ks, b0, b1);
    ue += (int64_t)h->h_rank[p] * (a1 - a0);
    ve += (int64_t)h->h_rank[p] * (b1 - b0);
    fe += (int64_t)h->h_rank[p] * ((a1 - a0) + (b1 - b0));
    if (j < d) {
      const int nsl = 1 << (3 * (d - 1 - j));
      for (int sl = 0; sl < nsl; ++sl) {
        items.push_back((int32_t)p);
        items.push_back(sl);
      }
    }
    if (j < d - 1) {
      po[p] = pacc;
      pacc += (int64_t)h->h_rank[p] << (3 * (d - 1 - j));
      upper.push_back((int32_t)p);
    }
  }
  h->max_slice = 0;
  if (d >= 1) {
    for (int64_t b = 0; b < (int64_t(1) << (3 * (d - 1))); ++b)
      h->max_slice = std::max(h->max_slice, h->h_leaf_off[(b + 1) << 3] - h->h_leaf_off[b << 3]);
  }
  // table sizes of the tensor-core T blocks: per level d - 1 box the pairs of
  // its ancestors (interaction lists are symmetric, so as many by source as
  // by target); the leaf kernel reads its block list from global memory
  h->tc_entries = 0;
  {
    auto cnt = [&](int j, int64_t b) {
      const int64_t gb = h3d::level_base(j) + b;
      return (int)(h->h_il_ptr[gb + 1] - h->h_il_ptr[gb]);
    };
    if (d >= 2)
      for (int64_t b = 0; b < (int64_t(1) << (3 * (d - 1))); ++b) {
        int n = 0;
        for (int j = 1; j <= d - 1; ++j) n += cnt(j, b >> (3 * (d - 1 - j)));
        h->tc_entries = std::max(h->tc_entries, n);
      }
  }
  h->sum_rank = acc;
  h->sum_rank4 = acc4;
  h->part_total = pacc;
  h->n_items = (int64_t)items.size() / 2;
  h->n_upper = (int64_t)upper.size();
  h->factor_entries = fe;
  h->u_entries = ue;
  h->v_entries = ve;
  cudaStream_t s = h->stream;
  const size_t npb = std::max<int64_t>(np, 1);
  H3D_CUDA(h->rank.ensure(sizeof(int32_t) * npb));
  H3D_CUDA(h->u64.ensure(sizeof(void*) * npb));
  H3D_CUDA(h->v64.ensure(sizeof(void*) * npb));
  H3D_CUDA(h->u32.ensure(sizeof(void*) * npb));
  H3D_CUDA(h->v32.ensure(sizeof(void*) * npb));
  H3D_CUDA(h->tr_off.ensure(sizeof(int64_t) * npb));
  H3D_CUDA(h->part_off.ensure(sizeof(int64_t) * npb));
  H3D_CUDA(h->items.ensure(sizeof(int32_t) * std::max<size_t>(items.size(), 2)));
  H3D_CUDA(h->upper.ensure(sizeof(int32_t) * std::max<size_t>(upper.size(), 1)));
  H3D_CUDA(h->pair_level.ensure(sizeof(int32_t) * npb));
  if (np) {
    H3D_CUDA(cudaMemcpyAsync(h->rank.p, h->h_rank.data(), sizeof(int32_t) * np, cudaMemcpyHostToDevice, s));
    H3D_CUDA(cudaMemcpyAsync(h->u64.p, h->h_u64.data(), sizeof(void*) * np, cudaMemcpyHostToDevice, s));
    H3D_CUDA(cudaMemcpyAsync(h->v64.p, h->h_v64.data(), sizeof(void*) * np, cudaMemcpyHostToDevice, s));
    H3D_CUDA(cudaMemcpyAsync(h->u32.p, h->h_u32.data(), sizeof(void*) * np, cudaMemcpyHostToDevice, s));
    H3D_CUDA(cudaMemcpyAsync(h->v32.p, h->h_v32.data(), sizeof(void*) * np, cudaMemcpyHostToDevice, s));
    H3D_CUDA(cudaMemcpyAsync(h->tr_off.p, tr.data(), sizeof(int64_t) * np, cudaMemcpyHostToDevice, s));
    H3D_CUDA(cudaMemcpyAsync(h->part_off.p, po.data(), sizeof(int64_t) * np, cudaMemcpyHostToDevice, s));
    H3D_CUDA(cudaMemcpyAsync(h->pair_level.p, h->h_pair_level.data(), sizeof(int32_t) * np,
                             cudaMemcpyHostToDevice, s));
  }
  if (!items.empty())
    H3D_CUDA(cudaMemcpyAsync(h->items.p, items.data(), sizeof(int32_t) * items.size(),
                             cudaMemcpyHostToDevice, s));
  if (!upper.empty())
    H3D_CUDA(cudaMemcpyAsync(h->upper.p, upper.data(), sizeof(int32_t) * upper.size(),
                             cudaMemcpyHostToDevice, s));
  H3D_CUDA(cudaStreamSynchronize(s));
  h->mv_nrhs_cap = 0;
  // the tensor-core engine's near-field blocks and tensor maps (which point
  // at the factors) are rebuilt on its next use
  h->near_built = false;
  h->maps_built = false;
  h->gemv_built = false;
  h->f64_built = false;
  h->f64_unavailable = false;
  h->assembled = true;
  h->finish_seconds = now_s() - t_finish;
  h->assemble_seconds = now_s() - t_start;
  return HODLR3D_OK;
}

}  // namespace hodlr3d_host
