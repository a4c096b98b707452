// Host side of the hodlr3d_gb300 C ABI: handle life cycle, device memory,
// tree build, batched ACA orchestration, matvec and GMRES drivers.
//
// Reference interfaces replaced: HODLR3D (include/HODLR3D.hpp:12-21,
// src/HODLR3D.cpp), HODLR3DTree (include/HODLR3DTree.hpp, src/HODLR3DTree.cpp),
// LowRank (src/ACA.cpp), classGMRES (include/gmres.hpp, src/gmres.cpp).
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <mutex>
#include <thread>
#include <chrono>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <memory>
#include <new>
#include <numeric>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/hodlr3d.h"
#include "aca.h"
#include "common.cuh"
#include "gmres.h"
#include "matvec.h"
#include "noalloc.h"
#include "tree.h"

namespace {

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

#define H3D_CUDA(call)                                                                   \
  do {                                                                                   \
    cudaError_t e_ = (call);                                                             \
    if (e_ != cudaSuccess) {                                                             \
      if (e_ == cudaErrorMemoryAllocation)                                               \
        return set_error(HODLR3D_ERR_OUT_OF_MEMORY, "%s: %s (%s:%d)", #call,             \
                         cudaGetErrorString(e_), __FILE__, __LINE__);                    \
      return set_error(HODLR3D_ERR_CUDA, "%s: %s (%s:%d)", #call, cudaGetErrorString(e_), \
                       __FILE__, __LINE__);                                              \
    }                                                                                    \
  } while (0)

#define H3D_TRY(call)           \
  do {                          \
    int s_ = (call);            \
    if (s_ != HODLR3D_OK) return s_; \
  } while (0)

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

struct DevBuf {
  void* p = nullptr;
  size_t bytes = 0;
  ~DevBuf() { release(); }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    bytes = 0;
  }
  cudaError_t ensure(size_t b) {
    if (b <= bytes && p) return cudaSuccess;
    release();
    cudaError_t e = cudaMalloc(&p, b ? b : 16);
    if (e == cudaSuccess) bytes = b;
    return e;
  }
  template <class T>
  T* as() const {
    return static_cast<T*>(p);
  }
};

// two CUDA events for a timed span, destroyed with the scope
struct EventPair {
  cudaEvent_t a = nullptr, b = nullptr;
  ~EventPair() {
    if (a) cudaEventDestroy(a);
    if (b) cudaEventDestroy(b);
  }
};

}  // namespace

struct hodlr3d_handle {
  // problem
  int64_t N = 0;
  int nP1D = 0;
  double L = 1.0;
  int tol_pow = 0;
  double tol = 0.0;
  int levels = 0;
  int64_t nleaf = 0;
  int64_t nbox_all = 0;
  hodlr3d_options opt{};
  h3d::KernelDesc kd{};
  int device = 0;
  int num_sms = 0;
  cudaStream_t stream = nullptr;
  int64_t launches = 0;
  // tree (device)
  DevBuf xyz, perm, leaf_off, xs, ys, zs, xl, yl, zl, centre, nbr_all, nbr_leaf, il_ptr, pair_tgt,
      pair_src, rev;
  std::vector<int32_t> h_perm, h_leaf_off, h_pair_tgt, h_pair_src, h_pair_level;
  std::vector<int64_t> h_il_ptr;
  int max_leaf = 0;
  int64_t npairs = 0;
  double tree_seconds = 0.0;
  // factors
  bool assembled = false;
  std::vector<int32_t> h_rank;
  std::vector<std::vector<int32_t>> h_piv_rows, h_piv_cols;  // local pivots per pair
  std::vector<DevBuf*> pools;
  std::vector<int64_t> h_fac_off;       // per pair: element offset of its FP64 U in its pool (V follows)
  std::vector<int32_t> h_fac_pool;      // per pair: index of its FP64 pool in `pools` (-1: rank 0 or none)
  std::vector<double*> h_u64, h_v64;
  std::vector<float*> h_u32, h_v32;
  // FP32 V of the pairs of each source box, contiguous in the order of its
  // reverse list: per box (all levels numbered together) the float offset in
  // v32_pool of its first pair and its rows (the sum of the ranks)
  DevBuf* v32_pool = nullptr;
  std::vector<int64_t> h_vbox_off;
  std::vector<int32_t> h_vbox_rows;
  // FP32 U of the pairs of each target box side by side: one row-major
  // n_b x R_b matrix per box (R_b = sum of the padded ranks of its pairs) at
  // u32_pool + h_ubox_off[b]; pair p at column h_coff[p], row stride
  // h_ustride[p] = R_b.  The tensor-core T uses the same grouping: T of box b
  // is 32 x R_b at 32-wide offset h_tbox_off[b].
  DevBuf* u32_pool = nullptr;
  // FP64-accurate form: lo parts of the FP32 copies (FP64 value minus the
  // FP32 value, rounded), same layouts; built on first use
  DevBuf u32lo_pool, v32lo_pool, knearlo;
  bool lo_built = false;
  bool lo_unavailable = false;  // the lo parts did not fit: fp64x is the FP64 form
  std::vector<int32_t> h_pair_m, h_pair_n;  // per pair: source and target box sizes
  std::vector<int64_t> h_ubox_off, h_tbox_off;
  std::vector<int32_t> h_rbox, h_ustride, h_coff;
  DevBuf ustride, tc_toff, tc_tld, tc_tbox, tc_rbox;
  DevBuf rank, u64, v64, u32, v32, tr_off, part_off, items, upper, pair_level;
  int64_t sum_rank = 0, sum_rank4 = 0, part_total = 0, n_items = 0, n_upper = 0, factor_entries = 0;
  int tc_entries = 0;  // largest table of a tensor-core block
  int64_t u_entries = 0, v_entries = 0;
  int max_slice = 0;
  int max_rank = 0;
  double assemble_seconds = 0.0;
  int aca_batches = 0;
  double aca_kernel_seconds = 0.0;  // device time of the ACA kernels of the last assembly
  double finish_seconds = 0.0;      // finish_assembly of the last assembly or load
  // matvec work buffers
  DevBuf xsorted, tbuf, pbuf, ynl, stage_x, stage_y, stage_t;
  int mv_nrhs_cap = 0;
  // optional per-kernel timing of matvec launches
  struct Prof : h3d::MatvecProfiler {
    std::vector<cudaEvent_t> pool;
    size_t used = 0;
    std::vector<std::pair<const char*, std::pair<cudaEvent_t, cudaEvent_t>>> spans;
    cudaEvent_t last = nullptr;
    cudaEvent_t next_event() {
      if (used == pool.size()) {
        cudaEvent_t e;
        cudaEventCreate(&e);
        pool.push_back(e);
      }
      return pool[used++];
    }
    void begin(cudaStream_t s) override {
      last = next_event();
      cudaEventRecord(last, s);
    }
    void mark(cudaStream_t s, const char* name) override {
      cudaEvent_t e = next_event();
      cudaEventRecord(e, s);
      spans.push_back({name, {last, e}});
      last = e;
    }
    ~Prof() {
      for (cudaEvent_t e : pool) cudaEventDestroy(e);
    }
  };
  bool profiling = false;
  Prof prof;
  int engine = 0;   // 0 auto, 1 SIMT kernels, 2 tensor-core kernels, 3 few-column kernels
  // automatic choice for the mixed product, per (transpose, nrhs), from the
  // timings of hodlr3d_autotune: 0 = the column-count rules, else an engine
  int8_t tuned[2][65] = {};
  DevBuf dev_err;   // set by kernels whose bounded waits gave up
  bool leaves_aligned = false;  // every leaf population a multiple of 4
  DevBuf knear, near_off;       // FP32 near-field blocks of the tensor-core engine
  DevBuf tct;                   // X and T of the tensor-core engine (split-exact FP32)
  DevBuf tmaps;                 // tensor maps of the tensor-core engine: U, V, near blocks
  bool maps_built = false;
  bool near_built = false;
  std::vector<int32_t> h_nbr_leaf;  // host copy (tensor maps of the near-field blocks)
  std::vector<int64_t> h_near_off;  // 27 per leaf: near-block offsets, -1 for no neighbour
  std::vector<int64_t> h_near_base;  // per leaf: its near-field matrix (blocks side by side)
  std::vector<int32_t> h_near_ld;    // per leaf: row length of that matrix
  DevBuf near_base, near_ld;
  int64_t near_floats = 0;
  // few-column engine (matvec_gemv.cu): tables over the grouped FP32 layouts
  bool gemv_built = false;
  bool gemv_ok = false;          // tree and layouts fit the few-column kernels
  bool gemv8_ok = false;         // ... in passes of 8 columns (mixed form)
  DevBuf gv_ubox_off, gv_vbox_off, gv_vbox_rows, gv_vrow0, gv_vrow_t, gv_trow_v, gv_tbase, gv_vpofs,
      gv_upofs, gv_vt_items, gv_vt_upper, gv_ut_items, gv_ut_upper, gv_x, gv_t, gv_tt, gv_p, gv_pt,
      gv_xl, gv_tl, gv_ttl, gv_pd, gv_ptd;
  int64_t gv_n_vt_items = 0, gv_n_vt_upper = 0, gv_n_ut_items = 0, gv_n_ut_upper = 0;
  // GMRES work buffers
  DevBuf g_Q, g_w, g_r, g_x, g_b, g_H, g_cs, g_sn, g_beta, g_hk, g_bnorm, g_err, g_part, g_y,
      g_kcol, g_brk, g_scal, g_d, g_coef;

  ~hodlr3d_handle() {
    for (DevBuf* b : pools) delete b;
    if (stream) cudaStreamDestroy(stream);
  }
};

namespace {

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

// range [start, end) in tree order of box k at level j
inline void box_range(const hodlr3d_t h, int j, int64_t k, int64_t& a, int64_t& b) {
  const int sh = 3 * (h->levels - j);
  a = h->h_leaf_off[k << sh];
  b = h->h_leaf_off[(k + 1) << sh];
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

int run_aca_batch(hodlr3d_t h, std::vector<HostTask>& batch, std::vector<HostTask>& retry,
                  bool small_kernel) {
  cudaStream_t s = h->stream;
  const int nt = (int)batch.size();
  std::vector<h3d::AcaTask> tasks(nt);
  int64_t ws = 0, fl = 0, pv = 0;
  int cap_max = 1;
  for (int i = 0; i < nt; ++i) {
    const HostTask& b = batch[i];
    h3d::AcaTask& t = tasks[i];
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
  DevBuf d_tasks, d_ws, d_fl, d_pv, d_rank, d_status, d_counter, d_off;
  H3D_CUDA(d_tasks.ensure(sizeof(h3d::AcaTask) * nt));
  H3D_CUDA(d_ws.ensure(sizeof(double) * std::max<int64_t>(ws, 1)));
  H3D_CUDA(d_fl.ensure(std::max<int64_t>(fl, 1)));
  H3D_CUDA(d_pv.ensure(sizeof(int32_t) * std::max<int64_t>(pv, 1)));
  H3D_CUDA(d_rank.ensure(sizeof(int32_t) * nt));
  H3D_CUDA(d_status.ensure(sizeof(int32_t) * nt));
  H3D_CUDA(d_counter.ensure(sizeof(int32_t)));
  H3D_CUDA(cudaMemcpyAsync(d_tasks.p, tasks.data(), sizeof(h3d::AcaTask) * nt, cudaMemcpyHostToDevice, s));
  H3D_CUDA(cudaMemsetAsync(d_counter.p, 0, sizeof(int32_t), s));
  const int block = small_kernel ? 64 : 256;
  const size_t shm = h3d::aca_shared_bytes(cap_max);
  int per_sm = small_kernel ? 16 : 4;
  if (shm > 0) {
    const int by_shm = (int)std::max<size_t>(1, (200 * 1024) / (shm + 2048));
    per_sm = std::max(1, std::min(per_sm, by_shm));
  }
  const int grid = std::max(1, std::min(nt, h->num_sms * per_sm));
  h3d::PointsF64 P{h->xs.as<double>(), h->ys.as<double>(), h->zs.as<double>()};
  EventPair ev;
  H3D_CUDA(cudaEventCreate(&ev.a));
  H3D_CUDA(cudaEventCreate(&ev.b));
  H3D_CUDA(cudaEventRecord(ev.a, s));
  H3D_CUDA(h3d::launch_aca(s, block, grid, d_tasks.as<h3d::AcaTask>(), nt, d_counter.as<int>(), P,
                           h->kd, h->tol, d_ws.as<double>(), d_fl.as<unsigned char>(),
                           d_pv.as<int32_t>(), d_rank.as<int32_t>(), d_status.as<int32_t>(),
                           cap_max));
  H3D_CUDA(cudaEventRecord(ev.b, s));
  ++h->launches;
  std::vector<int32_t> rk(nt), st(nt), pvh(pv);
  H3D_CUDA(cudaMemcpyAsync(rk.data(), d_rank.p, sizeof(int32_t) * nt, cudaMemcpyDeviceToHost, s));
  H3D_CUDA(cudaMemcpyAsync(st.data(), d_status.p, sizeof(int32_t) * nt, cudaMemcpyDeviceToHost, s));
  if (pv) H3D_CUDA(cudaMemcpyAsync(pvh.data(), d_pv.p, sizeof(int32_t) * pv, cudaMemcpyDeviceToHost, s));
  H3D_CUDA(cudaStreamSynchronize(s));
  H3D_CUDA(cudaGetLastError());
  float aca_ms = 0.f;
  H3D_CUDA(cudaEventElapsedTime(&aca_ms, ev.a, ev.b));
  h->aca_kernel_seconds += 1e-3 * aca_ms;
  // finished tasks -> exact-size pools; capacity overflows -> retried with twice the capacity
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
  H3D_CUDA(d_off.ensure(sizeof(int64_t) * nt));
  H3D_CUDA(cudaMemcpyAsync(d_off.p, dst.data(), sizeof(int64_t) * nt, cudaMemcpyHostToDevice, s));
  H3D_CUDA(cudaMemcpyAsync(d_rank.p, rk.data(), sizeof(int32_t) * nt, cudaMemcpyHostToDevice, s));
  H3D_CUDA(h3d::launch_aca_compact(s, nt, d_tasks.as<h3d::AcaTask>(), d_rank.as<int32_t>(),
                                   d_off.as<int64_t>(), d_ws.as<double>(), pool64->as<double>()));
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
    const int32_t* pr = pvh.data() + tasks[i].piv_off;
    h->h_piv_rows[p].assign(pr, pr + r);
    h->h_piv_cols[p].assign(pr + tasks[i].cap, pr + tasks[i].cap + r);
  }
  H3D_CUDA(cudaStreamSynchronize(s));
  ++h->aca_batches;
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
  // first rank capacity above leaf size: pairs that reach it run again with
  // twice the capacity (same ranks and pivots).  128 and the workspace below:
  // at 64^3 (1/r, tol 1e-10) 4 batches and 6.7-7.7 s against 20 and
  // 8.9-11.1 s with 256 and 8 GiB in the same process (each batch waits for
  // its slowest pair); 96 costs more in repeated pairs than it saves.
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
    t.cap = (t.leaf || mn <= cap0) ? mn : cap0;
    todo.push_back(t);
  }
  size_t budget = h->opt.aca_workspace_bytes;
  if (!budget) {  // 32 GiB, or a quarter of the free device memory when less
    size_t free_b = 0, total_b = 0;
    H3D_CUDA(cudaMemGetInfo(&free_b, &total_b));
    budget = std::max<size_t>(size_t(1) << 30, std::min<size_t>(size_t(32) << 30, free_b / 4));
  }
  while (!todo.empty()) {
    // largest blocks first
    std::stable_sort(todo.begin(), todo.end(), [](const HostTask& a, const HostTask& b) {
      return (int64_t)a.n * a.m > (int64_t)b.n * b.m;
    });
    std::vector<HostTask> retry;
    size_t i = 0;
    while (i < todo.size()) {
      const bool small = std::max(todo[i].n, todo[i].m) <= 128;
      std::vector<HostTask> batch;
      size_t bytes = 0;
      while (i < todo.size()) {
        const HostTask& t = todo[i];
        if ((std::max(t.n, t.m) <= 128) != small) break;
        const size_t tb = sizeof(double) * (size_t)t.cap * (t.n + t.m) + (t.n + t.m) + 8 * t.cap + 64;
        if (!batch.empty() && bytes + tb > budget) break;
        batch.push_back(t);
        bytes += tb;
        ++i;
      }
      H3D_TRY(run_aca_batch(h, batch, retry, small));
    }
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
  // table sizes of the tensor-core blocks: per level d - 1 box the pairs of
  // its ancestors (interaction lists are symmetric, so as many by source as
  // by target), per leaf its pairs plus 27 near-field blocks
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
    for (int64_t k = 0; k < h->nleaf; ++k) h->tc_entries = std::max(h->tc_entries, cnt(d, k) + 27);
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
  h->assembled = true;
  h->finish_seconds = now_s() - t_finish;
  h->assemble_seconds = now_s() - t_start;
  return HODLR3D_OK;
}

// ---------------------------------------------------------------------------
// factor files (hodlr3d_save / hodlr3d_load)
// ---------------------------------------------------------------------------
// Version 1, host byte order (little-endian on both supported hosts):
//   "H3DFACT1", FileHeader, points (n x 3 FP64, original order),
//   per pair {rank, pool, offset of U in the pool} (PairRec), the pivots of
//   every pair (rank row then rank column local indices), per pool its FP64
//   element count, the pool contents (per pair U n x r then V m x r,
//   column-major, as the assembly wrote them), a 64-bit checksum of all of it.
// The tree and interaction lists are rebuilt from the points on load and
// must hash to lists_hash: the factors belong to exactly those pairs.
constexpr char kFactMagic[8] = {'H', '3', 'D', 'F', 'A', 'C', 'T', '1'};

struct FileHeader {
  uint32_t version, header_bytes;
  int64_t n;
  int32_t nP1D, tol_pow;
  double L;
  int32_t kernel, levels;
  double diag;
  int64_t npairs;
  int32_t npools, reserved;
  uint64_t lists_hash;
};

struct PairRec {
  int32_t rank, pool;
  int64_t off;
};

// word-wise mixing hash (multiply-xorshift); trailing bytes folded in one word
struct Hasher {
  uint64_t x = 0x243F6A8885A308D3ull;
  void add(const void* p, size_t bytes) {
    const unsigned char* b = static_cast<const unsigned char*>(p);
    size_t i = 0;
    for (; i + 8 <= bytes; i += 8) {
      uint64_t w;
      std::memcpy(&w, b + i, 8);
      x = (x ^ w) * 0x9E3779B97F4A7C15ull;
      x ^= x >> 29;
    }
    if (i < bytes) {
      uint64_t w = 0;
      std::memcpy(&w, b + i, bytes - i);
      x = (x ^ w ^ (uint64_t)(bytes - i) << 56) * 0x9E3779B97F4A7C15ull;
      x ^= x >> 29;
    }
  }
};

uint64_t lists_hash(const hodlr3d_t h) {
  Hasher hs;
  hs.add(h->h_pair_level.data(), sizeof(int32_t) * h->h_pair_level.size());
  hs.add(h->h_pair_tgt.data(), sizeof(int32_t) * h->h_pair_tgt.size());
  hs.add(h->h_pair_src.data(), sizeof(int32_t) * h->h_pair_src.size());
  hs.add(h->h_leaf_off.data(), sizeof(int32_t) * h->h_leaf_off.size());
  return hs.x;
}

struct File {
  std::FILE* f = nullptr;
  Hasher hs;
  ~File() {
    if (f) std::fclose(f);
  }
  bool write(const void* p, size_t bytes) {
    hs.add(p, bytes);
    return std::fwrite(p, 1, bytes, f) == bytes;
  }
  bool read(void* p, size_t bytes) {
    if (std::fread(p, 1, bytes, f) != bytes) return false;
    hs.add(p, bytes);
    return true;
  }
};

constexpr size_t kFileChunk = size_t(64) << 20;

int save_factors(hodlr3d_t h, const char* path) {
  if (!h->assembled) return set_error(HODLR3D_ERR_NOT_ASSEMBLED, "hodlr3d_assemble has not run");
  const int64_t np = h->npairs;
  // the FP64 pools the pairs use, renumbered in order
  std::vector<int> remap(h->pools.size(), -1), used;
  for (int64_t p = 0; p < np; ++p) {
    const int q = h->h_fac_pool[p];
    if (q >= 0 && remap[q] < 0) {
      remap[q] = 0;
    }
  }
  for (size_t q = 0; q < h->pools.size(); ++q)
    if (remap[q] == 0) {
      remap[q] = (int)used.size();
      used.push_back((int)q);
    }
  File F;
  F.f = std::fopen(path, "wb");
  if (!F.f) return set_error(HODLR3D_ERR_IO, "cannot open %s for writing", path);
  if (std::fwrite(kFactMagic, 1, 8, F.f) != 8) return set_error(HODLR3D_ERR_IO, "write failed: %s", path);
  FileHeader hd{};
  hd.version = 1;
  hd.header_bytes = sizeof(FileHeader);
  hd.n = h->N;
  hd.nP1D = h->nP1D;
  hd.tol_pow = h->tol_pow;
  hd.L = h->L;
  hd.kernel = h->kd.kind;
  hd.levels = h->levels;
  hd.diag = h->kd.diag;
  hd.npairs = np;
  hd.npools = (int32_t)used.size();
  hd.lists_hash = lists_hash(h);
  std::vector<double> xyz(3 * h->N);
  H3D_CUDA(cudaMemcpy(xyz.data(), h->xyz.p, sizeof(double) * xyz.size(), cudaMemcpyDeviceToHost));
  std::vector<PairRec> pr(np);
  for (int64_t p = 0; p < np; ++p)
    pr[p] = {h->h_rank[p], h->h_fac_pool[p] >= 0 ? remap[h->h_fac_pool[p]] : -1, h->h_fac_off[p]};
  bool ok = F.write(&hd, sizeof hd) && F.write(xyz.data(), sizeof(double) * xyz.size()) &&
            F.write(pr.data(), sizeof(PairRec) * pr.size());
  for (int64_t p = 0; ok && p < np; ++p)
    ok = F.write(h->h_piv_rows[p].data(), sizeof(int32_t) * h->h_piv_rows[p].size()) &&
         F.write(h->h_piv_cols[p].data(), sizeof(int32_t) * h->h_piv_cols[p].size());
  std::vector<int64_t> counts;
  for (int q : used) counts.push_back((int64_t)(h->pools[q]->bytes / sizeof(double)));
  ok = ok && F.write(counts.data(), sizeof(int64_t) * counts.size());
  std::vector<unsigned char> buf;
  for (size_t u = 0; ok && u < used.size(); ++u) {
    const DevBuf* b = h->pools[used[u]];
    for (size_t o = 0; ok && o < b->bytes; o += kFileChunk) {
      const size_t len = std::min(kFileChunk, b->bytes - o);
      buf.resize(len);
      H3D_CUDA(cudaMemcpy(buf.data(), static_cast<const unsigned char*>(b->p) + o, len,
                          cudaMemcpyDeviceToHost));
      ok = F.write(buf.data(), len);
    }
  }
  const uint64_t sum = F.hs.x;
  ok = ok && std::fwrite(&sum, 1, 8, F.f) == 8;
  if (!ok || std::fflush(F.f) != 0) return set_error(HODLR3D_ERR_IO, "write failed: %s", path);
  return HODLR3D_OK;
}

int load_factors(const char* path, const hodlr3d_options* opt, hodlr3d_t* out) {
  const double t_start = now_s();
  File F;
  F.f = std::fopen(path, "rb");
  if (!F.f) return set_error(HODLR3D_ERR_IO, "cannot open %s", path);
  char magic[8];
  if (std::fread(magic, 1, 8, F.f) != 8 || std::memcmp(magic, kFactMagic, 8) != 0)
    return set_error(HODLR3D_ERR_IO, "%s is not a hodlr3d factor file (version 1)", path);
  FileHeader hd{};
  // sizes are checked before anything is allocated from them: the point count
  // within what hodlr3d_create takes, at most one pool per pair
  if (!F.read(&hd, sizeof hd) || hd.version != 1 || hd.header_bytes != sizeof(FileHeader) || hd.n < 2 ||
      hd.n > INT32_MAX / 2 || hd.npairs < 0 || hd.npools < 0 || hd.npools > std::max<int64_t>(hd.npairs, 1))
    return set_error(HODLR3D_ERR_IO, "%s: unreadable header", path);
  std::vector<double> xyz(3 * (size_t)hd.n);
  if (!F.read(xyz.data(), sizeof(double) * xyz.size())) return set_error(HODLR3D_ERR_IO, "%s: truncated", path);
  hodlr3d_options o;
  if (opt) o = *opt;
  else hodlr3d_default_options(&o);
  o.diag_override = hd.diag;
  hodlr3d_t h = nullptr;
  H3D_TRY(hodlr3d_create(xyz.data(), hd.n, hd.nP1D, hd.L, hd.tol_pow, hd.kernel, &o, &h));
  std::unique_ptr<hodlr3d_handle, void (*)(hodlr3d_t)> guard(h, hodlr3d_destroy);
  if (h->levels != hd.levels || h->npairs != hd.npairs || lists_hash(h) != hd.lists_hash)
    return set_error(HODLR3D_ERR_IO, "%s: the tree rebuilt from its points differs from the saved one", path);
  const int64_t np = hd.npairs;
  std::vector<PairRec> pr(np);
  if (!F.read(pr.data(), sizeof(PairRec) * pr.size())) return set_error(HODLR3D_ERR_IO, "%s: truncated", path);
  h->h_rank.assign(np, 0);
  h->h_piv_rows.assign(np, {});
  h->h_piv_cols.assign(np, {});
  h->h_u64.assign(np, nullptr);
  h->h_v64.assign(np, nullptr);
  h->h_u32.assign(np, nullptr);
  h->h_v32.assign(np, nullptr);
  h->h_fac_pool.assign(np, -1);
  h->h_fac_off.assign(np, 0);
  for (int64_t p = 0; p < np; ++p) {
    const int r = pr[p].rank;
    if (r < 0 || r > h->N || pr[p].pool < -1 || pr[p].pool >= hd.npools || (pr[p].pool < 0 && r > 0))
      return set_error(HODLR3D_ERR_IO, "%s: corrupt pair record %lld", path, (long long)p);
    h->h_rank[p] = r;
    h->h_piv_rows[p].resize(r);
    h->h_piv_cols[p].resize(r);
    if (!F.read(h->h_piv_rows[p].data(), sizeof(int32_t) * r) ||
        !F.read(h->h_piv_cols[p].data(), sizeof(int32_t) * r))
      return set_error(HODLR3D_ERR_IO, "%s: truncated", path);
  }
  std::vector<int64_t> counts(hd.npools);
  if (!F.read(counts.data(), sizeof(int64_t) * counts.size())) return set_error(HODLR3D_ERR_IO, "%s: truncated", path);
  std::vector<unsigned char> buf;
  for (int q = 0; q < hd.npools; ++q) {
    if (counts[q] < 0) return set_error(HODLR3D_ERR_IO, "%s: corrupt pool size", path);
    DevBuf* b = new DevBuf();
    h->pools.push_back(b);
    const size_t bytes = sizeof(double) * (size_t)counts[q];
    H3D_CUDA(b->ensure(bytes));
    for (size_t o = 0; o < bytes; o += kFileChunk) {
      const size_t len = std::min(kFileChunk, bytes - o);
      buf.resize(len);
      if (!F.read(buf.data(), len)) return set_error(HODLR3D_ERR_IO, "%s: truncated", path);
      H3D_CUDA(cudaMemcpy(static_cast<unsigned char*>(b->p) + o, buf.data(), len, cudaMemcpyHostToDevice));
    }
  }
  const uint64_t want = F.hs.x;
  uint64_t sum = 0;
  if (std::fread(&sum, 1, 8, F.f) != 8 || sum != want)
    return set_error(HODLR3D_ERR_IO, "%s: checksum mismatch", path);
  for (int64_t p = 0; p < np; ++p) {
    if (pr[p].pool < 0) continue;
    const int j = h->h_pair_level[p];
    int64_t a0, a1, b0, b1;
    box_range(h, j, h->h_pair_tgt[p] - h3d::level_base(j), a0, a1);
    box_range(h, j, h->h_pair_src[p] - h3d::level_base(j), b0, b1);
    const int64_t r = pr[p].rank;
    if (pr[p].off < 0 || pr[p].off + r * ((a1 - a0) + (b1 - b0)) > counts[pr[p].pool])
      return set_error(HODLR3D_ERR_IO, "%s: pair %lld lies outside its pool", path, (long long)p);
    for (int l = 0; l < r; ++l)
      if (h->h_piv_rows[p][l] < 0 || h->h_piv_rows[p][l] >= a1 - a0 || h->h_piv_cols[p][l] < 0 ||
          h->h_piv_cols[p][l] >= b1 - b0)
        return set_error(HODLR3D_ERR_IO, "%s: pivot of pair %lld outside its boxes", path, (long long)p);
    double* base = h->pools[pr[p].pool]->as<double>() + pr[p].off;
    h->h_fac_pool[p] = pr[p].pool;
    h->h_fac_off[p] = pr[p].off;
    h->h_u64[p] = base;
    h->h_v64[p] = base + r * (a1 - a0);
  }
  h->aca_batches = 0;
  h->aca_kernel_seconds = 0.0;
  H3D_TRY(finish_assembly(h, t_start));
  *out = guard.release();
  return HODLR3D_OK;
}

// ---------------------------------------------------------------------------
// matvec
// ---------------------------------------------------------------------------
int ensure_matvec_buffers(hodlr3d_t h, int nrhs) {
  const int nr = h3d::padded_nrhs(nrhs);
  if (nr <= h->mv_nrhs_cap) return HODLR3D_OK;
  H3D_CUDA(h->xsorted.ensure(sizeof(double) * h->N * nr));
  H3D_CUDA(h->tbuf.ensure(sizeof(double) * std::max<int64_t>(h->sum_rank, 1) * nr));
  H3D_CUDA(h->pbuf.ensure(sizeof(double) * std::max<int64_t>(h->part_total, 1) * nr));
  H3D_CUDA(h->ynl.ensure(sizeof(double) * h->N * nr));
  h->mv_nrhs_cap = nr;
  return HODLR3D_OK;
}

// Tensor maps (2D tiled, FP32, 128-byte swizzle, zero fill outside) of the
// tensor-core engine's A operands, box 32 x 128: per target box the U of its
// pairs side by side (n x R_b), per source box the V of its pairs (sum of
// ranks x round4(m)), per leaf and neighbour slot the near-field block
// (nk x round4(ne)).  Maps of empty operands stay zero and are never used.
int build_tensor_maps(hodlr3d_t h, const std::vector<int64_t>& near_off) {
  static PFN_cuTensorMapEncodeTiled_v12000 encode = nullptr;
  if (!encode) {
    cudaDriverEntryPointQueryResult q;
    H3D_CUDA(cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", (void**)&encode, 12000,
                                              cudaEnableDefault, &q));
    if (!encode || q != cudaDriverEntryPointSuccess)
      return set_error(HODLR3D_ERR_CUDA, "cuTensorMapEncodeTiled is not available");
  }
  const int64_t nbox = (int64_t)h->h_vbox_rows.size();
  const int64_t nm = 2 * nbox + 27 * h->nleaf;
  std::vector<CUtensorMap> maps((size_t)std::max<int64_t>(nm, 1));
  std::memset(maps.data(), 0, sizeof(CUtensorMap) * maps.size());
  std::atomic<int> bad{0};
  std::mutex bad_mu;
  char bad_msg[160] = {0};
  auto enc = [&](CUtensorMap* m, const float* base, int64_t inner, int64_t rows, uint32_t box_rows,
                 int64_t ld) {
    if (!base || inner <= 0 || rows <= 0) return;
    const cuuint64_t dim[2] = {(cuuint64_t)inner, (cuuint64_t)rows};
    const cuuint64_t stride[1] = {(cuuint64_t)ld * sizeof(float)};
    const cuuint32_t box[2] = {32, box_rows}, es[2] = {1, 1};
    const CUresult r = encode(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, (void*)base, dim, stride, box, es,
                              CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                              CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS && !bad.exchange(1)) {
      std::lock_guard<std::mutex> g(bad_mu);
      std::snprintf(bad_msg, sizeof(bad_msg), "code %d, %lld x %lld at %p, box 32 x %u, map at %p",
                    (int)r, (long long)rows, (long long)inner, (const void*)base, box_rows, (void*)m);
    }
  };
  const float* knear = h->knear.as<float>();
  const int nthr = (int)std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
  std::vector<std::thread> th;
  for (int t = 0; t < nthr; ++t)
    th.emplace_back([&, t] {
      cudaSetDevice(h->opt.device);  // the encoder wants the device's context current
      for (int64_t b = t; b < nbox; b += nthr) {
        int j = 0;
        while (j < h->levels && h3d::level_base(j + 1) <= b) ++j;
        int64_t b0, b1;
        box_range(h, j, b - h3d::level_base(j), b0, b1);
        if (h->h_rbox[b] > 0)
          enc(&maps[b], h->u32_pool->as<float>() + h->h_ubox_off[b], h->h_rbox[b], b1 - b0, 128,
              h->h_rbox[b]);
        if (h->h_vbox_rows[b] > 0)
          enc(&maps[nbox + b], h->v32_pool->as<float>() + h->h_vbox_off[b],
              ((b1 - b0) + 3) & ~int64_t(3), h->h_vbox_rows[b], 128, ((b1 - b0) + 3) & ~int64_t(3));
      }
      for (int64_t k = t; k < h->nleaf; k += nthr) {
        const int64_t nk = h->h_leaf_off[k + 1] - h->h_leaf_off[k];
        for (int sl = 0; sl < 27; ++sl) {
          const int64_t off = near_off[27 * k + sl];
          if (off < 0) continue;
          const int64_t nn = sl < 26 ? h->h_nbr_leaf[26 * k + sl] : k;
          const int64_t ne = h->h_leaf_off[nn + 1] - h->h_leaf_off[nn];
          enc(&maps[2 * nbox + 27 * k + sl], knear + off, (ne + 3) & ~int64_t(3), nk, 128,
              h->h_near_ld[k]);
        }
      }
    });
  for (auto& x : th) x.join();
  if (bad) {
    std::lock_guard<std::mutex> g(bad_mu);
    return set_error(HODLR3D_ERR_CUDA, "a tensor map could not be encoded (%s)", bad_msg);
  }
  H3D_CUDA(h->tmaps.ensure(sizeof(CUtensorMap) * maps.size()));
  H3D_CUDA(cudaMemcpy(h->tmaps.p, maps.data(), sizeof(CUtensorMap) * maps.size(),
                      cudaMemcpyHostToDevice));
  h->maps_built = true;
  return HODLR3D_OK;
}

// FP32 near-field blocks of every leaf (both FP32 engines), evaluated once
// per assembly.  The blocks of leaf k (slots 0..25 the neighbours, 26
// itself; absent neighbours skipped) sit side by side in one row-major
// nk x Rn_k matrix at h_near_base[k] (Rn_k = h_near_ld[k], the sum of their
// round4(ne)); slot s's block starts at h_near_off[27 k + s] (-1: absent).
int ensure_near_blocks(hodlr3d_t h, const h3d::NearOp& nr, cudaStream_t s) {
  if (h->near_built) return HODLR3D_OK;
  h->h_nbr_leaf.resize(26 * h->nleaf);
  H3D_CUDA(cudaMemcpy(h->h_nbr_leaf.data(), h->nbr_leaf.p, sizeof(int32_t) * 26 * h->nleaf,
                      cudaMemcpyDeviceToHost));
  const std::vector<int32_t>& nbl = h->h_nbr_leaf;
  std::vector<int64_t>& off = h->h_near_off;
  off.assign(27 * h->nleaf, -1);
  h->h_near_base.assign(h->nleaf, 0);
  h->h_near_ld.assign(h->nleaf, 0);
  int64_t tot = 0;
  for (int64_t k = 0; k < h->nleaf; ++k) {
    const int64_t nk = h->h_leaf_off[k + 1] - h->h_leaf_off[k];
    int64_t col = 0;
    for (int sl = 0; sl < 27; ++sl) {
      const int64_t nn = sl < 26 ? nbl[26 * k + sl] : k;
      if (nn < 0) continue;
      const int64_t ne = h->h_leaf_off[nn + 1] - h->h_leaf_off[nn];
      off[27 * k + sl] = tot + col;
      col += (ne + 3) & ~int64_t(3);
    }
    h->h_near_base[k] = tot;
    h->h_near_ld[k] = (int32_t)col;
    tot += nk * col;
  }
  H3D_CUDA(h->knear.ensure(sizeof(float) * std::max<int64_t>(tot, 4)));
  H3D_CUDA(h->near_off.ensure(sizeof(int64_t) * off.size()));
  H3D_CUDA(cudaMemcpy(h->near_off.p, off.data(), sizeof(int64_t) * off.size(),
                      cudaMemcpyHostToDevice));
  H3D_CUDA(h->near_base.ensure(sizeof(int64_t) * h->nleaf));
  H3D_CUDA(cudaMemcpy(h->near_base.p, h->h_near_base.data(), sizeof(int64_t) * h->nleaf,
                      cudaMemcpyHostToDevice));
  H3D_CUDA(h->near_ld.ensure(sizeof(int32_t) * h->nleaf));
  H3D_CUDA(cudaMemcpy(h->near_ld.p, h->h_near_ld.data(), sizeof(int32_t) * h->nleaf,
                      cudaMemcpyHostToDevice));
  h->launches += h3d::launch_near_blocks(s, h->nleaf, h->leaf_off.as<int32_t>(), nr,
                                         h->near_off.as<int64_t>(), h->near_ld.as<int32_t>(),
                                         h->knear.as<float>());
  H3D_CUDA(cudaGetLastError());
  h->near_floats = tot;
  h->near_built = true;
  h->maps_built = false;
  return HODLR3D_OK;
}

// Work lists and index tables of the few-column engine (matvec_gemv.cu) over
// the grouped FP32 layouts; leaves it off (gemv_ok false) when the tree does
// not fit its shared memory or 32-bit row numbers.
int ensure_gemv(hodlr3d_t h, cudaStream_t s) {
  if (h->gemv_built) return HODLR3D_OK;
  h->gemv_built = true;
  h->gemv_ok = false;
  const int ml4 = (h->max_leaf + 3) & ~3;
  if (h3d::gemv_smem_bytes(ml4, 4, true) > 200 * 1024) return HODLR3D_OK;
  const int64_t np = h->npairs;
  const int64_t nbox = (int64_t)h->h_vbox_rows.size();
  const int64_t trows = h->h_tbox_off[nbox] / 32;
  std::vector<int64_t> vrow0(nbox + 1, 0), tbase(nbox, 0), vpofs(nbox, -1), upofs(nbox, -1);
  for (int64_t b = 0; b < nbox; ++b) {
    tbase[b] = h->h_tbox_off[b] / 32;
    vrow0[b + 1] = vrow0[b] + h->h_vbox_rows[b];
  }
  const int64_t vrows = vrow0[nbox];
  if (trows >= INT32_MAX || vrows >= INT32_MAX) return HODLR3D_OK;
  std::vector<int32_t> rev(std::max<int64_t>(np, 1)), tgt(std::max<int64_t>(np, 1));
  if (np) H3D_CUDA(cudaMemcpy(rev.data(), h->rev.p, sizeof(int32_t) * np, cudaMemcpyDeviceToHost));
  for (int64_t b = 0; b < nbox; ++b)
    for (int64_t p = h->h_il_ptr[b]; p < h->h_il_ptr[b + 1]; ++p) tgt[p] = (int32_t)b;
  std::vector<int32_t> vrow_t(std::max<int64_t>(vrows, 1)), trow_v(std::max<int64_t>(trows, 1), -1);
  std::vector<int32_t> vt_upper, ut_upper;
  std::vector<int32_t> vt_items, ut_items;  // int4 / int2 records
  int64_t pv = 0, pu = 0;
  for (int64_t b = 0; b < nbox; ++b) {
    int j = 0;
    while (j < h->levels && h3d::level_base(j + 1) <= b) ++j;
    int64_t a0, a1;
    box_range(h, j, b - h3d::level_base(j), a0, a1);
    const int64_t m = a1 - a0, m4 = (m + 3) & ~int64_t(3);
    // V stack of b as a source box: rows map to T rows of the pairs' targets
    int64_t v = vrow0[b];
    for (int64_t q = h->h_il_ptr[b]; q < h->h_il_ptr[b + 1]; ++q) {
      const int p = rev[q];
      const int64_t base = tbase[tgt[p]] + h->h_coff[p];
      for (int l = 0; l < h->h_rank[p]; ++l) {
        trow_v[base + l] = (int32_t)v;
        vrow_t[v++] = (int32_t)(base + l);
      }
    }
    const int rows = h->h_vbox_rows[b];
    if (rows > 0 && m > 0) {
      const int nch = (int)((m4 + h3d::kGemvCols - 1) / h3d::kGemvCols);
      if (nch > 1) {
        vpofs[b] = pv;
        pv += (int64_t)rows * nch;
        vt_upper.push_back((int32_t)b);
      }
      for (int ci = 0; ci < nch; ++ci)
        for (int r0 = 0; r0 < rows; r0 += h3d::kGemvRowChunk) {
          const int rec[4] = {(int32_t)b, ci, r0, std::min(h3d::kGemvRowChunk, rows - r0)};
          vt_items.insert(vt_items.end(), rec, rec + 4);
        }
    }
    // U of b as a target box
    const int R = h->h_rbox[b];
    if (R > 0 && m > 0) {
      const int nch = (int)((m + h3d::kGemvRowsT - 1) / h3d::kGemvRowsT);
      if (nch > 1) {
        upofs[b] = pu;
        pu += (int64_t)R * nch;
        ut_upper.push_back((int32_t)b);
      }
      for (int ci = 0; ci < nch; ++ci) {
        ut_items.push_back((int32_t)b);
        ut_items.push_back(ci);
      }
    }
  }
  auto put = [](DevBuf& d, const void* src, size_t bytes) -> cudaError_t {
    cudaError_t e = d.ensure(std::max<size_t>(bytes, 16));
    if (e != cudaSuccess || bytes == 0) return e;
    return cudaMemcpy(d.p, src, bytes, cudaMemcpyHostToDevice);
  };
  H3D_CUDA(put(h->gv_ubox_off, h->h_ubox_off.data(), sizeof(int64_t) * nbox));
  H3D_CUDA(put(h->gv_vbox_off, h->h_vbox_off.data(), sizeof(int64_t) * nbox));
  H3D_CUDA(put(h->gv_vbox_rows, h->h_vbox_rows.data(), sizeof(int32_t) * nbox));
  H3D_CUDA(put(h->gv_vrow0, vrow0.data(), sizeof(int64_t) * (nbox + 1)));
  H3D_CUDA(put(h->gv_vrow_t, vrow_t.data(), sizeof(int32_t) * vrows));
  H3D_CUDA(put(h->gv_trow_v, trow_v.data(), sizeof(int32_t) * trows));
  H3D_CUDA(put(h->gv_tbase, tbase.data(), sizeof(int64_t) * nbox));
  H3D_CUDA(put(h->gv_vpofs, vpofs.data(), sizeof(int64_t) * nbox));
  H3D_CUDA(put(h->gv_upofs, upofs.data(), sizeof(int64_t) * nbox));
  H3D_CUDA(put(h->gv_vt_items, vt_items.data(), sizeof(int32_t) * vt_items.size()));
  H3D_CUDA(put(h->gv_vt_upper, vt_upper.data(), sizeof(int32_t) * vt_upper.size()));
  H3D_CUDA(put(h->gv_ut_items, ut_items.data(), sizeof(int32_t) * ut_items.size()));
  H3D_CUDA(put(h->gv_ut_upper, ut_upper.data(), sizeof(int32_t) * ut_upper.size()));
  h->gv_n_vt_items = (int64_t)vt_items.size() / 4;
  h->gv_n_vt_upper = (int64_t)vt_upper.size();
  h->gv_n_ut_items = (int64_t)ut_items.size() / 2;
  h->gv_n_ut_upper = (int64_t)ut_upper.size();
  // 8 columns (mixed); the fp64x form's 4 columns of FP32 pairs fit too
  H3D_CUDA(h->gv_x.ensure(sizeof(float) * 8 * h->N));
  H3D_CUDA(h->gv_t.ensure(sizeof(float) * 8 * std::max<int64_t>(trows, 1)));
  H3D_CUDA(cudaMemsetAsync(h->gv_t.p, 0, sizeof(float) * 8 * std::max<int64_t>(trows, 1), s));
  H3D_CUDA(h->gv_tt.ensure(sizeof(float) * 8 * std::max<int64_t>(vrows, 1)));
  H3D_CUDA(h->gv_p.ensure(sizeof(float) * 8 * std::max<int64_t>(pv, 1)));
  H3D_CUDA(h->gv_pt.ensure(sizeof(float) * 8 * std::max<int64_t>(pu, 1)));
  h->gemv8_ok = h3d::gemv_smem_bytes(ml4, 8, false) <= 200 * 1024;
  h->gemv_ok = true;
  return HODLR3D_OK;
}

// The FP64-accurate form's lo parts (U, V, near field) and its work buffers,
// built on first use after each assembly.
int ensure_lo(hodlr3d_t h, const h3d::NearOp& nr, cudaStream_t s) {
  if (h->lo_built) return HODLR3D_OK;
  const int64_t np = h->npairs;
  const float* ubase = h->u32_pool->as<float>();
  const float* vbase = h->v32_pool->as<float>();
  H3D_CUDA(h->u32lo_pool.ensure(h->u32_pool->bytes));
  H3D_CUDA(h->v32lo_pool.ensure(h->v32_pool->bytes));
  if (np) {
    std::vector<float*> ulo(np), vlo(np);
    for (int64_t p = 0; p < np; ++p) {
      ulo[p] = h->u32lo_pool.as<float>() + (h->h_u32[p] - ubase);
      vlo[p] = h->v32lo_pool.as<float>() + (h->h_v32[p] - vbase);
    }
    DevBuf d64, dlo, dsz, dr, dus;
    H3D_CUDA(d64.ensure(sizeof(void*) * np));
    H3D_CUDA(dlo.ensure(sizeof(void*) * np));
    H3D_CUDA(dsz.ensure(sizeof(int32_t) * np));
    H3D_CUDA(dr.ensure(sizeof(int32_t) * np));
    H3D_CUDA(dus.ensure(sizeof(int32_t) * np));
    H3D_CUDA(cudaMemcpy(dr.p, h->h_rank.data(), sizeof(int32_t) * np, cudaMemcpyHostToDevice));
    H3D_CUDA(cudaMemcpy(dus.p, h->h_ustride.data(), sizeof(int32_t) * np, cudaMemcpyHostToDevice));
    // V
    H3D_CUDA(cudaMemcpy(d64.p, h->h_v64.data(), sizeof(void*) * np, cudaMemcpyHostToDevice));
    H3D_CUDA(cudaMemcpy(dlo.p, vlo.data(), sizeof(void*) * np, cudaMemcpyHostToDevice));
    H3D_CUDA(cudaMemcpy(dsz.p, h->h_pair_m.data(), sizeof(int32_t) * np, cudaMemcpyHostToDevice));
    H3D_CUDA(h3d::launch_v32(s, np, d64.as<const double* const>(), dlo.as<float* const>(),
                             dsz.as<int32_t>(), dr.as<int32_t>(), 1));
    H3D_CUDA(cudaStreamSynchronize(s));
    // U
    H3D_CUDA(cudaMemcpy(d64.p, h->h_u64.data(), sizeof(void*) * np, cudaMemcpyHostToDevice));
    H3D_CUDA(cudaMemcpy(dlo.p, ulo.data(), sizeof(void*) * np, cudaMemcpyHostToDevice));
    H3D_CUDA(cudaMemcpy(dsz.p, h->h_pair_n.data(), sizeof(int32_t) * np, cudaMemcpyHostToDevice));
    H3D_CUDA(h3d::launch_u32(s, np, d64.as<const double* const>(), dlo.as<float* const>(),
                             dsz.as<int32_t>(), dus.as<int32_t>(), dr.as<int32_t>(), 1));
    H3D_CUDA(cudaStreamSynchronize(s));
    h->launches += 2;
  }
  H3D_CUDA(h->knearlo.ensure(sizeof(float) * std::max<int64_t>(h->near_floats, 4)));
  h->launches += h3d::launch_near_lo(s, h->nleaf, h->leaf_off.as<int32_t>(), nr,
                                     h->near_off.as<int64_t>(), h->near_ld.as<int32_t>(),
                                     h->knear.as<float>(), h->knearlo.as<float>());
  H3D_CUDA(cudaGetLastError());
  const int64_t nbox = (int64_t)h->h_vbox_rows.size();
  const int64_t trows = std::max<int64_t>(h->h_tbox_off[nbox] / 32, 1);
  const size_t gp = h->gv_p.bytes / sizeof(float), gpt = h->gv_pt.bytes / sizeof(float);
  H3D_CUDA(h->gv_xl.ensure(sizeof(float) * 4 * h->N));
  H3D_CUDA(h->gv_tl.ensure(sizeof(float) * 4 * trows));
  H3D_CUDA(cudaMemsetAsync(h->gv_tl.p, 0, sizeof(float) * 4 * trows, s));
  H3D_CUDA(h->gv_ttl.ensure(h->gv_tt.bytes));
  H3D_CUDA(h->gv_pd.ensure(sizeof(double) * gp));
  H3D_CUDA(h->gv_ptd.ensure(sizeof(double) * gpt));
  h->lo_built = true;
  return HODLR3D_OK;
}

// The few-column engine (matvec_gemv.cu) over this handle's tables, in passes
// of 4 (or 8) columns; its tables and, for fp64x, the lo parts exist.
int run_gemv(hodlr3d_t h, const double* x, double* y, int nrhs, int64_t ld, cudaStream_t s,
             bool trans, bool fp64x) {
  h3d::GemvOp g{};
  g.levels = h->levels;
  g.max_leaf4 = (h->max_leaf + 3) & ~3;
  g.nleaf = h->nleaf;
  g.N = h->N;
  g.leaf_off = h->leaf_off.as<int32_t>();
  g.perm = h->perm.as<int32_t>();
  g.nbr_leaf = h->nbr_leaf.as<int32_t>();
  g.u32 = h->u32_pool->as<float>();
  g.v32 = h->v32_pool->as<float>();
  g.ubox_off = h->gv_ubox_off.as<int64_t>();
  g.rbox = h->tc_rbox.as<int32_t>();
  g.vbox_off = h->gv_vbox_off.as<int64_t>();
  g.vbox_rows = h->gv_vbox_rows.as<int32_t>();
  g.vrow0 = h->gv_vrow0.as<int64_t>();
  g.vrow_t = h->gv_vrow_t.as<int32_t>();
  g.trow_v = h->gv_trow_v.as<int32_t>();
  g.tbase = h->gv_tbase.as<int64_t>();
  g.vpofs = h->gv_vpofs.as<int64_t>();
  g.upofs = h->gv_upofs.as<int64_t>();
  g.knear = h->knear.as<float>();
  g.u32lo = fp64x ? h->u32lo_pool.as<float>() : nullptr;
  g.v32lo = fp64x ? h->v32lo_pool.as<float>() : nullptr;
  g.knearlo = fp64x ? h->knearlo.as<float>() : nullptr;
  g.near_base = h->near_base.as<int64_t>();
  g.near_ld = h->near_ld.as<int32_t>();
  g.near_off = h->near_off.as<int64_t>();
  h3d::GemvBuffers gb{};
  gb.xg = h->gv_x.as<float>();
  gb.t = h->gv_t.as<float>();
  gb.tt = h->gv_tt.as<float>();
  gb.p = h->gv_p.as<float>();
  gb.pt = h->gv_pt.as<float>();
  gb.xl = h->gv_xl.as<float>();
  gb.tl = h->gv_tl.as<float>();
  gb.ttl = h->gv_ttl.as<float>();
  gb.pd = h->gv_pd.as<double>();
  gb.ptd = h->gv_ptd.as<double>();
  gb.vt_items = h->gv_vt_items.as<int4>();
  gb.n_vt_items = h->gv_n_vt_items;
  gb.vt_upper = h->gv_vt_upper.as<int32_t>();
  gb.n_vt_upper = h->gv_n_vt_upper;
  gb.ut_items = h->gv_ut_items.as<int2>();
  gb.n_ut_items = h->gv_n_ut_items;
  gb.ut_upper = h->gv_ut_upper.as<int32_t>();
  gb.n_ut_upper = h->gv_n_ut_upper;
  // passes of 8 columns for the mixed transpose (when the leaves'
  // near-field inputs fit the shared memory: 8 columns 11.6 ms against two
  // passes of 4, 14.1 ms, at 64^3), else of 4 (the forward kernels read the
  // vector with a lane stride of 4 NR floats, which 8 columns turn into
  // serialised shared-memory and L1 accesses: 16.8 ms against 11.4)
  const int width = (!fp64x && trans && nrhs > 4 && h->gemv8_ok) ? 8 : 4;
  for (int c0 = 0; c0 < nrhs; c0 += width)
    h->launches += h3d::launch_matvec_gemv(s, g, gb, x + c0 * ld, ld, y + c0 * ld, ld,
                                           std::min(width, nrhs - c0), trans, fp64x,
                                           h->profiling ? &h->prof : nullptr);
  H3D_CUDA(cudaGetLastError());
  return HODLR3D_OK;
}

// The tensor-core engine (matvec_tc.cu) in batches of 32 columns; builds its
// near-field blocks and tensor maps on first use.
int run_tc(hodlr3d_t h, const h3d::FarOp& far, const h3d::NearOp& nr, const double* x, double* y,
           int nrhs, int64_t ld, cudaStream_t s) {
  H3D_TRY(ensure_matvec_buffers(h, 32));  // slice partials and level sums of 32 columns
  if (!h->dev_err.p) {
    H3D_CUDA(h->dev_err.ensure(sizeof(int)));
    H3D_CUDA(cudaMemsetAsync(h->dev_err.p, 0, sizeof(int), s));
  }
  H3D_TRY(ensure_near_blocks(h, nr, s));
  if (!h->maps_built) H3D_TRY(build_tensor_maps(h, h->h_near_off));
  // [X | T], the B operands in the split-exact form
  H3D_CUDA(h->tct.ensure(sizeof(float) * 32 * (h->N + std::max<int64_t>(h->sum_rank4, 1))));
  h3d::TcBuffers T{};
  T.xt = h->tct.as<float>();
  T.t = T.xt + 32 * h->N;
  T.p = reinterpret_cast<float*>(h->pbuf.p);
  T.ynl = h->ynl.as<double>();
  T.err = h->dev_err.as<int>();
  T.upper_pairs = h->upper.as<int32_t>();
  T.n_upper = h->n_upper;
  T.max_slice = h->max_slice;
  T.knear = h->knear.as<float>();
  T.near_off = h->near_off.as<int64_t>();
  const CUtensorMap* tm = h->tmaps.as<CUtensorMap>();
  const int64_t nbox = (int64_t)h->h_vbox_rows.size();
  T.umaps = tm;
  T.vmaps = tm + nbox;
  T.nmaps = tm + 2 * nbox;
  for (int c0 = 0; c0 < nrhs; c0 += 32)
    h->launches += h3d::launch_matvec_tc(s, h->N, h->perm.as<int32_t>(), far, nr, T, x + c0 * ld,
                                         ld, y + c0 * ld, ld, std::min(32, nrhs - c0),
                                         h->profiling ? &h->prof : nullptr);
  H3D_CUDA(cudaGetLastError());
  return HODLR3D_OK;
}

// largest column counts the few-column engine takes in the automatic choice
// (measured at 64^3: 5.7 ms for 4 columns against 10.4 ms for the tensor
// cores' 32; transposed, 7.0 ms for 4 and 46 ms for 32 columns against 28
// and 53 ms for the CUDA-core transpose)
constexpr int kGemvForwardMax = 4;
constexpr int kGemvTransposeMax = 32;
// on trees the tensor-core engine does not take, passes of 4 columns beat the
// CUDA-core kernels' single pass up to 32 columns (64^3: ~6 ms per pass
// against 54 ms for 32 columns)
constexpr int kGemvForwardNoTcMax = 32;

// The operator as the matvec kernels see it: pair tables and factors (FP32
// copies when f32, else the FP64 factors), and the near field.
h3d::FarOp far_op(hodlr3d_t h, bool f32) {
  h3d::FarOp far{};
  far.levels = h->levels;
  far.nleaf = h->nleaf;
  far.leaf_off = h->leaf_off.as<int32_t>();
  far.il_ptr = h->il_ptr.as<int64_t>();
  far.rev = h->rev.as<int32_t>();
  far.rank = h->rank.as<int32_t>();
  far.pair_level = h->pair_level.as<int32_t>();
  far.pair_tgt = h->pair_tgt.as<int32_t>();
  far.pair_src = h->pair_src.as<int32_t>();
  far.tr_off = h->tr_off.as<int64_t>();
  far.ustride = h->ustride.as<int32_t>();
  far.tc_toff = h->tc_toff.as<int64_t>();
  far.tc_tld = h->tc_tld.as<int32_t>();
  far.tc_tbox = h->tc_tbox.as<int64_t>();
  far.tc_rbox = h->tc_rbox.as<int32_t>();
  far.part_off = h->part_off.as<int64_t>();
  far.ufac = f32 ? h->u32.as<const void*>() : h->u64.as<const void*>();
  far.vfac = f32 ? h->v32.as<const void*>() : h->v64.as<const void*>();
  return far;
}

h3d::NearOp near_op(hodlr3d_t h) {
  h3d::NearOp nr{};
  nr.nbr_leaf = h->nbr_leaf.as<int32_t>();
  nr.xs = h->xs.as<double>();
  nr.ys = h->ys.as<double>();
  nr.zs = h->zs.as<double>();
  nr.xl = h->xl.as<float>();
  nr.yl = h->yl.as<float>();
  nr.zl = h->zl.as<float>();
  nr.centre = h->centre.as<double>();
  nr.kd = h->kd;
  return nr;
}

int matvec_device(hodlr3d_t h, const double* x, double* y, int nrhs, int64_t ld, int precision,
                  cudaStream_t s, bool trans) {
  if (!h->assembled) return set_error(HODLR3D_ERR_NOT_ASSEMBLED, "hodlr3d_assemble has not run");
  if (!x || !y) return set_error(HODLR3D_ERR_INVALID_ARG, "null vector");
  if (nrhs < 1 || nrhs > 64) return set_error(HODLR3D_ERR_INVALID_ARG, "nrhs must be in 1..64");
  if (ld < h->N) return set_error(HODLR3D_ERR_INVALID_ARG, "ld < n");
  if (precision != HODLR3D_FP64 && precision != HODLR3D_MIXED && precision != HODLR3D_FP64X)
    return set_error(HODLR3D_ERR_INVALID_ARG, "unknown precision %d", precision);
  if (precision == HODLR3D_MIXED && !h->opt.keep_fp32)
    return set_error(HODLR3D_ERR_INVALID_ARG, "mixed precision needs keep_fp32");
  // the FP64-accurate form builds on the FP32 copies; without them, or on a
  // tree the few-column kernels do not take, it is the FP64 form
  if (precision == HODLR3D_FP64X && !h->opt.keep_fp32) precision = HODLR3D_FP64;
  H3D_TRY(ensure_matvec_buffers(h, nrhs));
  const bool f32 = precision == HODLR3D_MIXED;
  h3d::FarOp far = far_op(h, f32);
  const h3d::NearOp nr = near_op(h);
  h3d::MatvecBuffers B{};
  B.xsorted = h->xsorted.p;
  B.tbuf = h->tbuf.p;
  B.pbuf = h->pbuf.as<double>();
  B.ynl = h->ynl.as<double>();
  B.items = h->items.as<int32_t>();
  B.n_items = h->n_items;
  B.upper_pairs = h->upper.as<int32_t>();
  B.n_upper = h->n_upper;
  B.max_slice = h->max_slice;
  // Mixed form: the few-column engine streams the FP32 factors once per 4
  // right-hand sides; the tensor-core engine once per 32 at a higher cost per
  // factor entry, so it takes the forward product from kGemvForwardMax + 1
  // columns on.  The transpose has no tensor-core form: past
  // kGemvTransposeMax columns the CUDA-core kernels (all columns in one pass)
  // are faster.
  const bool mixed = precision == HODLR3D_MIXED;
  const bool fp64x = precision == HODLR3D_FP64X;
  // the engine of this call: forced, tuned (automatic choice after
  // hodlr3d_autotune, mixed form) or 0 for the rules below
  const int engine = h->engine == 0 && mixed ? h->tuned[trans ? 1 : 0][nrhs] : h->engine;
  // trees the tensor-core engine takes (16-byte aligned leaf rows, bounded tables)
  const bool tc_tree = h->max_leaf <= 128 && h->leaves_aligned && h->tc_entries <= h3d::tc_max_entries();
  const int gemv_max = trans ? kGemvTransposeMax : (tc_tree ? kGemvForwardMax : kGemvForwardNoTcMax);
  bool use_gemv = false;
  // fp64x: the few-column kernels (automatic or forced); forcing the CUDA-core
  // kernels gives the FP64 form; the tensor cores have no FP64-accurate form
  if (fp64x && engine == 2)
    return set_error(HODLR3D_ERR_UNSUPPORTED,
                     "the tensor-core engine has no FP64-accurate form (use HODLR3D_MIXED or "
                     "another engine)");
  if ((fp64x && engine != 1) ||
      (mixed && (engine == 3 || (engine == 0 && nrhs <= gemv_max)))) {
    H3D_TRY(ensure_near_blocks(h, nr, s));
    H3D_TRY(ensure_gemv(h, s));
    use_gemv = h->gemv_ok;
    if (use_gemv && fp64x && !h->lo_unavailable) {
      const int st = ensure_lo(h, nr, s);
      if (st == HODLR3D_ERR_OUT_OF_MEMORY) {
        // the lo parts (as large as the FP32 copies) do not fit: the FP64 form
        // serves instead, now and for the rest of this assembly
        cudaGetLastError();
        h->u32lo_pool.release();
        h->v32lo_pool.release();
        h->knearlo.release();
        h->lo_unavailable = true;
      } else if (st != HODLR3D_OK) {
        return st;
      }
    }
    if (fp64x && h->lo_unavailable) use_gemv = false;
  }
  if (fp64x && !use_gemv) {
    precision = HODLR3D_FP64;
    far = far_op(h, false);
  }
  if (engine == 3 && !use_gemv && !fp64x)
    return set_error(HODLR3D_ERR_UNSUPPORTED,
                     "the few-column engine needs the mixed form, leaves whose near-field inputs "
                     "fit its shared memory and fewer than 2^31 rows of T");
  if (use_gemv) return run_gemv(h, x, y, nrhs, ld, s, trans, fp64x);
  const bool tc_ok = mixed && !trans && tc_tree;
  if (engine == 2 && !tc_ok)
    return set_error(HODLR3D_ERR_UNSUPPORTED,
                     "the tensor-core engine needs A x (not the transpose) in the mixed form, "
                     "leaves of at most 128 points, each a multiple of 4, and at most %d pairs per "
                     "block (this tree: %d)", h3d::tc_max_entries(), h->tc_entries);
  if (tc_ok && engine != 1) return run_tc(h, far, nr, x, y, nrhs, ld, s);
  // the CUDA-core engine (matvec.cu)
  h->launches += h3d::launch_matvec(s, h->N, h->perm.as<int32_t>(), far, nr, B, x, ld, y, ld, nrhs,
                                    precision, trans ? 1 : 0, h->profiling ? &h->prof : nullptr);
  H3D_CUDA(cudaGetLastError());
  return HODLR3D_OK;
}

// ---------------------------------------------------------------------------
// autotuning of the automatic engine choice
// ---------------------------------------------------------------------------
// Column counts timed; a count between two of them takes the choice of the
// next one up (the engines' costs step at powers of two: the tensor cores pad
// to 32 columns, the CUDA-core kernels to the next power of two, the
// few-column kernels run passes of 4 or 8).
constexpr int kTuneCounts[] = {1, 2, 4, 8, 16, 32, 64};
constexpr int kNumTuneCounts = sizeof(kTuneCounts) / sizeof(kTuneCounts[0]);

// Times every engine that runs the mixed product of this operator (A x: CUDA
// cores, tensor cores, few-column kernels; A^T x: CUDA cores, few-column) at
// each count of kTuneCounts, `reps` timed products after one untimed, the
// median kept; the fastest fills h->tuned.  The inputs are one constant (every
// byte 0x3F: 4.8e-4; no kernel branches on values).  The forced engine
// (hodlr3d_set_engine) is restored.
int autotune(hodlr3d_t h, int reps, std::string& report) {
  std::memset(h->tuned, 0, sizeof h->tuned);
  report.clear();
  if (reps == 0) return HODLR3D_OK;
  if (!h->assembled) return set_error(HODLR3D_ERR_NOT_ASSEMBLED, "hodlr3d_assemble has not run");
  if (!h->opt.keep_fp32) return set_error(HODLR3D_ERR_INVALID_ARG, "the mixed form needs keep_fp32");
  const int64_t N = h->N;
  const size_t bytes = sizeof(double) * N * 64;
  DevBuf X, Y;
  H3D_CUDA(X.ensure(bytes));
  H3D_CUDA(Y.ensure(bytes));
  cudaStream_t s = h->stream;
  H3D_CUDA(cudaMemsetAsync(X.p, 0x3F, bytes, s));
  EventPair ev;
  H3D_CUDA(cudaEventCreate(&ev.a));
  H3D_CUDA(cudaEventCreate(&ev.b));
  const int forced = h->engine;
  int8_t choice[2][kNumTuneCounts] = {};
  char line[160];
  report = "transpose nrhs engine ms\n";
  int st = HODLR3D_OK;
  for (int tr = 0; tr < 2 && st == HODLR3D_OK; ++tr) {
    for (int ci = 0; ci < kNumTuneCounts && st == HODLR3D_OK; ++ci) {
      const int nrhs = kTuneCounts[ci];
      float best = 0.f;
      for (int eng = 1; eng <= 3; ++eng) {
        if (tr && eng == 2) continue;  // no tensor-core transpose
        h->engine = eng;
        // untimed product: builds the engine's tables and buffers
        st = matvec_device(h, X.as<double>(), Y.as<double>(), nrhs, N, HODLR3D_MIXED, s, tr != 0);
        if (st == HODLR3D_ERR_UNSUPPORTED) {  // this tree does not suit the engine
          st = HODLR3D_OK;
          continue;
        }
        if (st != HODLR3D_OK) break;
        std::vector<float> ms(reps);
        for (int r = 0; r < reps && st == HODLR3D_OK; ++r) {
          cudaError_t e = cudaEventRecord(ev.a, s);
          if (e == cudaSuccess) {
            st = matvec_device(h, X.as<double>(), Y.as<double>(), nrhs, N, HODLR3D_MIXED, s, tr != 0);
            e = cudaEventRecord(ev.b, s);
          }
          if (e == cudaSuccess) e = cudaEventSynchronize(ev.b);
          if (e == cudaSuccess) e = cudaEventElapsedTime(&ms[r], ev.a, ev.b);
          if (e != cudaSuccess && st == HODLR3D_OK)
            st = set_error(HODLR3D_ERR_CUDA, "autotune timing: %s", cudaGetErrorString(e));
        }
        if (st != HODLR3D_OK) break;
        std::sort(ms.begin(), ms.end());
        const float med = ms[reps / 2];
        std::snprintf(line, sizeof line, "%d %d %d %.6f\n", tr, nrhs, eng, med);
        report += line;
        if (choice[tr][ci] == 0 || med < best) {
          choice[tr][ci] = (int8_t)eng;
          best = med;
        }
      }
    }
  }
  h->engine = forced;
  if (st != HODLR3D_OK) return st;
  for (int tr = 0; tr < 2; ++tr) {
    int ci = 0;
    for (int n = 1; n <= 64; ++n) {
      while (kTuneCounts[ci] < n) ++ci;
      h->tuned[tr][n] = choice[tr][ci];
    }
  }
  return HODLR3D_OK;
}

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

}  // namespace

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

int hodlr3d_gmres(hodlr3d_t h, const double* b, double* x, int nrhs, int64_t ld,
                  const hodlr3d_gmres_params* prm, hodlr3d_gmres_result* res, double* hist,
                  int hist_cap, int* n_hist, void* stream) try {
  H3D_TRY(check_handle(h));
  if (!h->assembled) return set_error(HODLR3D_ERR_NOT_ASSEMBLED, "hodlr3d_assemble has not run");
  if (!b || !x || !prm || nrhs < 1 || nrhs > 64 || ld < h->N || prm->maxit < 1 || !(prm->tol > 0))
    return set_error(HODLR3D_ERR_INVALID_ARG, "bad GMRES arguments");
  // inputs may still be in flight on the caller's stream
  H3D_CUDA(cudaStreamSynchronize((cudaStream_t)stream));
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
  if (v == 2)
    return set_error(HODLR3D_ERR_CUDA, "a tensor-core block's operand table overflowed (results of that call are invalid)");
  if (v) return set_error(HODLR3D_ERR_CUDA, "a tensor-core wait gave up (results of that call are invalid)");
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
