// Host side of the hodlr3d_gb300 C ABI, internal header (not installed): the
// handle with its device buffers, the error helpers, and the functions the
// host translation units share.
//   setup.cpp    handle checks, tree build, batched ACA, post-ACA tables
//   factors.cpp  factor files (hodlr3d_save / hodlr3d_load)
//   product.cpp  the three matvec engines' host drivers, engine autotuning
//   solve.cpp    GMRES cycles
//   capi.cpp     the extern "C" entry points
//
// Reference interfaces replaced: HODLR3D (include/HODLR3D.hpp:12-21,
// src/HODLR3D.cpp), HODLR3DTree (include/HODLR3DTree.hpp, src/HODLR3DTree.cpp),
// LowRank (src/ACA.cpp), classGMRES (include/gmres.hpp, src/gmres.cpp).
#pragma once
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

namespace hodlr3d_host {

// message of the last failure of the calling thread (hodlr3d_last_error)
extern thread_local std::string g_last_error;
// records a printf-style message and returns code
int set_error(int code, const char* fmt, ...);
// the C entry points are function-try-blocks whose handler returns this: an
// exception (a host allocation that failed) becomes a status code instead of
// crossing the C ABI
int exception_status() noexcept;
double now_s();
// diagonal of Qchoice 16 (include/kernel.hpp:43-61)
double quadrature_kii(int64_t N);

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

}  // namespace hodlr3d_host

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


// the handle (include/hodlr3d.h's opaque hodlr3d_t) owns its device buffers
using hodlr3d_host::DevBuf;

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
  // blocks per level d-1 slice of the tensor-core T kernel chosen by
  // hodlr3d_autotune (0: the rule of launch_matvec_tc)
  int tc_split = 0;
  DevBuf dev_err;   // set by kernels whose bounded waits gave up
  bool leaves_aligned = false;  // every leaf population a multiple of 4
  DevBuf knear, near_off;       // FP32 near-field blocks of the tensor-core engine
  DevBuf tct;                   // X, T and their low parts (tensor-core engine, split-exact FP32)
  DevBuf tmaps;                 // tensor maps of the tensor-core engine: U, V, leaf rows
  // leaf rows of the tensor-core engine (product.cpp ensure_leaf_rows): per
  // leaf its dense FP32 blocks (near field, then the leaf-level interaction
  // list) side by side, nk x W_k at krow + h_row_base[k]; built once per handle
  DevBuf krow, leaf_blocks, block_ptr, row_base, row_ld;
  std::vector<int64_t> h_row_base;
  std::vector<int32_t> h_row_ld;
  int max_blocks = 0;
  int64_t row_floats = 0;
  bool rows_built = false;
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
  int64_t gv_trows = 0, gv_vrows = 0, gv_pv = 0, gv_pu = 0;  // T rows, V-stack rows, partial rows
  // FP64 streaming engine (matvec_f64.cu): FP64 factors grouped like the FP32
  // copies, FP64 near-field blocks, FP64 work buffers; built on first use
  // after each assembly, left out (the CUDA-core FP64 kernels serve) when
  // they do not fit in device memory
  DevBuf u64g_pool, v64g_pool, knear64, f64_x, f64_t, f64_tt, f64_p, f64_pt;
  bool f64_built = false;
  bool f64_unavailable = false;
  // GMRES work buffers
  DevBuf g_Q, g_w, g_r, g_x, g_b, g_H, g_cs, g_sn, g_beta, g_hk, g_bnorm, g_err, g_part, g_y,
      g_kcol, g_brk, g_scal, g_d, g_coef;

  ~hodlr3d_handle() {
    for (DevBuf* b : pools) delete b;
    if (stream) cudaStreamDestroy(stream);
  }
};

namespace hodlr3d_host {

// range [start, end) in tree order of box k at level j
inline void box_range(const hodlr3d_t h, int j, int64_t k, int64_t& a, int64_t& b) {
  const int sh = 3 * (h->levels - j);
  a = h->h_leaf_off[k << sh];
  b = h->h_leaf_off[(k + 1) << sh];
}

// setup.cpp
int check_handle(hodlr3d_t h);
bool kernel_supported(int k);
int build_tree(hodlr3d_t h, const double* xyz_host);
int assemble(hodlr3d_t h);
int finish_assembly(hodlr3d_t h, double t_start);
// factors.cpp
int save_factors(hodlr3d_t h, const char* path);
int load_factors(const char* path, const hodlr3d_options* opt, hodlr3d_t* out);
// product.cpp
int ensure_matvec_buffers(hodlr3d_t h, int nrhs);
h3d::FarOp far_op(hodlr3d_t h, bool f32);
h3d::NearOp near_op(hodlr3d_t h);
int matvec_device(hodlr3d_t h, const double* x, double* y, int nrhs, int64_t ld, int precision,
                  cudaStream_t s, bool trans);
int autotune(hodlr3d_t h, int reps, std::string& report);
// solve.cpp
int gmres_cycle(hodlr3d_t h, const double* b, double* x, int nrhs, int m, double tol, int prec,
                bool trans, bool x_is_zero, const std::vector<double>& bnorm_h, int* iters,
                std::vector<double>& err_out, std::vector<double>* hist, bool* breakdown_any);

}  // namespace hodlr3d_host
