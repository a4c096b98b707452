// Matvec launchers (matvec.cu).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "common.cuh"

namespace h3d {

// The compressed (far-field) part of the operator: per pair its rank and the
// factors U (n x r) and V (m x r), column-major; n, m are the sizes of the
// target and source boxes.  Pairs are sorted by target box; il_ptr indexes
// them by box (all levels numbered together), rev lists them by source box.
struct FarOp {
  int levels;
  int64_t nleaf;
  const int32_t* leaf_off;    // nleaf + 1
  const int64_t* il_ptr;      // boxes of all levels + 1
  const int32_t* rev;         // rev[q]: pair whose source is the box owning list slot q
  const int32_t* rank;
  const int32_t* pair_level;
  const int32_t* pair_tgt;    // all-levels box numbers
  const int32_t* pair_src;
  const int64_t* tr_off;      // per pair: offset of its r rows in T (times the padded nrhs)
  const int64_t* part_off;    // per pair above level d - 1: offset of its slice partials
  const void* const* ufac;    // per pair U pointer (double* or float*)
  const void* const* vfac;    // per pair V pointer
};

// The dense near field: every leaf with its face/edge neighbours and itself.
struct NearOp {
  const int32_t* nbr_leaf;  // nleaf x 26, leaf ids or -1
  const double* xs;         // tree-ordered points, FP64
  const double* ys;
  const double* zs;
  const float* xl;          // FP32 offsets from the leaf centre
  const float* yl;
  const float* zl;
  const double* centre;     // nleaf x 3 leaf centres
  KernelDesc kd;
};

// Work buffers.  xsorted: N * NR reals; tbuf: sum_rank * NR reals; pbuf:
// part_total * NR doubles; ynl: N * NR doubles (NR = padded nrhs).
struct MatvecBuffers {
  void* xsorted;
  void* tbuf;
  double* pbuf;
  double* ynl;
  const int32_t* items;        // (pair, slice) work items of the non-leaf pairs
  int64_t n_items;
  const int32_t* upper_pairs;  // pairs above level d - 1
  int64_t n_upper;
  int max_slice;               // largest population of a level d - 1 box
};

// Optional per-kernel timing: begin() before the first launch, mark() after
// each, on the launch stream.
struct MatvecProfiler {
  virtual ~MatvecProfiler() {}
  virtual void begin(cudaStream_t s) = 0;
  virtual void mark(cudaStream_t s, const char* name) = 0;
};

int padded_nrhs(int nrhs);

// precision: 0 = FP64, 1 = mixed.  X, Y column-major in the original order.
// Returns the number of kernel launches.
int launch_matvec(cudaStream_t s, int64_t N, const int32_t* perm, const FarOp& far,
                  const NearOp& near, const MatvecBuffers& B, const double* X, int64_t ldx,
                  double* Y, int64_t ldy, int nrhs, int precision, int trans,
                  MatvecProfiler* prof);

void launch_dense_rows(cudaStream_t s, int64_t N, const double* xyz, KernelDesc kd,
                       const int64_t* rows, int64_t nrows, const double* X, int64_t ldx,
                       double* Y, int nrhs);

}  // namespace h3d
