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
  const int32_t* leaf_off;  // nleaf + 1
  const int64_t* il_ptr;    // boxes of all levels + 1
  const int32_t* rev;       // rev[q]: pair whose source is the box owning list slot q
  const int32_t* rank;
  const int64_t* tr_off;    // per pair: offset of its r values in T (times nrhs)
  const int64_t* part_off;  // per pair: offset of its chunk partials (levels < leaf level)
  const void* const* ufac;  // per pair U pointer (double* or float*)
  const void* const* vfac;  // per pair V pointer
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

// precision: 0 = FP64 factors/near field, 1 = FP32 factors/near field with
// FP64 accumulation across tiles.  trans: apply A^T.
// X, Y: column-major, original point order, nrhs columns, leading dims.
// Work buffers (device): xs_buf (N * nrhs * 8 bytes), tbuf (sum_rank * nrhs
// doubles), pbuf (partials, part_total * nrhs doubles).
struct MatvecBuffers {
  void* xsorted;
  double* tbuf;
  double* pbuf;
  const int32_t* nonleaf_pairs;  // pairs above the leaf level
  int64_t n_nonleaf;
  const int32_t* pair_level;     // level of every pair
  int max_leaf;                  // largest leaf population
};

int launch_matvec(cudaStream_t s, int64_t N, const int32_t* perm, const FarOp& far,
                  const NearOp& near, const MatvecBuffers& B, const double* X, int64_t ldx,
                  double* Y, int64_t ldy, int nrhs, int precision, int trans);

void launch_dense_rows(cudaStream_t s, int64_t N, const double* xyz, KernelDesc kd,
                       const int64_t* rows, int64_t nrows, const double* X, int64_t ldx,
                       double* Y, int nrhs);

}  // namespace h3d
