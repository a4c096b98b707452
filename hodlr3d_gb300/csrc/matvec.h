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
  const int32_t* ustride;     // per pair: row stride of its FP32 U (the FP32 U of a box share rows)
  // tensor-core T, grouped by target box: box b's T is 32 x R_b (R_b = sum of
  // round4(r) over its pairs) at tc_tbox[b], element (c, k) at + c R_b + k;
  // pair p's columns start at tc_toff[p] (row stride tc_tld[p] = R_b)
  const int64_t* tc_toff;
  const int32_t* tc_tld;
  const int64_t* tc_tbox;
  const int32_t* tc_rbox;
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

// Index of element (i, l) of a pair's factor with rank r over a box of n
// points.  FP64 factors are column-major with leading dimension n.  In the
// FP32 copies U is row-major with row stride us (the FP32 U of the pairs of a
// target box sit side by side, each rank padded to a multiple of 4) and V is
// column-major with n padded to a multiple of 4 (zero padding), so that every
// row of U and column of V starts on 16 bytes for the tensor-core kernels;
// their values are in the split-exact TF32 form (tf32_split_value), and the
// FP32 V of the pairs of one source box are stored one after the other.
template <typename FT, bool IS_U>
__host__ __device__ __forceinline__ int64_t fac_idx(int64_t i, int l, int r, int64_t n, int64_t us) {
  if (sizeof(FT) == 8) return (int64_t)l * n + i;
  if (IS_U) return i * us + l;
  return (int64_t)l * ((n + 3) & ~3) + i;
}

// One dense block of a leaf row (tensor-core engine): the block of leaf k
// with source leaf `src` (its near field or its leaf-level interaction list)
// at column x0 of leaf k's row matrix, nk x round4(len); X of the source
// starts at tree position src_off.
struct LeafBlock {
  int32_t x0;
  int32_t src_off;
  int32_t len;
  int32_t src;
};

// Work buffers of the tensor-core form (32 right-hand sides, FP32):
// xt: 32 * N floats, X in tree order, x(t, c) at xt[c N + t]; t: 32 * sum of
// round4(rank) floats, pair p's T_p (c, l) at t[tc_toff[p] + c tc_tld[p] + l],
// zero padded (grouped by target box: FarOp::tc_*); both in the
// split-exact TF32 form.  p: 32 * part_total floats;
// ynl: 32 * N doubles;
// err: device flag, 1 when an mbarrier wait gave up, 2 when a block's table
// exceeded tc_max_entries().
struct TcBuffers {
  float* xt;
  float* t;
  int64_t lo_off;  // the low parts of X and T, lo_off floats after them
  int ta_split;    // blocks per slice of the T kernel (0: the default rule)
  float* p;
  double* ynl;
  int* err;
  const int32_t* upper_pairs;
  int64_t n_upper;
  int max_slice;
  // leaf rows: per leaf its dense blocks (near field, then the leaf-level
  // interaction list) blocks[block_ptr[k] .. block_ptr[k + 1])
  const LeafBlock* blocks;
  const int32_t* block_ptr;
  // 2D tensor maps (CUtensorMap, 128 bytes each) of the FP32 operands A,
  // 128-byte swizzle, zero fill; boxes of all levels numbered together:
  // umaps[b]: the U of the pairs of target box b side by side, as n x R_b
  // (FarOp::tc_rbox), box 32 x 128; vmaps[b]: the V of the pairs whose source
  // is box b, stacked in the order of its reverse list, as (sum of ranks) x
  // round4(m), box 32 x 128; rmaps[k]: leaf k's row matrix, nk x W_k, box
  // 32 x 64.
  const void* umaps;
  const void* vmaps;
  const void* rmaps;
};

// Tensor-core mixed-precision product A X for 1..32 right-hand sides (zero
// padded to 32); leaves of at most 64 points whose populations are multiples of 4
// (16-byte aligned operand rows).  Returns the number of launches.
int launch_matvec_tc(cudaStream_t s, int64_t N, const int32_t* perm, const FarOp& far,
                     const NearOp& near, const TcBuffers& B, const double* X, int64_t ldx,
                     double* Y, int64_t ldy, int nrhs, MatvecProfiler* prof);
// Largest number of table entries (pairs of all levels a block multiplies)
// one tensor-core block takes.
int tc_max_entries();
// Largest number of dense blocks in one leaf row of the tensor-core engine.
int tc_max_row_blocks();
// Test hook: the next T-kernel launch's block (0, 0) stops copying before
// chunk `chunk` (-1: off), so that its bounded waits give up.
cudaError_t tc_set_drop_chunk(int chunk);
// Evaluates the dense FP32 blocks of the leaf rows (split-exact form): block
// i of leaf k at column blocks[block_ptr[k] + i].x0 of the nk x row_ld[k]
// row-major matrix at Krow + row_base[k]; max_blocks = the largest count.
int launch_row_blocks(cudaStream_t s, int64_t nleaf, int max_blocks, const int32_t* leaf_off,
                      const NearOp& near, const LeafBlock* blocks, const int32_t* block_ptr,
                      const int64_t* row_base, const int32_t* row_ld, float* Krow);
// Evaluates the FP32 near-field blocks of every leaf: block (k, slot) (slots
// 0..25 the neighbours, 26 the leaf itself) is nk x round4(ne) at
// near_off[27 k + slot] with row stride near_ld[k] (the blocks of a leaf side
// by side in one row-major matrix).
int launch_near_blocks(cudaStream_t s, int64_t nleaf, const int32_t* leaf_off, const NearOp& near,
                       const int64_t* near_off, const int32_t* near_ld, float* Knear);

// The few-column form (matvec_gemv.cu): 1, 2, 4 or 8 right-hand sides, A X
// or A^T X, from the box-grouped FP32 factors and near-field blocks.
constexpr int kGemvCols = 1024;     // columns of a V-stack chunk (forward)
constexpr int kGemvRowChunk = 2048;  // V-stack rows per forward work item
constexpr int kGemvRowsT = 256;     // U rows per transposed work item

struct GemvOp {
  int levels;
  int max_leaf4;              // round4 of the largest leaf population
  int64_t nleaf;
  int64_t N;
  const int32_t* leaf_off;
  const int32_t* perm;
  const int32_t* nbr_leaf;    // nleaf x 26
  const float* u32;           // grouped FP32 U pool
  const float* v32;           // grouped FP32 V pool
  const int64_t* ubox_off;    // per box: U_b at u32 + ubox_off[b], n_b x rbox[b]
  const int32_t* rbox;
  const int64_t* vbox_off;    // per box: V stack at v32 + vbox_off[a], vbox_rows[a] x round4(m_a)
  const int32_t* vbox_rows;
  const int64_t* vrow0;       // per box: first row of its V stack in the global row numbering
  const int32_t* vrow_t;      // per global V-stack row: its row of T
  const int32_t* trow_v;      // per row of T: its global V-stack row, -1 for padding
  const int64_t* tbase;       // per box: first row of its T (R_b rows)
  const int64_t* vpofs;       // per box: chunk partials of its V stack (floats / NR), -1 when one chunk
  const int64_t* upofs;       // per box: chunk partials of its U^T X (floats / NR), -1 when one chunk
  const float* knear;         // FP32 near-field blocks (launch_near_blocks)
  const float* u32lo;         // fp64x: lo parts (FP64 value - FP32 copy), same layouts
  const float* v32lo;
  const float* knearlo;
  const int64_t* near_base;   // per leaf: its blocks side by side, nk x near_ld[k] row-major
  const int32_t* near_ld;
  const int64_t* near_off;    // 27 per leaf: start of each block (column near_off - near_base), -1 absent
};

// Work buffers: xg N x 8 floats; t: T rows x 8 floats (zeroed once: its
// padding rows are never written); tt: V-stack rows x 8 floats (the
// transposed T in stack order); p, pt: chunk partials x 8 floats.  The fp64x
// form (4 columns) adds the lo parts xl, tl (zeroed once), ttl and the chunk
// partials as FP32 pairs pd, ptd.
// Work lists: vt_items (source box, chunk, first row, rows); vt_upper: boxes
// with chunk partials; ut_items (target box, row chunk); ut_upper likewise.
struct GemvBuffers {
  float* xg;
  float* t;
  float* tt;
  float* p;
  float* pt;
  float* xl;
  float* tl;
  float* ttl;
  double* pd;
  double* ptd;
  const int4* vt_items;
  int64_t n_vt_items;
  const int32_t* vt_upper;
  int64_t n_vt_upper;
  const int2* ut_items;
  int64_t n_ut_items;
  const int32_t* ut_upper;
  int64_t n_ut_upper;
};

// Largest dynamic shared memory a few-column launch of nr (<= 4 or <= 8)
// columns asks for.
size_t gemv_smem_bytes(int max_leaf4, int nr, bool fp64x);
// nrhs in 1..8 (fp64x: 1..4, the FP64-accurate form from the FP32 pairs).
// Returns the number of launches (0: nrhs out of range).
int launch_matvec_gemv(cudaStream_t s, const GemvOp& op, const GemvBuffers& B, const double* X,
                       int64_t ldx, double* Y, int64_t ldy, int nrhs, bool trans, bool fp64x,
                       MatvecProfiler* prof);
// The FP64 form streamed (matvec_f64.cu): one right-hand side per pass over
// FP64 copies of the factors grouped exactly like the FP32 ones (the same
// element offsets, so GemvOp's tables serve; its float pointers are unused)
// and FP64 near-field blocks in the near-field layout.  Work buffers: xg N,
// t the rows of T (zeroed once: padding rows are never written), tt the
// V-stack rows, p / pt the chunk partials, all FP64.
struct F64Buffers {
  const double* u64;
  const double* v64;
  const double* knear64;
  double* xg;
  double* t;
  double* tt;
  double* p;
  double* pt;
  const int4* vt_items;
  int64_t n_vt_items;
  const int32_t* vt_upper;
  int64_t n_vt_upper;
  const int2* ut_items;
  int64_t n_ut_items;
  const int32_t* ut_upper;
  int64_t n_ut_upper;
};
size_t f64_smem_bytes(int max_leaf4);
// y = A x (trans: A^T x) for one column, device pointers; returns the launches.
int launch_matvec_f64(cudaStream_t s, const GemvOp& op, const F64Buffers& B, const double* x,
                      double* y, bool trans, MatvecProfiler* prof);
// FP64 grouped copies of every pair's U (row stride us[p], zeros up to
// round4(r)) and V (leading dimension round4(m)) at ug[p], vg[p].
int launch_group_f64(cudaStream_t s, int64_t npairs, const double* const* u64, double* const* ug,
                     const int32_t* nsize, const int32_t* us, const double* const* v64,
                     double* const* vg, const int32_t* msize, const int32_t* rank);
// FP64 near-field blocks (the FP64 form's entries) in the near-field layout.
int launch_near64(cudaStream_t s, int64_t nleaf, const int32_t* leaf_off, const NearOp& near,
                  const int64_t* near_off, const int32_t* near_ld, double* Knear64);

// fp64x: lo parts of the near-field blocks, knearlo = K (FP64, as the FP64
// near field evaluates it) - Knear, same layout.
int launch_near_lo(cudaStream_t s, int64_t nleaf, const int32_t* leaf_off, const NearOp& near,
                   const int64_t* near_off, const int32_t* near_ld, const float* Knear,
                   float* Knearlo);

// precision: 0 = FP64, 1 = mixed.  X, Y column-major in the original order.
// Returns the number of kernel launches.
int launch_matvec(cudaStream_t s, int64_t N, const int32_t* perm, const FarOp& far,
                  const NearOp& near, const MatvecBuffers& B, const double* X, int64_t ldx,
                  double* Y, int64_t ldy, int nrhs, int precision, int trans,
                  MatvecProfiler* prof);

// out[c * rows + r] = in[r * cols + c] (rows x cols row-major -> column-major)
void launch_transpose(cudaStream_t s, const double* in, int64_t rows, int64_t cols, double* out);

void launch_dense_rows(cudaStream_t s, int64_t N, const double* xyz, KernelDesc kd,
                       const int64_t* rows, int64_t nrows, const double* X, int64_t ldx,
                       double* Y, int nrhs);

// out[e] = K(rc[e], rc[n + e]) for e < n (device arrays), FP64
void launch_entries(cudaStream_t s, int64_t N, const double* xyz, KernelDesc kd, const int64_t* rc,
                    int64_t n, double* out);

}  // namespace h3d
