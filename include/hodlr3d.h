/* hodlr3d_gb300 -- C ABI of the GB300-native HODLR3D path (tree build, ACA
 * assembly, fast matvec, GMRES) on one GPU.
 *
 * Plain pointers and sizes only.  Every call returns an int status
 * (HODLR3D_OK = 0); nothing aborts.  hodlr3d_last_error() describes the last
 * failure of the calling thread.
 *
 * Each entry point names the reference interface it replaces (paths inside the
 * SAFRAN-LAB/HODLR3D source tree).
 */
#ifndef HODLR3D_GB300_H
#define HODLR3D_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define HODLR3D_ABI_VERSION 3

typedef struct hodlr3d_handle* hodlr3d_t;

enum hodlr3d_status {
  HODLR3D_OK = 0,
  HODLR3D_ERR_INVALID_ARG = 1,   /* bad size, pointer, kernel id or option */
  HODLR3D_ERR_CUDA = 2,          /* a CUDA call failed (message in last_error) */
  HODLR3D_ERR_OUT_OF_MEMORY = 3, /* device or host allocation failed */
  HODLR3D_ERR_NOT_ASSEMBLED = 4, /* matvec / solve before hodlr3d_assemble */
  HODLR3D_ERR_NONFINITE = 5,     /* NaN or Inf met in kernel entries or vectors */
  HODLR3D_ERR_BREAKDOWN = 6,     /* GMRES Arnoldi breakdown (h(k+1,k) == 0) */
  HODLR3D_ERR_NO_CONVERGENCE = 7,/* GMRES stopped at maxit above the tolerance */
  HODLR3D_ERR_UNSUPPORTED = 8,   /* kernel or feature not available on the device */
  HODLR3D_ERR_NO_DEVICE = 9,     /* no usable CUDA device */
  HODLR3D_ERR_IO = 10            /* factor file missing, unreadable, corrupt or not matching */
};

enum hodlr3d_precision {
  HODLR3D_FP64 = 0,  /* FP64 end to end (matches the reference's FP64 matvec) */
  HODLR3D_MIXED = 1, /* FP32 factors and near field, FP64 accumulation across tiles */
  HODLR3D_FP64X = 2  /* FP64-accurate products in FP32-pair arithmetic: every FP64 entry
                        as hi + lo FP32 values (relative error 2^-46), exact FP32 products
                        and compensated sums, FP64 across tiles; needs keep_fp32 and device
                        memory for the lo parts (as much as the FP32 copies), built on first
                        use; without them, or on a tree the few-column kernels do not take:
                        HODLR3D_FP64.
                        Agrees with the FP64 form to ~1e-13 relative. */
};

/* Options of hodlr3d_create; fill with hodlr3d_default_options first. */
typedef struct hodlr3d_options {
  int device;                 /* CUDA device ordinal (0) */
  double diag_override;       /* NaN: the reference diagonal (Kii for kernel 16, else 0) */
  int keep_fp32;              /* also keep FP32 copies of the factors for HODLR3D_MIXED (1) */
  size_t aca_workspace_bytes; /* device workspace for one assembly batch (0: 32 GiB or a
                                 quarter of the free device memory, whichever is less) */
  int rank_cap;               /* first per-pair rank capacity above leaf size (0: 128); a pair
                                 that reaches it runs again with twice the capacity */
} hodlr3d_options;

typedef struct hodlr3d_stats {
  int64_t n_points;
  int levels;               /* octree depth (reference nLevels, src/HODLR3D.cpp:7) */
  int64_t n_pairs;          /* compressed interaction-list pairs, levels 1..levels */
  int64_t n_near_blocks;    /* dense leaf blocks (self + face/edge neighbours) */
  int max_rank;             /* reference HODLR3DTree::getMaxRank */
  int64_t sum_rank;         /* sum of pair ranks */
  double memory_entries;    /* reference HODLR3DTree::findMemory count */
  int64_t factor_entries;   /* sum over pairs of rank * (n + m) */
  int64_t u_entries;        /* sum over pairs of rank * n (target-side factors) */
  int64_t v_entries;        /* sum over pairs of rank * m (source-side factors) */
  int64_t factor_bytes_fp64;
  int64_t factor_bytes_fp32;
  int64_t near_entries;     /* sum over near blocks of n * m */
  double tree_seconds;      /* last hodlr3d_create, device tree + lists */
  double assemble_seconds;  /* last hodlr3d_assemble */
  int aca_batches;          /* assembly batches of the last hodlr3d_assemble */
  double aca_kernel_seconds; /* device time of its ACA kernels (CUDA events) */
  double finish_seconds;    /* FP32 grouping and matvec tables of the last
                               hodlr3d_assemble or hodlr3d_load */
} hodlr3d_stats;

typedef struct hodlr3d_gmres_params {
  int maxit;        /* Krylov iterations (unrestarted) or per cycle when restart > 0 */
  int restart;      /* 0: unrestarted as the reference; m > 0: GMRES(m) */
  double tol;       /* relative residual |r| / |b| to reach */
  int precision;    /* HODLR3D_FP64 (or HODLR3D_FP64X): plain GMRES with products of that
                       form; HODLR3D_MIXED: FP32 inner GMRES(restart) with an FP64-accurate
                       outer residual (HODLR3D_FP64X products; iterative refinement) */
  int max_outer;    /* HODLR3D_MIXED: refinement steps (0: 20) */
  double inner_tol; /* HODLR3D_MIXED: inner relative tolerance (0: 1e-5) */
  int transpose;    /* solve A^T x = b (adjoint) instead of A x = b */
} hodlr3d_gmres_params;

typedef struct hodlr3d_gmres_result {
  int iterations;        /* total Krylov iterations (max over right-hand sides) */
  int outer;             /* refinement steps (mixed) */
  double rel_residual;   /* max over RHS of the final estimate |r| / |b| */
  int converged;         /* all right-hand sides reached tol */
} hodlr3d_gmres_result;

/* ---- life cycle ------------------------------------------------------ */
int hodlr3d_abi_version(void);
void hodlr3d_default_options(hodlr3d_options* opt);
const char* hodlr3d_last_error(void);

/* Builds the kernel and the uniform octree with its neighbour slots and
 * interaction lists on the device.  Replaces HODLR3D::HODLR3D(nParticlesInLeafAlong1D,
 * L, TOL_POW, Qchoice, particles) (include/HODLR3D.hpp:18, src/HODLR3D.cpp:3-15).
 * xyz: host array of n points, x y z interleaved (the reference's pts3D).
 * kernel_id: the reference's Qchoice 0-16 (src/kernel.cpp:65-227), all evaluated on
 * the device (11, 12: J0, Y0 of CUDA's math library; 14: K_{1/2}(r)/sqrt(r) in
 * its closed form sqrt(pi/2) e^{-r} / r). */
int hodlr3d_create(const double* xyz, int64_t n, int nP1D, double L, int tol_pow, int kernel_id,
                   const hodlr3d_options* opt, hodlr3d_t* out);

/* Frees everything (HODLR3D::~HODLR3D, src/HODLR3D.cpp:29-32). */
void hodlr3d_destroy(hodlr3d_t h);

/* Partially pivoted ACA of every interaction-list pair.  Replaces
 * HODLR3D::assemble -> HODLR3DTree::getUVtTree (src/HODLR3D.cpp:17-19,
 * src/HODLR3DTree.cpp:1621-1645, src/ACA.cpp:127-238). */
int hodlr3d_assemble(hodlr3d_t h);

/* Factor persistence (no reference counterpart: the reference re-assembles
 * every run).  hodlr3d_save writes an assembled operator -- parameters,
 * points, ranks, pivots and FP64 factors -- to a versioned binary file with a
 * checksum; hodlr3d_load rebuilds the tree from the saved points, checks that
 * its interaction lists are the saved ones and returns an assembled handle
 * (FP32 copies re-derived) without running ACA.  opt as hodlr3d_create (its
 * diag_override is replaced by the saved diagonal).  HODLR3D_ERR_IO on a
 * missing, truncated, corrupt or mismatching file. */
int hodlr3d_save(hodlr3d_t h, const char* path);
int hodlr3d_load(const char* path, const hodlr3d_options* opt, hodlr3d_t* out);

/* ---- products -------------------------------------------------------- */
/* y = A x for nrhs columns (column-major, leading dimension ld >= n), device
 * pointers, enqueued on `stream` (a cudaStream_t; NULL is the CUDA default
 * stream); the call returns once the work is enqueued.  Calls on one handle
 * share its work buffers and must not overlap in time (as the reference's
 * facade, which is not re-entrant).  Replaces HODLR3D::MatVecProduct(b, Ab)
 * (src/HODLR3D.cpp:21-27).  1 <= nrhs <= 64. */
int hodlr3d_matvec(hodlr3d_t h, const double* x, double* y, int nrhs, int64_t ld, int precision,
                   void* stream);
/* The same product for callers that cannot allocate device memory while they
 * run (a caller held to a memory budget fixed up front, or one whose
 * allocator must not be re-entered from the computing thread).  No
 * counterpart in the reference.  It never allocates: its work buffers come
 * from one fixed 64 MiB device array that every GPU loading the library holds
 * until exit, and sizes needing more are refused with HODLR3D_ERR_INVALID_ARG.
 * The first call on a device looks the array's address up (make it before
 * any stream capture).  All calls share the array, so calls that overlap on
 * the GPU race.  It runs the CUDA-core kernels only: HODLR3D_FP64X is
 * computed in the FP64 form.  Device pointers, enqueued on `stream`. */
int hodlr3d_matvec_noalloc(hodlr3d_t h, const double* x, double* y, int nrhs, int64_t ld,
                           int precision, void* stream);
/* Same with host pointers (pageable or pinned): copies in, multiplies,
 * copies out, synchronises. */
int hodlr3d_matvec_host(hodlr3d_t h, const double* x, double* y, int nrhs, int64_t ld,
                        int precision);
/* Same for host arrays stored by rows: x and y are n x nrhs, element (i, c)
 * at [i * nrhs + c] (the layout of a C-ordered (n, nrhs) array); the GPU
 * reorders them.  No reference counterpart (the reference multiplies one
 * vector at a time). */
int hodlr3d_matvec_host_rows(hodlr3d_t h, const double* x, double* y, int nrhs, int precision);
/* y = A^T x with the transposed operator (V (U^T x) on compressed pairs,
 * transposed near field).  No reference counterpart (the reference has no
 * transpose product); device pointers. */
int hodlr3d_matvec_transpose(hodlr3d_t h, const double* x, double* y, int nrhs, int64_t ld,
                             int precision, void* stream);
/* y[r] = sum_j K(rows[r], j) x[j], the dense FP64 product of sampled rows
 * (the reference drivers' check by columns, kernel::getCol,
 * src/kernel.cpp:27-35; K symmetric).  Device pointers, nrhs columns; y is
 * nrhs x nrows (column c at y + c nrows).  A row id outside [0, n) gives NaN
 * in its outputs (the ids are on the device, so they are checked there). */
int hodlr3d_dense_rows(hodlr3d_t h, const int64_t* rows, int64_t nrows, const double* x,
                       double* y, int nrhs, int64_t ldx, void* stream);

/* out[e] = K(rows[e], cols[e]) for e < n: the matrix entries the device
 * evaluates (the FP64 product's formula for the handle's kernel, its
 * diagonal value where the ids are equal), original point ids, host arrays;
 * synchronous.  The batched counterpart of the reference's
 * userkernel::getMatrixEntry(i, j) (include/kernel.hpp:112; kernel::getRow,
 * getCol, getMatrix gather it, src/kernel.cpp:7-62); the C++ facade uses it
 * to check that an application's own getMatrixEntry is the kernel the device
 * evaluates.  HODLR3D_ERR_INVALID_ARG for an id outside [0, n). */
int hodlr3d_entries(hodlr3d_t h, const int64_t* rows, const int64_t* cols, int64_t n, double* out);
/* The diagonal of kernel 16 for n points: 1 + the integral of 1/(4 pi r)
 * over a point's cell of side h = 1/cbrt(n) (16^3 Gauss-Legendre points on
 * each octant).  Replaces the Kii computation of the reference's userkernel
 * constructor (include/kernel.hpp:43-61, src/Integral3D.cpp:9-43); host only,
 * no device needed. */
int hodlr3d_quadrature_kii(int64_t n, double* kii);
/* ---- solve ----------------------------------------------------------- */
/* GMRES from x0 = 0 for nrhs right-hand sides (device pointers, column-major).
 * Replaces classGMRES::gmres(M, b, maxIterations, threshold, x, error,
 * noOfIterations, e) (include/gmres.hpp:23, src/gmres.cpp:40-94).
 * hist (optional, host, hist_cap values): relative residual estimates of
 * the first right-hand side, as the reference's e vector; *n_hist receives
 * the count.  Waits for `stream` before it starts and returns with x ready. */
int hodlr3d_gmres(hodlr3d_t h, const double* b, double* x, int nrhs, int64_t ld,
                  const hodlr3d_gmres_params* prm, hodlr3d_gmres_result* res, double* hist,
                  int hist_cap, int* n_hist, void* stream);

/* ---- introspection (parity tests, statistics) --------------------------- */
int hodlr3d_get_stats(hodlr3d_t h, hodlr3d_stats* s);
/* perm[t]: original index of the t-th point in tree order (host, n values);
 * leaf_off: 8^levels + 1 offsets of the leaves in tree order (host). */
int hodlr3d_get_tree(hodlr3d_t h, int32_t* perm, int64_t* leaf_off);
/* neighbour slots of every box of one level, 8^level x 26 (host; -1 = none);
 * the reference's HODLR3DBox::neighborNumbers (include/HODLR3DTree.hpp:16). */
int hodlr3d_get_neighbors(hodlr3d_t h, int level, int32_t* nbr);
/* (level, target box, source box) of every pair, sorted (host, 3 x n_pairs);
 * the reference's HODLR3DBox::interactionList (include/HODLR3DTree.hpp:17). */
int hodlr3d_get_pairs(hodlr3d_t h, int32_t* level_tgt_src);
/* per-pair rank (host, n_pairs) and the global ids of the row and column
 * pivots concatenated in pair order (host, sum_rank each); the reference's
 * L[i].cols(), row_basis[i], col_basis[i] (include/HODLR3DTree.hpp:20-21). */
int hodlr3d_get_ranks(hodlr3d_t h, int32_t* rank);
int hodlr3d_get_pivots(hodlr3d_t h, int32_t* rows, int32_t* cols);
/* U (n x r) and V (m x r) FP64 factors of one pair, column-major (host). */
int hodlr3d_get_pair_factors(hodlr3d_t h, int64_t pair, double* U, double* V);
/* number of kernel launches issued by the library since creation */
int64_t hodlr3d_launch_count(hodlr3d_t h);
/* Matvec engine: 0 = automatic (mixed form: the few-column FP32 kernels for
 * A x with 1..4 right-hand sides (1..32 on trees the tensor cores do not
 * take) and A^T x with 1..32, the tensor cores, tcgen05 3xTF32, for A x with
 * more; HODLR3D_FP64X: the few-column kernels; HODLR3D_FP64: the few-column
 * FP64 streaming kernels, one column per pass, over FP64 factors grouped by
 * box (built on first use; where they do not fit in device memory, and
 * otherwise, the CUDA-core kernels), 1 = CUDA-core kernels only
 * (HODLR3D_FP64X becomes HODLR3D_FP64), 2 = tensor cores only, 3 =
 * few-column kernels only (HODLR3D_ERR_UNSUPPORTED where the chosen engine
 * does not apply).  After hodlr3d_autotune the automatic
 * choice of the mixed form follows its timings instead of these rules. */
int hodlr3d_set_engine(hodlr3d_t h, int engine);
/* Autotuner of the automatic engine choice over this operator's own rank
 * histogram: times every engine that runs the mixed-precision product (A x:
 * CUDA cores, tensor cores, few-column kernels; A^T x: CUDA cores and
 * few-column kernels) at 1, 2, 4, 8, 16, 32 and 64 right-hand sides, `reps`
 * timed products each after an untimed one (median), and makes engine 0 use
 * the fastest; a count between two timed ones takes the choice of the next
 * one up.  Blocks the calling thread; allocates two n x 64 work arrays for
 * its duration.  reps = 0 returns to the column-count rules; a new assembly
 * or load does too.  report (optional, cap bytes, NUL-terminated, truncated):
 * one line "transpose nrhs engine ms" per timing, then the launch shapes it
 * times on the tensor-core engine (32 columns): "launch ta_split k ms" for
 * k = 1, 2, 4, 8, 16, 32 blocks per slice of its T kernel and
 * "launch ta_split_chosen k ms" (the results do not depend on k).  No
 * reference counterpart. */
int hodlr3d_autotune(hodlr3d_t h, int reps, char* report, int cap);
/* The automatic choice after hodlr3d_autotune: choice[64 t + nrhs - 1] for
 * t = 0 (A x) and 1 (A^T x), nrhs 1..64; an engine number, or 0 where the
 * column-count rules apply. */
int hodlr3d_get_tuning(hodlr3d_t h, int32_t* choice);
/* Synchronises the device and reports HODLR3D_ERR_CUDA if a bounded
 * tensor-core wait gave up in an earlier call on this handle, then clears
 * that flag (the products of later calls are checked afresh). */
int hodlr3d_device_status(hodlr3d_t h);
/* Testing of the bounded waits: in the next tensor-core product on this
 * handle's device, block (0, 0) of the T kernel copies its chunks only up to
 * chunk `chunk` (one-shot; -1: off).  The chunk's "landed" barrier is never
 * completed, the block's waits give up after about a second each, the block
 * drains its copies and products in flight and frees its tensor memory, and
 * hodlr3d_device_status reports the failure; that product's results are
 * invalid.  No reference counterpart. */
int hodlr3d_test_drop_copy(hodlr3d_t h, int chunk);
/* Per-kernel timing of the matvec launches with CUDA events recorded between
 * them on the launch stream (off by default).  The report lists one line per
 * kernel, "name launches total_ms", accumulated since the last report. */
int hodlr3d_set_profiling(hodlr3d_t h, int enable);
int hodlr3d_profile_report(hodlr3d_t h, char* buf, int cap);

#ifdef __cplusplus
}
#endif
#endif
