/* CPU restatement of the HODLR3D reference algorithm (tree, interaction
 * lists, partially pivoted ACA, matvec, GMRES, dense direct sum).
 *
 * TEST INFRASTRUCTURE ONLY.  This is the oracle: the parity tests, the smoke
 * check and the CPU-baseline leg of the benchmark check the CUDA path
 * against it.  The product (hodlr3d_gb300) never links or calls it.
 *
 * It is pinned against the reference's own sources compiled here (see
 * oracle/Makefile.ref and tests/golden/make_golden.py).
 */
#ifndef HODLR3D_ORACLE_H
#define HODLR3D_ORACLE_H
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_problem orc_problem;

/* Builds the kernel and the uniform octree (reference HODLR3D::HODLR3D,
 * src/HODLR3D.cpp:3-15).  xyz is N x 3 interleaved.  diag_override: NaN to
 * keep the reference diagonal (Kii for kernel 16, 0 otherwise). */
orc_problem* orc_create(const double* xyz, int64_t N, int nP1D, double L, int tol_pow,
                        int kernel_id, double diag_override);
void orc_destroy(orc_problem* p);
void orc_set_threads(int n);

int orc_levels(const orc_problem* p);
double orc_kii(const orc_problem* p);
double orc_entry(const orc_problem* p, int64_t i, int64_t j);
/* leaf order: perm[t] = original index of the t-th point in tree order */
void orc_perm(const orc_problem* p, int32_t* perm);
/* offsets of the boxes of level j in tree order: 8^j + 1 values */
void orc_box_offsets(const orc_problem* p, int level, int64_t* off);
/* neighbour slots of every box at level j: 8^j x 26 (-1 = none) */
void orc_neighbors(const orc_problem* p, int level, int32_t* nbr);
/* number of interaction-list pairs over levels 1..nLevels */
int64_t orc_num_pairs(const orc_problem* p);
/* pair table in (level, target, source ascending) order: 3 ints per pair */
void orc_pairs(const orc_problem* p, int32_t* level_tgt_src);

/* Lean storage for later assemblies: pivots and the r x r L, R only (the
 * reference's storage, include/HODLR3DTree.hpp:20-21); the residual-vector
 * forms (orc_pair_factors, orc_matvec_uv, orc_matvec_uv_t) then refuse. */
void orc_set_lean(orc_problem* p, int lean);
int orc_is_lean(const orc_problem* p);
/* ACA of every pair (reference HODLR3DTree::getUVtTree, src/HODLR3DTree.cpp:1621-1645).
 * Selection (optional, n_sel > 0): assemble only the pairs whose target box is
 * one of the listed (level, box) targets. */
int orc_assemble(orc_problem* p, const int32_t* sel_level, const int32_t* sel_box, int n_sel);
void orc_ranks(const orc_problem* p, int32_t* rank);
int64_t orc_total_pivots(const orc_problem* p);
/* global ids of row / column pivots, concatenated in pair order */
void orc_pivots(const orc_problem* p, int32_t* rows, int32_t* cols);
/* U (n x r) and V (m x r) column-major of one pair (ACA residual vectors) */
void orc_pair_factors(const orc_problem* p, int64_t pair, double* U, double* V);

/* y = A x (reference HODLR3D::MatVecProduct, src/HODLR3D.cpp:21-27) in the
 * reference's CUR form: Ac R^-1 L^-1 Ar x with Ac, Ar re-evaluated.
 * Selection (optional, n_sel > 0): evaluate only the far field of the listed
 * (level, box) targets and the near field of the listed leaf boxes. */
void orc_matvec(const orc_problem* p, const double* x, double* y, const int32_t* sel_level,
                const int32_t* sel_box, int n_sel);
/* y = A x with the stored ACA factors, U (V^T x). */
void orc_matvec_uv(const orc_problem* p, const double* x, double* y);
/* y = A^T x with the stored ACA factors, V (U^T x), and the near field transposed. */
void orc_matvec_uv_t(const orc_problem* p, const double* x, double* y);
/* y[r] = sum_j K(rows[r], j) x[j], the dense FP64 product (reference
 * kernel::getCol, src/kernel.cpp:27-35, summed over columns) */
void orc_dense_rows(const orc_problem* p, const int64_t* rows, int64_t nrows, const double* x,
                    double* y);
/* Unrestarted GMRES from x0 = 0 (reference classGMRES::gmres, src/gmres.cpp:40-94).
 * hist must hold maxit + 1 values; returns the iteration count. */
int orc_gmres(const orc_problem* p, const double* b, int maxit, double tol, double* x,
              double* hist, int* nhist);
/* entries of the ACA factors held: the reference's findMemory count
 * (src/HODLR3DTree.cpp:1757-1778), and the largest rank (getMaxRank, :1807-1818) */
double orc_memory_entries(const orc_problem* p);
int orc_max_rank(const orc_problem* p);

#ifdef __cplusplus
}
#endif
#endif
