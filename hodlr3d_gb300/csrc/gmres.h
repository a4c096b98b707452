// Batched GMRES device helpers (gmres.cu).  Each returns the launch count.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "common.cuh"

namespace h3d {

// out[c] = (q[:,c] -= coef[c] u[:,c] if upd) . (self ? q : w)[:,c]; partial
// needs nrhs * 1024 doubles.
int gmres_dot(cudaStream_t s, int64_t N, int nrhs, double* q, const double* u, const double* coef,
              const double* w, int upd, int self, double* partial, double* out, int take_sqrt);
int gmres_scale_copy(cudaStream_t s, int64_t N, int nrhs, const double* x, const double* sc,
                     double* y);
int gmres_sub(cudaStream_t s, int64_t n, const double* a, const double* b, double* y);
int gmres_add(cudaStream_t s, int64_t n, const double* x, double* y);
int gmres_givens(cudaStream_t s, int k, int m, int nrhs, const double* hk, double* H, double* cs,
                 double* sn, double* beta, const double* bnorm, double* err, int* breakdown);
int gmres_solve_update(cudaStream_t s, int64_t N, int nrhs, int m, const double* H,
                       const double* beta, const int* kcol, double* y, const double* Q, int nvec,
                       double* x, int64_t ldx);
int gmres_pack(cudaStream_t s, int64_t N, int nrhs, const double* a, int64_t lda, double* b,
               int64_t ldb);

}  // namespace h3d
