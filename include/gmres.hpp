// C++ drop-in facade of the reference's classGMRES (include/gmres.hpp:13-26 of
// SAFRAN-LAB/HODLR3D) over the hodlr3d_gb300 C ABI.  Header only.
//
// gmres(M, b, maxIterations, threshold, x, error, noOfIterations, e) keeps
// the reference's signature and semantics (unrestarted GMRES from x0 = 0,
// modified Gram-Schmidt, Givens rotations, e = residual estimates starting
// with 1); the Krylov vectors live on the GPU.  Vec needs data(), size(),
// resize().
#ifndef HODLR3D_GB300_GMRES_FACADE_HPP
#define HODLR3D_GB300_GMRES_FACADE_HPP

#include <cuda_runtime.h>

#include <vector>

#include "HODLR3D.hpp"

class classGMRES {
 public:
  classGMRES() {}

  template <class Vec>
  void gmres(HODLR3D* M, Vec b, int maxIterations, double threshold, Vec& x, double& error,
             int& noOfIterations, std::vector<double>& e) {
    const int n = M->N;
    double *db = nullptr, *dx = nullptr;
    if (cudaMalloc(&db, sizeof(double) * n) != cudaSuccess ||
        cudaMalloc(&dx, sizeof(double) * n) != cudaSuccess) {
      cudaFree(db);
      throw hodlr3d_gb300::Error(HODLR3D_ERR_OUT_OF_MEMORY, "device vectors for GMRES");
    }
    cudaMemcpy(db, b.data(), sizeof(double) * n, cudaMemcpyHostToDevice);
    hodlr3d_gmres_params prm{};
    prm.maxit = maxIterations;
    prm.restart = 0;
    prm.tol = threshold;
    prm.precision = HODLR3D_FP64;
    hodlr3d_gmres_result res{};
    std::vector<double> hist(maxIterations + 1);
    int nh = 0;
    const int code = hodlr3d_gmres(M->handle(), db, dx, 1, n, &prm, &res, hist.data(),
                                   (int)hist.size(), &nh, nullptr);
    x.resize(n);
    cudaMemcpy(x.data(), dx, sizeof(double) * n, cudaMemcpyDeviceToHost);
    cudaFree(db);
    cudaFree(dx);
    if (code != HODLR3D_OK && code != HODLR3D_ERR_NO_CONVERGENCE) hodlr3d_gb300::check(code);
    error = res.rel_residual;
    noOfIterations = res.iterations;
    e.assign(hist.begin(), hist.begin() + nh);
  }
};

#endif
