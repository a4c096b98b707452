// An application that defines userkernel::getMatrixEntry itself, as the
// reference's applications do (include/kernel.hpp:112 leaves it to them;
// examples/testHODLR3D.cpp:33-71 defines it), built against the
// hodlr3d_gb300 C++ facade.
//
//   user_kernel_example <cubeRootN> same    -> the exp(-r) kernel with a unit
//        diagonal (Qchoice 1, diag_override 1): the facade accepts it, and the
//        product matches the dense sum of the kernel's columns; exit 0
//   user_kernel_example <cubeRootN> other   -> exp(-2r), which the device does
//        not evaluate for Qchoice 1: construction throws
//        HODLR3D_ERR_UNSUPPORTED; exit 3
#define HODLR3D_GB300_USER_GETMATRIXENTRY
#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

#include "HODLR3D.hpp"

static bool g_other = false;

double userkernel::getMatrixEntry(const unsigned i, const unsigned j) {
  if (i == j) return 1.0;
  const double r = std::sqrt(R2(i, j));
  return g_other ? std::exp(-2.0 * r) : RBF_Exponential(i, j) + 0.0 * r;
}

int main(int argc, char** argv) {
  const int n = argc > 1 ? atoi(argv[1]) : 16;
  g_other = argc > 2 && std::strcmp(argv[2], "other") == 0;
  std::vector<pts3D> particles;
  for (int j = 0; j < n; ++j)
    for (int k = 0; k < n; ++k)
      for (int i = 0; i < n; ++i)
        particles.push_back({-1.0 + (2.0 * k + 1.0) / n, -1.0 + (2.0 * j + 1.0) / n,
                             -1.0 + (2.0 * i + 1.0) / n});
  HODLR3D* H = nullptr;
  try {
    H = new HODLR3D(4, 1.0, 8, 1, particles, 1.0);
  } catch (const hodlr3d_gb300::Error& e) {
    printf("refused: code=%d %s\n", e.code, e.what());
    return e.code == HODLR3D_ERR_UNSUPPORTED ? 3 : 1;
  }
  H->assemble();
  const int N = H->N;
  std::vector<double> b(N, 0.0), Hb;
  for (int i = 0; i < N; i += 500) b[i] = 1.0;
  H->MatVecProduct(b, Hb);
  hodlr3d_gb300::VectorXd truth = hodlr3d_gb300::VectorXd::Zero(N);
  for (int i = 0; i < N; i += 500) truth += H->mykernel->getCol(i);
  double num = 0.0;
  for (int t = 0; t < N; ++t) num += (truth(t) - Hb[t]) * (truth(t) - Hb[t]);
  const double err = std::sqrt(num) / truth.norm();
  printf("accepted: N=%d matvec_rel_err=%.3e\n", N, err);
  delete H;
  return err < 1e-6 ? 0 : 1;
}
