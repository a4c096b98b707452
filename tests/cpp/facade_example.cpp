// The reference's drivers (examples/testHODLR3D.cpp, examples/testHODLR3Dsolve.cpp)
// written against the hodlr3d_gb300 C++ facade: a uniform grid, the matvec
// checked against the dense sum of columns, and the GMRES solve of
// b = K x_true.  Exit status 0 when both meet their tolerances.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <vector>

#include "HODLR3D.hpp"
#include "gmres.hpp"

int main(int argc, char** argv) {
  const int cubeRootN = argc > 1 ? atoi(argv[1]) : 16;
  const int nP1D = 4, TOL_POW = 10, Qchoice = 16;
  const double L = 1.0;
  std::vector<pts3D> particles;
  for (int j = 0; j < cubeRootN; ++j)
    for (int k = 0; k < cubeRootN; ++k)
      for (int i = 0; i < cubeRootN; ++i) {
        const double c = 2.0 / cubeRootN;
        particles.push_back({-L + c * (k + 0.5), -L + c * (j + 0.5), -L + c * (i + 0.5)});
      }
  HODLR3D* H = new HODLR3D(nP1D, L, TOL_POW, Qchoice, particles);
  H->assemble();
  const int N = H->N;
  // b: ones at every 500th point, as the reference drivers (deterministic here)
  std::vector<double> b(N, 0.0), Hb;
  for (int i = 0; i < N; i += 500) b[i] = 1.0;
  H->MatVecProduct(b, Hb);
  // dense check as the reference driver does it (examples/testHODLR3D.cpp:140-147):
  // the sum of the kernel's columns at the ones, from the host kernel object
  hodlr3d_gb300::VectorXd truth = hodlr3d_gb300::VectorXd::Zero(N);
  for (int i = 0; i < N; i += 500) truth = truth + H->mykernel->getCol(i);
  double num = 0.0;
  for (int t = 0; t < N; ++t) num += (truth(t) - Hb[t]) * (truth(t) - Hb[t]);
  const double err = std::sqrt(num) / truth.norm();
  // the same column through the tree's kernel pointer, and the diagonal Kii
  // of the kernel object against the device's entry
  const bool same_kernel = H->A->K == H->mykernel && H->A->N == N &&
                           H->mykernel->Kii == hodlr3d_gb300::device_entry(H->handle(), 0, 0);
  double mem = 0.0;
  H->A->findMemory(mem);
  // solve A x = b_true with x_true = 1
  std::vector<double> xt(N, 1.0), bt, x;
  H->MatVecProduct(xt, bt);
  classGMRES G;
  double gerr = 0.0;
  int nit = 0;
  std::vector<double> e;
  G.gmres(H, bt, 400, 1e-10, x, gerr, nit, e);
  double fe = 0.0, fn = 0.0;
  for (int t = 0; t < N; ++t) {
    fe += (x[t] - 1.0) * (x[t] - 1.0);
    fn += 1.0;
  }
  printf("N=%d matvec_rel_err=%.3e max_rank=%d memory_entries=%.0f gmres_it=%d gmres_res=%.3e fwd_err=%.3e "
         "same_kernel=%d matVecTime=%.3es\n",
         N, err, H->A->getMaxRank(), mem, nit, gerr, std::sqrt(fe / fn), (int)same_kernel,
         H->A->matVecTime);
  // factor file round trip: the loaded operator gives the same product
  const std::string path = std::string(argc > 2 ? argv[2] : "/tmp") + "/facade_example.h3d";
  H->save(path);
  std::unique_ptr<HODLR3D> G2 = HODLR3D::load(path);
  std::vector<double> Hb2;
  G2->MatVecProduct(b, Hb2);
  bool same = Hb2.size() == Hb.size();
  for (int t = 0; same && t < N; ++t) same = Hb2[t] == Hb[t];
  // the FP64-accurate FP32-pair form against the FP64 form
  G2->precision = HODLR3D_FP64X;
  std::vector<double> Hbx;
  G2->MatVecProduct(b, Hbx);
  double dx = 0.0, dn = 0.0;
  for (int t = 0; t < N; ++t) {
    dx += (Hbx[t] - Hb[t]) * (Hbx[t] - Hb[t]);
    dn += Hb[t] * Hb[t];
  }
  std::remove(path.c_str());
  printf("loaded_same=%d fp64x_rel_diff=%.3e\n", (int)same, std::sqrt(dx / dn));
  // engine autotuning: the mixed product under the tuned automatic choice
  const std::string table = G2->autotune(1);
  G2->precision = HODLR3D_MIXED;
  std::vector<double> Hbm;
  G2->MatVecProduct(b, Hbm);
  double dm = 0.0;
  for (int t = 0; t < N; ++t) dm += (Hbm[t] - Hb[t]) * (Hbm[t] - Hb[t]);
  const bool tuned = table.find("transpose nrhs engine ms") == 0 && std::sqrt(dm / dn) < 2e-6;
  printf("autotune_lines=%d mixed_rel_diff=%.3e\n", (int)std::count(table.begin(), table.end(), '\n'),
         std::sqrt(dm / dn));
  const bool ok = err < 1e-8 && gerr <= 1e-10 && std::sqrt(fe / fn) < 1e-8 && same &&
                  std::sqrt(dx / dn) < 1e-12 && tuned && same_kernel && H->A->matVecTime > 0.0;
  delete H;
  return ok ? 0 : 1;
}
