// Harness around the HODLR3D reference sources, compiled against the
// project-written API shim in oracle/shim.  Test infrastructure only: it runs
// the reference's own tree build, ACA assembly, matvec and GMRES on a point
// set read from disk and dumps every intermediate that parity tests compare
// against (tree keys, leaf order, neighbour slots, interaction lists, ACA
// ranks and pivots, the matvec, the GMRES history).
//
// It plays the role of the application translation unit of the reference:
// the reference declares userkernel::getMatrixEntry (include/kernel.hpp:112)
// and leaves its definition to the application; the definition below is the
// dispatch of examples/testHODLR3Dsolve.cpp:32-75 (diagonal 0 unless
// Qchoice == 16), plus an optional diagonal override used by the exp(-r)
// workload (diagonal 1).
//
// usage: hodlr3d_ref <in_dir> <out_dir> <nP1D> <L> <TOL_POW> <Qchoice>
//                    <diag_override|nan> <gmres_maxit> <gmres_tol>
// in_dir holds points.f64 (N x 3, xyz interleaved) and charges.f64 (N).
#include <bits/stdc++.h>
#include <Eigen/Dense>
#include "definitions.hpp"
#include "kernel.hpp"
#include "ACA.hpp"
#include "HODLR3DTree.hpp"
#include "HODLR3D.hpp"
#include "gmres.hpp"

static double g_diag_override = NAN;

double userkernel::getMatrixEntry(const unsigned i, const unsigned j) {
  if (i == j && !std::isnan(g_diag_override)) return g_diag_override;
  if (Qchoice != 16) {
    if (i == j) return 0.0;
    switch (Qchoice) {
      case 0: return RBF_Logarithm(i, j);
      case 1: return RBF_Exponential(i, j);
      case 2: return RBF_Inverse_Quadric(i, j);
      case 3: return RBF_Quadric(i, j);
      case 4: return RBF_Inverse_Multi_Quadric(i, j);
      case 5: return RBF_Gaussian(i, j);
      case 6: return RBF_Multi_quadric(i, j);
      case 7: return Laplacian_3D(i, j);
      case 8: return oneOverR4(i, j);
      case 9: return Laplacian_2D(i, j);
      case 10: return RBF_spline(i, j);
      case 11: return kernel_besselJ(i, j);
      case 12: return kernel_besselY(i, j);
      case 13: return Helmholtz_cos(i, j);
      case 14: return Feynman(i, j);
      case 15: return Yukawa(i, j);
    }
    return 0.0;
  }
  return IE_CUBE_3D(i, j);
}

template <class T>
static std::vector<T> read_all(const std::string& path) {
  std::ifstream f(path, std::ios::binary);
  if (!f) { fprintf(stderr, "cannot open %s\n", path.c_str()); exit(2); }
  f.seekg(0, std::ios::end);
  size_t bytes = f.tellg();
  f.seekg(0);
  std::vector<T> v(bytes / sizeof(T));
  f.read(reinterpret_cast<char*>(v.data()), bytes);
  return v;
}

template <class T>
static void write_all(const std::string& path, const std::vector<T>& v) {
  std::ofstream f(path, std::ios::binary);
  f.write(reinterpret_cast<const char*>(v.data()), v.size() * sizeof(T));
}

static double now() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

int main(int argc, char** argv) {
  if (argc < 10) {
    fprintf(stderr, "usage: %s in_dir out_dir nP1D L TOL_POW Qchoice diag gmres_maxit gmres_tol\n", argv[0]);
    return 2;
  }
  std::string in = argv[1], out = argv[2];
  int nP1D = atoi(argv[3]);
  double L = atof(argv[4]);
  int TOL_POW = atoi(argv[5]);
  int Qchoice = atoi(argv[6]);
  g_diag_override = strcmp(argv[7], "nan") == 0 ? NAN : atof(argv[7]);
  int gmres_maxit = atoi(argv[8]);
  double gmres_tol = atof(argv[9]);

  std::vector<double> xyz = read_all<double>(in + "/points.f64");
  std::vector<double> q = read_all<double>(in + "/charges.f64");
  const int N = (int)(xyz.size() / 3);
  std::vector<pts3D> particles(N);
  for (int i = 0; i < N; ++i) particles[i] = {xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2]};

  std::vector<double> times;
  double t0 = now();
  HODLR3D* H = new HODLR3D(nP1D, L, TOL_POW, Qchoice, particles);
  double t1 = now();
  H->assemble();
  double t2 = now();
  times.push_back(t1 - t0);
  times.push_back(t2 - t1);

  HODLR3DTree* T = H->A;
  const int nLevels = T->nLevels;
  // ---- tree dump --------------------------------------------------------
  std::vector<int> meta = {N, nLevels};
  write_all(out + "/meta.i32", meta);
  std::vector<double> kii = {H->mykernel->Kii, H->mykernel->h3};
  write_all(out + "/kii.f64", kii);
  // leaf order (concatenation of leaf chargeLocations) and leaf sizes
  std::vector<int> perm, leaf_count;
  for (int k = 0; k < T->nBoxesPerLevel[nLevels]; ++k) {
    const auto& cl = T->tree[nLevels][k].chargeLocations;
    perm.insert(perm.end(), cl.begin(), cl.end());
    leaf_count.push_back((int)cl.size());
  }
  write_all(out + "/perm.i32", perm);
  write_all(out + "/leaf_count.i32", leaf_count);
  // per level: centres, neighbour slots, interaction lists (CSR), ACA output
  std::vector<double> centers;
  std::vector<int> nbr, il_ptr, il_idx, il_level, il_box;
  std::vector<int> rank, piv_ptr, row_piv, col_piv;
  il_ptr.push_back(0);
  piv_ptr.push_back(0);
  for (int j = 0; j <= nLevels; ++j) {
    for (int k = 0; k < T->nBoxesPerLevel[j]; ++k) {
      const HODLR3DBox& b = T->tree[j][k];
      centers.push_back(b.center.x);
      centers.push_back(b.center.y);
      centers.push_back(b.center.z);
      for (int s = 0; s < 26; ++s) nbr.push_back(b.neighborNumbers[s]);
      for (size_t i = 0; i < b.interactionList.size(); ++i) {
        il_idx.push_back(b.interactionList[i]);
        il_level.push_back(j);
        il_box.push_back(k);
        if (j >= 1) {
          rank.push_back((int)b.L[i].cols());
          for (size_t r = 0; r < b.row_basis[i].size(); ++r) {
            row_piv.push_back(b.row_basis[i][r]);
            col_piv.push_back(b.col_basis[i][r]);
          }
        } else {
          rank.push_back(0);
        }
        piv_ptr.push_back((int)row_piv.size());
      }
      il_ptr.push_back((int)il_idx.size());
    }
  }
  write_all(out + "/centers.f64", centers);
  write_all(out + "/nbr.i32", nbr);
  write_all(out + "/il_ptr.i32", il_ptr);
  write_all(out + "/il_idx.i32", il_idx);
  write_all(out + "/il_level.i32", il_level);
  write_all(out + "/il_box.i32", il_box);
  write_all(out + "/rank.i32", rank);
  write_all(out + "/piv_ptr.i32", piv_ptr);
  write_all(out + "/row_piv.i32", row_piv);
  write_all(out + "/col_piv.i32", col_piv);

  // ---- matvec -----------------------------------------------------------
  Eigen::VectorXd b(N), Ab;
  for (int i = 0; i < N; ++i) b(i) = q[i];
  double t3 = now();
  H->MatVecProduct(b, Ab);
  double t4 = now();
  times.push_back(t4 - t3);
  write_all(out + "/matvec.f64", Ab.d);

  // ---- GMRES (optional) -------------------------------------------------
  if (gmres_maxit > 0) {
    classGMRES* G = new classGMRES();  // never deleted, as in the reference driver
    Eigen::VectorXd x;
    double err = 0.0;
    int nit = 0;
    std::vector<double> e;
    double t5 = now();
    G->gmres(H, b, gmres_maxit, gmres_tol, x, err, nit, e);
    double t6 = now();
    times.push_back(t6 - t5);
    write_all(out + "/gmres_x.f64", x.d);
    write_all(out + "/gmres_hist.f64", e);
    std::vector<int> it = {nit};
    write_all(out + "/gmres_nit.i32", it);
  }
  write_all(out + "/times.f64", times);
  double mem = 0.0;
  T->findMemory(mem);
  std::vector<double> stats = {mem, (double)T->getMaxRank()};
  write_all(out + "/stats.f64", stats);
  printf("N=%d levels=%d tree=%.3fs assemble=%.3fs matvec=%.3fs maxrank=%d\n", N, nLevels,
         times[0], times[1], times[2], T->getMaxRank());
  // classGMRES's destructor is declared but never defined by the reference
  // (include/gmres.hpp:25), so the solver object above is leaked on purpose.
  delete H;
  return 0;
}
