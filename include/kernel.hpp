// C++ drop-in for the reference's matrix-entry classes `kernel` and
// `userkernel` (include/kernel.hpp:12-117 of SAFRAN-LAB/HODLR3D, bodies in
// src/kernel.cpp).  Header only; host code, FP64.
//
// What it keeps:
//   * kernel: `particles`, the virtual getMatrixEntry(i, j), getRow, getCol
//     (by rows and whole), getMatrix (by index lists and by ranges), which
//     gather getMatrixEntry exactly as the reference does (src/kernel.cpp:7-62);
//   * userkernel: `Qchoice`, `Kii`, `h3`, the 16 named formulas the
//     reference's applications dispatch to (IE_CUBE_3D, RBF_Logarithm, ...,
//     Yukawa; src/kernel.cpp:65-227) and getMatrixEntry.
//
// getMatrixEntry: the reference leaves its definition to the application
// (include/kernel.hpp:112, defined in examples/testHODLR3D.cpp:33-71).  Here
// the header defines it as the reference drivers' dispatch (the formula of
// Qchoice, diagonal 0 except Kii for Qchoice 16, or diag_override when set).
// An application that defines its own, as with the reference, defines
// HODLR3D_GB300_USER_GETMATRIXENTRY before including this header and keeps its
// definition `double userkernel::getMatrixEntry(const unsigned i, const
// unsigned j) { ... }` in one of its source files.
//
// The GPU cannot call host code: the device evaluates the built-in formula of
// the handle's Qchoice (plus a diagonal override).  The HODLR3D facade
// therefore compares the application's getMatrixEntry with the device's
// entries (hodlr3d_entries) on sampled pairs when it is constructed, and
// refuses an operator that differs (hodlr3d_gb300::Error,
// HODLR3D_ERR_UNSUPPORTED) rather than compressing another matrix.  A new
// kernel enters the device as a new kernel id: its formula added to the
// entry functions of hodlr3d_gb300/csrc/common.cuh (entry64_offdiag for the
// FP64 forms, entry32_offdiag for the FP32 near field) and accepted by
// kernel_supported() in csrc/setup.cpp, then the same formula here.
//
// Vector types: Eigen::VectorXd / Eigen::MatrixXd when Eigen's headers are
// included first (as in the reference's applications), else the small
// column-major stand-ins below.
#ifndef HODLR3D_GB300_KERNEL_HPP
#define HODLR3D_GB300_KERNEL_HPP

#include <cmath>
#include <stdexcept>
#include <string>
#include <vector>

#include "hodlr3d.h"

#ifndef HODLR3D_GB300_PTS3D
#define HODLR3D_GB300_PTS3D
struct pts3D {  // include/definitions.hpp:7-9
  double x, y, z;
};
#endif

namespace hodlr3d_gb300 {

#if defined(EIGEN_CORE_H) || defined(EIGEN_CORE_MODULE_H)
using VectorXd = Eigen::VectorXd;
using MatrixXd = Eigen::MatrixXd;
#else
// Dense FP64 vector with the parts of Eigen::VectorXd the reference's
// drivers use on kernel results (element access, sums, norm).
class VectorXd {
 public:
  std::vector<double> v;
  VectorXd() {}
  explicit VectorXd(long n) : v((size_t)n, 0.0) {}
  static VectorXd Zero(long n) { return VectorXd(n); }
  long size() const { return (long)v.size(); }
  void resize(long n) { v.assign((size_t)n, 0.0); }
  double* data() { return v.data(); }
  const double* data() const { return v.data(); }
  double& operator()(long i) { return v[(size_t)i]; }
  double operator()(long i) const { return v[(size_t)i]; }
  double& operator[](long i) { return v[(size_t)i]; }
  double operator[](long i) const { return v[(size_t)i]; }
  double norm() const {
    double s = 0.0;
    for (double x : v) s += x * x;
    return std::sqrt(s);
  }
  VectorXd& operator+=(const VectorXd& o) {
    for (size_t i = 0; i < v.size(); ++i) v[i] += o.v[i];
    return *this;
  }
  VectorXd& operator-=(const VectorXd& o) {
    for (size_t i = 0; i < v.size(); ++i) v[i] -= o.v[i];
    return *this;
  }
  friend VectorXd operator+(VectorXd a, const VectorXd& b) { return a += b; }
  friend VectorXd operator-(VectorXd a, const VectorXd& b) { return a -= b; }
};

// Dense FP64 column-major matrix (element access only).
class MatrixXd {
 public:
  long nr = 0, nc = 0;
  std::vector<double> v;
  MatrixXd() {}
  MatrixXd(long r, long c) : nr(r), nc(c), v((size_t)(r * c), 0.0) {}
  long rows() const { return nr; }
  long cols() const { return nc; }
  double* data() { return v.data(); }
  double& operator()(long i, long j) { return v[(size_t)(j * nr + i)]; }
  double operator()(long i, long j) const { return v[(size_t)(j * nr + i)]; }
};
#endif

// The built-in formulas by Qchoice at squared distance R2 > 0 (the
// reference's src/kernel.cpp:76-227; Qchoice 16 is h3 / R, its off-diagonal).
inline double builtin_entry(int q, double R2, double h3) {
  const double R = std::sqrt(R2);
  switch (q) {
    case 0: return std::log(1.0 + R);
    case 1: return std::exp(-R);
    case 2: return 1.0 / (1.0 + R * R);
    case 3: return 1.0 + R * R;
    case 4: return 1.0 / std::sqrt(R * R + 1.0);
    case 5: return std::exp(-(R * R));
    case 6: return std::sqrt(R * R + 1.0);
    case 7: return 1.0 / R;
    case 8: return 1.0 / (R2 * R2);
    case 9: return std::log(R);
    case 10: return R * R * std::log(R);
    case 11: return std::cyl_bessel_j(0.0, R);
    case 12: return std::cyl_neumann(0.0, R);
    case 13: return std::cos(R) / R;
    case 14: return std::cyl_bessel_k(0.5, R) / std::sqrt(R);
    case 15: return std::exp(-50.0 * R) / R;
    case 16: return h3 * (1.0 / R);
  }
  throw std::invalid_argument("Qchoice must be in 0..16, got " + std::to_string(q));
}

}  // namespace hodlr3d_gb300

class kernel {
 public:
  double a = 0.0;
  std::vector<pts3D> particles;

  explicit kernel(std::vector<pts3D>& p) : particles(p) {}
  virtual ~kernel() {}

  // the reference's base class prints a notice and returns 0
  virtual double getMatrixEntry(const unsigned, const unsigned) { return 0.0; }

  hodlr3d_gb300::VectorXd getRow(const int j, std::vector<int> col_indices) {
    hodlr3d_gb300::VectorXd row((long)col_indices.size());
    for (long k = 0; k < (long)col_indices.size(); ++k) row(k) = getMatrixEntry(j, col_indices[k]);
    return row;
  }
  hodlr3d_gb300::VectorXd getCol(const int k, std::vector<int> row_indices) {
    hodlr3d_gb300::VectorXd col((long)row_indices.size());
    for (long j = 0; j < (long)row_indices.size(); ++j) col(j) = getMatrixEntry(row_indices[j], k);
    return col;
  }
  // the whole column k (the reference drivers' dense check)
  hodlr3d_gb300::VectorXd getCol(const int k) {
    hodlr3d_gb300::VectorXd col((long)particles.size());
    for (long j = 0; j < (long)particles.size(); ++j) col(j) = getMatrixEntry((unsigned)j, k);
    return col;
  }
  hodlr3d_gb300::MatrixXd getMatrix(std::vector<int> row_indices, std::vector<int> col_indices) {
    hodlr3d_gb300::MatrixXd m((long)row_indices.size(), (long)col_indices.size());
    for (long j = 0; j < (long)row_indices.size(); ++j)
      for (long k = 0; k < (long)col_indices.size(); ++k)
        m(j, k) = getMatrixEntry(row_indices[j], col_indices[k]);
    return m;
  }
  // rows [row_start, row_end) x columns [col_start, col_end), stored from
  // (0, 0) (the reference writes the block at its global indices,
  // src/kernel.cpp:52-62, which stays inside the matrix only from (0, 0))
  hodlr3d_gb300::MatrixXd getMatrix(int row_start_index, int col_start_index, int row_end_index,
                                    int col_end_index) {
    hodlr3d_gb300::MatrixXd m(row_end_index - row_start_index, col_end_index - col_start_index);
    for (int j = row_start_index; j < row_end_index; ++j)
      for (int k = col_start_index; k < col_end_index; ++k)
        m(j - row_start_index, k - col_start_index) = getMatrixEntry(j, k);
    return m;
  }
};

class userkernel : public kernel {
 public:
  int Qchoice;
  double Kii = 0.0;
  double h3 = 0.0;
  // diagonal value replacing the reference's (Kii for Qchoice 16, else 0)
  // when not NaN; the HODLR3D facade sets it from its diag_override argument
  double diag_override = NAN;

  userkernel(std::vector<pts3D> particles, int Qchoice) : kernel(particles), Qchoice(Qchoice) {
    if (Qchoice == 16) {
      // include/kernel.hpp:43-61: Kii = 1 + the integral of 1/(4 pi r) over a
      // point's cell of side 1/cbrt(N) (the library's quadrature)
      if (hodlr3d_quadrature_kii((int64_t)this->particles.size(), &Kii) != HODLR3D_OK)
        throw std::invalid_argument(hodlr3d_last_error());
      h3 = 1.0 / double(this->particles.size());
    }
  }

  double R2(const unsigned i, const unsigned j) const {
    const pts3D& p = particles[i];
    const pts3D& q = particles[j];
    return (p.x - q.x) * (p.x - q.x) + (p.y - q.y) * (p.y - q.y) + (p.z - q.z) * (p.z - q.z);
  }
  double f(int q, const unsigned i, const unsigned j) const {
    return hodlr3d_gb300::builtin_entry(q, R2(i, j), h3);
  }

  double IE_CUBE_3D(const unsigned i, const unsigned j) { return i == j ? Kii : h3 * Laplacian_3D(i, j); }
  double RBF_Logarithm(const unsigned i, const unsigned j) { return f(0, i, j); }
  double RBF_Exponential(const unsigned i, const unsigned j) { return f(1, i, j); }
  double RBF_Inverse_Quadric(const unsigned i, const unsigned j) { return f(2, i, j); }
  double RBF_Quadric(const unsigned i, const unsigned j) { return f(3, i, j); }
  double RBF_Inverse_Multi_Quadric(const unsigned i, const unsigned j) { return f(4, i, j); }
  double RBF_Gaussian(const unsigned i, const unsigned j) { return f(5, i, j); }
  double RBF_Multi_quadric(const unsigned i, const unsigned j) { return f(6, i, j); }
  double Laplacian_3D(const unsigned i, const unsigned j) { return f(7, i, j); }
  double oneOverR4(const unsigned i, const unsigned j) { return f(8, i, j); }
  double Laplacian_2D(const unsigned i, const unsigned j) { return f(9, i, j); }
  double RBF_spline(const unsigned i, const unsigned j) { return f(10, i, j); }
  double kernel_besselJ(const unsigned i, const unsigned j) { return f(11, i, j); }
  double kernel_besselY(const unsigned i, const unsigned j) { return f(12, i, j); }
  double Helmholtz_cos(const unsigned i, const unsigned j) { return f(13, i, j); }
  double Feynman(const unsigned i, const unsigned j) { return f(14, i, j); }
  double Yukawa(const unsigned i, const unsigned j) { return f(15, i, j); }

  double getMatrixEntry(const unsigned i, const unsigned j) override;
};

#ifndef HODLR3D_GB300_USER_GETMATRIXENTRY
// The dispatch of the reference drivers (examples/testHODLR3Dsolve.cpp:32-75):
// the formula of Qchoice off the diagonal; on it Kii for Qchoice 16, else 0.
inline double userkernel::getMatrixEntry(const unsigned i, const unsigned j) {
  if (i == j && !std::isnan(diag_override)) return diag_override;
  if (Qchoice == 16) return IE_CUBE_3D(i, j);
  if (i == j) return 0.0;
  return f(Qchoice, i, j);
}
#endif

#endif
