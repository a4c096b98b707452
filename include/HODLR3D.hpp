// C++ drop-in facade of the reference's HODLR3D class (include/HODLR3D.hpp:12-21
// of SAFRAN-LAB/HODLR3D) over the hodlr3d_gb300 C ABI.  Header only.
//
// The reference's constructor, assemble() and MatVecProduct(b, Ab) keep their
// signatures; the vector type is a template parameter so Eigen::VectorXd (or
// std::vector<double>) works unchanged: it needs data(), size() and resize().
// The kernel is chosen by Qchoice (src/kernel.cpp:65-227) instead of a
// user-compiled getMatrixEntry; every Qchoice 0-16 runs on the GPU.
// Errors are thrown as hodlr3d_gb300::Error (the reference has no error path).
#ifndef HODLR3D_GB300_FACADE_HPP
#define HODLR3D_GB300_FACADE_HPP

#include <cmath>
#include <cstring>
#include <stdexcept>
#include <memory>
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

struct Error : std::runtime_error {
  int code;
  Error(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

inline void check(int code) {
  if (code != HODLR3D_OK) throw Error(code, hodlr3d_last_error());
}

// Statistics the reference drivers read from the tree (findMemory, getMaxRank).
struct TreeView {
  hodlr3d_t h;
  int nLevels() const {
    hodlr3d_stats s;
    check(hodlr3d_get_stats(h, &s));
    return s.levels;
  }
  void findMemory(double& sum) const {
    hodlr3d_stats s;
    check(hodlr3d_get_stats(h, &s));
    sum = s.memory_entries;
  }
  int getMaxRank() const {
    hodlr3d_stats s;
    check(hodlr3d_get_stats(h, &s));
    return s.max_rank;
  }
};

}  // namespace hodlr3d_gb300

class HODLR3D {
 public:
  hodlr3d_gb300::TreeView tree;  // stands in for the reference's A (HODLR3DTree*)
  hodlr3d_gb300::TreeView* A;
  int N;
  // HODLR3D_MIXED selects the FP32 factors; HODLR3D_FP64X FP64-accurate
  // products in FP32-pair arithmetic
  int precision = HODLR3D_FP64;

  HODLR3D(int nParticlesInLeafAlong1D, double L, int TOL_POW, int Qchoice,
          std::vector<pts3D>& particles, double diag_override = NAN) {
    hodlr3d_options opt;
    hodlr3d_default_options(&opt);
    opt.diag_override = diag_override;
    N = (int)particles.size();
    hodlr3d_t h = nullptr;
    hodlr3d_gb300::check(hodlr3d_create(reinterpret_cast<const double*>(particles.data()), N,
                                        nParticlesInLeafAlong1D, L, TOL_POW, Qchoice, &opt, &h));
    tree.h = h;
    A = &tree;
  }
  HODLR3D(const HODLR3D&) = delete;
  HODLR3D& operator=(const HODLR3D&) = delete;
  ~HODLR3D() { hodlr3d_destroy(tree.h); }

  void assemble() { hodlr3d_gb300::check(hodlr3d_assemble(tree.h)); }

  // Factor files (no reference counterpart): save an assembled operator,
  // or build one from a file without running ACA.
  void save(const std::string& path) const { hodlr3d_gb300::check(hodlr3d_save(tree.h, path.c_str())); }
  static std::unique_ptr<HODLR3D> load(const std::string& path) {
    hodlr3d_t h = nullptr;
    hodlr3d_gb300::check(hodlr3d_load(path.c_str(), nullptr, &h));
    return std::unique_ptr<HODLR3D>(new HODLR3D(h));
  }

  // Engine autotuning for this operator (no reference counterpart): the
  // automatic choice of the mixed form follows the timings; reps = 0 returns
  // to the column-count rules.  Returns the timing table as text.
  std::string autotune(int reps = 3) {
    std::string report(1 << 14, '\0');
    hodlr3d_gb300::check(hodlr3d_autotune(tree.h, reps, &report[0], (int)report.size()));
    report.resize(std::strlen(report.c_str()));
    return report;
  }

  // Ab = A b (host vectors); Ab is resized like the reference's (src/HODLR3DTree.cpp:1782).
  template <class Vec>
  void MatVecProduct(Vec& b, Vec& AFMM_Ab) {
    AFMM_Ab.resize(N);
    hodlr3d_gb300::check(hodlr3d_matvec_host(tree.h, b.data(), AFMM_Ab.data(), 1, N, precision));
  }

  hodlr3d_t handle() const { return tree.h; }

 private:
  explicit HODLR3D(hodlr3d_t h) {
    hodlr3d_stats st;
    hodlr3d_gb300::check(hodlr3d_get_stats(h, &st));
    N = (int)st.n_points;
    tree.h = h;
    A = &tree;
  }
};

#endif
