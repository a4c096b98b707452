// C++ drop-in facade of the reference's HODLR3D class (include/HODLR3D.hpp:12-21
// of SAFRAN-LAB/HODLR3D) over the hodlr3d_gb300 C ABI.  Header only.
//
// The reference's constructor, assemble() and MatVecProduct(b, Ab) keep their
// signatures; the vector type is a template parameter so Eigen::VectorXd (or
// std::vector<double>) works unchanged: it needs data(), size() and resize().
// The members the reference's drivers read keep their names: N, mykernel
// (userkernel*, include/kernel.hpp here), A->N, A->K, A->assTime,
// A->matVecTime, A->findMemory, A->getMaxRank (examples/testHODLR3D.cpp:107-153).
// The device evaluates the built-in formula of Qchoice (src/kernel.cpp:65-227;
// every Qchoice 0-16 runs on the GPU); the constructor checks on sampled
// entries that mykernel->getMatrixEntry -- the header's dispatch, or the
// application's own definition -- is that kernel, and throws otherwise.
// Errors are thrown as hodlr3d_gb300::Error (the reference has no error path).
#ifndef HODLR3D_GB300_FACADE_HPP
#define HODLR3D_GB300_FACADE_HPP

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <stdexcept>
#include <memory>
#include <string>
#include <vector>

#include "hodlr3d.h"
#include "kernel.hpp"

namespace hodlr3d_gb300 {

struct Error : std::runtime_error {
  int code;
  Error(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

inline void check(int code) {
  if (code != HODLR3D_OK) throw Error(code, hodlr3d_last_error());
}

inline double device_entry(hodlr3d_t h, int64_t i, int64_t j) {
  double v = NAN;
  check(hodlr3d_entries(h, &i, &j, 1, &v));
  return v;
}

// What the reference drivers read from the tree (HODLR3DTree,
// include/HODLR3DTree.hpp:24-60): N, the kernel K, the timers, findMemory,
// getMaxRank.
struct TreeView {
  hodlr3d_t h = nullptr;
  int N = 0;
  userkernel* K = nullptr;
  // the reference's split of a matvec: assTime, the kernel evaluations of
  // the far-field factors and near blocks (zero here: the factors are
  // stored and the near field is part of the product's kernels), and
  // matVecTime, the product itself (wall clock of the last MatVecProduct,
  // copies included)
  double assTime = 0.0;
  double matVecTime = 0.0;
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
  userkernel* mykernel = nullptr;  // the reference's kernel object (also A->K)
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
    tree.N = N;
    A = &tree;
    try {
      mykernel = new userkernel(particles, Qchoice);
      mykernel->diag_override = diag_override;
      tree.K = mykernel;
      check_kernel();
    } catch (...) {
      delete mykernel;
      hodlr3d_destroy(h);
      throw;
    }
  }
  HODLR3D(const HODLR3D&) = delete;
  HODLR3D& operator=(const HODLR3D&) = delete;
  ~HODLR3D() {
    hodlr3d_destroy(tree.h);
    delete mykernel;
  }

  // mykernel->getMatrixEntry against the entries the device evaluates, on
  // the diagonal and on pseudo-random pairs: an application whose own
  // getMatrixEntry is not the device's kernel is refused (the GPU cannot
  // run host code).  Agreement within 1e-12 of the largest sampled entry
  // (host and device math libraries differ in the last bits for the
  // transcendental kernels).
  void check_kernel(int samples = 64) {
    if (N < 1) return;
    std::vector<int64_t> r, c;
    uint64_t st = 0x9E3779B97F4A7C15ull;
    for (int s = 0; s < samples; ++s) {
      st = st * 6364136223846793005ull + 1442695040888963407ull;
      const int64_t i = (int64_t)((st >> 33) % (uint64_t)N);
      st = st * 6364136223846793005ull + 1442695040888963407ull;
      const int64_t j = s < 4 ? i : (int64_t)((st >> 33) % (uint64_t)N);
      r.push_back(i);
      c.push_back(j);
    }
    std::vector<double> dev(r.size());
    hodlr3d_gb300::check(hodlr3d_entries(tree.h, r.data(), c.data(), (int64_t)r.size(), dev.data()));
    double scale = 0.0, worst = 0.0;
    int64_t wi = 0, wj = 0;
    std::vector<double> host(r.size());
    for (size_t e = 0; e < r.size(); ++e) {
      host[e] = mykernel->getMatrixEntry((unsigned)r[e], (unsigned)c[e]);
      scale = std::max(scale, std::max(std::fabs(host[e]), std::fabs(dev[e])));
    }
    for (size_t e = 0; e < r.size(); ++e) {
      const double d = std::fabs(host[e] - dev[e]);
      if (!(d <= worst)) {
        worst = d;
        wi = r[e];
        wj = c[e];
      }
    }
    if (!(worst <= 1e-12 * scale))
      throw hodlr3d_gb300::Error(
          HODLR3D_ERR_UNSUPPORTED,
          "getMatrixEntry(" + std::to_string(wi) + ", " + std::to_string(wj) + ") = " +
              std::to_string(mykernel->getMatrixEntry((unsigned)wi, (unsigned)wj)) +
              " is not the device's kernel for this Qchoice (" +
              std::to_string(hodlr3d_gb300::device_entry(tree.h, wi, wj)) +
              "); give the diagonal through diag_override, or add the kernel to the device");
  }

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
    const auto t0 = std::chrono::steady_clock::now();
    AFMM_Ab.resize(N);
    hodlr3d_gb300::check(hodlr3d_matvec_host(tree.h, b.data(), AFMM_Ab.data(), 1, N, precision));
    tree.matVecTime = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  }

  hodlr3d_t handle() const { return tree.h; }

 private:
  explicit HODLR3D(hodlr3d_t h) {
    hodlr3d_stats st;
    hodlr3d_gb300::check(hodlr3d_get_stats(h, &st));
    N = (int)st.n_points;
    tree.h = h;
    tree.N = N;
    A = &tree;
  }
};

#endif
