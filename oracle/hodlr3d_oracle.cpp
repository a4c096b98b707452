// CPU restatement of the HODLR3D reference algorithm -- TEST INFRASTRUCTURE.
//
// This file is the oracle: a plain C++/OpenMP restatement of the reference
// path (tree, interaction lists, ACA, matvec, GMRES) that the parity tests,
// the smoke check and the CPU-baseline leg of the benchmark compare the CUDA
// product with.  The product never links it.  Every function cites the
// reference file:line it follows.  It is pinned against the reference's own
// sources compiled in this repository's test environment (oracle/Makefile.ref,
// tests/golden/make_golden.py): identical leaf order, neighbour slots,
// interaction-list sets, ACA ranks and pivots, and the matvec to rounding.
//
// Arithmetic is kept free of fused multiply-adds (built with
// -ffp-contract=off).  The ACA's norms and dot products use the canonical
// reduction order of canonical_sum.h (the order of the CUDA kernels); the
// other reductions run sequentially in index order.  Ranks and pivots are
// therefore reproducible bit for bit on every host and on the GPU.
#include "hodlr3d_oracle.h"
#include "canonical_sum.h"

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <numeric>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

constexpr double kPi = 3.1415926535897932384;  // include/definitions.hpp:4

// Gauss-Legendre nodes (ascending) and weights on [-1,1] by Newton iteration
// on the Legendre recurrence (the classical method of e.g. Press et al.,
// "gauleg").  Replaces the tabulated case of
// src/Gauss_Legendre_Nodes_and_Weights.cpp:457-510 (n = 16).
void gauss_legendre(int n, std::vector<double>& x, std::vector<double>& w) {
  x.assign(n, 0.0);
  w.assign(n, 0.0);
  const int m = (n + 1) / 2;
  for (int i = 0; i < m; ++i) {
    long double z = std::cos(kPi * (i + 0.75) / (n + 0.5));
    long double pp = 0.0;
    for (int it = 0; it < 100; ++it) {
      long double p1 = 1.0, p2 = 0.0;
      for (int j = 1; j <= n; ++j) {
        long double p3 = p2;
        p2 = p1;
        p1 = ((2.0L * j - 1.0L) * z * p2 - (j - 1.0L) * p3) / j;
      }
      pp = n * (z * p1 - p2) / (z * z - 1.0L);
      long double z1 = z;
      z = z1 - p1 / pp;
      if (std::fabs((double)(z - z1)) < 1e-19) break;
    }
    x[i] = (double)(-z);
    x[n - 1 - i] = (double)z;
    long double wi = 2.0L / ((1.0L - z * z) * pp * pp);
    w[i] = (double)wi;
    w[n - 1 - i] = (double)wi;
  }
}

// Kii = 8 * int_{[0,h/2]^3} 1/(4 pi r) + 1 with 16^3 tensor Gauss-Legendre
// points: include/kernel.hpp:43-61 and src/Integral3D.cpp:3-43 (the
// accumulator there is uninitialised; it is taken as 0).
double quadrature_kii(int64_t N) {
  const double h = 1.0 / std::cbrt(double(N));
  std::vector<double> nodes, weights;
  gauss_legendre(16, nodes, weights);
  const double a = 0.0, b = h * 0.5;
  const double c = 0.5 * (b - a), l = 0.5 * (b + a);
  double result = 0.0;
  for (int i = 0; i < 16; ++i) {
    const double tx = c * nodes[i] + l;
    for (int j = 0; j < 16; ++j) {
      const double ty = c * nodes[j] + l;
      for (int k = 0; k < 16; ++k) {
        const double tz = c * nodes[k] + l;
        const double f = 1.0 / ((4 * kPi) * std::sqrt(tx * tx + ty * ty + tz * tz));
        result += (weights[i] * weights[j] * weights[k] * f);
      }
    }
  }
  result *= (c * c * c);
  result *= 8;
  return result + 1.0;
}

struct PairFactors {
  int rank = 0;
  std::vector<int32_t> rows, cols;  // local pivot indices
  std::vector<double> U, V;          // n x rank, m x rank (column-major)
  // lean storage (the reference's own, include/HODLR3DTree.hpp:20-21): the
  // r x r factors L(a,b) = U(row_a, b) and R(a,b) = V(col_b, a), row-major,
  // with U and V dropped after the ACA
  std::vector<double> Lm, Rm;
};

}  // namespace

struct orc_problem {
  int64_t N = 0;
  int nP1D = 0;
  double L = 1.0;
  int tol_pow = 0;
  double tol = 0.0;
  int kernel = 16;
  double diag = NAN;
  double Kii = 0.0, h3 = 0.0;
  std::vector<double> x, y, z;  // original order
  int nLevels = 0;
  std::vector<int32_t> perm;                   // tree order -> original id
  std::vector<std::vector<int64_t>> off;       // off[j][k], 8^j + 1 values
  std::vector<std::vector<int32_t>> nbr;       // nbr[j][26 k + s]
  std::vector<std::vector<int64_t>> il_ptr;    // il_ptr[j][k] into pair arrays
  std::vector<int32_t> p_level, p_tgt, p_src;  // pair table
  std::vector<PairFactors> fac;
  bool lean = false;
};

namespace {

// Kernel entry: the dispatch of the application-defined getMatrixEntry
// (examples/testHODLR3Dsolve.cpp:32-75) over the formulas of
// src/kernel.cpp:65-227, with an optional diagonal override.
inline double entry(const orc_problem& p, int64_t i, int64_t j) {
  if (i == j) {
    if (!std::isnan(p.diag)) return p.diag;
    return p.kernel == 16 ? p.Kii : 0.0;
  }
  const double dx = p.x[i] - p.x[j], dy = p.y[i] - p.y[j], dz = p.z[i] - p.z[j];
  const double R2 = dx * dx + dy * dy + dz * dz;
  const double R = std::sqrt(R2);
  switch (p.kernel) {
    case 0: return std::log(1.0 + R / 1.0);
    case 1: return std::exp(-R / 1.0);
    case 2: return 1.0 / (1.0 + (R / 1.0) * (R / 1.0));
    case 3: return 1.0 + (R / 1.0) * (R / 1.0);
    case 4: return 1.0 / std::sqrt((R / 1.0) * (R / 1.0) + 1);
    case 5: return std::exp(-(R / 1.0) * (R / 1.0));
    case 6: return std::sqrt((R / 1.0) * (R / 1.0) + 1);
    case 7: return 1 / R;
    case 8: return 1.0 / (R2 * R2);
    case 9: return std::log(R);
    case 10: return R * R * std::log(R);
    case 11: return std::cyl_bessel_j(0.0, 1.0 * R);
    case 12: return std::cyl_neumann(0.0, 1.0 * R);
    case 13: return std::cos(1.0 * R) / R;
    case 14: return std::cyl_bessel_k(0.5, R) / std::sqrt(R);
    case 15: return std::exp(-50.0 * R) / R;
    case 16: return p.h3 * (1 / R);
  }
  return 0.0;
}

// Child digit -> octant bits, the layout of assign_Center_Location
// (src/HODLR3DTree.cpp:1528-1553): 0:(-,-,-) 1:(+,-,-) 2:(+,+,-) 3:(-,+,-)
// 4:(-,-,+) 5:(+,-,+) 6:(+,+,+) 7:(-,+,+).
constexpr int kDigitX[8] = {0, 1, 1, 0, 0, 1, 1, 0};
constexpr int kDigitY[8] = {0, 0, 1, 1, 0, 0, 1, 1};
constexpr int kDigitZ[8] = {0, 0, 0, 0, 1, 1, 1, 1};

inline int digit_of(int bx, int by, int bz) {
  static const int tab[8] = {0, 1, 3, 2, 4, 5, 7, 6};  // index bx + 2 by + 4 bz
  return tab[bx + 2 * by + 4 * bz];
}

inline void box_coords(int level, int64_t k, int& ix, int& iy, int& iz) {
  ix = iy = iz = 0;
  for (int t = level - 1; t >= 0; --t) {
    const int d = (int)((k >> (3 * t)) & 7);
    ix = 2 * ix + kDigitX[d];
    iy = 2 * iy + kDigitY[d];
    iz = 2 * iz + kDigitZ[d];
  }
}

inline int64_t box_id(int level, int ix, int iy, int iz) {
  int64_t k = 0;
  for (int t = level - 1; t >= 0; --t) {
    const int d = digit_of((ix >> t) & 1, (iy >> t) & 1, (iz >> t) & 1);
    k = 8 * k + d;
  }
  return k;
}

// Tree: depth (src/HODLR3D.cpp:6-7), leaf assignment by recursive octant
// comparison against box centres with ties to the low side
// (assignChargeLocations, src/HODLR3DTree.cpp:1558-1608; centres as in
// assign_Center_Location :1518-1556), stable leaf order, parent ranges as
// concatenations of children (assignNonLeafChargeLocations :1610-1619).
void build_tree(orc_problem& p) {
  const double cubeRootN = std::pow(double(p.N), 1.0 / 3.0);
  p.nLevels = (int)std::ceil(3 * std::log(double(cubeRootN) / p.nP1D) / std::log(8));
  if (p.nLevels < 0) p.nLevels = 0;
  const int d = p.nLevels;
  std::vector<double> radius(d + 1);
  radius[0] = p.L;
  for (int k = 1; k <= d; ++k) radius[k] = 0.5 * radius[k - 1];
  std::vector<int64_t> leaf(p.N);
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < p.N; ++i) {
    double cx = 0.0, cy = 0.0, cz = 0.0;
    int64_t k = 0;
    for (int j = 0; j < d; ++j) {
      const double shift = 0.5 * radius[j];
      const int bz = p.z[i] <= cz ? 0 : 1;
      const int bx = p.x[i] <= cx ? 0 : 1;
      const int by = p.y[i] <= cy ? 0 : 1;
      k = 8 * k + digit_of(bx, by, bz);
      cx = bx ? cx + shift : cx - shift;
      cy = by ? cy + shift : cy - shift;
      cz = bz ? cz + shift : cz - shift;
    }
    leaf[i] = k;
  }
  const int64_t nleaf = int64_t(1) << (3 * d);
  std::vector<int64_t> cnt(nleaf + 1, 0);
  for (int64_t i = 0; i < p.N; ++i) cnt[leaf[i] + 1]++;
  for (int64_t k = 0; k < nleaf; ++k) cnt[k + 1] += cnt[k];
  p.perm.assign(p.N, 0);
  std::vector<int64_t> pos(cnt.begin(), cnt.end() - 1);
  for (int64_t i = 0; i < p.N; ++i) p.perm[pos[leaf[i]]++] = (int32_t)i;  // stable
  p.off.assign(d + 1, {});
  for (int j = 0; j <= d; ++j) {
    const int64_t nb = int64_t(1) << (3 * j);
    const int64_t stride = int64_t(1) << (3 * (d - j));
    p.off[j].resize(nb + 1);
    for (int64_t k = 0; k <= nb; ++k) p.off[j][k] = cnt[k * stride];
  }
}

// Neighbour slots and interaction lists: the geometric content of
// assign_Child0..7_Interaction (src/HODLR3DTree.cpp:111-1490).  The children
// of the parent's near boxes (the parent and its face/edge neighbours; vertex
// slots are never filled, :123-125) are the box's face/edge neighbours (slot
// 9(dz+1)+3(dy+1)+(dx+1), minus one above the centre) or, when not face/edge
// adjacent (vertex-adjacent included), its interaction list.  Lists are kept
// in ascending box order.
void build_lists(orc_problem& p) {
  const int d = p.nLevels;
  p.nbr.assign(d + 1, {});
  p.il_ptr.assign(d + 1, {});
  p.p_level.clear();
  p.p_tgt.clear();
  p.p_src.clear();
  p.nbr[0].assign(26, -1);
  p.il_ptr[0].assign(2, 0);
  int64_t npairs = 0;
  for (int j = 1; j <= d; ++j) {
    const int64_t nb = int64_t(1) << (3 * j);
    const int side = 1 << j, pside = 1 << (j - 1);
    p.nbr[j].assign(nb * 26, -1);
    std::vector<std::vector<int32_t>> il(nb);
#pragma omp parallel for schedule(static)
    for (int64_t k = 0; k < nb; ++k) {
      int ix, iy, iz;
      box_coords(j, k, ix, iy, iz);
      const int px = ix >> 1, py = iy >> 1, pz = iz >> 1;
      for (int ez = -1; ez <= 1; ++ez)
        for (int ey = -1; ey <= 1; ++ey)
          for (int ex = -1; ex <= 1; ++ex) {
            if (ex != 0 && ey != 0 && ez != 0) continue;  // parent's vertex neighbour
            const int qx = px + ex, qy = py + ey, qz = pz + ez;
            if (qx < 0 || qy < 0 || qz < 0 || qx >= pside || qy >= pside || qz >= pside) continue;
            for (int c = 0; c < 8; ++c) {
              const int bx = 2 * qx + kDigitX[c], by = 2 * qy + kDigitY[c], bz = 2 * qz + kDigitZ[c];
              const int dx = bx - ix, dy = by - iy, dz = bz - iz;
              if (dx == 0 && dy == 0 && dz == 0) continue;
              const int64_t b = box_id(j, bx, by, bz);
              const bool adj = std::abs(dx) <= 1 && std::abs(dy) <= 1 && std::abs(dz) <= 1 &&
                               !(dx != 0 && dy != 0 && dz != 0);
              if (adj) {
                int s = 9 * (dz + 1) + 3 * (dy + 1) + (dx + 1);
                if (s > 13) --s;
                p.nbr[j][26 * k + s] = (int32_t)b;
              } else {
                il[k].push_back((int32_t)b);
              }
            }
          }
      std::sort(il[k].begin(), il[k].end());
      (void)side;
    }
    p.il_ptr[j].resize(nb + 1);
    for (int64_t k = 0; k < nb; ++k) {
      p.il_ptr[j][k] = npairs;
      for (int32_t s : il[k]) {
        p.p_level.push_back(j);
        p.p_tgt.push_back((int32_t)k);
        p.p_src.push_back(s);
        ++npairs;
      }
    }
    p.il_ptr[j][nb] = npairs;
  }
  p.fac.assign(npairs, PairFactors());
}

// First index of the largest |v| over the allowed indices
// (LowRank::maxAbsVector, src/ACA.cpp:10-23).  -1 if none is allowed.
inline int argmax_abs(const std::vector<double>& v, const std::vector<char>& used) {
  int idx = -1;
  double mx = 0.0;
  for (size_t s = 0; s < v.size(); ++s) {
    if (used[s]) continue;
    const double a = std::fabs(v[s]);
    if (idx < 0 || a > mx) {
      idx = (int)s;
      mx = a;
    }
  }
  return idx;
}

inline double seq_norm(const std::vector<double>& v) {
  return std::sqrt(hodlr3d_canonical_sum([&](long i) { return v[i] * v[i]; }, (long)v.size()));
}

inline double seq_dot(const double* a, const std::vector<double>& b) {
  return hodlr3d_canonical_sum([&](long i) { return a[i] * b[i]; }, (long)b.size());
}

// Partially pivoted ACA of the block K(rows, cols)
// (LowRank::ACA_only_nodesCUR, src/ACA.cpp:127-238).  Keeps the residual
// vectors u_l (columns of U) and v_l (columns of V); the reference's L and R
// are L(i,j) = U(row_i, j), R(j,i) = V(col_i, j).
void aca(const orc_problem& p, const int32_t* rows, int n, const int32_t* cols, int m,
         PairFactors& f) {
  f = PairFactors();
  if (n == 0 || m == 0) return;
  const int mn = std::min(n, m);
  std::vector<char> used_r(n, 0), used_c(m, 0);
  std::vector<double> row(m), col(n), u(n), v(m);
  int row_index = 0, col_index = -1;
  int l_local;
  for (l_local = 0; l_local < n; ++l_local) {  // :153-159
    row_index = l_local;
    for (int s = 0; s < m; ++s) row[s] = entry(p, rows[row_index], cols[s]);
    col_index = argmax_abs(row, used_c);
    if (std::fabs(row[col_index]) > 1e-16) break;
  }
  if (l_local == n) return;
  v = row;
  f.rows.push_back(row_index);
  f.cols.push_back(col_index);
  for (int t = 0; t < n; ++t) col[t] = entry(p, rows[t], cols[col_index]);
  for (int t = 0; t < n; ++t) u[t] = col[t] / row[col_index];
  f.U.insert(f.U.end(), u.begin(), u.end());
  f.V.insert(f.V.end(), v.begin(), v.end());
  used_c[col_index] = 1;
  used_r[row_index] = 1;
  int r = 1;
  double normS = 0.0;
  row_index = argmax_abs(col, used_r);
  while (seq_norm(u) * seq_norm(v) > p.tol * normS && r < mn) {  // :178
    f.rows.push_back(row_index);
    for (int s = 0; s < m; ++s) row[s] = entry(p, rows[row_index], cols[s]);
    for (int l = 0; l < r; ++l) {
      const double a = f.U[(size_t)l * n + row_index];
      const double* Vl = &f.V[(size_t)l * m];
      for (int s = 0; s < m; ++s) row[s] -= a * Vl[s];
    }
    col_index = argmax_abs(row, used_c);
    f.cols.push_back(col_index);
    v = row;
    for (int t = 0; t < n; ++t) col[t] = entry(p, rows[t], cols[col_index]);
    for (int l = 0; l < r; ++l) {
      const double a = f.V[(size_t)l * m + col_index];
      const double* Ul = &f.U[(size_t)l * n];
      for (int t = 0; t < n; ++t) col[t] -= a * Ul[t];
    }
    for (int t = 0; t < n; ++t) u[t] = col[t] / row[col_index];
    if (seq_norm(u) < 1e-16 || seq_norm(v) < 1e-16) {  // :199-203
      f.rows.pop_back();
      f.cols.pop_back();
      break;
    }
    f.U.insert(f.U.end(), u.begin(), u.end());
    f.V.insert(f.V.end(), v.begin(), v.end());
    ++r;
    used_c[col_index] = 1;
    used_r[row_index] = 1;
    const double nu = seq_norm(u), nv = seq_norm(v);  // :211-215
    normS = normS * normS + (nu * nv) * (nu * nv);
    for (int l = 0; l < r; ++l)
      normS += 2 * std::fabs(seq_dot(&f.U[(size_t)l * n], u) * seq_dot(&f.V[(size_t)l * m], v));
    normS = std::sqrt(normS);
    row_index = argmax_abs(col, used_r);
  }
  f.rank = r;
}

inline bool selected(const int32_t* sl, const int32_t* sb, int n, int level, int64_t box) {
  if (n <= 0) return true;
  for (int i = 0; i < n; ++i)
    if (sl[i] == level && sb[i] == box) return true;
  return false;
}

}  // namespace

extern "C" {

void orc_set_threads(int n) {
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
#else
  (void)n;
#endif
}

orc_problem* orc_create(const double* xyz, int64_t N, int nP1D, double L, int tol_pow,
                        int kernel_id, double diag_override) {
  orc_problem* p = new orc_problem();
  p->N = N;
  p->nP1D = nP1D;
  p->L = L;
  p->tol_pow = tol_pow;
  p->tol = std::pow(10, -1.0 * tol_pow);  // src/ACA.cpp:5
  p->kernel = kernel_id;
  p->diag = diag_override;
  p->x.resize(N);
  p->y.resize(N);
  p->z.resize(N);
  for (int64_t i = 0; i < N; ++i) {
    p->x[i] = xyz[3 * i];
    p->y[i] = xyz[3 * i + 1];
    p->z[i] = xyz[3 * i + 2];
  }
  if (kernel_id == 16) {
    p->Kii = quadrature_kii(N);
    p->h3 = 1.0 / double(N);
  }
  build_tree(*p);
  build_lists(*p);
  return p;
}

void orc_destroy(orc_problem* p) { delete p; }
int orc_levels(const orc_problem* p) { return p->nLevels; }
double orc_kii(const orc_problem* p) { return p->Kii; }
double orc_entry(const orc_problem* p, int64_t i, int64_t j) { return entry(*p, i, j); }
void orc_perm(const orc_problem* p, int32_t* perm) {
  std::copy(p->perm.begin(), p->perm.end(), perm);
}
void orc_box_offsets(const orc_problem* p, int level, int64_t* off) {
  std::copy(p->off[level].begin(), p->off[level].end(), off);
}
void orc_neighbors(const orc_problem* p, int level, int32_t* nbr) {
  std::copy(p->nbr[level].begin(), p->nbr[level].end(), nbr);
}
int64_t orc_num_pairs(const orc_problem* p) { return (int64_t)p->p_level.size(); }
void orc_pairs(const orc_problem* p, int32_t* lts) {
  for (size_t i = 0; i < p->p_level.size(); ++i) {
    lts[3 * i] = p->p_level[i];
    lts[3 * i + 1] = p->p_tgt[i];
    lts[3 * i + 2] = p->p_src[i];
  }
}

int orc_assemble(orc_problem* p, const int32_t* sel_level, const int32_t* sel_box, int n_sel) {
  const int64_t np = (int64_t)p->p_level.size();
  // largest blocks first so the dynamic schedule balances
  std::vector<int64_t> order;
  for (int64_t i = 0; i < np; ++i)
    if (selected(sel_level, sel_box, n_sel, p->p_level[i], p->p_tgt[i])) order.push_back(i);
  std::stable_sort(order.begin(), order.end(),
                   [&](int64_t a, int64_t b) { return p->p_level[a] < p->p_level[b]; });
#pragma omp parallel for schedule(dynamic, 1)
  for (int64_t oi = 0; oi < (int64_t)order.size(); ++oi) {
    const int64_t i = order[oi];
    const int j = p->p_level[i];
    const int64_t t0 = p->off[j][p->p_tgt[i]], t1 = p->off[j][p->p_tgt[i] + 1];
    const int64_t s0 = p->off[j][p->p_src[i]], s1 = p->off[j][p->p_src[i] + 1];
    PairFactors& f = p->fac[i];
    aca(*p, &p->perm[t0], (int)(t1 - t0), &p->perm[s0], (int)(s1 - s0), f);
    if (p->lean) {
      const int r = f.rank, n = (int)(t1 - t0), m = (int)(s1 - s0);
      f.Lm.assign((size_t)r * r, 0.0);
      f.Rm.assign((size_t)r * r, 0.0);
      for (int a = 0; a < r; ++a)
        for (int b = 0; b < r; ++b) {
          f.Lm[(size_t)a * r + b] = f.U[(size_t)b * n + f.rows[a]];
          f.Rm[(size_t)a * r + b] = f.V[(size_t)a * m + f.cols[b]];
        }
      std::vector<double>().swap(f.U);
      std::vector<double>().swap(f.V);
    }
  }
  return 0;
}

// Lean storage for the assemblies that follow: only pivots and the r x r L, R
// are kept (the CUR product needs nothing else); the residual-vector forms
// (orc_pair_factors, orc_matvec_uv, orc_matvec_uv_t) are then unavailable.
void orc_set_lean(orc_problem* p, int lean) { p->lean = lean != 0; }
int orc_is_lean(const orc_problem* p) { return p->lean ? 1 : 0; }

void orc_ranks(const orc_problem* p, int32_t* rank) {
  for (size_t i = 0; i < p->fac.size(); ++i) rank[i] = p->fac[i].rank;
}
int64_t orc_total_pivots(const orc_problem* p) {
  int64_t s = 0;
  for (const auto& f : p->fac) s += f.rank;
  return s;
}
void orc_pivots(const orc_problem* p, int32_t* rows, int32_t* cols) {
  int64_t w = 0;
  for (size_t i = 0; i < p->fac.size(); ++i) {
    const int j = p->p_level[i];
    const int64_t t0 = p->off[j][p->p_tgt[i]], s0 = p->off[j][p->p_src[i]];
    for (int r = 0; r < p->fac[i].rank; ++r) {
      rows[w] = p->perm[t0 + p->fac[i].rows[r]];
      cols[w] = p->perm[s0 + p->fac[i].cols[r]];
      ++w;
    }
  }
}
void orc_pair_factors(const orc_problem* p, int64_t pair, double* U, double* V) {
  std::copy(p->fac[pair].U.begin(), p->fac[pair].U.end(), U);
  std::copy(p->fac[pair].V.begin(), p->fac[pair].V.end(), V);
}

// Far field per level in CUR form with re-evaluated Ac, Ar
// (evaluateFarField, src/HODLR3DTree.cpp:1660-1706), leaf near field over
// slots 0..25 then self (evaluate_NearField :1708-1755), level sum in level
// order (collectPotential :1781-1793) and scatter to the original order
// (reorder :1795-1805).
void orc_matvec(const orc_problem* p, const double* xin, double* yout, const int32_t* sel_level,
                const int32_t* sel_box, int n_sel) {
  const int d = p->nLevels;
  const int64_t N = p->N;
  std::vector<double> xs(N), total(N, 0.0);
  for (int64_t t = 0; t < N; ++t) xs[t] = xin[p->perm[t]];
  for (int j = 1; j <= d || (j == 1 && d == 0); ++j) {
    const int lev = d == 0 ? 0 : j;
    std::vector<double> pot(N, 0.0);
    const int64_t nb = int64_t(1) << (3 * lev);
#pragma omp parallel for schedule(dynamic, 1)
    for (int64_t k = 0; k < nb; ++k) {
      const int64_t t0 = p->off[lev][k], n = p->off[lev][k + 1] - t0;
      const bool sel = selected(sel_level, sel_box, n_sel, lev, k);
      if (sel && lev >= 1) {
        for (int64_t i = p->il_ptr[lev][k]; i < p->il_ptr[lev][k + 1]; ++i) {
          const PairFactors& f = p->fac[i];
          const int r = f.rank;
          if (r == 0) continue;
          const int64_t s0 = p->off[lev][p->p_src[i]], m = p->off[lev][p->p_src[i] + 1] - s0;
          std::vector<double> t(r, 0.0), t1(r), t2(r);
          for (int l = 0; l < r; ++l) {  // t0 = Ar x
            const int32_t gi = p->perm[t0 + f.rows[l]];
            double s = 0.0;
            for (int64_t c = 0; c < m; ++c) s += entry(*p, gi, p->perm[s0 + c]) * xs[s0 + c];
            t[l] = s;
          }
          // L(a,b) = U(row_a, b), R(a,b) = V(col_b, a) (or their lean copies)
          auto Lab = [&](int a, int b) {
            return p->lean ? f.Lm[(size_t)a * r + b] : f.U[(size_t)b * n + f.rows[a]];
          };
          auto Rab = [&](int a, int b) {
            return p->lean ? f.Rm[(size_t)a * r + b] : f.V[(size_t)a * m + f.cols[b]];
          };
          for (int a = 0; a < r; ++a) {  // t1 = L^-1 t0
            double s = t[a];
            for (int b = 0; b < a; ++b) s -= Lab(a, b) * t1[b];
            t1[a] = s / 1.0;
          }
          for (int a = r - 1; a >= 0; --a) {  // t2 = R^-1 t1
            double s = t1[a];
            for (int b = a + 1; b < r; ++b) s -= Rab(a, b) * t2[b];
            t2[a] = s / Rab(a, a);
          }
          for (int64_t c = 0; c < n; ++c) {  // potential += Ac t2
            const int32_t gi = p->perm[t0 + c];
            double s = 0.0;
            for (int l = 0; l < r; ++l) s += entry(*p, gi, p->perm[s0 + f.cols[l]]) * t2[l];
            pot[t0 + c] += s;
          }
        }
      }
      if (lev == d && sel) {
        std::vector<double> acc(n);
        for (int sl = 0; sl <= 26; ++sl) {
          const int64_t nn = sl < 26 ? p->nbr[d][26 * k + sl] : k;
          if (nn < 0) continue;
          const int64_t q0 = p->off[d][nn], m = p->off[d][nn + 1] - q0;
          for (int64_t c = 0; c < n; ++c) {
            const int32_t gi = p->perm[t0 + c];
            double s = 0.0;
            for (int64_t e = 0; e < m; ++e) s += entry(*p, gi, p->perm[q0 + e]) * xs[q0 + e];
            pot[t0 + c] += s;
          }
        }
      }
    }
    for (int64_t t = 0; t < N; ++t) total[t] = total[t] + pot[t];
    if (d == 0) break;
  }
  for (int64_t t = 0; t < N; ++t) yout[p->perm[t]] = total[t];
}

// Same operator applied from the stored residual vectors: y_k += U (V^T x).
void orc_matvec_uv(const orc_problem* p, const double* xin, double* yout) {
  const int d = p->nLevels;
  const int64_t N = p->N;
  std::vector<double> xs(N), total(N, 0.0);
  for (int64_t t = 0; t < N; ++t) xs[t] = xin[p->perm[t]];
  for (int j = 1; j <= d; ++j) {
    const int64_t nb = int64_t(1) << (3 * j);
#pragma omp parallel for schedule(dynamic, 1)
    for (int64_t k = 0; k < nb; ++k) {
      const int64_t t0 = p->off[j][k], n = p->off[j][k + 1] - t0;
      for (int64_t i = p->il_ptr[j][k]; i < p->il_ptr[j][k + 1]; ++i) {
        const PairFactors& f = p->fac[i];
        const int r = f.rank;
        const int64_t s0 = p->off[j][p->p_src[i]], m = p->off[j][p->p_src[i] + 1] - s0;
        std::vector<double> t(r);
        for (int l = 0; l < r; ++l) {
          double s = 0.0;
          for (int64_t c = 0; c < m; ++c) s += f.V[(size_t)l * m + c] * xs[s0 + c];
          t[l] = s;
        }
        for (int64_t c = 0; c < n; ++c) {
          double s = 0.0;
          for (int l = 0; l < r; ++l) s += f.U[(size_t)l * n + c] * t[l];
          total[t0 + c] += s;
        }
      }
    }
  }
#pragma omp parallel for schedule(dynamic, 1)
  for (int64_t k = 0; k < (int64_t(1) << (3 * d)); ++k) {
    const int64_t t0 = p->off[d][k], n = p->off[d][k + 1] - t0;
    for (int sl = 0; sl <= 26; ++sl) {
      const int64_t nn = sl < 26 ? p->nbr[d][26 * k + sl] : k;
      if (nn < 0) continue;
      const int64_t q0 = p->off[d][nn], m = p->off[d][nn + 1] - q0;
      for (int64_t c = 0; c < n; ++c) {
        const int32_t gi = p->perm[t0 + c];
        double s = 0.0;
        for (int64_t e = 0; e < m; ++e) s += entry(*p, gi, p->perm[q0 + e]) * xs[q0 + e];
        total[t0 + c] += s;
      }
    }
  }
  for (int64_t t = 0; t < N; ++t) yout[p->perm[t]] = total[t];
}

// Transpose of the stored operator: for every pair (k, s) the source box s
// receives V (U^T x_k); the near field contributes K(i, j) x_i to row j.
void orc_matvec_uv_t(const orc_problem* p, const double* xin, double* yout) {
  const int d = p->nLevels;
  const int64_t N = p->N;
  std::vector<double> xs(N), total(N, 0.0);
  for (int64_t t = 0; t < N; ++t) xs[t] = xin[p->perm[t]];
  for (int j = 1; j <= d; ++j) {
    const int64_t nb = int64_t(1) << (3 * j);
    for (int64_t k = 0; k < nb; ++k) {
      const int64_t t0 = p->off[j][k], n = p->off[j][k + 1] - t0;
      for (int64_t i = p->il_ptr[j][k]; i < p->il_ptr[j][k + 1]; ++i) {
        const PairFactors& f = p->fac[i];
        const int r = f.rank;
        const int64_t s0 = p->off[j][p->p_src[i]], m = p->off[j][p->p_src[i] + 1] - s0;
        std::vector<double> t(r);
        for (int l = 0; l < r; ++l) {
          double s = 0.0;
          for (int64_t c = 0; c < n; ++c) s += f.U[(size_t)l * n + c] * xs[t0 + c];
          t[l] = s;
        }
        for (int64_t c = 0; c < m; ++c) {
          double s = 0.0;
          for (int l = 0; l < r; ++l) s += f.V[(size_t)l * m + c] * t[l];
          total[s0 + c] += s;
        }
      }
    }
  }
  for (int64_t k = 0; k < (int64_t(1) << (3 * d)); ++k) {
    const int64_t t0 = p->off[d][k], n = p->off[d][k + 1] - t0;
    for (int sl = 0; sl <= 26; ++sl) {
      const int64_t nn = sl < 26 ? p->nbr[d][26 * k + sl] : k;
      if (nn < 0) continue;
      const int64_t q0 = p->off[d][nn], m = p->off[d][nn + 1] - q0;
      for (int64_t e = 0; e < m; ++e) {
        const int32_t gj = p->perm[q0 + e];
        double s = 0.0;
        for (int64_t c = 0; c < n; ++c) s += entry(*p, p->perm[t0 + c], gj) * xs[t0 + c];
        total[q0 + e] += s;
      }
    }
  }
  for (int64_t t = 0; t < N; ++t) yout[p->perm[t]] = total[t];
}

void orc_dense_rows(const orc_problem* p, const int64_t* rows, int64_t nrows, const double* x,
                    double* y) {
#pragma omp parallel for schedule(dynamic, 4)
  for (int64_t r = 0; r < nrows; ++r) {
    double s = 0.0;
    for (int64_t j = 0; j < p->N; ++j) s += entry(*p, rows[r], j) * x[j];
    y[r] = s;
  }
}

// classGMRES::gmres (src/gmres.cpp:40-94) with arnoldi (:29-38), Givens
// rotations (:5-26) and the final triangular solve of the rotated Hessenberg.
int orc_gmres(const orc_problem* p, const double* b, int maxit, double tol, double* x,
              double* hist, int* nhist) {
  const int64_t N = p->N;
  std::vector<double> r(b, b + N);  // x0 = 0, A x0 = 0
  double b_norm = 0.0;
  for (int64_t i = 0; i < N; ++i) b_norm += b[i] * b[i];
  b_norm = std::sqrt(b_norm);
  const double r_norm = b_norm;
  int nh = 0;
  hist[nh++] = r_norm / b_norm;
  const int m = maxit;
  std::vector<std::vector<double>> Q;
  Q.emplace_back(N);
  for (int64_t i = 0; i < N; ++i) Q[0][i] = r[i] / r_norm;
  std::vector<std::vector<double>> H;  // columns of the rotated Hessenberg
  std::vector<double> cs(m, 0.0), sn(m, 0.0), beta(m + 1, 0.0);
  beta[0] = r_norm;
  int K = m - 1;
  std::vector<double> q(N);
  for (int k = 0; k < m; ++k) {
    orc_matvec(p, Q[k].data(), q.data(), nullptr, nullptr, 0);
    std::vector<double> h(k + 2, 0.0);
    for (int i = 0; i <= k; ++i) {  // modified Gram-Schmidt
      double s = 0.0;
      for (int64_t t = 0; t < N; ++t) s += q[t] * Q[i][t];
      h[i] = s;
      for (int64_t t = 0; t < N; ++t) q[t] = q[t] - h[i] * Q[i][t];
    }
    double qn = 0.0;
    for (int64_t t = 0; t < N; ++t) qn += q[t] * q[t];
    h[k + 1] = std::sqrt(qn);
    Q.emplace_back(N);
    for (int64_t t = 0; t < N; ++t) Q[k + 1][t] = q[t] / h[k + 1];
    for (int i = 0; i < k; ++i) {
      const double tmp = cs[i] * h[i] + sn[i] * h[i + 1];
      h[i + 1] = -sn[i] * h[i] + cs[i] * h[i + 1];
      h[i] = tmp;
    }
    const double tn = std::sqrt(h[k] * h[k] + h[k + 1] * h[k + 1]);
    cs[k] = h[k] / tn;
    sn[k] = h[k + 1] / tn;
    h[k] = cs[k] * h[k] + sn[k] * h[k + 1];
    h[k + 1] = 0.0;
    H.push_back(h);
    beta[k + 1] = -sn[k] * beta[k];
    beta[k] = cs[k] * beta[k];
    const double err = std::fabs(beta[k + 1]) / b_norm;
    hist[nh++] = err;
    if (err <= tol) {
      K = k;
      break;
    }
  }
  const int n = K + 1;
  std::vector<double> yv(n);
  for (int i = n - 1; i >= 0; --i) {
    double s = beta[i];
    for (int j = i + 1; j < n; ++j) s -= H[j][i] * yv[j];
    yv[i] = s / H[i][i];
  }
  for (int64_t t = 0; t < N; ++t) {
    double s = 0.0;
    for (int l = 0; l < n; ++l) s += Q[l][t] * yv[l];
    x[t] = 0.0 + s;
  }
  *nhist = nh;
  return n;
}

double orc_memory_entries(const orc_problem* p) {
  double sum = 0.0;
  const int d = p->nLevels;
  for (size_t i = 0; i < p->fac.size(); ++i) {
    const int j = p->p_level[i];
    const double n = double(p->off[j][p->p_tgt[i] + 1] - p->off[j][p->p_tgt[i]]);
    const double m = double(p->off[j][p->p_src[i] + 1] - p->off[j][p->p_src[i]]);
    const double r = p->fac[i].rank;
    sum += r * n + r * r + m * r;
  }
  for (int64_t k = 0; k < (int64_t(1) << (3 * d)); ++k) {
    const double n = double(p->off[d][k + 1] - p->off[d][k]);
    sum += n * n;
    for (int s = 0; s < 26; ++s) {
      const int64_t nn = p->nbr[d][26 * k + s];
      if (nn >= 0) sum += n * double(p->off[d][nn + 1] - p->off[d][nn]);
    }
  }
  return sum;
}

int orc_max_rank(const orc_problem* p) {
  int r = 0;
  for (const auto& f : p->fac) r = std::max(r, f.rank);
  return r;
}

}  // extern "C"
