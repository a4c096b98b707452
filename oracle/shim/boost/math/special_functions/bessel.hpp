// Project-written stand-in for the three Boost.Math Bessel functions that the
// HODLR3D reference kernels call (src/kernel.cpp Qchoice 11, 12, 14).  It maps
// them to the C++17 special functions of libstdc++.  Test infrastructure only.
#ifndef HODLR3D_ORACLE_BOOST_BESSEL_SHIM
#define HODLR3D_ORACLE_BOOST_BESSEL_SHIM
#include <cmath>
namespace boost {
namespace math {
inline double cyl_bessel_j(double nu, double x) { return std::cyl_bessel_j(nu, x); }
inline double cyl_neumann(double nu, double x) { return std::cyl_neumann(nu, x); }
inline double cyl_bessel_k(double nu, double x) { return std::cyl_bessel_k(nu, x); }
}  // namespace math
}  // namespace boost
#endif
