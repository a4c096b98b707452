"""The C++ facade headers compile against the library and, on a GPU, run the
reference's driver flow (matvec vs dense columns, GMRES solve)."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CUDA = "/usr/local/cuda"


def build_example(tmpdir, name="facade_example"):
    from hodlr3d_gb300 import _lib
    lib = _lib.ensure_built()
    exe = os.path.join(tmpdir, name)
    cmd = [shutil.which("g++") or "g++", "-std=c++17", "-O2",
           os.path.join(ROOT, "tests", "cpp", name + ".cpp"), "-I", os.path.join(ROOT, "include"),
           "-I", os.path.join(CUDA, "include"), "-L", os.path.dirname(lib), "-lhodlr3d_gb300",
           "-L", os.path.join(CUDA, "lib64"), "-lcudart", "-Wl,-rpath," + os.path.dirname(lib),
           "-o", exe]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    return exe


def test_facade_compiles_and_links(tmp_path):
    exe = build_example(str(tmp_path))
    assert os.path.exists(exe)
    assert os.path.exists(build_example(str(tmp_path), "user_kernel_example"))


def test_host_kernel_formulas_and_kii(tmp_path):
    """include/kernel.hpp on the host alone (no GPU): the 16 named formulas of
    userkernel against their definitions, getRow / getCol / getMatrix against
    getMatrixEntry, and Kii from the library's quadrature."""
    src = tmp_path / "k.cpp"
    src.write_text(r"""
#include <cmath>
#include <cstdio>
#include "kernel.hpp"
int main() {
  std::vector<pts3D> p = {{0, 0, 0}, {0.3, -0.2, 0.1}, {1.0, 0.5, -0.5}};
  userkernel k16(p, 16), k7(p, 7);
  const double r = std::sqrt(0.09 + 0.04 + 0.01);
  int bad = 0;
  bad += std::fabs(k16.getMatrixEntry(0, 1) - (1.0 / 3.0) / r) > 1e-15;
  bad += !(k16.getMatrixEntry(1, 1) == k16.Kii) || !(k16.Kii > 1.0);
  bad += std::fabs(k7.getMatrixEntry(1, 0) - 1.0 / r) > 1e-15 || k7.getMatrixEntry(2, 2) != 0.0;
  bad += std::fabs(k7.Feynman(0, 1) - std::sqrt(3.14159265358979323846 / 2) * std::exp(-r) / r) > 1e-14;
  bad += std::fabs(k7.Yukawa(0, 1) - std::exp(-50 * r) / r) > 1e-15;
  bad += std::fabs(k7.kernel_besselJ(0, 1) - std::cyl_bessel_j(0.0, r)) > 0;
  auto col = k16.getCol(1);
  auto row = k16.getRow(1, {0, 2});
  auto m = k16.getMatrix({0, 1}, {1, 2});
  auto blk = k16.getMatrix(1, 1, 3, 3);
  bad += col.size() != 3 || col(0) != k16.getMatrixEntry(0, 1) || row(1) != k16.getMatrixEntry(1, 2);
  bad += m(1, 1) != k16.getMatrixEntry(1, 2) || blk(0, 1) != k16.getMatrixEntry(1, 2);
  double kii = 0;
  bad += hodlr3d_quadrature_kii(3, &kii) != 0 || kii != k16.Kii;
  printf("bad=%d Kii=%.17g\n", bad, k16.Kii);
  return bad;
}
""")
    from hodlr3d_gb300 import _lib
    lib = _lib.ensure_built()
    exe = str(tmp_path / "k")
    subprocess.run([shutil.which("g++") or "g++", "-std=c++17", "-O2", str(src), "-I",
                    os.path.join(ROOT, "include"), "-L", os.path.dirname(lib), "-lhodlr3d_gb300",
                    "-L", os.path.join(CUDA, "lib64"), "-lcudart", "-Wl,-rpath," + os.path.dirname(lib),
                    "-o", exe], check=True, capture_output=True, text=True)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0, r.stdout + r.stderr


@pytest.mark.gpu
def test_user_defined_getmatrixentry(tmp_path):
    """An application's own getMatrixEntry: accepted when it is the device's
    kernel (product checked against its dense columns), refused with
    HODLR3D_ERR_UNSUPPORTED when it is not."""
    exe = build_example(str(tmp_path), "user_kernel_example")
    r = subprocess.run([exe, "16", "same"], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0 and "accepted" in r.stdout, r.stdout + r.stderr
    r = subprocess.run([exe, "16", "other"], capture_output=True, text=True, timeout=300)
    assert r.returncode == 3 and "refused: code=8" in r.stdout, r.stdout + r.stderr


@pytest.mark.gpu
def test_facade_runs_reference_driver_flow(tmp_path):
    exe = build_example(str(tmp_path))
    r = subprocess.run([exe, "16"], capture_output=True, text=True, timeout=300)
    print(r.stdout, r.stderr)
    assert r.returncode == 0, r.stdout + r.stderr
