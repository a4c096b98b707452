"""The C++ facade headers compile against the library and, on a GPU, run the
reference's driver flow (matvec vs dense columns, GMRES solve)."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CUDA = "/usr/local/cuda"


def build_example(tmpdir):
    from hodlr3d_gb300 import _lib
    lib = _lib.ensure_built()
    exe = os.path.join(tmpdir, "facade_example")
    cmd = [shutil.which("g++") or "g++", "-std=c++17", "-O2",
           os.path.join(ROOT, "tests", "cpp", "facade_example.cpp"), "-I", os.path.join(ROOT, "include"),
           "-I", os.path.join(CUDA, "include"), "-L", os.path.dirname(lib), "-lhodlr3d_gb300",
           "-L", os.path.join(CUDA, "lib64"), "-lcudart", "-Wl,-rpath," + os.path.dirname(lib),
           "-o", exe]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    return exe


def test_facade_compiles_and_links(tmp_path):
    exe = build_example(str(tmp_path))
    assert os.path.exists(exe)


@pytest.mark.gpu
def test_facade_runs_reference_driver_flow(tmp_path):
    exe = build_example(str(tmp_path))
    r = subprocess.run([exe, "16"], capture_output=True, text=True, timeout=300)
    print(r.stdout, r.stderr)
    assert r.returncode == 0, r.stdout + r.stderr
