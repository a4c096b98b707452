"""The C-ABI library builds, loads and exports every entry point that
include/*.h declares; host-only calls behave (no GPU needed)."""
import ctypes
import glob
import math
import os
import re

import pytest

from hodlr3d_gb300 import _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        src = open(h).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        for m in re.finditer(r"\b(hodlr3d_[a-z0-9_]+)\s*\(", src):
            names.add(m.group(1))
    return sorted(names)


def test_headers_declare_the_abi():
    names = declared_functions()
    for must in ("hodlr3d_create", "hodlr3d_assemble", "hodlr3d_matvec", "hodlr3d_gmres",
                 "hodlr3d_destroy", "hodlr3d_last_error", "hodlr3d_matvec_transpose"):
        assert must in names


def test_library_exports_every_declared_symbol():
    L = _lib.lib()
    missing = [n for n in declared_functions() if not hasattr(L, n)]
    assert not missing, missing


def test_abi_version_and_default_options():
    L = _lib.lib()
    assert L.hodlr3d_abi_version() == 3
    o = _lib.Options()
    L.hodlr3d_default_options(ctypes.byref(o))
    assert o.device == 0 and o.keep_fp32 == 1 and math.isnan(o.diag_override)


def test_invalid_arguments_fail_cleanly():
    L = _lib.lib()
    h = ctypes.c_void_p()
    import numpy as np
    pts = np.zeros((10, 3))
    # bad kernel id
    code = L.hodlr3d_create(pts.ctypes.data, 10, 4, 1.0, 10, 42, None, ctypes.byref(h))
    assert code == _lib.ERR_INVALID_ARG and not h.value
    code = L.hodlr3d_create(pts.ctypes.data, 10, 4, 1.0, 10, -1, None, ctypes.byref(h))
    assert code == _lib.ERR_INVALID_ARG and not h.value
    # null handle: every entry point that takes one refuses it
    assert L.hodlr3d_assemble(None) == _lib.ERR_INVALID_ARG
    buf = ctypes.create_string_buffer(64)
    choice = np.zeros(128, np.int32)
    assert L.hodlr3d_autotune(None, 3, buf, 64) == _lib.ERR_INVALID_ARG
    assert L.hodlr3d_get_tuning(None, choice.ctypes.data) == _lib.ERR_INVALID_ARG
    assert L.hodlr3d_set_engine(None, 0) == _lib.ERR_INVALID_ARG
    assert L.hodlr3d_matvec(None, None, None, 1, 10, 0, None) == _lib.ERR_INVALID_ARG
    assert L.hodlr3d_dense_rows(None, None, 0, None, None, 1, 10, None) == _lib.ERR_INVALID_ARG
    assert L.hodlr3d_get_stats(None, None) == _lib.ERR_INVALID_ARG
    assert L.hodlr3d_device_status(None) == _lib.ERR_INVALID_ARG
    assert L.hodlr3d_launch_count(None) == 0
    L.hodlr3d_destroy(None)  # a no-op
    # factor files: bad arguments and a missing file fail before any device work
    assert L.hodlr3d_save(None, b"x.h3d") == _lib.ERR_INVALID_ARG
    assert L.hodlr3d_load(None, None, ctypes.byref(h)) == _lib.ERR_INVALID_ARG
    assert L.hodlr3d_load(b"/nonexistent/op.h3d", None, ctypes.byref(h)) == _lib.ERR_IO
    assert not h.value and b"cannot open" in L.hodlr3d_last_error()


def test_no_device_or_tree_error_is_reported():
    """Without a GPU creation reports ERR_NO_DEVICE; with one, a too-shallow tree is refused."""
    import numpy as np
    L = _lib.lib()
    h = ctypes.c_void_p()
    pts = np.random.default_rng(0).uniform(-1, 1, (64, 3))
    code = L.hodlr3d_create(pts.ctypes.data, 64, 4, 1.0, 10, 16, None, ctypes.byref(h))
    assert code in (_lib.ERR_NO_DEVICE, _lib.ERR_INVALID_ARG)
    assert not h.value


def _factor_header(version=1, n=64, npairs=0, npools=0):
    import struct
    # FileHeader (hodlr3d_gb300/csrc/factors.cpp): version, header bytes, n, nP1D, tol_pow, L, kernel, levels,
    # diag, npairs, npools, reserved, lists hash
    return b"H3DFACT1" + struct.pack("<IIqiidiidqiiQ", version, 72, n, 4, 10, 1.0, 16, 1, 0.5,
                                     npairs, npools, 0, 0x1234)


def test_factor_header_reader(tmp_path):
    p = tmp_path / "h.h3d"
    p.write_bytes(_factor_header(n=4096, npairs=2808) + b"\0" * 64)
    h = _lib.read_factor_header(p)
    assert (h["version"], h["header_bytes"], h["n"], h["nP1D"], h["tol_pow"], h["kernel"]) == (1, 72, 4096, 4, 10, 16)
    assert h["L"] == 1.0 and h["diag"] == 0.5 and h["npairs"] == 2808 and h["lists_hash"] == 0x1234


def test_factor_file_validation_before_any_device_work(tmp_path):
    """Wrong magic, wrong version, truncated points and header sizes that no
    saved operator has (more points than hodlr3d_create takes, more pools
    than pairs, negative counts) are refused with HODLR3D_ERR_IO while
    reading, before anything is allocated from them or the tree is rebuilt
    on a device."""
    L = _lib.lib()
    h = ctypes.c_void_p()
    cases = {
        "magic.h3d": b"H3DFACT9" + _factor_header()[8:],
        "version.h3d": _factor_header(version=2),
        "truncated.h3d": _factor_header(n=64) + b"\0" * 100,  # 64 points need 1536 bytes
        "huge_n.h3d": _factor_header(n=1 << 60),
        "one_point.h3d": _factor_header(n=1),
        "pools.h3d": _factor_header(npairs=10, npools=11),
        "neg_pairs.h3d": _factor_header(npairs=-1),
        "neg_pools.h3d": _factor_header(npools=-3),
    }
    for name, data in cases.items():
        p = tmp_path / name
        p.write_bytes(data)
        assert L.hodlr3d_load(str(p).encode(), None, ctypes.byref(h)) == _lib.ERR_IO, name
        assert not h.value
