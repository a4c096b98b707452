"""ctypes wrapper of the CPU oracle (oracle/hodlr3d_oracle.cpp).

TEST INFRASTRUCTURE ONLY: imported by tests/, by ``__graft_entry__.smoke()``
and by the CPU-baseline leg of ``bench.py``, to check the CUDA path against.
The product package never imports it.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "build", "liboracle_hodlr3d.so")
_lib = None

_i32p = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")
_i64p = np.ctypeslib.ndpointer(np.int64, flags="C_CONTIGUOUS")
_f64p = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")


def build(force: bool = False) -> str:
    """Compiles the oracle library with its Makefile (seconds)."""
    src = os.path.join(_HERE, "hodlr3d_oracle.cpp")
    if force or not os.path.exists(_LIB_PATH) or os.path.getmtime(_LIB_PATH) < os.path.getmtime(src):
        subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB_PATH


def lib():
    global _lib
    if _lib is not None:
        return _lib
    build()
    L = ctypes.CDLL(_LIB_PATH)
    vp = ctypes.c_void_p
    L.orc_create.restype = vp
    L.orc_create.argtypes = [_f64p, ctypes.c_int64, ctypes.c_int, ctypes.c_double, ctypes.c_int,
                             ctypes.c_int, ctypes.c_double]
    L.orc_destroy.argtypes = [vp]
    L.orc_set_threads.argtypes = [ctypes.c_int]
    L.orc_levels.argtypes = [vp]
    L.orc_levels.restype = ctypes.c_int
    L.orc_kii.argtypes = [vp]
    L.orc_kii.restype = ctypes.c_double
    L.orc_entry.argtypes = [vp, ctypes.c_int64, ctypes.c_int64]
    L.orc_entry.restype = ctypes.c_double
    L.orc_perm.argtypes = [vp, _i32p]
    L.orc_box_offsets.argtypes = [vp, ctypes.c_int, _i64p]
    L.orc_neighbors.argtypes = [vp, ctypes.c_int, _i32p]
    L.orc_num_pairs.argtypes = [vp]
    L.orc_num_pairs.restype = ctypes.c_int64
    L.orc_pairs.argtypes = [vp, _i32p]
    L.orc_set_lean.argtypes = [vp, ctypes.c_int]
    L.orc_is_lean.argtypes = [vp]
    L.orc_is_lean.restype = ctypes.c_int
    L.orc_assemble.argtypes = [vp, vp, vp, ctypes.c_int]
    L.orc_assemble.restype = ctypes.c_int
    L.orc_ranks.argtypes = [vp, _i32p]
    L.orc_total_pivots.argtypes = [vp]
    L.orc_total_pivots.restype = ctypes.c_int64
    L.orc_pivots.argtypes = [vp, _i32p, _i32p]
    L.orc_pair_factors.argtypes = [vp, ctypes.c_int64, _f64p, _f64p]
    L.orc_matvec.argtypes = [vp, _f64p, _f64p, vp, vp, ctypes.c_int]
    L.orc_matvec_uv.argtypes = [vp, _f64p, _f64p]
    L.orc_matvec_uv_t.argtypes = [vp, _f64p, _f64p]
    L.orc_dense_rows.argtypes = [vp, _i64p, ctypes.c_int64, _f64p, _f64p]
    L.orc_gmres.argtypes = [vp, _f64p, ctypes.c_int, ctypes.c_double, _f64p, _f64p,
                            ctypes.POINTER(ctypes.c_int)]
    L.orc_gmres.restype = ctypes.c_int
    L.orc_memory_entries.argtypes = [vp]
    L.orc_memory_entries.restype = ctypes.c_double
    L.orc_max_rank.argtypes = [vp]
    L.orc_max_rank.restype = ctypes.c_int
    _lib = L
    return L


def set_threads(n: int) -> None:
    lib().orc_set_threads(int(n))


class Oracle:
    """The reference algorithm on the CPU in FP64 (restated; see the C++ file)."""

    def __init__(self, points, nP1D=4, L=1.0, tol_pow=10, kernel=16, diag=float("nan"),
                 lean=False):
        """lean: keep only the pivots and the r x r L, R per pair (the
        reference's own storage; what the CUR product needs) instead of the
        residual vectors U, V as well -- 62 GB less host memory at 64^3."""
        self._L = lib()
        pts = np.ascontiguousarray(points, dtype=np.float64).reshape(-1, 3)
        self.N = pts.shape[0]
        self.points = pts
        self.h = self._L.orc_create(pts.ravel(), self.N, int(nP1D), float(L), int(tol_pow),
                                    int(kernel), float(diag))
        self.levels = self._L.orc_levels(self.h)
        self.assembled = False
        self._L.orc_set_lean(self.h, 1 if lean else 0)

    def __del__(self):
        h = getattr(self, "h", None)
        if h:
            self._L.orc_destroy(h)
            self.h = None

    def _need_vectors(self):
        if self._L.orc_is_lean(self.h):
            raise RuntimeError("the residual vectors U, V are not kept in lean mode")

    # tree -------------------------------------------------------------
    @property
    def kii(self) -> float:
        return self._L.orc_kii(self.h)

    def entry(self, i: int, j: int) -> float:
        return self._L.orc_entry(self.h, int(i), int(j))

    def perm(self) -> np.ndarray:
        out = np.empty(self.N, np.int32)
        self._L.orc_perm(self.h, out)
        return out

    def box_offsets(self, level: int) -> np.ndarray:
        out = np.empty((1 << (3 * level)) + 1, np.int64)
        self._L.orc_box_offsets(self.h, int(level), out)
        return out

    def neighbors(self, level: int) -> np.ndarray:
        out = np.empty((1 << (3 * level)) * 26, np.int32)
        self._L.orc_neighbors(self.h, int(level), out)
        return out.reshape(-1, 26)

    def pairs(self) -> np.ndarray:
        n = self._L.orc_num_pairs(self.h)
        out = np.empty(3 * n, np.int32)
        self._L.orc_pairs(self.h, out)
        return out.reshape(-1, 3)

    # assembly ----------------------------------------------------------
    def assemble(self, sel_level=None, sel_box=None):
        if sel_level is None:
            self._L.orc_assemble(self.h, None, None, 0)
        else:
            sl = np.ascontiguousarray(sel_level, np.int32)
            sb = np.ascontiguousarray(sel_box, np.int32)
            self._L.orc_assemble(self.h, sl.ctypes.data, sb.ctypes.data, len(sl))
        self.assembled = True

    def ranks(self) -> np.ndarray:
        out = np.empty(self._L.orc_num_pairs(self.h), np.int32)
        self._L.orc_ranks(self.h, out)
        return out

    def pivots(self):
        n = self._L.orc_total_pivots(self.h)
        r = np.empty(n, np.int32)
        c = np.empty(n, np.int32)
        self._L.orc_pivots(self.h, r, c)
        return r, c

    def pair_factors(self, pair: int, n: int, m: int, rank: int):
        self._need_vectors()
        U = np.empty(n * rank, np.float64)
        V = np.empty(m * rank, np.float64)
        self._L.orc_pair_factors(self.h, int(pair), U, V)
        return U.reshape(rank, n).T, V.reshape(rank, m).T

    def memory_entries(self) -> float:
        return self._L.orc_memory_entries(self.h)

    def max_rank(self) -> int:
        return self._L.orc_max_rank(self.h)

    # products ----------------------------------------------------------
    def matvec(self, x, sel_level=None, sel_box=None) -> np.ndarray:
        x = np.ascontiguousarray(x, np.float64)
        y = np.zeros(self.N, np.float64)
        if sel_level is None:
            self._L.orc_matvec(self.h, x, y, None, None, 0)
        else:
            sl = np.ascontiguousarray(sel_level, np.int32)
            sb = np.ascontiguousarray(sel_box, np.int32)
            self._L.orc_matvec(self.h, x, y, sl.ctypes.data, sb.ctypes.data, len(sl))
        return y

    def matvec_uv(self, x) -> np.ndarray:
        self._need_vectors()
        x = np.ascontiguousarray(x, np.float64)
        y = np.zeros(self.N, np.float64)
        self._L.orc_matvec_uv(self.h, x, y)
        return y

    def matvec_uv_t(self, x) -> np.ndarray:
        self._need_vectors()
        x = np.ascontiguousarray(x, np.float64)
        y = np.zeros(self.N, np.float64)
        self._L.orc_matvec_uv_t(self.h, x, y)
        return y

    def dense_rows(self, rows, x) -> np.ndarray:
        rows = np.ascontiguousarray(rows, np.int64)
        x = np.ascontiguousarray(x, np.float64)
        y = np.empty(len(rows), np.float64)
        self._L.orc_dense_rows(self.h, rows, len(rows), x, y)
        return y

    def gmres(self, b, maxit=400, tol=1e-10):
        b = np.ascontiguousarray(b, np.float64)
        x = np.zeros(self.N, np.float64)
        hist = np.zeros(maxit + 1, np.float64)
        nh = ctypes.c_int(0)
        nit = self._L.orc_gmres(self.h, b, int(maxit), float(tol), x, hist, ctypes.byref(nh))
        return x, hist[: nh.value], nit
