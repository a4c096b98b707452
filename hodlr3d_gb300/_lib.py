"""ctypes binding of the C ABI in include/hodlr3d.h (libhodlr3d_gb300.so).

The library is the only compute path: if it cannot be loaded the import of
any function that needs it raises, there is no CPU fallback.
"""
from __future__ import annotations

import ctypes
import math
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "lib", "libhodlr3d_gb300.so")

OK = 0
ERR_INVALID_ARG = 1
ERR_CUDA = 2
ERR_OUT_OF_MEMORY = 3
ERR_NOT_ASSEMBLED = 4
ERR_NONFINITE = 5
ERR_BREAKDOWN = 6
ERR_NO_CONVERGENCE = 7
ERR_UNSUPPORTED = 8
ERR_NO_DEVICE = 9
ERR_IO = 10

FP64 = 0
MIXED = 1
FP64X = 2  # FP64-accurate products in FP32-pair arithmetic


class Options(ctypes.Structure):
    _fields_ = [("device", ctypes.c_int), ("diag_override", ctypes.c_double),
                ("keep_fp32", ctypes.c_int), ("aca_workspace_bytes", ctypes.c_size_t),
                ("rank_cap", ctypes.c_int)]


class Stats(ctypes.Structure):
    _fields_ = [("n_points", ctypes.c_int64), ("levels", ctypes.c_int), ("n_pairs", ctypes.c_int64),
                ("n_near_blocks", ctypes.c_int64), ("max_rank", ctypes.c_int),
                ("sum_rank", ctypes.c_int64), ("memory_entries", ctypes.c_double),
                ("factor_entries", ctypes.c_int64), ("u_entries", ctypes.c_int64),
                ("v_entries", ctypes.c_int64), ("factor_bytes_fp64", ctypes.c_int64),
                ("factor_bytes_fp32", ctypes.c_int64), ("near_entries", ctypes.c_int64),
                ("tree_seconds", ctypes.c_double), ("assemble_seconds", ctypes.c_double),
                ("aca_batches", ctypes.c_int), ("aca_kernel_seconds", ctypes.c_double),
                ("finish_seconds", ctypes.c_double)]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


class GmresParams(ctypes.Structure):
    _fields_ = [("maxit", ctypes.c_int), ("restart", ctypes.c_int), ("tol", ctypes.c_double),
                ("precision", ctypes.c_int), ("max_outer", ctypes.c_int),
                ("inner_tol", ctypes.c_double), ("transpose", ctypes.c_int)]


class GmresResult(ctypes.Structure):
    _fields_ = [("iterations", ctypes.c_int), ("outer", ctypes.c_int),
                ("rel_residual", ctypes.c_double), ("converged", ctypes.c_int)]


class HODLR3DError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"hodlr3d error {code}: {msg}")
        self.code = code


_lib = None


def ensure_built() -> str:
    if not os.path.exists(LIB_PATH):
        from . import build
        build.build()
    return LIB_PATH


def lib() -> ctypes.CDLL:
    global _lib
    if _lib is not None:
        return _lib
    path = ensure_built()
    L = ctypes.CDLL(path)
    vp, i32, i64, dbl = ctypes.c_void_p, ctypes.c_int, ctypes.c_int64, ctypes.c_double
    sigs = {
        "hodlr3d_abi_version": ([], i32),
        "hodlr3d_default_options": ([ctypes.POINTER(Options)], None),
        "hodlr3d_last_error": ([], ctypes.c_char_p),
        "hodlr3d_create": ([vp, i64, i32, dbl, i32, i32, ctypes.POINTER(Options),
                            ctypes.POINTER(vp)], i32),
        "hodlr3d_destroy": ([vp], None),
        "hodlr3d_assemble": ([vp], i32),
        "hodlr3d_save": ([vp, ctypes.c_char_p], i32),
        "hodlr3d_load": ([ctypes.c_char_p, ctypes.POINTER(Options), ctypes.POINTER(vp)], i32),
        "hodlr3d_matvec": ([vp, vp, vp, i32, i64, i32, vp], i32),
        "hodlr3d_matvec_host": ([vp, vp, vp, i32, i64, i32], i32),
        "hodlr3d_matvec_host_rows": ([vp, vp, vp, i32, i32], i32),
        "hodlr3d_matvec_transpose": ([vp, vp, vp, i32, i64, i32, vp], i32),
        "hodlr3d_dense_rows": ([vp, vp, i64, vp, vp, i32, i64, vp], i32),
        "hodlr3d_entries": ([vp, vp, vp, i64, vp], i32),
        "hodlr3d_quadrature_kii": ([i64, ctypes.POINTER(dbl)], i32),
        "hodlr3d_gmres": ([vp, vp, vp, i32, i64, ctypes.POINTER(GmresParams),
                           ctypes.POINTER(GmresResult), vp, i32, ctypes.POINTER(i32), vp], i32),
        "hodlr3d_get_stats": ([vp, ctypes.POINTER(Stats)], i32),
        "hodlr3d_get_tree": ([vp, vp, vp], i32),
        "hodlr3d_get_neighbors": ([vp, i32, vp], i32),
        "hodlr3d_get_pairs": ([vp, vp], i32),
        "hodlr3d_get_ranks": ([vp, vp], i32),
        "hodlr3d_get_pivots": ([vp, vp, vp], i32),
        "hodlr3d_get_pair_factors": ([vp, i64, vp, vp], i32),
        "hodlr3d_launch_count": ([vp], i64),
        "hodlr3d_set_profiling": ([vp, i32], i32),
        "hodlr3d_set_engine": ([vp, i32], i32),
        "hodlr3d_autotune": ([vp, i32, ctypes.c_char_p, i32], i32),
        "hodlr3d_get_tuning": ([vp, vp], i32),
        "hodlr3d_device_status": ([vp], i32),
        "hodlr3d_test_drop_copy": ([vp, i32], i32),
        "hodlr3d_matvec_noalloc": ([vp, vp, vp, i32, i64, i32, vp], i32),
        "hodlr3d_profile_report": ([vp, ctypes.c_char_p, i32], i32),
    }
    for name, (args, res) in sigs.items():
        f = getattr(L, name)
        f.argtypes = args
        f.restype = res
    _lib = L
    return L


def check(code: int) -> None:
    if code != OK:
        msg = lib().hodlr3d_last_error()
        raise HODLR3DError(code, msg.decode() if msg else "")


def default_options(device: int = 0, diag_override: float = math.nan, keep_fp32: bool = True,
                    aca_workspace_bytes: int = 0, rank_cap: int = 0) -> Options:
    o = Options()
    lib().hodlr3d_default_options(ctypes.byref(o))
    o.device = device
    o.diag_override = diag_override
    o.keep_fp32 = 1 if keep_fp32 else 0
    o.aca_workspace_bytes = aca_workspace_bytes
    o.rank_cap = rank_cap
    return o


def read_factor_header(path) -> dict:
    """The parameters stored in a factor file (include/hodlr3d.h, hodlr3d_save):
    magic, then {version, header bytes, n, nP1D, tol_pow, L, kernel, levels,
    diag, npairs, npools, reserved, lists hash}."""
    import struct
    with open(path, "rb") as f:
        head = f.read(8 + 72)
    if len(head) < 80 or head[:8] != b"H3DFACT1":
        raise HODLR3DError(ERR_IO, f"{path}: not a hodlr3d factor file")
    v = struct.unpack("<IIqiidiidqiiQ", head[8:80])
    keys = ("version", "header_bytes", "n", "nP1D", "tol_pow", "L", "kernel", "levels", "diag",
            "npairs", "npools", "reserved", "lists_hash")
    return dict(zip(keys, v))
