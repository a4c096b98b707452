"""Python mirror of the reference's HODLR3D C++ API over the CUDA library.

``HODLR3D(nParticlesInLeafAlong1D, L, TOL_POW, Qchoice, particles)``,
``assemble()`` and ``MatVecProduct(b)`` follow include/HODLR3D.hpp:12-21;
``classGMRES().gmres(M, b, maxIterations, threshold)`` follows
include/gmres.hpp:13-26.  The work runs in libhodlr3d_gb300.so on one GPU;
numpy arrays go through the host entry points, CUDA torch tensors through the
device entry points on torch's current stream.
"""
from __future__ import annotations

import ctypes
import math
import os
from typing import Optional

import numpy as np

from . import _lib
from ._lib import FP64, FP64X, MIXED, HODLR3DError, check

_PREC = {"fp64": FP64, "mixed": MIXED, "fp64x": FP64X, FP64: FP64, MIXED: MIXED, FP64X: FP64X}


def _prec(p) -> int:
    try:
        return _PREC[p]
    except KeyError:
        raise ValueError(f"precision must be 'fp64', 'mixed' or 'fp64x', got {p!r}") from None


def parse_tune_report(text: str, engines) -> tuple:
    """The report of hodlr3d_autotune (include/hodlr3d.h): a header line, one
    "transpose nrhs engine ms" line per engine timing, then "launch ta_split k
    ms" lines and "launch ta_split_chosen k ms".  Returns ([(transpose, nrhs,
    engine name, ms)], {"ta_split": {k: ms}, "ta_split_chosen": k or None})."""
    rows = []
    launch = {"ta_split": {}, "ta_split_chosen": None}
    for line in text.splitlines()[1:]:
        if line.startswith("launch "):
            _, key, k, ms = line.split()
            if key == "ta_split":
                launch["ta_split"][int(k)] = float(ms)
            elif key == "ta_split_chosen":
                launch["ta_split_chosen"] = int(k)
            continue
        t, n, e, ms = line.split()
        rows.append((bool(int(t)), int(n), engines[int(e)], float(ms)))
    return rows, launch


class HODLR3D:
    """The HODLR3D operator on one GPU (reference: src/HODLR3D.cpp:3-32).

    particles: (N, 3) array of points.  Qchoice: the reference's kernel choice
    (src/kernel.cpp:65-227); 16 is 1/r with the quadrature diagonal.
    diag_override: optional diagonal value (e.g. 1.0 for exp(-r)).
    """

    def __init__(self, nParticlesInLeafAlong1D: int, L: float, TOL_POW: int, Qchoice: int,
                 particles, *, diag_override: float = math.nan, device: int = 0,
                 keep_fp32: bool = True, aca_workspace_bytes: int = 0, rank_cap: int = 0):
        L_ = _lib.lib()
        pts = np.ascontiguousarray(np.asarray(particles, dtype=np.float64).reshape(-1, 3))
        self.N = int(pts.shape[0])
        self.nParticlesInLeafAlong1D = int(nParticlesInLeafAlong1D)
        self.L = float(L)
        self.TOL_POW = int(TOL_POW)
        self.Qchoice = int(Qchoice)
        self.device = int(device)
        opt = _lib.default_options(device, diag_override, keep_fp32, aca_workspace_bytes, rank_cap)
        h = ctypes.c_void_p()
        check(L_.hodlr3d_create(pts.ctypes.data, self.N, self.nParticlesInLeafAlong1D, self.L,
                                self.TOL_POW, self.Qchoice, ctypes.byref(opt), ctypes.byref(h)))
        self._h = h
        self._L = L_
        self.assembled = False

    def close(self) -> None:
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            self._L.hodlr3d_destroy(h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self) -> ctypes.c_void_p:
        if self._h is None:
            raise HODLR3DError(_lib.ERR_INVALID_ARG, "closed")
        return self._h

    # ---- reference API ----------------------------------------------------
    def assemble(self) -> None:
        """ACA of every interaction-list pair (HODLR3D::assemble)."""
        check(self._L.hodlr3d_assemble(self.handle))
        self.assembled = True

    # ---- factor persistence (no reference counterpart) ----------------------
    def save(self, path) -> None:
        """Writes the assembled operator (parameters, points, ranks, pivots,
        FP64 factors) to a versioned binary file (hodlr3d_save)."""
        check(self._L.hodlr3d_save(self.handle, os.fsencode(path)))

    @classmethod
    def load(cls, path, *, device: int = 0, keep_fp32: bool = True) -> "HODLR3D":
        """An assembled operator from a file written by save(): the tree is
        rebuilt from the saved points and checked against the saved lists; no
        ACA runs (hodlr3d_load)."""
        L_ = _lib.lib()
        opt = _lib.default_options(device, math.nan, keep_fp32, 0, 0)
        h = ctypes.c_void_p()
        check(L_.hodlr3d_load(os.fsencode(path), ctypes.byref(opt), ctypes.byref(h)))
        self = cls.__new__(cls)
        self._h = h
        self._L = L_
        self.device = int(device)
        st = _lib.Stats()
        check(L_.hodlr3d_get_stats(h, ctypes.byref(st)))
        self.N = int(st.n_points)
        hdr = _lib.read_factor_header(path)
        self.nParticlesInLeafAlong1D = hdr["nP1D"]
        self.L = hdr["L"]
        self.TOL_POW = hdr["tol_pow"]
        self.Qchoice = hdr["kernel"]
        self.assembled = True
        return self

    def MatVecProduct(self, b, precision="fp64", out=None) -> np.ndarray:
        """Ab = A b for host arrays b of shape (N,) or (N, nrhs) (HODLR3D::MatVecProduct).

        A C-ordered (N, nrhs) array goes to the GPU as it is (rows of
        right-hand sides, reordered there); other layouts by columns.  out: an
        optional float64 array of b's shape and layout to write the result to."""
        a = np.asarray(b, dtype=np.float64)
        if a.ndim not in (1, 2) or a.shape[0] != self.N:
            raise ValueError(f"expected shape ({self.N},) or ({self.N}, nrhs), got {np.shape(b)}")
        if a.ndim == 2 and a.shape[1] > 1 and a.flags.c_contiguous:
            y = np.empty_like(a) if out is None else out
            if y.shape != a.shape or y.dtype != np.float64 or not y.flags.c_contiguous:
                raise ValueError("out must be a C-ordered float64 array of b's shape")
            check(self._L.hodlr3d_matvec_host_rows(self.handle, a.ctypes.data, y.ctypes.data,
                                                   a.shape[1], _prec(precision)))
            return y
        x, nrhs, shape = self._host_cols(a)
        y = np.empty_like(x)
        check(self._L.hodlr3d_matvec_host(self.handle, x.ctypes.data, y.ctypes.data, nrhs, self.N,
                                          _prec(precision)))
        if out is not None:
            out[...] = y.T.reshape(shape)
            return out
        return y.T.reshape(shape)

    # ---- device API (torch tensors on this GPU) --------------------------
    def matvec(self, x, precision="fp64", transpose: bool = False):
        """y = A x (or A^T x) for a CUDA float64 tensor of shape (N,) or (N, nrhs)."""
        import torch
        xc, nrhs, shape = self._dev_cols(x)
        y = torch.empty_like(xc)
        fn = self._L.hodlr3d_matvec_transpose if transpose else self._L.hodlr3d_matvec
        check(fn(self.handle, xc.data_ptr(), y.data_ptr(), nrhs, self.N, _prec(precision),
                 torch.cuda.current_stream(xc.device).cuda_stream))
        return y.T.reshape(shape)

    def matvec_transpose(self, x, precision="fp64"):
        return self.matvec(x, precision, transpose=True)

    def gmres(self, b, maxit: int = 400, tol: float = 1e-10, restart: int = 0,
              precision="fp64", transpose: bool = False, max_outer: int = 0,
              inner_tol: float = 0.0, hist_cap: int = 0, raise_on_failure: bool = True):
        """Solves A x = b (or A^T x = b) from x0 = 0 for a CUDA float64 tensor b
        of shape (N,) or (N, nrhs).  Returns (x, info)."""
        import torch
        bc, nrhs, shape = self._dev_cols(b)
        x = torch.empty_like(bc)
        prm = _lib.GmresParams(int(maxit), int(restart), float(tol), _prec(precision),
                               int(max_outer), float(inner_tol), 1 if transpose else 0)
        res = _lib.GmresResult()
        hist = np.zeros(max(hist_cap, 1), np.float64)
        nh = ctypes.c_int(0)
        code = self._L.hodlr3d_gmres(self.handle, bc.data_ptr(), x.data_ptr(), nrhs, self.N,
                                     ctypes.byref(prm), ctypes.byref(res),
                                     hist.ctypes.data if hist_cap else None, int(hist_cap),
                                     ctypes.byref(nh), torch.cuda.current_stream(bc.device).cuda_stream)
        info = {"iterations": res.iterations, "outer": res.outer,
                "rel_residual": res.rel_residual, "converged": bool(res.converged),
                "history": hist[: nh.value].copy(), "status": code}
        if code != _lib.OK and raise_on_failure and code not in (_lib.ERR_NO_CONVERGENCE,):
            check(code)
        return x.T.reshape(shape), info

    def entries(self, rows, cols) -> np.ndarray:
        """K(rows[e], cols[e]) as the device evaluates it (FP64; the diagonal
        value where the ids are equal); original point ids."""
        r = np.ascontiguousarray(np.asarray(rows, np.int64).reshape(-1))
        c = np.ascontiguousarray(np.asarray(cols, np.int64).reshape(-1))
        if r.shape != c.shape:
            raise ValueError("rows and cols differ in length")
        out = np.empty(len(r), np.float64)
        check(self._L.hodlr3d_entries(self.handle, r.ctypes.data, c.ctypes.data, len(r),
                                      out.ctypes.data))
        return out

    def dense_rows(self, rows, x):
        """FP64 direct sum of sampled rows: y[r] = sum_j K(rows[r], j) x[j]."""
        import torch
        xc, nrhs, shape = self._dev_cols(x)
        rows_np = np.asarray(rows, np.int64).reshape(-1)
        if rows_np.size and (rows_np.min() < 0 or rows_np.max() >= self.N):
            raise ValueError(f"row ids must lie in [0, {self.N})")
        rows_t = torch.as_tensor(rows_np, device=xc.device)
        y = torch.empty((nrhs, len(rows_t)), dtype=torch.float64, device=xc.device)
        check(self._L.hodlr3d_dense_rows(self.handle, rows_t.data_ptr(), len(rows_t), xc.data_ptr(),
                                         y.data_ptr(), nrhs, self.N,
                                         torch.cuda.current_stream(xc.device).cuda_stream))
        return y.T if len(shape) == 2 else y[0]

    # ---- introspection ----------------------------------------------------
    def stats(self) -> dict:
        s = _lib.Stats()
        check(self._L.hodlr3d_get_stats(self.handle, ctypes.byref(s)))
        return s.as_dict()

    @property
    def levels(self) -> int:
        return int(self.stats()["levels"])

    def perm(self) -> np.ndarray:
        p = np.empty(self.N, np.int32)
        check(self._L.hodlr3d_get_tree(self.handle, p.ctypes.data, None))
        return p

    def leaf_offsets(self) -> np.ndarray:
        off = np.empty((1 << (3 * self.levels)) + 1, np.int64)
        check(self._L.hodlr3d_get_tree(self.handle, None, off.ctypes.data))
        return off

    def neighbors(self, level: int) -> np.ndarray:
        out = np.empty((1 << (3 * level)) * 26, np.int32)
        check(self._L.hodlr3d_get_neighbors(self.handle, int(level), out.ctypes.data))
        return out.reshape(-1, 26)

    def pairs(self) -> np.ndarray:
        n = int(self.stats()["n_pairs"])
        out = np.empty(3 * n, np.int32)
        check(self._L.hodlr3d_get_pairs(self.handle, out.ctypes.data))
        return out.reshape(-1, 3)

    def ranks(self) -> np.ndarray:
        n = int(self.stats()["n_pairs"])
        out = np.empty(n, np.int32)
        check(self._L.hodlr3d_get_ranks(self.handle, out.ctypes.data))
        return out

    def pivots(self):
        n = int(self.stats()["sum_rank"])
        r = np.empty(max(n, 1), np.int32)
        c = np.empty(max(n, 1), np.int32)
        check(self._L.hodlr3d_get_pivots(self.handle, r.ctypes.data, c.ctypes.data))
        return r[:n], c[:n]

    def pair_factors(self, pair: int, n: int, m: int, rank: int):
        U = np.empty(max(n * rank, 1), np.float64)
        V = np.empty(max(m * rank, 1), np.float64)
        check(self._L.hodlr3d_get_pair_factors(self.handle, int(pair), U.ctypes.data, V.ctypes.data))
        return U[: n * rank].reshape(rank, n).T, V[: m * rank].reshape(rank, m).T

    def launch_count(self) -> int:
        return int(self._L.hodlr3d_launch_count(self.handle))

    def set_engine(self, engine: str) -> None:
        """'auto', 'simt' (CUDA cores, every form), 'tc' (tcgen05 tensor cores,
        mixed A x) or 'gemv' (few-column streaming kernels: mixed and fp64x
        A x and A^T x from the FP32 copies, the FP64 form from FP64 copies
        grouped the same way)."""
        check(self._L.hodlr3d_set_engine(self.handle, {"auto": 0, "simt": 1, "tc": 2, "gemv": 3}[engine]))

    ENGINES = ("auto", "simt", "tc", "gemv")

    def autotune(self, reps: int = 3) -> list:
        """Times every engine that runs the mixed product of this operator at
        1, 2, 4, 8, 16, 32 and 64 right-hand sides (A x and A^T x) and makes
        the automatic choice follow the fastest; reps=0 returns to the
        column-count rules.  Returns the timings as (transpose, nrhs, engine,
        ms) tuples."""
        buf = ctypes.create_string_buffer(1 << 14)
        check(self._L.hodlr3d_autotune(self.handle, int(reps), buf, len(buf)))
        rows, self._launch = parse_tune_report(buf.value.decode(), self.ENGINES)
        return rows

    def launch_tuning(self) -> dict:
        """The launch shapes the last autotune() timed on the tensor-core
        engine: {"ta_split": {blocks per slice: ms}, "ta_split_chosen": k}
        (None where it did not run)."""
        return getattr(self, "_launch", {"ta_split": {}, "ta_split_chosen": None})

    def tuning(self) -> dict:
        """The automatic engine per column count after autotune():
        {"forward": [...], "transpose": [...]} over nrhs = 1..64, None where the
        column-count rules apply."""
        c = np.zeros(128, np.int32)
        check(self._L.hodlr3d_get_tuning(self.handle, c.ctypes.data))
        names = [None if v == 0 else self.ENGINES[v] for v in c]
        return {"forward": names[:64], "transpose": names[64:]}

    def device_status(self) -> None:
        """Raises if a bounded device wait gave up in an earlier call."""
        check(self._L.hodlr3d_device_status(self.handle))

    def set_profiling(self, enable: bool) -> None:
        """Records CUDA events between the matvec's kernel launches."""
        check(self._L.hodlr3d_set_profiling(self.handle, 1 if enable else 0))

    def profile_report(self) -> dict:
        """{kernel: (launches, total_ms)} accumulated since the last report."""
        buf = ctypes.create_string_buffer(4096)
        check(self._L.hodlr3d_profile_report(self.handle, buf, len(buf)))
        out = {}
        for line in buf.value.decode().splitlines():
            name, n, ms = line.split()
            out[name] = (int(n), float(ms))
        return out

    # ---- helpers --------------------------------------------------------------
    def _host_cols(self, b):
        a = np.asarray(b, dtype=np.float64)
        if a.ndim == 1:
            a = a.reshape(-1, 1)
        if a.ndim != 2 or a.shape[0] != self.N:
            raise ValueError(f"expected shape ({self.N},) or ({self.N}, nrhs), got {np.shape(b)}")
        return np.ascontiguousarray(a.T), a.shape[1], np.shape(b)

    def _dev_cols(self, x):
        import torch
        if not isinstance(x, torch.Tensor) or not x.is_cuda:
            raise TypeError("expected a CUDA torch tensor")
        if x.dtype != torch.float64:
            raise TypeError("expected float64")
        if x.device.index != self.device:
            raise ValueError(f"the operator lives on cuda:{self.device}, the tensor on {x.device}")
        shape = tuple(x.shape)
        xx = x.reshape(-1, 1) if x.dim() == 1 else x
        if xx.dim() != 2 or xx.shape[0] != self.N:
            raise ValueError(f"expected shape ({self.N},) or ({self.N}, nrhs), got {shape}")
        return xx.T.contiguous(), int(xx.shape[1]), shape


class classGMRES:
    """classGMRES::gmres (include/gmres.hpp:23, src/gmres.cpp:40-94): unrestarted
    GMRES from x0 = 0; returns (x, error, noOfIterations, e) where e holds the
    residual estimates |beta(k+1)| / |b| starting with 1."""

    def gmres(self, M: HODLR3D, b, maxIterations: int, threshold: float):
        import torch
        host = not isinstance(b, torch.Tensor)
        bt = torch.as_tensor(np.asarray(b, np.float64) if host else b, dtype=torch.float64)
        if not bt.is_cuda:
            bt = bt.to(f"cuda:{M.device}")
        x, info = M.gmres(bt, maxit=maxIterations, tol=threshold, restart=0, precision="fp64",
                          hist_cap=maxIterations + 1)
        e = list(info["history"])
        xo = x.cpu().numpy() if host else x
        return xo, info["rel_residual"], info["iterations"], e
