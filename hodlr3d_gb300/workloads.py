"""Seeded synthetic point sets and charge vectors for the HODLR3D workloads.

Points follow the ordering of the reference's ``set_Uniform_Nodes``
(examples/testHODLR3D.cpp:15-31): index ``p = j*n*n + k*n + i`` has
``x = node[k], y = node[j], z = node[i]`` (z fastest, y slowest).
"""
from __future__ import annotations

import numpy as np


def grid_cell_centres(n: int, L: float = 1.0) -> np.ndarray:
    """n^3 cell centres of a uniform grid on [-L, L]^3: ``-L + L(2i+1)/n``."""
    nodes = -L + L * (2.0 * np.arange(n) + 1.0) / n
    return _tensor(nodes)


def grid_reference_nodes(n: int, L: float = 1.0) -> np.ndarray:
    """The reference's interior nodes ``-L + 2L(k+1)/(n+1)`` (examples/testHODLR3D.cpp:17-19)."""
    nodes = np.array([-L + 2.0 * L * (k + 1.0) / (n + 1.0) for k in range(n)])
    return _tensor(nodes)


def _tensor(nodes: np.ndarray) -> np.ndarray:
    n = len(nodes)
    j, k, i = np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing="ij")
    return np.ascontiguousarray(
        np.stack([nodes[k.ravel()], nodes[j.ravel()], nodes[i.ravel()]], axis=1), dtype=np.float64)


def uniform_random(N: int, seed: int = 1, L: float = 1.0) -> np.ndarray:
    """N points i.i.d. uniform in [-L, L]^3."""
    rng = np.random.default_rng(seed)
    return np.ascontiguousarray(rng.uniform(-L, L, size=(N, 3)), dtype=np.float64)


def charges_uniform(N: int, nrhs: int = 1, seed: int = 1) -> np.ndarray:
    """i.i.d. uniform[0,1) charges, shape (N,) for one column else (N, nrhs)."""
    q = np.random.default_rng(seed).random((nrhs, N)).T
    return np.ascontiguousarray(q[:, 0] if nrhs == 1 else q)


def charges_normal(N: int, nrhs: int = 1, seed: int = 1) -> np.ndarray:
    """i.i.d. N(0,1) charges, shape (N,) for one column else (N, nrhs)."""
    q = np.random.default_rng(seed).standard_normal((nrhs, N)).T
    return np.ascontiguousarray(q[:, 0] if nrhs == 1 else q)
