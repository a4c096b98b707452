"""Helpers shared by the tests that read the golden fixtures of tests/golden/."""
from __future__ import annotations

import glob
import hashlib
import os
import zlib

import numpy as np

from hodlr3d_gb300 import workloads

GOLDEN_DIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


# fixtures above this many points (the 64^3 operators) are checked by their
# own GPU module, tests/test_gpu_parity_large.py, with one assembly per case;
# the CPU oracle and the per-engine modules take the smaller ones
LARGE_N = 40000


def _npz_points(path: str) -> int:
    with np.load(path) as d:
        return int(d["N"])


def golden_names(large: bool = False):
    names = sorted(glob.glob(os.path.join(GOLDEN_DIR, "*.npz")))
    return [os.path.basename(p)[:-4] for p in names if (_npz_points(p) > LARGE_N) == large]


def load(name: str) -> dict:
    d = np.load(os.path.join(GOLDEN_DIR, name + ".npz"))
    return {k: d[k] for k in d.files}


def points_of(g: dict) -> np.ndarray:
    gen = str(g["generator"])
    args = g["gen_args"]
    if gen == "uniform_random":
        pts = workloads.uniform_random(int(args[0]), int(args[1]))
    elif len(args) > 1:
        pts = getattr(workloads, gen)(int(args[0]), float(args[1]))
    else:
        pts = getattr(workloads, gen)(int(args[0]))
    assert hashlib.sha256(pts.tobytes()).hexdigest() == str(g["points_sha256"]), "point generator drifted"
    return pts


def pair_keys(pairs: np.ndarray) -> np.ndarray:
    p = pairs.astype(np.int64)
    return (p[:, 0] << 40) | (p[:, 1] << 20) | p[:, 2]


def pivot_crc_per_box(pairs: np.ndarray, ranks: np.ndarray, rows: np.ndarray, cols: np.ndarray):
    """One CRC32 per (level, target box) over the pivots of its pairs in pair
    order, boxes in increasing (level, box) order."""
    ptr = np.concatenate([[0], np.cumsum(ranks.astype(np.int64))])
    key = pairs[:, 0].astype(np.int64) * (1 << 32) + pairs[:, 1]
    order = np.argsort(key, kind="stable")
    ks = key[order]
    starts = np.concatenate([[0], np.nonzero(np.diff(ks))[0] + 1, [len(ks)]])
    out = []
    for a, b in zip(starts[:-1], starts[1:]):
        sel = order[a:b]
        r = np.concatenate([rows[ptr[i]:ptr[i + 1]] for i in sel]).astype(np.int32)
        c = np.concatenate([cols[ptr[i]:ptr[i + 1]] for i in sel]).astype(np.int32)
        out.append(zlib.crc32(np.ascontiguousarray(np.stack([r, c])).tobytes()))
    return np.array(out, dtype=np.uint32)
