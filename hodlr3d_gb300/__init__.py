"""hodlr3d_gb300: GB300-native HODLR3D (uniform-octree ACA assembly, fast
matvec, GMRES) on one GPU, behind the reference's API.

The compute path is libhodlr3d_gb300.so (hand-written sm_103a CUDA, C ABI in
include/hodlr3d.h); this package is its Python host mirror.
"""
from ._lib import FP64, FP64X, MIXED, HODLR3DError
from .hodlr3d import HODLR3D, classGMRES

__all__ = ["HODLR3D", "classGMRES", "HODLR3DError", "FP64", "FP64X", "MIXED"]
