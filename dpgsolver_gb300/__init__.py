"""GB300-native (sm_103a, FP64) explicit DG residual for DPGSolver.

The product is libdgpu.so (CUDA, C ABI in include/dgpu.h); ``solver`` mirrors the reference's explicit DG entry
points over that ABI and ``host`` builds the caller-side set-up (meshes, TP operators, geometry) for the
synthetic workloads.
"""
from ._lib import build, load, LIB_PATH  # noqa: F401

__all__ = ["build", "load", "LIB_PATH"]
