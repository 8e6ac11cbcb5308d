"""mulskips_gb300 — GB300-native KMC event loop of MulSKIPS.

The compute path is libmulskips_gpu.so (CUDA, sm_103a) behind the C ABI in
include/mulskips_gpu.h; this package holds its build step, the ctypes
binding, the start.dat front end and the pymulskips-style wrapper.
"""
from .engine import Lattice, Batch, arrhenius_tables, coordination  # noqa: F401

__all__ = ["Lattice", "Batch", "arrhenius_tables", "coordination"]
