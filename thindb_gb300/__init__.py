"""thindb_gb300 — GB300-native grouped-aggregation path of thinDB.

The CUDA engine lives in libthindb_gpu.so behind the plain-C boundary
include/thindb_gpu.h; this package holds the sources (csrc/), the in-tree
build, and the host-side mirror of thinDB's operator interface (engine.py).
"""
from . import abi  # noqa: F401

__all__ = ["abi", "engine", "datagen", "build"]
