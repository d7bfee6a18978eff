"""GB300 (sm_103a) implementation of immunodbscan's DBSCAN clone-collapsing path.

The clustering runs in libimmunodbscan_gb300.so (hand-written CUDA behind the C
ABI of include/immunodbscan_gb300.h).  This package holds the build recipe, the
ctypes binding, a Python mirror of the reference's InterlinkClass and the
seeded synthetic repertoire generators used by the tests and the benchmark.
"""
from ._lib import IdbError, LIB_PATH, lib  # noqa: F401
from .interlink import (Context, DeviceBatch, Interlink, Result, cluster_workload,  # noqa: F401
                        make_params)

__all__ = ["IdbError", "LIB_PATH", "lib", "Context", "DeviceBatch", "Interlink", "Result",
           "cluster_workload", "make_params"]
