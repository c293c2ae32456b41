"""mdacp_gb300: GB300-native (sm_103a) Lennard-Jones short-range hot path of MDACP.

The compute lives in libmdg.so (CUDA, C ABI in include/mdg.h); this package is
the host side: the ctypes binding (`native`), an MDManager mirror
(`manager`), the .cfg semantics (`config`) and initial conditions (`lattice`).
"""
from . import config, lattice  # noqa: F401

__all__ = ["config", "lattice", "native", "manager"]
