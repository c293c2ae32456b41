"""The reference's output and restart formats (ctypes over include/mdg.h).

write_dump      MDManager::SaveAsDumpFile (mdmanager.cc:475-505)
write_cdview    MDUnit::SaveAsCdview (mdunit.cc:52-67)
write_configuration  Variables::SaveConfiguration (variables.cc:45-56), real particles
write_stream / read_stream  Variables::SaveToStream / LoadFromStream (variables.cc:111-131)

Positions and momenta are (n, 3) or (n, 4) arrays in the caller's order; the
files are byte for byte what the reference writes for the same particles.
"""
import ctypes

import numpy as np

from . import native

_D = ctypes.POINTER(ctypes.c_double)


def _four(a, n=None):
    a = np.asarray(a, dtype=np.float64)
    out = np.zeros((len(a) if n is None else n, 4))
    out[:, :a.shape[1]] = a
    return np.ascontiguousarray(out)


def _ck(rc, what):
    if rc != native.MDG_OK:
        raise native.MDGError("%s: %s" % (what, native.ERRORS.get(rc, rc)))


def write_dump(path, q, p, append=False):
    q4, p4 = _four(q), _four(p)
    _ck(native.load().mdg_write_dump(str(path).encode(), q4.ctypes.data_as(_D), p4.ctypes.data_as(_D), len(q4),
                                     1 if append else 0), "write_dump")


def write_cdview(path, q, p, types=None, append=False):
    q4, p4 = _four(q), _four(p)
    t = None
    if types is not None:
        t = np.ascontiguousarray(types, dtype=np.int32)
    _ck(native.load().mdg_write_cdview(str(path).encode(), q4.ctypes.data_as(_D), p4.ctypes.data_as(_D),
                                       t.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)) if t is not None else None,
                                       len(q4), 1 if append else 0), "write_cdview")


def write_configuration(path, q, p):
    q4, p4 = _four(q), _four(p)
    _ck(native.load().mdg_write_configuration(str(path).encode(), q4.ctypes.data_as(_D), p4.ctypes.data_as(_D),
                                              len(q4)), "write_configuration")


def write_stream(path, q, p, append=False):
    q4, p4 = _four(q), _four(p)
    _ck(native.load().mdg_write_stream(str(path).encode(), q4.ctypes.data_as(_D), p4.ctypes.data_as(_D), len(q4),
                                       1 if append else 0), "write_stream")


def read_stream(path, capacity):
    """Returns (q4, p4, time, zeta) of a LoadFromStream file ([n][4] arrays)."""
    q4 = np.zeros((capacity, 4))
    p4 = np.zeros((capacity, 4))
    n = ctypes.c_int32()
    t, z = ctypes.c_double(), ctypes.c_double()
    _ck(native.load().mdg_read_stream(str(path).encode(), q4.ctypes.data_as(_D), p4.ctypes.data_as(_D), capacity,
                                      ctypes.byref(n), ctypes.byref(t), ctypes.byref(z)), "read_stream")
    return q4[:n.value], p4[:n.value], t.value, z.value
