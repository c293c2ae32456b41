"""The C-ABI library: builds for sm_103a, loads, and exports every entry point of include/mdg.h.

No compute calls here (no GPU on the CPU runner)."""
import ctypes
import os
import re
import shutil

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    names = []
    for h in os.listdir(os.path.join(ROOT, "include")):
        if h.endswith(".h"):
            text = open(os.path.join(ROOT, "include", h)).read()
            names += re.findall(r"^\s*(?:const\s+)?\w+\s*\*?\s*(mdg_\w+)\s*\(", text, re.M)
    return sorted(set(names))


@pytest.fixture(scope="module")
def lib():
    from mdacp_gb300 import build, native
    if not os.path.exists(native.LIB_PATH):
        if not shutil.which("nvcc") and not os.path.exists("/usr/local/cuda/bin/nvcc"):
            pytest.skip("nvcc not available")
        build.build()
    return ctypes.CDLL(native.LIB_PATH)


def test_header_declares_entry_points():
    names = _declared()
    assert "mdg_create" in names and "mdg_calculate" in names and len(names) >= 15


def test_every_declared_symbol_is_exported(lib):
    for name in _declared():
        assert hasattr(lib, name), name


def test_binding_covers_header():
    from mdacp_gb300 import adjoint, batch, native
    assert set(_declared()) <= set(native.SIGNATURES) | set(batch.SIGNATURES) | set(adjoint.SIGNATURES)


def test_version_and_defaults_without_gpu(lib):
    from mdacp_gb300 import native
    L = native.load()
    assert b"sm_103a" in L.mdg_version()
    p = native.Params()
    L.mdg_params_default(ctypes.byref(p))
    assert p.cutoff == 3.0 and abs(p.margin - 0.3) < 1e-15 and p.dt == 0.001 and p.langevin_half_drift_compat == 1
    # the half-margin rule by default; the reference policy's candidate limit
    # at CheckListLength's default (simulationinfo.cc:27)
    assert p.rebuild_policy == native.REBUILD_HALFMARGIN and p.check_list_length == 500
    assert ctypes.sizeof(native.Params) == 128  # sizeof(mdg_params) on the C side


def test_invalid_parameters_rejected_before_device_use(lib):
    from mdacp_gb300 import native
    L = native.load()
    p = native.Params()
    L.mdg_params_default(ctypes.byref(p))
    p.capacity = -5
    h = ctypes.c_void_p()
    assert L.mdg_create(ctypes.byref(p), ctypes.byref(h)) == 1
    assert not h.value
    assert L.mdg_destroy(None) == 0
    # the reason stays readable after the failed create, per calling thread
    assert b"capacity" in L.mdg_last_error(None)
    p.capacity = 100
    p.dt = 0.0
    assert L.mdg_create(ctypes.byref(p), ctypes.byref(h)) == 1
    assert b"dt" in L.mdg_last_error(None)
    p.dt = 0.001
    p.rebuild_policy = 7
    assert L.mdg_create(ctypes.byref(p), ctypes.byref(h)) == 1
    assert b"rebuild policy" in L.mdg_last_error(None)
    p.rebuild_policy = native.REBUILD_REFERENCE
    p.check_list_length = 0
    assert L.mdg_create(ctypes.byref(p), ctypes.byref(h)) == 1
    assert b"check_list_length" in L.mdg_last_error(None)


def test_python_manager_reports_the_create_reason():
    from mdacp_gb300 import native
    from mdacp_gb300.manager import MDManager
    with pytest.raises(native.MDGError, match="dt must be"):
        MDManager(20.0, capacity=100, dt=0.0)


def test_adjoint_create_checks_before_device_use(lib):
    # particle count (list entries hold the index in 26 bits), box size
    # against 2 (cutoff sigma + margin) and the step parameters are checked
    # before any device call
    import mdacp_gb300.adjoint as adj
    L = adj._lib()
    p = adj.AdjointParams()
    L.mdg_adjoint_params_default(ctypes.byref(p))
    p.box[:] = [20.0, 20.0, 20.0]
    p.margin = 0.5
    h = ctypes.c_void_p()
    for n in (1, 1 << 26):
        assert L.mdg_adjoint_create(ctypes.byref(p), n, ctypes.byref(h)) == 1
        assert not h.value
    p.box[:] = [5.9, 20.0, 20.0]  # below 2 (2.5 + 0.5)
    assert L.mdg_adjoint_create(ctypes.byref(p), 4000, ctypes.byref(h)) == 1
    p.box[:] = [20.0, 20.0, 20.0]
    p.checkpoint_every = 0
    assert L.mdg_adjoint_create(ctypes.byref(p), 4000, ctypes.byref(h)) == 1
    assert not h.value


def test_batch_create_checks_before_device_use(lib):
    # box sizes against 2 (cutoff + margin), particle counts and the cell
    # limit are checked before any device call; the switches refuse a null
    # handle
    import numpy as np
    import mdacp_gb300.batch as bt
    L = bt._lib()
    p = bt.BatchParams()
    L.mdg_batch_params_default(ctypes.byref(p))
    p.margin = 0.4
    h = ctypes.c_void_p()

    def create(ns, boxes):
        n = np.asarray(ns, dtype=np.int32)
        b = np.asarray(boxes, dtype=np.float64).reshape(-1, 3)
        return L.mdg_batch_create(ctypes.byref(p), len(n), n.ctypes.data_as(bt._I), bt._dp(b), ctypes.byref(h))

    assert create([100], [[5.7, 10.0, 10.0]]) == 1      # an edge below 2 (2.5 + 0.4)
    assert create([0], [[10.0, 10.0, 10.0]]) == 1       # an empty box
    assert create([100, -1], [[10.0] * 3, [10.0] * 3]) == 1
    assert create([100], [[100.0, 100.0, 100.0]]) == 3  # 34^3 cells > the per-box limit
    assert not h.value
    assert L.mdg_batch_set_inner(None, 1) == 1
    assert L.mdg_batch_set_shape(None, 512, 1, 4) == 1


def test_noalloc_limits_checked_before_device_use(lib):
    # a huge box over a tiny cut-off would overflow the cell count; it is
    # refused (MDG_ERR_CAPACITY) before any conversion, product or launch, and
    # state arrays off a 32-byte boundary are refused (MDG_ERR_INVALID).  The
    # pointers are never dereferenced on these paths.
    from mdacp_gb300 import native
    L = native.load()
    aligned, odd = ctypes.c_void_p(0x10000), ctypes.c_void_p(0x10008)
    out = ctypes.c_void_p(0x20000)
    for box in ((1e30, 1e30, 1e30), (3e6, 3e6, 3e6), (2.0 ** 22, 2.0 ** 22, 2.0 ** 22), (600.0, 600.0, 600.0)):
        b = (ctypes.c_double * 3)(*box)
        assert L.mdg_observe_noalloc(aligned, aligned, 100, b, 1e-3 if box[0] > 1e6 else 1.0, out, None) == 3
    b = (ctypes.c_double * 3)(20.0, 20.0, 20.0)
    assert L.mdg_observe_noalloc(odd, aligned, 100, b, 2.5, out, None) == 1
    assert L.mdg_observe_noalloc(aligned, odd, 100, b, 2.5, out, None) == 1
    assert L.mdg_observe_noalloc(aligned, aligned, 100, b, 2.5, ctypes.c_void_p(0x20004), None) == 1
    b = (ctypes.c_double * 3)(float("inf"), 20.0, 20.0)
    assert L.mdg_observe_noalloc(aligned, aligned, 100, b, 2.5, out, None) == 1


def test_create_refuses_huge_boxes_before_device_use(lib):
    from mdacp_gb300 import native
    L = native.load()
    p = native.Params()
    L.mdg_params_default(ctypes.byref(p))
    p.capacity = 100
    h = ctypes.c_void_p()
    for side in (1e30, 2.0 ** 40, float("inf")):
        p.box[0] = side
        assert L.mdg_create(ctypes.byref(p), ctypes.byref(h)) == 1
        assert not h.value
        assert b"cells" in L.mdg_last_error(None)
