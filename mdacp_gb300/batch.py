"""Batched replica boxes through the C ABI (mdg_batch_* in include/mdg.h).

Also builds the batched workload: boxes with N drawn uniformly from a range,
each an FCC lattice filled to ceil((N/4)^(1/3))^3 unit cells and thinned to N
sites by a seeded permutation, density and temperature drawn uniformly.
"""
import ctypes

import numpy as np

from . import lattice, native


class BatchParams(ctypes.Structure):
    _fields_ = [("precision", ctypes.c_int32), ("device", ctypes.c_int32), ("cutoff", ctypes.c_double),
                ("margin", ctypes.c_double), ("dt", ctypes.c_double), ("list_capacity", ctypes.c_int32),
                ("use_graphs", ctypes.c_int32), ("prune_buffer", ctypes.c_double)]


class BatchStats(ctypes.Structure):
    _fields_ = [("steps", ctypes.c_int64), ("rebuilds", ctypes.c_int64), ("particles", ctypes.c_int64),
                ("boxes", ctypes.c_int32), ("list_capacity", ctypes.c_int32), ("threads", ctypes.c_int32),
                ("lanes_per_particle", ctypes.c_int32), ("ctas_per_sm", ctypes.c_int32), ("inner_list", ctypes.c_int32),
                ("elapsed_ms", ctypes.c_double), ("kernel_launches", ctypes.c_int64), ("flat", ctypes.c_int32),
                ("reserved", ctypes.c_int32), ("prune_buffer", ctypes.c_double)]


_P = ctypes.c_void_p
_D = ctypes.POINTER(ctypes.c_double)
_I = ctypes.POINTER(ctypes.c_int32)
SIGNATURES = {
    "mdg_batch_params_default": (None, [ctypes.POINTER(BatchParams)]),
    "mdg_batch_create": (ctypes.c_int, [ctypes.POINTER(BatchParams), ctypes.c_int32, _I, _D, ctypes.POINTER(_P)]),
    "mdg_batch_destroy": (ctypes.c_int, [_P]),
    "mdg_batch_last_error": (ctypes.c_char_p, [_P]),
    "mdg_batch_set_state": (ctypes.c_int, [_P, _D, _D]),
    "mdg_batch_get_state": (ctypes.c_int, [_P, _D, _D]),
    "mdg_batch_calculate": (ctypes.c_int, [_P, ctypes.c_int32]),
    "mdg_batch_observe": (ctypes.c_int, [_P, _D]),
    "mdg_batch_tune": (ctypes.c_int, [_P, ctypes.c_int32, _I, _I, _I]),
    "mdg_batch_set_shape": (ctypes.c_int, [_P, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32]),
    "mdg_batch_set_inner": (ctypes.c_int, [_P, ctypes.c_int32]),
    "mdg_batch_set_flat": (ctypes.c_int, [_P, ctypes.c_int32]),
    "mdg_batch_get_stats": (ctypes.c_int, [_P, ctypes.POINTER(BatchStats)]),
}


def _lib():
    lib = native.load()
    if not getattr(lib, "_mdg_batch_declared", False):
        for name, (res, args) in SIGNATURES.items():
            f = getattr(lib, name)
            f.restype = res
            f.argtypes = args
        lib._mdg_batch_declared = True
    return lib


def _dp(a):
    return a.ctypes.data_as(_D)


def make_replicas(nbox, seed=1, n_range=(500, 8000), rho_range=(0.3, 0.9), t_range=(0.7, 1.5)):
    """Returns (list of (q, p, L)) for nbox boxes drawn as the batched workload."""
    u = lattice.uniform53(seed, 3 * nbox, 21).reshape(nbox, 3)
    boxes = []
    for b in range(nbox):
        n = int(n_range[0] + u[b, 0] * (n_range[1] - n_range[0] + 1))
        n = min(max(n, n_range[0]), n_range[1])
        rho = rho_range[0] + u[b, 1] * (rho_range[1] - rho_range[0])
        T = t_range[0] + u[b, 2] * (t_range[1] - t_range[0])
        cells = int(np.ceil((n / 4.0) ** (1.0 / 3.0) - 1e-12))
        L = (4 * cells ** 3 / rho) ** (1.0 / 3.0)
        q, Lv = lattice.fcc(4 * cells ** 3 / L ** 3, L, cells=cells)
        q = lattice.thin(q, n, seed * 100003 + b)
        p = lattice.maxwell(n, T, seed * 7919 + b)
        boxes.append((q, p, Lv))
    return boxes


class Batch:
    def __init__(self, boxes, cutoff=2.5, margin=0.4, dt=0.002, precision="fp64", list_capacity=0, device=0,
                 use_graphs=True, prune_buffer=None):
        self.lib = _lib()
        prm = BatchParams()
        self.lib.mdg_batch_params_default(ctypes.byref(prm))
        prm.precision = native.PRECISIONS[precision]
        prm.device, prm.cutoff, prm.margin, prm.dt = device, cutoff, margin, dt
        prm.list_capacity, prm.use_graphs = list_capacity, 1 if use_graphs else 0
        if prune_buffer is not None:
            prm.prune_buffer = prune_buffer
        self.n = np.array([len(b[0]) for b in boxes], dtype=np.int32)
        Ls = np.ascontiguousarray(np.array([np.broadcast_to(b[2], (3,)) for b in boxes], dtype=np.float64))
        self.L = Ls
        h = ctypes.c_void_p()
        rc = self.lib.mdg_batch_create(ctypes.byref(prm), len(boxes), self.n.ctypes.data_as(_I), _dp(Ls),
                                       ctypes.byref(h))
        native.check(rc)
        self._h = h
        self.offsets = np.concatenate([[0], np.cumsum(self.n)])
        q4 = np.zeros((self.offsets[-1], 4))
        p4 = np.zeros((self.offsets[-1], 4))
        for k, (q, p, _) in enumerate(boxes):
            q4[self.offsets[k]:self.offsets[k + 1], :3] = q
            p4[self.offsets[k]:self.offsets[k + 1], :3] = p
        self._ck(self.lib.mdg_batch_set_state(self._h, _dp(q4), _dp(p4)))

    def _ck(self, rc):
        if rc != 0:
            raise native.MDGError("%s: %s" % (native.ERRORS.get(rc, rc), self.lib.mdg_batch_last_error(self._h).decode()))

    def close(self):
        if getattr(self, "_h", None):
            self.lib.mdg_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def calculate(self, nsteps):
        self._ck(self.lib.mdg_batch_calculate(self._h, int(nsteps)))

    def observe_raw(self):
        out = np.zeros((len(self.n), 3))
        self._ck(self.lib.mdg_batch_observe(self._h, _dp(out)))
        return out

    def state(self):
        q4 = np.zeros((self.offsets[-1], 4))
        p4 = np.zeros((self.offsets[-1], 4))
        self._ck(self.lib.mdg_batch_get_state(self._h, _dp(q4), _dp(p4)))
        return [(q4[a:b, :3], p4[a:b, :3]) for a, b in zip(self.offsets[:-1], self.offsets[1:])]

    def tune(self, trial_steps=20):
        t, lp, c = ctypes.c_int32(), ctypes.c_int32(), ctypes.c_int32()
        self._ck(self.lib.mdg_batch_tune(self._h, int(trial_steps), ctypes.byref(t), ctypes.byref(lp),
                                         ctypes.byref(c)))
        return t.value, lp.value, c.value

    def set_inner(self, on):
        """One lane per particle walks the inner list (True) or every listed pair."""
        self._ck(self.lib.mdg_batch_set_inner(self._h, 1 if on else 0))

    def set_shape(self, threads, lanes, ctas_per_sm):
        self._ck(self.lib.mdg_batch_set_shape(self._h, threads, lanes, ctas_per_sm))

    def set_flat(self, on):
        """Flat layout of the step (the grid strides over every box's particles)
        or each CTA stepping its own boxes (False)."""
        self._ck(self.lib.mdg_batch_set_flat(self._h, 1 if on else 0))

    def stats(self):
        s = BatchStats()
        self._ck(self.lib.mdg_batch_get_stats(self._h, ctypes.byref(s)))
        return {f: getattr(s, f) for f, _ in BatchStats._fields_}
