"""Adjoint of an NVE trajectory through the C ABI (mdg_adjoint_* in include/mdg.h).

`Adjoint(...).forward(q0, p0)` runs the horizon and returns the objective;
`.backward()` returns dJ/dq0, dJ/dp0, dJ/depsilon, dJ/dsigma.
"""
import ctypes

import numpy as np

from . import native


class AdjointParams(ctypes.Structure):
    _fields_ = [("box", ctypes.c_double * 3), ("cutoff", ctypes.c_double), ("margin", ctypes.c_double),
                ("dt", ctypes.c_double), ("epsilon", ctypes.c_double), ("sigma", ctypes.c_double),
                ("steps", ctypes.c_int32), ("checkpoint_every", ctypes.c_int32), ("objective", ctypes.c_int32),
                ("device", ctypes.c_int32)]


_P = ctypes.c_void_p
_D = ctypes.POINTER(ctypes.c_double)
SIGNATURES = {
    "mdg_adjoint_params_default": (None, [ctypes.POINTER(AdjointParams)]),
    "mdg_adjoint_create": (ctypes.c_int, [ctypes.POINTER(AdjointParams), ctypes.c_int32, ctypes.POINTER(_P)]),
    "mdg_adjoint_destroy": (ctypes.c_int, [_P]),
    "mdg_adjoint_last_error": (ctypes.c_char_p, [_P]),
    "mdg_adjoint_forward": (ctypes.c_int, [_P, _D, _D, _D]),
    "mdg_adjoint_backward": (ctypes.c_int, [_P, _D, _D, _D, _D]),
}
OBJECTIVES = {"pe": 0, "pressure": 1}


def _lib():
    lib = native.load()
    if not getattr(lib, "_mdg_adjoint_declared", False):
        for name, (res, args) in SIGNATURES.items():
            f = getattr(lib, name)
            f.restype = res
            f.argtypes = args
        lib._mdg_adjoint_declared = True
    return lib


def _dp(a):
    return a.ctypes.data_as(_D)


class Adjoint:
    def __init__(self, L, n, steps=200, checkpoint_every=20, dt=0.002, cutoff=2.5, margin=0.5, epsilon=1.0,
                 sigma=1.0, objective="pe", device=0):
        self.lib = _lib()
        prm = AdjointParams()
        self.lib.mdg_adjoint_params_default(ctypes.byref(prm))
        prm.box[:] = [float(x) for x in np.broadcast_to(np.asarray(L, dtype=np.float64), (3,))]
        prm.cutoff, prm.margin, prm.dt = cutoff, margin, dt
        prm.epsilon, prm.sigma = epsilon, sigma
        prm.steps, prm.checkpoint_every = steps, checkpoint_every
        prm.objective = OBJECTIVES[objective]
        prm.device = device
        self.n = n
        h = ctypes.c_void_p()
        native.check(self.lib.mdg_adjoint_create(ctypes.byref(prm), n, ctypes.byref(h)))
        self._h = h

    def _ck(self, rc):
        if rc != 0:
            raise native.MDGError("%s: %s" % (native.ERRORS.get(rc, rc),
                                              self.lib.mdg_adjoint_last_error(self._h).decode()))

    def close(self):
        if getattr(self, "_h", None):
            self.lib.mdg_adjoint_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def forward(self, q0, p0):
        q4 = np.zeros((self.n, 4))
        p4 = np.zeros((self.n, 4))
        q4[:, :3], p4[:, :3] = q0, p0
        J = ctypes.c_double()
        self._ck(self.lib.mdg_adjoint_forward(self._h, _dp(q4), _dp(p4), ctypes.byref(J)))
        return J.value

    def backward(self):
        dq = np.zeros((self.n, 4))
        dp = np.zeros((self.n, 4))
        de, ds = ctypes.c_double(), ctypes.c_double()
        self._ck(self.lib.mdg_adjoint_backward(self._h, _dp(dq), _dp(dp), ctypes.byref(de), ctypes.byref(ds)))
        return dq[:, :3], dp[:, :3], de.value, ds.value
