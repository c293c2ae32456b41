"""ctypes wrapper of the C restatement of the MDACP hot path (test infrastructure only).

The shared library is built by `build()` from mdacp_oracle.c with gcc
(-ffp-contract=off, so its arithmetic rounds like the reference's FMA-free build).
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libmdacp_oracle.so")

NVE, LANGEVIN, NOSEHOOVER = 0, 1, 2
REBUILD_REFERENCE, REBUILD_HALFMARGIN = 0, 1


def build(force=False):
    src = os.path.join(HERE, "mdacp_oracle.c")
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= max(
            os.path.getmtime(src), os.path.getmtime(os.path.join(HERE, "mdacp_oracle.h"))):
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    tmp = LIB + ".tmp%d" % os.getpid()
    subprocess.check_call(["gcc", "-O3", "-std=c11", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off",
                           "-Wall", "-Wno-unused-function", src, "-o", tmp, "-lm"])
    os.replace(tmp, LIB)
    return LIB


MAKERS_LIB = os.path.join(BUILD, "libmdacp_makers.so")


def build_makers(force=False):
    """Builds the C++ restatement of the reference's configuration makers."""
    src = os.path.join(HERE, "makers.cc")
    if not force and os.path.exists(MAKERS_LIB) and os.path.getmtime(MAKERS_LIB) >= os.path.getmtime(src):
        return MAKERS_LIB
    os.makedirs(BUILD, exist_ok=True)
    tmp = MAKERS_LIB + ".tmp%d" % os.getpid()
    subprocess.check_call(["g++", "-O3", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off", "-Wall", src,
                           "-o", tmp])
    os.replace(tmp, MAKERS_LIB)
    return MAKERS_LIB


_makers = None


def _mk():
    global _makers
    if _makers is None:
        lib = ctypes.CDLL(build_makers())
        dp = ctypes.POINTER(ctypes.c_double)
        lib.orc_make_fcc.restype = ctypes.c_long
        lib.orc_make_fcc.argtypes = [dp, ctypes.c_double, dp, ctypes.c_long]
        lib.orc_make_extract.restype = ctypes.c_long
        lib.orc_make_extract.argtypes = [dp, ctypes.c_double, ctypes.c_int, dp, ctypes.c_long]
        lib.orc_make_droplet.restype = ctypes.c_long
        lib.orc_make_droplet.argtypes = [dp, ctypes.c_double, ctypes.c_double, dp, ctypes.c_long]
        lib.orc_make_collision.restype = ctypes.c_long
        lib.orc_make_collision.argtypes = [dp, ctypes.c_double, ctypes.c_double, ctypes.c_double, dp, dp,
                                           ctypes.c_long]
        lib.orc_initial_velocity.restype = None
        lib.orc_initial_velocity.argtypes = [dp, ctypes.c_long, ctypes.c_double, ctypes.c_int]
        _makers = lib
    return _makers


def make_configuration(maker, L, density, unit_id=0):
    """ConfigurationMaker ("fcc") or ExtractConfigurationMaker ("extract") positions, (n, 3)."""
    L3 = np.ascontiguousarray(np.broadcast_to(np.asarray(L, dtype=np.float64), (3,)))
    dp = ctypes.POINTER(ctypes.c_double)
    lib = _mk()
    if maker == "fcc":
        n = lib.orc_make_fcc(L3.ctypes.data_as(dp), density, None, 0)
        q = np.zeros((n, 3))
        lib.orc_make_fcc(L3.ctypes.data_as(dp), density, q.ctypes.data_as(dp), n)
    else:
        n = lib.orc_make_extract(L3.ctypes.data_as(dp), density, unit_id, None, 0)
        q = np.zeros((n, 3))
        lib.orc_make_extract(L3.ctypes.data_as(dp), density, unit_id, q.ctypes.data_as(dp), n)
    return q


def make_state(maker, L, density, radius=0.0, v0=0.0, unit_id=0):
    """(q, p) as the reference sets them up: the maker's positions, then
    SetInitialVelocity(v0, unit_id) ("fcc", "extract", "droplet" as in
    Burst::Run), or the collision balls' own velocities +-v0 along x."""
    L3 = np.ascontiguousarray(np.broadcast_to(np.asarray(L, dtype=np.float64), (3,)))
    dp = ctypes.POINTER(ctypes.c_double)
    lib = _mk()
    if maker == "collision":
        n = lib.orc_make_collision(L3.ctypes.data_as(dp), density, radius, v0, None, None, 0)
        q, p = np.zeros((n, 3)), np.zeros((n, 3))
        lib.orc_make_collision(L3.ctypes.data_as(dp), density, radius, v0, q.ctypes.data_as(dp),
                               p.ctypes.data_as(dp), n)
        return q, p
    if maker == "droplet":
        n = lib.orc_make_droplet(L3.ctypes.data_as(dp), density, radius, None, 0)
        q = np.zeros((n, 3))
        lib.orc_make_droplet(L3.ctypes.data_as(dp), density, radius, q.ctypes.data_as(dp), n)
    else:
        q = make_configuration(maker, L3, density, unit_id)
    p = initial_velocity(len(q), v0, unit_id) if v0 != 0.0 else np.zeros_like(q)
    return q, p


def initial_velocity(n, v0, seed=0):
    """Variables::SetInitialVelocity(v0, seed) momenta, (n, 3)."""
    p = np.zeros((n, 3))
    _mk().orc_initial_velocity(p.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), n, v0, seed)
    return p


class _Params(ctypes.Structure):
    _fields_ = [("L", ctypes.c_double * 3), ("rc", ctypes.c_double), ("margin", ctypes.c_double),
                ("dt", ctypes.c_double), ("gamma", ctypes.c_double), ("temperature", ctypes.c_double),
                ("tau", ctypes.c_double), ("seed", ctypes.c_uint64), ("thermostat", ctypes.c_int),
                ("rebuild_policy", ctypes.c_int), ("check_list_length", ctypes.c_int),
                ("langevin_half_drift_compat", ctypes.c_int), ("threads", ctypes.c_int)]


_lib = None


def lib():
    global _lib
    if _lib is None:
        L = ctypes.CDLL(build())
        P = ctypes.c_void_p
        dp = ctypes.POINTER(ctypes.c_double)
        ip = ctypes.POINTER(ctypes.c_int32)
        L.orc_create.restype = P
        L.orc_create.argtypes = [ctypes.POINTER(_Params), ctypes.c_int, dp]
        L.orc_destroy.argtypes = [P]
        L.orc_make_pairlist.argtypes = [P]
        L.orc_calculate.argtypes = [P]
        L.orc_calculate.restype = ctypes.c_int
        L.orc_observe.argtypes = [P, dp]
        L.orc_forces.argtypes = [P, dp]
        L.orc_pairs.argtypes = [P, ip, ctypes.c_long]
        L.orc_pairs.restype = ctypes.c_long
        L.orc_get_state.argtypes = [P, dp]
        for f in ("orc_particle_count", "orc_ghost_count"):
            getattr(L, f).argtypes = [P]
            getattr(L, f).restype = ctypes.c_int
        L.orc_rebuild_count.argtypes = [P]
        L.orc_rebuild_count.restype = ctypes.c_long
        L.orc_zeta.argtypes = [P]
        L.orc_zeta.restype = ctypes.c_double
        L.orc_lj_constants.argtypes = [ctypes.c_double, dp, dp]
        L.orc_bruteforce_pairs.argtypes = [ctypes.c_int, dp, dp, ctypes.c_double, ip, ctypes.c_long]
        L.orc_bruteforce_pairs.restype = ctypes.c_long
        L.orc_langevin_normals.argtypes = [ctypes.c_uint64, ctypes.c_uint32, ctypes.c_uint64, dp]
        _lib = L
    return _lib


def _dp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def lj_constants(rc):
    c0, c2 = ctypes.c_double(), ctypes.c_double()
    lib().orc_lj_constants(rc, ctypes.byref(c0), ctypes.byref(c2))
    return c0.value, c2.value


def langevin_normals(seed, pid, step):
    z = np.zeros(3)
    lib().orc_langevin_normals(seed, pid, step, _dp(z))
    return z


def bruteforce_pairs(q, L, sl):
    q = np.ascontiguousarray(q[:, :3], dtype=np.float64)
    Lb = np.ascontiguousarray(L, dtype=np.float64)
    n = len(q)
    m = lib().orc_bruteforce_pairs(n, _dp(q), _dp(Lb), sl, None, 0)
    rec = np.zeros((m, 3), dtype=np.int32)
    lib().orc_bruteforce_pairs(n, _dp(q), _dp(Lb), sl, rec.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)), m)
    return rec


class System:
    """One MDACP unit spanning the whole periodic box, restated in C."""

    def __init__(self, q, p, L, rc=2.5, margin=0.5, dt=0.001, thermostat=NVE, gamma=0.1,
                 temperature=1.0, tau=0.1, seed=1, rebuild_policy=REBUILD_REFERENCE,
                 check_list_length=500, langevin_half_drift_compat=1, threads=1):
        q = np.asarray(q, dtype=np.float64)
        p = np.asarray(p, dtype=np.float64)
        self.n = len(q)
        qp = np.ascontiguousarray(np.hstack([q[:, :3], p[:, :3]]))
        prm = _Params()
        prm.L[:] = [float(x) for x in np.broadcast_to(np.asarray(L, dtype=np.float64), (3,))]
        prm.rc, prm.margin, prm.dt = rc, margin, dt
        prm.gamma, prm.temperature, prm.tau, prm.seed = gamma, temperature, tau, seed
        prm.thermostat, prm.rebuild_policy = thermostat, rebuild_policy
        prm.check_list_length, prm.langevin_half_drift_compat = check_list_length, langevin_half_drift_compat
        prm.threads = threads
        self.L = np.array(prm.L[:])
        self._h = lib().orc_create(ctypes.byref(prm), self.n, _dp(qp))

    def close(self):
        if self._h:
            lib().orc_destroy(self._h)
            self._h = None

    __del__ = close

    def make_pairlist(self):
        lib().orc_make_pairlist(self._h)

    def calculate(self, steps=1):
        rebuilt = 0
        for _ in range(steps):
            r = lib().orc_calculate(self._h)
            if r < 0:
                raise RuntimeError("Too fast particles exists. Try smaller time step")
            rebuilt += r
        return rebuilt

    def observe_raw(self):
        out = np.zeros(3)
        lib().orc_observe(self._h, _dp(out))
        return out  # KE sum, PE sum, virial sum / 3

    def observe(self):
        """(T, P, E, KE/N, PE/N, virial/N) as MDManager reports them (mdmanager.cc:390-429)."""
        ke, pe, vir = self.observe_raw()
        n = float(self.n)
        T = ke / n / 1.5
        V = self.L[0] * self.L[1] * self.L[2]
        P = (T - vir / n) * n / V
        return np.array([T, P, ke / n + pe / n, ke / n, pe / n, vir / n])

    def forces(self):
        f = np.zeros((self.n, 3))
        lib().orc_forces(self._h, _dp(f))
        return f

    def pairs(self):
        m = lib().orc_pairs(self._h, None, 0)
        rec = np.zeros((m, 3), dtype=np.int32)
        lib().orc_pairs(self._h, rec.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)), m)
        return rec

    def state(self):
        qp = np.zeros((self.n, 6))
        lib().orc_get_state(self._h, _dp(qp))
        return qp[:, :3].copy(), qp[:, 3:].copy()

    @property
    def ghosts(self):
        return lib().orc_ghost_count(self._h)

    @property
    def rebuilds(self):
        return lib().orc_rebuild_count(self._h)

    @property
    def zeta(self):
        return lib().orc_zeta(self._h)
