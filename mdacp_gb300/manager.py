"""Host-side mirror of MDACP's MDManager for one periodic box on one GPU.

Method names follow the reference (mdmanager.h:32-83): MakePairList ->
make_pairlist, Calculate -> calculate, Temperature / Pressure / TotalEnergy /
KineticEnergy / PotentialEnergy, SetSeed, SetControlTemperature,
SetAimedTemperature, GetTotalParticleNumber.  Every call goes through the C
ABI of libmdg.so (include/mdg.h); nothing here computes physics.
"""
import ctypes

import numpy as np

from . import native
from .config import Parameter, SimulationInfo


def _dp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _as4(x):
    """[n][4] float64 rows; a C-contiguous [n][4] float64 array (pinned host
    memory included) is passed on as it is."""
    if isinstance(x, np.ndarray) and x.dtype == np.float64 and x.ndim == 2 and x.shape[1] == 4 \
            and x.flags.c_contiguous:
        return x
    x = np.asarray(x, dtype=np.float64)
    out = np.zeros((len(x), 4), dtype=np.float64)
    out[:, :3] = x[:, :3]
    return out


class MDManager:
    def __init__(self, box, capacity=None, cutoff=3.0, margin=0.3, dt=0.001, precision="fp64",
                 thermostat="nve", temperature=1.0, gamma=0.1, tau=0.1, seed=1, langevin_half_drift_compat=True,
                 list_capacity=0, device=0, use_graphs=True, n=None, prune_buffer=None,
                 rebuild_policy="halfmargin", check_list_length=500):
        self.lib = native.load()
        prm = native.Params()
        self.lib.mdg_params_default(ctypes.byref(prm))
        box = np.broadcast_to(np.asarray(box, dtype=np.float64), (3,))
        prm.box[:] = [float(v) for v in box]
        prm.capacity = int(capacity or n or 1000000)
        prm.cutoff, prm.margin, prm.dt = float(cutoff), float(margin), float(dt)
        prm.precision = native.PRECISIONS[precision]
        prm.thermostat = {"nve": native.NVE, "langevin": native.LANGEVIN, "nosehoover": native.NOSEHOOVER}[thermostat]
        prm.temperature, prm.gamma, prm.tau = float(temperature), float(gamma), float(tau)
        prm.seed = int(seed)
        prm.langevin_half_drift_compat = 1 if langevin_half_drift_compat else 0
        prm.list_capacity = int(list_capacity)
        prm.device = int(device)
        prm.use_graphs = 1 if use_graphs else 0
        if prune_buffer is not None:
            prm.prune_buffer = float(prune_buffer)
        prm.rebuild_policy = native.REBUILD_POLICIES[rebuild_policy]
        prm.check_list_length = int(check_list_length)
        self.params = prm
        self.L = np.array(prm.box[:])
        h = ctypes.c_void_p()
        native.check(self.lib.mdg_create(ctypes.byref(prm), ctypes.byref(h)), create=True)
        self._h = h
        self.n = 0

    @classmethod
    def from_cfg(cls, param, n, **overrides):
        """Builds a manager from .cfg keys (SimulationInfo semantics plus the mdg keys)."""
        if not isinstance(param, Parameter):
            param = Parameter.from_file(param)
        si = SimulationInfo(param)
        kw = dict(box=si.L, capacity=n, cutoff=si.cutoff, margin=si.buffer_length, dt=si.time_step,
                  precision=si.precision, thermostat=si.thermostat, temperature=si.aimed_temperature,
                  gamma=si.heatbath_gamma, tau=si.heatbath_tau, seed=param.get_int("Seed", 1),
                  langevin_half_drift_compat=si.langevin_half_drift_compat, device=si.device,
                  rebuild_policy=si.rebuild_policy, check_list_length=si.check_list_length)
        kw.update(overrides)
        return cls(**kw)

    def close(self):
        if getattr(self, "_h", None):
            self.lib.mdg_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _ck(self, rc):
        native.check(rc, self._h)

    # state ---------------------------------------------------------------
    def set_state(self, q, p):
        q4, p4 = _as4(q), _as4(p)
        self.n = len(q4)
        self._ck(self.lib.mdg_set_state(self._h, _dp(q4), _dp(p4), self.n))

    def state(self, q4=None, p4=None):
        """Positions and momenta in the caller's order, as [n][3] views of
        [n][4] buffers; q4/p4 may be given (C-contiguous float64 [n][4], e.g.
        pinned host memory) to receive the state without an allocation."""
        q4 = np.zeros((self.n, 4)) if q4 is None else q4
        p4 = np.zeros((self.n, 4)) if p4 is None else p4
        for x in (q4, p4):
            if x.dtype != np.float64 or x.shape != (self.n, 4) or not x.flags.c_contiguous:
                raise ValueError("state buffers must be C-contiguous float64 [n][4]")
        self._ck(self.lib.mdg_get_state(self._h, _dp(q4), _dp(p4)))
        return q4[:, :3], p4[:, :3]

    def synchronize(self):
        """Waits for the steps calculate() left outstanding and reports their errors."""
        self._ck(self.lib.mdg_synchronize(self._h))

    def make_state(self, maker, density, radius=0.0, v0=0.0):
        """The reference's configuration makers and SetInitialVelocity, on the device.

        maker: "fcc" (ConfigurationMaker, confmaker.cc:9-44), "extract"
        (ExtractConfigurationMaker for one unit spanning the box,
        confmaker.cc:174-252), "droplet" (DropletMaker, burst.cc:10-61, sites
        within `radius` of the centre) or "collision" (the two BallAdder balls
        of Collision::Run, collision.cc:8-63, of `radius`, moving at +v0 and
        -v0 along x).  For the others v0 > 0 draws velocities as
        Variables::SetInitialVelocity(v0, 0) (variables.cc:82-108).
        """
        self._ck(self.lib.mdg_make_state(self._h, native.MAKERS[maker], float(density), float(radius), float(v0)))
        self.n = self.stats()["particles"]

    def save_dump(self, path):
        """MDManager::SaveAsDumpFile of the current state (mdmanager.cc:475-505)."""
        self._ck(self.lib.mdg_save_dump(self._h, str(path).encode()))

    def save_cdview(self, path):
        """MDManager::SaveAsCdview of the current state (mdmanager.cc:90-105)."""
        self._ck(self.lib.mdg_save_cdview(self._h, str(path).encode()))

    # hot path ------------------------------------------------------------
    def make_pairlist(self):
        self._ck(self.lib.mdg_make_pairlist(self._h))

    def calculate(self, nsteps=1):
        self._ck(self.lib.mdg_calculate(self._h, int(nsteps)))

    def calculate_profiled(self, nsteps):
        """Steps as mdg_calculate replays them, with CUDA events around every
        step kernel; returns the summed device ms of the fused step kernel."""
        ms = ctypes.c_double()
        self._ck(self.lib.mdg_calculate_profiled(self._h, int(nsteps), ctypes.byref(ms)))
        return ms.value

    def calculate_phases(self, nsteps):
        """Steps as mdg_calculate_profiled runs them; device ms per phase as the
        reference's StopWatch objects split Calculate: {"force", "pair", "all"}."""
        out = np.zeros(3)
        self._ck(self.lib.mdg_calculate_phases(self._h, int(nsteps), _dp(out)))
        return {"force": out[0], "pair": out[1], "all": out[2]}

    def forces(self):
        f4 = np.zeros((self.n, 4))
        self._ck(self.lib.mdg_forces(self._h, _dp(f4)))
        return f4[:, :3]

    def pairs(self):
        cnt = ctypes.c_int64()
        self._ck(self.lib.mdg_pairs(self._h, None, 0, ctypes.byref(cnt)))
        rec = np.zeros((cnt.value, 3), dtype=np.int32)
        self._ck(self.lib.mdg_pairs(self._h, rec.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)), cnt.value,
                                    ctypes.byref(cnt)))
        return rec

    # observation (mdmanager.cc:390-429) ------------------------------------
    def observe_raw(self):
        out = np.zeros(3)
        self._ck(self.lib.mdg_observe(self._h, _dp(out)))
        return out

    def observe(self):
        """(T, P, E, KE/N, PE/N, virial/N) as MDManager reports them."""
        ke, pe, vir = self.observe_raw()
        n = float(self.n)
        T = ke / n / 1.5
        V = float(self.L[0] * self.L[1] * self.L[2])
        P = (T - vir / n) * n / V
        return np.array([T, P, ke / n + pe / n, ke / n, pe / n, vir / n])

    def temperature(self):
        return self.observe()[0]

    def pressure(self):
        return self.observe()[1]

    def total_energy(self):
        return self.observe()[2]

    def kinetic_energy(self):
        return self.observe()[3]

    def potential_energy(self):
        return self.observe()[4]

    def get_total_particle_number(self):
        return self.n

    # control -------------------------------------------------------------
    def set_seed(self, seed):
        self._ck(self.lib.mdg_set_seed(self._h, int(seed)))

    def set_thermostat(self, thermostat, temperature):
        t = {"nve": native.NVE, "langevin": native.LANGEVIN, "nosehoover": native.NOSEHOOVER}[thermostat]
        self._ck(self.lib.mdg_set_thermostat(self._h, t, float(temperature)))

    def stats(self):
        s = native.Stats()
        self._ck(self.lib.mdg_get_stats(self._h, ctypes.byref(s)))
        return {"steps": s.steps, "rebuilds": s.rebuilds, "list_capacity": s.list_capacity,
                "max_neighbours": s.max_neighbours, "listed_pairs": s.listed_pairs, "cells": tuple(s.cells),
                "particles": s.particles, "zeta": s.zeta, "elapsed_ms": s.elapsed_ms,
                "kernel_launches": s.kernel_launches, "inner_pairs": s.inner_pairs, "prunes": s.prunes}
