"""Generates the golden fixtures of tests/golden/ by running the MDACP reference itself.

The reference binary is built from the reference sources by oracle/build_ref.sh
(rc = 2.5 via the generated mdconfig header, margin via OracleBufferLength).
Each fixture stores the injected input and the reference's outputs:

  c1_small.npz   2048 atoms (8^3 FCC at density 0.5, displaced by up to 0.15,
                 L = 16): half pair list (key id, partner id, image code) in the
                 reference's order, forces (p after one CalculateForce at dt=1),
                 PE and virial sums, E/T/P trace over 100 NVE steps every 10,
                 final state.
  rho08.npz      864 atoms (6^3 FCC at density 0.8): forces, observables, trace.
  langevin.npz   2048 atoms, the reference's Langevin project at T=0.9,
                 gamma=1.0, dt=0.005, Seed=12345 (mt19937 noise): temperature
                 trace over 3000 steps, for statistical comparison.
  io_small.npz   108 atoms: the bytes of the reference's writers for the
                 loaded state (SaveAsDumpFile, SaveAsCdview with type = input
                 index, MDUnit::SaveConfiguration, Variables::SaveToStream).
  makers.npz     the reference's ConfigurationMaker and ExtractConfigurationMaker
                 states (positions, then MDManager::SetInitialVelocity(1.5)) for
                 a few boxes and densities, in the unit's particle order.

Run from the repository root: python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import refrun  # noqa: E402
from tests.helpers import liquid_like  # noqa: E402

RC, MARGIN = 2.5, 0.5


def nve_fixture(name, density, cells, seed, steps=100, every=10):
    q, p, L = liquid_like(density, cells, seed=seed)
    pairs = refrun.run("pairs", q, p, L, rc=RC, margin=MARGIN)["pairs"]
    fo = refrun.run("force", q, p, L, rc=RC, margin=MARGIN)
    tr = refrun.run("trace", q, p, L, rc=RC, margin=MARGIN, dt=0.001, steps=steps, observe_every=every)
    np.savez_compressed(os.path.join(HERE, name), q=q, p=p, L=L, rc=RC, margin=MARGIN, dt=0.001,
                        pairs=pairs.astype(np.int32), force=fo["force"], obs=fo["obs"], trace=tr["trace"],
                        q_final=tr["q"], p_final=tr["p"], steps=steps, every=every)


def langevin_fixture():
    q, p, L = liquid_like(0.5, 8, seed=77, temperature=1.0)
    extra = {"ControlTemperature": "yes", "HeatbathType": "Langevin", "AimedTemperature": 0.9,
             "HeatbathGamma": 1.0, "Seed": 12345}
    tr = refrun.run("trace", q, p, L, rc=RC, margin=MARGIN, dt=0.005, steps=3000, observe_every=10, extra=extra)
    np.savez_compressed(os.path.join(HERE, "langevin"), q=q, p=p, L=L, rc=RC, margin=MARGIN, dt=0.005,
                        temperature=0.9, gamma=1.0, trace=tr["trace"])


def io_fixture():
    q, p, L = liquid_like(0.5, 3, seed=5)
    o = refrun.run("write", q, p, L, rc=RC, margin=MARGIN)
    blobs = {k: np.frombuffer(o[k], dtype=np.uint8) for k in ("dump", "cdview", "configuration", "stream")}
    np.savez_compressed(os.path.join(HERE, "io_small"), q=q, p=p, L=L, **blobs)


# (maker, box, density, radius, v0): v0 is SetInitialVelocity's speed, or the
# balls' speed for the collision maker (Collision::Run fixes it at 1.0, the
# radius at L_y / 4 and the density at 0.374, collision.cc:55-63)
MAKER_CASES = [("fcc", (10.0, 10.0, 10.0), 0.5, 0.0, 1.5), ("fcc", (10.0, 12.0, 11.0), 0.8, 0.0, 1.5),
               ("extract", (10.0,) * 3, 0.5, 0.0, 1.5), ("extract", (23.7,) * 3, 0.8, 0.0, 1.5),
               ("extract", (30.0,) * 3, 0.5, 0.0, 1.5),
               ("collision", (60.0, 30.0, 30.0), 0.374, 7.5, 1.0), ("collision", (50.0, 40.0, 36.0), 0.374, 10.0, 1.0),
               ("droplet", (20.0,) * 3, 0.6, 6.5, 1.5), ("droplet", (26.0,) * 3, 0.5, 9.0, 1.5)]


def makers_fixture():
    """Positions and velocities the reference's makers produce: its
    ConfigurationMaker / ExtractConfigurationMaker + SetInitialVelocity, and
    its Collision::Run / Burst::Run set-up (loops at zero)."""
    out = {}
    dummy = np.zeros((1, 3))
    for k, (maker, L, rho, radius, v0) in enumerate(MAKER_CASES):
        extra = {"OracleMaker": maker, "Density": rho, "InitialVelocity": v0, "TotalLoop": 0,
                 "ThermalizeLoop": 0, "Radius": radius}
        o = refrun.run("make", dummy, dummy, np.array(L), rc=RC, margin=MARGIN, extra=extra)
        out["q%d" % k], out["p%d" % k] = o["q"], o["p"]
        out["L%d" % k], out["rho%d" % k] = np.array(L), rho
        out["radius%d" % k], out["v0%d" % k] = radius, v0
    np.savez_compressed(os.path.join(HERE, "makers"), makers=np.array([c[0] for c in MAKER_CASES]), **out)


if __name__ == "__main__":
    if not refrun.available(RC):
        refrun.build()
    nve_fixture("c1_small", 0.5, 8, seed=1)
    nve_fixture("rho08", 0.8, 6, seed=2)
    langevin_fixture()
    io_fixture()
    makers_fixture()
    for f in sorted(os.listdir(HERE)):
        if f.endswith(".npz"):
            print(f, os.path.getsize(os.path.join(HERE, f)))
