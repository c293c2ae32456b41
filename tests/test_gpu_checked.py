"""The bounds-checked build (libmdg_check.so, -DMDG_CHECK=1) on the parity cases.

Every gather and scatter index of the single-box path is checked on the
device; a failed check would stop the run with MDG_ERR_STATE "bounds check
failed (site, index)".  The cases run in a child process that loads the
checked library (MDG_LIBRARY=check): pair set and FP64 forces against the
oracle, NVE traces in both forms with frequent inner-list re-selection, a list
overflow and its regrowth, Langevin and the observers.  Nothing is corrupted
on purpose: the checks must simply never fire on valid runs.
"""
import os
import subprocess
import sys

import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

CASES = r'''
import sys
sys.path.insert(0, sys.argv[1])
import numpy as np
from mdacp_gb300 import native
from mdacp_gb300.manager import MDManager
from oracle import port
from tests.helpers import directed_pair_keys, liquid_like
lib = native.load()
assert lib._name.endswith("libmdg_check.so"), lib._name
RC, MARGIN = 2.5, 0.5

def gpu(L, n, **kw):
    return MDManager(L, capacity=n, cutoff=RC, margin=MARGIN, **kw)

q, p, L = liquid_like(0.8, 8, seed=3)
ref = port.System(q, p, L, rc=RC, margin=MARGIN)
ref.make_pairlist()
m = gpu(L, len(q))
m.set_state(q, p)
m.make_pairlist()
assert np.array_equal(directed_pair_keys(m.pairs(), len(q), half=False), directed_pair_keys(ref.pairs(), len(q), half=True))
fr = ref.forces()
assert np.linalg.norm(m.forces() - fr) <= 1e-12 * np.linalg.norm(fr)

q, p, L = liquid_like(0.5, 10, seed=4)
for prec in ("fp64", "mixed"):
    ref = port.System(q, p, L, rc=RC, margin=MARGIN)
    ref.make_pairlist()
    m = gpu(L, len(q), precision=prec, prune_buffer=0.02)
    m.set_state(q, p)
    m.calculate(150)
    ref.calculate(150)
    tol = 1e-10 if prec == "fp64" else 1e-5
    np.testing.assert_allclose(m.observe(), ref.observe(), rtol=tol, atol=tol)
    assert m.stats()["prunes"] > m.stats()["rebuilds"]

m = gpu(L, len(q), list_capacity=8)
m.set_state(q, p)
m.calculate(20)
assert m.stats()["list_capacity"] > 8

m = gpu(L, len(q), dt=0.005, thermostat="langevin", temperature=0.9, gamma=1.0, seed=7, precision="mixed")
m.set_state(q, p)
m.calculate(200)
assert np.isfinite(m.observe()).all()
print("checked cases ok")
'''


def test_checked_build_runs_the_parity_cases():
    from mdacp_gb300 import build
    build.build(check=True)
    r = subprocess.run([sys.executable, "-c", CASES, ROOT], env=dict(os.environ, MDG_LIBRARY="check"),
                       capture_output=True, text=True, timeout=1200, cwd=ROOT)
    assert r.returncode == 0, r.stdout[-3000:] + r.stderr[-3000:]
    assert "checked cases ok" in r.stdout
