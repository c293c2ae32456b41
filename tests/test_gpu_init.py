"""Device initial conditions against the reference's own makers.

tests/golden/makers.npz holds the states the reference wrote (made by
tests/golden/make_golden.py): ConfigurationMaker (confmaker.cc:9-44) and
ExtractConfigurationMaker (confmaker.cc:174-252, mt19937(0) deletions), then
MDManager::SetInitialVelocity(1.5) (variables.cc:82-108); and the set-up of
the reference's Collision::Run (two BallAdder balls, collision.cc:8-63) and
Burst::Run (DropletMaker + SetInitialVelocity, burst.cc:10-61,103-109).
Positions must be bit-identical in the same order; velocities come from the
device's cos/sin and a parallel mean, so they agree to rounding (the
collision balls' +-speed exactly).  The droplet is also checked against a
numpy restatement of its loop.
"""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = np.load(os.path.join(HERE, "golden", "makers.npz"))


def _made(L, maker, rho, v0=1.5, radius=0.0, capacity=None):
    from mdacp_gb300.manager import MDManager
    m = MDManager(L, capacity=capacity or 20000, cutoff=2.5, margin=0.5, dt=0.001)
    m.make_state(maker, rho, radius=radius, v0=v0)
    q, p = m.state()
    m.close()
    return q, p


@pytest.mark.parametrize("k", range(len(GOLD["makers"])))
def test_makers_match_reference(k):
    maker = str(GOLD["makers"][k])
    q, p = _made(GOLD["L%d" % k], maker, float(GOLD["rho%d" % k]), v0=float(GOLD["v0%d" % k]),
                 radius=float(GOLD["radius%d" % k]))
    qr, pr = GOLD["q%d" % k], GOLD["p%d" % k]
    assert q.shape == qr.shape
    assert np.array_equal(q, qr), np.abs(q - qr).max()
    if maker == "collision":
        assert np.array_equal(p, pr)
    else:
        np.testing.assert_allclose(p, pr, rtol=0, atol=1e-13)
        assert np.abs(p.mean(axis=0)).max() < 1e-13


def test_droplet_matches_restated_loop():
    L, rho, radius = 20.0, 0.6, 6.5
    s = 1.0 / (rho * 0.25) ** (1.0 / 3.0)
    hs, e, c = s * 0.5, 0.0000001, L * 0.5
    n = int(L / s)
    ref = []
    for iz in range(n):          # burst.cc:30-60, site order and rounding
        for iy in range(n):
            for ix in range(n):
                for dx, dy, dz in ((0, 0, 0), (0, 1, 1), (1, 0, 1), (1, 1, 0)):
                    x = [ix * s + hs + e if dx else ix * s + e, iy * s + hs + e if dy else iy * s + e,
                         iz * s + hs + e if dz else iz * s + e]
                    ddx, ddy, ddz = x[0] - c, x[1] - c, x[2] - c
                    if ddx * ddx + ddy * ddy + ddz * ddz < radius * radius:
                        ref.append(x)
    ref = np.array(ref)
    q, p = _made(L, "droplet", rho, v0=0.0, radius=radius)
    assert np.array_equal(q, ref)
    assert not p.any()


def test_capacity_is_reported():
    from mdacp_gb300.manager import MDManager
    from mdacp_gb300.native import MDGError
    m = MDManager(10.0, capacity=100, cutoff=2.5, margin=0.5, dt=0.001)
    with pytest.raises(MDGError):
        m.make_state("fcc", 0.5)
    m.close()


def test_made_state_runs_like_the_oracle():
    # the made state steps like any other: 200 NVE steps against the oracle
    # (ConfigurationMaker; extract lattices put sites exactly on the box faces,
    # where the reference's ghost search misses images until the first rebuild)
    from oracle import port
    q, p = _made(12.0, "fcc", 0.5, v0=1.2)
    from mdacp_gb300.manager import MDManager
    m = MDManager(12.0, capacity=len(q), cutoff=2.5, margin=0.5, dt=0.001)
    m.set_state(q, p)
    m.calculate(200)
    s = port.System(q, p, 12.0, rc=2.5, margin=0.5, dt=0.001)
    s.make_pairlist()
    s.calculate(200)
    np.testing.assert_allclose(m.observe(), s.observe(), rtol=1e-10, atol=1e-12)
    m.close()
