"""The oracle (C restatement of the reference) pinned against the reference itself.

Golden fixtures (tests/golden/*.npz, made by make_golden.py from the reference
binary) must be reproduced bit for bit; when the reference binary is built
here, larger cases are compared live.  Independent checks: mesh search against
brute force, invariance under particle order, Philox known answers.
"""
import os

import numpy as np
import pytest

from oracle import port, refrun
from tests.helpers import directed_pair_keys, liquid_like

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def _fixture(name):
    return dict(np.load(os.path.join(GOLDEN, name + ".npz")))


def _trace(sys_, steps, every):
    rows = [sys_.observe()]
    for _ in range(steps // every):
        sys_.calculate(every)
        rows.append(sys_.observe())
    return np.array(rows)


@pytest.mark.parametrize("name", ["c1_small", "rho08"])
def test_port_reproduces_golden_bitwise(name):
    g = _fixture(name)
    s = port.System(g["q"], g["p"], g["L"], rc=float(g["rc"]), margin=float(g["margin"]), dt=float(g["dt"]))
    s.make_pairlist()
    if name == "c1_small":
        assert np.array_equal(s.pairs(), g["pairs"])
    assert np.array_equal(s.forces(), g["force"])
    ke, pe, vir = s.observe_raw()
    assert pe == g["obs"][0] and vir == g["obs"][1]
    tr = _trace(s, int(g["steps"]), int(g["every"]))
    assert np.array_equal(tr, g["trace"][:, 1:])
    qf, pf = s.state()
    assert np.array_equal(qf, g["q_final"]) and np.array_equal(pf, g["p_final"])


def test_golden_forces_are_not_trivial():
    g = _fixture("c1_small")
    assert np.abs(g["force"]).max() > 1.0
    assert len(g["pairs"]) > 20 * len(g["q"])


@pytest.mark.skipif(not refrun.available(2.5), reason="reference binary not built (oracle/build_ref.sh)")
@pytest.mark.parametrize("density,cells", [(0.5, 20), (0.8, 10)])
def test_port_matches_reference_live(density, cells):
    q, p, L = liquid_like(density, cells, seed=3 * cells)
    ref_pairs = refrun.run("pairs", q, p, L)["pairs"]
    ref_force = refrun.run("force", q, p, L)["force"]
    ref = refrun.run("trace", q, p, L, steps=100, observe_every=20)
    s = port.System(q, p, L, rc=2.5, margin=0.5)
    s.make_pairlist()
    assert np.array_equal(s.pairs(), ref_pairs)
    assert np.array_equal(s.forces(), ref_force)
    assert np.array_equal(_trace(s, 100, 20), ref["trace"][:, 1:])
    qf, pf = s.state()
    assert np.array_equal(qf, ref["q"]) and np.array_equal(pf, ref["p"])


@pytest.mark.skipif(not refrun.available(2.5), reason="reference binary not built (oracle/build_ref.sh)")
@pytest.mark.parametrize("density,cells", [(0.5, 10), (0.8, 8)])
def test_port_matches_reference_over_many_rebuilds(density, cells):
    """1,000 steps: the buffer-length countdown, the candidate-pair check and
    the rebuilds they trigger (PairList::UpdatePairListValidity,
    PairList::CheckByDisplacement, pairlist.cc:48-100; MDManager::Calculate,
    mdmanager.cc:116-126) fall on the same steps as the reference's, or the
    final state would not be bit-equal."""
    q, p, L = liquid_like(density, cells, seed=7 * cells)
    ref = refrun.run("trace", q, p, L, steps=1000, observe_every=100)
    s = port.System(q, p, L, rc=2.5, margin=0.5)
    s.make_pairlist()
    assert np.array_equal(_trace(s, 1000, 100), ref["trace"][:, 1:])
    qf, pf = s.state()
    assert np.array_equal(qf, ref["q"]) and np.array_equal(pf, ref["p"])
    assert s.rebuilds >= 10


@pytest.mark.skipif(not refrun.available(3.0), reason="reference binary not built (oracle/build_ref.sh)")
def test_port_matches_unpatched_reference_cutoff():
    """The reference's own compile-time constants: rc = 3.0, margin 0.3."""
    q, p, L = liquid_like(0.5, 10, seed=8)
    ref = refrun.run("force", q, p, L, rc=3.0, margin=0.3)["force"]
    s = port.System(q, p, L, rc=3.0, margin=0.3)
    s.make_pairlist()
    assert np.array_equal(s.forces(), ref)


@pytest.mark.parametrize("density,cells", [(0.5, 6), (0.8, 6)])
def test_mesh_search_equals_bruteforce(density, cells):
    q, p, L = liquid_like(density, cells, seed=4)
    s = port.System(q, p, L, rc=2.5, margin=0.5)
    s.make_pairlist()
    mesh = directed_pair_keys(s.pairs(), len(q), half=True)
    brute = directed_pair_keys(port.bruteforce_pairs(q, L, 3.0), len(q), half=False)
    assert np.array_equal(mesh, brute)


def test_order_invariance():
    """Variables::Shuffle (variables.cc:145-172) as a cross-check: same physics in any order."""
    q, p, L = liquid_like(0.5, 8, seed=6)
    perm = np.random.default_rng(0).permutation(len(q))
    a = port.System(q, p, L)
    b = port.System(q[perm], p[perm], L)
    a.make_pairlist()
    b.make_pairlist()
    ka = directed_pair_keys(a.pairs(), len(q))
    inv = np.argsort(perm)
    rb = b.pairs().astype(np.int64)
    rb[:, 0] = perm[rb[:, 0]]
    rb[:, 1] = perm[rb[:, 1]]
    assert np.array_equal(ka, directed_pair_keys(rb, len(q)))
    fa, fb = a.forces(), b.forces()[inv]
    assert np.abs(fa - fb).max() <= 1e-12 * np.abs(fa).max()


def test_philox_known_answers():
    import ctypes
    lib = port.lib()
    lib.orc_philox4x32_10.argtypes = [ctypes.POINTER(ctypes.c_uint32)] * 3

    def philox(c, k):
        C, K, O = (ctypes.c_uint32 * 4)(*c), (ctypes.c_uint32 * 2)(*k), (ctypes.c_uint32 * 4)()
        lib.orc_philox4x32_10(C, K, O)
        return list(O)

    assert philox([0, 0, 0, 0], [0, 0]) == [0x6627e8d5, 0xe169c58d, 0xbc57ac4c, 0x9b00dbd8]
    assert philox([0xffffffff] * 4, [0xffffffff] * 2) == [0x408f276d, 0x41c83b0e, 0xa20bc7c6, 0x6d5451fd]
    assert philox([0x243f6a88, 0x85a308d3, 0x13198a2e, 0x03707344], [0xa4093822, 0x299f31d0]) == [
        0xd16cfe09, 0x94fdcceb, 0x5001e420, 0x24126ea1]


def test_langevin_normals_are_standard():
    z = np.array([port.langevin_normals(99, i, s) for i in range(400) for s in range(25)]).ravel()
    assert abs(z.mean()) < 0.03 and abs(z.std() - 1.0) < 0.03


def test_langevin_statistics_match_reference():
    """Philox noise (oracle/GPU) vs the reference's mt19937 stream: same thermostat statistics."""
    g = _fixture("langevin")
    s = port.System(g["q"], g["p"], g["L"], rc=2.5, margin=0.5, dt=float(g["dt"]), thermostat=port.LANGEVIN,
                    temperature=float(g["temperature"]), gamma=float(g["gamma"]), seed=12345)
    s.make_pairlist()
    T = []
    for _ in range(300):
        s.calculate(10)
        T.append(s.observe()[0])
    T = np.array(T)
    Tr = g["trace"][1:, 1]
    half = len(T) // 2
    m, mr = T[half:].mean(), Tr[half:].mean()
    se = np.sqrt(T[half:].var() / (len(T) / 20) + Tr[half:].var() / (len(Tr) / 20))
    assert abs(m - mr) < 4 * se + 1e-3, (m, mr, se)
    assert abs(mr - 0.9) < 0.05 and abs(m - 0.9) < 0.05


def test_nosehoover_relaxes_temperature():
    q, p, L = liquid_like(0.5, 6, seed=9, temperature=1.5)
    s = port.System(q, p, L, thermostat=port.NOSEHOOVER, temperature=1.0, tau=0.1, dt=0.002)
    s.make_pairlist()
    s.calculate(2000)
    assert abs(s.observe()[0] - 1.0) < 0.2


def test_maker_restatement_matches_reference_fixture():
    # oracle/makers.cc against the states the reference's own makers wrote
    gold = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "makers.npz"))
    for k, maker in enumerate(gold["makers"]):
        q, p = port.make_state(str(maker), gold["L%d" % k], float(gold["rho%d" % k]), float(gold["radius%d" % k]),
                               float(gold["v0%d" % k]))
        assert np.array_equal(q, gold["q%d" % k]), maker
        np.testing.assert_allclose(p, gold["p%d" % k], rtol=0, atol=1e-15)
