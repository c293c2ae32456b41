"""Edge cases of the hot path: tiny and permuted inputs, particles on the box
faces, the smallest cell grids, capacity limits.

The reference has no tests of its own; its debug helpers suggest the checks
(MakeListBruteforce meshlist.cc:90-106 for the pair set, Variables::Shuffle
variables.cc:145-172 for order invariance).  Pair sets are compared bit-exact
with the brute-force enumeration of the oracle; forces within the FP64
tolerance of the parity tests.
"""
import numpy as np
import pytest

from oracle import port
from tests.helpers import directed_pair_keys, liquid_like

pytestmark = pytest.mark.gpu

RC, MARGIN = 2.5, 0.5


def _gpu(L, n, **kw):
    from mdacp_gb300.manager import MDManager
    kw.setdefault("cutoff", RC)
    kw.setdefault("margin", MARGIN)
    return MDManager(L, capacity=n, **kw)


def _lj_force(r):
    """Force factor of the smoothly truncated potential, variables.cc:16-28."""
    c2 = 6.0 / RC ** 14 - 3.0 / RC ** 8
    return 24.0 / r ** 8 - 48.0 / r ** 14 + 8.0 * c2


def test_one_particle_has_no_force_and_no_pairs():
    m = _gpu(8.0, 1)
    m.set_state(np.array([[1.0, 2.0, 3.0]]), np.array([[0.1, 0.0, -0.2]]))
    assert not m.forces().any()
    m.make_pairlist()
    assert len(m.pairs()) == 0
    m.calculate(10)
    q, p = m.state()
    np.testing.assert_allclose(q[0], [1.0 + 10 * 0.001 * 0.1, 2.0, 3.0 - 10 * 0.001 * 0.2], rtol=0, atol=1e-14)


def test_two_particles_across_the_periodic_face():
    L = 8.0
    for r in (1.05, 1.9, 2.49):
        q = np.array([[0.3, 4.0, 4.0], [0.3 - r + L, 4.0, 4.0]])  # the image at x = 0.3 - r
        m = _gpu(L, 2)
        m.set_state(q, np.zeros((2, 3)))
        f = m.forces()
        fx = _lj_force(r) * (-r)  # f(r) (q_j - q_i), q_j - q_i = -r along x
        np.testing.assert_allclose(f[0], [fx, 0.0, 0.0], rtol=1e-13, atol=1e-14)
        np.testing.assert_allclose(f[1], -f[0], rtol=1e-13, atol=1e-14)
        m.close()


def test_beyond_cutoff_gives_zero_force():
    q = np.array([[1.0, 1.0, 1.0], [1.0 + RC + 1e-9, 1.0, 1.0]])
    m = _gpu(12.0, 2)
    m.set_state(q, np.zeros((2, 3)))
    assert not m.forces().any()


def test_permuted_input_same_pairs_and_forces():
    q, p, L = liquid_like(0.5, 8, seed=71)
    n = len(q)
    perm = np.random.default_rng(5).permutation(n)
    m = _gpu(L, n)
    m.set_state(q, p)
    m.make_pairlist()
    k0 = directed_pair_keys(m.pairs(), n, half=False)
    f0 = m.forces()
    m.set_state(q[perm], p[perm])
    m.make_pairlist()
    rec = np.asarray(m.pairs()).copy()
    rec[:, 0], rec[:, 1] = perm[rec[:, 0]], perm[rec[:, 1]]  # back to the original indices
    assert np.array_equal(directed_pair_keys(rec, n, half=False), k0)
    f1 = np.empty_like(f0)
    f1[perm] = m.forces()
    assert np.abs(f1 - f0).max() <= 1e-12 * np.abs(f0).max()


def test_particles_on_the_faces():
    # Particles exactly on the lower faces (and one ulp below the upper ones)
    # get every periodic image: the pair set equals the brute-force one.  The
    # reference (and the oracle, which restates it) forms a ghost only for a
    # particle strictly inside the edge slab (q > s, mdrect.cc:24-44; mdunit.cc:137-176),
    # so a particle at exactly 0 loses the images the ghost cascade would give
    # it; every pair the oracle lacks involves one of these particles.
    q, p, L = liquid_like(0.5, 6, seed=81)
    side = float(np.ravel(L)[0])
    q[0] = [0.0, 0.0, 0.0]
    q[1] = [0.5 * side, 0.0, 0.5 * side]
    top = np.nextafter(side, 0.0)
    q[2] = [top, 1.0, top]
    n = len(q)
    m = _gpu(L, n)
    m.set_state(q, p)
    m.make_pairlist()
    gk = directed_pair_keys(m.pairs(), n, half=False)
    bk = directed_pair_keys(port.bruteforce_pairs(q, np.full(3, side), RC + MARGIN), n, half=False)
    assert np.array_equal(gk, bk)
    ref = port.System(q, p, L, rc=RC, margin=MARGIN)
    ref.make_pairlist()
    rk = directed_pair_keys(ref.pairs(), n, half=True)
    missing = np.setdiff1d(gk, rk)
    assert len(np.setdiff1d(rk, gk)) == 0
    a, b = (missing // 27) // n, (missing // 27) % n
    assert np.all(np.isin(a, [0, 1, 2]) | np.isin(b, [0, 1, 2]))


@pytest.mark.parametrize("side", [6.2, 9.1])  # two and three cells per side at SL = 3
def test_smallest_cell_grids_match_brute_force(side):
    rng = np.random.default_rng(int(side * 10))
    n = int(0.5 * side ** 3)
    q = rng.random((n, 3)) * side
    p = rng.normal(size=(n, 3))
    m = _gpu(side, n)
    m.set_state(q, p)
    m.make_pairlist()
    assert m.stats()["cells"][0] == int(side // (RC + MARGIN))
    gk = directed_pair_keys(m.pairs(), n, half=False)
    bk = directed_pair_keys(port.bruteforce_pairs(q, np.full(3, side), RC + MARGIN), n, half=False)
    assert np.array_equal(gk, bk)


def test_capacity_limits():
    from mdacp_gb300 import native
    q, p, L = liquid_like(0.5, 4, seed=91)
    m = _gpu(L, len(q))
    m.set_state(q, p)            # exactly the capacity
    with pytest.raises(native.MDGError):
        m.set_state(np.vstack([q, q[:1] + 0.5]), np.vstack([p, p[:1]]))
    m.set_state(q, p)
    m.calculate(3)


def test_box_below_two_search_lengths_is_refused():
    # the 27-cell stencil needs at least two cells per side (side > 2 (rc + margin))
    from mdacp_gb300 import native
    with pytest.raises(native.MDGError, match="twice the search length"):
        _gpu(5.9, 10)
    with pytest.raises(native.MDGError):
        _gpu(np.array([12.0, 12.0, 6.0]), 10)
    m = _gpu(6.2, 10)   # two cells per side: accepted
    m.close()


def test_empty_state_is_refused_and_the_handle_stays_usable():
    from mdacp_gb300 import native
    q, p, L = liquid_like(0.5, 4, seed=93)
    m = _gpu(L, len(q))
    with pytest.raises(native.MDGError):
        m.set_state(np.zeros((0, 3)), np.zeros((0, 3)))
    m.set_state(q, p)
    m.calculate(5)
    assert m.stats()["steps"] == 5
