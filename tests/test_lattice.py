import numpy as np

from mdacp_gb300 import lattice


def test_fcc_counts_match_reference_configuration_maker():
    q, L = lattice.fcc(0.5, 40.0)
    assert len(q) == 32000 and np.all(q > 0) and np.all(q < 40.0)
    q2, L2 = lattice.fcc_cube(10, 0.8)
    assert len(q2) == 4000 and abs(L2[0] - 17.09975946676697) < 1e-12


def test_maxwell_zero_momentum_and_temperature():
    v = lattice.maxwell(20000, 1.3, 5)
    assert np.abs(v.sum(0)).max() < 1e-9
    assert abs((v * v).sum() / (3 * len(v)) - 1.3) < 0.03
    assert np.array_equal(v, lattice.maxwell(20000, 1.3, 5))


def test_thin_keeps_sorted_subset():
    q, L = lattice.fcc(0.5, 20.0)
    t = lattice.thin(q, 500, 3)
    assert len(t) == 500 and len(np.unique(t, axis=0)) == 500
