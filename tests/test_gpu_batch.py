"""Batched replicas: every box of a batch against the oracle run on that box alone.

Boxes of uneven size (500..8000 atoms, the batched configuration's range, in
the FP64 comparison; 500..2000 elsewhere), density 0.3..0.9 (so some boxes
have only two cells per side) and temperature 0.7..1.5, rc 2.5, margin 0.4,
dt 0.002.  FP64: per-box observables rtol 1e-10 after 100 steps; mixed: within
1e-5 of FP64; overflow regrowth; autotuner leaves the state unchanged.
"""
import numpy as np
import pytest

from oracle import port

pytestmark = pytest.mark.gpu

RC, MARGIN, DT = 2.5, 0.4, 0.002


def _boxes(nbox=12, seed=3, n_range=(500, 2000)):
    """nbox drawn boxes plus one 500-atom box at density 0.9 (L = 8.2: two cells per side)."""
    from mdacp_gb300.batch import make_replicas
    return make_replicas(nbox, seed=seed, n_range=n_range) + make_replicas(
        1, seed=seed + 1000, n_range=(500, 500), rho_range=(0.9, 0.9))


def _oracle_obs(boxes, steps):
    out = []
    for q, p, L in boxes:
        s = port.System(q, p, L, rc=RC, margin=MARGIN, dt=DT)
        s.make_pairlist()
        s.calculate(steps)
        out.append(s.observe_raw())
    return np.array(out)


def test_batch_fp64_matches_oracle_per_box():
    from mdacp_gb300.batch import Batch
    boxes = _boxes(16, n_range=(500, 8000))
    assert any(L[0] < 3 * (RC + MARGIN) for _, _, L in boxes)   # two cells per side occurs
    assert max(len(q) for q, _, _ in boxes) > 6000
    b = Batch(boxes, cutoff=RC, margin=MARGIN, dt=DT)
    b.calculate(100)
    np.testing.assert_allclose(b.observe_raw(), _oracle_obs(boxes, 100), rtol=1e-10, atol=1e-10)
    st = b.stats()
    assert st["steps"] == 100 and st["rebuilds"] >= len(boxes)


@pytest.mark.parametrize("precision", ["mixed", "mixed_plain"])
def test_batch_mixed_close_to_fp64(precision):
    from mdacp_gb300.batch import Batch
    boxes = _boxes(8, seed=5, n_range=(500, 8000))
    a = Batch(boxes, cutoff=RC, margin=MARGIN, dt=DT, precision="fp64")
    m = Batch(boxes, cutoff=RC, margin=MARGIN, dt=DT, precision=precision)
    a.calculate(50)
    m.calculate(50)
    np.testing.assert_allclose(m.observe_raw(), a.observe_raw(), rtol=1e-5, atol=1e-5)


@pytest.mark.parametrize("shape", [(128, 1, 4), (256, 2, 2), (512, 4, 1), (128, 1, 8, "flat"), (256, 1, 5, "flat")])
def test_batch_shapes_agree(shape):
    # per-box CTAs in three shapes and the flat layout (the grid striding over
    # every box's particles, per-box flags applied after the step) in two
    from mdacp_gb300.batch import Batch
    boxes = _boxes(6, seed=7)
    b = Batch(boxes, cutoff=RC, margin=MARGIN, dt=DT)
    b.set_shape(*shape[:3])
    if len(shape) > 3:
        b.set_flat(True)
        assert b.stats()["flat"] == 1
    b.calculate(60)
    np.testing.assert_allclose(b.observe_raw(), _oracle_obs(boxes, 60), rtol=1e-10, atol=1e-10)
    st = b.stats()
    assert st["steps"] == 60 and st["rebuilds"] >= len(boxes)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_batch_flat_layout_matches_per_box_layout(precision):
    # the same boxes through both layouts, inner list on, with a tiny buffer so
    # the boxes re-select every few steps: the per-particle arithmetic and the
    # per-box rebuild / re-selection schedule are the same.  The mixed states
    # agree bit for bit; in FP64 the compiler may fuse the pair expressions
    # (r^2, the force factor) differently in the two kernels, so the states
    # agree to the rounding that grows from there (1e-9 after 70 steps)
    from mdacp_gb300.batch import Batch
    boxes = _boxes(8, seed=17, n_range=(500, 8000))
    runs = []
    for flat in (False, True):
        b = Batch(boxes, cutoff=RC, margin=MARGIN, dt=DT, precision=precision, prune_buffer=0.02)
        b.set_shape(256, 1, 2)
        b.set_flat(flat)
        b.calculate(70)
        st = b.stats()
        assert st["inner_list"] == 1 and st["flat"] == (1 if flat else 0)
        runs.append(([x.copy() for pair in b.state() for x in pair], st["rebuilds"]))
    (a, ra), (c, rc) = runs
    assert ra == rc
    for u, v in zip(a, c):
        if precision == "mixed":
            assert np.array_equal(u, v)
        else:
            np.testing.assert_allclose(v, u, rtol=1e-9, atol=1e-9)


def test_batch_overflow_regrows_and_catches_up():
    from mdacp_gb300.batch import Batch
    boxes = _boxes(6, seed=9)
    b = Batch(boxes, cutoff=RC, margin=MARGIN, dt=DT, list_capacity=8)
    b.calculate(40)
    assert b.stats()["list_capacity"] > 8
    np.testing.assert_allclose(b.observe_raw(), _oracle_obs(boxes, 40), rtol=1e-10, atol=1e-10)


def test_autotuner_restores_state():
    from mdacp_gb300.batch import Batch
    boxes = _boxes(6, seed=11)
    b = Batch(boxes, cutoff=RC, margin=MARGIN, dt=DT)
    b.calculate(10)
    before = [x.copy() for pair in b.state() for x in pair]
    t, lanes, c = b.tune(trial_steps=4)
    st = b.stats()
    assert t in (128, 256, 512) and lanes in (1, 2, 4) and st["flat"] in (0, 1)
    # every CTA resident: at most 2,048 threads per SM, the flat layout with
    # one lane per particle and at most 256 threads
    assert 1 <= st["ctas_per_sm"] and t * st["ctas_per_sm"] <= 2048
    assert not st["flat"] or (lanes == 1 and t <= 256)
    after = [x for pair in b.state() for x in pair]
    for u, v in zip(before, after):
        assert np.array_equal(u, v)
    b.calculate(30)
    np.testing.assert_allclose(b.observe_raw(), _oracle_obs([(q, p, L) for (q, p), (_, _, L) in
                                                             zip([(x, y) for x, y in zip(before[0::2], before[1::2])],
                                                                 boxes)], 30), rtol=1e-10, atol=1e-10)


@pytest.mark.parametrize("precision", ["fp64", "mixed_plain", "mixed"])
def test_inner_list_changes_nothing(precision):
    # the inner rows keep the outer rows' order and drop only pairs beyond rc,
    # whose terms are exactly zero: the trajectories agree bit for bit, also
    # when a tiny buffer makes the boxes re-select every few steps.  With
    # compensated sums (mixed) a zero term leaves the compensated value
    # unchanged but re-normalises the correction, so later additions round
    # differently: forces agree to about one float rounding and the states
    # after 80 steps to 1e-7, not bit for bit
    from mdacp_gb300.batch import Batch
    boxes = _boxes(6, seed=13)
    runs = []
    for buf in (0.0, None, 0.02, 0.2):  # 0.2: half the margin, a choice of the autotuner
        b = Batch(boxes, cutoff=RC, margin=MARGIN, dt=DT, precision=precision, prune_buffer=buf)
        b.set_shape(256, 1, 2)
        b.calculate(80)
        st = b.stats()
        assert st["inner_list"] == (0 if buf == 0.0 else 1)
        runs.append([x.copy() for pair in b.state() for x in pair])
    # the inner list switched off by hand walks every listed pair
    b = Batch(boxes, cutoff=RC, margin=MARGIN, dt=DT, precision=precision)
    b.set_shape(256, 1, 2)
    b.set_inner(False)
    b.calculate(80)
    assert b.stats()["inner_list"] == 0
    runs.append([x.copy() for pair in b.state() for x in pair])
    for other in runs[1:]:
        for u, v in zip(runs[0], other):
            if precision == "mixed":
                np.testing.assert_allclose(v, u, rtol=1e-7, atol=1e-7)
            else:
                assert np.array_equal(u, v)


@pytest.mark.parametrize("precision", ["mixed", "mixed_plain"])
def test_batch_mixed_state_readers(precision):
    # the mixed forms do not write q_end in the step; observers, get_state and
    # the autotuner's snapshot form it from each box's last q_mid slot, and
    # the padding lane (packed reference positions inside) comes back zero.
    # Reading between chunks leaves the run bit for bit where one call takes it
    import ctypes
    from mdacp_gb300.batch import Batch
    boxes = _boxes(6, seed=23)
    runs = []
    for chunks in ((70,), (25, 1, 44)):
        b = Batch(boxes, cutoff=RC, margin=MARGIN, dt=DT, precision=precision)
        b.set_shape(256, 1, 2)
        b.set_flat(True)
        for c in chunks:
            b.calculate(c)
            b.observe_raw()
            b.state()
        n = sum(len(x[0]) for x in boxes)
        q4 = np.full((n, 4), 7.0)
        p4 = np.full((n, 4), 7.0)
        dp = ctypes.POINTER(ctypes.c_double)
        assert b.lib.mdg_batch_get_state(b._h, q4.ctypes.data_as(dp), p4.ctypes.data_as(dp)) == 0
        assert not q4[:, 3].any() and not p4[:, 3].any()
        runs.append((q4, p4, b.observe_raw()))
    (qa, pa, oa), (qb, pb, ob) = runs
    assert np.array_equal(qa, qb) and np.array_equal(pa, pb)
    np.testing.assert_array_equal(oa, ob)
