"""GPU parity against the oracle (the C restatement pinned bitwise to the reference).

Tolerances: pair set bit-exact; FP64 forces |dF_i| <= 1e-12 max(|F_i|, sum_j |f_ij|)
and ||dF||/||F|| <= 1e-12; E/T/P traces over 100 steps relative 1e-10;
mixed-precision RMS relative force error <= 1e-5.
"""
import numpy as np
import pytest

from oracle import port
from tests.helpers import directed_pair_keys, liquid_like, pair_force_abs_sum

pytestmark = pytest.mark.gpu

RC, MARGIN = 2.5, 0.5


def _gpu(L, n, **kw):
    from mdacp_gb300.manager import MDManager
    kw.setdefault("cutoff", RC)
    kw.setdefault("margin", MARGIN)
    return MDManager(L, capacity=n, **kw)


@pytest.mark.parametrize("density,cells", [(0.5, 20), (0.8, 10), (0.5, 8)])
def test_pair_set_bit_exact(density, cells):
    q, p, L = liquid_like(density, cells, seed=cells)
    n = len(q)
    ref = port.System(q, p, L, rc=RC, margin=MARGIN)
    ref.make_pairlist()
    rk = directed_pair_keys(ref.pairs(), n, half=True)
    m = _gpu(L, n)
    m.set_state(q, p)
    m.make_pairlist()
    gk = directed_pair_keys(m.pairs(), n, half=False)
    assert len(gk) == len(rk)
    assert np.array_equal(gk, rk)


@pytest.mark.parametrize("density,cells", [(0.5, 20), (0.8, 10)])
def test_forces_fp64(density, cells):
    q, p, L = liquid_like(density, cells, seed=100 + cells)
    n = len(q)
    ref = port.System(q, p, L, rc=RC, margin=MARGIN)
    ref.make_pairlist()
    fr = ref.forces()
    scale = np.maximum(np.linalg.norm(fr, axis=1), pair_force_abs_sum(q, L, ref.pairs(), RC))
    m = _gpu(L, n)
    m.set_state(q, p)
    f = m.forces()
    df = np.linalg.norm(f - fr, axis=1)
    assert np.all(df <= 1e-12 * scale), (df / scale).max()
    assert np.linalg.norm(f - fr) <= 1e-12 * np.linalg.norm(fr)


def test_observables_match_reference_expression():
    q, p, L = liquid_like(0.5, 12, seed=5)
    ref = port.System(q, p, L, rc=RC, margin=MARGIN)
    ref.make_pairlist()
    m = _gpu(L, len(q))
    m.set_state(q, p)
    o, orf = m.observe_raw(), ref.observe_raw()
    np.testing.assert_allclose(o, orf, rtol=1e-13)


@pytest.mark.parametrize("use_graphs,prune", [(True, None), (False, None), (True, 0.0), (True, 0.02)])
def test_nve_trace_100_steps(use_graphs, prune):
    """prune: inner-list buffer (None = default 0.1; 0 = walk every listed pair;
    0.02 = re-select every few steps)."""
    q, p, L = liquid_like(0.5, 20, seed=9)
    ref = port.System(q, p, L, rc=RC, margin=MARGIN, dt=0.001)
    ref.make_pairlist()
    m = _gpu(L, len(q), dt=0.001, use_graphs=use_graphs, prune_buffer=prune)
    m.set_state(q, p)
    m.make_pairlist()
    rows, rrows = [m.observe()], [ref.observe()]
    for _ in range(10):
        m.calculate(10)
        ref.calculate(10)
        rows.append(m.observe())
        rrows.append(ref.observe())
    rows, rrows = np.array(rows), np.array(rrows)
    np.testing.assert_allclose(rows, rrows, rtol=1e-10, atol=1e-12)
    qg, pg = m.state()
    qr, pr = ref.state()
    dq = np.abs((qg - qr + L / 2) % L - L / 2).max()
    assert dq < 1e-10 and np.abs(pg - pr).max() < 1e-10
    st = m.stats()
    assert st["steps"] == 100
    if prune == 0.02:
        assert st["prunes"] > st["rebuilds"] and st["inner_pairs"] < st["listed_pairs"]


def test_mixed_force_error():
    q, p, L = liquid_like(0.5, 20, seed=21)
    ref = port.System(q, p, L, rc=RC, margin=MARGIN)
    ref.make_pairlist()
    fr = ref.forces()
    m = _gpu(L, len(q), precision="mixed")
    m.set_state(q, p)
    f = m.forces()
    rel = np.linalg.norm(f - fr, axis=1) / np.linalg.norm(fr, axis=1)
    rms = np.sqrt(np.mean(rel ** 2))
    assert rms <= 1e-5, rms


def test_mixed_trace_close():
    q, p, L = liquid_like(0.5, 16, seed=23)
    ref = port.System(q, p, L, rc=RC, margin=MARGIN)
    ref.make_pairlist()
    m = _gpu(L, len(q), precision="mixed")
    m.set_state(q, p)
    m.calculate(100)
    ref.calculate(100)
    np.testing.assert_allclose(m.observe(), ref.observe(), rtol=1e-5, atol=1e-6)


def test_mixed_observer_matches_fp64_observer():
    # the mixed form evaluates pair energies and virials in float from the
    # home-cell-local positions; on the same state the sums agree with the FP64
    # observer to float rounding (per-pair relative 1e-7, summed in double)
    q, p, L = liquid_like(0.8, 24, seed=29)
    a = _gpu(L, len(q), precision="mixed")
    b = _gpu(L, len(q))
    for m in (a, b):
        m.set_state(q, p)
    np.testing.assert_allclose(a.observe_raw(), b.observe_raw(), rtol=2e-6, atol=0)
    a.calculate(150)
    qa, pa = a.state()
    b.set_state(qa, pa)
    np.testing.assert_allclose(a.observe_raw(), b.observe_raw(), rtol=2e-6, atol=0)


def test_langevin_matches_oracle_stream():
    q, p, L = liquid_like(0.5, 12, seed=31)
    kw = dict(dt=0.005, thermostat="langevin", temperature=0.9, gamma=1.0, seed=12345)
    m = _gpu(L, len(q), **kw)
    m.set_state(q, p)
    ref = port.System(q, p, L, rc=RC, margin=MARGIN, dt=0.005, thermostat=port.LANGEVIN, temperature=0.9,
                      gamma=1.0, seed=12345)
    ref.make_pairlist()
    m.calculate(40)
    ref.calculate(40)
    qg, pg = m.state()
    qr, pr = ref.state()
    assert np.abs(pg - pr).max() < 1e-5
    np.testing.assert_allclose(m.observe(), ref.observe(), rtol=1e-5, atol=1e-6)


def test_nosehoover_matches_oracle():
    q, p, L = liquid_like(0.5, 12, seed=41, temperature=1.3)
    m = _gpu(L, len(q), thermostat="nosehoover", temperature=1.0, tau=0.1)
    m.set_state(q, p)
    ref = port.System(q, p, L, rc=RC, margin=MARGIN, thermostat=port.NOSEHOOVER, temperature=1.0, tau=0.1)
    ref.make_pairlist()
    m.calculate(50)
    ref.calculate(50)
    np.testing.assert_allclose(m.observe(), ref.observe(), rtol=1e-10, atol=1e-12)
    assert abs(m.stats()["zeta"] - ref.zeta) < 1e-10


def test_overflow_regrows_list():
    q, p, L = liquid_like(0.8, 8, seed=51)
    ref = port.System(q, p, L, rc=RC, margin=MARGIN)
    ref.make_pairlist()
    fr = ref.forces()
    m = _gpu(L, len(q), list_capacity=8)
    m.set_state(q, p)
    f = m.forces()
    assert m.stats()["list_capacity"] > 8
    assert np.linalg.norm(f - fr) <= 1e-12 * np.linalg.norm(fr)
    m.calculate(30)
    ref.calculate(30)
    np.testing.assert_allclose(m.observe(), ref.observe(), rtol=1e-10, atol=1e-12)


def test_outstanding_steps_recover_overflow():
    # single-step calls return before the steps run; the list overflow of the
    # first rebuild halts the device, and the next reader regrows the rows and
    # runs the owed steps
    q, p, L = liquid_like(0.8, 8, seed=52)
    ref = port.System(q, p, L, rc=RC, margin=MARGIN)
    ref.make_pairlist()
    m = _gpu(L, len(q), list_capacity=8)
    m.set_state(q, p)
    for _ in range(30):
        m.calculate(1)
    ref.calculate(30)
    np.testing.assert_allclose(m.observe(), ref.observe(), rtol=1e-10, atol=1e-12)
    st = m.stats()
    assert st["steps"] == 30 and st["list_capacity"] > 8


def test_single_step_calls_match_one_call():
    q, p, L = liquid_like(0.5, 10, seed=53)
    a = _gpu(L, len(q), precision="mixed")
    b = _gpu(L, len(q), precision="mixed")
    for m in (a, b):
        m.set_state(q, p)
    a.calculate(1500)
    for _ in range(1500):   # crosses the 1024-step confirmation bound once
        b.calculate(1)
    b.synchronize()
    qa, pa = a.state()
    qb, pb = b.state()
    assert np.array_equal(qa, qb) and np.array_equal(pa, pb)
    assert a.stats()["steps"] == b.stats()["steps"] == 1500


def test_bad_state_reported_by_the_next_reader():
    from mdacp_gb300 import native
    q, p, L = liquid_like(0.5, 6, seed=62)
    m = _gpu(L, len(q))
    bad = q.copy()
    bad[5, 0] = np.inf
    m.set_state(bad, p)
    m.calculate(5)           # enqueued only
    with pytest.raises(native.MDGError, match="bad particle state"):
        m.observe()
    m.set_state(q, p)
    m.calculate(5)
    m.synchronize()
    assert m.stats()["steps"] == 5


def test_state_roundtrip_and_bad_state():
    from mdacp_gb300 import native
    q, p, L = liquid_like(0.5, 6, seed=61)
    m = _gpu(L, len(q))
    m.set_state(q, p)
    qg, pg = m.state()
    assert np.array_equal(qg, q) and np.array_equal(pg, p)
    bad = q.copy()
    bad[3, 1] = np.nan
    m.set_state(bad, p)
    with pytest.raises(native.MDGError, match="bad particle state"):
        m.make_pairlist()
    m.set_state(q, p)   # the handle stays usable
    m.calculate(5)


def test_elapsed_time_is_the_last_calls_steps():
    # elapsed_ms covers the steps of the last calculate call only, also when
    # an earlier call's steps were still outstanding
    q, p, L = liquid_like(0.5, 24, seed=54)
    m = _gpu(L, len(q), precision="mixed")
    m.set_state(q, p)
    m.make_pairlist()
    m.calculate(300)
    m.calculate(30)
    t_short = m.stats()["elapsed_ms"]
    m.calculate(300)
    t_long = m.stats()["elapsed_ms"]
    assert 0 < t_short < 0.5 * t_long


def test_new_state_of_the_same_size_reuses_graphs_correctly():
    # the step graphs hold the geometry by value: a new state with the same
    # particle count keeps them, a different count rebuilds them
    qa, pa, L = liquid_like(0.5, 10, seed=55)
    qb, pb, _ = liquid_like(0.5, 10, seed=56)
    m = _gpu(L, len(qa))
    m.set_state(qa, pa)
    m.calculate(20)
    for q, p in ((qb, pb), (qa[:-7], pa[:-7])):
        m.set_state(q, p)
        m.calculate(40)
        ref = port.System(q, p, L, rc=RC, margin=MARGIN)
        ref.make_pairlist()
        ref.calculate(40)
        np.testing.assert_allclose(m.observe(), ref.observe(), rtol=1e-10, atol=1e-12)


def test_phase_times_split_the_run():
    # StopWatch-like split: step kernels ("force"), rebuild sequences ("pair")
    # and the whole run; the first step after set_state rebuilds
    q, p, L = liquid_like(0.5, 12, seed=57)
    m = _gpu(L, len(q), precision="mixed")
    m.set_state(q, p)
    ph = m.calculate_phases(60)
    assert ph["force"] > 0 and ph["pair"] > 0
    assert ph["force"] + ph["pair"] <= ph["all"] * 1.001
    assert m.stats()["steps"] == 60
    ref = port.System(q, p, L, rc=RC, margin=MARGIN)
    ref.make_pairlist()
    ref.calculate(60)
    np.testing.assert_allclose(m.observe(), ref.observe(), rtol=1e-5, atol=1e-6)


@pytest.mark.parametrize("precision", ["mixed", "mixed_plain"])
def test_mixed_readers_leave_the_trajectory_alone(precision):
    # the mixed form keeps mid-step positions relative to the home cell and
    # does not write the step-boundary positions; readers (observers, forces,
    # get_state) and rebuilds form them from q_mid and p.  Reading between
    # steps must not perturb the run: 300 steps in one call and the same steps
    # in chunks with every reader in between end bit for bit in the same
    # state, with several list rebuilds on the way
    q, p, L = liquid_like(0.5, 16, seed=37)
    a = _gpu(L, len(q), precision=precision)
    b = _gpu(L, len(q), precision=precision)
    for m in (a, b):
        m.set_state(q, p)
        m.make_pairlist()
    a.calculate(300)
    done = 0
    for chunk in (37, 1, 62, 100, 100):
        b.calculate(chunk)
        done += chunk
        b.observe_raw()
        b.forces()
        b.state()
    assert done == 300
    qa, pa = a.state()
    qb, pb = b.state()
    assert np.array_equal(qa, qb) and np.array_equal(pa, pb)
    assert a.stats()["rebuilds"] == b.stats()["rebuilds"] >= 3
    np.testing.assert_array_equal(a.observe_raw(), b.observe_raw())


@pytest.mark.parametrize("precision", ["mixed", "mixed_plain"])
def test_mixed_reference_positions_in_the_padding_lane(precision):
    # the mixed form carries its build and prune reference positions in the
    # padding lane of q_mid and p (21-bit fixed point per axis, displacement
    # thresholds lowered by two units of the packing); the lane comes back
    # zero from mdg_get_state, and the list rebuilds fall on the steps the
    # FP64 form takes them (the thresholds move by micro-sigma, the
    # trajectories differ by float rounding of the forces)
    q, p, L = liquid_like(0.5, 16, seed=41)
    a = _gpu(L, len(q), precision=precision)
    b = _gpu(L, len(q))
    for m in (a, b):
        m.set_state(q, p)
        m.make_pairlist()
    for chunk in (60, 60, 80):
        a.calculate(chunk)
        b.calculate(chunk)
        sa, sb = a.stats(), b.stats()
        assert sa["rebuilds"] == sb["rebuilds"]
        assert abs(sa["prunes"] - sb["prunes"]) <= 1
    assert a.stats()["rebuilds"] >= 3
    q4 = np.full((len(q), 4), 7.0)
    p4 = np.full((len(q), 4), 7.0)
    a.state(q4, p4)
    assert not q4[:, 3].any() and not p4[:, 3].any()
    qb, pb = b.state()
    np.testing.assert_allclose(q4[:, :3], qb, rtol=0, atol=1e-6 * L[0])


@pytest.mark.parametrize("use_graphs", [True, False])
def test_reference_rebuild_policy_matches_oracle(use_graphs):
    # RebuildPolicy=reference: the buffer budget (2 max|p| dt per step) and,
    # once it is spent, the displacement check of PairList (pairlist.cc:26-121)
    # over the particles and their ghost images (the images at the previous
    # mid-step, as the reference refreshes them), evaluated at each step's
    # start as the oracle does: the rebuilds fall on the same steps, and the
    # FP64 trajectory matches the oracle's
    q, p, L = liquid_like(0.5, 10, seed=43)
    ref = port.System(q, p, L, rc=RC, margin=MARGIN, dt=0.002)
    ref.make_pairlist()
    m = _gpu(L, len(q), dt=0.002, rebuild_policy="reference", use_graphs=use_graphs)
    m.set_state(q, p)
    m.make_pairlist()
    r = m.stats()["rebuilds"]
    ref_steps, gpu_steps = [], []
    for k in range(300):
        if ref.calculate(1):
            ref_steps.append(k + 1)
        m.calculate(1)
        r2 = m.stats()["rebuilds"]
        if r2 != r:
            gpu_steps.append(k + 1)
        r = r2
    assert gpu_steps == ref_steps and len(ref_steps) >= 6
    np.testing.assert_allclose(m.observe_raw(), ref.observe_raw(), rtol=1e-10, atol=1e-10)


def test_reference_rebuild_policy_mixed_and_too_fast():
    # the mixed form under the reference policy rebuilds on the FP64 form's
    # steps; a momentum with 2 |p| dt above the margin stops the run with the
    # reference's "too fast particles" error, and the handle takes a new state
    from mdacp_gb300 import native
    q, p, L = liquid_like(0.5, 10, seed=47)
    a = _gpu(L, len(q), dt=0.002, rebuild_policy="reference", precision="mixed")
    b = _gpu(L, len(q), dt=0.002, rebuild_policy="reference")
    for m in (a, b):
        m.set_state(q, p)
        m.make_pairlist()
    for chunk in (100, 100):
        a.calculate(chunk)
        b.calculate(chunk)
        assert a.stats()["rebuilds"] == b.stats()["rebuilds"]
    assert b.stats()["rebuilds"] >= 3
    fast = p.copy()
    fast[0] = [130.0, 0.0, 0.0]  # 2 x 130 x 0.002 = 0.52 > margin 0.5
    for m in (a, b):
        m.set_state(q, fast)
        with pytest.raises(native.MDGError, match="too fast"):
            m.calculate(3)
            m.synchronize()
        m.set_state(q, p)
        m.calculate(5)
        m.synchronize()
