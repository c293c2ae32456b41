"""The CPU reference gradient (oracle/adjoint_ref.py) against central finite differences."""
import numpy as np
import pytest

from oracle.adjoint_ref import Model
from tests.helpers import liquid_like


@pytest.mark.parametrize("objective", ["pe", "pressure"])
def test_reference_gradient_matches_finite_differences(objective):
    q, p, L = liquid_like(0.8, 3, amp=0.1, seed=4)          # 108 atoms
    m = Model(L, dt=0.002, objective=objective)
    steps = 12
    J, gq, gp, ge, gs = m.gradient(q, p, steps)
    # central differences: steps small enough for the O(h^2) error of the steep
    # sigma dependence, large enough to stay clear of roundoff in the state
    hp, h = 1e-6, 1e-5

    def J_at(eps=1.0, sig=1.0, q0=q, p0=p):
        mm = Model(L, dt=0.002, eps=eps, sig=sig, objective=objective)
        return mm.run(q0, p0, steps)[0]

    fd_e = (J_at(eps=1 + hp) - J_at(eps=1 - hp)) / (2 * hp)
    fd_s = (J_at(sig=1 + hp) - J_at(sig=1 - hp)) / (2 * hp)
    assert abs(ge - fd_e) <= 1e-6 * max(1.0, abs(fd_e))
    assert abs(gs - fd_s) <= 1e-6 * max(1.0, abs(fd_s))
    for (a, k) in [(5, 0), (17, 1), (60, 2)]:
        qp, qm = q.copy(), q.copy()
        qp[a, k] += h
        qm[a, k] -= h
        fd = (J_at(q0=qp) - J_at(q0=qm)) / (2 * h)
        assert abs(gq[a, k] - fd) <= 1e-6 * max(abs(fd), 1e-3), (a, k, gq[a, k], fd)
        pp, pm = p.copy(), p.copy()
        pp[a, k] += h
        pm[a, k] -= h
        fd = (J_at(p0=pp) - J_at(p0=pm)) / (2 * h)
        assert abs(gp[a, k] - fd) <= 1e-6 * max(abs(fd), 1e-3), (a, k, gp[a, k], fd)
