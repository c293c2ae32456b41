"""GPU adjoint: against the FP64 CPU reference gradient and against central finite differences.

Reference: oracle/adjoint_ref.py (numpy discrete adjoint, itself pinned to
finite differences in tests/test_adjoint_ref.py) on 500 atoms, 40 steps,
relative 1e-9.  Finite differences (h = 1e-6) on the 4000-atom box at density
0.8 over 200 steps, checkpoint every 20: relative 1e-4 for epsilon, sigma and
initial-position components.  The torch.autograd.Function below exists for
these tests only.
"""
import numpy as np
import pytest

from oracle.adjoint_ref import Model
from tests.helpers import liquid_like

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("objective", ["pe", "pressure"])
def test_adjoint_matches_reference_gradient(objective):
    from mdacp_gb300.adjoint import Adjoint
    q, p, L = liquid_like(0.8, 5, amp=0.1, seed=12)          # 500 atoms, L = 8.55
    steps, K = 40, 10
    ref = Model(L, dt=0.002, objective=objective)
    J0, gq0, gp0, ge0, gs0 = ref.gradient(q, p, steps)
    a = Adjoint(L, len(q), steps=steps, checkpoint_every=K, dt=0.002, margin=1.0, objective=objective)
    J = a.forward(q, p)
    gq, gp, ge, gs = a.backward()
    assert abs(J - J0) <= 1e-12 * abs(J0)
    assert np.linalg.norm(gq - gq0) <= 1e-9 * np.linalg.norm(gq0)
    assert np.linalg.norm(gp - gp0) <= 1e-9 * np.linalg.norm(gp0)
    assert abs(ge - ge0) <= 1e-9 * abs(ge0) and abs(gs - gs0) <= 1e-9 * abs(gs0)


def _c5(seed=5):
    return liquid_like(0.8, 10, amp=0.1, seed=seed)           # 4000 atoms, L = 17.1


@pytest.mark.parametrize("objective", ["pe", "pressure"])
def test_adjoint_matches_finite_differences_c5(objective):
    from mdacp_gb300.adjoint import Adjoint
    q, p, L = _c5()
    n, h = len(q), 1e-6
    kw = dict(steps=200, checkpoint_every=20, dt=0.002, margin=2.0, objective=objective)
    a = Adjoint(L, n, **kw)
    J = a.forward(q, p)
    gq, gp, ge, gs = a.backward()

    def Jp(eps=1.0, sig=1.0, q0=q):
        b = Adjoint(L, n, epsilon=eps, sigma=sig, **kw)
        v = b.forward(q0, p)
        b.close()
        return v

    fd_e = (Jp(eps=1 + h) - Jp(eps=1 - h)) / (2 * h)
    fd_s = (Jp(sig=1 + h) - Jp(sig=1 - h)) / (2 * h)
    assert abs(ge - fd_e) <= 1e-4 * abs(fd_e), (ge, fd_e)
    assert abs(gs - fd_s) <= 1e-4 * abs(fd_s), (gs, fd_s)
    # the three largest components of dJ/dq0 (so FD noise is negligible)
    flat = np.argsort(-np.abs(gq).ravel())[:3]
    for f in flat:
        i, k = divmod(int(f), 3)
        qp_, qm_ = q.copy(), q.copy()
        qp_[i, k] += h
        qm_[i, k] -= h
        fd = (Jp(q0=qp_) - Jp(q0=qm_)) / (2 * h)
        assert abs(gq[i, k] - fd) <= 1e-4 * abs(fd), (i, k, gq[i, k], fd)


@pytest.mark.parametrize("objective", ["pe", "pressure"])
def test_adjoint_finite_differences_margin_half(objective):
    """The C5 case at the list margin of the large NVE runs (0.5, a new list
    every 20-step segment): epsilon, sigma, the three largest components of
    dJ/dq0 and three drawn from the larger half, against central differences
    (h = 1e-6 for epsilon and sigma, 1e-5 for positions, so the rounding of J
    stays far below the difference of the smaller components)."""
    from mdacp_gb300.adjoint import Adjoint
    q, p, L = _c5(seed=6)
    n, h = len(q), 1e-6
    kw = dict(steps=200, checkpoint_every=20, dt=0.002, margin=0.5, objective=objective)
    a = Adjoint(L, n, **kw)
    a.forward(q, p)
    gq, gp, ge, gs = a.backward()
    a.close()

    def Jp(eps=1.0, sig=1.0, q0=q):
        b = Adjoint(L, n, epsilon=eps, sigma=sig, **kw)
        v = b.forward(q0, p)
        b.close()
        return v

    fd_e = (Jp(eps=1 + h) - Jp(eps=1 - h)) / (2 * h)
    fd_s = (Jp(sig=1 + h) - Jp(sig=1 - h)) / (2 * h)
    assert abs(ge - fd_e) <= 1e-4 * abs(fd_e), (ge, fd_e)
    assert abs(gs - fd_s) <= 1e-4 * abs(fd_s), (gs, fd_s)
    order = np.argsort(-np.abs(gq).ravel())
    picks = list(order[:3]) + list(np.random.default_rng(2).choice(order[3:len(order) // 2], 3, replace=False))
    hq = 1e-5
    for f in picks:
        i, k = divmod(int(f), 3)
        qp_, qm_ = q.copy(), q.copy()
        qp_[i, k] += hq
        qm_[i, k] -= hq
        fd = (Jp(q0=qp_) - Jp(q0=qm_)) / (2 * hq)
        assert abs(gq[i, k] - fd) <= 1e-4 * abs(fd), (i, k, gq[i, k], fd)


def test_autograd_function_wrapper():
    import torch
    from mdacp_gb300.adjoint import Adjoint

    class MeanPotential(torch.autograd.Function):
        """J(q0, p0) of the adjoint engine; gradients from its backward pass (tests only)."""

        @staticmethod
        def forward(ctx, q0, p0, engine):
            J = engine.forward(q0.detach().numpy(), p0.detach().numpy())
            ctx.engine = engine
            return torch.tensor(J, dtype=torch.float64)

        @staticmethod
        def backward(ctx, g):
            gq, gp, _, _ = ctx.engine.backward()
            return g * torch.from_numpy(gq), g * torch.from_numpy(gp), None

    q, p, L = liquid_like(0.8, 5, amp=0.1, seed=13)
    eng = Adjoint(L, len(q), steps=20, checkpoint_every=5, margin=1.0)
    qt = torch.tensor(q, requires_grad=True)
    pt = torch.tensor(p, requires_grad=True)
    J = MeanPotential.apply(qt, pt, eng)
    J.backward()
    ref = Model(L, dt=0.002).gradient(q, p, 20)
    assert np.linalg.norm(qt.grad.numpy() - ref[1]) <= 1e-9 * np.linalg.norm(ref[1])
    assert np.linalg.norm(pt.grad.numpy() - ref[2]) <= 1e-9 * np.linalg.norm(ref[2])
