"""FP64 reference gradient of a trajectory-averaged LJ observable (test infrastructure only).

Plain numpy, all pairs with the minimum image (small systems only), the
reference's smoothly truncated potential written as V(r) = eps phi(r/sigma)
(variables.cc:16-28 in sigma units) and its drift-kick-drift step
(mdmanager.cc:151-157).  The gradient is the discrete adjoint: every state is
kept (no checkpointing) and the pair Hessian is applied as explicit 3x3 blocks.
It is checked against central finite differences in tests/test_adjoint_ref.py
and used as the reference for the GPU adjoint.
"""
import numpy as np


def lj_constants(xc):
    s2 = 1.0 / (xc * xc)
    s6 = s2 * s2 * s2
    s8, s12 = s6 * s2, s6 * s6
    s14 = s12 * s2
    c2 = 6.0 * s14 - 3.0 * s8
    c0 = -s12 + s6 - c2 / s2
    return c0, c2


class Model:
    def __init__(self, L, xc=2.5, eps=1.0, sig=1.0, dt=0.002, objective="pe"):
        self.L = np.broadcast_to(np.asarray(L, dtype=np.float64), (3,)).copy()
        self.xc, self.eps, self.sig, self.dt = xc, eps, sig, dt
        self.c0, self.c2 = lj_constants(xc)
        self.objective = objective

    def _pairs(self, q):
        n = len(q)
        i, j = np.triu_indices(n, 1)
        d = q[j] - q[i]
        d -= self.L * np.rint(d / self.L)
        r2 = (d * d).sum(1)
        m = r2 <= (self.xc * self.sig) ** 2
        return i[m], j[m], d[m], r2[m]

    def _terms(self, r2):
        e, s, c0, c2 = self.eps, self.sig, self.c0, self.c2
        x2 = r2 / (s * s)
        x = np.sqrt(x2)
        phi = 4 * (x ** -12 - x ** -6 + c2 * x2 + c0)
        dphi = 4 * (-12 * x ** -13 + 6 * x ** -7 + 2 * c2 * x)           # phi'(x)
        d2phi = 4 * (156 * x ** -14 - 42 * x ** -8 + 2 * c2)             # phi''(x)
        r = np.sqrt(r2)
        V = e * phi
        Vp = e / s * dphi                                                # dV/dr
        Vpp = e / s ** 2 * d2phi
        dV_ds = -e / s * x * dphi                                        # dV/dsigma at fixed r
        dVp_ds = -e / s ** 2 * (dphi + x * d2phi)                        # d(dV/dr)/dsigma
        return r, V, Vp, Vpp, dV_ds, dVp_ds

    def force(self, q):
        i, j, d, r2 = self._pairs(q)
        r, V, Vp, *_ = self._terms(r2)
        fij = (Vp / r)[:, None] * d            # force on i from j
        F = np.zeros_like(q)
        np.add.at(F, i, fij)
        np.add.at(F, j, -fij)
        return F

    def objective_and_grads(self, q, p):
        """j, dj/dq, dj/dp, dj/deps, dj/dsigma at one state."""
        n = len(q)
        i, j, d, r2 = self._pairs(q)
        r, V, Vp, Vpp, dV_ds, dVp_ds = self._terms(r2)
        u = d / r[:, None]                     # unit vector i -> j
        gq = np.zeros_like(q)
        gp = np.zeros_like(p)
        if self.objective == "pe":
            val = V.sum() / n
            # dU/dq_i = -V'(r) u ; dU/dq_j = +V'(r) u
            np.add.at(gq, i, -(Vp[:, None] * u) / n)
            np.add.at(gq, j, (Vp[:, None] * u) / n)
            return val, gq, gp, V.sum() / self.eps / n, dV_ds.sum() / n
        vol = self.L.prod()
        W = r * Vp                              # pair virial term f r^2 with f = V'/r
        G = W.sum()
        KE = 0.5 * (p * p).sum()
        val = (2 * KE - G) / (3 * vol)
        dW_dr = Vp + r * Vpp
        np.add.at(gq, i, (dW_dr[:, None] * u) / (3 * vol))
        np.add.at(gq, j, -(dW_dr[:, None] * u) / (3 * vol))
        gp = 2 * p / (3 * vol)
        dW_ds = r * dVp_ds
        return val, gq, gp, -G / self.eps / (3 * vol), -dW_ds.sum() / (3 * vol)

    def hvp(self, q, v):
        """Hessian of the potential energy applied to v (3x3 pair blocks)."""
        i, j, d, r2 = self._pairs(q)
        r, V, Vp, Vpp, *_ = self._terms(r2)
        u = d / r[:, None]
        # block K = V'' u u^T + (V'/r)(I - u u^T); (H v)_i += K (v_i - v_j), (H v)_j -= ...
        w = v[i] - v[j]
        uw = (u * w).sum(1)
        Kw = (Vpp * uw)[:, None] * u + (Vp / r)[:, None] * (w - uw[:, None] * u)
        out = np.zeros_like(v)
        np.add.at(out, i, Kw)
        np.add.at(out, j, -Kw)
        return out

    def dforce_dparams(self, q):
        """dF/deps and dF/dsigma (n x 3 each)."""
        i, j, d, r2 = self._pairs(q)
        r, V, Vp, Vpp, dV_ds, dVp_ds = self._terms(r2)
        u = d / r[:, None]
        fe = (Vp / self.eps)[:, None] * u
        fs = dVp_ds[:, None] * u
        Fe = np.zeros_like(q)
        Fs = np.zeros_like(q)
        np.add.at(Fe, i, fe)
        np.add.at(Fe, j, -fe)
        np.add.at(Fs, i, fs)
        np.add.at(Fs, j, -fs)
        return Fe, Fs

    def run(self, q0, p0, steps):
        dt, h = self.dt, 0.5 * self.dt
        q, p = q0.copy(), p0.copy()
        J = 0.0
        states, halves = [(q.copy(), p.copy())], []
        for _ in range(steps):
            qh = q + p * h
            p = p + self.force(qh) * dt
            q = qh + p * h
            halves.append(qh)
            states.append((q.copy(), p.copy()))
            J += self.objective_and_grads(q, p)[0] / steps
        return J, states, halves

    def gradient(self, q0, p0, steps):
        J, states, halves = self.run(q0, p0, steps)
        dt, h, w = self.dt, 0.5 * self.dt, 1.0 / steps
        aq = np.zeros_like(q0)
        ap = np.zeros_like(p0)
        ge = gs = 0.0
        for n in range(steps, 0, -1):
            q, p = states[n]
            _, gq, gp, je, js = self.objective_and_grads(q, p)
            aq += w * gq
            ap += w * gp
            ge += w * je
            gs += w * js
            qh = halves[n - 1]
            ap_k = ap + h * aq                 # through q_n = qh + dt/2 p_n
            aqh = aq - dt * self.hvp(qh, ap_k)  # through p_n = p_{n-1} + dt F(qh)
            Fe, Fs = self.dforce_dparams(qh)
            ge += dt * (ap_k * Fe).sum()
            gs += dt * (ap_k * Fs).sum()
            aq = aqh                           # through qh = q_{n-1} + dt/2 p_{n-1}
            ap = ap_k + h * aqh
        return J, aq, ap, ge, gs
