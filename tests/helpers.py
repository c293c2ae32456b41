"""Seeded inputs shared by the tests."""
import numpy as np

from mdacp_gb300 import lattice


def wrap(q, L):
    q = np.mod(q, L)
    return np.where(q >= L, q - L, q)


def liquid_like(density, cells, amp=0.15, temperature=1.0, seed=1):
    """FCC of cells^3 unit cells at `density`, each site displaced by a seeded
    uniform offset in [-amp, amp]^3 and wrapped into [0, L); Maxwell momenta."""
    q, L = lattice.fcc_cube(cells, density)
    u = lattice.uniform53(seed, q.size, 11).reshape(q.shape)
    q = wrap(q + amp * (2.0 * u - 1.0), L)
    p = lattice.maxwell(len(q), temperature, seed)
    return q, p, L


def directed_pair_keys(rec, n, half=True):
    """int64 keys of directed image pairs.  A half list (the reference's) lists a
    real-real pair once (code 13) and each real-ghost pair from its real side."""
    rec = np.asarray(rec, dtype=np.int64)
    a, b, c = rec[:, 0], rec[:, 1], rec[:, 2]
    keys = [(a * n + b) * 27 + c]
    if half:
        rr = c == 13
        keys.append((b[rr] * n + a[rr]) * 27 + 13)
    k = np.concatenate(keys)
    k.sort()
    return k


def pair_force_abs_sum(q, L, rec, rc, half=True):
    """Per-particle sum of |f_ij| over the pairs within rc (scale for force tolerances)."""
    rec = np.asarray(rec, dtype=np.int64)
    a, b, c = rec[:, 0], rec[:, 1], rec[:, 2]
    sh = np.stack([c % 3 - 1, (c // 3) % 3 - 1, c // 9 - 1], axis=1) * np.asarray(L)
    d = q[b] + sh - q[a]
    r2 = (d * d).sum(1)
    m = r2 <= rc * rc
    r2 = r2[m]
    f = np.abs(24.0 / r2 ** 4 - 48.0 / r2 ** 7) * np.sqrt(r2)
    out = np.zeros(len(q))
    np.add.at(out, a[m], f)
    if half:
        np.add.at(out, b[m], f)
    return out
