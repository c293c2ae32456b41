"""GPU parity at the large NVE configuration: 100^3 FCC cells = 4,000,000 atoms
at density 0.5 (L = 200) and 0.8 (L = 170.99759466766969), rc 2.5, margin 0.5.

Against the oracle (the C restatement pinned bitwise to the reference) on the
same state: every FCC site displaced by a seeded uniform offset in
[-0.15, 0.15]^3, Maxwell momenta at T = 1.
  * pair list: the number of directed image pairs within rc + margin equal,
    and the rows of 20,000 sampled particles bit-exact as sets of
    (i, j, image);
  * FP64 forces: |dF_i| <= 1e-12 max(|F_i|, sum_j |f_ij|) per atom and
    ||dF|| <= 1e-12 ||F||;
  * mixed forms: RMS relative force error <= 1e-5 for the compensated
    (MDG_MIXED) and the plain (MDG_MIXED_PLAIN) float sums.
Cases of the reference these follow: meshlist.cc:219-271 (pair search),
fcalculator.cc:229-290 (force).
"""
import numpy as np
import pytest

from oracle import port
from tests.helpers import liquid_like

pytestmark = pytest.mark.gpu

RC, MARGIN, CELLS = 2.5, 0.5, 100


def _row_keys(rec, n, rows, half):
    """Sorted int64 keys (i, j, image) of the directed pairs whose first
    particle is in the boolean mask `rows`.  A half list (the oracle's) holds a
    real-real pair once (image 13): its reverse is added."""
    rec = np.asarray(rec)
    a, b, c = (rec[:, k].astype(np.int64) for k in range(3))
    sel = rows[a]
    keys = [(a[sel] * n + b[sel]) * 27 + c[sel]]
    if half:
        rr = (c == 13) & rows[b]
        keys.append((b[rr] * n + a[rr]) * 27 + 13)
    k = np.concatenate(keys)
    k.sort()
    return k


def _directed_count(rec, half):
    rec = np.asarray(rec)
    return len(rec) + (int(np.count_nonzero(rec[:, 2] == 13)) if half else 0)


def _abs_force_sum(q, L, rec, n, chunk=1 << 24):
    """Per-particle sum of |f_ij| over the half list's pairs within rc (the
    scale of the per-atom force tolerance), in chunks."""
    out = np.zeros(n)
    for s in range(0, len(rec), chunk):
        r = np.asarray(rec[s:s + chunk], dtype=np.int64)
        a, b, c = r[:, 0], r[:, 1], r[:, 2]
        sh = np.stack([c % 3 - 1, (c // 3) % 3 - 1, c // 9 - 1], axis=1) * np.asarray(L)
        d = q[b] + sh - q[a]
        r2 = (d * d).sum(1)
        m = r2 <= RC * RC
        r2 = r2[m]
        f = np.abs(24.0 / r2 ** 4 - 48.0 / r2 ** 7) * np.sqrt(r2)
        out += np.bincount(a[m], weights=f, minlength=n) + np.bincount(b[m], weights=f, minlength=n)
    return out


@pytest.fixture(scope="module", params=[0.5, 0.8], ids=["rho0.5", "rho0.8"])
def headline(request):
    density = request.param
    q, p, L = liquid_like(density, CELLS, seed=41 if density == 0.5 else 43)
    n = len(q)
    assert n == 4_000_000
    ref = port.System(q, p, L, rc=RC, margin=MARGIN)
    ref.make_pairlist()
    rec = ref.pairs()
    fr = ref.forces()
    ref.close()
    return {"density": density, "q": q, "p": p, "L": L, "n": n, "rec": rec, "fr": fr}


def _gpu(case, precision):
    from mdacp_gb300.manager import MDManager
    m = MDManager(case["L"], capacity=case["n"], cutoff=RC, margin=MARGIN, dt=0.001, precision=precision)
    m.set_state(case["q"], case["p"])
    m.make_pairlist()
    return m


def test_headline_pair_list(headline):
    n = headline["n"]
    m = _gpu(headline, "fp64")
    g = m.pairs()
    m.close()
    assert len(g) == _directed_count(headline["rec"], half=True)
    rows = np.zeros(n, dtype=bool)
    rows[np.random.default_rng(7).choice(n, 20_000, replace=False)] = True
    gk = _row_keys(g, n, rows, half=False)
    rk = _row_keys(headline["rec"], n, rows, half=True)
    assert len(gk) == len(rk) > 20_000 * 20
    assert np.array_equal(gk, rk)


def test_headline_forces_fp64(headline):
    q, L, n, fr = headline["q"], headline["L"], headline["n"], headline["fr"]
    m = _gpu(headline, "fp64")
    f = m.forces()
    m.close()
    scale = np.maximum(np.linalg.norm(fr, axis=1), _abs_force_sum(q, L, headline["rec"], n))
    df = np.linalg.norm(f - fr, axis=1)
    assert np.all(df <= 1e-12 * scale), (df / scale).max()
    assert np.linalg.norm(f - fr) <= 1e-12 * np.linalg.norm(fr)


@pytest.mark.parametrize("precision", ["mixed", "mixed_plain"])
def test_headline_mixed_force_error(headline, precision):
    fr = headline["fr"]
    m = _gpu(headline, precision)
    f = m.forces()
    m.close()
    rel = np.linalg.norm(f - fr, axis=1) / np.linalg.norm(fr, axis=1)
    rms = float(np.sqrt(np.mean(rel ** 2)))
    assert rms <= 1e-5, rms
