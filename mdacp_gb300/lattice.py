"""Initial conditions: FCC lattices and seeded Maxwell velocities.

`fcc` places sites the way MDACP's ConfigurationMaker does (confmaker.cc:9-44):
lattice constant s = (4/rho)^(1/3), floor(L/s) unit cells per side, four sites
per cell in the order (0,0,0), (0,h,h), (h,0,h), (h,h,0), each shifted by
e = 1e-7 so no site sits exactly on a face (a site on a face gets no ghost
image in the reference until the first rebuild).

`maxwell` draws velocities from a counter-based generator (splitmix64 ->
Box-Muller), scaled to temperature T and with the net momentum removed, so the
same (n, T, seed) gives the same array on any machine.
"""
import numpy as np

_M64 = np.uint64(0xFFFFFFFFFFFFFFFF)


def fcc(density, L, offset=1e-7, cells=None):
    """Returns (positions [n,3], box [3]).  `cells` forces the cell count per side."""
    L = np.broadcast_to(np.asarray(L, dtype=np.float64), (3,)).copy()
    s = 1.0 / pow(density * 0.25, 1.0 / 3.0)
    hs = s * 0.5
    if cells is None:
        nc = [int(L[d] / s) for d in range(3)]
    else:
        nc = list(np.broadcast_to(cells, (3,)))
    iz, iy, ix = np.meshgrid(np.arange(nc[2], dtype=np.float64), np.arange(nc[1], dtype=np.float64),
                             np.arange(nc[0], dtype=np.float64), indexing="ij")
    bx, by, bz = (ix * s).ravel(), (iy * s).ravel(), (iz * s).ravel()
    sites = [(bx + offset, by + offset, bz + offset),
             (bx + offset, by + hs + offset, bz + hs + offset),
             (bx + hs + offset, by + offset, bz + hs + offset),
             (bx + hs + offset, by + hs + offset, bz + offset)]
    q = np.empty((bx.size, 4, 3))
    for k, (x, y, z) in enumerate(sites):
        q[:, k, 0], q[:, k, 1], q[:, k, 2] = x, y, z
    return q.reshape(-1, 3), L


def fcc_cube(cells, density, offset=1e-7):
    """cells^3 FCC unit cells (4*cells^3 atoms) filling a cube at `density`."""
    L = cells * (4.0 / density) ** (1.0 / 3.0)
    # guard against floor(L/s) rounding down to cells-1
    return fcc(density, L, offset, cells=cells)


def _splitmix64(x):
    x = (x + np.uint64(0x9E3779B97F4A7C15)) & _M64
    z = x
    z = ((z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)) & _M64
    z = ((z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)) & _M64
    return z ^ (z >> np.uint64(31))


def uniform53(seed, count, stream=0):
    """count doubles in (0, 1) from a counter-based splitmix64 stream."""
    base = np.uint64((seed * 0x100000001B3 + stream * 0x9E3779B1) & 0xFFFFFFFFFFFFFFFF)
    with np.errstate(over="ignore"):
        ctr = base + np.arange(count, dtype=np.uint64)
        bits = _splitmix64(ctr) >> np.uint64(11)
    return (bits.astype(np.float64) + 0.5) * (1.0 / 9007199254740992.0)


def maxwell(n, temperature, seed):
    """n x 3 velocities with <v^2>/3 = T (mass 1), zero net momentum."""
    m = 3 * n + (3 * n) % 2
    u1 = uniform53(seed, m // 2, 1)
    u2 = uniform53(seed, m // 2, 2)
    r = np.sqrt(-2.0 * np.log(u1))
    z = np.concatenate([r * np.cos(2 * np.pi * u2), r * np.sin(2 * np.pi * u2)])[:3 * n]
    v = z.reshape(n, 3) * np.sqrt(temperature)
    v -= v.mean(axis=0)
    return v


def thin(q, n_keep, seed):
    """Keeps n_keep sites chosen by a seeded permutation (replica boxes)."""
    u = uniform53(seed, len(q), 7)
    keep = np.sort(np.argsort(u, kind="stable")[:n_keep])
    return q[keep]
