"""Seeded synthetic initial conditions.

The reference seeds ``rand()`` with the wall clock (include/MMSP.main.hpp:55),
so its examples are not reproducible.  These generators replace it with a
counter-based SplitMix64 stream (Steele, Lea and Flood, "Fast splittable
pseudorandom number generators", OOPSLA 2014): value ``i`` of stream ``seed``
depends only on ``(seed, i)``, so every run, machine and thread count sees
the same bytes.  Doubles take the top 53 bits: ``u = (z >> 11) * 2**-53``.
"""
from __future__ import annotations

import numpy as np

_GAMMA = np.uint64(0x9E3779B97F4A7C15)
_M1 = np.uint64(0xBF58476D1CE4E5B9)
_M2 = np.uint64(0x94D049BB133111EB)


def splitmix64(seed: int, n: int, start: int = 0) -> np.ndarray:
    """Values ``start .. start+n-1`` of the SplitMix64 stream for ``seed``."""
    with np.errstate(over="ignore"):
        idx = np.arange(start + 1, start + n + 1, dtype=np.uint64)
        z = np.uint64(seed & 0xFFFFFFFFFFFFFFFF) + idx * _GAMMA
        z = (z ^ (z >> np.uint64(30))) * _M1
        z = (z ^ (z >> np.uint64(27))) * _M2
        z = z ^ (z >> np.uint64(31))
    return z


def uniform(seed: int, n: int, start: int = 0) -> np.ndarray:
    """Doubles in [0, 1)."""
    z = splitmix64(seed, n, start)
    return (z >> np.uint64(11)).astype(np.float64) * (2.0 ** -53)


def noisy_composition(shape, mean: float, amplitude: float, seed: int) -> np.ndarray:
    """``c = mean + amplitude * U(-1, 1)`` i.i.d. per cell, node order."""
    n = int(np.prod(shape))
    u = uniform(seed, n)
    return (mean + amplitude * (2.0 * u - 1.0)).reshape(shape)


def voronoi_grain_ids(shape, points: int, seed: int) -> np.ndarray:
    """Grain index of every cell of a periodic Voronoi tessellation of
    ``points`` seeds drawn uniformly in the box (one stream value per
    coordinate): the seed nearest by the periodic minimum-image distance,
    the lowest index on a tie.  Returns an int64 array of shape ``shape``."""
    shape = tuple(int(s) for s in shape)
    dim = len(shape)
    u = uniform(seed, points * dim).reshape(points, dim)
    pts = u * np.asarray(shape, dtype=np.float64)
    ncell = int(np.prod(shape))
    grain = np.empty(ncell, dtype=np.int64)
    grids = np.indices(shape).reshape(dim, -1).T.astype(np.float64)
    L = np.asarray(shape, dtype=np.float64)
    chunk = max(1, (1 << 22) // max(points, 1))
    for s in range(0, ncell, chunk):
        x = grids[s:s + chunk]
        d2 = np.zeros((x.shape[0], points))
        for a in range(dim):
            d = np.abs(x[:, a:a + 1] - pts[None, :, a])
            d = np.minimum(d, L[a] - d)
            d2 += d * d
        grain[s:s + chunk] = np.argmin(d2, axis=1)
    return grain.reshape(shape)


def voronoi_grains(shape, points: int, fields: int, seed: int) -> np.ndarray:
    """Order parameters of a periodic Voronoi tessellation.

    ``points`` seeds are drawn uniformly in the box (one stream value per
    coordinate).  Each cell belongs to the seed nearest by the periodic
    minimum-image distance (lowest seed index on a tie); ``eta_k = 1`` for
    ``k = grain % fields`` and 0 otherwise.  Returns shape ``shape + (fields,)``.
    """
    shape = tuple(int(s) for s in shape)
    ncell = int(np.prod(shape))
    grain = voronoi_grain_ids(shape, points, seed).ravel()
    eta = np.zeros((ncell, fields), dtype=np.float64)
    eta[np.arange(ncell), grain % fields] = 1.0
    return eta.reshape(shape + (fields,))


def batched_cahn_hilliard(count: int = 256, seed: int = 4, sides=tuple(range(64, 513, 32)),
                          amplitude: float = 0.01):
    """The batched 2D Cahn-Hilliard workload: `count` square grids with sides
    drawn uniformly from `sides`, each with its own kappa ~ U(0.5, 2) and mean
    composition ~ U(0.3, 0.7), c = mean + amplitude*U(-1, 1) per cell.

    Returns a list of (c0, kappa) pairs.  Stream `seed` gives the per-grid
    draws (3 values per grid); grid i's cells use stream seed*1000003 + i.
    """
    u = uniform(seed, 3 * count).reshape(count, 3)
    out = []
    for i in range(count):
        side = int(sides[min(int(u[i, 0] * len(sides)), len(sides) - 1)])
        kappa = 0.5 + 1.5 * u[i, 1]
        mean = 0.3 + 0.4 * u[i, 2]
        c0 = noisy_composition((side, side), mean, amplitude, seed * 1000003 + i)
        out.append((c0, float(kappa)))
    return out


def graingrowth_circles(shape, fields: int = 2) -> np.ndarray:
    """The shipped grain-growth start state (graingrowth.cpp:34-51 in 2D/3D,
    :18-30 in 1D): field 1 inside circles of radius 16 on a period-64
    lattice of the first two axes, field 0 elsewhere."""
    shape = tuple(int(s) for s in shape)
    x = np.indices(shape)
    if len(shape) == 1:
        inside = (32 - x[0] % 64) < 16.0
    else:
        r = np.sqrt((32 - x[0] % 64) ** 2.0 + (32 - x[1] % 64) ** 2.0)
        inside = r < 16.0
    eta = np.zeros(shape + (fields,), dtype=np.float64)
    eta[..., 0] = np.where(inside, 0.0, 1.0)
    eta[..., 1] = np.where(inside, 1.0, 0.0)
    return eta


def zener_particles(shape, particles: int, seed: int) -> np.ndarray:
    """The shipped Zener-pinning start state
    (examples/coarsening/zener_pinning/isotropic/phase_field/zener.cpp:14-95),
    with seeded positions: field 0 holds the particles, fields 1 and 2 the
    matrix grain and the period-64 circles of graingrowth_circles; each
    particle sets a 3-cell cube (3 cells per axis, wrapped periodically)
    to (1, 0, 0)."""
    shape = tuple(int(s) for s in shape)
    eta = np.zeros(shape + (3,), dtype=np.float64)
    eta[..., 1:] = graingrowth_circles(shape, 2)
    n = int(np.prod(shape))
    centre = (uniform(seed, particles) * n).astype(np.int64)
    for c in centre:
        x = np.unravel_index(int(c), shape)
        offs = np.indices((3,) * len(shape)).reshape(len(shape), -1).T - 1
        for o in offs:
            p = tuple((xi + oi) % si for xi, oi, si in zip(x, o, shape))
            eta[p] = (1.0, 0.0, 0.0)
    return eta


def ostwald_start(shape, fields: int, seed: int) -> np.ndarray:
    """The shipped Ostwald-ripening start state
    (examples/coarsening/ostwald_ripening/isotropic/phase_field/ostwald.cpp:13-54),
    with a seeded stream: composition r ~ U(0, 1) per cell and the first
    order parameter 1 - r; further order parameters (beyond the example's
    two fields) start at 0.1 * U(0, 1)."""
    shape = tuple(int(s) for s in shape)
    n = int(np.prod(shape))
    eta = np.zeros(shape + (fields,), dtype=np.float64)
    r = uniform(seed, n).reshape(shape)
    eta[..., 0] = r
    eta[..., 1] = 1.0 - r
    for j in range(2, fields):
        eta[..., j] = 0.1 * uniform(seed, n, start=j * n).reshape(shape)
    return eta


def convex_start(shape, seed=None, C0: float = 0.45, K: float = 2.0, Ca: float = 0.05, Cb: float = 0.95,
                 A: float = 2.0) -> np.ndarray:
    """Start state of the convex-splitting Cahn-Hilliard example
    (examples/phase_transitions/cahn-hilliard/convex_splitting/cahn-hilliard.cpp:
    229-250): c = C0 (1 + 0.1 cos(q . x)) with q = 0.1 (sqrt 2, sqrt 3, sqrt 5)
    (the 2D benchmark stripes) or, with a seed, c = C0 + 0.25 U(0,1) - 0.125;
    then mu = f'(c) - K lap c with the parametric f of :57-96 (periodic,
    dx = 1).  Shape grid_shape + (2,), cell-major (c, mu)."""
    shape = tuple(int(s) for s in shape)
    if seed is None:
        q = (0.1 * np.sqrt(2.0), 0.1 * np.sqrt(3.0), 0.1 * np.sqrt(5.0))
        x = np.indices(shape).astype(np.float64)
        wave = sum(x[a] * q[a] for a in range(len(shape)))
        c = C0 * (1.0 + 0.1 * np.cos(wave))
    else:
        c = C0 + 0.25 * uniform(seed, int(np.prod(shape))).reshape(shape) - 0.125
    B = A / (Ca - C0) ** 2
    dfdc = -A * (c - C0) + B * (c - C0) ** 3 + Ca * (c - Ca) ** 3 + Cb * (c - Cb) ** 3
    lap = sum(np.roll(c, 1, a) + np.roll(c, -1, a) - 2.0 * c for a in range(len(shape)))
    out = np.empty(shape + (2,))
    out[..., 0] = c
    out[..., 1] = dfdc - K * lap
    return out


def sparse_grains(shape, points: int, seed: int, capacity: int):
    """A sparse grain start state (grid<dim,sparse<double>>): each cell holds one
    item (its periodic Voronoi grain index, 1.0), as the sparsePF example's
    cells start with one set() each (sparsePF/graingrowth.cpp:14-56).
    Returns (count, index, value) with `capacity` slots per cell."""
    shape = tuple(int(s) for s in shape)
    cnt = np.ones(shape, np.int32)
    idx = np.zeros(shape + (capacity,), np.int32)
    val = np.zeros(shape + (capacity,), np.float64)
    idx[..., 0] = voronoi_grain_ids(shape, points, seed)
    val[..., 0] = 1.0
    return cnt, idx, val


def sparse_circles(shape, capacity: int):
    """The sparsePF example's own start state (sparsePF/graingrowth.cpp:14-56):
    index 1 where the distance r < 16 (2D/3D: r from (32, 32) on a period-64
    lattice of the first two axes; 1D: r = 32 - x), index 0 elsewhere, value 1.0."""
    shape = tuple(int(s) for s in shape)
    x = np.indices(shape)
    if len(shape) == 1:
        r = 32.0 - x[0]
    else:
        r = np.sqrt((32 - x[0] % 64) ** 2.0 + (32 - x[1] % 64) ** 2.0)
    cnt = np.ones(shape, np.int32)
    idx = np.zeros(shape + (capacity,), np.int32)
    val = np.zeros(shape + (capacity,), np.float64)
    idx[..., 0] = (r < 16.0).astype(np.int32)
    val[..., 0] = 1.0
    return cnt, idx, val
