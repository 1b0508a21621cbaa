"""ctypes front end of the CPU oracle (TEST INFRASTRUCTURE).

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline legs
import this module; the product never does.  It loads
``oracle/_build/libpf_oracle.so`` (built by ``make -C oracle``) and exposes
numpy-level wrappers of the functions declared in ``pf_oracle.h``.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libpf_oracle.so")
REF_BIN = os.path.join(HERE, "_ref", "ref_update")

PERIODIC = 2


class _Grid(ctypes.Structure):
    _fields_ = [("dim", ctypes.c_int), ("n", ctypes.c_int * 3),
                ("dx", ctypes.c_double * 3), ("bc", (ctypes.c_int * 2) * 3)]


_lib = None


def build() -> None:
    subprocess.run(["make", "-s", "-C", HERE], check=True)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = ctypes.CDLL(LIB_PATH)
        dp = ctypes.POINTER(ctypes.c_double)
        gp = ctypes.POINTER(_Grid)
        for name, args in [
            ("pfo_ch_baseline", [gp, dp, ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_int]),
            ("pfo_ch_shipped", [gp, dp, ctypes.c_int] + [ctypes.c_double] * 5 + [ctypes.c_int]),
            ("pfo_ac_baseline", [gp, ctypes.c_int, dp, ctypes.c_int] + [ctypes.c_double] * 4 + [ctypes.c_int]),
            ("pfo_ac_graingrowth", [gp, ctypes.c_int, dp, ctypes.c_int, ctypes.c_double, ctypes.c_int]),
            ("pfo_ac_zener", [gp, ctypes.c_int, dp, ctypes.c_int, ctypes.c_double, ctypes.c_int]),
            ("pfo_ostwald", [gp, ctypes.c_int, dp, ctypes.c_int] + [ctypes.c_double] * 9 + [ctypes.c_int]),
            ("pfo_ch_convex", [gp, dp, ctypes.c_int] + [ctypes.c_double] * 9 + [ctypes.POINTER(ctypes.c_int)]),
            ("pfo_ch_shipped_noise", [gp, dp, ctypes.c_int] + [ctypes.c_double] * 6
             + [ctypes.c_uint64, ctypes.c_longlong, ctypes.c_int]),
            ("pfo_ac_scalar_noise", [gp, dp, ctypes.c_int] + [ctypes.c_double] * 6
             + [ctypes.c_uint64, ctypes.c_longlong, ctypes.c_int]),
            ("pfo_ac_scalar_shipped", [gp, dp, ctypes.c_int] + [ctypes.c_double] * 5 + [ctypes.c_int]),
            ("pfo_laplacian", [gp, dp, dp]),
            ("pfo_sparse_gg", [gp, ctypes.c_int, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int), dp,
                               ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.c_int,
                               ctypes.POINTER(ctypes.c_int)]),
            ("pfo_ch_mass_energy", [gp, dp, ctypes.c_double, dp, dp]),
            ("pfo_ac_mass_energy", [gp, ctypes.c_int, dp, ctypes.c_double, ctypes.c_double, dp, dp]),
        ]:
            f = getattr(L, name)
            f.argtypes = args
            f.restype = ctypes.c_int
        L.pfo_pow3.argtypes = [dp, dp, ctypes.c_long]
        L.pfo_pow3.restype = None
        L.pfo_gaussian.argtypes = [ctypes.c_uint64, ctypes.c_uint64]
        L.pfo_gaussian.restype = ctypes.c_double
        _lib = L
    return _lib


def _grid(shape, dx=None, bc=None) -> _Grid:
    g = _Grid()
    g.dim = len(shape)
    for a, s in enumerate(shape):
        g.n[a] = int(s)
        g.dx[a] = 1.0 if dx is None else float(dx[a])
        lo, hi = (PERIODIC, PERIODIC) if bc is None else bc[a]
        g.bc[a][0] = lo
        g.bc[a][1] = hi
    return g


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _check(rc, name):
    if rc != 0:
        raise ValueError("%s: oracle refused the arguments (%d)" % (name, rc))


def ch_baseline(c, steps, kappa=1.0, M=1.0, dt=0.005, dx=None, bc=None, threads=0):
    out = np.array(c, dtype=np.float64, order="C", copy=True)
    g = _grid(out.shape, dx, bc)
    _check(lib().pfo_ch_baseline(ctypes.byref(g), _ptr(out), int(steps), kappa, M, dt, threads), "ch_baseline")
    return out


def ch_shipped(c, steps, r=1.0, u=1.0, K=1.0, M=1.0, dt=0.01, dx=None, bc=None, threads=0):
    out = np.array(c, dtype=np.float64, order="C", copy=True)
    g = _grid(out.shape, dx, bc)
    _check(lib().pfo_ch_shipped(ctypes.byref(g), _ptr(out), int(steps), r, u, K, M, dt, threads), "ch_shipped")
    return out


def ac_baseline(eta, steps, gamma=1.5, kappa=2.0, L=1.0, dt=0.05, dx=None, bc=None, threads=0):
    """``eta`` has shape grid_shape + (N,) (cell-major)."""
    out = np.array(eta, dtype=np.float64, order="C", copy=True)
    g = _grid(out.shape[:-1], dx, bc)
    _check(lib().pfo_ac_baseline(ctypes.byref(g), out.shape[-1], _ptr(out), int(steps),
                                 gamma, kappa, L, dt, threads), "ac_baseline")
    return out


def ac_graingrowth(eta, steps, dt=0.01, dx=None, bc=None, threads=0):
    out = np.array(eta, dtype=np.float64, order="C", copy=True)
    g = _grid(out.shape[:-1], dx, bc)
    _check(lib().pfo_ac_graingrowth(ctypes.byref(g), out.shape[-1], _ptr(out), int(steps), dt, threads),
           "ac_graingrowth")
    return out


def ac_zener(eta, steps, dt=0.01, dx=None, bc=None, threads=0):
    """Zener pinning as shipped: grain growth with field 0 (particles) fixed."""
    out = np.array(eta, dtype=np.float64, order="C", copy=True)
    g = _grid(out.shape[:-1], dx, bc)
    _check(lib().pfo_ac_zener(ctypes.byref(g), out.shape[-1], _ptr(out), int(steps), dt, threads), "ac_zener")
    return out


def ostwald(eta, steps, dt=0.001, L=1.0, D=1.0, Calpha=0.05, Cbeta=0.95, A=2.0, delta=1.0, epsilon=3.0,
            kappa=2.0, dx=None, bc=None, threads=0):
    """Ostwald ripening as shipped; ``eta`` has shape grid_shape + (N,), field 0 the composition."""
    out = np.array(eta, dtype=np.float64, order="C", copy=True)
    g = _grid(out.shape[:-1], dx, bc)
    _check(lib().pfo_ostwald(ctypes.byref(g), out.shape[-1], _ptr(out), int(steps), dt, L, D, Calpha, Cbeta, A,
                             delta, epsilon, kappa, threads), "ostwald")
    return out


def ch_convex(cm, steps, dt=None, D=None, K=2.0, C0=0.45, Ca=0.05, Cb=0.95, A=2.0, omega=1.2, tolerance=1e-14,
              dx=None, bc=None, return_iters=False):
    """Convex-splitting Cahn-Hilliard as shipped; ``cm`` has shape grid_shape + (2,) (c, mu).
    Defaults are the example's: D = 2/(Cb-Ca), dt = 1/(D*K)."""
    if D is None:
        D = 2.0 / (Cb - Ca)
    if dt is None:
        dt = 1.0 / (D * K)
    out = np.array(cm, dtype=np.float64, order="C", copy=True)
    g = _grid(out.shape[:-1], dx, bc)
    it = ctypes.c_int(0)
    rc = lib().pfo_ch_convex(ctypes.byref(g), _ptr(out), int(steps), dt, D, K, C0, Ca, Cb, A, omega, tolerance,
                             ctypes.byref(it))
    if rc == -2:
        raise RuntimeError("convex splitting stagnated (10000 iterations)")
    _check(rc, "ch_convex")
    return (out, it.value) if return_iters else out


def gaussian(seed, k):
    """Deviate k of the counter-based normal stream `seed` (pfo_gaussian)."""
    return lib().pfo_gaussian(int(seed), int(k))


def ch_shipped_noise(c, steps, r=1.0, u=1.0, K=1.0, M=1.0, dt=0.01, noise=0.0, seed=0, step0=0, dx=None, bc=None,
                     threads=0):
    """Shipped Cahn-Hilliard with gaussian(0, noise) added to mu (model B, spinodal)."""
    out = np.array(c, dtype=np.float64, order="C", copy=True)
    g = _grid(out.shape, dx, bc)
    _check(lib().pfo_ch_shipped_noise(ctypes.byref(g), _ptr(out), int(steps), r, u, K, M, dt, noise, int(seed),
                                      int(step0), threads), "ch_shipped_noise")
    return out


def ac_scalar_noise(phi, steps, r=1.0, u=1.0, K=1.0, M=1.0, dt=0.01, noise=0.0, seed=0, step0=0, dx=None, bc=None,
                    threads=0):
    """Shipped scalar Allen-Cahn with gaussian(0, noise) in the bracket (model A)."""
    out = np.array(phi, dtype=np.float64, order="C", copy=True)
    g = _grid(out.shape, dx, bc)
    _check(lib().pfo_ac_scalar_noise(ctypes.byref(g), _ptr(out), int(steps), r, u, K, M, dt, noise, int(seed),
                                     int(step0), threads), "ac_scalar_noise")
    return out


def ac_scalar_shipped(phi, steps, r=1.0, u=1.0, K=1.0, M=1.0, dt=0.01, dx=None, bc=None, threads=0):
    out = np.array(phi, dtype=np.float64, order="C", copy=True)
    g = _grid(out.shape, dx, bc)
    _check(lib().pfo_ac_scalar_shipped(ctypes.byref(g), _ptr(out), int(steps), r, u, K, M, dt, threads),
           "ac_scalar_shipped")
    return out


def laplacian(f, dx=None, bc=None):
    f = np.ascontiguousarray(f, dtype=np.float64)
    out = np.empty_like(f)
    g = _grid(f.shape, dx, bc)
    _check(lib().pfo_laplacian(ctypes.byref(g), _ptr(f), _ptr(out)), "laplacian")
    return out


def ch_mass_energy(c, kappa=1.0, dx=None, bc=None):
    c = np.ascontiguousarray(c, dtype=np.float64)
    g = _grid(c.shape, dx, bc)
    m = ctypes.c_double()
    e = ctypes.c_double()
    _check(lib().pfo_ch_mass_energy(ctypes.byref(g), _ptr(c), kappa, ctypes.byref(m), ctypes.byref(e)),
           "ch_mass_energy")
    return m.value, e.value


def ac_mass_energy(eta, gamma=1.5, kappa=2.0, dx=None, bc=None):
    eta = np.ascontiguousarray(eta, dtype=np.float64)
    N = eta.shape[-1]
    g = _grid(eta.shape[:-1], dx, bc)
    m = np.zeros(N)
    e = ctypes.c_double()
    _check(lib().pfo_ac_mass_energy(ctypes.byref(g), N, _ptr(eta), gamma, kappa, _ptr(m), ctypes.byref(e)),
           "ac_mass_energy")
    return m, e.value


def pow3(x):
    x = np.ascontiguousarray(x, dtype=np.float64)
    y = np.empty_like(x)
    lib().pfo_pow3(_ptr(x), _ptr(y), x.size)
    return y


def ref_available() -> bool:
    return os.path.exists(REF_BIN)


def sparse_gg(cnt, idx, val, steps, dt=0.01, eps=1e-8, dx=None, bc=None, threads=0):
    """Sparse phase-field grain growth (pfo_sparse_gg): one update() call of
    the sparsePF example.  cnt has the grid's shape (items per cell); idx and
    val have shape + (K,), the first cnt items of each cell in stored order.
    Returns (cnt, idx, val, longest list seen)."""
    cnt = np.array(cnt, dtype=np.int32, order="C", copy=True)
    K = int(np.asarray(idx).shape[-1])
    idx = np.array(idx, dtype=np.int32, order="C", copy=True)
    val = np.array(val, dtype=np.float64, order="C", copy=True)
    assert idx.shape == cnt.shape + (K,) and val.shape == idx.shape
    g = _grid(cnt.shape, dx, bc)
    longest = ctypes.c_int(0)
    ip = ctypes.POINTER(ctypes.c_int)
    rc = lib().pfo_sparse_gg(ctypes.byref(g), K, cnt.ctypes.data_as(ip), idx.ctypes.data_as(ip), _ptr(val),
                             int(steps), float(dt), float(eps), int(threads), ctypes.byref(longest))
    if rc == -3:
        raise OverflowError("a sparse cell list exceeded %d items" % K)
    _check(rc, "sparse_gg")
    return cnt, idx, val, longest.value
