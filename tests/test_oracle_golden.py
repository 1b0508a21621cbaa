"""The CPU oracle against the reference's own outputs (golden vectors).

tests/golden/*.npz were produced by the reference's grid/laplacian/update
loops (oracle/ref_api/ref_update.cpp compiled from the reference headers,
tests/golden/make_golden.py).  The C restatement must reproduce every one
bit for bit.  When the reference program is built in this checkout, random
extra cases are run through it directly as well.
"""
import glob
import hashlib
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN

FIXTURES = sorted(f for f in glob.glob(os.path.join(GOLDEN, "*.npz"))
                  if not os.path.basename(f).startswith("sparse"))
SPARSE_FIXTURES = sorted(glob.glob(os.path.join(GOLDEN, "sparse*.npz")))


def run_oracle(o, z, x=None, steps=None):
    m = str(z["model"])
    p = [float(v) for v in z["params"]]
    st = int(z["steps"]) if steps is None else steps
    dx = z["dx"].tolist()
    bc = z["bc"].tolist()
    x = z["start"] if x is None else x
    if m == "ch_baseline":
        return o.ch_baseline(x, st, *p, dx=dx, bc=bc)
    if m == "ch_shipped":
        return o.ch_shipped(x, st, *p, dx=dx, bc=bc)
    if m == "ac_scalar":
        return o.ac_scalar_shipped(x, st, *p, dx=dx, bc=bc)
    if m == "ac_baseline":
        return o.ac_baseline(x, st, *p, dx=dx, bc=bc)
    if m == "graingrowth":
        return o.ac_graingrowth(x, st, *p, dx=dx, bc=bc)
    if m == "zener":
        return o.ac_zener(x, st, *p, dx=dx, bc=bc)
    if m == "ostwald":
        return o.ostwald(x, st, *p, dx=dx, bc=bc)
    if m == "ch_convex":
        keys = ("dt", "D", "K", "C0", "Ca", "Cb", "A", "omega", "tolerance")
        out, iters = o.ch_convex(x, st, dx=dx, bc=bc, return_iters=True, **dict(zip(keys, p)))
        if "iterations" in z.files and steps is None:
            assert iters == int(z["iterations"]), (iters, int(z["iterations"]))
        return out
    raise ValueError(m)


def test_fixtures_present():
    assert len(FIXTURES) >= 12


@pytest.mark.parametrize("path", FIXTURES, ids=[os.path.basename(f)[:-4] for f in FIXTURES])
def test_oracle_matches_reference_bitwise(oracle, path):
    z = np.load(path)
    got = run_oracle(oracle, z)
    want = z["result"]
    assert got.shape == want.shape
    assert np.array_equal(got, want), "max |diff| %g" % np.abs(got - want).max()
    # the fixture must actually move: a fixed point would pin nothing
    assert np.abs(want - z["start"]).max() > 1e-6


def test_threads_do_not_change_bits(oracle):
    from mmsp_gb300 import inputs

    c = inputs.noisy_composition((9, 10, 11), 0.4, 0.02, 5)
    a = oracle.ch_baseline(c, 7, threads=1)
    b = oracle.ch_baseline(c, 7, threads=4)
    assert np.array_equal(a, b)
    e = inputs.voronoi_grains((6, 7, 8), 5, 3, 6)
    assert np.array_equal(oracle.ac_baseline(e, 5, threads=1), oracle.ac_baseline(e, 5, threads=3))


def test_full_size_2d_checksum(oracle):
    """2D Cahn-Hilliard 256x256, 2000 steps: the oracle reproduces the
    reference's result (SHA-256 recorded when the reference ran it)."""
    from mmsp_gb300 import inputs

    meta = json.load(open(os.path.join(GOLDEN, "full_size.json")))["ch2d_256_2000"]
    assert meta["source"] == "reference"
    c0 = inputs.noisy_composition(tuple(meta["shape"]), meta["mean"], meta["amplitude"], meta["seed"])
    out = oracle.ch_baseline(c0, meta["steps"], meta["kappa"], meta["M"], meta["dt"])
    assert hashlib.sha256(np.ascontiguousarray(out, "<f8").tobytes()).hexdigest() == meta["sha256"]
    m, e = oracle.ch_mass_energy(out, meta["kappa"])
    assert m == pytest.approx(meta["mass"], rel=1e-13)
    assert e == pytest.approx(meta["energy"], rel=1e-13)


def test_mass_energy_definitions(oracle):
    # uniform state: no gradient, energy = N * f(c), mass = N * c * dV
    c = np.full((4, 5), 0.3)
    m, e = oracle.ch_mass_energy(c, 1.0, dx=[0.5, 2.0])
    assert m == pytest.approx(20 * 0.3 * 1.0)
    assert e == pytest.approx(20 * (0.3 ** 2 * 0.7 ** 2) * 1.0)
    eta = np.zeros((3, 3, 2))
    eta[..., 0] = 1.0
    m2, e2 = oracle.ac_mass_energy(eta, 1.5, 2.0)
    assert list(m2) == [9.0, 0.0]
    assert e2 == pytest.approx(9 * (-0.5 + 0.25))


def test_oracle_rejects_undefined_mapping(oracle):
    # mirror on an extent-1 axis would index outside the grid in the reference
    with pytest.raises(ValueError):
        oracle.ch_baseline(np.zeros((1, 4)), 1, bc=[[0, 0], [2, 2]])


@pytest.mark.skipif(not os.path.exists(os.path.join(os.path.dirname(GOLDEN), "..", "oracle", "_ref", "ref_update")),
                    reason="reference program not built in this checkout")
@pytest.mark.parametrize("case", range(4))
def test_oracle_random_cases_against_reference_program(oracle, case):
    import sys
    sys.path.insert(0, GOLDEN)
    import make_golden
    from mmsp_gb300 import inputs

    rng = np.random.default_rng(100 + case)
    dim = 1 + case % 3
    shape = tuple(int(s) for s in rng.integers(2, 9, size=dim))
    if case % 2 == 0:
        x0 = inputs.noisy_composition(shape, 0.45, 0.05, 200 + case)
        ref, _ = make_golden.run_ref("ch_baseline", x0, False, 0, 13, (0.9, 1.1, 0.004))
        got = oracle.ch_baseline(x0, 13, 0.9, 1.1, 0.004)
    else:
        x0 = inputs.voronoi_grains(shape, 4, 3, 300 + case)
        ref, _ = make_golden.run_ref("ac_baseline", x0, True, 3, 11, (1.5, 2.0, 1.0, 0.05))
        got = oracle.ac_baseline(x0, 11, 1.5, 2.0, 1.0, 0.05)
    assert np.array_equal(ref, got)


def sparse_slots(z, capacity):
    """Start state of a sparse fixture in `capacity` slots per cell."""
    c0 = z["start_count"]
    k = z["start_index"].shape[-1]
    idx = np.zeros(c0.shape + (capacity,), np.int32)
    val = np.zeros(c0.shape + (capacity,), np.float64)
    idx[..., :k] = z["start_index"]
    val[..., :k] = z["start_value"]
    return c0, idx, val


@pytest.mark.parametrize("path", SPARSE_FIXTURES, ids=[os.path.basename(f)[:-4] for f in SPARSE_FIXTURES])
def test_sparse_oracle_matches_reference_fixture(oracle, path):
    """Sparse phase-field grain growth: counts, indices (in stored order) and
    values bit for bit against the reference's grid<dim,sparse<double>>."""
    z = np.load(path)
    dt, eps = [float(v) for v in z["params"]]
    c0, i0, v0 = sparse_slots(z, 16)
    cnt, idx, val, _ = oracle.sparse_gg(c0, i0, v0, int(z["steps"]), dt, eps)
    k = z["index"].shape[-1]
    assert np.array_equal(cnt, z["count"])
    live = np.arange(k) < cnt[..., None]
    assert np.array_equal(np.where(live, idx[..., :k], 0), np.where(live, z["index"], 0))
    assert np.array_equal(np.where(live, val[..., :k], 0.0), np.where(live, z["value"], 0.0))


def test_sparse_oracle_overflow_and_threads(oracle):
    """A list that would outgrow its slots is an error, not a silent drop;
    threaded runs equal the serial one."""
    from mmsp_gb300 import inputs

    c0, i0, v0 = inputs.sparse_grains((24, 20), 9, 5, 3)
    with pytest.raises(OverflowError):
        oracle.sparse_gg(c0, i0, v0, 60)
    c0, i0, v0 = inputs.sparse_grains((24, 20), 9, 5, 16)
    a = oracle.sparse_gg(c0, i0, v0, 30, threads=1)
    b = oracle.sparse_gg(c0, i0, v0, 30, threads=4)
    for x, y in zip(a[:3], b[:3]):
        assert np.array_equal(x, y)
