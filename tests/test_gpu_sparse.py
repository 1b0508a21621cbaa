"""Sparse phase-field grain growth on the device, through the C ABI.

The reference's sparsePF update (examples/coarsening/grain_growth/isotropic/
sparsePF/graingrowth.cpp:58-120) on grid<dim,sparse<double>>: per cell a list
of (grain index, value) items in insertion order.  Against the fixtures made
by the reference itself (tests/golden/sparse*.npz) and against the oracle on
seeded grain structures: counts and indices in their stored order exactly,
values within 1e-12 relative (pow(x,3) is a compensated cube on the device).
"""
import ctypes
import glob
import os

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu

SPARSE_FIXTURES = sorted(glob.glob(os.path.join(GOLDEN, "sparse*.npz")))
TOL = 1e-12


def slots(count, index, value, K):
    """Pad (or cut) the slot axis to K; slots past a cell's count are zero."""
    idx = np.zeros(count.shape + (K,), np.int32)
    val = np.zeros(count.shape + (K,), np.float64)
    k = min(K, index.shape[-1])
    idx[..., :k] = index[..., :k]
    val[..., :k] = value[..., :k]
    live = np.arange(K) < count[..., None]
    return np.where(live, idx, 0), np.where(live, val, 0.0)


def assert_same_lists(got, want, K):
    gc, gi, gv = got
    wc, wi, wv = want
    assert np.array_equal(gc, wc), "counts differ in %d cells" % int((gc != wc).sum())
    gi, gv = slots(gc, gi, gv, K)
    wi, wv = slots(wc, wi, wv, K)
    assert np.array_equal(gi, wi), "indices differ"
    scale = max(np.abs(wv).max(), 1e-300)
    assert np.abs(gv - wv).max() / scale <= TOL, np.abs(gv - wv).max()


def run(native, shape, K, start, steps_list, dx=None, **kw):
    d = native.make_desc(shape, K, np.float64, "sparse_gg", dx=dx, **kw)
    with native.Stepper(d) as s:
        c0, i0, v0 = start
        i0, v0 = slots(c0, i0, v0, K)
        s.sparse_upload(c0, i0, v0)
        for n in steps_list:
            s.step(n)
        return s.sparse_download()


@pytest.mark.parametrize("K", [16, 32])
@pytest.mark.parametrize("path", SPARSE_FIXTURES, ids=[os.path.basename(f)[:-4] for f in SPARSE_FIXTURES])
def test_sparse_matches_reference_fixture(gpu, path, K):
    z = np.load(path)
    dt, eps = [float(v) for v in z["params"]]
    shape = z["start_count"].shape
    got = run(gpu, shape, K, (z["start_count"], z["start_index"], z["start_value"]), [int(z["steps"])],
              dt=dt, epsilon=eps)
    assert_same_lists(got, (z["count"], z["index"], z["value"]), K)


CASES = [((40, 36), 10, 5, 130, None), ((33, 17), 7, 6, 60, [1.2, 0.9]), ((12, 14, 10), 9, 7, 40, None),
         ((9, 8, 16), 5, 8, 25, [1.0, 1.5, 0.8]), ((200,), 6, 9, 150, None)]


@pytest.mark.parametrize("shape,grains,seed,steps,dx", CASES, ids=["x".join(map(str, c[0])) for c in CASES])
def test_sparse_against_oracle(gpu, oracle, shape, grains, seed, steps, dx):
    """Seeded grain structures, ragged shapes, dx != 1, 1D-3D, graph-replayed
    runs (>= 128 steps)."""
    from mmsp_gb300 import inputs

    K = 24
    start = inputs.sparse_grains(shape, grains, seed, K)
    want = oracle.sparse_gg(*start, steps, 0.01, 1e-8, dx=dx)[:3]
    got = run(gpu, shape, K, start, [steps], dx=dx)
    assert_same_lists(got, want, K)


def test_sparse_each_call_starts_a_fresh_newgrid(gpu, oracle):
    """Two step calls equal two update() calls (each builds an empty newGrid),
    not one call of the summed steps: the stale items differ."""
    from mmsp_gb300 import inputs

    K = 24
    start = inputs.sparse_grains((30, 28), 9, 11, K)
    mid = oracle.sparse_gg(*start, 17, 0.01, 1e-8)[:3]
    want = oracle.sparse_gg(*mid, 23, 0.01, 1e-8)[:3]
    got = run(gpu, (30, 28), K, start, [17, 23])
    assert_same_lists(got, want, K)
    one_call = oracle.sparse_gg(*start, 40, 0.01, 1e-8)[:3]
    assert not (np.array_equal(one_call[0], want[0]) and np.array_equal(one_call[1], want[1]) and
                np.array_equal(one_call[2], want[2]))


def test_sparse_overflow_is_reported(gpu):
    from mmsp_gb300 import inputs

    K = 3
    start = inputs.sparse_grains((24, 20), 9, 5, K)
    d = gpu.make_desc((24, 20), K, np.float64, "sparse_gg")
    with gpu.Stepper(d) as s:
        s.sparse_upload(*start)
        s.step(60)
        with pytest.raises(gpu.GpuError) as ei:
            s.sparse_download()
        assert ei.value.code == gpu.EOVERFLOW


def test_sparse_refusals(gpu):
    import torch

    from mmsp_gb300 import inputs

    K = 4
    d = gpu.make_desc((16, 16), K, np.float64, "sparse_gg")
    L = gpu.load()
    with gpu.Stepper(d) as s:
        c, i, v = inputs.sparse_grains((16, 16), 4, 1, K)
        bad = c.copy()
        bad[3, 3] = K + 1
        with pytest.raises(gpu.GpuError) as ei:
            s.sparse_upload(bad, i, v)
        assert ei.value.code == gpu.EINVAL
        s.sparse_upload(c, i, v)
        x = np.zeros(16 * 16 * K)
        assert L.mmsp_gpu_upload(s.h, x.ctypes.data, x.nbytes, gpu.CELL_MAJOR) == gpu.EUNSUPPORTED
        st = gpu.Stats()
        assert L.mmsp_gpu_reduce(s.h, ctypes.byref(st)) == gpu.EUNSUPPORTED
        assert L.mmsp_gpu_output(s.h, b"/tmp/never_written.dat", None) == gpu.EUNSUPPORTED
    a = torch.zeros(16 * 16 * 4, dtype=torch.float64, device="cuda")
    assert L.mmsp_gpu_step_noalloc(ctypes.byref(d), ctypes.c_void_p(a.data_ptr()), ctypes.c_void_p(a.data_ptr()), 1,
                                   None) == gpu.EUNSUPPORTED
    arr = (gpu.Desc * 1)(d)
    b = ctypes.c_void_p()
    assert L.mmsp_gpu_batch_create(ctypes.byref(b), 1, arr) == gpu.EUNSUPPORTED
    x = np.zeros(16 * 16 * K)
    assert L.mmsp_gpu_update(ctypes.byref(d), x.ctypes.data, x.nbytes, gpu.CELL_MAJOR, 1, None) == gpu.EUNSUPPORTED
