"""The batched form (mmsp_gpu_batch_*): many uneven grids advanced together.

Each grid of a batch must end exactly where a loop of single-grid update()
calls would: FP64 batches are compared bit for bit with the oracle, FP32
batches within 1e-5 of it.  The batch mixes grids the persistent kernel
takes (2D Cahn-Hilliard, rows a multiple of 32 cells) with grids it does not
(3D, odd rows, grain growth), which advance through their own kernels.
"""
import json
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL_F32 = 1e-5


def mixed_members(dtype):
    from mmsp_gb300 import inputs

    members = []
    # (shape, kappa, M, dt) of 2D CH grids the persistent kernel takes, incl. tiny row counts
    for k, (shape, kappa) in enumerate([((3, 32), 1.0), ((64, 64), 0.7), ((40, 96), 1.9), ((5, 160), 1.2),
                                        ((130, 512), 0.5), ((1, 64), 1.0), ((77, 224), 1.4)]):
        c0 = inputs.noisy_composition(shape, 0.45, 0.03, 900 + k)
        members.append(("ch", c0, dict(kappa=kappa, mobility=1.0, dt=0.004)))
    # grids that fall back to their own kernels
    members.append(("ch", inputs.noisy_composition((10, 12, 14), 0.4, 0.02, 950), dict(kappa=1.0, mobility=1.0, dt=0.002)))
    members.append(("ch", inputs.noisy_composition((20, 33), 0.5, 0.02, 951), dict(kappa=1.0, mobility=1.0, dt=0.004)))
    members.append(("ac", inputs.voronoi_grains((9, 10, 11), 6, 3, 952), dict(gamma=1.5, kappa=2.0, mobility=1.0, dt=0.05)))
    return members


def oracle_run(oracle, model, x, steps, p):
    if model == "ch":
        return oracle.ch_baseline(x, steps, p["kappa"], p["mobility"], p["dt"])
    return oracle.ac_baseline(x, steps, p["gamma"], p["kappa"], p["mobility"], p["dt"])


def make_batch(gpu, members, dtype):
    descs = []
    for model, x, p in members:
        fields = x.shape[-1] if model == "ac" else 1
        shape = x.shape[:-1] if model == "ac" else x.shape
        descs.append(gpu.make_desc(shape, fields, dtype, model, **p))
    b = gpu.Batch(descs)
    for i, (_, x, _) in enumerate(members):
        b.upload(i, x.astype(dtype))
    return b


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_batch_whole_transfers(gpu, dtype):
    """upload_all / download_all (every grid in one call, one synchronisation)
    move the same bytes as the per-grid calls, cell-major vector grids
    included, before and after steps."""
    members = mixed_members(dtype)
    b = make_batch(gpu, members, dtype)
    try:
        xs = [x.astype(dtype) for _, x, _ in members]
        assert all(np.array_equal(o, x) for o, x in zip(b.download_all(), xs))
        b.step(37)
        one = [b.download(i) for i in range(len(members))]
        allv = b.download_all()
        assert all(np.array_equal(o, a) for o, a in zip(one, allv))
        b.upload_all(xs)
        b.step(37)
        again = b.download_all()
        assert all(np.array_equal(o, a) for o, a in zip(one, again))
        with pytest.raises(ValueError):
            b.upload_all(xs[:-1])
    finally:
        b.close()


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_batch_matches_single_grid_updates(gpu, oracle, dtype):
    members = mixed_members(dtype)
    b = make_batch(gpu, members, dtype)
    info_before = b.info()
    b.step(1)
    b.step(200)      # graph replay from the odd pool, then a remainder
    b.step(3)
    info = b.info()
    assert info.instances == len(members) and info.persistent == 7 and info.fallback == 3
    assert info.rows_per_item > 0 and info.threads_per_block in (64, 128) and info.items > 0
    assert info_before.rows_per_item == 0
    for i, (model, x, p) in enumerate(members):
        got = b.download(i).astype(np.float64)
        want = oracle_run(oracle, model, x, 204, p)
        if dtype == np.float64:
            assert np.array_equal(got, want), (i, np.abs(got - want).max())
        else:
            assert np.abs(got - want).max() <= TOL_F32, (i, np.abs(got - want).max())
        if model == "ch":
            m, e = oracle.ch_mass_energy(want, p["kappa"])
            st = b.reduce(i)
            assert st.mass == pytest.approx(m, rel=1e-12 if dtype == np.float64 else 1e-6)
    b.close()


def test_batch_config_workload_sample(gpu, oracle):
    """A sample of the batched configuration's grids (sides 64..512, own kappa
    and mean), FP32 for 1000 steps, each within 1e-5 of the FP64 oracle."""
    from mmsp_gb300 import inputs

    work = inputs.batched_cahn_hilliard(count=12, seed=4)
    descs = [gpu.make_desc(c0.shape, 1, np.float32, "ch", kappa=k, mobility=1.0, dt=0.005) for c0, k in work]
    with gpu.Batch(descs) as b:
        for i, (c0, _) in enumerate(work):
            b.upload(i, c0.astype(np.float32))
        b.step(1000)
        for i in (0, 5, 11):
            c0, k = work[i]
            want = oracle.ch_baseline(c0, 1000, k, 1.0, 0.005)
            got = b.download(i).astype(np.float64)
            assert np.abs(got - want).max() <= TOL_F32
            assert np.abs(want - c0).max() > 1e-4


def test_autotune_cache(gpu, tmp_path, monkeypatch):
    from mmsp_gb300 import inputs

    path = tmp_path / "tune.json"
    monkeypatch.setenv("MMSP_GPU_TUNE_CACHE", str(path))
    work = inputs.batched_cahn_hilliard(count=5, seed=9)
    descs = [gpu.make_desc(c0.shape, 1, np.float32, "ch", kappa=k, dt=0.005) for c0, k in work]
    with gpu.Batch(descs) as b:
        b.tune(force=True)
        first = b.info()
        assert first.tuned_from_cache == 0 and first.tune_ms > 0
    saved = json.loads(path.read_text())
    assert any(v[:2] == [first.rows_per_item, first.threads_per_block] and v[2] in (0, first.temporal_depth)
               for v in saved.values())
    with gpu.Batch(descs) as b:
        b.tune()
        again = b.info()
        assert again.tuned_from_cache == 1
        assert (again.rows_per_item, again.threads_per_block) == (first.rows_per_item, first.threads_per_block)
        assert (again.temporal_depth, again.tile_rows, again.tile_cols) == \
            (first.temporal_depth, first.tile_rows, first.tile_cols)


def test_batch_rejects_mixed_dtypes(gpu):
    d1 = gpu.make_desc((32, 32), 1, np.float32, "ch")
    d2 = gpu.make_desc((32, 32), 1, np.float64, "ch")
    with pytest.raises(gpu.GpuError) as ei:
        gpu.Batch([d1, d2])
    assert ei.value.code == gpu.EINVAL


TILINGS = [(2, 0), (4, 0), (8, 0), (2, 1), (4, 1), (8, 1), (2, 2), (4, 2), (8, 2), (2, 3), (4, 3), (8, 3), (0, 0)]
TILE_SHAPES = [(64, 128), (96, 128), (128, 128), (128, 128)]


@pytest.mark.parametrize("ks,shape", TILINGS, ids=["depth%d-shape%d" % t for t in TILINGS])
def test_batch_temporal_blocking(gpu, oracle, monkeypatch, ks, shape):
    """The temporally blocked kernel on every region shape and depth: grids
    smaller than a tile (rows and columns wrap more than once), ragged edge
    tiles, non-unit spacing, both Cahn-Hilliard forms; step counts that are
    not multiples of the depth; within 1e-5 of the FP64 oracle, and within
    FP32 rounding of the per-step kernel."""
    from mmsp_gb300 import inputs

    monkeypatch.setenv("MMSP_GPU_BATCH_TILE", "%d,%d" % (ks, shape))
    grids = [((3, 32), "ch", {}), ((64, 64), "ch", {}), ((40, 96), "ch", dict(kappa=1.9)),
             ((130, 512), "ch", dict(kappa=0.5)), ((77, 224), "ch", dict(kappa=1.4)), ((200, 160), "ch", {}),
             ((33, 64), "ch", dict(dx=[1.1, 0.9]))]
    members = [(inputs.noisy_composition(sh, 0.45, 0.03, 700 + k), m, p) for k, (sh, m, p) in enumerate(grids)]
    descs = [gpu.make_desc(x.shape, 1, np.float32, m, mobility=1.0, dt=0.004, **p) for x, m, p in members]
    with gpu.Batch(descs) as b:
        for i, (x, _, _) in enumerate(members):
            b.upload(i, x.astype(np.float32))
        b.step(3)
        b.step(150)      # graph replay, then blocked launches and single steps
        info = b.info()
        assert info.temporal_depth == max(ks, 1)
        if ks:
            assert (info.tile_rows, info.tile_cols) == TILE_SHAPES[shape] and info.tiles > 0
        for i, (x, _, p) in enumerate(members):
            got = b.download(i).astype(np.float64)
            want = oracle.ch_baseline(x, 153, p.get("kappa", 1.0), 1.0, 0.004, dx=p.get("dx"))
            assert np.abs(got - want).max() <= TOL_F32, (i, np.abs(got - want).max())


def test_batch_tuner_considers_temporal_blocking(gpu, monkeypatch):
    """Tuning an all-FP32 2D batch scores the blocked kernel too; whatever
    wins is reported, and a bad override is refused."""
    from mmsp_gb300 import inputs

    monkeypatch.delenv("MMSP_GPU_TUNE_CACHE", raising=False)
    work = inputs.batched_cahn_hilliard(count=16, seed=5)
    descs = [gpu.make_desc(c0.shape, 1, np.float32, "ch", kappa=k, dt=0.005) for c0, k in work]
    with gpu.Batch(descs) as b:
        for i, (c0, _) in enumerate(work):
            b.upload(i, c0.astype(np.float32))
        b.tune(force=True)
        info = b.info()
        assert info.temporal_depth in (1, 2, 4, 8)
        assert (info.tile_rows > 0) == (info.temporal_depth > 1)
    monkeypatch.setenv("MMSP_GPU_BATCH_TILE", "3,0")
    with gpu.Batch(descs) as b:
        with pytest.raises(gpu.GpuError) as ei:
            b.tune(force=True)
        assert ei.value.code == gpu.EINVAL
