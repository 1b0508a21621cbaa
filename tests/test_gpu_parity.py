"""Parity of the device step with the reference, through the C ABI.

FP64 (plain form): bit-identical to the reference's own update() on the
golden fixtures, and to the CPU oracle on seeded random grids of ragged
shapes.  The shipped examples' pow(x,3) is evaluated on the device by a
compensated cube, so those forms are held to 1e-12 relative instead.
FP32 (precision form): max error against the FP64 oracle within 1e-5.
"""
import glob
import hashlib
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu

FIXTURES = sorted(f for f in glob.glob(os.path.join(GOLDEN, "*.npz"))
                  if not os.path.basename(f).startswith("sparse"))
SPARSE_FIXTURES = sorted(glob.glob(os.path.join(GOLDEN, "sparse*.npz")))
TOL_SHIPPED = 1e-12   # relative, forms with pow(x,3)
TOL_F32 = 1e-5        # absolute, FP32 against FP64 after the stated steps


def desc_for(native, model, params, shape, fields, dtype, dx=None, bc=None):
    p = [float(v) for v in params]
    kw = dict(dx=dx, bc=bc)
    if model == "ch_baseline":
        return native.make_desc(shape, 1, dtype, "ch", kappa=p[0], mobility=p[1], dt=p[2], **kw)
    if model == "ch_shipped":
        return native.make_desc(shape, 1, dtype, "ch_poly", r=p[0], u=p[1], kappa=p[2], mobility=p[3], dt=p[4], **kw)
    if model == "ac_scalar":
        return native.make_desc(shape, 1, dtype, "ac_poly", r=p[0], u=p[1], kappa=p[2], mobility=p[3], dt=p[4], **kw)
    if model == "ac_baseline":
        return native.make_desc(shape, fields, dtype, "ac", gamma=p[0], kappa=p[1], mobility=p[2], dt=p[3], **kw)
    if model == "graingrowth":
        return native.make_desc(shape, fields, dtype, "gg", dt=p[0], **kw)
    if model == "zener":
        return native.make_desc(shape, fields, dtype, "zener", dt=p[0], **kw)
    if model == "ostwald":
        return native.make_desc(shape, fields, dtype, "ostwald", dt=p[0], mobility=p[1], D=p[2], Calpha=p[3],
                                Cbeta=p[4], A=p[5], delta=p[6], epsilon=p[7], kappa=p[8], **kw)
    if model == "ch_convex":
        return native.make_desc(shape, fields, dtype, "ch_convex", dt=p[0], mobility=p[1], kappa=p[2], C0=p[3],
                                Ca=p[4], Cb=p[5], A=p[6], omega=p[7], tolerance=p[8], **kw)
    raise ValueError(model)


def run_gpu(native, desc, x, steps, layout=0):
    with native.Stepper(desc) as s:
        s.upload(x, layout)
        s.step(steps)
        return s.download(layout)


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a, "<f8").tobytes()).hexdigest()


@pytest.mark.parametrize("path", FIXTURES, ids=[os.path.basename(f)[:-4] for f in FIXTURES])
def test_fp64_matches_reference_fixture(gpu, path):
    z = np.load(path)
    model = str(z["model"])
    x = z["start"]
    vector = model in ("ac_baseline", "graingrowth", "zener", "ostwald", "ch_convex")
    shape = x.shape[:-1] if vector else x.shape
    fields = x.shape[-1] if vector else 1
    bc = z["bc"].tolist()
    d = desc_for(gpu, model, z["params"], shape, fields, np.float64, dx=z["dx"].tolist(), bc=bc)
    if any(b != [2, 2] for b in bc):
        with pytest.raises(gpu.GpuError) as ei:
            gpu.Stepper(d)
        assert ei.value.code == gpu.EUNSUPPORTED
        return
    got = run_gpu(gpu, d, x, int(z["steps"]))
    want = z["result"]
    if model in ("ch_baseline", "ac_baseline"):
        assert np.array_equal(got, want), "max |diff| %g" % np.abs(got - want).max()
    else:
        rel = np.abs(got - want).max() / np.abs(want).max()
        assert rel <= TOL_SHIPPED, rel


RAGGED = [(7,), (1, 9), (5, 7), (33, 45), (2, 3, 5), (1, 4, 6), (17, 33, 45), (40, 3, 70), (3, 50, 33)]


@pytest.mark.parametrize("shape", RAGGED, ids=["x".join(map(str, s)) for s in RAGGED])
def test_fp64_ch_ragged_shapes_bitwise(gpu, oracle, shape):
    from mmsp_gb300 import inputs

    c0 = inputs.noisy_composition(shape, 0.45, 0.03, 1000 + len(shape))
    d = gpu.make_desc(shape, 1, np.float64, "ch", kappa=1.0, mobility=1.0, dt=0.002)
    got = run_gpu(gpu, d, c0, 9)
    want = oracle.ch_baseline(c0, 9, 1.0, 1.0, 0.002)
    assert np.array_equal(got, want), "max |diff| %g" % np.abs(got - want).max()


@pytest.mark.parametrize("shape,fields", [((6,), 2), ((9, 11), 3), ((5, 6, 7), 8), ((20, 9, 37), 5), ((2, 40, 3), 16)])
def test_fp64_ac_ragged_shapes_bitwise(gpu, oracle, shape, fields):
    from mmsp_gb300 import inputs

    e0 = inputs.voronoi_grains(shape, 6, fields, 77)
    d = gpu.make_desc(shape, fields, np.float64, "ac", gamma=1.5, kappa=2.0, mobility=1.0, dt=0.05)
    got = run_gpu(gpu, d, e0, 7)
    want = oracle.ac_baseline(e0, 7, 1.5, 2.0, 1.0, 0.05)
    assert np.array_equal(got, want), "max |diff| %g" % np.abs(got - want).max()


def test_fp64_nonunit_spacing_and_parameters(gpu, oracle):
    from mmsp_gb300 import inputs

    c0 = inputs.noisy_composition((12, 14, 16), 0.5, 0.02, 9)
    d = gpu.make_desc(c0.shape, 1, np.float64, "ch", kappa=0.7, mobility=1.3, dt=0.0005, dx=[0.9, 1.1, 1.7])
    got = run_gpu(gpu, d, c0, 11)
    want = oracle.ch_baseline(c0, 11, 0.7, 1.3, 0.0005, dx=[0.9, 1.1, 1.7])
    assert np.array_equal(got, want)


def test_graph_replay_long_run_bitwise(gpu, oracle):
    """Runs long enough for CUDA-graph replay (64-step graphs), started from
    both ping-pong buffers, match a plain run."""
    from mmsp_gb300 import inputs

    c0 = inputs.noisy_composition((16, 20, 24), 0.4, 0.02, 12)
    d = gpu.make_desc(c0.shape, 1, np.float64, "ch", dt=0.002)
    with gpu.Stepper(d) as s:
        s.upload(c0)
        s.step(1)
        s.step(300)    # odd buffer start: one plain step, graphs, remainder
        s.step(129)
        got = s.download()
    want = oracle.ch_baseline(c0, 430, 1.0, 1.0, 0.002)
    assert np.array_equal(got, want)


def test_layouts_and_transfers(gpu, oracle):
    from mmsp_gb300 import inputs

    e0 = inputs.voronoi_grains((8, 9, 10), 5, 4, 3)
    d = gpu.make_desc(e0.shape[:-1], 4, np.float64, "ac", gamma=1.5, kappa=2.0, dt=0.05)
    a = run_gpu(gpu, d, e0, 3, layout=gpu.CELL_MAJOR)
    b = run_gpu(gpu, d, np.moveaxis(e0, -1, 0).copy(), 3, layout=gpu.FIELD_MAJOR)
    assert np.array_equal(a, np.moveaxis(b, 0, -1))
    with gpu.Stepper(d) as s:
        with pytest.raises(ValueError):
            s.upload(e0[:-1])
        import ctypes
        buf = np.zeros(10)
        rc = gpu.load().mmsp_gpu_upload(s.h, buf.ctypes.data, buf.nbytes, 0)
        assert rc == gpu.EINVAL
        assert b"bytes" in gpu.load().mmsp_gpu_last_error(s.h)


def test_one_shot_update_matches_handle(gpu, oracle):
    from mmsp_gb300 import inputs

    c0 = inputs.noisy_composition((30, 31), 0.5, 0.01, 4)
    d = gpu.make_desc(c0.shape, 1, np.float64, "ch", dt=0.005)
    out, st = gpu.update(c0, 150, d)
    want = oracle.ch_baseline(c0, 150, 1.0, 1.0, 0.005)
    assert np.array_equal(out, want)
    m, e = oracle.ch_mass_energy(want, 1.0)
    assert st.mass == pytest.approx(m, rel=1e-12)
    assert st.energy == pytest.approx(e, rel=1e-12)
    assert st.steps == 150 and st.gpu_ms > 0


@pytest.mark.parametrize("model", ["ch", "ac"])
def test_reductions_match_oracle(gpu, oracle, model):
    from mmsp_gb300 import inputs

    if model == "ch":
        x = inputs.noisy_composition((21, 34, 19), 0.4, 0.05, 21)
        d = gpu.make_desc(x.shape, 1, np.float64, "ch", kappa=0.8, dx=[0.5, 1.0, 2.0])
        m, e = oracle.ch_mass_energy(x, 0.8, dx=[0.5, 1.0, 2.0])
    else:
        x = inputs.voronoi_grains((14, 15, 16), 9, 5, 22) * 0.9 + 0.01
        d = gpu.make_desc(x.shape[:-1], 5, np.float64, "ac", gamma=1.5, kappa=2.0)
        ms, e = oracle.ac_mass_energy(x, 1.5, 2.0)
        m = float(np.sum(ms))
    with gpu.Stepper(d) as s:
        s.upload(x)
        st = s.reduce()
    assert st.mass == pytest.approx(m, rel=1e-12)
    assert st.energy == pytest.approx(e, rel=1e-12)


def test_fp32_precision_form_small(gpu, oracle):
    from mmsp_gb300 import inputs

    c0 = inputs.noisy_composition((32, 40, 48), 0.4, 0.02, 31)
    d = gpu.make_desc(c0.shape, 1, np.float32, "ch", dt=0.002)
    got = run_gpu(gpu, d, c0.astype(np.float32), 200).astype(np.float64)
    want = oracle.ch_baseline(c0, 200, 1.0, 1.0, 0.002)
    assert np.abs(got - want).max() <= TOL_F32
    e0 = inputs.voronoi_grains((20, 24, 28), 15, 8, 32)
    d = gpu.make_desc(e0.shape[:-1], 8, np.float32, "ac", gamma=1.5, kappa=2.0, dt=0.05)
    got = run_gpu(gpu, d, e0.astype(np.float32), 50).astype(np.float64)
    want = oracle.ac_baseline(e0, 50, 1.5, 2.0, 1.0, 0.05)
    assert np.abs(got - want).max() <= TOL_F32


def test_errors_are_codes_not_crashes(gpu):
    d = gpu.make_desc((8, 8), 1, np.float64, "ch", bc=[[1, 1], [2, 2]])
    with pytest.raises(gpu.GpuError) as ei:
        gpu.Stepper(d)
    assert ei.value.code == gpu.EUNSUPPORTED
    d = gpu.make_desc((8, 8), 2, np.float64, "ch")
    with pytest.raises(gpu.GpuError) as ei:
        gpu.Stepper(d)
    assert ei.value.code == gpu.EINVAL
    d = gpu.make_desc((8, 8), 1, np.float64, "ch")
    with gpu.Stepper(d) as s:
        assert gpu.load().mmsp_gpu_step(s.h, -1) == gpu.EINVAL
        s.step(0)


# ---------------------------------------------------------------- full size

FULL = json.load(open(os.path.join(GOLDEN, "full_size.json")))


def test_full_2d_256_fp64_matches_reference_checksum(gpu):
    from mmsp_gb300 import inputs

    m = FULL["ch2d_256_2000"]
    c0 = inputs.noisy_composition(tuple(m["shape"]), m["mean"], m["amplitude"], m["seed"])
    d = gpu.make_desc(c0.shape, 1, np.float64, "ch", kappa=m["kappa"], mobility=m["M"], dt=m["dt"])
    out, st = gpu.update(c0, m["steps"], d)
    assert sha(out) == m["sha256"]
    assert st.mass == pytest.approx(m["mass"], rel=1e-12)
    assert st.energy == pytest.approx(m["energy"], rel=1e-12)


def test_full_3d_256_fp64_checksum_and_fp32_error(gpu):
    """256^3 Cahn-Hilliard, 1000 steps: FP64 bit-identical to the oracle
    (checksum); FP32 max error <= 1e-5 against that FP64 state; mass drift."""
    from mmsp_gb300 import inputs

    m = FULL["ch3d_256_1000"]
    c0 = inputs.noisy_composition(tuple(m["shape"]), m["mean"], m["amplitude"], m["seed"])
    d64 = gpu.make_desc(c0.shape, 1, np.float64, "ch", kappa=m["kappa"], mobility=m["M"], dt=m["dt"])
    out64, st64 = gpu.update(c0, m["steps"], d64)
    assert sha(out64) == m["sha256"]
    assert st64.energy == pytest.approx(m["energy"], rel=1e-12)
    d32 = gpu.make_desc(c0.shape, 1, np.float32, "ch", kappa=m["kappa"], mobility=m["M"], dt=m["dt"])
    out32, st32 = gpu.update(c0.astype(np.float32), m["steps"], d32)
    err = np.abs(out32.astype(np.float64) - out64)
    assert err.max() <= TOL_F32, err.max()
    assert abs(st32.mass - m["mass0"]) / m["mass0"] < 1e-6


CONTRACT_CASES = [
    ("ch", (9, 11), dict(kappa=1.0, mobility=1.0, dt=0.005)),
    ("ch", (40, 3, 70), dict(kappa=1.0, mobility=1.0, dt=0.002)),
    ("ch", (17, 33, 45), dict(kappa=0.7, mobility=1.3, dt=0.0005, dx=[0.9, 1.1, 1.7])),
    ("ch", (1, 4, 6), dict(kappa=1.0, mobility=1.0, dt=0.002)),
    ("ch_poly", (24, 20, 36), dict(r=1.0, u=1.0, kappa=1.0, mobility=1.0, dt=0.005)),
    ("ch_poly", (33, 45), dict(r=0.8, u=1.2, kappa=1.0, mobility=0.5, dt=0.01, dx=[1.2, 0.8])),
]


@pytest.mark.parametrize("model,shape,prm", CONTRACT_CASES,
                         ids=["%s-%s" % (m, "x".join(map(str, s))) for m, s, _ in CONTRACT_CASES])
def test_fp64_contracted_against_oracle(gpu, oracle, model, shape, prm):
    """FP64 with MMSP_GPU_FLAG_CONTRACT (fused multiply-adds, regrouped
    Laplacian): within TOL_SHIPPED relative of the oracle, which is
    bit-identical to the reference; the flag-free run stays bitwise."""
    from mmsp_gb300 import inputs

    c0 = inputs.noisy_composition(shape, 0.45 if model == "ch" else 0.0, 0.03 if model == "ch" else 0.1,
                                  300 + len(shape))
    steps = 150    # past the graph threshold
    d = gpu.make_desc(shape, 1, np.float64, model, contract=True, **prm)
    got = run_gpu(gpu, d, c0, steps)
    dx = prm.get("dx")
    if model == "ch":
        want = oracle.ch_baseline(c0, steps, prm["kappa"], prm["mobility"], prm["dt"], dx=dx)
    else:
        want = oracle.ch_shipped(c0, steps, prm["r"], prm["u"], prm["kappa"], prm["mobility"], prm["dt"], dx=dx)
    assert np.isfinite(want).all()    # a stable case
    rel = np.abs(got - want).max() / np.abs(want).max()
    assert rel <= TOL_SHIPPED, rel
    if model == "ch":
        exact = run_gpu(gpu, gpu.make_desc(shape, 1, np.float64, model, **prm), c0, steps)
        assert np.array_equal(exact, want)


def test_full_2d_256_fp64_contracted(gpu):
    """2D 256^2 x 2000 steps: the contracted FP64 form within 1e-12 relative
    of the reference (whose result the exact form reproduces bit for bit:
    checksum), and the reference's own sampled values."""
    from mmsp_gb300 import inputs

    m = FULL["ch2d_256_2000"]
    c0 = inputs.noisy_composition(tuple(m["shape"]), m["mean"], m["amplitude"], m["seed"])
    kw = dict(kappa=m["kappa"], mobility=m["M"], dt=m["dt"])
    exact, _ = gpu.update(c0, m["steps"], gpu.make_desc(c0.shape, 1, np.float64, "ch", **kw))
    assert sha(exact) == m["sha256"]
    fast, st = gpu.update(c0, m["steps"], gpu.make_desc(c0.shape, 1, np.float64, "ch", contract=True, **kw))
    rel = np.abs(fast - exact).max() / np.abs(exact).max()
    assert rel <= TOL_SHIPPED, rel
    sample = fast.ravel()[::m["sample_stride"]][:len(m["sample"])]
    assert np.abs(sample - np.array(m["sample"])).max() <= TOL_SHIPPED * np.abs(exact).max()
    assert st.mass == pytest.approx(m["mass"], rel=1e-12)
    assert st.energy == pytest.approx(m["energy"], rel=1e-12)


def test_full_3d_256_fp64_contracted(gpu):
    """3D 256^3 x 1000 steps: the contracted FP64 form within 1e-12 relative
    of the exact form, which matches the oracle's checksum."""
    from mmsp_gb300 import inputs

    m = FULL["ch3d_256_1000"]
    c0 = inputs.noisy_composition(tuple(m["shape"]), m["mean"], m["amplitude"], m["seed"])
    kw = dict(kappa=m["kappa"], mobility=m["M"], dt=m["dt"])
    exact, _ = gpu.update(c0, m["steps"], gpu.make_desc(c0.shape, 1, np.float64, "ch", **kw))
    assert sha(exact) == m["sha256"]
    fast, st = gpu.update(c0, m["steps"], gpu.make_desc(c0.shape, 1, np.float64, "ch", contract=True, **kw))
    rel = np.abs(fast - exact).max() / np.abs(exact).max()
    assert rel <= TOL_SHIPPED, rel
    assert st.mass == pytest.approx(m["mass"], rel=1e-12)
    assert st.energy == pytest.approx(m["energy"], rel=1e-12)


def test_full_3d_ac_128_n8(gpu):
    """128^3 x 8 grain growth (Voronoi, 200 seeds): dt=0.05 FP64 bit-identical
    to the oracle after 500 steps, FP32 within 1e-5; dt=0.1 diverges at the
    same step as in the oracle."""
    from mmsp_gb300 import inputs

    m = FULL["ac3d_128_n8_dt0.05_500"]
    e0 = inputs.voronoi_grains(tuple(m["shape"]), m["points"], m["fields"], m["seed"])
    d64 = gpu.make_desc(e0.shape[:-1], 8, np.float64, "ac", gamma=m["gamma"], kappa=m["kappa"],
                        mobility=m["L"], dt=m["dt"])
    out64, st = gpu.update(e0, m["steps"], d64)
    assert sha(out64) == m["sha256"]
    d32 = gpu.make_desc(e0.shape[:-1], 8, np.float32, "ac", gamma=m["gamma"], kappa=m["kappa"],
                        mobility=m["L"], dt=m["dt"])
    out32, _ = gpu.update(e0.astype(np.float32), m["steps"], d32)
    assert np.abs(out32.astype(np.float64) - out64).max() <= TOL_F32
    div = FULL["ac3d_128_n8_dt0.1_divergence"]
    d = gpu.make_desc(e0.shape[:-1], 8, np.float64, "ac", gamma=1.5, kappa=2.0, dt=0.1)
    first_bad = None
    with gpu.Stepper(d) as s:
        s.upload(e0)
        for k in range(1, 41):
            s.step(1)
            x = s.download()
            if not np.isfinite(x).all():
                first_bad = k
                break
            assert np.abs(x).max() == pytest.approx(div["max_abs_per_step"][k - 1], rel=1e-12)
    assert first_bad == div["first_nonfinite_step"]


# FP32 3D grids with rows of 32 to 512 cells and at least 12 rows per plane
# take the register-streaming kernel; cover its strip/segment edge cases
# (partial last strip, periodic Y wrap at both ends, the smallest allowed Y,
# a single warp per row, few X planes) and its row forms: compile-time rows
# of 32..512 in powers of two; runtime rows with bulk copies (multiples of 4
# cells), with per-thread 8-byte copies (even rows), odd rows (a padded
# shared row whose extra cell is the row's cell 0); a last warp that the row
# fills only in part (the warp-end mu exchange and the periodic wrap from its
# last real lane), down to lane 0 alone.
STREAM_SHAPES = [(16, 24, 64), (20, 13, 32), (5, 12, 96), (3, 40, 256), (33, 17, 128), (1, 16, 32),
                 (7, 13, 243), (4, 12, 33), (6, 20, 50), (3, 14, 198), (2, 12, 300), (2, 12, 301), (3, 17, 190),
                 (4, 12, 36), (3, 12, 63), (2, 13, 65), (3, 22, 242)]


@pytest.mark.parametrize("shape", STREAM_SHAPES, ids=["x".join(map(str, s)) for s in STREAM_SHAPES])
@pytest.mark.parametrize("model", ["ch", "ch_poly"])
def test_fp32_stream_kernel_against_fp64_oracle(gpu, oracle, shape, model):
    from mmsp_gb300 import inputs

    steps = 60
    if model == "ch":
        c0 = inputs.noisy_composition(shape, 0.4, 0.05, 500 + shape[0])
        d = gpu.make_desc(shape, 1, np.float32, "ch", kappa=0.9, mobility=1.1, dt=0.002, dx=[1.0, 0.9, 1.1])
        want = oracle.ch_baseline(c0, steps, 0.9, 1.1, 0.002, dx=[1.0, 0.9, 1.1])
    else:
        c0 = inputs.noisy_composition(shape, 0.0, 0.5, 600 + shape[0])
        d = gpu.make_desc(shape, 1, np.float32, "ch_poly", r=1.0, u=1.0, kappa=1.0, mobility=1.0, dt=0.002)
        want = oracle.ch_shipped(c0, steps, 1.0, 1.0, 1.0, 1.0, 0.002)
    got = run_gpu(gpu, d, c0.astype(np.float32), steps).astype(np.float64)
    assert np.abs(got - want).max() <= TOL_F32 * max(1.0, np.abs(want).max())
    # the state must move, or the comparison pins nothing
    assert np.abs(want - c0).max() > 1e-4


def test_handles_of_one_kernel_with_different_shared_memory(gpu, oracle):
    """Two live handles that use the same kernel with different shared-memory
    needs (16 and 3 fields): planning the second must not break the first."""
    from mmsp_gb300 import inputs

    big = inputs.voronoi_grains((10, 11, 12), 7, 16, 61)
    small = inputs.voronoi_grains((10, 11, 12), 7, 3, 62)
    d_big = gpu.make_desc(big.shape[:-1], 16, np.float64, "ac", gamma=1.5, kappa=2.0, dt=0.05)
    d_small = gpu.make_desc(small.shape[:-1], 3, np.float64, "ac", gamma=1.5, kappa=2.0, dt=0.05)
    with gpu.Stepper(d_big) as a:
        a.upload(big)
        with gpu.Stepper(d_small) as b:
            b.upload(small)
            a.step(4)
            b.step(4)
            got_a, got_b = a.download(), b.download()
    assert np.array_equal(got_a, oracle.ac_baseline(big, 4, 1.5, 2.0, 1.0, 0.05))
    assert np.array_equal(got_b, oracle.ac_baseline(small, 4, 1.5, 2.0, 1.0, 0.05))


# FP32 3D Allen-Cahn grids with rows of up to 256 cells take the streaming
# kernel: all fields staged per plane by bulk copies where rows are 16-byte
# multiples (Z % 4 == 0), by per-thread 4-byte asynchronous copies otherwise.
# Partial strips, Y wrap at both ends, strips of 4, 2 and 1 rows (Y = 3..5),
# 1 to 16 fields, each model.
AC_STREAM = [((6, 13, 32), 3, "ac"), ((9, 7, 64), 8, "ac"), ((5, 20, 128), 16, "ac"), ((3, 10, 256), 2, "gg"),
             ((7, 9, 32), 1, "ac_poly"), ((12, 6, 64), 5, "gg"),
             ((8, 11, 37), 4, "ac"), ((5, 9, 100), 8, "ac"), ((4, 6, 255), 3, "gg"), ((10, 3, 1), 2, "ac"),
             ((6, 4, 3), 5, "ac_poly"), ((9, 5, 200), 6, "gg"), ((3, 17, 61), 16, "ac"), ((2, 7, 12), 2, "ac"),
             ((7, 9, 150), 12, "ac"), ((6, 10, 200), 6, "gg"),   # 4-slot rings (per-thread / bulk copies)
             ((8, 12, 64), 3, "zener"), ((5, 9, 45), 6, "zener")]


@pytest.mark.parametrize("shape,fields,model", AC_STREAM, ids=["%s-%d-%s" % ("x".join(map(str, s)), f, m) for s, f, m in AC_STREAM])
def test_fp32_ac_stream_kernel_against_fp64_oracle(gpu, oracle, shape, fields, model):
    from mmsp_gb300 import inputs

    steps = 40
    if model == "ac_poly":
        x = inputs.noisy_composition(shape, 0.0, 0.8, 700 + shape[0])
        d = gpu.make_desc(shape, 1, np.float32, "ac_poly", r=1.0, u=1.0, kappa=1.0, mobility=1.0, dt=0.01)
        want = oracle.ac_scalar_shipped(x, steps, 1.0, 1.0, 1.0, 1.0, 0.01)
    else:
        x = inputs.voronoi_grains(shape, 7, fields, 710 + shape[0]) * 0.8 + 0.05
        if model == "ac":
            d = gpu.make_desc(shape, fields, np.float32, "ac", gamma=1.5, kappa=2.0, mobility=1.0, dt=0.05,
                              dx=[1.0, 1.1, 0.9])
            want = oracle.ac_baseline(x, steps, 1.5, 2.0, 1.0, 0.05, dx=[1.0, 1.1, 0.9])
        elif model == "gg":
            d = gpu.make_desc(shape, fields, np.float32, "gg", dt=0.01)
            want = oracle.ac_graingrowth(x, steps, 0.01)
        else:
            d = gpu.make_desc(shape, fields, np.float32, "zener", dt=0.01)
            want = oracle.ac_zener(x, steps, 0.01)
    got = run_gpu(gpu, d, x.astype(np.float32), steps).astype(np.float64)
    assert np.abs(got - want).max() <= TOL_F32
    assert np.abs(want - x).max() > 1e-3


# Rows of 64, 128 and 256 cells take the warp-per-row form of the streaming
# kernel; MMSP_GPU_AC3_SHAPE fixes its strip rows, ring depth, warps per row
# and (fourth value 1) the producer/consumer form ("0,0": the per-cell
# form): 2- and 4-row strips (Y = 4, 5 fall back to 2 rows), rings of 3 to 6
# slots, 1, 2 and 4 warps per row (uneven field shares, a warp with none),
# partial strips and Y wraps, a single X plane, every model.
AC_VEC = [("2,3", (7, 9, 64), 3, "ac"), ("2,5", (5, 11, 128), 8, "gg"), ("4,6", (6, 13, 128), 4, "zener"),
          ("4,4", (4, 6, 256), 6, "ac"), ("0,0", (5, 9, 128), 8, "ac"), ("4,3", (3, 5, 128), 1, "ac_poly"),
          ("4,4", (9, 4, 64), 16, "gg"), ("2,4", (4, 14, 256), 12, "ac"), ("4,4,2", (6, 9, 128), 8, "ac"),
          ("2,3,4", (5, 7, 64), 5, "gg"), ("4,4,4", (4, 6, 128), 3, "zener"), ("4,3,2", (5, 10, 256), 7, "ac"),
          ("4,4,2,1", (6, 9, 128), 8, "ac"), ("4,3,1,1", (5, 7, 64), 5, "gg"), ("2,4,2,1", (4, 14, 256), 12, "ac"),
          ("4,5,4,1", (4, 6, 128), 3, "zener"), ("4,3,1,1", (1, 7, 128), 2, "ac")]


@pytest.mark.parametrize("tile,shape,fields,model", AC_VEC,
                         ids=["%s-%s-%d-%s" % (t, "x".join(map(str, s)), f, m) for t, s, f, m in AC_VEC])
def test_fp32_ac_row_warp_kernel_shapes(gpu, oracle, monkeypatch, tile, shape, fields, model):
    monkeypatch.setenv("MMSP_GPU_AC3_SHAPE", tile)
    test_fp32_ac_stream_kernel_against_fp64_oracle(gpu, oracle, shape, fields, model)


# 2D FP32 Cahn-Hilliard handles step in blocks of 4 steps per launch of the
# temporally blocked kernel (64 x 128 regions), the leftover steps of a call
# one per launch: rows of a multiple of 4 cells (16-byte copies) and not,
# grids smaller than a region (wraps inside it), ragged edge tiles, a single
# row, non-unit spacing, both models; graph replays, a start from the second
# buffer at an even launch count (no graph), and calls of multiples of 4
# steps equal one call bit for bit.
TB_HANDLE = [(50, 77), (64, 64), (130, 512), (3, 33), (200, 1024), (97, 100), (1, 40), (33, 130)]


@pytest.mark.parametrize("shape", TB_HANDLE, ids=["x".join(map(str, s)) for s in TB_HANDLE])
def test_fp32_2d_blocked_handle(gpu, oracle, shape):
    from mmsp_gb300 import inputs

    poly = shape[0] % 2 == 1
    x = inputs.noisy_composition(shape, 0.0 if poly else 0.45, 0.5 if poly else 0.05, 900 + shape[0])
    if poly:
        d = gpu.make_desc(shape, 1, np.float32, "ch_poly", r=1.0, u=1.0, kappa=1.0, mobility=1.0, dt=0.004)
    else:
        d = gpu.make_desc(shape, 1, np.float32, "ch", kappa=0.8, mobility=1.2, dt=0.003, dx=[1.0, 1.1])
    x32 = x.astype(np.float32)
    with gpu.Stepper(d) as s:
        s.upload(x32)
        for n in (8, 16, 13):          # 9 blocked launches, then one single step
            s.step(n)
        a = s.download()
        s.upload(x32)
        s.step(24)
        s.step(13)
        b = s.download()
        s.upload(x32)
        s.step(3)                      # three single steps: buffer 1 at an even launch count
        s.step(300)                    # 75 blocked launches without the graph
        c = s.download()
        s.upload(x32)
        s.step(300)                    # graph replays
        s.step(3)
        e = s.download()
    assert np.array_equal(a, b)
    if poly:
        want37 = oracle.ch_shipped(x, 37, 1.0, 1.0, 1.0, 1.0, 0.004)
        want303 = oracle.ch_shipped(x, 303, 1.0, 1.0, 1.0, 1.0, 0.004)
    else:
        want37 = oracle.ch_baseline(x, 37, 0.8, 1.2, 0.003, dx=[1.0, 1.1])
        want303 = oracle.ch_baseline(x, 303, 0.8, 1.2, 0.003, dx=[1.0, 1.1])
    scale = max(1.0, np.abs(want303).max())
    assert np.abs(a.astype(np.float64) - want37).max() <= TOL_F32 * scale
    assert np.abs(c.astype(np.float64) - want303).max() <= TOL_F32 * scale
    assert np.abs(e.astype(np.float64) - want303).max() <= TOL_F32 * scale
    assert np.abs(want303 - x).max() > 1e-3


# FP32 Cahn-Hilliard grids that the streaming kernel does not take use the row
# kernel (any row length, plain loads): 2D rows up to 1024 cells, 3D grids
# with fewer than 12 rows per plane or rows shorter than 32 cells.
ROWS = [(50, 77), (7, 1024), (3, 33), (1, 100), (20, 9, 45), (6, 3, 70), (11, 1, 33), (5, 40, 500), (9, 30, 1)]


@pytest.mark.parametrize("shape", ROWS, ids=["x".join(map(str, s)) for s in ROWS])
def test_fp32_rows_kernel_against_fp64_oracle(gpu, oracle, shape):
    from mmsp_gb300 import inputs

    steps = 50
    dt = 0.004 if len(shape) == 2 else 0.002
    c0 = inputs.noisy_composition(shape, 0.45, 0.05, 800 + sum(shape))
    d = gpu.make_desc(shape, 1, np.float32, "ch", kappa=1.2, mobility=0.9, dt=dt, dx=[1.0, 1.1, 0.95][: len(shape)])
    got = run_gpu(gpu, d, c0.astype(np.float32), steps).astype(np.float64)
    want = oracle.ch_baseline(c0, steps, 1.2, 0.9, dt, dx=[1.0, 1.1, 0.95][: len(shape)])
    assert np.abs(got - want).max() <= TOL_F32
    assert np.abs(want - c0).max() > 1e-4


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
@pytest.mark.parametrize("shape", [(40, 36), (20, 16, 64), (9, 11, 37)])
def test_zener_particles_do_not_move(gpu, oracle, dtype, shape):
    """Zener pinning: field 0 (the particles) is copied bit for bit every step
    while the grains (fields 1, 2) evolve around it (zener.cpp:134)."""
    from mmsp_gb300 import inputs

    x = inputs.zener_particles(shape, 12, 40 + len(shape)).astype(dtype)
    d = gpu.make_desc(shape, 3, dtype, "zener", dt=0.01)
    got = run_gpu(gpu, d, x, 60)
    assert np.array_equal(got[..., 0], x[..., 0])
    want = oracle.ac_zener(x.astype(np.float64), 60, 0.01)
    tol = TOL_SHIPPED if dtype == np.float64 else TOL_F32
    assert np.abs(got.astype(np.float64) - want).max() <= tol * max(1.0, np.abs(want).max())
    assert np.abs(want[..., 1:] - x[..., 1:]).max() > 1e-3


OSTWALD = [((96, 64), 2), ((20, 16, 12), 3), ((7, 9, 13), 4), ((200,), 2)]


@pytest.mark.parametrize("shape,fields", OSTWALD, ids=["%s-%d" % ("x".join(map(str, s)), f) for s, f in OSTWALD])
def test_ostwald_fp32_and_fp64_against_oracle(gpu, oracle, shape, fields):
    """Ostwald ripening (two kernels per step): FP64 within the shipped-form
    tolerance of the oracle (pow(x,3) by the compensated cube), FP32 within
    the precision-form tolerance."""
    from mmsp_gb300 import inputs

    x = inputs.ostwald_start(shape, fields, 50 + len(shape))
    steps = 100
    want = oracle.ostwald(x, steps)
    d64 = gpu.make_desc(shape, fields, np.float64, "ostwald")
    got64 = run_gpu(gpu, d64, x, steps)
    assert np.abs(got64 - want).max() <= TOL_SHIPPED * np.abs(want).max()
    d32 = gpu.make_desc(shape, fields, np.float32, "ostwald")
    got32 = run_gpu(gpu, d32, x.astype(np.float32), steps).astype(np.float64)
    assert np.abs(got32 - want).max() <= TOL_F32
    assert np.abs(want - x).max() > 1e-3
    # the composition is conserved: its sum moves by rounding only
    assert abs(want[..., 0].sum() - x[..., 0].sum()) < 1e-9 * x[..., 0].size
    assert abs(got64[..., 0].sum() - x[..., 0].sum()) < 1e-9 * x[..., 0].size


# FP32 3D grids with rows of 32, 64 or 128 cells and 2..4 fields take the
# one-kernel streaming step (strips of 16 rows, 8 for 128-cell rows): ragged
# last strips, short plane runs, non-unit spacing.
OST_STREAM = [((6, 21, 32), 2, None), ((5, 40, 64), 3, None), ((4, 13, 128), 4, None), ((9, 20, 64), 2, None),
              ((7, 24, 64), 2, (1.0, 0.8, 1.25))]


@pytest.mark.parametrize("shape,fields,dx", OST_STREAM,
                         ids=["%s-%d-%s" % ("x".join(map(str, s)), f, "unit" if h is None else "dx")
                              for s, f, h in OST_STREAM])
def test_ostwald_stream_kernel_against_oracle(gpu, oracle, shape, fields, dx):
    """The one-kernel FP32 Ostwald step within the precision-form tolerance
    of the FP64 oracle, and close to the two-kernel FP32 path (selected by
    MMSP_GPU_OST_TWO_KERNELS at planning)."""
    from mmsp_gb300 import inputs

    x = inputs.ostwald_start(shape, fields, 70 + fields)
    steps = 120
    want = oracle.ostwald(x, steps, dx=dx)
    d32 = gpu.make_desc(shape, fields, np.float32, "ostwald", dx=dx)
    got = run_gpu(gpu, d32, x.astype(np.float32), steps).astype(np.float64)
    assert np.abs(got - want).max() <= TOL_F32
    assert np.abs(want - x).max() > 1e-3
    os.environ["MMSP_GPU_OST_TWO_KERNELS"] = "1"
    try:
        two = run_gpu(gpu, d32, x.astype(np.float32), steps).astype(np.float64)
    finally:
        del os.environ["MMSP_GPU_OST_TWO_KERNELS"]
    assert np.abs(two - want).max() <= TOL_F32
    assert np.abs(got - two).max() <= 2e-6


def ostwald_energy(x, dx, Ca=0.05, Cb=0.95, A=2.0, delta=1.0, eps=3.0, kappa=2.0):
    """The free energy the library reports for the Ostwald model, in numpy:
    -A/2 (C-Cm)^2 + B/4 (C-Cm)^4 + Da/4 (C-Ca)^4 + Db/4 (C-Cb)^4 - g/2 (C-Ca)^2 sum e^2
    + delta/4 sum e^4 + eps/2 sum_{i<j} e_i^2 e_j^2 + kappa/2 sum |grad|^2 (central differences)."""
    Cm = 0.5 * (Ca + Cb)
    B = A / (Cb - Cm) ** 2
    g = 2.0 / (Cb - Ca) ** 2
    Da = Db = g / delta ** 2
    C = x[..., 0]
    e = x[..., 1:]
    e2 = e * e
    sq = e2.sum(-1)
    pair = 0.5 * (sq * sq - (e2 * e2).sum(-1))
    f = (-0.5 * A * (C - Cm) ** 2 + 0.25 * B * (C - Cm) ** 4 + 0.25 * Da * (C - Ca) ** 4
         + 0.25 * Db * (C - Cb) ** 4 - 0.5 * g * (C - Ca) ** 2 * sq + 0.25 * delta * (e2 * e2).sum(-1)
         + 0.5 * eps * pair)
    grad = np.zeros_like(C)
    for j in range(x.shape[-1]):
        for a in range(C.ndim):
            gi = (np.roll(x[..., j], -1, a) - np.roll(x[..., j], 1, a)) / (2.0 * dx[a])
            grad += gi * gi
    dV = float(np.prod(dx))
    return dV * x.sum(), dV * (f + 0.5 * kappa * grad).sum()


def test_ostwald_reductions(gpu):
    from mmsp_gb300 import inputs

    shape, dx = (24, 20, 16), [1.0, 0.9, 1.1]
    x = inputs.ostwald_start(shape, 3, 61)
    d = gpu.make_desc(shape, 3, np.float64, "ostwald", dx=dx)
    with gpu.Stepper(d) as s:
        s.upload(x)
        s.step(20)
        st = s.reduce()
        y = s.download()
    m, e = ostwald_energy(y, dx)
    assert abs(st.mass - m) <= 1e-12 * abs(m)
    assert abs(st.energy - e) <= 1e-11 * abs(e)


# Stochastic forms: the shipped polynomial models plus thermal noise from a
# counter-based stream (the oracle draws the same deviates).
# (name, model, shape, dtype, params, steps)
KT, DT, DV = 0.01, 0.01, 1.0
SIGMA_AB = float(np.sqrt(2.0 * KT / (DT * DV)))      # model_A.cpp:99, model_B.cpp:100: sqrt(2 kT/(dt dV))
SIGMA_SPIN = float(np.sqrt(0.05 * DT / DV))           # spinodal.cpp:95: sqrt(epsilon dt/dV)
NOISY = [
    ("modelA_2d", "ac_poly", (48, 40), dict(r=1.0, u=1.0, kappa=1.0, mobility=1.0, dt=DT, noise=SIGMA_AB), 60),
    ("modelA_3d_graph_length", "ac_poly", (12, 10, 14), dict(r=1.0, u=1.0, kappa=1.0, mobility=1.0, dt=DT,
                                                          noise=SIGMA_AB), 150),
    ("modelB_2d", "ch_poly", (40, 36), dict(r=1.0, u=1.0, kappa=1.0, mobility=1.0, dt=DT, noise=SIGMA_AB), 60),
    ("modelB_3d", "ch_poly", (10, 12, 9), dict(r=1.0, u=1.0, kappa=1.0, mobility=1.0, dt=DT, noise=SIGMA_AB), 40),
    ("spinodal_2d", "ch_poly", (64, 48), dict(r=1.0, u=1.0, kappa=1.0, mobility=0.5 / DV, dt=DT, noise=SIGMA_SPIN),
     80),
]


def noisy_oracle(oracle, model, x, steps, prm, seed, step0=0):
    kw = dict(r=prm["r"], u=prm["u"], K=prm["kappa"], M=prm["mobility"], dt=prm["dt"], noise=prm["noise"],
              seed=seed, step0=step0)
    if model == "ac_poly":
        return oracle.ac_scalar_noise(x, steps, **kw)
    return oracle.ch_shipped_noise(x, steps, **kw)


@pytest.mark.parametrize("name,model,shape,prm,steps", NOISY, ids=[n[0] for n in NOISY])
def test_stochastic_forms_against_oracle(gpu, oracle, name, model, shape, prm, steps):
    from mmsp_gb300 import inputs

    seed = 1234 + len(name)
    x = inputs.noisy_composition(shape, 0.0, 0.2, 77 + len(shape))
    want = noisy_oracle(oracle, model, x, steps, prm, seed)
    d64 = gpu.make_desc(shape, 1, np.float64, model, seed=seed, **prm)
    got = run_gpu(gpu, d64, x, steps)
    assert np.abs(got - want).max() <= TOL_SHIPPED * max(1.0, np.abs(want).max())
    d32 = gpu.make_desc(shape, 1, np.float32, model, seed=seed, **prm)
    got32 = run_gpu(gpu, d32, x.astype(np.float32), steps).astype(np.float64)
    assert np.abs(got32 - want).max() <= TOL_F32
    # the noise acts: the deterministic form ends elsewhere
    plain = dict(prm, noise=0.0)
    assert np.abs(noisy_oracle(oracle, model, x, steps, plain, seed) - want).max() > 1e-4


def test_stochastic_stream_is_deterministic_and_continues(gpu, oracle):
    from mmsp_gb300 import inputs

    shape = (32, 24)
    prm = dict(r=1.0, u=1.0, kappa=1.0, mobility=1.0, dt=DT, noise=SIGMA_AB)
    x = inputs.noisy_composition(shape, 0.0, 0.2, 5)
    d = gpu.make_desc(shape, 1, np.float64, "ch_poly", seed=9, **prm)
    a = run_gpu(gpu, d, x, 30)
    assert np.array_equal(a, run_gpu(gpu, d, x, 30))                  # same seed, same bits
    with gpu.Stepper(d) as s:                                         # steps split over calls
        s.upload(x)
        s.step(12)
        s.step(18)
        assert np.array_equal(s.download(), a)
    d2 = gpu.make_desc(shape, 1, np.float64, "ch_poly", seed=10, **prm)
    assert not np.array_equal(run_gpu(gpu, d2, x, 30), a)             # another seed, another path
    # a new upload restarts the stream at step 0
    with gpu.Stepper(d) as s:
        s.upload(x)
        s.step(7)
        s.upload(x)
        s.step(30)
        assert np.array_equal(s.download(), a)


def test_stochastic_forms_are_refused_where_no_step_index_travels(gpu):
    d = gpu.make_desc((64, 64), 1, np.float32, "ch_poly", noise=0.1, seed=1)
    with pytest.raises(gpu.GpuError) as e:
        gpu.Batch([d, d])
    assert e.value.code == gpu.EUNSUPPORTED
    bad = gpu.make_desc((8, 8), 1, np.float64, "ch_poly", noise=-1.0)
    with pytest.raises(gpu.GpuError) as e:
        gpu.Stepper(bad)
    assert e.value.code == gpu.EINVAL


# Convex-splitting Cahn-Hilliard: an implicit solve per step (red-black SOR to
# a 1e-14 relative residual).  FP64 is compared with the oracle, which matches
# the reference program bit for bit including its iteration counts.
CONVEX = [((40, 20), None, 4), ((64, 48), 5, 6), ((12, 10, 8), 31, 3), ((128,), 7, 10)]


@pytest.mark.parametrize("shape,seed,steps", CONVEX, ids=["x".join(map(str, s)) for s, _, _ in CONVEX])
def test_convex_splitting_against_oracle(gpu, oracle, shape, seed, steps):
    from mmsp_gb300 import inputs

    x = inputs.convex_start(shape, seed)
    want, iters = oracle.ch_convex(x, steps, return_iters=True)
    d = gpu.make_desc(shape, 2, np.float64, "ch_convex")
    with gpu.Stepper(d) as s:
        s.upload(x)
        states = [x]
        for k in range(steps):
            s.step(1)
            states.append(s.download())
        st = s.reduce()
        got = states[-1]
    assert abs(st.solver_iterations - iters) <= 5           # residual sums differ only in rounding
    assert np.abs(got - want).max() <= 1e-10 * max(1.0, np.abs(want).max())
    # convex splitting (Eyre) is energy-stable for the discrete energy of its
    # Laplacian, the one with forward-difference gradients
    fd = [convex_energy(y[..., 0], forward=True) for y in states]
    assert all(b <= a + 1e-10 * abs(a) for a, b in zip(fd, fd[1:])), fd
    # the reduction reports the example's reportEnergy (central differences) and the mass of c
    assert abs(st.energy - convex_energy(got[..., 0])) <= 1e-11 * abs(st.energy)
    assert abs(st.mass - x[..., 0].sum()) <= 1e-9 * abs(x[..., 0].sum())   # c is conserved


def convex_energy(c, forward=False, C0=0.45, Ca=0.05, Cb=0.95, A=2.0, K=2.0):
    """sum of energy_density(c) + K/2 |grad c|^2 (cahn-hilliard.cpp:57-80, 172-200), dx = 1:
    central differences as reportEnergy's grad, or forward differences."""
    B = A / (Ca - C0) ** 2
    f = -0.5 * A * (c - C0) ** 2 + 0.25 * B * (c - C0) ** 4 + 0.25 * Ca * (c - Ca) ** 4 + 0.25 * Cb * (c - Cb) ** 4
    g2 = np.zeros_like(c)
    for a in range(c.ndim):
        g = np.roll(c, -1, a) - c if forward else 0.5 * (np.roll(c, -1, a) - np.roll(c, 1, a))
        g2 += g * g
    return float((f + 0.5 * K * g2).sum())


def test_convex_splitting_refusals(gpu):
    with pytest.raises(gpu.GpuError) as e:
        gpu.Stepper(gpu.make_desc((40, 20), 2, np.float32, "ch_convex"))
    assert e.value.code == gpu.EUNSUPPORTED                   # FP64 only
    with pytest.raises(gpu.GpuError) as e:
        gpu.Stepper(gpu.make_desc((41, 20), 2, np.float64, "ch_convex"))
    assert e.value.code == gpu.EUNSUPPORTED                   # odd extent
    with pytest.raises(gpu.GpuError) as e:
        gpu.Stepper(gpu.make_desc((40, 20), 1, np.float64, "ch_convex"))
    assert e.value.code == gpu.EINVAL                         # c and mu
