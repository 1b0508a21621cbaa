"""Snapshots of a device state as MMSP grid files (mmsp_gpu_output).

A snapshot queued between steps must hold the state at that point of the
stream even though later steps are already queued behind it, and its file
must be the one mmsp_gpu_write_grid writes for the same values (the host
writer is pinned to the reference's grid::output on the CPU).
"""
import os

import numpy as np
import pytest

from mmsp_gb300 import gridfile, inputs, native

pytestmark = pytest.mark.gpu

CASES = [
    ("ch2d_f64", (64, 48), 1, np.float64, "ch", dict(dt=0.005)),
    ("ch3d_f32_chunked", (80, 64, 64), 1, np.float32, "ch", dict(dt=0.002)),
    ("ac3d_f32", (24, 20, 32), 5, np.float32, "ac", dict(dt=0.05, gamma=1.5, kappa=2.0)),
    ("ac3d_f64_chunked", (32, 32, 40), 4, np.float64, "gg", dict(dt=0.01)),
]


def start(shape, fields, dtype):
    if fields == 1:
        return inputs.noisy_composition(shape, 0.45, 0.05, 31).astype(dtype)
    return (inputs.voronoi_grains(shape, 9, fields, 32) * 0.8 + 0.05).astype(dtype)


def state_after(d, x, steps):
    with native.Stepper(d) as s:
        s.upload(x)
        s.step(steps)
        return s.download()


@pytest.mark.parametrize("name,shape,fields,dtype,model,params", CASES, ids=[c[0] for c in CASES])
def test_snapshots_between_queued_steps(gpu, tmp_path, name, shape, fields, dtype, model, params):
    d = native.make_desc(shape, fields, dtype, model, **params)
    x = start(shape, fields, dtype)
    with native.Stepper(d) as s:
        s.upload(x)
        s.step(7)
        s.output(str(tmp_path / "a.dat"))
        s.step(5)                          # queued while snapshot a is still copied and written
        s.output(str(tmp_path / "b.dat"), level=1)
        s.step(3)
        s.output(str(tmp_path / "c.dat"), level=0)
        s.output_wait()
        final = s.download()
    want = {"a": state_after(d, x, 7), "b": state_after(d, x, 12), "c": final}
    for k, v in want.items():
        g = gridfile.read(str(tmp_path / (k + ".dat")))
        assert g.vector == (fields > 1)
        assert np.array_equal(g.data, v), k
    # the same bytes as the host writer's file of the same values
    gpu.write_grid(str(tmp_path / "a_host.dat"), want["a"], d)
    assert (tmp_path / "a.dat").read_bytes() == (tmp_path / "a_host.dat").read_bytes()


def test_many_snapshots_reuse_the_buffers(gpu, tmp_path):
    shape = (96, 96, 64)
    d = native.make_desc(shape, 1, np.float32, "ch", dt=0.002)
    x = start(shape, 1, np.float32)
    with native.Stepper(d) as s:
        s.upload(x)
        for i in range(6):
            s.step(2)
            s.output(str(tmp_path / ("s%d.dat" % i)), threads=4)
        s.output_wait()
        states = [gridfile.read(str(tmp_path / ("s%d.dat" % i))).data for i in range(6)]
        last = s.download()
    assert np.array_equal(states[-1], last)
    assert np.array_equal(states[0], state_after(d, x, 2))
    assert all(not np.array_equal(states[i], states[i + 1]) for i in range(5))


def test_write_failure_is_reported_by_wait(gpu, tmp_path):
    d = native.make_desc((32, 32), 1, np.float64, "ch")
    with native.Stepper(d) as s:
        s.upload(start((32, 32), 1, np.float64))
        s.output(str(tmp_path / "missing_dir" / "x.dat"))
        with pytest.raises(native.GpuError) as e:
            s.output_wait()
        assert e.value.code == native.EIO
        s.output_wait()                            # the failure is reported once
        s.output(str(tmp_path / "ok.dat"))
        s.output_wait()
    assert os.path.exists(tmp_path / "ok.dat")
    with native.Stepper(d) as s:
        s.upload(start((32, 32), 1, np.float64))
        with pytest.raises(native.GpuError) as e:
            s.output(str(tmp_path / "bad.dat"), level=11)
        assert e.value.code == native.EINVAL


def test_destroy_waits_for_queued_snapshots(gpu, tmp_path):
    shape = (64, 64, 64)
    d = native.make_desc(shape, 1, np.float32, "ch", dt=0.002)
    x = start(shape, 1, np.float32)
    s = native.Stepper(d)
    s.upload(x)
    s.step(4)
    s.output(str(tmp_path / "z.dat"))
    s.close()                                      # no output_wait
    assert np.array_equal(gridfile.read(str(tmp_path / "z.dat")).data, state_after(d, x, 4))
