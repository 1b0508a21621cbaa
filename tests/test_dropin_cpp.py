"""The C++ drop-in (include/MMSP.gpu.hpp) used the way a plugin uses it.

tests/cpp/dropin_main.cpp defines the plugin's update() by forwarding to
MMSP::gpu::update.  Where the reference headers exist it is built against the
reference's own grid (oracle/_ref/dropin_ref, by ``make -C oracle ref``);
elsewhere it is built against tests/cpp/mini_grid.hpp, a stand-in with the
same free-function interface.
"""
import os
import shutil
import subprocess
import tempfile

import numpy as np
import pytest

from conftest import ROOT

REF_DROPIN = os.path.join(ROOT, "oracle", "_ref", "dropin_ref")


def build_mini(tmp):
    from mmsp_gb300 import build

    exe = os.path.join(tmp, "dropin_mini")
    cxx = shutil.which("g++") or "g++"
    subprocess.run([cxx, "-O2", "-std=c++11", "-Wall", "-I", os.path.join(ROOT, "tests", "cpp"),
                    "-I", os.path.join(ROOT, "include"), os.path.join(ROOT, "tests", "cpp", "dropin_main.cpp"),
                    "-o", exe, "-L", build.LIBDIR, "-lmmsp_gpu", "-Wl,-rpath," + build.LIBDIR],
                   check=True, capture_output=True)
    return exe


def run(exe, mode, x, steps, shape, fields=None):
    with tempfile.TemporaryDirectory() as td:
        fi = os.path.join(td, "in.raw")
        fo = os.path.join(td, "out.raw")
        np.ascontiguousarray(x).tofile(fi)
        args = [exe, mode, fi, fo, str(steps)] + [str(s) for s in shape]
        if fields:
            args.append(str(fields))
        r = subprocess.run(args, capture_output=True, text=True)
        out = np.fromfile(fo, dtype=x.dtype).reshape(x.shape) if r.returncode == 0 else None
    return r, out


def test_stand_in_builds(tmp_path):
    from mmsp_gb300 import build

    if not os.path.exists(build.LIB):
        build.build()
    assert os.path.exists(build_mini(str(tmp_path)))


@pytest.mark.skipif(not os.path.exists(REF_DROPIN), reason="reference headers not present in this checkout")
def test_reference_grid_build_reports_errors_like_the_reference():
    """Built against the reference's grid; without a GPU the wrapper prints
    the library's message and exits through MMSP::Abort(code) (utility.cpp:30-36)."""
    import ctypes

    from mmsp_gb300 import native

    try:
        has_gpu = ctypes.CDLL("libcuda.so.1") is not None
    except OSError:
        has_gpu = False
    x = np.zeros((4, 4, 4))
    r, out = run(REF_DROPIN, "ch", x, 1, x.shape)
    if has_gpu and r.returncode == 0:
        assert np.array_equal(out, x)   # a uniform state is a fixed point
    else:
        assert r.returncode == (native.ENODEV & 0xFF)
        assert "no suitable CUDA device" in r.stderr


@pytest.mark.gpu
def test_dropin_scalar_and_vector_grids_on_device(gpu, oracle, tmp_path):
    from mmsp_gb300 import inputs

    exe = build_mini(str(tmp_path))
    c0 = inputs.noisy_composition((20, 24, 28), 0.4, 0.02, 41)
    r, out = run(exe, "ch", c0, 25, c0.shape)
    assert r.returncode == 0, r.stderr
    assert np.array_equal(out, oracle.ch_baseline(c0, 25, 1.0, 1.0, 0.002))
    r, out = run(exe, "ch_f32", c0.astype(np.float32), 25, c0.shape)
    assert r.returncode == 0, r.stderr
    assert np.abs(out.astype(np.float64) - oracle.ch_baseline(c0, 25, 1.0, 1.0, 0.002)).max() <= 1e-5
    e0 = inputs.graingrowth_circles((40, 40, 6), 2)
    r, out = run(exe, "gg", e0, 30, e0.shape[:-1], 2)
    assert r.returncode == 0, r.stderr
    want = oracle.ac_graingrowth(e0, 30, 0.01)
    assert np.abs(out - want).max() <= 1e-12 * np.abs(want).max()


@pytest.mark.gpu
def test_run_loop_writes_the_snapshots_of_main(gpu, oracle, tmp_path):
    """MMSP::gpu::run replaces MMSP.main.hpp's update/output loop with the state
    on the device: one file per increment, named base.<step zero-padded to the
    digits of the step count>.dat, holding the state after that many steps."""
    from mmsp_gb300 import gridfile, inputs

    exe = build_mini(str(tmp_path))
    c0 = inputs.noisy_composition((12, 14, 16), 0.4, 0.02, 42)
    fi, fo, base = str(tmp_path / "in.raw"), str(tmp_path / "out.raw"), str(tmp_path / "ch")
    c0.tofile(fi)
    r = subprocess.run([exe, "run_ch", fi, base, fo, "120", "40", "12", "14", "16"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    for k in (40, 80, 120):
        g = gridfile.read(base + ".%03d.dat" % k)
        assert g.type_name == "grid:double" and g.shape == (12, 14, 16)
        assert np.array_equal(g.data, oracle.ch_baseline(c0, k, 1.0, 1.0, 0.002))
    assert np.array_equal(np.fromfile(fo).reshape(c0.shape), oracle.ch_baseline(c0, 120, 1.0, 1.0, 0.002))
    e0 = inputs.graingrowth_circles((20, 20, 4), 2)
    e0.tofile(fi)
    r = subprocess.run([exe, "run_gg", fi, str(tmp_path / "gg"), fo, "30", "10", "20", "20", "4", "2"],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    g = gridfile.read(str(tmp_path / "gg") + ".30.dat")
    want = oracle.ac_graingrowth(e0, 30, 0.01)
    assert g.vector and g.fields == 2 and np.abs(g.data - want).max() <= 1e-12 * np.abs(want).max()


@pytest.mark.gpu
def test_dropin_sparse_grid_on_device(gpu, oracle, tmp_path):
    """update(grid<3,sparse<double>>&, steps) through MMSP::gpu::update: the
    items of every cell, in stored order, as the oracle's sparsePF update."""
    from mmsp_gb300 import inputs

    exe = build_mini(str(tmp_path))
    shape, K = (10, 12, 8), 32
    c0, i0, v0 = inputs.sparse_grains(shape, 7, 12, K)
    fi, fo = str(tmp_path / "in.bin"), str(tmp_path / "out.bin")
    with open(fi, "wb") as f:
        f.write(np.asarray([3] + list(shape), np.int32).tobytes())
        for c, ii, vv in zip(c0.ravel(), i0.reshape(-1, K), v0.reshape(-1, K)):
            f.write(np.int32(c).tobytes())
            for h in range(c):
                f.write(np.int32(ii[h]).tobytes() + np.float64(vv[h]).tobytes())
    r = subprocess.run([exe, "sparse", fi, fo, "30"] + [str(s) for s in shape], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    wc, wi, wv, _ = oracle.sparse_gg(c0, i0, v0, 30)
    b = open(fo, "rb").read()
    p = 16
    wi, wv = wi.reshape(-1, K), wv.reshape(-1, K)
    for k, n in enumerate(wc.ravel()):
        assert int(np.frombuffer(b, np.int32, 1, p)[0]) == n
        p += 4
        for h in range(n):
            assert int(np.frombuffer(b, np.int32, 1, p)[0]) == wi[k, h]
            v = float(np.frombuffer(b, np.float64, 1, p + 4)[0])
            assert abs(v - wv[k, h]) <= 1e-12 * max(1.0, abs(wv[k, h]))
            p += 12
    assert p == len(b)
