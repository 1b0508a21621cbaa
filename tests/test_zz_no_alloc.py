"""mmsp_gpu_step_noalloc: the entry point for callers that cannot allocate.

Callers whose device memory belongs to another allocator or a fixed budget,
or whose hot loops must not call cudaMalloc/cudaFree (they may synchronise
the whole device), pass their own device buffers and the library keeps a
multi-step run's intermediate state in a fixed, process-wide device array.
These tests call it through the C ABI twice in a row (the second call finds
the first call's leftovers in the shared array) and compare each result with
the handle-based entry points (mmsp_gpu_create/upload/step/download): bit
for bit in FP64, within the FP32 tolerance of the other parity tests.

This file is collected last, so a run that stops at the first failure has
run every other test before it.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL_F32 = 1e-5


def reference_run(native, desc, x, steps_list):
    """States after each cumulative step count, through a handle."""
    outs = []
    with native.Stepper(desc) as s:
        s.upload(x, native.FIELD_MAJOR)
        done = 0
        for n in steps_list:
            s.step(n - done)
            done = n
            outs.append(s.download(native.FIELD_MAJOR))
    return outs


def noalloc(native, desc, src, dst, steps, stream=0):
    L = native.load()
    return L.mmsp_gpu_step_noalloc(ctypes.byref(desc), ctypes.c_void_p(src.data_ptr()),
                                   ctypes.c_void_p(dst.data_ptr()), int(steps), ctypes.c_void_p(stream))


@pytest.mark.parametrize("case", ["ch3d_f64", "ch3d_f32_stream", "ac3d_f64", "ch2d_f32"])
def test_noalloc_matches_handle_path_two_calls(gpu, case):
    import torch

    from mmsp_gb300 import inputs

    native = gpu
    if case == "ch3d_f64":
        x = inputs.noisy_composition((24, 20, 36), 0.4, 0.02, 71)
        d = native.make_desc(x.shape, 1, np.float64, "ch", dt=0.002)
    elif case == "ch3d_f32_stream":
        x = inputs.noisy_composition((40, 24, 64), 0.4, 0.02, 72).astype(np.float32)
        d = native.make_desc(x.shape, 1, np.float32, "ch", dt=0.002)
    elif case == "ac3d_f64":
        e = inputs.voronoi_grains((12, 14, 16), 8, 4, 73)
        x = np.ascontiguousarray(np.moveaxis(e, -1, 0))    # field-major, the device layout
        d = native.make_desc(e.shape[:-1], 4, np.float64, "ac", gamma=1.5, kappa=2.0, dt=0.05)
    else:
        x = inputs.noisy_composition((96, 64), 0.5, 0.01, 74).astype(np.float32)
        d = native.make_desc(x.shape, 1, np.float32, "ch", dt=0.005)
    want7, want12 = reference_run(native, d, x, [7, 12])

    dev_in = torch.from_numpy(np.ascontiguousarray(x)).cuda()
    dev_a = torch.empty_like(dev_in)
    torch.cuda.synchronize()
    # first call: 7 steps, distinct input and output
    assert noalloc(native, d, dev_in, dev_a, 7) == native.OK
    got7 = dev_a.cpu().numpy()
    # second call: 5 more steps in place, on top of the first call's scratch contents
    assert noalloc(native, d, dev_a, dev_a, 5) == native.OK
    got12 = dev_a.cpu().numpy()
    assert np.array_equal(dev_in.cpu().numpy(), x)    # the input is not written
    for got, want in ((got7, want7), (got12, want12)):
        assert got.shape == want.shape
        if x.dtype == np.float64:
            assert np.array_equal(got, want), np.abs(got - want).max()
        else:
            assert np.abs(got.astype(np.float64) - want).max() <= TOL_F32


def test_noalloc_rejects_grids_beyond_the_scratch(gpu):
    import torch

    native = gpu
    # 2^22 + 2^16 FP32 cells: above the 16 MiB scratch
    shape = (64 + 1, 256, 256)
    d = native.make_desc(shape, 1, np.float32, "ch", dt=0.002)
    assert np.prod(shape) * 4 > native.NOALLOC_MAX_BYTES
    a = torch.zeros(shape, dtype=torch.float32, device="cuda")
    b = torch.empty_like(a)
    assert noalloc(native, d, a, b, 2) == native.ENOMEM      # needs the scratch: refused
    assert noalloc(native, d, a, a, 1) == native.ENOMEM      # in place needs it too
    assert noalloc(native, d, a, b, 1) == native.OK          # one step in -> out needs none
    assert bool(torch.isfinite(b).all())                      # finished, finite result
    bad = native.make_desc((8, 8), 2, np.float64, "ch")      # invalid descriptor
    assert noalloc(native, bad, a, b, 1) == native.EINVAL
