"""The C ABI library on a machine without a GPU: it loads, exports every
symbol include/MMSP.gpu.h declares, and its host-only entry points work."""
import ctypes
import os
import re

import numpy as np
import pytest

from conftest import ROOT


def header_symbols():
    src = open(os.path.join(ROOT, "include", "MMSP.gpu.h")).read()
    return sorted(set(re.findall(r"\b(mmsp_gpu_[a-z_0-9]+)\s*\(", src)))


@pytest.fixture(scope="module")
def lib():
    from mmsp_gb300 import build, native

    if not os.path.exists(build.LIB):
        build.build()
    return native.load()


def test_header_and_binding_agree():
    from mmsp_gb300 import native

    assert header_symbols() == sorted(native.EXPORTS)


def test_library_exports_every_declared_symbol(lib):
    for name in header_symbols():
        assert hasattr(lib, name), name


def test_version_and_strerror(lib):
    assert lib.mmsp_gpu_version() == 3
    assert lib.mmsp_gpu_strerror(0) == b"ok"
    assert lib.mmsp_gpu_strerror(-4) == b"unsupported configuration"


def test_desc_init_defaults(lib):
    from mmsp_gb300 import native

    d = native.Desc()
    n = (ctypes.c_int * 3)(256, 256, 1)
    assert lib.mmsp_gpu_desc_init(ctypes.byref(d), 2, n, 1, native.F64, native.CH) == 0
    assert (d.dim, d.n[0], d.n[1], d.n[2], d.fields) == (2, 256, 256, 1, 1)
    assert [d.bc[a][s] for a in range(3) for s in range(2)] == [native.BC_PERIODIC] * 6
    assert d.dt == 0.005 and d.kappa == 1.0 and d.mobility == 1.0
    assert lib.mmsp_gpu_desc_init(ctypes.byref(d), 3, n, 2, native.F32, native.GG) == 0
    assert d.dt == 0.01 and d.kappa == 2.0
    assert lib.mmsp_gpu_desc_init(ctypes.byref(d), 2, n, 3, native.F64, native.OSTWALD) == 0
    assert (d.dt, d.kappa, d.mobility) == (0.001, 2.0, 1.0)              # ostwald.cpp:66-80
    assert list(d.aux) == [1.0, 0.05, 0.95, 2.0, 1.0, 3.0]
    assert ctypes.sizeof(native.Desc) == 4 * 14 + 8 * 15          # C layout: 14 ints, 15 doubles
    assert native.Desc.dx.offset == 56                             # where ABI version 2 had it
    assert d.flags == 0
    d.flags = 2
    assert lib.mmsp_gpu_validate(ctypes.byref(d)) == native.EINVAL   # unknown flag
    d.flags = native.FLAG_CONTRACT
    assert lib.mmsp_gpu_validate(ctypes.byref(d)) == native.OK


def test_ostwald_validation_and_footprint(lib):
    from mmsp_gb300 import native

    d = native.make_desc((16, 16), fields=1, model="ostwald")
    assert lib.mmsp_gpu_validate(ctypes.byref(d)) == native.EINVAL          # needs an order parameter
    d = native.make_desc((16, 16), fields=3, model="ostwald", Cbeta=0.05)
    assert lib.mmsp_gpu_validate(ctypes.byref(d)) == native.EINVAL          # Calpha == Cbeta
    d = native.make_desc((16, 16), fields=3, model="ostwald")
    assert lib.mmsp_gpu_validate(ctypes.byref(d)) == native.OK
    b = ctypes.c_size_t()
    assert lib.mmsp_gpu_footprint(ctypes.byref(d), ctypes.byref(b)) == 0
    assert b.value >= 2 * 3 * 256 * 8 + 256 * 8                              # two states and the work grid
    x = np.zeros(16 * 16 * 3)
    assert lib.mmsp_gpu_step_noalloc(ctypes.byref(d), x.ctypes.data, x.ctypes.data, 1, None) == native.EUNSUPPORTED


def test_validation_without_device(lib):
    from mmsp_gb300 import native

    d = native.make_desc((8, 8), model="ch")
    assert lib.mmsp_gpu_validate(ctypes.byref(d)) == native.OK
    d.bc[0][0] = native.BC_NEUMANN
    assert lib.mmsp_gpu_validate(ctypes.byref(d)) == native.EUNSUPPORTED
    d = native.make_desc((8, 8), fields=2, model="ch")
    assert lib.mmsp_gpu_validate(ctypes.byref(d)) == native.EINVAL
    d = native.make_desc((8, 8, 8), fields=40, model="ac")
    assert lib.mmsp_gpu_validate(ctypes.byref(d)) == native.EUNSUPPORTED
    d = native.make_desc((8, 0), model="ch")
    assert lib.mmsp_gpu_validate(ctypes.byref(d)) == native.EINVAL
    d = native.make_desc((8, 8), model="ch", dx=[0.0, 1.0])
    assert lib.mmsp_gpu_validate(ctypes.byref(d)) == native.EINVAL
    d = native.make_desc((8, 8), model="ch", dt=float("nan"))
    assert lib.mmsp_gpu_validate(ctypes.byref(d)) == native.EINVAL
    d.dim = 4
    assert lib.mmsp_gpu_validate(ctypes.byref(d)) == native.EINVAL
    assert lib.mmsp_gpu_validate(None) == native.EINVAL


def test_footprint(lib):
    from mmsp_gb300 import native

    d = native.make_desc((256, 256, 256), model="ch", dtype=np.float32)
    b = ctypes.c_size_t()
    assert lib.mmsp_gpu_footprint(ctypes.byref(d), ctypes.byref(b)) == 0
    assert b.value >= 2 * 256 ** 3 * 4
    assert b.value < 2 * 256 ** 3 * 4 + (1 << 20)


def test_null_arguments_are_rejected(lib):
    from mmsp_gb300 import native

    assert lib.mmsp_gpu_create(None, None) == native.EINVAL
    assert lib.mmsp_gpu_destroy(None) == native.OK
    assert lib.mmsp_gpu_step(None, 1) == native.EINVAL
    assert lib.mmsp_gpu_reduce(None, None) == native.EINVAL
    assert lib.mmsp_gpu_last_error(None) == b"NULL handle"


def test_batch_and_server_refuse_without_a_device(lib):
    """On a machine with no CUDA device the batched and serving entry points
    return MMSP_GPU_ENODEV instead of failing later."""
    import ctypes

    from mmsp_gb300 import native

    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a CUDA device is present")
    except ImportError:
        pass
    d = native.make_desc((32, 32), 1, np.float32, "ch")
    arr = (native.Desc * 1)(d)
    b = ctypes.c_void_p()
    assert lib.mmsp_gpu_batch_create(ctypes.byref(b), 1, arr) == native.ENODEV
    s = ctypes.c_void_p()
    cfg = native.ServerConfig(0, 0, 0)
    assert lib.mmsp_gpu_server_start(ctypes.byref(s), ctypes.byref(cfg)) == native.ENODEV
    assert lib.mmsp_gpu_batch_create(ctypes.byref(b), 0, arr) == native.EINVAL


def test_noalloc_refuses_misaligned_and_overlapping_pointers(lib):
    """mmsp_gpu_step_noalloc checks the caller's pointers on the host, before
    it touches a device: the FP32 3D kernels stage planes with bulk copies
    that need 16-byte-aligned addresses, and an output that partly overlaps
    the input would be written while it is still read.  The addresses below
    are never dereferenced (no device work is queued for a refused call),
    so the test runs without a GPU."""
    from mmsp_gb300 import native

    d = native.make_desc((40, 24, 64), 1, np.float32, "ch", dt=0.002)
    nbytes = 40 * 24 * 64 * 4
    base = 1 << 32
    call = lambda i, o, steps=1: lib.mmsp_gpu_step_noalloc(ctypes.byref(d), ctypes.c_void_p(i),
                                                           ctypes.c_void_p(o), steps, None)
    assert call(base + 4, base + nbytes + 256) == native.EINVAL        # input 4 bytes off a 16-byte boundary
    assert call(base, base + nbytes + 260) == native.EINVAL            # output misaligned
    assert call(base + 8, base + 8) == native.EINVAL                   # in place, misaligned
    assert call(base, base + nbytes - 16) == native.EINVAL             # output overlaps the input's tail
    assert call(base + 4096, base) == native.EINVAL                    # input overlaps the output's tail
    assert call(base, base + 16, 0) == native.EINVAL                   # a zero-step copy checks too
    assert call(0, base) == native.EINVAL                              # NULL


def test_sparse_descriptor_validation(lib):
    """Sparse grain growth: FP64 only, 1..32 slots per cell, finite epsilon;
    defaults of the sparsePF example (dt 0.01, epsilon 1e-8)."""
    from mmsp_gb300 import native

    d = native.make_desc((32, 16), 8, np.float64, "sparse_gg")
    assert (d.dt, d.aux[0]) == (0.01, 1e-8)
    assert lib.mmsp_gpu_validate(ctypes.byref(d)) == native.OK
    b = ctypes.c_size_t()
    assert lib.mmsp_gpu_footprint(ctypes.byref(d), ctypes.byref(b)) == 0
    assert b.value >= 2 * 32 * 16 * (4 + 8 * 12)
    d = native.make_desc((32, 16), 8, np.float32, "sparse_gg")
    assert lib.mmsp_gpu_validate(ctypes.byref(d)) == native.EUNSUPPORTED
    d = native.make_desc((32, 16), 40, np.float64, "sparse_gg")
    assert lib.mmsp_gpu_validate(ctypes.byref(d)) == native.EUNSUPPORTED
    d = native.make_desc((32, 16), 8, np.float64, "sparse_gg", epsilon=float("inf"))
    assert lib.mmsp_gpu_validate(ctypes.byref(d)) == native.EINVAL
    assert lib.mmsp_gpu_strerror(native.EOVERFLOW) == b"sparse cell list outgrew its slots"
