"""ctypes binding of libmmsp_gpu.so (the C ABI declared in include/MMSP.gpu.h).

There is no CPU fallback: if the library is missing or no CUDA device is
present, the calls raise.  The binding mirrors the header one to one; the
Pythonic helpers (``Stepper``, ``update``) only marshal numpy arrays.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from . import build as _build

OK, EINVAL, ENOMEM, ECUDA, EUNSUPPORTED, ETIMEDOUT, ENODEV, ENOTFOUND, ECANCELED, ESTOPPED, EIO, ENOCONV, \
    EOVERFLOW = 0, -1, -2, -3, -4, -5, -6, -7, -8, -9, -10, -11, -12
BC_MIRROR, BC_NEUMANN, BC_PERIODIC, BC_PARALLEL, BC_DIRICHLET = 0, 1, 2, 3, 4
F64, F32 = 0, 1
FLAG_CONTRACT = 1   # MMSP_GPU_FLAG_CONTRACT
CH, CH_POLY, AC, GG, AC_POLY, ZENER, OSTWALD, CH_CONVEX, SPARSE_GG = 0, 1, 2, 3, 4, 5, 6, 7, 8
CELL_MAJOR, FIELD_MAJOR = 0, 1

MODELS = {"ch": CH, "ch_poly": CH_POLY, "ac": AC, "gg": GG, "ac_poly": AC_POLY, "zener": ZENER,
          "ostwald": OSTWALD, "ch_convex": CH_CONVEX, "sparse_gg": SPARSE_GG}
OSTWALD_AUX = ("D", "Calpha", "Cbeta", "A", "delta", "epsilon")   # mmsp_gpu_desc.aux of MMSP_GPU_OSTWALD
NOISE_AUX = ("noise", "seed")   # mmsp_gpu_desc.aux of MMSP_GPU_CH_POLY / MMSP_GPU_AC_POLY
CONVEX_AUX = ("C0", "Ca", "Cb", "A", "omega", "tolerance")   # mmsp_gpu_desc.aux of MMSP_GPU_CH_CONVEX
SPARSE_AUX = ("epsilon",)   # mmsp_gpu_desc.aux of MMSP_GPU_SPARSE_GG
DTYPES = {np.dtype(np.float64): F64, np.dtype(np.float32): F32}

# Every symbol include/MMSP.gpu.h declares (checked by the CPU test suite).
EXPORTS = [
    "mmsp_gpu_version", "mmsp_gpu_strerror", "mmsp_gpu_desc_init", "mmsp_gpu_validate",
    "mmsp_gpu_footprint", "mmsp_gpu_create", "mmsp_gpu_destroy", "mmsp_gpu_set_stream",
    "mmsp_gpu_upload", "mmsp_gpu_download", "mmsp_gpu_upload_device", "mmsp_gpu_download_device",
    "mmsp_gpu_step", "mmsp_gpu_synchronize", "mmsp_gpu_reduce", "mmsp_gpu_state",
    "mmsp_gpu_last_error", "mmsp_gpu_update", "mmsp_gpu_step_noalloc", "mmsp_gpu_fp64_rate",
    "mmsp_gpu_sparse_upload", "mmsp_gpu_sparse_download",
    "mmsp_gpu_output_opts_init", "mmsp_gpu_write_grid", "mmsp_gpu_output", "mmsp_gpu_output_wait",
    "mmsp_gpu_batch_create", "mmsp_gpu_batch_destroy", "mmsp_gpu_batch_set_stream", "mmsp_gpu_batch_upload",
    "mmsp_gpu_batch_download", "mmsp_gpu_batch_upload_all", "mmsp_gpu_batch_download_all", "mmsp_gpu_batch_step", "mmsp_gpu_batch_synchronize", "mmsp_gpu_batch_reduce",
    "mmsp_gpu_batch_tune", "mmsp_gpu_batch_get_info", "mmsp_gpu_batch_last_error",
    "mmsp_gpu_server_start", "mmsp_gpu_server_submit", "mmsp_gpu_server_poll", "mmsp_gpu_server_wait",
    "mmsp_gpu_server_fetch", "mmsp_gpu_server_cancel", "mmsp_gpu_server_get_stats", "mmsp_gpu_server_stop",
]
REQ_QUEUED, REQ_RUNNING, REQ_DONE = 0, 1, 2
NOALLOC_MAX_BYTES = 16 << 20   # MMSP_GPU_NOALLOC_MAX_BYTES


class Desc(ctypes.Structure):
    _fields_ = [("dim", ctypes.c_int), ("n", ctypes.c_int * 3), ("fields", ctypes.c_int),
                ("dtype", ctypes.c_int), ("model", ctypes.c_int), ("bc", (ctypes.c_int * 2) * 3),
                ("flags", ctypes.c_int), ("dx", ctypes.c_double * 3), ("dt", ctypes.c_double), ("kappa", ctypes.c_double),
                ("mobility", ctypes.c_double), ("gamma", ctypes.c_double), ("r", ctypes.c_double),
                ("u", ctypes.c_double), ("aux", ctypes.c_double * 6)]


class OutputOpts(ctypes.Structure):
    _fields_ = [("level", ctypes.c_int), ("threads", ctypes.c_int), ("vector", ctypes.c_int),
                ("fields_line", ctypes.c_int), ("g0", ctypes.c_int * 3)]


class Stats(ctypes.Structure):
    _fields_ = [("mass", ctypes.c_double), ("energy", ctypes.c_double), ("gpu_ms", ctypes.c_double),
                ("steps", ctypes.c_int64), ("solver_iterations", ctypes.c_int64)]


class BatchInfo(ctypes.Structure):
    _fields_ = [("instances", ctypes.c_int), ("persistent", ctypes.c_int), ("fallback", ctypes.c_int),
                ("rows_per_item", ctypes.c_int), ("threads_per_block", ctypes.c_int), ("blocks", ctypes.c_int),
                ("items", ctypes.c_int), ("tuned_from_cache", ctypes.c_int), ("tune_ms", ctypes.c_double),
                ("device_bytes", ctypes.c_size_t), ("temporal_depth", ctypes.c_int), ("tile_rows", ctypes.c_int),
                ("tile_cols", ctypes.c_int), ("tiles", ctypes.c_int)]


class ServerConfig(ctypes.Structure):
    _fields_ = [("hbm_budget_bytes", ctypes.c_size_t), ("chunk_steps", ctypes.c_int), ("max_active", ctypes.c_int)]


class RequestStatus(ctypes.Structure):
    _fields_ = [("state", ctypes.c_int), ("steps_total", ctypes.c_int), ("steps_done", ctypes.c_int64),
                ("submit_s", ctypes.c_double), ("admit_s", ctypes.c_double), ("finish_s", ctypes.c_double),
                ("mass", ctypes.c_double), ("energy", ctypes.c_double), ("message", ctypes.c_char * 160)]


class ServerStats(ctypes.Structure):
    _fields_ = [("submitted", ctypes.c_int64), ("admitted", ctypes.c_int64), ("completed", ctypes.c_int64),
                ("failed", ctypes.c_int64), ("cancelled", ctypes.c_int64), ("queued", ctypes.c_int),
                ("active", ctypes.c_int), ("device_bytes_in_use", ctypes.c_size_t),
                ("device_bytes_budget", ctypes.c_size_t), ("rounds", ctypes.c_int64)]


class GpuError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__("%s (%d)%s" % (strerror(code), code, (": " + msg) if msg else ""))
        self.code = code


_lib = None


def lib_path() -> str:
    return _build.LIB


def load(build_if_missing: bool = False):
    """Load libmmsp_gpu.so; raises if it is absent (no fallback)."""
    global _lib
    if _lib is not None:
        return _lib
    path = lib_path()
    if not os.path.exists(path):
        if not build_if_missing:
            raise ImportError("libmmsp_gpu.so is not built (%s); run __graft_entry__.build()" % path)
        _build.build()
    L = ctypes.CDLL(path)
    vp, sz, i = ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int
    dp = ctypes.POINTER(Desc)
    sig = {
        "mmsp_gpu_version": (i, []),
        "mmsp_gpu_strerror": (ctypes.c_char_p, [i]),
        "mmsp_gpu_desc_init": (i, [dp, i, ctypes.POINTER(ctypes.c_int), i, i, i]),
        "mmsp_gpu_validate": (i, [dp]),
        "mmsp_gpu_footprint": (i, [dp, ctypes.POINTER(ctypes.c_size_t)]),
        "mmsp_gpu_create": (i, [ctypes.POINTER(vp), dp]),
        "mmsp_gpu_destroy": (i, [vp]),
        "mmsp_gpu_set_stream": (i, [vp, vp]),
        "mmsp_gpu_upload": (i, [vp, vp, sz, i]),
        "mmsp_gpu_download": (i, [vp, vp, sz, i]),
        "mmsp_gpu_upload_device": (i, [vp, vp, sz, i]),
        "mmsp_gpu_download_device": (i, [vp, vp, sz, i]),
        "mmsp_gpu_step": (i, [vp, i]),
        "mmsp_gpu_synchronize": (i, [vp]),
        "mmsp_gpu_reduce": (i, [vp, ctypes.POINTER(Stats)]),
        "mmsp_gpu_state": (i, [vp, ctypes.POINTER(vp)]),
        "mmsp_gpu_last_error": (ctypes.c_char_p, [vp]),
        "mmsp_gpu_update": (i, [dp, vp, sz, i, i, ctypes.POINTER(Stats)]),
        "mmsp_gpu_step_noalloc": (i, [dp, vp, vp, i, vp]),
        "mmsp_gpu_fp64_rate": (i, [vp, vp]),
        "mmsp_gpu_sparse_upload": (i, [vp, vp, vp, vp]),
        "mmsp_gpu_sparse_download": (i, [vp, vp, vp, vp]),
        "mmsp_gpu_output_opts_init": (i, [ctypes.POINTER(OutputOpts)]),
        "mmsp_gpu_write_grid": (i, [ctypes.c_char_p, dp, vp, sz, i, ctypes.POINTER(OutputOpts)]),
        "mmsp_gpu_output": (i, [vp, ctypes.c_char_p, ctypes.POINTER(OutputOpts)]),
        "mmsp_gpu_output_wait": (i, [vp]),
        "mmsp_gpu_batch_create": (i, [ctypes.POINTER(vp), i, dp]),
        "mmsp_gpu_batch_destroy": (i, [vp]),
        "mmsp_gpu_batch_set_stream": (i, [vp, vp]),
        "mmsp_gpu_batch_upload": (i, [vp, i, vp, sz, i]),
        "mmsp_gpu_batch_download": (i, [vp, i, vp, sz, i]),
        "mmsp_gpu_batch_upload_all": (i, [vp, ctypes.POINTER(vp), i]),
        "mmsp_gpu_batch_download_all": (i, [vp, ctypes.POINTER(vp), i]),
        "mmsp_gpu_batch_step": (i, [vp, i]),
        "mmsp_gpu_batch_synchronize": (i, [vp]),
        "mmsp_gpu_batch_reduce": (i, [vp, i, ctypes.POINTER(Stats)]),
        "mmsp_gpu_batch_tune": (i, [vp, i]),
        "mmsp_gpu_batch_get_info": (i, [vp, ctypes.POINTER(BatchInfo)]),
        "mmsp_gpu_batch_last_error": (ctypes.c_char_p, [vp]),
        "mmsp_gpu_server_start": (i, [ctypes.POINTER(vp), ctypes.POINTER(ServerConfig)]),
        "mmsp_gpu_server_submit": (i, [vp, dp, vp, sz, i, i, ctypes.POINTER(ctypes.c_uint64)]),
        "mmsp_gpu_server_poll": (i, [vp, ctypes.c_uint64, ctypes.POINTER(RequestStatus)]),
        "mmsp_gpu_server_wait": (i, [vp, ctypes.c_uint64, ctypes.c_double, ctypes.POINTER(RequestStatus)]),
        "mmsp_gpu_server_fetch": (i, [vp, ctypes.c_uint64, vp, sz, i]),
        "mmsp_gpu_server_cancel": (i, [vp, ctypes.c_uint64]),
        "mmsp_gpu_server_get_stats": (i, [vp, ctypes.POINTER(ServerStats)]),
        "mmsp_gpu_server_stop": (i, [vp]),
    }
    for name, (res, args) in sig.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    _lib = L
    return L


def strerror(code: int) -> str:
    try:
        return load().mmsp_gpu_strerror(code).decode()
    except Exception:
        return "status"


def make_desc(shape, fields=1, dtype=np.float64, model="ch", dx=None, bc=None, dt=None, kappa=None,
              mobility=None, gamma=None, r=None, u=None, contract=False, **aux) -> Desc:
    """A descriptor with the model's defaults (mmsp_gpu_desc_init), then overrides.
    Ostwald-ripening parameters go by name (D, Calpha, Cbeta, A, delta, epsilon);
    the polynomial models take a thermal noise standard deviation and seed
    (noise, seed).  contract=True sets MMSP_GPU_FLAG_CONTRACT (FP64
    Cahn-Hilliard with fused multiply-adds, within 1e-12 of the reference)."""
    L = load()
    shape = tuple(int(s) for s in shape)
    d = Desc()
    n = (ctypes.c_int * 3)(*(list(shape) + [1] * (3 - len(shape))))
    m = MODELS[model] if isinstance(model, str) else int(model)
    # defaults only: mmsp_gpu_create validates the final descriptor
    L.mmsp_gpu_desc_init(ctypes.byref(d), len(shape), n, int(fields), DTYPES[np.dtype(dtype)], m)
    if dx is not None:
        for a, v in enumerate(dx):
            d.dx[a] = float(v)
    if bc is not None:
        for a, (lo, hi) in enumerate(bc):
            d.bc[a][0] = int(lo)
            d.bc[a][1] = int(hi)
    if contract:
        d.flags |= FLAG_CONTRACT
    for name, v in (("dt", dt), ("kappa", kappa), ("mobility", mobility), ("gamma", gamma), ("r", r), ("u", u)):
        if v is not None:
            setattr(d, name, float(v))
    names = OSTWALD_AUX if m == OSTWALD else CONVEX_AUX if m == CH_CONVEX else SPARSE_AUX if m == SPARSE_GG \
        else NOISE_AUX
    for name, v in aux.items():
        if name not in names:
            raise TypeError("unknown model parameter %r" % name)
        d.aux[names.index(name)] = float(v)
    return d


def _check(rc: int, h=None, what: str = ""):
    if rc != OK:
        msg = ""
        if h is not None:
            try:
                msg = load().mmsp_gpu_last_error(h).decode()
            except Exception:
                msg = ""
        raise GpuError(rc, (what + ": " + msg) if what else msg)


class Stepper:
    """A device-resident grid (one mmsp_gpu_handle)."""

    def __init__(self, desc: Desc):
        self.L = load()
        self.desc = desc
        h = ctypes.c_void_p()
        _check(self.L.mmsp_gpu_create(ctypes.byref(h), ctypes.byref(desc)), None, "create")
        self.h = h
        self.dtype = np.float64 if desc.dtype == F64 else np.float32
        self.shape = tuple(desc.n[a] for a in range(desc.dim))
        self.fields = desc.fields

    def close(self):
        if getattr(self, "h", None):
            self.L.mmsp_gpu_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _host_shape(self, layout):
        if self.fields == 1:
            return self.shape
        return self.shape + (self.fields,) if layout == CELL_MAJOR else (self.fields,) + self.shape

    def upload(self, arr: np.ndarray, layout: int = CELL_MAJOR):
        a = np.ascontiguousarray(arr, dtype=self.dtype)
        if a.shape != self._host_shape(layout):
            raise ValueError("shape %s, expected %s" % (a.shape, self._host_shape(layout)))
        _check(self.L.mmsp_gpu_upload(self.h, a.ctypes.data, a.nbytes, layout), self.h, "upload")

    def download(self, layout: int = CELL_MAJOR, out: np.ndarray | None = None) -> np.ndarray:
        if out is None:
            out = np.empty(self._host_shape(layout), dtype=self.dtype)
        _check(self.L.mmsp_gpu_download(self.h, out.ctypes.data, out.nbytes, layout), self.h, "download")
        return out

    def step(self, steps: int):
        _check(self.L.mmsp_gpu_step(self.h, int(steps)), self.h, "step")

    def synchronize(self):
        _check(self.L.mmsp_gpu_synchronize(self.h), self.h, "synchronize")

    def reduce(self) -> Stats:
        st = Stats()
        _check(self.L.mmsp_gpu_reduce(self.h, ctypes.byref(st)), self.h, "reduce")
        return st

    def set_stream(self, stream_ptr: int | None):
        _check(self.L.mmsp_gpu_set_stream(self.h, ctypes.c_void_p(stream_ptr or 0)), self.h, "set_stream")

    def state_ptr(self) -> int:
        p = ctypes.c_void_p()
        _check(self.L.mmsp_gpu_state(self.h, ctypes.byref(p)), self.h, "state")
        return p.value

    def output(self, filename: str, **opts):
        """mmsp_gpu_output: queue a snapshot of the state as an MMSP grid file."""
        o = output_opts(**opts)
        _check(self.L.mmsp_gpu_output(self.h, os.fsencode(filename), ctypes.byref(o)), self.h, "output")

    def output_wait(self):
        _check(self.L.mmsp_gpu_output_wait(self.h), self.h, "output_wait")

    def sparse_upload(self, count, index, value):
        """A sparse grid's lists (mmsp_gpu_sparse_upload): count has the grid's
        shape, index and value shape + (K,) with K = desc.fields."""
        K = self.fields
        c = np.ascontiguousarray(count, dtype=np.int32)
        ix = np.ascontiguousarray(index, dtype=np.int32)
        v = np.ascontiguousarray(value, dtype=np.float64)
        if c.shape != self.shape or ix.shape != self.shape + (K,) or v.shape != ix.shape:
            raise ValueError("sparse arrays of shape %s / %s, grid %s with %d slots" % (c.shape, ix.shape, self.shape, K))
        _check(self.L.mmsp_gpu_sparse_upload(self.h, c.ctypes.data, ix.ctypes.data, v.ctypes.data), self.h,
               "sparse_upload")

    def sparse_download(self):
        """(count, index, value) of a sparse grid (mmsp_gpu_sparse_download)."""
        K = self.fields
        c = np.empty(self.shape, np.int32)
        ix = np.empty(self.shape + (K,), np.int32)
        v = np.empty(self.shape + (K,), np.float64)
        _check(self.L.mmsp_gpu_sparse_download(self.h, c.ctypes.data, ix.ctypes.data, v.ctypes.data), self.h,
               "sparse_download")
        return c, ix, v

    def upload_device(self, ptr: int, nbytes: int, layout: int = FIELD_MAJOR):
        _check(self.L.mmsp_gpu_upload_device(self.h, ctypes.c_void_p(ptr), nbytes, layout), self.h, "upload_device")

    def download_device(self, ptr: int, nbytes: int, layout: int = FIELD_MAJOR):
        _check(self.L.mmsp_gpu_download_device(self.h, ctypes.c_void_p(ptr), nbytes, layout), self.h,
               "download_device")


def output_opts(level: int = 9, threads: int = 0, vector: int = -1, fields_line: int = -1, g0=None) -> OutputOpts:
    """mmsp_gpu_output_opts_init, then overrides."""
    o = OutputOpts()
    load().mmsp_gpu_output_opts_init(ctypes.byref(o))
    o.level, o.threads, o.vector, o.fields_line = int(level), int(threads), int(vector), int(fields_line)
    for a, v in enumerate(g0 or []):
        o.g0[a] = int(v)
    return o


def write_grid(filename: str, arr: np.ndarray, desc: Desc, layout: int = CELL_MAJOR, **opts):
    """mmsp_gpu_write_grid: host values as an MMSP grid file (no device needed)."""
    L = load()
    a = np.ascontiguousarray(arr)
    if a.dtype != (np.float64 if desc.dtype == F64 else np.float32):
        raise ValueError("array dtype does not match the descriptor")
    o = output_opts(**opts)
    _check(L.mmsp_gpu_write_grid(os.fsencode(filename), ctypes.byref(desc), a.ctypes.data_as(ctypes.c_void_p),
                                 a.nbytes, layout, ctypes.byref(o)), None, "write_grid")


def update(arr: np.ndarray, steps: int, desc: Desc, layout: int = CELL_MAJOR):
    """mmsp_gpu_update: one call per update(grid&, steps); returns (result, Stats)."""
    L = load()
    dt = np.float64 if desc.dtype == F64 else np.float32
    a = np.array(arr, dtype=dt, order="C", copy=True)
    st = Stats()
    rc = L.mmsp_gpu_update(ctypes.byref(desc), a.ctypes.data, a.nbytes, layout, int(steps), ctypes.byref(st))
    _check(rc, None, "update")
    return a, st


def _bcheck(rc: int, b=None, what: str = ""):
    if rc != OK:
        msg = ""
        if b is not None:
            try:
                msg = load().mmsp_gpu_batch_last_error(b).decode()
            except Exception:
                msg = ""
        raise GpuError(rc, (what + ": " + msg) if what else msg)


class Batch:
    """Many grids advanced together (mmsp_gpu_batch_*)."""

    def __init__(self, descs):
        self.L = load()
        arr = (Desc * len(descs))(*descs)
        b = ctypes.c_void_p()
        _bcheck(self.L.mmsp_gpu_batch_create(ctypes.byref(b), len(descs), arr), None, "batch_create")
        self.b = b
        self.descs = list(descs)
        self.dtype = np.float64 if descs[0].dtype == F64 else np.float32

    def close(self):
        if getattr(self, "b", None):
            self.L.mmsp_gpu_batch_destroy(self.b)
            self.b = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _shape(self, i):
        d = self.descs[i]
        s = tuple(d.n[a] for a in range(d.dim))
        return s if d.fields == 1 else s + (d.fields,)

    def upload(self, i: int, arr: np.ndarray):
        a = np.ascontiguousarray(arr, dtype=self.dtype)
        if a.shape != self._shape(i):
            raise ValueError("shape %s, expected %s" % (a.shape, self._shape(i)))
        _bcheck(self.L.mmsp_gpu_batch_upload(self.b, i, a.ctypes.data, a.nbytes, CELL_MAJOR), self.b, "upload")

    def download(self, i: int, out: np.ndarray = None) -> np.ndarray:
        """Grid i's state; into `out` (C-contiguous, the grid's shape and
        dtype, e.g. a view of pinned memory) when given."""
        if out is None:
            out = np.empty(self._shape(i), dtype=self.dtype)
        elif out.shape != self._shape(i) or out.dtype != self.dtype or not out.flags.c_contiguous:
            raise ValueError("out: expected a C-contiguous %s array of shape %s" % (self.dtype, self._shape(i)))
        _bcheck(self.L.mmsp_gpu_batch_download(self.b, i, out.ctypes.data, out.nbytes, CELL_MAJOR), self.b,
                "download")
        return out

    def upload_all(self, arrs):
        """Every grid's state in one call (one synchronisation)."""
        keep = []
        for i, arr in enumerate(arrs):
            a = np.ascontiguousarray(arr, dtype=self.dtype)
            if a.shape != self._shape(i):
                raise ValueError("grid %d: shape %s, expected %s" % (i, a.shape, self._shape(i)))
            keep.append(a)
        if len(keep) != len(self.descs):
            raise ValueError("expected %d arrays" % len(self.descs))
        ptrs = (ctypes.c_void_p * len(keep))(*[a.ctypes.data for a in keep])
        _bcheck(self.L.mmsp_gpu_batch_upload_all(self.b, ptrs, CELL_MAJOR), self.b, "upload_all")

    def download_all(self, outs=None):
        """Every grid's state in one call; into `outs` (C-contiguous arrays of
        each grid's shape and dtype) when given."""
        if outs is None:
            outs = [np.empty(self._shape(i), dtype=self.dtype) for i in range(len(self.descs))]
        if len(outs) != len(self.descs):
            raise ValueError("expected %d arrays" % len(self.descs))
        for i, o in enumerate(outs):
            if o.shape != self._shape(i) or o.dtype != self.dtype or not o.flags.c_contiguous:
                raise ValueError("grid %d: expected a C-contiguous %s array of shape %s" % (i, self.dtype, self._shape(i)))
        ptrs = (ctypes.c_void_p * len(outs))(*[o.ctypes.data for o in outs])
        _bcheck(self.L.mmsp_gpu_batch_download_all(self.b, ptrs, CELL_MAJOR), self.b, "download_all")
        return outs

    def step(self, steps: int):
        _bcheck(self.L.mmsp_gpu_batch_step(self.b, int(steps)), self.b, "step")

    def synchronize(self):
        _bcheck(self.L.mmsp_gpu_batch_synchronize(self.b), self.b, "synchronize")

    def reduce(self, i: int) -> Stats:
        st = Stats()
        _bcheck(self.L.mmsp_gpu_batch_reduce(self.b, i, ctypes.byref(st)), self.b, "reduce")
        return st

    def tune(self, force: bool = False):
        _bcheck(self.L.mmsp_gpu_batch_tune(self.b, 1 if force else 0), self.b, "tune")

    def set_stream(self, stream_ptr):
        _bcheck(self.L.mmsp_gpu_batch_set_stream(self.b, ctypes.c_void_p(stream_ptr or 0)), self.b, "set_stream")

    def info(self) -> BatchInfo:
        inf = BatchInfo()
        _bcheck(self.L.mmsp_gpu_batch_get_info(self.b, ctypes.byref(inf)), self.b, "info")
        return inf


class Server:
    """The request loop (mmsp_gpu_server_*)."""

    def __init__(self, budget_bytes: int = 0, chunk_steps: int = 0, max_active: int = 0):
        self.L = load()
        cfg = ServerConfig(budget_bytes, chunk_steps, max_active)
        s = ctypes.c_void_p()
        _check(self.L.mmsp_gpu_server_start(ctypes.byref(s), ctypes.byref(cfg)), None, "server_start")
        self.s = s
        self.shapes = {}

    def submit(self, desc: Desc, arr: np.ndarray, steps: int) -> int:
        dt = np.float64 if desc.dtype == F64 else np.float32
        a = np.ascontiguousarray(arr, dtype=dt)
        rid = ctypes.c_uint64()
        _check(self.L.mmsp_gpu_server_submit(self.s, ctypes.byref(desc), a.ctypes.data, a.nbytes, CELL_MAJOR,
                                             int(steps), ctypes.byref(rid)), None, "submit")
        self.shapes[rid.value] = (a.shape, dt)
        return rid.value

    def poll(self, rid: int) -> RequestStatus:
        st = RequestStatus()
        _check(self.L.mmsp_gpu_server_poll(self.s, rid, ctypes.byref(st)), None, "poll")
        return st

    def wait(self, rid: int, timeout: float = 600.0) -> RequestStatus:
        st = RequestStatus()
        rc = self.L.mmsp_gpu_server_wait(self.s, rid, float(timeout), ctypes.byref(st))
        if rc not in (OK, ETIMEDOUT):
            _check(rc, None, "wait")
        return st

    def fetch(self, rid: int) -> np.ndarray:
        shape, dt = self.shapes[rid]
        out = np.empty(shape, dtype=dt)
        _check(self.L.mmsp_gpu_server_fetch(self.s, rid, out.ctypes.data, out.nbytes, CELL_MAJOR), None, "fetch")
        del self.shapes[rid]
        return out

    def cancel(self, rid: int):
        _check(self.L.mmsp_gpu_server_cancel(self.s, rid), None, "cancel")

    def stats(self) -> ServerStats:
        st = ServerStats()
        _check(self.L.mmsp_gpu_server_get_stats(self.s, ctypes.byref(st)), None, "stats")
        return st

    def stop(self):
        if getattr(self, "s", None):
            self.L.mmsp_gpu_server_stop(self.s)
            self.s = None

    def __del__(self):
        try:
            self.stop()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.stop()


def fp64_rate(stream: int = 0) -> float:
    """FP64 operations per second of the current device (mmsp_gpu_fp64_rate)."""
    v = ctypes.c_double()
    _check(load().mmsp_gpu_fp64_rate(ctypes.c_void_p(stream), ctypes.byref(v)), None, "fp64_rate")
    return v.value
