"""MMSP grid file format: reader and writer.

The byte layout is the reference's, so files written here are read by the
reference's ``grid::input`` (and hence by ``mmsp2png`` / ``mmsp2tsv``), and
files written by the reference are read here:

* ASCII header (``grid::output``, include/MMSP.grid.cpp:1370-1399):
  ``grid:<type>\\n``, ``dim\\n``, ``fields\\n``, ``g0 g1\\n`` per axis and
  ``dx\\n`` per axis in C++ ostream default formatting (``%g``).
  Type names: include/MMSP.grid.h:593-596, include/MMSP.utility.h:208-213,
  include/MMSP.vector.h:115-117.
* ``int32 nblocks`` then, per block (``grid::write_buffer``,
  include/MMSP.grid.cpp:1818-1909): ``int32 x0,x1`` per axis, ``int32 b0,b1``
  per axis, ``uint64 size_in_mem``, ``uint64 size_on_disk`` and a zlib
  ``compress2`` level-9 payload (raw when the two sizes are equal).
* Payload (``to_buffer``, include/MMSP.grid.cpp:1146-1157): cells with the
  last index fastest; a scalar cell is one ``T``; a ``vector<T>`` cell is
  ``int32 N`` followed by ``N`` values (include/MMSP.vector.cpp:95-117).

Reading follows ``grid::read`` (include/MMSP.grid.cpp:1248-1356): every block
is copied into its own region of the global grid, and the block's boundary
conditions replace the defaults on the faces it touches.
"""
from __future__ import annotations

import struct
import zlib
from dataclasses import dataclass, field

import numpy as np

# Boundary-condition codes, include/MMSP.utility.h:23-29.
MIRROR, NEUMANN, PERIODIC, PARALLEL, DIRICHLET = 0, 1, 2, 3, 4

_SCALAR_NAMES = {
    np.dtype(np.float64): "double",
    np.dtype(np.float32): "float",
    np.dtype(np.int32): "int",
    np.dtype(np.int64): "long",
    np.dtype(np.int16): "short",
    np.dtype(np.int8): "char",
    np.dtype(np.uint8): "unsigned char",
    np.dtype(np.uint32): "unsigned int",
    np.dtype(np.uint64): "unsigned long",
    np.dtype(np.uint16): "unsigned short",
}
_NAME_TO_DTYPE = {v: k for k, v in _SCALAR_NAMES.items()}


class GridFileError(ValueError):
    """A grid file that cannot be read (the reference exits with -1..-3)."""


@dataclass
class GridData:
    """A grid as stored in a file: global extents, spacing, BCs and values.

    ``data`` has shape ``(n0, ..., n_{dim-1})`` for scalar grids and
    ``(n0, ..., n_{dim-1}, N)`` for ``vector<T>`` grids (cell-major values).
    """

    dim: int
    g0: list
    g1: list
    dx: list
    data: np.ndarray
    vector: bool = False
    fields: int = 0
    b0: list = field(default_factory=list)
    b1: list = field(default_factory=list)

    def __post_init__(self):
        if not self.b0:
            self.b0 = [PERIODIC] * self.dim
        if not self.b1:
            self.b1 = [PERIODIC] * self.dim

    @property
    def shape(self):
        return tuple(int(b - a) for a, b in zip(self.g0, self.g1))

    @property
    def type_name(self) -> str:
        base = _SCALAR_NAMES[np.dtype(self.data.dtype)]
        return ("grid:vector:" if self.vector else "grid:") + base


def _fmt_g(x: float) -> str:
    """C++ ``ostream << double`` with default flags (precision 6, %g)."""
    return "%g" % x


def header_bytes(g: GridData) -> bytes:
    lines = [g.type_name, str(g.dim), str(g.fields)]
    lines += ["%d %d" % (a, b) for a, b in zip(g.g0, g.g1)]
    lines += [_fmt_g(d) for d in g.dx]
    return ("\n".join(lines) + "\n").encode("ascii")


def payload_bytes(g: GridData) -> bytes:
    """``to_buffer`` of the whole grid (last index fastest)."""
    arr = np.ascontiguousarray(g.data)
    if not g.vector:
        return arr.astype(arr.dtype.newbyteorder("<"), copy=False).tobytes()
    n = arr.shape[-1]
    cells = arr.reshape(-1, n)
    rec = np.dtype([("n", "<i4"), ("v", arr.dtype.newbyteorder("<"), (n,))])
    out = np.empty(cells.shape[0], dtype=rec)
    out["n"] = n
    out["v"] = cells
    return out.tobytes()


def write(filename: str, g: GridData, level: int = 9, raw: bool = False) -> None:
    """``grid::output`` (serial, include/MMSP.grid.cpp:1358-1402)."""
    raw_payload = payload_bytes(g)
    body = raw_payload if raw else zlib.compress(raw_payload, level)
    blk = bytearray()
    for a, b in zip(g.g0, g.g1):
        blk += struct.pack("<ii", int(a), int(b))
    for a, b in zip(g.b0, g.b1):
        blk += struct.pack("<ii", int(a), int(b))
    blk += struct.pack("<QQ", len(raw_payload), len(body))
    with open(filename, "wb") as f:
        f.write(header_bytes(g))
        f.write(struct.pack("<i", 1))
        f.write(bytes(blk))
        f.write(body)


def _readline(buf: bytes, pos: int):
    end = buf.index(b"\n", pos)
    return buf[pos:end].decode("ascii"), end + 1


def read(filename: str, expect_type: str | None = None, expect_dim: int | None = None) -> GridData:
    """``grid::input`` + ``grid::read`` for a serial reader."""
    try:
        with open(filename, "rb") as f:
            buf = f.read()
    except OSError as e:
        raise GridFileError("File input error: could not open %s." % filename) from e
    try:
        pos = 0
        type_name, pos = _readline(buf, pos)
        dim_s, pos = _readline(buf, pos)
        fields_s, pos = _readline(buf, pos)
        dim = int(dim_s)
        fields_n = int(fields_s)
        if dim < 1 or dim > 3:
            raise GridFileError("File read error: wrong dimension (%d)." % dim)
        g0, g1, dx = [], [], []
        for _ in range(dim):
            s, pos = _readline(buf, pos)
            a, b = s.split()
            g0.append(int(a))
            g1.append(int(b))
        for _ in range(dim):
            s, pos = _readline(buf, pos)
            dx.append(float(s))
    except (ValueError, IndexError) as e:
        if isinstance(e, GridFileError):
            raise
        raise GridFileError("File read error: malformed header in %s." % filename) from e
    if expect_type is not None and type_name != expect_type:
        raise GridFileError("File read error: wrong data type (%s), expected (%s)." % (type_name, expect_type))
    if expect_dim is not None and dim != expect_dim:
        raise GridFileError("File read error: wrong dimension (%d)." % dim)
    if type_name.startswith("grid:vector:"):
        vector, base = True, type_name[len("grid:vector:"):]
    elif type_name.startswith("grid:scalar:"):
        vector, base = False, type_name[len("grid:scalar:"):]
    elif type_name.startswith("grid:"):
        vector, base = False, type_name[len("grid:"):]
    else:
        raise GridFileError("File read error: wrong data type (%s)." % type_name)
    if base not in _NAME_TO_DTYPE:
        raise GridFileError("File read error: unsupported data type (%s)." % type_name)
    dt = _NAME_TO_DTYPE[base].newbyteorder("<")
    shape = tuple(b - a for a, b in zip(g0, g1))
    if any(s <= 0 for s in shape):
        raise GridFileError("File read error: empty extent in %s." % filename)

    data = None
    b0 = [PERIODIC] * dim
    b1 = [PERIODIC] * dim

    def need(n):
        if pos + n > len(buf):
            raise GridFileError("File read error: truncated file %s." % filename)

    need(4)
    (blocks,) = struct.unpack_from("<i", buf, pos)
    pos += 4
    if blocks < 1:
        raise GridFileError("File read error: no data blocks in %s." % filename)
    for _ in range(blocks):
        need(16 * dim + 16)
        lim = struct.unpack_from("<%di" % (2 * dim), buf, pos)
        pos += 8 * dim
        bcs = struct.unpack_from("<%di" % (2 * dim), buf, pos)
        pos += 8 * dim
        size_in_mem, size_on_disk = struct.unpack_from("<QQ", buf, pos)
        pos += 16
        need(size_on_disk)
        body = buf[pos:pos + size_on_disk]
        pos += size_on_disk
        if size_in_mem != size_on_disk:
            try:
                body = zlib.decompress(body)
            except zlib.error as e:
                raise GridFileError("Uncompress: corrupt data in %s." % filename) from e
        if len(body) != size_in_mem:
            raise GridFileError("Uncompress: size mismatch in %s." % filename)
        lmin = [lim[2 * j] for j in range(dim)]
        lmax = [lim[2 * j + 1] for j in range(dim)]
        bshape = tuple(b - a for a, b in zip(lmin, lmax))
        ncell = int(np.prod(bshape))
        if vector:
            if ncell == 0:
                continue
            (n,) = struct.unpack_from("<i", body, 0)
            if n < 0 or len(body) != ncell * (4 + n * dt.itemsize):
                raise GridFileError("File read error: inconsistent vector block in %s." % filename)
            rec = np.dtype([("n", "<i4"), ("v", dt, (n,))])
            cells = np.frombuffer(body, dtype=rec, count=ncell)
            if np.any(cells["n"] != n):
                raise GridFileError("File read error: ragged vector cells in %s." % filename)
            blockdata = cells["v"].reshape(bshape + (n,)).astype(dt.newbyteorder("="))
            if data is None:
                data = np.zeros(shape + (n,), dtype=blockdata.dtype)
        else:
            if len(body) != ncell * dt.itemsize:
                raise GridFileError("File read error: inconsistent block size in %s." % filename)
            blockdata = np.frombuffer(body, dtype=dt, count=ncell).reshape(bshape).astype(dt.newbyteorder("="))
            if data is None:
                data = np.zeros(shape, dtype=blockdata.dtype)
        sl = tuple(slice(a - o, b - o) for a, b, o in zip(lmin, lmax, g0))
        data[sl] = blockdata
        for j in range(dim):
            if lmin[j] == g0[j]:
                b0[j] = bcs[2 * j]
            if lmax[j] == g1[j]:
                b1[j] = bcs[2 * j + 1]
    if data is None:
        raise GridFileError("File read error: no cells in %s." % filename)
    return GridData(dim=dim, g0=g0, g1=g1, dx=dx, data=data, vector=vector,
                    fields=fields_n, b0=b0, b1=b1)
