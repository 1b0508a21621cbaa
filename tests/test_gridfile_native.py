"""The native grid-file writer (mmsp_gpu_write_grid), on the CPU.

The files must be the reference's grid::output of a serial run: same header
and block layout, the payload in to_buffer order, compressed by one
compress2 call at level 9 when it is at most 1 MiB (then byte-identical to
what the reference writes) and as one chunked zlib stream above that.  Where
the reference program is built (oracle/_ref/ref_update, the reference's own
grid::input and grid::output), it reads each file back and writes it again
after 0 steps.
"""
import os
import struct
import subprocess
import zlib

import numpy as np
import pytest

from mmsp_gb300 import gridfile, native
from oracle import pf_oracle

CHUNK = 1 << 20


def desc(shape, fields, dtype, dx=None):
    return native.make_desc(shape, fields, dtype, "ch" if fields == 1 else "ac", dx=dx)


def python_file(path, x, dx, vector, fields):
    dim = x.ndim - (1 if vector else 0)
    g = gridfile.GridData(dim=dim, g0=[0] * dim, g1=list(x.shape[:dim]), dx=list(dx), data=x, vector=vector,
                          fields=fields)
    gridfile.write(str(path), g)
    return path.read_bytes()


def block(path, dim):
    """(header text, size_in_mem, size_on_disk, body) of a one-block file."""
    b = path.read_bytes()
    pos = 0
    for _ in range(3 + 2 * dim):
        pos = b.index(b"\n", pos) + 1
    head = b[:pos]
    nblocks, = struct.unpack_from("<i", b, pos)
    assert nblocks == 1
    pos += 4 + 16 * dim
    mem, disk = struct.unpack_from("<QQ", b, pos)
    return head, mem, disk, b[pos + 16:]


def test_small_scalar_is_byte_identical_to_compress2(tmp_path):
    x = np.random.default_rng(1).random((17, 23))
    native.write_grid(str(tmp_path / "n.dat"), x, desc(x.shape, 1, np.float64, dx=[1.0, 0.5]))
    want = python_file(tmp_path / "p.dat", x, [1.0, 0.5], False, 0)
    assert (tmp_path / "n.dat").read_bytes() == want
    head, mem, disk, body = block(tmp_path / "n.dat", 2)
    assert head == b"grid:double\n2\n0\n0 17\n0 23\n1\n0.5\n"
    assert mem == x.nbytes and disk == len(body) and zlib.decompress(body) == x.tobytes()


@pytest.mark.parametrize("layout", [native.CELL_MAJOR, native.FIELD_MAJOR])
def test_vector_cells_in_both_layouts(tmp_path, layout):
    x = np.random.default_rng(2).random((9, 7, 5, 4)).astype(np.float32)   # cell-major values
    host = x if layout == native.CELL_MAJOR else np.ascontiguousarray(np.moveaxis(x, -1, 0))
    native.write_grid(str(tmp_path / "n.dat"), host, desc(x.shape[:3], 4, np.float32), layout)
    g = gridfile.read(str(tmp_path / "n.dat"))
    assert g.vector and g.fields == 4 and g.type_name == "grid:vector:float"
    assert np.array_equal(g.data, x)
    assert (tmp_path / "n.dat").read_bytes() == python_file(tmp_path / "p.dat", x, [1.0] * 3, True, 4)


def test_large_payload_is_one_chunked_stream_independent_of_threads(tmp_path):
    x = np.random.default_rng(3).random((40, 64, 64))    # 1.31 MB: two pieces
    d = desc(x.shape, 1, np.float64)
    native.write_grid(str(tmp_path / "t1.dat"), x, d, threads=1)
    native.write_grid(str(tmp_path / "t8.dat"), x, d, threads=8)
    assert (tmp_path / "t1.dat").read_bytes() == (tmp_path / "t8.dat").read_bytes()
    _, mem, disk, body = block(tmp_path / "t1.dat", 3)
    assert mem == x.nbytes > CHUNK and disk == len(body)
    assert body[:2] == b"\x78\xda" and zlib.decompress(body) == x.tobytes()
    assert np.array_equal(gridfile.read(str(tmp_path / "t1.dat")).data, x)


def test_levels_on_a_constant_field(tmp_path):
    z = np.full((64, 64, 64), 0.25, dtype=np.float32)    # 1 MiB: one compress2 call
    d = desc(z.shape, 1, np.float32)
    for lv, head in ((1, b"\x78\x01"), (5, b"\x78\x5e"), (6, b"\x78\x9c"), (9, b"\x78\xda")):
        p = tmp_path / ("l%d.dat" % lv)
        native.write_grid(str(p), z, d, level=lv)
        _, mem, disk, body = block(p, 3)
        assert body[:2] == head and zlib.decompress(body) == z.tobytes() and disk < mem // 50
    big = np.full((80, 64, 64), 0.25, dtype=np.float32)  # 1.25 MiB: chunked stream, same header rule
    for lv, head in ((1, b"\x78\x01"), (5, b"\x78\x5e"), (6, b"\x78\x9c")):
        p = tmp_path / ("b%d.dat" % lv)
        native.write_grid(str(p), big, desc(big.shape, 1, np.float32), level=lv)
        _, mem, disk, body = block(p, 3)
        assert body[:2] == head and zlib.decompress(body) == big.tobytes()


def test_level_zero_writes_the_raw_form(tmp_path):
    x = np.random.default_rng(4).random((5, 6)).astype(np.float32)
    native.write_grid(str(tmp_path / "r.dat"), x, desc(x.shape, 1, np.float32), level=0)
    _, mem, disk, body = block(tmp_path / "r.dat", 2)
    assert mem == disk == x.nbytes and body == x.tobytes()
    assert np.array_equal(gridfile.read(str(tmp_path / "r.dat")).data, x)


def test_options_and_errors(tmp_path):
    x = np.zeros((4, 4, 4, 2))
    d = desc((4, 4, 4), 2, np.float64)
    native.write_grid(str(tmp_path / "g.dat"), x, d, g0=[10, -4, 0], fields_line=7)
    head, _, _, _ = block(tmp_path / "g.dat", 3)
    assert head == b"grid:vector:double\n3\n7\n10 14\n-4 0\n0 4\n1\n1\n1\n"
    with pytest.raises(native.GpuError) as e:
        native.write_grid(str(tmp_path / "no_such_dir" / "x.dat"), x, d)
    assert e.value.code == native.EIO
    with pytest.raises(native.GpuError) as e:
        native.write_grid(str(tmp_path / "v.dat"), x, d, vector=0)    # two values per cell in a scalar file
    assert e.value.code == native.EINVAL
    with pytest.raises(native.GpuError) as e:
        native.write_grid(str(tmp_path / "s.dat"), x[..., :1], d)     # wrong size
    assert e.value.code == native.EINVAL
    with pytest.raises(native.GpuError) as e:
        native.write_grid(str(tmp_path / "l.dat"), x, d, level=10)
    assert e.value.code == native.EINVAL


REF = pf_oracle.REF_BIN
CASES = [("scalar_small", (24, 31), 0), ("scalar_chunked", (48, 64, 64), 0),
         ("vector_small", (6, 7, 9), 3), ("vector_chunked", (40, 40, 40), 3)]


@pytest.mark.skipif(not os.path.exists(REF), reason="reference program not built in this checkout")
@pytest.mark.parametrize("case,shape,fields", CASES, ids=[c[0] for c in CASES])
def test_reference_reads_native_files(tmp_path, case, shape, fields):
    rng = np.random.default_rng(5)
    x = rng.random(shape + ((fields,) if fields else ()))
    d = desc(shape, max(fields, 1), np.float64, dx=[0.5] * len(shape))
    fin, fout = tmp_path / "in.dat", tmp_path / "out.dat"
    native.write_grid(str(fin), x, d)
    model, params = ("graingrowth", ["0.01"]) if fields else ("ch_baseline", ["1.0", "1.0", "0.01"])
    subprocess.run([REF, model, str(fin), str(fout), "0"] + params, check=True, capture_output=True)
    _, mem, _, _ = block(fin, len(shape))
    if mem <= CHUNK:
        assert fout.read_bytes() == fin.read_bytes()   # the reference writes the same bytes
    else:
        hi, mi, _, bi = block(fin, len(shape))
        ho, mo, _, bo = block(fout, len(shape))
        assert hi == ho and mi == mo and zlib.decompress(bi) == zlib.decompress(bo)
    g = gridfile.read(str(fout))
    assert np.array_equal(g.data, x)
