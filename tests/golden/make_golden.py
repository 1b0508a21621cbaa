"""Generate the golden vectors in tests/golden/ from the reference itself.

Run in a container that holds the reference source (its headers are compiled
by ``make -C oracle ref`` into ``oracle/_ref/ref_update``):

    python tests/golden/make_golden.py            # small fixtures (*.npz)
    python tests/golden/make_golden.py --full     # + full-size checksums

Small fixtures: seeded start states are written as MMSP grid files with
``mmsp_gb300.gridfile``, advanced by the reference's own ``grid``,
``laplacian`` and ``swap`` (ref_update.cpp), and the reference's output file
is read back.  Each ``.npz`` holds the start state, the reference's result,
the model, its parameters and the step count.

Sparse fixtures (``sparse*.npz``): sparse phase-field grain growth through
the reference's own ``grid<dim,sparse<double>>``, ``laplacian`` and ``swap``
(ref_update's sparsepf mode, fed a plain list file); the C oracle is checked
against each before it is saved.

Full-size checksums (``full_size.json``): 2D CH 256x256 x 2000 steps is run
through the reference itself; the 3D configurations (256^3 CH, 128^3 x 8 AC)
would take hours through the reference's per-cell allocations, so they are
run through the C oracle, which the small fixtures pin bit for bit to the
reference.  Each entry stores the SHA-256 of the final float64 array (node
order, little-endian), mass/energy and a strided sample.
"""
import argparse
import hashlib
import json
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from mmsp_gb300 import gridfile, inputs  # noqa: E402
from oracle import pf_oracle  # noqa: E402

# (name, model, shape, fields, start, params, steps, extra)
SMALL = [
    ("ch2d_baseline", "ch_baseline", (40, 56), 0, ("noise", 0.5, 0.01, 11), (1.0, 1.0, 0.005), 200, {}),
    ("ch3d_baseline", "ch_baseline", (12, 16, 20), 0, ("noise", 0.4, 0.02, 12), (1.0, 1.0, 0.002), 60, {}),
    ("ch1d_baseline", "ch_baseline", (64,), 0, ("noise", 0.5, 0.05, 13), (1.0, 1.0, 0.005), 300, {}),
    ("ch2d_baseline_dx", "ch_baseline", (24, 36), 0, ("noise", 0.5, 0.01, 14), (0.7, 1.3, 0.001), 100,
     {"dx": [0.5, 2.0]}),
    ("ch2d_baseline_neumann", "ch_baseline", (20, 28), 0, ("noise", 0.5, 0.02, 15), (1.0, 1.0, 0.005), 80,
     {"bc": [[1, 1], [4, 0]]}),
    ("ch2d_shipped", "ch_shipped", (32, 24), 0, ("noise", 0.0, 1.0, 16), (1.0, 1.0, 1.0, 1.0, 0.01), 50, {}),
    ("ch3d_shipped", "ch_shipped", (10, 8, 12), 0, ("noise", 0.0, 1.0, 17), (1.0, 1.0, 1.0, 1.0, 0.01), 20, {}),
    ("ac_scalar2d_shipped", "ac_scalar", (32, 32), 0, ("noise", 0.0, 1.0, 18), (1.0, 1.0, 1.0, 1.0, 0.01), 50, {}),
    ("ac3d_baseline", "ac_baseline", (10, 12, 14), 8, ("voronoi", 20, 19), (1.5, 2.0, 1.0, 0.05), 30, {}),
    ("ac2d_baseline", "ac_baseline", (24, 20), 4, ("voronoi", 12, 20), (1.5, 2.0, 1.0, 0.05), 40, {}),
    ("ac3d_baseline_n3", "ac_baseline", (8, 9, 10), 3, ("voronoi", 9, 21), (1.2, 1.5, 0.8, 0.04), 25, {}),
    ("gg2d_shipped", "graingrowth", (64, 64), 2, ("circles",), (0.01,), 100, {}),
    ("gg3d_shipped", "graingrowth", (36, 36, 4), 2, ("circles",), (0.01,), 40, {}),
    ("zener2d_shipped", "zener", (64, 64), 3, ("zener", 40, 22), (0.01,), 100, {}),
    ("zener3d_shipped", "zener", (24, 24, 12), 3, ("zener", 30, 23), (0.01,), 40, {}),
    ("ostwald2d_shipped", "ostwald", (64, 32), 2, ("ostwald", 24), (0.001, 1.0, 1.0, 0.05, 0.95, 2.0, 1.0, 3.0, 2.0), 60, {}),
    ("ostwald3d_shipped", "ostwald", (16, 12, 8), 4, ("ostwald", 25), (0.001, 1.0, 1.0, 0.05, 0.95, 2.0, 1.0, 3.0, 2.0), 40, {}),
    ("convex2d_shipped", "ch_convex", (40, 20), 2, ("convex", None), (0.225, 2.0 / 0.9, 2.0, 0.45, 0.05, 0.95, 2.0, 1.2, 1e-14), 4, {}),
    ("convex3d_shipped", "ch_convex", (12, 10, 8), 2, ("convex", 31), (0.225, 2.0 / 0.9, 2.0, 0.45, 0.05, 0.95, 2.0, 1.2, 1e-14), 3, {}),
]


def start_state(shape, fields, spec):
    kind = spec[0]
    if kind == "noise":
        _, mean, amp, seed = spec
        return inputs.noisy_composition(shape, mean, amp, seed)
    if kind == "voronoi":
        _, pts, seed = spec
        return inputs.voronoi_grains(shape, pts, fields, seed)
    if kind == "circles":
        return inputs.graingrowth_circles(shape, fields)
    if kind == "zener":
        _, particles, seed = spec
        return inputs.zener_particles(shape, particles, seed)
    if kind == "ostwald":
        return inputs.ostwald_start(shape, fields, spec[1])
    if kind == "convex":
        return inputs.convex_start(shape, spec[1])
    raise ValueError(kind)


def run_ref(model, data, vector, fields, steps, params, dx=None, bc=None, want_stdout=False):
    dim = data.ndim - (1 if vector else 0)
    shape = data.shape[:dim]
    g = gridfile.GridData(dim=dim, g0=[0] * dim, g1=list(shape),
                          dx=list(dx) if dx else [1.0] * dim, data=data,
                          vector=vector, fields=fields,
                          b0=[b[0] for b in bc] if bc else [],
                          b1=[b[1] for b in bc] if bc else [])
    with tempfile.TemporaryDirectory() as td:
        fin = os.path.join(td, "in.dat")
        fout = os.path.join(td, "out.dat")
        gridfile.write(fin, g)
        res = subprocess.run([pf_oracle.REF_BIN, model, fin, fout, str(steps)] + [repr(float(p)) for p in params],
                             check=True, capture_output=True, text=True)
        secs = float(res.stdout.split()[-1])
        out = gridfile.read(fout)
    if want_stdout:
        return out.data, secs, res.stdout
    return out.data, secs


# sparse phase-field grain growth: (name, shape, start, steps); dt 0.01, epsilon 1e-8 as shipped
SPARSE = [
    ("sparse2d_grains", (48, 40), ("grains", 12, 3), 150),
    ("sparse3d_grains", (16, 12, 10), ("grains", 8, 4), 40),
    ("sparse2d_circles", (128, 64), ("circles",), 200),
    ("sparse3d_circles", (64, 32, 4), ("circles",), 40),
]
SPARSE_CAPACITY = 32


def write_sparse(path, cnt, idx, val):
    """The plain list file ref_update's sparsepf mode reads: int32 dim, int32
    extents, then per cell int32 count and count x (int32 index, float64 value)."""
    with open(path, "wb") as f:
        f.write(np.int32(cnt.ndim).tobytes())
        f.write(np.asarray(cnt.shape, np.int32).tobytes())
        c = cnt.ravel()
        ii = idx.reshape(c.size, -1)
        vv = val.reshape(c.size, -1)
        for k in range(c.size):
            f.write(np.int32(c[k]).tobytes())
            for h in range(c[k]):
                f.write(np.int32(ii[k, h]).tobytes())
                f.write(np.float64(vv[k, h]).tobytes())


def read_sparse(path, capacity):
    b = open(path, "rb").read()
    dim = int(np.frombuffer(b, np.int32, 1, 0)[0])
    shape = tuple(int(v) for v in np.frombuffer(b, np.int32, dim, 4))
    p = 4 + 4 * dim
    n = int(np.prod(shape))
    cnt = np.zeros(n, np.int32)
    idx = np.zeros((n, capacity), np.int32)
    val = np.zeros((n, capacity), np.float64)
    item = np.dtype([("i", "<i4"), ("v", "<f8")])
    for k in range(n):
        c = int(np.frombuffer(b, np.int32, 1, p)[0])
        p += 4
        if c > capacity:
            raise OverflowError("list of %d items" % c)
        it = np.frombuffer(b, item, c, p)
        p += 12 * c
        cnt[k] = c
        idx[k, :c] = it["i"]
        val[k, :c] = it["v"]
    return cnt.reshape(shape), idx.reshape(shape + (capacity,)), val.reshape(shape + (capacity,))


def make_sparse(only=None):
    """Sparse fixtures: the reference's sparse update (ref_update sparsepf) on
    grid<dim,sparse<double>>; the C oracle must agree bit for bit."""
    for name, shape, spec, steps in SPARSE:
        if only and name not in only:
            continue
        if spec[0] == "grains":
            c0, i0, v0 = inputs.sparse_grains(shape, spec[1], spec[2], SPARSE_CAPACITY)
        else:
            c0, i0, v0 = inputs.sparse_circles(shape, SPARSE_CAPACITY)
        with tempfile.TemporaryDirectory() as td:
            fin, fout = os.path.join(td, "in.bin"), os.path.join(td, "out.bin")
            write_sparse(fin, c0, i0, v0)
            res = subprocess.run([pf_oracle.REF_BIN, "sparsepf", fin, fout, str(steps), "0.01", "1e-08"],
                                 check=True, capture_output=True, text=True)
            cr, ir, vr = read_sparse(fout, SPARSE_CAPACITY)
        co, io, vo, longest = pf_oracle.sparse_gg(c0, i0, v0, steps, 0.01, 1e-8)
        assert np.array_equal(cr, co) and np.array_equal(ir, io) and np.array_equal(vr, vo), name
        k = max(int(cr.max()), int(c0.max()))   # slots in use
        np.savez_compressed(os.path.join(HERE, name + ".npz"), model="sparsepf", steps=steps,
                            params=np.asarray([0.01, 1e-8]), start_count=c0, start_index=i0[..., :k],
                            start_value=v0[..., :k], count=cr, index=ir[..., :k], value=vr[..., :k])
        print("%-24s %s steps=%d longest list %d, ref %s" % (name, shape, steps, longest, res.stdout.split()[-1]))


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a, dtype="<f8").tobytes()).hexdigest()


def make_small(only=None):
    for name, model, shape, fields, spec, params, steps, extra in SMALL:
        if only and name not in only:
            continue
        x0 = start_state(shape, fields, spec)
        vector = fields > 0
        out, secs, text = run_ref(model, x0, vector, fields, steps, params, extra.get("dx"), extra.get("bc"),
                                  want_stdout=True)
        more = {}
        if "iterations" in text:   # the implicit solve reports the last step's iterations
            more["iterations"] = int(text.split("iterations")[1].split()[0])
        np.savez_compressed(os.path.join(HERE, name + ".npz"), start=x0, result=out, model=model,
                            params=np.asarray(params, dtype=np.float64), steps=steps,
                            dx=np.asarray(extra.get("dx", [1.0] * len(shape))),
                            bc=np.asarray(extra.get("bc", [[2, 2]] * len(shape))), **more)
        print("%-24s %s steps=%d ref %.3fs" % (name, shape, steps, secs))


def make_full():
    out = {}
    # configuration 1: 2D CH 256^2 float64, 2000 steps, through the reference itself
    c0 = inputs.noisy_composition((256, 256), 0.5, 0.01, 1)
    t = time.time()
    ref, secs = run_ref("ch_baseline", c0, False, 0, 2000, (1.0, 1.0, 0.005))
    port = pf_oracle.ch_baseline(c0, 2000, 1.0, 1.0, 0.005)
    assert np.array_equal(ref, port), "C oracle differs from the reference on 2D CH 256^2"
    m, e = pf_oracle.ch_mass_energy(ref, 1.0)
    m0, e0 = pf_oracle.ch_mass_energy(c0, 1.0)
    out["ch2d_256_2000"] = dict(shape=[256, 256], seed=1, mean=0.5, amplitude=0.01, kappa=1.0, M=1.0,
                                dt=0.005, steps=2000, source="reference", ref_update_seconds=secs,
                                sha256=sha(ref), mass0=m0, energy0=e0, mass=m, energy=e,
                                sample_stride=97, sample=ref.ravel()[::97][:64].tolist())
    print("ch2d_256_2000 ref %.1fs (total %.1fs)" % (secs, time.time() - t))
    # configuration 2: 3D CH 256^3 float64, 1000 steps, through the pinned C oracle
    c0 = inputs.noisy_composition((256, 256, 256), 0.4, 0.02, 2)
    t = time.time()
    res = pf_oracle.ch_baseline(c0, 1000, 1.0, 1.0, 0.002)
    dt_s = time.time() - t
    m0, e0 = pf_oracle.ch_mass_energy(c0, 1.0)
    m, e = pf_oracle.ch_mass_energy(res, 1.0)
    out["ch3d_256_1000"] = dict(shape=[256, 256, 256], seed=2, mean=0.4, amplitude=0.02, kappa=1.0, M=1.0,
                                dt=0.002, steps=1000, source="oracle", oracle_seconds=dt_s,
                                sha256=sha(res), mass0=m0, energy0=e0, mass=m, energy=e,
                                sample_stride=1000003, sample=res.ravel()[::1000003].tolist())
    print("ch3d_256_1000 oracle %.1fs" % dt_s)
    # configuration 3: 3D AC 128^3 x 8, Voronoi 200 seeds; dt=0.05 (stable) and dt=0.1 (as stated)
    e0 = inputs.voronoi_grains((128, 128, 128), 200, 8, 3)
    t = time.time()
    res = pf_oracle.ac_baseline(e0, 500, 1.5, 2.0, 1.0, 0.05)
    dt_s = time.time() - t
    m, e = pf_oracle.ac_mass_energy(res, 1.5, 2.0)
    out["ac3d_128_n8_dt0.05_500"] = dict(shape=[128, 128, 128], fields=8, points=200, seed=3, gamma=1.5,
                                         kappa=2.0, L=1.0, dt=0.05, steps=500, source="oracle",
                                         oracle_seconds=dt_s, sha256=sha(res), mass=m.tolist(), energy=e,
                                         sample_stride=999983, sample=res.ravel()[::999983].tolist())
    print("ac3d dt=0.05 oracle %.1fs" % dt_s)
    x = e0.copy()
    first_bad = None
    maxabs = []
    for s in range(1, 41):
        x = pf_oracle.ac_baseline(x, 1, 1.5, 2.0, 1.0, 0.1)
        mx = float(np.nanmax(np.abs(x))) if np.isfinite(x).any() else float("nan")
        maxabs.append(mx)
        if first_bad is None and not np.isfinite(x).all():
            first_bad = s
            break
    out["ac3d_128_n8_dt0.1_divergence"] = dict(dt=0.1, first_nonfinite_step=first_bad, max_abs_per_step=maxabs,
                                               source="oracle")
    print("ac3d dt=0.1 first non-finite step", first_bad)
    with open(os.path.join(HERE, "full_size.json"), "w") as f:
        json.dump(out, f, indent=1)


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--full", action="store_true")
    ap.add_argument("--only", nargs="*", help="names of the small fixtures to (re)make")
    args = ap.parse_args()
    if not pf_oracle.ref_available():
        sys.exit("build the reference program first: make -C oracle ref")
    make_small(set(args.only) if args.only else None)
    make_sparse(set(args.only) if args.only else None)
    if args.full:
        make_full()
