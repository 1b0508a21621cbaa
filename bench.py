"""Benchmark of the explicit phase-field step (one JSON line on stdout).

Default workload: 3D Cahn-Hilliard, f=c^2(1-c)^2, 256^3 cells, dt=0.002,
kappa=M=1, periodic, 1000 explicit steps per bench step, in FP64 -- the
arithmetic of the reference's own update() -- with fused multiply-adds
(MMSP_GPU_FLAG_CONTRACT: within 1e-12 relative of the reference).  ``value``
is cell-updates/s with the state resident in HBM; ``e2e`` is the same metric
through the C ABI call a user's update(grid&, steps) makes (mmsp_gpu_update:
pinned host buffer in, device steps, host buffer out, all inside the timed
region).  The FP64 step is bound by the FP64 pipe, so ``roofline`` compares
its FP64 operations per second with the device's measured FP64 rate
(mmsp_gpu_fp64_rate).

Beside the headline the line carries, measured in the same run:
``forms``    the bit-identical FP64 form and the FP32 precision form (HBM
             roofline, e2e, error and mass drift against FP64);
``batched``  256 2D Cahn-Hilliard grids of sides 64..512 in FP32, against
             the same 256 solves one at a time in FP64;
``serving``  a Poisson stream of mixed requests through the request loop,
             p50/p99 latency, against the same requests one at a time in FP64;
``configs``  the other single-grid configurations and models.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

``--impl reference`` times the reference's serial update() restated as the
C oracle (the reference itself cannot be compiled on the GPU host: its
source is not there) on all host cores, in FP64, on bounded samples of the
same grid.  Under torchrun each rank runs an independent replica (the grid
does not shard across devices in this build): ``scaling`` is "weak".
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

# The request loop runs each admitted request on its own stream (128 of
# them); more hardware work queues than the default 8 let their kernels start
# independently.  Read when the process creates its CUDA context.
os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "cell-updates/s (3D Cahn-Hilliard 256^3, 1000 explicit steps, FP64)"
SHAPE = (256, 256, 256)
SOLVE_STEPS = 1000
DT, KAPPA, MOB = 0.002, 1.0, 1.0
MEAN, AMP, SEED = 0.4, 0.02, 2
WORKLOAD = "ch3d_256_f64"
# FP64 pipe operations (add, multiply or fused multiply-add) per cell-step of
# the two FP64 forms (pf_ch64.cu: 9 + 7 contracted, 13 + 10 exact)
F64_OPS_CONTRACT = 16
F64_OPS_EXACT = 23


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def max_over_ranks(x: float, device=None) -> float:
    """The largest value of x over the ranks of the default process group
    (x itself without one).  Replicas time their own solves; the job's time is
    the slowest rank's."""
    import torch
    import torch.distributed as dist

    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return x
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_throughput(units_per_rank: float, slowest_seconds: float, world: int) -> float:
    """Whole-job throughput of independent replicas: all ranks' units over
    the slowest rank's time (weak scaling)."""
    return world * units_per_rank / slowest_seconds


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def profile_traffic(kernel_tag: str):
    """DRAM bytes per launch of the named kernel, from the ncu summary in profiles/."""
    p = os.path.join(ROOT, "profiles", kernel_tag + ".txt")
    if not os.path.exists(p):
        return None
    for line in open(p):
        line = line.strip()
        if line.startswith("traffic_bytes_per_launch:"):
            try:
                return float(line.split(":", 1)[1].split()[0])
            except ValueError:
                return None
    return None


class Clocks:
    """nvidia-smi samples during the timed region."""

    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap,utilization.gpu")

    def __init__(self, index: int):
        self.index = index
        self.p = None
        self.path = None

    def start(self):
        try:
            import tempfile
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.f = open(self.path, "w")
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                                       "--format=csv,noheader,nounits", "-lms", "100"],
                                      stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.p = None

    def stop(self):
        if self.p is None:
            return None
        self.p.terminate()
        try:
            self.p.wait(timeout=5)
        except Exception:
            self.p.kill()
        self.f.close()
        sm, smax, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            v = [x.strip() for x in line.split(",")]
            if len(v) < 8:
                continue
            try:
                util = float(v[7])
                if util > 0:
                    sm.append(float(v[0]))
                smax = max(smax, float(v[1]))
            except ValueError:
                continue
            for n, x in zip(names, v[3:7]):
                if x.lower() == "active":
                    reasons.add(n)
        os.unlink(self.path)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax or None,
                "reasons": sorted(reasons), "samples_under_load": len(sm)}


def cpu_sample(threads: int, target_s: float = 10.0):
    """The oracle (the reference's update() restated in C, FP64) on the full
    grid for as many steps as fit in about target_s seconds."""
    from mmsp_gb300 import inputs
    from oracle import pf_oracle

    c = inputs.noisy_composition(SHAPE, MEAN, AMP, SEED)
    t0 = time.perf_counter()
    pf_oracle.ch_baseline(c, 1, KAPPA, MOB, DT, threads=threads)
    t1 = time.perf_counter() - t0
    n = max(1, int(target_s / max(t1, 1e-3)))
    t0 = time.perf_counter()
    pf_oracle.ch_baseline(c, n, KAPPA, MOB, DT, threads=threads)
    el = time.perf_counter() - t0
    cells = int(np.prod(SHAPE))
    return cells * n / el, n, el


def run_reference(args):
    ws, rank, _ = dist_env()
    if rank != 0:
        return 0
    threads = os.cpu_count() or 1
    from mmsp_gb300 import inputs
    from oracle import pf_oracle

    c = inputs.noisy_composition(SHAPE, MEAN, AMP, SEED)
    t0 = time.perf_counter()
    pf_oracle.ch_baseline(c, 1, KAPPA, MOB, DT, threads=threads)
    per = time.perf_counter() - t0
    sample_steps = max(1, int(4.0 / max(per, 1e-3)))   # about 4 s per bench step
    for _ in range(args.warmup):
        pf_oracle.ch_baseline(c, sample_steps, KAPPA, MOB, DT, threads=threads)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        pf_oracle.ch_baseline(c, sample_steps, KAPPA, MOB, DT, threads=threads)
    el = time.perf_counter() - t0
    cells = int(np.prod(SHAPE))
    v = cells * sample_steps * args.steps / el
    sample = "%d of the %d explicit steps of the 256^3 grid per bench step, FP64" % (sample_steps, SOLVE_STEPS)
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": "cell-updates/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": el / args.steps * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": WORKLOAD, "grid": list(SHAPE), "steps_per_solve": SOLVE_STEPS,
                   "dt": DT, "kappa": KAPPA, "M": MOB, "parallelism": "host threads"},
        "cpu_baseline": {"value": v, "unit": "cell-updates/s", "cores": threads, "kind": "port",
                         "sample": sample},
        "e2e": {"value": v, "unit": "cell-updates/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def other_configs(native, inputs, stream):
    """The other single-grid configurations, timed with CUDA events on
    `stream`: 2D CH 256^2 FP64 (2000 steps) and 3D AC 128^3 x 8 (500 steps,
    dt 0.05; dt 0.1 diverges) in FP32 and FP64."""
    import torch

    def timed(desc, x, steps):
        s = native.Stepper(desc)
        s.set_stream(stream.cuda_stream)
        s.upload(x)
        s.step(min(steps, 64))
        s.synchronize()
        s.upload(x)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        with torch.cuda.stream(stream):
            e0.record(stream)
            s.step(steps)
            e1.record(stream)
        stream.synchronize()
        out = s.download()
        s.close()
        return e0.elapsed_time(e1), out

    res = {}
    c2 = inputs.noisy_composition((256, 256), 0.5, 0.01, 1)
    ms, _ = timed(native.make_desc((256, 256), 1, np.float64, "ch", dt=0.005), c2, 2000)
    msc, _ = timed(native.make_desc((256, 256), 1, np.float64, "ch", dt=0.005, contract=True), c2, 2000)
    res["ch2d_256_f64_2000"] = {"ms": ms, "cell_updates_per_s": 256 * 256 * 2000 / (ms / 1e3),
                                "contracted_ms": msc, "contracted_cell_updates_per_s": 256 * 256 * 2000 / (msc / 1e3)}
    e = inputs.voronoi_grains((128, 128, 128), 200, 8, 3)
    ms32, o32 = timed(native.make_desc((128, 128, 128), 8, np.float32, "ac", gamma=1.5, kappa=2.0, dt=0.05),
                      e.astype(np.float32), 500)
    ms64, o64 = timed(native.make_desc((128, 128, 128), 8, np.float64, "ac", gamma=1.5, kappa=2.0, dt=0.05), e, 500)
    vals = 128 ** 3 * 8 * 500
    res["ac3d_128_n8_500"] = {"f32_ms": ms32, "f64_ms": ms64, "f32_value_updates_per_s": vals / (ms32 / 1e3),
                              "f64_value_updates_per_s": vals / (ms64 / 1e3),
                              "f32_roofline_frac": 2 * 4 * vals / (ms32 / 1e3) / 1e9 / peaks()[0],
                              "f32_max_err_vs_f64": float(np.abs(o32.astype(np.float64) - o64).max())}
    res.update(other_models(native, inputs, timed))
    return res


def other_models(native, inputs, timed):
    """The further explicit models on the same device path: Zener pinning
    (grain growth with the particle field fixed) on 128^3 x 3 fields,
    Ostwald ripening (composition + order parameter; one kernel per step in
    FP32, two in FP64) on 256 x 128 x 64 x 2 fields (the example's 128 x 64 x 16, doubled per
    axis) and model B (Cahn-Hilliard with thermal noise) on 1024^2, 500
    steps each in FP32 and FP64, beside the oracle (the reference's loops
    restated in C, FP64, one thread) on 2 steps."""
    from oracle import pf_oracle

    peak = peaks()[0]
    out = {}
    sigma = float(np.sqrt(2.0 * 0.01 / 0.01))   # model B: sqrt(2 kT/(dt dV)), kT = dt = 0.01, dV = 1
    cases = [
        ("zener3d_128_n3_500", (128, 128, 128), 3, "zener", {}, inputs.zener_particles((128, 128, 128), 400, 9),
         lambda x, n: pf_oracle.ac_zener(x, n, 0.01, threads=1)),
        ("ostwald3d_256x128x64_n2_500", (256, 128, 64), 2, "ostwald", {},
         inputs.ostwald_start((256, 128, 64), 2, 9), lambda x, n: pf_oracle.ostwald(x, n, threads=1)),
        ("modelB2d_1024_noise_500", (1024, 1024), 1, "ch_poly", dict(dt=0.01, noise=sigma, seed=3),
         inputs.noisy_composition((1024, 1024), 0.0, 0.1, 9),
         lambda x, n: pf_oracle.ch_shipped_noise(x, n, dt=0.01, noise=sigma, seed=3, threads=1)),
    ]
    for name, shape, fields, model, kw, x, cpu in cases:
        steps = 500
        d32 = native.make_desc(shape, fields, np.float32, model, **kw)
        d64 = native.make_desc(shape, fields, np.float64, model, **kw)
        ms32, o32 = timed(d32, x.astype(np.float32), steps)
        ms64, o64 = timed(d64, x, steps)
        vals = int(np.prod(shape)) * fields * steps
        t0 = time.perf_counter()
        cpu(x, 2)
        cpu_s = (time.perf_counter() - t0) / 2
        cpu_rate = int(np.prod(shape)) * fields / cpu_s
        out[name] = {"f32_ms": ms32, "f64_ms": ms64, "f32_value_updates_per_s": vals / (ms32 / 1e3),
                     "f64_value_updates_per_s": vals / (ms64 / 1e3),
                     "f32_roofline_frac": 2 * 4 * vals / (ms32 / 1e3) / 1e9 / peak,
                     "f32_max_err_vs_f64": float(np.abs(o32.astype(np.float64) - o64).max()),
                     "cpu_oracle_value_updates_per_s": cpu_rate, "cpu_sample": "2 FP64 steps, 1 thread",
                     "f64_speedup_vs_cpu": vals / (ms64 / 1e3) / cpu_rate}
    out.update(convex_splitting(native, inputs, timed))
    out.update(sparse_grain_growth(native, inputs))
    return out


def sparse_grain_growth(native, inputs):
    """Sparse phase-field grain growth (the sparsePF example's update, FP64)
    on a 2048^2 grid of 32 periodic Voronoi grains, 16 item slots per
    cell, 100 steps in one call, beside the oracle (the example's loops
    restated in C, one thread) on 2 steps.  Algorithmic bytes of a step:
    every cell's list read and the new list written once (int32 count, then
    int32 index + float64 value per item), at the lists' mean length (about
    190 MB per step: above the 129 MB L2)."""
    import torch

    from oracle import pf_oracle

    shape, K, steps = (2048, 2048), 16, 100
    c0, i0, v0 = inputs.sparse_grains(shape, 32, 21, K)
    d = native.make_desc(shape, K, np.float64, "sparse_gg")
    stream = torch.cuda.Stream()
    with native.Stepper(d) as s:
        s.set_stream(stream.cuda_stream)    # the events below are recorded on the handle's stream
        s.sparse_upload(c0, i0, v0)
        s.step(8)
        s.synchronize()
        s.sparse_upload(c0, i0, v0)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        s.step(steps)
        e1.record(stream)
        stream.synchronize()
        ms = e0.elapsed_time(e1)
        cnt, _, _ = s.sparse_download()
    cells = int(np.prod(shape))
    mean_items = 0.5 * (float(c0.mean()) + float(cnt.mean()))
    alg = cells * 2 * (4 + 12 * mean_items)
    peak = peaks()[0]
    t0 = time.perf_counter()
    pf_oracle.sparse_gg(c0, i0, v0, 2, 0.01, 1e-8, threads=1)
    cpu_s = (time.perf_counter() - t0) / 2
    rate = cells * steps / (ms / 1e3)
    return {"sparse2d_2048_g32_100": {"f64_ms": ms, "cell_updates_per_s": rate, "mean_items_per_cell": mean_items,
                                     "longest_list": int(cnt.max()),
                                     "roofline": {"bound": "hbm", "alg_bytes_per_step": alg,
                                                  "achieved_gbs": alg / (ms / 1e3 / steps) / 1e9, "peak": peak,
                                                  "frac": alg / (ms / 1e3 / steps) / 1e9 / peak},
                                     "cpu_oracle_cell_updates_per_s": cells / cpu_s, "cpu_sample": "2 steps, 1 thread",
                                     "speedup_vs_cpu": rate / (cells / cpu_s)}}


def convex_splitting(native, inputs, timed):
    """Convex-splitting Cahn-Hilliard on the example's 400 x 200 grid (stripes
    start, parametric energy, dt = 1/(D K)): 20 semi-implicit steps in FP64,
    each a red-black SOR solve to a 1e-14 residual, beside the oracle (the
    example's loops restated in C, one thread) on 2 steps."""
    from oracle import pf_oracle

    shape = (400, 200)
    x = inputs.convex_start(shape)
    d = native.make_desc(shape, 2, np.float64, "ch_convex")
    steps = 20
    ms, _ = timed(d, x, steps)
    with native.Stepper(d) as s:
        s.upload(x)
        s.step(steps)
        iters = s.reduce().solver_iterations
    t0 = time.perf_counter()
    _, cpu_iters = pf_oracle.ch_convex(x, 2, return_iters=True)
    cpu_s = (time.perf_counter() - t0) / 2
    return {"convex2d_400x200_f64_20": {"ms_per_step": ms / steps, "iterations_last_step": iters,
                                        "cpu_oracle_ms_per_step": cpu_s * 1e3,
                                        "cpu_oracle_iterations_step2": cpu_iters,
                                        "speedup_vs_cpu": cpu_s * 1e3 / (ms / steps),
                                        "cpu_sample": "2 steps, 1 thread, FP64"}}


def output_path(native, inputs):
    """Snapshots of the 256^3 FP32 grid as MMSP grid files (zlib level 9, as
    the reference writes them): three snapshots 100 steps apart through
    mmsp_gpu_output, timed from the first step call until the last file is
    on disk, against one compress2 call on one thread of the same payload
    (the reference's write_buffer)."""
    import shutil
    import tempfile
    import zlib

    td = tempfile.mkdtemp(prefix="mmsp_out_")
    try:
        x = inputs.noisy_composition(SHAPE, MEAN, AMP, SEED).astype(np.float32)
        d = native.make_desc(SHAPE, 1, np.float32, "ch", dt=DT, kappa=KAPPA, mobility=MOB)
        with native.Stepper(d) as s:
            s.upload(x)
            s.output(os.path.join(td, "warm.dat"))   # first use allocates the buffers
            s.output_wait()
            t0 = time.perf_counter()
            for i in range(3):
                s.step(100)
                s.output(os.path.join(td, "s%d.dat" % i))
            s.output_wait()
            wall = time.perf_counter() - t0
            raw = s.download().tobytes()
        size = os.path.getsize(os.path.join(td, "s2.dat"))
        t1 = time.perf_counter()
        zlib.compress(raw, 9)
        ref = time.perf_counter() - t1
    finally:
        shutil.rmtree(td, ignore_errors=True)
    return {"grid": "256^3 f32", "snapshots": 3, "steps_between": 100, "level": 9, "wall_s": wall,
            "s_per_snapshot": wall / 3, "payload_mb": len(raw) / 1e6, "file_mb": size / 1e6,
            "host_threads": os.cpu_count(), "reference_write_s": ref,
            "reference_write": "one compress2 (zlib level 9) call on one thread, as write_buffer does",
            "speedup_vs_reference_write": ref / (wall / 3)}


def timed_solver(native, stream, flush):
    """One bench step on `stream`: reset the state from a device copy
    (untimed), flush L2 (untimed), then `steps` steps between CUDA events on
    the same stream."""
    import torch

    def solve(s, init, nbytes, steps=SOLVE_STEPS):
        with torch.cuda.stream(stream):
            s.upload_device(init.data_ptr(), nbytes, native.FIELD_MAJOR)
            flush.zero_()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            s.step(steps)
            e1.record(stream)
        return e0, e1

    return solve


def e2e_update(native, desc, host, reps, warmup, flush):
    """mmsp_gpu_update (create, upload from the pinned host buffer, 1000
    steps, reduction, download into it, destroy), timed on the host around
    the call; the host buffer is refilled (untimed) before every call."""
    import ctypes

    import torch

    L = native.load()
    stats = native.Stats()
    hv, c0 = host
    nbytes = hv.nbytes
    times = []
    for i in range(warmup + reps):
        hv[:] = c0
        flush.zero_()
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        rc = L.mmsp_gpu_update(ctypes.byref(desc), hv.ctypes.data, nbytes, native.CELL_MAJOR, SOLVE_STEPS,
                               ctypes.byref(stats))
        t2 = time.perf_counter()
        if rc != 0:
            raise native.GpuError(rc, "mmsp_gpu_update")
        if i >= warmup:
            times.append(t2 - t1)
    return float(np.mean(times)), nbytes


def run_gpu(args):
    import torch

    from mmsp_gb300 import inputs, native

    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    def barrier():
        if ws > 1:
            import torch.distributed as dist
            dist.barrier()

    native.load()
    cells = int(np.prod(SHAPE))
    c0 = inputs.noisy_composition(SHAPE, MEAN, AMP, SEED)
    c0_32 = c0.astype(np.float32)
    stream = torch.cuda.Stream()
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    solve = timed_solver(native, stream, flush)

    def make(dtype, contract=False):
        d = native.make_desc(SHAPE, 1, dtype, "ch", kappa=KAPPA, mobility=MOB, dt=DT, contract=contract)
        s = native.Stepper(d)
        s.set_stream(stream.cuda_stream)
        return d, s

    # ---- headline: FP64 (contracted) on the device -------------------------------------------
    d64, s64 = make(np.float64, contract=True)
    init64 = torch.from_numpy(c0).cuda()
    nbytes64 = init64.numel() * 8
    for _ in range(args.warmup):
        solve(s64, init64, nbytes64)
    stream.synchronize()
    torch.cuda.synchronize()
    barrier()
    clocks = Clocks(local)
    clocks.start()
    evs = []
    t0 = time.perf_counter()
    for _ in range(args.steps):
        evs.append(solve(s64, init64, nbytes64))
    stream.synchronize()
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    barrier()
    clk = clocks.stop()
    ms = [a.elapsed_time(b) for a, b in evs]
    ms_step = max_over_ranks(float(np.mean(ms)), "cuda")
    value = job_throughput(cells * SOLVE_STEPS, ms_step / 1e3, ws)
    st64 = s64.reduce()
    out64c = s64.download()
    s64.close()
    m0 = float(np.sum(c0))

    # FP64 roofline: FP64 pipe operations per step over the measured FP64 rate
    fp64_peak = native.fp64_rate(stream.cuda_stream)
    step_s = ms_step / 1e3 / SOLVE_STEPS
    fp64_achieved = F64_OPS_CONTRACT * cells / step_s
    hbm_peak, peak_kind = peaks()

    # ---- bit-identical FP64 form (the reference's operation order) ----------------------------
    dx64, sx64 = make(np.float64, contract=False)
    solve(sx64, init64, nbytes64)
    a, b = solve(sx64, init64, nbytes64)
    stream.synchronize()
    ms_exact = a.elapsed_time(b)
    stx = sx64.reduce()
    out64 = sx64.download()
    sx64.close()
    rel_contract = float(np.abs(out64c - out64).max() / np.abs(out64).max())

    # ---- e2e FP64 through mmsp_gpu_update with pinned host buffers ----------------------------
    host64 = torch.empty(cells, dtype=torch.float64, pin_memory=True)
    e2e_s, _ = e2e_update(native, d64, (host64.numpy(), c0.ravel()), args.steps, 1, flush)
    e2e_s = max_over_ranks(e2e_s, "cuda")
    e2e_val = job_throughput(cells * SOLVE_STEPS, e2e_s, ws)

    # ---- FP32 precision form -------------------------------------------------------------------
    d32, s32 = make(np.float32)
    init32 = torch.from_numpy(c0_32).cuda()
    nbytes32 = init32.numel() * 4
    for _ in range(args.warmup):
        solve(s32, init32, nbytes32)
    ev32 = [solve(s32, init32, nbytes32) for _ in range(args.steps)]
    stream.synchronize()
    ms32 = float(np.mean([a.elapsed_time(b) for a, b in ev32]))
    st32 = s32.reduce()
    out32 = s32.download().astype(np.float64)
    s32.close()
    err = np.abs(out32 - out64)
    host32 = torch.empty(cells, dtype=torch.float32, pin_memory=True)
    e2e32_s, _ = e2e_update(native, d32, (host32.numpy(), c0_32.ravel()), min(args.steps, 5), 1, flush)
    alg32 = cells * 2 * 4                      # one read + one write of the FP32 state per step
    ach32 = alg32 / (ms32 / 1e3 / SOLVE_STEPS) / 1e9

    line = {
        "metric": METRIC, "value": value, "unit": "cell-updates/s", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded SplitMix64, c=0.4+0.02*U(-1,1))",
        "config": {"workload": WORKLOAD, "grid": list(SHAPE), "steps_per_solve": SOLVE_STEPS, "dt": DT,
                   "kappa": KAPPA, "M": MOB, "bc": "periodic", "parallelism": "replicas" if ws > 1 else "1 GPU",
                   "form": "FP64, fused multiply-adds (MMSP_GPU_FLAG_CONTRACT), <= 1e-12 relative of the reference",
                   "l2": "flushed (256 MiB write) before every timed solve; FP64 working set 403 MB (state, "
                         "newGrid, temp)"},
        "roofline": {"bound": "fp64", "achieved": fp64_achieved / 1e12, "peak": fp64_peak / 1e12,
                     "unit": "T FP64 ops/s", "frac": fp64_achieved / fp64_peak,
                     "traffic": profile_traffic("ch64_step_f64_256"),
                     "kernel": "ch64_mu + ch64_update (one step: two launches)",
                     "peak_source": "measured live: mmsp_gpu_fp64_rate (independent FP64 FMA chains, all SMs)",
                     "ops_per_launch": F64_OPS_CONTRACT * cells, "ops_per_cell": F64_OPS_CONTRACT,
                     "hbm": {"alg_bytes_per_step": cells * 40,
                             "achieved_gbs": cells * 40 / step_s / 1e9, "peak_gbs": hbm_peak,
                             "note": "read c, write mu; read mu and c, write c' (40 B per cell)"}},
        "e2e": {"value": e2e_val, "unit": "cell-updates/s", "h2d_bytes_per_step": nbytes64,
                "d2h_bytes_per_step": nbytes64 + 16, "ms_per_step": e2e_s * 1e3},
        "gpu_launches": args.steps * SOLVE_STEPS * 2,
        "forms": {
            "f64_contracted": {"cell_updates_per_s": value, "ms_per_solve": ms_step,
                               "max_rel_err_vs_exact": rel_contract, "mass_drift": (st64.mass - m0) / m0},
            "f64_exact": {"cell_updates_per_s": cells * SOLVE_STEPS / (ms_exact / 1e3), "ms_per_solve": ms_exact,
                          "mass_drift": (stx.mass - m0) / m0,
                          "fp64_frac": F64_OPS_EXACT * cells / (ms_exact / 1e3 / SOLVE_STEPS) / fp64_peak,
                          "note": "bit-identical to the reference's update()"},
            "f32_precision": {"cell_updates_per_s": cells * SOLVE_STEPS / (ms32 / 1e3), "ms_per_solve": ms32,
                              "max_err_vs_f64": float(err.max()), "l2_err_vs_f64": float(np.sqrt(np.mean(err ** 2))),
                              "mass_drift": (st32.mass - m0) / m0,
                              "roofline": {"bound": "hbm", "achieved": ach32, "peak": hbm_peak, "unit": "GB/s",
                                           "frac": ach32 / hbm_peak, "traffic": profile_traffic("ch3_stream_f32_256"),
                                           "kernel": "ch3_stream_f32<8,256,2,CH,unit>", "peak_source": peak_kind,
                                           "alg_bytes_per_launch": alg32},
                              "e2e": {"value": cells * SOLVE_STEPS / e2e32_s, "unit": "cell-updates/s",
                                      "h2d_bytes_per_step": nbytes32, "d2h_bytes_per_step": nbytes32 + 16}},
        },
        "clocks": clk,
        "wall_s_timed_region": wall,
    }
    line["configs"] = other_configs(native, inputs, stream)
    if rank == 0:
        line["output"] = output_path(native, inputs)
        line["batched"] = batched(native, inputs, stream, max(3, args.steps // 4), flush)
        line["serving"] = serving(native, args.serve_requests, 200.0, 5, sequential=True)
        # a sustainable rate: 0.7 x the offered-load throughput, another draw of the mix
        sus = serving(native, max(50, args.serve_requests // 2), max(1.0, 0.7 * line["serving"]["value"]), 6,
                      sequential=False)
        line["serving"]["sustainable"] = {k: sus[k] for k in ("rate_offered", "requests", "value", "p50_s", "p99_s",
                                                              "span_s")}
    if rank == 0 and args.cpu_baseline:
        v, n, el = cpu_sample(1)
        line["cpu_baseline"] = {"value": v, "unit": "cell-updates/s", "cores": 1, "kind": "port",
                                "sample": "%d explicit FP64 steps of the 256^3 grid (%.1f s), serial C oracle" % (n, el)}
    if rank == 0:
        print(json.dumps(line), flush=True)
    if ws > 1:
        import torch.distributed as dist
        dist.destroy_process_group()
    return 0


BATCH_STEPS = 1000


def batched(native, inputs, stream, reps, flush):
    """Batched 2D Cahn-Hilliard (256 grids, sides 64..512, own kappa and mean
    composition, dt 0.005, 1000 steps each) in FP32 through mmsp_gpu_batch_*,
    against the same 256 solves one at a time in FP64 (contracted form) on
    the same GPU: the device time with the states resident, and end to end
    with host buffers in and out (mmsp_gpu_update per grid for the sequential
    side).  The FP32 results' largest deviation from FP64 is the accuracy."""
    import torch

    work = inputs.batched_cahn_hilliard(count=256, seed=4)
    cells = sum(c0.size for c0, _ in work)
    host = [c0.astype(np.float32) for c0, _ in work]
    descs = [native.make_desc(c0.shape, 1, np.float32, "ch", kappa=k, mobility=1.0, dt=0.005) for c0, k in work]
    b = native.Batch(descs)
    b.set_stream(stream.cuda_stream)
    for i, h in enumerate(host):
        b.upload(i, h)
    b.tune()
    info = b.info()
    times = []
    for it in range(1 + reps):
        for i, h in enumerate(host):          # reset (untimed)
            b.upload(i, h)
        flush.zero_()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        with torch.cuda.stream(stream):
            e0.record(stream)
            b.step(BATCH_STEPS)
            e1.record(stream)
        stream.synchronize()
        if it >= 1:
            times.append(e0.elapsed_time(e1))
    ms = float(np.mean(times))
    out32 = [b.download(i).astype(np.float64) for i in range(len(work))]
    # end to end: inputs from and results to pinned host memory
    pin_in = [torch.from_numpy(h).pin_memory().numpy() for h in host]
    pin_out = [torch.empty(h.shape, dtype=torch.float32).pin_memory().numpy() for h in host]
    e2e = []
    for _ in range(max(2, reps // 2)):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        b.upload_all(pin_in)
        b.step(BATCH_STEPS)
        res = b.download_all(pin_out)
        e2e.append(time.perf_counter() - t0)
    e2e_s = float(np.mean(e2e))
    b.close()
    del res
    # one at a time, FP64: resident (device time of the steps) and end to end (mmsp_gpu_update)
    seq_dev = 0.0
    seq_e2e = 0.0
    err = 0.0
    for i, (c0, k) in enumerate(work):
        d = native.make_desc(c0.shape, 1, np.float64, "ch", kappa=k, mobility=1.0, dt=0.005, contract=True)
        with native.Stepper(d) as s:
            s.upload(c0)
            s.synchronize()
            t1 = time.perf_counter()
            s.step(BATCH_STEPS)
            s.synchronize()
            seq_dev += time.perf_counter() - t1
        t1 = time.perf_counter()
        o64, _ = native.update(c0, BATCH_STEPS, d)
        seq_e2e += time.perf_counter() - t1
        err = max(err, float(np.abs(o64 - out32[i]).max()))
    solves = len(work) / (ms / 1e3)
    achieved = cells * 8 * BATCH_STEPS / (ms / 1e3) / 1e9      # FP32 read + write per cell-step
    peak, peak_kind = peaks()
    return {
        "metric": "solves/s (256 x 2D Cahn-Hilliard, sides 64-512, 1000 steps, FP32)", "value": solves,
        "unit": "solves/s", "ms_per_batch": ms, "reps": reps, "dtype": "f32",
        "config": {"workload": "ch2d_batch256_f32", "grids": len(work), "cells": cells,
                   "steps_per_solve": BATCH_STEPS, "dt": 0.005,
                   "data": "synthetic (seeded; kappa~U(0.5,2), mean~U(0.3,0.7), c=mean+0.01*U(-1,1))",
                   "tuning": {"rows_per_item": info.rows_per_item, "threads_per_block": info.threads_per_block,
                              "blocks": info.blocks, "items": info.items, "tune_ms": info.tune_ms,
                              "temporal_depth": info.temporal_depth, "tile_rows": info.tile_rows,
                              "tile_cols": info.tile_cols, "tiles": info.tiles}},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": profile_traffic("ch2_tb_f32_256grids" if info.temporal_depth > 1
                                                else "ch2_batch_f32_256grids"),
                     "kernel": ("ch2_tb_kernel<region %dx%d, KS=%d, CH, unit> (%d steps per launch)" % (
                         info.tile_rows, info.tile_cols, info.temporal_depth, info.temporal_depth)
                                if info.temporal_depth > 1 else "ch2_batch_kernel<float,CH>"),
                     "peak_source": peak_kind, "alg_bytes_per_step": cells * 8,
                     "note": "achieved = the per-step algorithmic bytes (one read + one write of every cell) over the "
                             "step time; the blocked kernel moves less (traffic is per launch of temporal_depth steps)"},
        "e2e": {"value": len(work) / e2e_s, "unit": "solves/s", "h2d_bytes_per_step": cells * 4,
                "d2h_bytes_per_step": cells * 4},
        "sequential_f64": {"solves_per_s": len(work) / seq_dev, "seconds": seq_dev,
                           "e2e_solves_per_s": len(work) / seq_e2e, "e2e_seconds": seq_e2e,
                           "how": "256 solves one at a time, FP64 contracted form: device-resident step time, and "
                                  "mmsp_gpu_update per grid (host buffers)"},
        "speedup_vs_sequential_f64": solves / (len(work) / seq_dev),
        "e2e_speedup_vs_sequential_f64": (len(work) / e2e_s) / (len(work) / seq_e2e),
        "max_err_vs_f64": err,
        "gpu_launches_per_batch": BATCH_STEPS // max(1, info.temporal_depth),
    }


def run_batch(args):
    """`--workload batch`: the batched form alone as a bench line."""
    import torch

    from mmsp_gb300 import inputs, native

    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    native.load()
    stream = torch.cuda.Stream()
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    r = batched(native, inputs, stream, args.steps, flush)
    line = dict(r)
    line.update({"n_gpus": ws, "steps": args.steps, "warmup": args.warmup, "ms_per_step": r["ms_per_batch"],
                 "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                 "data": r["config"]["data"], "gpu_launches": args.steps * r["gpu_launches_per_batch"]})
    if rank == 0:
        print(json.dumps(line), flush=True)
    return 0


def serve_requests(n, seed):
    """The serving mix: 50% 2D CH (sides 64-1024), 30% 3D CH (sides 32-256),
    20% 3D AC (4-16 order parameters, sides 32-128); steps log-uniform in
    [100, 10000]; FP32.  dt: 0.005 (2D CH), 0.002 (3D CH), 0.05 (AC)."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        kind = rng.random()
        steps = int(round(10 ** rng.uniform(2.0, 4.0)))
        if kind < 0.5:
            s = int(rng.integers(64, 1025))
            shape, fields, model, p = (s, s), 1, "ch", dict(dt=0.005, kappa=1.0, mobility=1.0)
        elif kind < 0.8:
            s = int(rng.integers(32, 257))
            shape, fields, model, p = (s, s, s), 1, "ch", dict(dt=0.002, kappa=1.0, mobility=1.0)
        else:
            s = int(rng.integers(32, 129))
            fields = int(rng.integers(4, 17))
            shape, model, p = (s, s, s), "ac", dict(dt=0.05, kappa=2.0, mobility=1.0, gamma=1.5)
        out.append((shape, fields, model, p, steps, int(rng.integers(0, 2**31))))
    return out


def make_state(shape, fields, seed):
    rng = np.random.default_rng(seed)
    if fields == 1:
        return (0.4 + 0.02 * (2 * rng.random(shape, dtype=np.float32) - 1)).astype(np.float32)
    # grains: each cell one random order parameter at 1
    g = rng.integers(0, fields, size=shape)
    e = np.zeros(shape + (fields,), np.float32)
    np.put_along_axis(e, g[..., None], 1.0, axis=-1)
    return e


def serving(native, n, rate, seed, sequential=True):
    """Poisson arrivals (`rate` per second) of `n` mixed FP32 requests into the
    request loop (mmsp_gpu_server_*): host buffers in at submit, results
    fetched to the host; p50/p99 latency from submit to finish and solves/s
    over the span from the first submit to the last finish.  With
    `sequential`, the same requests are then solved one at a time in FP64
    (contracted form) through mmsp_gpu_update on the same GPU, which gives
    the measured one-at-a-time baseline and the FP32 results' accuracy."""
    import threading

    reqs = serve_requests(n, seed)
    rng = np.random.default_rng(seed + 1)
    arrivals = np.cumsum(rng.exponential(1.0 / rate, size=n))
    states = [make_state(sh, f, s) for sh, f, _, _, _, s in reqs]
    descs = [native.make_desc(sh, f, np.float32, m, **p) for sh, f, m, p, _, _ in reqs]
    srv = native.Server()
    ids = [None] * n

    def feeder():
        t0 = time.perf_counter()
        for i in range(n):
            dt = arrivals[i] - (time.perf_counter() - t0)
            if dt > 0:
                time.sleep(dt)
            ids[i] = srv.submit(descs[i], states[i], reqs[i][4])

    th = threading.Thread(target=feeder)
    th.start()
    th.join()
    lat, fin, sub, results = [], [], [], []
    for i in range(n):
        st = srv.wait(ids[i], 3600.0)
        assert st.state == native.REQ_DONE, (st.state, st.message, reqs[i])
        lat.append(st.finish_s - st.submit_s)
        fin.append(st.finish_s)
        sub.append(st.submit_s)
        results.append(srv.fetch(ids[i]) if sequential else None)
    stats = srv.stats()
    srv.stop()
    span = max(fin) - min(sub)
    work = sum(int(np.prod(sh)) * f * st for sh, f, _, _, st, _ in reqs)
    out = {"metric": "served solves/s, p50/p99 latency (mixed CH/AC requests, Poisson arrivals, FP32)",
           "value": n / span, "unit": "solves/s", "dtype": "f32", "rate_offered": rate, "requests": n,
           "p50_s": float(np.percentile(lat, 50)), "p99_s": float(np.percentile(lat, 99)), "span_s": span,
           "value_updates_per_s": work / span, "rounds": int(stats.rounds),
           "arrival_window_s": float(arrivals[-1]),
           "config": {"workload": "serve_mix_f32", "mix": "50% 2D CH sides 64-1024, 30% 3D CH sides 32-256, "
                      "20% 3D AC N=4-16 sides 32-128; steps log-uniform 100-10000", "seed": seed},
           "e2e": {"value": n / span, "unit": "solves/s",
                   "h2d_bytes_per_step": int(sum(x.nbytes for x in states)),
                   "d2h_bytes_per_step": int(sum(x.nbytes for x in states)),
                   "note": "requests submitted from host buffers and fetched to host buffers"}}
    if sequential:
        seq = 0.0
        err = 0.0
        by_kind = {}
        for (sh, f, m, p, st, _), x, r in zip(reqs, states, results):
            d = native.make_desc(sh, f, np.float64, m, contract=True, **p)
            t0 = time.perf_counter()
            o64, _ = native.update(x.astype(np.float64), st, d)
            seq += time.perf_counter() - t0
            e = float(np.abs(o64 - r.astype(np.float64)).max())
            err = max(err, e)
            kind = "ac3d" if m == "ac" else "ch%dd" % len(sh)
            k = by_kind.setdefault(kind, {"requests": 0, "max_err_vs_f64": 0.0, "within_1e-5": 0})
            k["requests"] += 1
            k["max_err_vs_f64"] = max(k["max_err_vs_f64"], e)
            k["within_1e-5"] += int(e <= 1e-5)
        out["sequential_f64"] = {"solves_per_s": n / seq, "seconds": seq,
                                 "how": "the same requests one at a time in FP64 (contracted form) through "
                                        "mmsp_gpu_update: host buffer in, steps, host buffer out"}
        out["speedup_vs_sequential_f64"] = (n / span) / (n / seq)
        out["max_err_vs_f64"] = err
        out["err_by_kind"] = by_kind
    return out


def run_serve(args):
    """`--workload serve`: the serving form at the offered rate (with the
    measured sequential FP64 baseline) and at a sustainable rate."""
    from mmsp_gb300 import native

    native.load()
    offered = serving(native, args.serve_requests, 200.0, 5, sequential=True)
    sustained = serving(native, max(50, args.serve_requests // 2), max(1.0, 0.7 * offered["value"]), 6,
                        sequential=False)
    line = dict(offered)
    line.update({"n_gpus": 1, "steps": 1, "warmup": 0, "ms_per_step": offered["span_s"] * 1e3,
                 "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                 "data": "synthetic (seeded request mix and states)", "sustainable": sustained})
    print(json.dumps(line), flush=True)
    return 0


CASES = {
    # name: (shape, fields, dtype, model, params)
    "ch3d_f32": (SHAPE, 1, np.float32, "ch", dict(dt=DT, kappa=KAPPA, mobility=MOB)),
    "ch3d_f64": (SHAPE, 1, np.float64, "ch", dict(dt=DT, kappa=KAPPA, mobility=MOB)),
    "ch3d_f64c": (SHAPE, 1, np.float64, "ch", dict(dt=DT, kappa=KAPPA, mobility=MOB, contract=True)),
    "ch3d208_f32": ((208, 208, 208), 1, np.float32, "ch", dict(dt=DT, kappa=KAPPA, mobility=MOB)),
    "ch3d243_f32": ((243, 243, 243), 1, np.float32, "ch", dict(dt=DT, kappa=KAPPA, mobility=MOB)),
    "ac3d74_n14_f32": ((74, 74, 74), 14, np.float32, "ac", dict(dt=0.05, kappa=2.0, mobility=1.0, gamma=1.5)),
    "modelB2d_f32": ((1024, 1024), 1, np.float32, "ch_poly", dict(dt=0.01, noise=float(np.sqrt(2.0)), seed=3)),
    "ch2d_f64": ((256, 256), 1, np.float64, "ch", dict(dt=0.005, kappa=1.0, mobility=1.0)),
    "ac3d_f32": ((128, 128, 128), 8, np.float32, "ac", dict(dt=0.05, kappa=2.0, mobility=1.0, gamma=1.5)),
    "ac3d_f64": ((128, 128, 128), 8, np.float64, "ac", dict(dt=0.05, kappa=2.0, mobility=1.0, gamma=1.5)),
    "ostwald3d_f32": ((256, 128, 64), 2, np.float32, "ostwald", {}),
    "convex2d_f64": ((400, 200), 2, np.float64, "ch_convex", {}),
    "sparse2d_f64": ((2048, 2048), 16, np.float64, "sparse_gg", {}),
}


def run_case(name: str, steps: int):
    """Run `steps` explicit steps of one workload once, untimed: the command
    the ncu summaries under profiles/ are captured from."""
    from mmsp_gb300 import inputs, native

    if name == "batch_f32":
        work = inputs.batched_cahn_hilliard(count=256, seed=4)
        descs = [native.make_desc(c0.shape, 1, np.float32, "ch", kappa=k, mobility=1.0, dt=0.005) for c0, k in work]
        with native.Batch(descs) as b:
            for i, (c0, _) in enumerate(work):
                b.upload(i, c0.astype(np.float32))
            b.tune()          # 10 candidates x 4 launches before the measured steps
            b.step(steps)
            b.synchronize()
            inf = b.info()
        print("case batch_f32: %d steps, rows/item %d, threads %d" % (steps, inf.rows_per_item, inf.threads_per_block))
        return 0
    shape, fields, dtype, model, params = CASES[name]
    if model == "sparse_gg":
        d = native.make_desc(shape, fields, dtype, model, **params)
        with native.Stepper(d) as s:
            s.sparse_upload(*inputs.sparse_grains(shape, 32, 21, fields))
            s.step(steps)
            cnt, _, _ = s.sparse_download()
        print("case %s: %d steps, mean items %.3f" % (name, steps, float(cnt.mean())))
        return 0
    if fields == 1:
        x = inputs.noisy_composition(shape, MEAN, AMP, SEED)
    elif model == "ostwald":
        x = inputs.ostwald_start(shape, fields, 9)
    elif model == "ch_convex":
        x = inputs.convex_start(shape)
    else:
        x = inputs.voronoi_grains(shape, 200, fields, 3)
    d = native.make_desc(shape, fields, dtype, model, **params)
    with native.Stepper(d) as s:
        s.upload(x.astype(dtype))
        s.step(steps)
        s.synchronize()
        st = s.reduce()
    print("case %s: %d steps, mass %.12g energy %.12g" % (name, steps, st.mass, st.energy))
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu-baseline", dest="cpu_baseline", action="store_false")
    ap.add_argument("--case", choices=sorted(CASES) + ["batch_f32"], help="run one workload untimed (for ncu)")
    ap.add_argument("--case-steps", type=int, default=5)
    ap.add_argument("--workload", default="ch3d", choices=["ch3d", "batch", "serve"])
    ap.add_argument("--serve-requests", type=int, default=100)
    args = ap.parse_args()
    if args.case:
        return run_case(args.case, args.case_steps)
    if args.workload == "batch" and args.impl != "reference":
        if args.warmup < 3:
            args.warmup = 3
        return run_batch(args)
    if args.workload == "serve" and args.impl != "reference":
        return run_serve(args)
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        return run_reference(args)
    return run_gpu(args)


if __name__ == "__main__":
    sys.exit(main())
