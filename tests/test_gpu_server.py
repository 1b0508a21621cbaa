"""The serving form (mmsp_gpu_server_*): continuous batching of mixed solves.

A request's result must be the same alone and in the mix: every request is
compared with the same solve run alone through mmsp_gpu_update (bit for
bit: the same kernels run the same step sequence on each request's own
buffers).  Admission must respect the HBM budget, and the failure paths
(over-budget requests, cancellation, stop with work outstanding, waits that
time out) end requests with status codes, on the host.
"""
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def mixed_requests(gpu):
    from mmsp_gb300 import inputs

    reqs = []
    reqs.append((gpu.make_desc((96, 80), 1, np.float32, "ch", dt=0.005), inputs.noisy_composition((96, 80), 0.5, 0.02, 1), 350))
    reqs.append((gpu.make_desc((64, 64), 1, np.float64, "ch", dt=0.005, kappa=1.7), inputs.noisy_composition((64, 64), 0.4, 0.02, 2), 120))
    reqs.append((gpu.make_desc((20, 24, 32), 1, np.float32, "ch", dt=0.002), inputs.noisy_composition((20, 24, 32), 0.4, 0.02, 3), 500))
    e = inputs.voronoi_grains((16, 18, 20), 10, 5, 4)
    reqs.append((gpu.make_desc((16, 18, 20), 5, np.float32, "ac", dt=0.05, kappa=2.0, gamma=1.5), e, 260))
    reqs.append((gpu.make_desc((33, 47), 1, np.float64, "ch", dt=0.004), inputs.noisy_composition((33, 47), 0.5, 0.05, 5), 0))
    reqs.append((gpu.make_desc((128, 128), 1, np.float32, "ch", dt=0.005), inputs.noisy_composition((128, 128), 0.35, 0.02, 6), 1000))
    return reqs


def alone(gpu, desc, x, steps):
    dt = np.float64 if desc.dtype == gpu.F64 else np.float32
    out, st = gpu.update(x.astype(dt), steps, desc)
    return out, st


def test_results_same_alone_and_in_the_mix(gpu):
    reqs = mixed_requests(gpu)
    with gpu.Server(chunk_steps=100) as srv:
        ids = [srv.submit(d, x, n) for d, x, n in reqs]
        for rid in ids:
            st = srv.wait(rid, 120.0)
            assert st.state == gpu.REQ_DONE, st.state
        outs = [srv.fetch(rid) for rid in ids]
        stats = srv.stats()
        assert stats.completed == len(reqs) and stats.failed == 0 and stats.device_bytes_in_use == 0
    for (d, x, n), got in zip(reqs, outs):
        want, _ = alone(gpu, d, x, n)
        assert np.array_equal(got, want)


def test_further_models_same_alone_and_in_the_mix(gpu):
    """Zener pinning, Ostwald ripening (two kernels and a work grid per step),
    a noisy model-B grid (step-indexed noise, no graph replay) and a
    convex-splitting grid (an implicit solve per step) run through the server
    in chunks and must equal the same solves run alone in one call."""
    from mmsp_gb300 import inputs

    reqs = [
        (gpu.make_desc((24, 20, 16), 3, np.float32, "zener", dt=0.01), inputs.zener_particles((24, 20, 16), 8, 11), 230),
        (gpu.make_desc((32, 24, 16), 2, np.float64, "ostwald"), inputs.ostwald_start((32, 24, 16), 2, 12), 150),
        (gpu.make_desc((48, 40), 1, np.float64, "ch_poly", dt=0.01, noise=1.4, seed=77),
         inputs.noisy_composition((48, 40), 0.0, 0.2, 13), 260),
        (gpu.make_desc((40, 20), 2, np.float64, "ch_convex"), inputs.convex_start((40, 20)), 3),
        (gpu.make_desc((96, 80), 1, np.float32, "ch", dt=0.005), inputs.noisy_composition((96, 80), 0.5, 0.02, 14), 300),
    ]
    with gpu.Server(chunk_steps=100) as srv:
        ids = [srv.submit(d, x, n) for d, x, n in reqs]
        for rid in ids:
            st = srv.wait(rid, 120.0)
            assert st.state == gpu.REQ_DONE, (st.state, st.message)
        outs = [srv.fetch(rid) for rid in ids]
    for (d, x, n), got in zip(reqs, outs):
        want, _ = alone(gpu, d, x, n)
        assert np.array_equal(got, want)


def test_budget_admission_and_memory_release(gpu):
    from mmsp_gb300 import inputs
    import ctypes

    d = gpu.make_desc((64, 64, 64), 1, np.float32, "ch", dt=0.002)
    fp = ctypes.c_size_t()
    assert gpu.load().mmsp_gpu_footprint(ctypes.byref(d), ctypes.byref(fp)) == 0
    budget = 2 * fp.value + 1024          # room for two requests at a time
    x = inputs.noisy_composition((64, 64, 64), 0.4, 0.02, 8)
    with gpu.Server(budget_bytes=budget, chunk_steps=50) as srv:
        ids = [srv.submit(d, x, 300) for _ in range(6)]
        peak_active = 0
        while True:
            st = srv.stats()
            assert st.device_bytes_in_use <= budget
            peak_active = max(peak_active, st.active)
            if st.completed == 6:
                break
            time.sleep(0.002)
        assert peak_active <= 2
        outs = [srv.fetch(r) for r in ids]
        # too big for the whole budget: refused at submission
        big = gpu.make_desc((128, 128, 128), 1, np.float32, "ch", dt=0.002)
        with pytest.raises(gpu.GpuError) as ei:
            srv.submit(big, np.zeros((128, 128, 128), np.float32), 10)
        assert ei.value.code == gpu.ENOMEM
    for o in outs[1:]:
        assert np.array_equal(o, outs[0])


def test_cancel_timeout_and_stop(gpu):
    from mmsp_gb300 import inputs

    d = gpu.make_desc((128, 128, 128), 1, np.float32, "ch", dt=0.002)
    x = inputs.noisy_composition((128, 128, 128), 0.4, 0.02, 9)
    srv = gpu.Server(chunk_steps=20, max_active=1)
    long_id = srv.submit(d, x, 200000)
    queued_id = srv.submit(d, x, 10)
    st = srv.wait(long_id, 0.05)                  # far from done: times out, keeps running
    assert st.state in (gpu.REQ_QUEUED, gpu.REQ_RUNNING)
    srv.cancel(queued_id)                         # still queued behind max_active=1
    srv.cancel(long_id)                           # running: stops at the next round
    assert srv.wait(long_id, 60.0).state == gpu.ECANCELED
    assert srv.wait(queued_id, 60.0).state == gpu.ECANCELED
    with pytest.raises(gpu.GpuError) as ei:
        srv.fetch(long_id)
    assert ei.value.code == gpu.ECANCELED
    srv.submit(d, x, 200000)
    srv.submit(d, x, 200000)
    t0 = time.perf_counter()
    srv.stop()                   # outstanding work ends (ESTOPPED) at the next round boundary
    assert time.perf_counter() - t0 < 10.0
