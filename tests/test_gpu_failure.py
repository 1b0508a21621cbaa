"""Failure detection on the device without a fault: a bounded wait that runs out.

The FP32 3D streaming kernel stages planes with bulk copies on mbarriers and
bounds every wait.  MMSP_GPU_TEST_STALL_LAUNCHES=1 makes the next launch's
fills expect their bytes without issuing any copy and caps its waits at 4
polls, so the waits run out with no copy in flight: the kernel sets the
error word, drains (bounded) and returns, the host reports
MMSP_GPU_ETIMEDOUT, and the context stays usable -- a new upload and steps
afterwards match the oracle.  Run in a child process so the variable does
not reach other tests.
"""
import os
import subprocess
import sys

import pytest

from conftest import ROOT

pytestmark = pytest.mark.gpu

CHILD = r"""
import sys
import numpy as np
sys.path.insert(0, %r)
from mmsp_gb300 import inputs, native
from oracle import pf_oracle
L = native.load()
x = inputs.noisy_composition((40, 24, 64), 0.4, 0.02, 5)
d = native.make_desc(x.shape, 1, np.float32, "ch", dt=0.002)
with native.Stepper(d) as s:
    s.upload(x.astype(np.float32))
    s.step(1)                                   # the stalled launch
    print("first", L.mmsp_gpu_synchronize(s.h), flush=True)
    print("again", L.mmsp_gpu_synchronize(s.h), flush=True)   # the error word was cleared
    s.upload(x.astype(np.float32))
    s.step(20)
    got = s.download().astype(np.float64)
want = pf_oracle.ch_baseline(x, 20, 1.0, 1.0, 0.002)
print("err", float(np.abs(got - want).max()), flush=True)
"""


def test_bounded_wait_runs_out_and_the_context_stays_usable(gpu):
    env = dict(os.environ, MMSP_GPU_TEST_STALL_LAUNCHES="1")
    r = subprocess.run([sys.executable, "-c", CHILD % ROOT], env=env, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    lines = dict(line.split(None, 1) for line in r.stdout.splitlines() if line.strip())
    assert int(lines["first"]) == gpu.ETIMEDOUT
    assert int(lines["again"]) == gpu.OK
    assert float(lines["err"]) <= 1e-5
