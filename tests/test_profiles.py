"""The ncu summaries under profiles/ name the commands they were captured
from; each command must run committed code: a bench.py case that exists, and
no path outside the repository."""
import glob
import os
import re

import bench

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PROFILES = sorted(glob.glob(os.path.join(ROOT, "profiles", "*.txt")))


def test_profiles_exist():
    assert PROFILES


def test_profile_commands_name_existing_cases():
    cases = set(bench.CASES) | {"batch_f32"}
    for path in PROFILES:
        text = open(path).read()
        assert "Command" in text, path
        assert "--clock-control none" in text, path
        for name in re.findall(r"bench\.py --case (\S+)", text):
            assert name in cases, (path, name)
        assert "/root/" not in text, path


def test_profiles_state_traffic_and_kernel():
    for path in PROFILES:
        text = open(path).read()
        assert re.search(r"^Kernels?:", text, re.M), path
        assert "traffic_bytes_per_launch" in text or "dram__bytes" in text, path
