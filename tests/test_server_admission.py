"""Host logic of the stitch server: the admission policy (reuse, create, LRU eviction of idle
stitchers, waiting behind busy ones, the per-configuration limit) compiled and run on the CPU."""
from __future__ import annotations

import shutil
import subprocess
from pathlib import Path

import pytest

REPO = Path(__file__).resolve().parents[1]


def test_admission_policy(tmp_path):
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    exe = tmp_path / "admission_test"
    r = subprocess.run([cxx, "-std=c++17", "-O1", "-Wall", str(REPO / "tests" / "cpp" / "admission_test.cpp"), "-I",
                        str(REPO / "hm-cupano_gb300" / "csrc"), "-o", str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0 and r.stdout.strip().endswith("OK"), r.stdout
