"""The integer hi/lo split of the mixed path (shamrock_gb300/csrc/split64.cuh) against the
FP64 conversions it replaces, compiled for the host with g++ (the header is plain C++)."""

import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


def test_split64_matches_fp64_conversions(tmp_path):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not available")
    exe = tmp_path / "split64_check"
    subprocess.run([gxx, "-O2", "-std=c++17", "-o", str(exe),
                    os.path.join(HERE, "native", "split64_check.cpp")], check=True)
    r = subprocess.run([str(exe), "3000000"], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "mismatches 0" in r.stdout
