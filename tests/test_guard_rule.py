"""The estimate refresh rule of the error-controlled mixed precision
(shamrock_gb300/csrc/guard_rule.h, plain C++ used by the step driver), compiled for the
host with g++ and checked on its cases."""

import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


def test_refresh_rule_cases(tmp_path):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not available")
    exe = tmp_path / "guard_rule_check"
    subprocess.run([gxx, "-O2", "-std=c++17", "-o", str(exe),
                    os.path.join(HERE, "native", "guard_rule_check.cpp")], check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "failures 0" in r.stdout
