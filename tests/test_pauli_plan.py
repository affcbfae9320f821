"""The tiled Pauli-expectation kernel's plan (quest_gb300/csrc/qg_pauli_plan.h),
compiled for the host: the grouping of strings into passes and each pass's tile
coordinates, evaluated with the kernel's own index expressions on random states and
string lists (low-only, high-only, Z-only and repeated strings), against the direct sum."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "..", "quest_gb300", "csrc")


def test_pauli_tile_plan(tmp_path):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not available")
    exe = str(tmp_path / "pauli_plan_check")
    subprocess.run([gxx, "-O2", "-std=c++17", "-Wall", "-I", CSRC, os.path.join(HERE, "pauli_plan_check.cpp"), "-o", exe],
                   check=True)
    out = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stdout + out.stderr
    assert out.stdout.startswith("OK"), out.stdout
