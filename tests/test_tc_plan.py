"""The tensor-core block kernel's plan (quest_gb300/csrc/qg_tc_plan.h), compiled for
the host: the mode chosen for a target set, and the staged modes' index tables
(address-order loads and stores through shared memory) evaluated with the kernel's
own expressions on whole tiles of measured and random target sets."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "..", "quest_gb300", "csrc")


def test_block_plan_tables(tmp_path):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not available")
    exe = str(tmp_path / "tc_plan_check")
    subprocess.run([gxx, "-O2", "-std=c++17", "-I", CSRC, os.path.join(HERE, "tc_plan_check.cpp"), "-o", exe], check=True)
    out = subprocess.run([exe], capture_output=True, text=True)
    assert out.returncode == 0, out.stdout + out.stderr
    assert out.stdout.startswith("OK"), out.stdout
