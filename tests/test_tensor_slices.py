"""The exact 8-bit slice arithmetic of the tensor-core dense kernel
(quest_gb300/csrc/qg_slices.h), compiled for the host: digits that add back to each
value, digit sums below 2^22, outputs within (KR + 2) 2^-53 of the group's and the
operator's largest magnitudes against long double, and the groups that must go to FP64.
Also the process-wide switch (qg_set_tensor_slices)."""
import ctypes
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "..", "quest_gb300", "csrc")


def test_slices_within_bound(tmp_path):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not available")
    exe = str(tmp_path / "slices_check")
    subprocess.run([gxx, "-O2", "-std=c++17", "-I", CSRC, os.path.join(HERE, "slices_check.cpp"), "-o", exe], check=True)
    out = subprocess.run([exe], capture_output=True, text=True)
    assert out.returncode == 0, out.stdout + out.stderr
    assert out.stdout.startswith("OK"), out.stdout


def test_tensor_slices_switch(built_lib):
    from quest_gb300._lib import lib
    L = lib()
    mode = ctypes.c_int(-1)
    assert L.qg_get_tensor_slices(ctypes.byref(mode)) == 0 and mode.value == 1
    assert L.qg_set_tensor_slices(3) != 0
    assert L.qg_set_tensor_slices(-1) != 0
    for m in (0, 2, 1):
        assert L.qg_set_tensor_slices(m) == 0
        assert L.qg_get_tensor_slices(ctypes.byref(mode)) == 0 and mode.value == m
