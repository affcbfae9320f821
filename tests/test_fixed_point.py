"""The block-floating fixed-point pair arithmetic (quest_gb300/csrc/qg_fixed.cuh),
compiled for the host and checked against long-double evaluation: Haar and general
2x2 operators, pairs whose members differ by up to 2^80 in magnitude, zeros,
denormals, and the cases that must go to FP64 (Inf, NaN, results outside the
normal range)."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "..", "quest_gb300", "csrc")


def test_fixed_point_pairs_within_bound(tmp_path):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not available")
    exe = str(tmp_path / "fx_check")
    subprocess.run([gxx, "-O2", "-std=c++17", "-I", CSRC, os.path.join(HERE, "fx_check.cpp"), "-o", exe], check=True)
    out = subprocess.run([exe], capture_output=True, text=True)
    assert out.returncode == 0, out.stdout + out.stderr
    assert out.stdout.startswith("OK"), out.stdout


def test_product_mode_switch(built_lib):
    import ctypes
    from quest_gb300._lib import lib
    L = lib()
    mode = ctypes.c_int(-1)
    assert L.qg_get_fp64_products(ctypes.byref(mode)) == 0 and mode.value == 0
    assert L.qg_set_fp64_products(2) != 0
    assert L.qg_set_fp64_products(1) == 0
    assert L.qg_get_fp64_products(ctypes.byref(mode)) == 0 and mode.value == 1
    assert L.qg_set_fp64_products(0) == 0


def test_kernel_shape_table_and_tuning_file(built_lib, tmp_path):
    import ctypes
    from quest_gb300._lib import lib
    L = lib()
    ppt, thr = ctypes.c_int(), ctypes.c_int()
    assert L.qg_get_kernel_shape(0, ctypes.byref(ppt), ctypes.byref(thr)) == 0
    assert (ppt.value, thr.value) == (1, 256)
    assert L.qg_set_kernel_shape(0, 3, 256) != 0          # not a compiled shape
    assert L.qg_set_kernel_shape(3, 1, 256) != 0          # no such kernel
    assert L.qg_set_kernel_shape(0, 2, 128) == 0
    path = str(tmp_path / "tune.txt").encode()
    assert L.qg_tune_save(path) == 0
    text = open(path.decode()).read().splitlines()
    assert text[0] == "qg-tune 1" and text[1].split()[1:] == ["dense1_fx", "2", "128"]
    assert text[2].split()[1:] == ["diag1_fx", "1", "256"]
    assert text[3].split()[1:] == ["dense2_fx", "1", "256"]
    assert L.qg_set_kernel_shape(0, 1, 256) == 0
    n = ctypes.c_int(-1)
    assert L.qg_tune_load(path, ctypes.byref(n)) == 0 and n.value == 3
    assert L.qg_get_kernel_shape(0, ctypes.byref(ppt), ctypes.byref(thr)) == 0
    assert (ppt.value, thr.value) == (2, 128)
    # lines for another device are skipped
    with open(path.decode(), "w") as f:
        f.write("qg-tune 1\nOther_GPU dense1_fx 2 256\n")
    assert L.qg_tune_load(path, ctypes.byref(n)) == 0 and n.value == 0
    bad = str(tmp_path / "bad.txt").encode()
    open(bad.decode(), "w").write("something else\n")
    assert L.qg_tune_load(bad, ctypes.byref(n)) != 0
    assert L.qg_set_kernel_shape(0, 1, 256) == 0
