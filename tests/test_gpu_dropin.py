"""The drop-in itself: QuEST's own host code (API, localiser, accelerator -- the reference's
unchanged sources) over this repository's backend.  The QuEST sources are built with the
two shims of quest_gb300/shim in place of quest/src/gpu/ (COMPILE_CUDA=1, no MPI, no
cuQuantum), and the circuit runner of oracle/ref_harness.cpp is linked against the result
with GPU-accelerated Quregs.  The committed golden fixtures (outputs of QuEST's CPU build)
then run through QuEST's API -> localiser -> accelerator -> shim -> GB300 kernels:
amplitudes and reductions within 1e-12 of the fixtures, sampled measurement outcomes
bit-exact.  Random circuits of every op are checked against the oracle the same way.

Needs a checkout of the QuEST sources, named by QUEST_SOURCES; skipped where there is none."""
import glob
import os
import subprocess

import numpy as np
import pytest

import qcircuits as qc

pytestmark = pytest.mark.gpu
TOL = 1e-12
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.environ.get("QUEST_SOURCES", "")
GOLDEN = sorted(glob.glob(os.path.join(os.path.dirname(__file__), "golden", "*.npz")))
DEFS = ["-DFLOAT_PRECISION=2", "-DCOMPILE_MPI=0", "-DCOMPILE_OPENMP=1", "-DCOMPILE_CUDA=1", "-DCOMPILE_CUQUANTUM=0"]

needs_sources = pytest.mark.skipif(not os.path.isdir(os.path.join(SRC, "quest", "src")),
                                   reason="QuEST sources not present (QUEST_SOURCES)")


@pytest.fixture(scope="module")
def quest_on_gb300(built_lib, tmp_path_factory):
    jobs = str(max(1, os.cpu_count() or 1))
    r = subprocess.run(["make", "-s", "-j" + jobs, "-C", os.path.join(ROOT, "quest_gb300", "shim"), "REF=" + SRC],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    shim_build = os.path.join(ROOT, "quest_gb300", "shim", "_build")
    out = str(tmp_path_factory.mktemp("dropin") / "libqref_gb300.so")
    cmd = ["g++", "-O2", "-std=c++17", "-fopenmp", "-fPIC", "-shared", "-w", "-I" + SRC] + DEFS + [
        "-DREF_HARNESS_GPU=1", os.path.join(ROOT, "oracle", "ref_harness.cpp"), "-o", out,
        "-L" + shim_build, "-lQuEST_gb300", "-Wl,-rpath," + shim_build]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    return qc.CircuitLib(out, "ref_run_circuit")


@needs_sources
@pytest.mark.parametrize("path", GOLDEN, ids=[os.path.basename(p)[:-4] for p in GOLDEN])
def test_golden_fixtures_through_quest_host_code(quest_on_gb300, path):
    z = np.load(path)
    out, res, outs = quest_on_gb300.run(str(z["text"]), int(z["nq"]), int(z["is_dm"]), z["amps_in"])
    assert np.max(np.abs(out - z["amps_out"])) <= TOL
    assert res.shape == z["results"].shape and np.max(np.abs(res - z["results"]), initial=0) <= TOL
    assert outs.tolist() == z["outcomes"].tolist()


@needs_sources
@pytest.mark.parametrize("nq,is_dm,seed", [(5, 0, 301), (11, 0, 302), (16, 0, 303), (4, 1, 304), (7, 1, 305)])
def test_every_op_through_quest_host_code(quest_on_gb300, nq, is_dm, seed):
    text = qc.every_op_circuit(nq, is_dm, seed)
    amps = qc.random_density_matrix(nq, seed) if is_dm else qc.random_statevector(nq, seed)
    a1, r1, o1 = qc.oracle().run(text, nq, is_dm, amps)
    a2, r2, o2 = quest_on_gb300.run(text, nq, is_dm, amps)
    assert np.max(np.abs(a1 - a2)) <= TOL
    assert np.max(np.abs(r1 - r2)) <= TOL
    assert o1.tolist() == o2.tolist()
