"""QuEST's own host code links against this backend: the reference's api/,
core/, cpu/ and comm/ sources plus the two shims in quest_gb300/shim/ build into
one library with no undefined symbols, exporting QuEST's public API.  Needs the
QuEST sources; skipped elsewhere (they do not exist on the GPU machine)."""
import ctypes
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF = os.environ.get("QUEST_SOURCES", "/root/reference")   # a checkout of the QuEST sources, where one exists


@pytest.mark.skipif(not os.path.isdir(os.path.join(REF, "quest", "src")), reason="QuEST sources not present")
def test_quest_host_code_links_with_the_backend(built_lib):
    r = subprocess.run(["make", "-s", "-j8", "-C", os.path.join(ROOT, "quest_gb300", "shim"), "REF=" + REF],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    so = os.path.join(ROOT, "quest_gb300", "shim", "_build", "libQuEST_gb300.so")
    lib = ctypes.CDLL(so)
    for name in ("createQureg", "applyCompMatr1", "applyHadamard", "mixDepolarising", "mixKrausMap",
                 "calcTotalProb", "calcExpecPauliStr", "calcProbOfQubitOutcome", "applyQuantumFourierTransform"):
        assert hasattr(lib, name), name
