"""Host-side logic of the API layer that runs without a GPU: Pauli-string
packing, Kraus superoperator construction, matrix structs, error handler."""
import ctypes

import numpy as np
import pytest

import qcircuits as qc


@pytest.fixture(scope="module")
def api(built_lib):
    from quest_gb300 import api as A
    A.Q._get("setInputErrorHandler")(A._handler)   # raising handler; no GPU environment needed
    return A


def test_pauli_str_packing_matches_reference_layout(api):
    # paulis.h:53-60: base-4 digits, qubit q at bits 2q (low mask) / 2(q-32) (high mask)
    p = api.pauli_str([0, 1, 2, 3])
    assert p.lowPaulis == (1 << 2) | (2 << 4) | (3 << 6) and p.highPaulis == 0
    codes = [0] * 40
    codes[33] = 2
    codes[5] = 3
    p = api.pauli_str(codes)
    assert p.lowPaulis == 3 << 10 and p.highPaulis == 2 << 2


def test_pauli_code_validation_raises(api):
    with pytest.raises(api.QuESTError):
        api.Q.getPauliStrFromCodes(api.ints([5]), api.ints([0]), 1)


def test_kraus_superoperator_built_on_host(api):
    rng = np.random.default_rng(3)
    for k in (1, 2):
        ops = np.stack(qc.random_kraus(k, 4, rng))
        km = api.kraus_map(ops)
        sd = 1 << (2 * k)
        got = np.ctypeslib.as_array(ctypes.cast(km.superop.cpuElemsFlat, ctypes.POINTER(ctypes.c_double)), shape=(sd * sd * 2,))
        got = (got[0::2] + 1j * got[1::2]).reshape(sd, sd)
        expect = sum(np.kron(o.conj(), o) for o in ops)
        assert np.max(np.abs(got - expect)) < 1e-14
        api.Q.destroyKrausMap(km)


def test_comp_matr_roundtrip(api):
    rng = np.random.default_rng(4)
    u = qc.haar_unitary(8, rng)
    m = api.comp_matr(u)
    assert m.numQubits == 3 and m.numRows == 8
    flat = np.ctypeslib.as_array(ctypes.cast(m.cpuElemsFlat, ctypes.POINTER(ctypes.c_double)), shape=(128,))
    assert np.array_equal(flat[0::2] + 1j * flat[1::2], u.reshape(-1))
    api.Q.destroyCompMatr(m)


def test_api_without_env_reports_error(api):
    """Calls before initQuESTEnv go to the input-error handler, like the reference."""
    if api.Q._get("isQuESTEnvInit")():
        pytest.skip("environment already initialised in this process")
    with pytest.raises(api.QuESTError):
        api.Q.createQureg(3)


def test_deferred_statevector_gates_on_the_host(built_lib, tmp_path):
    """The API's deferral of one-qubit gates and controlled phases on statevectors
    (tests/deferral_check.cpp): the API source compiled against CPU stand-ins of the pass
    kernels, random layered circuits through the public calls equal the gate-by-gate product,
    and benchmark-shaped layers take the expected number of passes and no phase pass."""
    import os
    import shutil
    import subprocess
    from quest_gb300 import build
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not available")
    here = os.path.dirname(os.path.abspath(__file__))
    root = os.path.dirname(here)
    libdir = os.path.dirname(built_lib)
    cuda = build._cuda_home()
    exe = str(tmp_path / "deferral_check")
    subprocess.run([gxx, "-O2", "-std=c++17", "-I", os.path.join(root, "include"), "-I", os.path.join(root, "quest_gb300", "csrc"),
                    "-I", os.path.join(cuda, "include"), os.path.join(here, "deferral_check.cpp"), "-o", exe,
                    "-L", libdir, "-lquest_gb300", "-L", os.path.join(cuda, "lib64"), "-lcudart",
                    "-Wl,-rpath," + libdir], check=True)
    out = subprocess.run([exe], capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stdout[-3000:]
    assert out.stdout.strip().splitlines()[-1].startswith("OK")
