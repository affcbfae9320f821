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
