"""The CPU oracle against golden fixtures produced by the reference QuEST
library itself (tests/golden/make_golden.py) and, where the reference was built
in this checkout, against the reference directly on fresh random circuits."""
import glob
import os

import numpy as np
import pytest

import qcircuits as qc

GOLDEN = sorted(glob.glob(os.path.join(os.path.dirname(__file__), "golden", "*.npz")))


def load(path):
    z = np.load(path)
    return str(z["text"]), int(z["nq"]), int(z["is_dm"]), z["amps_in"], z["amps_out"], z["results"], z["outcomes"]


def test_golden_fixtures_exist():
    assert len(GOLDEN) >= 10


@pytest.mark.parametrize("path", GOLDEN, ids=[os.path.basename(p)[:-4] for p in GOLDEN])
def test_oracle_matches_reference_golden(path):
    text, nq, is_dm, amps_in, amps_out, results, outcomes = load(path)
    out, res, outs = qc.oracle().run(text, nq, is_dm, amps_in)
    # FP64 parity bar: 1e-12 max-abs per amplitude and per reduction; outcomes bit-exact
    assert np.max(np.abs(out - amps_out)) <= 1e-12
    assert res.shape == results.shape and np.max(np.abs(res - results), initial=0) <= 1e-12
    assert outs.tolist() == outcomes.tolist()


REF = qc.reference()


@pytest.mark.skipif(REF is None, reason="reference library not built in this checkout (make -C oracle ref REF=...)")
@pytest.mark.parametrize("nq,is_dm,seed", [(3, 0, 101), (7, 0, 102), (9, 0, 103), (3, 1, 104), (4, 1, 105), (6, 1, 106)])
def test_oracle_matches_reference_live(nq, is_dm, seed):
    text = qc.every_op_circuit(nq, is_dm, seed)
    amps = qc.random_density_matrix(nq, seed) if is_dm else qc.random_statevector(nq, seed)
    a1, r1, o1 = qc.oracle().run(text, nq, is_dm, amps)
    a2, r2, o2 = REF.run(text, nq, is_dm, amps)
    assert np.max(np.abs(a1 - a2)) <= 1e-12
    assert np.max(np.abs(r1 - r2)) <= 1e-12
    assert o1.tolist() == o2.tolist()


def test_oracle_planted_mistake_is_caught():
    """A wrong gate constant in the circuit (planted on the CPU) must break parity."""
    path = [p for p in GOLDEN if "sv5_every" in p][0]
    text, nq, is_dm, amps_in, amps_out, results, outcomes = load(path)
    bad = text.replace("\nT ", "\nS ", 1)
    assert bad != text
    out, _, _ = qc.oracle().run(bad, nq, is_dm, amps_in)
    assert np.max(np.abs(out - amps_out)) > 1e-6


def test_superoperator_matches_numpy():
    rng = np.random.default_rng(5)
    ops = qc.random_kraus(2, 3, rng)
    import ctypes
    lib = qc.oracle().lib
    flat = np.ascontiguousarray(np.stack(ops))
    out = np.zeros((16, 16), dtype=np.complex128)
    lib.orc_build_superop(out.ctypes.data_as(ctypes.c_void_p), flat.ctypes.data_as(ctypes.c_void_p), 3, 2)
    expect = sum(np.kron(o.conj(), o) for o in ops)
    assert np.max(np.abs(out - expect)) < 1e-14
