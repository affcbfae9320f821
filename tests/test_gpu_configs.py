"""GPU parity at the benchmark configurations' own circuits and sizes, against the
CPU oracle (pinned to the reference library by the golden fixtures).

* the plain method at its stated size: 20 qubits, 10 layers, total probability and
  16 Pauli expectation values;
* the 30-qubit benchmark's circuit (depth-20 Haar layers with 15 controlled phases
  each, then the full QFT) at 26 qubits, in both product modes of the one-target
  gates (block-floating fixed point, the default, and IEEE FP64);
* the density-matrix method (30 layers of unitaries, depolarising on every qubit and
  a two-qubit Kraus map, then purity and 16 Pauli expectation values) at 12 and
  14 qubits (a 4 GiB Choi vector at 14);
* outcome histograms of statevectors and density matrices, and their determinism.

Bar: FP64 max-abs difference per amplitude and per reduction <= 1e-12."""
import ctypes

import numpy as np
import pytest

import qcircuits as qc

pytestmark = pytest.mark.gpu
TOL = 1e-12


def run_gpu(env, text, nq, is_dm, amps):
    from quest_gb300.circuit import run_text
    Q = env.Q
    q = Q.createDensityQureg(nq) if is_dm else Q.createQureg(nq)
    try:
        env.set_amps(q, amps)
        res, outs = run_text("SEED 0\n" + text, q)
        out = env.get_amps(q)
    finally:
        Q.destroyQureg(q)
    return out, res, outs


benchmark_circuit_text = qc.benchmark_circuit_text


def test_config1_full_size(env):
    """The plain method at its stated size: 20 qubits, 10 x (H on all, RX/RY/RZ on every
    qubit, CNOT ladder), then calcTotalProb and 16 Pauli expectation values."""
    nq = 20
    text = qc.config1_circuit(nq, 10, 0x5155455354 + 1)
    amps = qc.random_statevector(nq, 0x5155455354 + 1)
    a1, r1, _ = qc.oracle().run(text, nq, 0, amps)
    a2, r2, _ = run_gpu(env, text, nq, 0, amps)
    assert len(text.splitlines()) == 10 * (20 + 60 + 19) + 17
    assert r1.size == 17
    assert np.max(np.abs(a1 - a2)) <= TOL
    assert np.max(np.abs(r1 - r2)) <= TOL


def test_benchmark_circuit_26q_both_product_modes(env):
    """The 30-qubit benchmark circuit (depth 20, 15 controlled phases per layer, QFT) at
    26 qubits (1 GiB) in the default fixed-point mode and with IEEE FP64 products."""
    from quest_gb300 import _lib
    L = _lib.lib()
    nq = 26
    text = benchmark_circuit_text(nq, 20, 0x5155455354 + 2)
    amps = qc.random_statevector(nq, 0x5155455354 + 2)
    a_orc, r_orc, _ = qc.oracle().run(text, nq, 0, amps)
    outs = {}
    mode = ctypes.c_int(-1)
    _lib.check(L.qg_get_fp64_products(ctypes.byref(mode)))
    try:
        for m in (0, 1):
            _lib.check(L.qg_set_fp64_products(m))
            outs[m] = run_gpu(env, text, nq, 0, amps)
    finally:
        _lib.check(L.qg_set_fp64_products(mode.value))
    errs = {m: float(np.max(np.abs(outs[m][0] - a_orc))) for m in outs}
    between = float(np.max(np.abs(outs[0][0] - outs[1][0])))
    print(f"\n26q benchmark circuit: max-abs vs oracle fixed-point {errs[0]:.3e}, IEEE FP64 {errs[1]:.3e}; "
          f"between the modes {between:.3e}; total prob {outs[0][1][0]!r} / {outs[1][1][0]!r}")
    for m in outs:
        assert errs[m] <= TOL, (m, errs[m])
        assert abs(outs[m][1][0] - r_orc[0]) <= TOL
    assert between <= TOL


@pytest.mark.parametrize("nq", [12, 14])
def test_config3_density_matrix(env, nq):
    """The density-matrix method: 30 layers of random 1-/2-qubit unitaries, each followed
    by mixDepolarising(0.01) on every qubit and a random 2-qubit 4-operator Kraus map,
    then calcPurity and 16 Pauli expectation values."""
    text = qc.config3_circuit(nq, 30, 0x5155455354 + 3)
    amps = qc.random_density_matrix(nq, 0x5155455354 + 3)
    a1, r1, _ = qc.oracle().run(text, nq, 1, amps)
    a2, r2, _ = run_gpu(env, text, nq, 1, amps)
    assert r1.size == 17
    assert np.max(np.abs(a1 - a2)) <= TOL
    assert np.max(np.abs(r1 - r2)) <= TOL


@pytest.mark.parametrize("nq,is_dm,qubits", [(14, 0, [3]), (14, 0, [13, 0, 6]), (20, 0, [19, 2, 11, 5, 0, 7, 14]),
                                             (9, 0, list(range(9))), (6, 1, [5, 1]), (7, 1, [0, 2, 4, 6]),
                                             (5, 1, [4, 3, 2, 1, 0])])
def test_probs_of_all_outcomes(env, nq, is_dm, qubits):
    """calcProbsOfAllMultiQubitOutcomes against the oracle's histogram (bin b holds the
    outcome whose bit i is qubits[i]); a second call gives identical bits."""
    amps = qc.random_density_matrix(nq, nq) if is_dm else qc.random_statevector(nq, nq)
    k = len(qubits)
    text = f"PROBALL {k} {' '.join(map(str, qubits))}\n"
    _, r1, _ = qc.oracle().run(text, nq, is_dm, amps)
    Q = env.Q
    q = Q.createDensityQureg(nq) if is_dm else Q.createQureg(nq)
    try:
        env.set_amps(q, amps)
        got = []
        for _ in range(2):
            out = (ctypes.c_double * (1 << k))()
            Q.calcProbsOfAllMultiQubitOutcomes(out, q, env.ints(qubits), k)
            got.append(np.array(out[:]))
        # the other reductions still work after the histogram (its scratch is kept apart)
        tp = Q.calcTotalProb(q)
    finally:
        Q.destroyQureg(q)
    assert np.max(np.abs(got[0] - r1)) <= TOL
    assert got[0].tobytes() == got[1].tobytes()
    assert abs(tp - np.sum(r1)) <= 1e-12


def test_multi_qubit_measurement_outcomes_bit_exact(env):
    """applyMultiQubitMeasurement[AndGetProb] and the forced forms: outcomes equal the
    oracle's under the same seeds (bit-exact), probabilities and states within 1e-12."""
    rng = np.random.default_rng(404)
    for trial in range(12):
        nq = int(rng.integers(4, 12))
        is_dm = trial % 3 == 2
        if is_dm:
            nq = min(nq, 6)
        amps = qc.random_density_matrix(nq, 500 + trial) if is_dm else qc.random_statevector(nq, 500 + trial)
        qs = [int(v) for v in rng.choice(nq, size=int(rng.integers(1, nq + 1)), replace=False)]
        lines = [f"SEED {int(rng.integers(1 << 31))} {int(rng.integers(1 << 31))}",
                 f"MEASM {len(qs)} {' '.join(map(str, qs))}", "TOTALPROB"]
        rest = [q for q in range(nq) if q not in qs]
        if rest:
            lines.append(f"FMEAS {rest[0]} {int(rng.integers(2))}")
        lines.append(f"MEASM 1 {int(rng.integers(nq))}")
        text = "\n".join(lines) + "\n"
        a1, r1, o1 = qc.oracle().run(text, nq, is_dm, amps)
        a2, r2, o2 = run_gpu(env, text, nq, is_dm, amps)
        assert o1.tolist() == o2.tolist(), (trial, o1, o2)
        assert np.max(np.abs(r1 - r2)) <= TOL
        assert np.max(np.abs(a1 - a2)) <= TOL


@pytest.mark.parametrize("nq,is_dm,terms", [(10, 0, 3), (18, 0, 40), (5, 1, 7), (8, 1, 33)])
def test_pauli_str_sum_vs_oracle(env, nq, is_dm, terms):
    """calcExpecPauliStrSum (several strings per pass) against the oracle's per-string loop,
    with more terms than one pass takes."""
    rng = np.random.default_rng(nq * 7 + terms)
    amps = qc.random_density_matrix(nq, 9) if is_dm else qc.random_statevector(nq, 9)
    text = qc.expsum_line(nq, terms, rng) + "\n" + f"EXPSUM 1 0.25 0.0 {'I' * nq}\n"
    _, r1, _ = qc.oracle().run(text, nq, is_dm, amps)
    _, r2, _ = run_gpu(env, text, nq, is_dm, amps)
    assert np.max(np.abs(r1 - r2)) <= TOL


def test_pauli_str_sum_validation(env):
    Q = env.Q
    q = Q.createQureg(4)
    try:
        bad = env.pauli_str_sum([1.0, 0.5j], ["XIII", "ZZII"])
        with pytest.raises(env.QuESTError):
            Q.calcExpecPauliStrSum(q, bad)
        Q.destroyPauliStrSum(bad)
        wide = env.pauli_str_sum([1.0], ["IIIIX"])
        with pytest.raises(env.QuESTError):
            Q.calcExpecPauliStrSum(q, wide)
        Q.destroyPauliStrSum(wide)
    finally:
        Q.destroyQureg(q)


@pytest.mark.parametrize("nq,seed,slices", [(3, 1, 1), (6, 2, 1), (9, 3, 1), (3, 4, 2), (6, 5, 2), (9, 6, 2)])
def test_deferred_density_matrix_superoperators(env, nq, seed, slices):
    """One-qubit unitaries and channels on a density matrix are multiplied into one
    pending superoperator per qubit and applied when something needs the state; random
    interleavings with two-qubit operations (which apply only the qubits they touch),
    controlled gates, rotations and reductions in between, against the oracle applying
    every operation at once.  With the tensor-core kernel forced (slices = 2) the pending
    qubits pair up, and a two-qubit unitary or Kraus map takes its qubits' pending
    superoperators into its own pass."""
    rng = np.random.default_rng(900 + seed)
    L = []
    for step in range(60):
        q = int(rng.integers(nq))
        kind = int(rng.integers(12))
        if kind == 0:
            L.append(f"U1 {q} {qc.mat_tokens(qc.haar_unitary(2, rng))}")
        elif kind == 1:
            L.append(f"DEPOL {q} {qc.fmt(rng.uniform(0, 0.3))}")
        elif kind == 2:
            L.append(f"DEPHASE {q} {qc.fmt(rng.uniform(0, 0.3))}")
        elif kind == 3:
            L.append(f"DAMP {q} {qc.fmt(rng.uniform(0, 0.5))}")
        elif kind == 4:
            px, py, pz = rng.uniform(0, 0.1, 3)
            L.append(f"PAULIS {q} {qc.fmt(px)} {qc.fmt(py)} {qc.fmt(pz)}")
        elif kind == 5:
            L.append(f"KRAUS 1 {q} 3 " + " ".join(qc.mat_tokens(o) for o in qc.random_kraus(1, 3, rng)))
        elif kind == 6:
            L.append(f"H {q}")
        elif kind == 7 and nq >= 2:
            a, b = (int(v) for v in rng.choice(nq, 2, replace=False))
            L.append(f"U2 {a} {b} {qc.mat_tokens(qc.haar_unitary(4, rng))}")
        elif kind == 8 and nq >= 2:
            a, b = (int(v) for v in rng.choice(nq, 2, replace=False))
            L.append(rng.choice([f"DEPOL2 {a} {b} {qc.fmt(rng.uniform(0, 0.3))}",
                                 f"DEPHASE2 {a} {b} {qc.fmt(rng.uniform(0, 0.3))}",
                                 f"KRAUS 2 {a} {b} 2 " + " ".join(qc.mat_tokens(o) for o in qc.random_kraus(2, 2, rng))]))
        elif kind == 9 and nq >= 2:
            a, b = (int(v) for v in rng.choice(nq, 2, replace=False))
            L.append(f"CU1 1 {a} 1 {b} {qc.mat_tokens(qc.haar_unitary(2, rng))}")
        elif kind == 10:
            L.append(f"RY {q} {qc.fmt(rng.uniform(0, 6.3))}")
        else:
            L.append(rng.choice(["TOTALPROB", "PURITY", f"PROBQ {q} 0",
                                 f"EXPEC {qc.pauli_text([int(v) for v in rng.integers(0, 4, nq)])}"]))
    L += ["PURITY", f"EXPEC {'X' * nq}", "TOTALPROB"]
    text = "\n".join(L) + "\n"
    amps = qc.random_density_matrix(nq, 950 + seed)
    a1, r1, _ = qc.oracle().run(text, nq, 1, amps)
    from quest_gb300 import _lib
    L = _lib.lib()
    before = ctypes.c_int(1)
    _lib.check(L.qg_get_tensor_slices(ctypes.byref(before)))
    _lib.check(L.qg_set_tensor_slices(slices))
    try:
        a2, r2, _ = run_gpu(env, text, nq, 1, amps)
    finally:
        _lib.check(L.qg_set_tensor_slices(before.value))
    assert np.max(np.abs(a1 - a2)) <= TOL
    assert np.max(np.abs(r1 - r2)) <= TOL


def test_deferred_superoperators_applied_by_sync_and_overwritten_by_set(env):
    """syncQuESTEnv applies the pending superoperators of every density matrix; a full
    setDensityQuregFlatAmps replaces the state, pending operations included."""
    import ctypes
    Q = env.Q
    nq = 4
    amps = qc.random_density_matrix(nq, 77)
    rng = np.random.default_rng(78)
    u = qc.haar_unitary(2, rng)
    text = f"U1 2 {qc.mat_tokens(u)}\nDEPOL 2 0.125\nDAMP 0 0.25\n"
    want, _, _ = qc.oracle().run(text, nq, 1, amps)
    q = Q.createDensityQureg(nq)
    try:
        env.set_amps(q, amps)
        Q.applyCompMatr1(q, 2, env.comp_matr1(u))
        Q.mixDepolarising(q, 2, 0.125)
        Q.mixDamping(q, 0, 0.25)
        Q.syncQuESTEnv()
        raw = np.empty(1 << (2 * nq), dtype=np.complex128)     # the device state, read without the API
        from quest_gb300 import _lib
        _lib.check(_lib.lib().qg_copy_d2h(raw.ctypes.data, ctypes.cast(q.gpuAmps, ctypes.c_void_p), raw.nbytes, None))
        assert np.max(np.abs(raw - want)) <= TOL
        Q.mixDepolarising(q, 1, 0.3)         # pending, then overwritten
        env.set_amps(q, amps)
        assert np.max(np.abs(env.get_amps(q) - amps)) == 0
    finally:
        Q.destroyQureg(q)
