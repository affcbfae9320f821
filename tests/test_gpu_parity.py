"""GPU parity: the GB300 path (QuEST-named API over the C ABI) against the
CPU oracle and the reference's golden fixtures.

Bar (FP64): max-abs difference per amplitude and per reduction <= 1e-12;
index/permutation work and sampled measurement outcomes bit-exact."""
import glob
import os

import numpy as np
import pytest

import qcircuits as qc

pytestmark = pytest.mark.gpu
TOL = 1e-12
GOLDEN = sorted(glob.glob(os.path.join(os.path.dirname(__file__), "golden", "*.npz")))


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


@pytest.mark.parametrize("path", GOLDEN, ids=[os.path.basename(p)[:-4] for p in GOLDEN])
def test_golden_fixture_on_gpu(env, path):
    z = np.load(path)
    out, res, outs = run_gpu(env, str(z["text"]), int(z["nq"]), int(z["is_dm"]), z["amps_in"])
    assert np.max(np.abs(out - z["amps_out"])) <= TOL
    assert np.max(np.abs(res - z["results"]), initial=0) <= TOL
    assert outs.tolist() == z["outcomes"].tolist()


@pytest.mark.parametrize("nq,is_dm,seed", [(3, 0, 1), (4, 0, 2), (7, 0, 3), (10, 0, 4), (13, 0, 5), (16, 0, 6),
                                           (3, 1, 7), (5, 1, 8), (7, 1, 9)])
def test_every_op_vs_oracle(env, nq, is_dm, seed):
    text = qc.every_op_circuit(nq, is_dm, seed)
    amps = qc.random_density_matrix(nq, seed) if is_dm else qc.random_statevector(nq, seed)
    a1, r1, o1 = qc.oracle().run(text, nq, is_dm, amps)
    a2, r2, o2 = run_gpu(env, text, nq, is_dm, amps)
    assert np.max(np.abs(a1 - a2)) <= TOL
    assert np.max(np.abs(r1 - r2)) <= TOL
    assert o1.tolist() == o2.tolist()


@pytest.mark.parametrize("nq,layers", [(4, 6), (7, 4)])
def test_config3_shape_vs_oracle(env, nq, layers):
    """The density-matrix method's circuit shape (Haar layers, depolarising on every
    qubit, a 2-qubit Kraus map per layer, purity, 16 Pauli expectations) at small size."""
    text = qc.config3_circuit(nq, layers, 33 + nq)
    amps = qc.random_density_matrix(nq, 33 + nq)
    a1, r1, _ = qc.oracle().run(text, nq, 1, amps)
    a2, r2, _ = run_gpu(env, text, nq, 1, amps)
    assert np.max(np.abs(a1 - a2)) <= TOL
    assert r1.size == 17 and np.max(np.abs(r1 - r2)) <= TOL


def test_config1_shape_vs_oracle(env):
    """The plain method's circuit shape at 14 qubits, 4 layers."""
    nq = 14
    text = qc.config1_circuit(nq, 4, 77)
    amps = qc.random_statevector(nq, 77)
    a1, r1, _ = qc.oracle().run(text, nq, 0, amps)
    a2, r2, _ = run_gpu(env, text, nq, 0, amps)
    assert np.max(np.abs(a1 - a2)) <= TOL
    assert np.max(np.abs(r1 - r2)) <= TOL


def _all_ctrl_targ_cases(n, rng):
    """Every target (and target pair) with 0, 1 and 2 controls in random states."""
    cases = []
    for t in range(n):
        others = [q for q in range(n) if q != t]
        cases.append(([], [], [t]))
        for c in others:
            cases.append(([c], [int(rng.integers(2))], [t]))
        c2 = [int(v) for v in rng.choice(others, 2, replace=False)]
        cases.append((c2, [int(v) for v in rng.integers(0, 2, 2)], [t]))
    for t1 in range(n):
        for t2 in range(n):
            if t1 != t2:
                others = [q for q in range(n) if q not in (t1, t2)]
                c = [int(rng.choice(others))]
                cases.append(([], [], [t1, t2]))
                cases.append((c, [int(rng.integers(2))], [t1, t2]))
    return cases


def test_every_ctrl_and_target_permutation(env):
    """All single/pair target placements with controls, for dense, diagonal,
    swap and Pauli ops, at 7 qubits (the reference's unit tests enumerate
    ctrl/target permutations the same way)."""
    n = 7
    rng = np.random.default_rng(2024)
    lines = []
    for c, s, t in _all_ctrl_targ_cases(n, rng):
        nc = len(c)
        pre = f"{nc} {' '.join(map(str, c))} {' '.join(map(str, s))}".replace("  ", " ")
        if len(t) == 1:
            m = qc.mat_tokens(qc.haar_unitary(2, rng))
            lines.append(f"CU1 {pre} {t[0]} {m}" if nc else f"U1 {t[0]} {m}")
            d = qc.mat_tokens(np.exp(1j * rng.uniform(0, 6.3, 2)))
            lines.append(f"CDK {pre} 1 {t[0]} {d}" if nc else f"D1 {t[0]} {d}")
            codes = [0] * n
            codes[t[0]] = int(rng.integers(1, 4))
            lines.append(f"CPSTR {pre} {qc.pauli_text(codes)}" if nc else f"PSTR {qc.pauli_text(codes)}")
            lines.append(f"CPG {pre} {qc.pauli_text(codes)} {qc.fmt(rng.uniform(0, 6.3))}" if nc else f"PG {qc.pauli_text(codes)} {qc.fmt(rng.uniform(0, 6.3))}")
        else:
            m = qc.mat_tokens(qc.haar_unitary(4, rng))
            lines.append(f"CU2 {pre} {t[0]} {t[1]} {m}" if nc else f"U2 {t[0]} {t[1]} {m}")
            lines.append(f"CSWAP {pre} {t[0]} {t[1]}" if nc else f"SWAP {t[0]} {t[1]}")
            d = qc.mat_tokens(np.exp(1j * rng.uniform(0, 6.3, 4)))
            lines.append(f"CDK {pre} 2 {t[0]} {t[1]} {d}" if nc else f"D2 {t[0]} {t[1]} {d}")
    lines.append("TOTALPROB")
    text = "\n".join(lines) + "\n"
    for is_dm, nq in ((0, n), (1, 3)):
        if is_dm:
            # density matrices use only qubits < 3 from the same op kinds
            sub = [l for l in lines if all(int(tok) < 3 for tok in _qubit_tokens(l))]
            text_dm = "\n".join(sub) + "\n"
            amps = qc.random_density_matrix(nq, 9)
            a1, r1, _ = qc.oracle().run(text_dm, nq, 1, amps)
            a2, r2, _ = run_gpu(env, text_dm, nq, 1, amps)
        else:
            amps = qc.random_statevector(nq, 9)
            a1, r1, _ = qc.oracle().run(text, nq, 0, amps)
            a2, r2, _ = run_gpu(env, text, nq, 0, amps)
        assert np.max(np.abs(a1 - a2)) <= TOL
        assert np.max(np.abs(r1 - r2)) <= TOL


def _qubit_tokens(line):
    tok = line.split()
    op = tok[0]
    if op in ("U1", "D1"):
        return [tok[1]]
    if op in ("U2", "SWAP", "D2"):
        return tok[1:3]
    if op in ("PSTR", "PG"):
        return [str(i) for i, ch in enumerate(tok[1]) if ch != "I"]
    if op.startswith("C"):
        nc = int(tok[1])
        qs = tok[2:2 + nc]
        rest = tok[2 + 2 * nc:]
        if op in ("CU1",):
            return qs + [rest[0]]
        if op in ("CU2", "CSWAP"):
            return qs + rest[:2]
        if op == "CDK":
            k = int(rest[0])
            return qs + rest[1:1 + k]
        if op in ("CPSTR", "CPG"):
            return qs + [str(i) for i, ch in enumerate(rest[0]) if ch != "I"]
    return []


def test_dense_many_targets_vs_oracle(env):
    """Dense matrices of 3..8 targets (register, parameter-space and shared-memory paths)."""
    rng = np.random.default_rng(11)
    n = 10
    lines = []
    for k in (3, 4, 5, 6, 7, 8):
        t = [int(v) for v in rng.choice(n, k, replace=False)]
        lines.append(f"UK {k} {' '.join(map(str, t))} {qc.mat_tokens(qc.haar_unitary(1 << k, rng))}")
    c = [int(v) for v in rng.choice(n, 7, replace=False)]
    lines.append(f"CUK 1 {c[0]} 0 6 {' '.join(map(str, c[1:]))} {qc.mat_tokens(qc.haar_unitary(64, rng))}")
    text = "\n".join(lines) + "\nTOTALPROB\n"
    amps = qc.random_statevector(n, 12)
    a1, r1, _ = qc.oracle().run(text, n, 0, amps)
    a2, r2, _ = run_gpu(env, text, n, 0, amps)
    assert np.max(np.abs(a1 - a2)) <= TOL
    assert np.max(np.abs(r1 - r2)) <= TOL


def test_measurement_outcomes_bit_exact_under_shared_seed(env):
    nq = 12
    rng = np.random.default_rng(5)
    lines = [f"SEED {int(rng.integers(1 << 30))} {int(rng.integers(1 << 30))}"]
    for _ in range(3):
        for t in range(nq):
            lines.append(f"U1 {t} {qc.mat_tokens(qc.haar_unitary(2, rng))}")
        for t in range(0, nq - 1, 2):
            lines.append(f"CZ {t} {t + 1}")
        for t in rng.choice(nq, 3, replace=False):
            lines.append(f"MEAS {int(t)}")
    text = "\n".join(lines) + "\nTOTALPROB\n"
    amps = qc.random_statevector(nq, 6)
    a1, r1, o1 = qc.oracle().run(text, nq, 0, amps)
    a2, r2, o2 = run_gpu(env, text, nq, 0, amps)
    assert o1.tolist() == o2.tolist() and len(o1) == 9
    assert np.max(np.abs(a1 - a2)) <= TOL


def test_reductions_are_deterministic(env):
    Q = env.Q
    nq = 22
    q = Q.createQureg(nq)
    try:
        env.set_amps(q, qc.random_statevector(nq, 3))
        p = env.pauli_str("XYZI" * 5 + "XY")
        vals = [(Q.calcTotalProb(q), Q.calcExpecPauliStr(q, p), Q.calcProbOfQubitOutcome(q, 17, 1)) for _ in range(3)]
        assert vals[0] == vals[1] == vals[2]
    finally:
        Q.destroyQureg(q)


def test_large_state_properties(env):
    """Size-independent properties at 26 qubits (1 GiB): involutions and
    permutations are bit-exact, unitary layers keep the norm."""
    Q = env.Q
    nq = 26
    amps = qc.random_statevector(nq, 42)
    q = Q.createQureg(nq)
    try:
        env.set_amps(q, amps)
        for t in (0, 5, 13, 25):
            Q.applyPauliX(q, t)
            Q.applyPauliX(q, t)
        Q.applySwap(q, 3, 24)
        Q.applySwap(q, 24, 3)
        Q.applyControlledPauliX(q, 25, 0)
        Q.applyControlledPauliX(q, 25, 0)
        out = env.get_amps(q)
        assert np.array_equal(out, amps)
        # CNOT 0 -> 25 permutes amplitudes exactly like the numpy index map
        Q.applyControlledPauliX(q, 0, 25)
        out = env.get_amps(q)
        idx = np.arange(1 << nq)
        perm = np.where(idx & 1, idx ^ (1 << 25), idx)
        assert np.array_equal(out, amps[perm])
        rng = np.random.default_rng(1)
        for t in range(nq):
            Q.applyCompMatr1(q, t, env.comp_matr1(qc.haar_unitary(2, rng)))
        assert abs(Q.calcTotalProb(q) - 1) < 1e-11
    finally:
        Q.destroyQureg(q)


def test_invalid_input_raises(env):
    Q = env.Q
    q = Q.createQureg(4)
    try:
        with pytest.raises(env.QuESTError):
            Q.applyHadamard(q, 4)
        with pytest.raises(env.QuESTError):
            Q.applyControlledPauliX(q, 2, 2)
        with pytest.raises(env.QuESTError):
            Q.applyCompMatr1(q, 0, env.comp_matr1([[1, 1], [0, 1]]))   # not unitary
        with pytest.raises(env.QuESTError):
            Q.mixDepolarising(q, 0, 0.1)   # statevector
        d = Q.createDensityQureg(2)
        with pytest.raises(env.QuESTError):
            Q.mixDepolarising(d, 0, 0.8)   # beyond maximal mixing
        Q.destroyQureg(d)
    finally:
        Q.destroyQureg(q)


def test_abi_rejects_bad_arguments(env):
    from quest_gb300 import _lib
    L = _lib.lib()
    q = env.Q.createQureg(3)
    try:
        m = _lib.cplx_array([1, 0, 0, 1])
        assert L.qg_sv_anyCtrlOneTargDenseMatr(q.gpuAmps, 3, None, None, 0, 3, m, None) == -2
        assert L.qg_sv_anyCtrlSwap(q.gpuAmps, 3, None, None, 0, 1, 1, None) == -2
        assert L.qg_sv_anyCtrlOneTargDenseMatr(None, 3, None, None, 0, 0, m, None) == -2
    finally:
        env.Q.destroyQureg(q)


def test_l2_fetch_granularity_hint(env):
    # initialisation leaves the context at 32-byte L2 fetches; the setter takes only the
    # documented values
    import ctypes
    from quest_gb300 import _lib
    L = _lib.lib()
    v = ctypes.c_int(-1)
    _lib.check(L.qg_get_l2_fetch_granularity(ctypes.byref(v)))
    assert v.value == 32
    try:
        _lib.check(L.qg_set_l2_fetch_granularity(128))
        _lib.check(L.qg_get_l2_fetch_granularity(ctypes.byref(v)))
        assert v.value == 128
        assert L.qg_set_l2_fetch_granularity(48) == -2
        # the restore puts back what the context had before initialisation changed it
        _lib.check(L.qg_restore_l2_fetch_granularity())
        _lib.check(L.qg_get_l2_fetch_granularity(ctypes.byref(v)))
        assert v.value != 128
    finally:
        _lib.check(L.qg_set_l2_fetch_granularity(32))


@pytest.mark.parametrize("nq,is_dm,seed", [(1, 0, 61), (5, 0, 62), (12, 0, 63), (1, 1, 64), (4, 1, 65), (6, 1, 66)])
def test_fullstate_diag_vs_oracle(env, nq, is_dm, seed):
    """FullStateDiagMatr: apply / multiply with and without powers, and the four
    expectation forms, on statevectors and density matrices."""
    text = qc.fullstate_diag_circuit(nq, is_dm, seed)
    amps = qc.random_density_matrix(nq, seed) if is_dm else qc.random_statevector(nq, seed)
    a1, r1, _ = qc.oracle().run(text, nq, is_dm, amps)
    a2, r2, _ = run_gpu(env, text, nq, is_dm, amps)
    assert np.max(np.abs(a1 - a2)) <= TOL
    assert r1.size == r2.size and np.max(np.abs(r1 - r2)) <= TOL


def test_fullstate_diag_validation(env):
    """The reference's checks: apply needs a unitary diagonal, the Hermitian expectation a
    real one, and a negative power of a zero element diverges."""
    from quest_gb300.api import QuESTError, full_state_diag
    from quest_gb300._lib import qg_cplx
    Q = env.Q
    q = Q.createQureg(3)
    try:
        bad = full_state_diag(np.full(8, 0.5 + 0j))
        with pytest.raises(QuESTError):
            Q.applyFullStateDiagMatr(q, bad)
        Q.multiplyFullStateDiagMatr(q, bad)            # non-unitary is fine for multiply
        Q.destroyFullStateDiagMatr(bad)
        cplx = full_state_diag(np.full(8, 1j))
        with pytest.raises(QuESTError):
            Q.calcExpecFullStateDiagMatr(q, cplx)
        Q.destroyFullStateDiagMatr(cplx)
        zero = full_state_diag(np.zeros(8, dtype=complex))
        with pytest.raises(QuESTError):
            Q.multiplyFullStateDiagMatrPower(q, zero, qg_cplx(-1.0, 0.0))
        Q.destroyFullStateDiagMatr(zero)
        wrong = full_state_diag(np.ones(16, dtype=complex))
        with pytest.raises(QuESTError):
            Q.applyFullStateDiagMatr(q, wrong)
        Q.destroyFullStateDiagMatr(wrong)
    finally:
        Q.destroyQureg(q)


@pytest.mark.parametrize("nq,is_dm", [(9, 0), (5, 1), (7, 1)])
def test_pauli_batch_matches_oracle(env, nq, is_dm):
    """calcExpecPauliStrs (one pass per 16 strings, statevector and density matrix)
    against the oracle's one-string-at-a-time expectations; 40 strings cross a pass
    boundary."""
    import ctypes
    rng = np.random.default_rng(70 + nq + is_dm)
    codes = [[int(v) for v in rng.integers(0, 4, nq)] for _ in range(40)]
    amps = qc.random_density_matrix(nq, 70 + nq) if is_dm else qc.random_statevector(nq, 70 + nq)
    _, want, _ = qc.oracle().run("".join(f"EXPEC {qc.pauli_text(c)}\n" for c in codes), nq, is_dm, amps)
    Q = env.Q
    q = Q.createDensityQureg(nq) if is_dm else Q.createQureg(nq)
    try:
        env.set_amps(q, amps)
        strs = (env.PauliStr * len(codes))(*[env.pauli_str(c) for c in codes])
        got = (ctypes.c_double * len(codes))()
        Q.calcExpecPauliStrs(got, q, strs, len(codes))
    finally:
        Q.destroyQureg(q)
    assert np.max(np.abs(np.array(list(got)) - want)) <= TOL


def _string_set(nq, count, style, rng):
    codes = []
    for s in range(count):
        c = [int(v) for v in rng.integers(0, 4, nq)]
        if style == "low":        # X/Y only on the lowest qubits (partners in the same row)
            c = [v if q < 3 or v in (0, 3) else 3 for q, v in enumerate(c)]
        elif style == "high":     # X/Y only on the highest qubits (partners far away)
            c = [v if q >= nq - 3 or v in (0, 3) else 0 for q, v in enumerate(c)]
        elif style == "zi":       # Z-only and identity strings between general ones
            if s % 2 == 0:
                c = [3 * (v & 1) if s % 4 == 0 else 0 for v in c]
        elif style == "repeat" and s % 2 == 1:
            c = codes[-1]
        codes.append(c)
    return codes


@pytest.mark.parametrize("nq", [1, 3, 6, 12, 17, 22])
@pytest.mark.parametrize("style", ["random", "low", "high", "zi", "repeat"])
def test_tiled_pauli_batch_string_shapes(env, nq, style):
    """The statevector batch (tiles of 2^t contiguous columns times the span of the
    strings' row parts, every amplitude read once per pass) on strings whose partners
    are near, far, absent (Z/I) or repeated, 1 to 22 qubits, against the oracle."""
    import ctypes
    rng = np.random.default_rng(hash((nq, style)) & 0xffff)
    codes = _string_set(nq, 37, style, rng)
    amps = qc.random_statevector(nq, 80 + nq)
    _, want, _ = qc.oracle().run("".join(f"EXPEC {qc.pauli_text(c)}\n" for c in codes), nq, 0, amps)
    Q = env.Q
    q = Q.createQureg(nq)
    try:
        env.set_amps(q, amps)
        strs = (env.PauliStr * len(codes))(*[env.pauli_str(c) for c in codes])
        got = (ctypes.c_double * len(codes))()
        Q.calcExpecPauliStrs(got, q, strs, len(codes))
        again = (ctypes.c_double * len(codes))()
        Q.calcExpecPauliStrs(again, q, strs, len(codes))
    finally:
        Q.destroyQureg(q)
    assert np.max(np.abs(np.array(list(got)) - want)) <= TOL
    assert bytes(got) == bytes(again)       # deterministic


@pytest.mark.parametrize("nq,text", [
    (12, "FQFT\n"),
    (21, "FQFT\nTOTALPROB\n"),
    (14, "QFT 5 3 4 5 6 7\n"),            # contiguous targets above qubit 0: one pass per step
    (14, "QFT 4 9 2 12 5\n"),             # not contiguous: the gate-by-gate form
    (10, "X 0\nFQFT\nFQFT\n"),
    (16, "QFT 11 0 1 2 3 4 5 6 7 8 9 10\n"),   # from qubit 0, below the top: closing swaps in one pass
    (14, "QFT 9 0 1 2 3 4 5 6 7 8\n"),        # fewer than 10 targets: the swaps one by one
])
def test_qft_steps_vs_oracle(env, nq, text):
    """The quantum Fourier transform with each step (Hadamard and its controlled phases)
    as one fixed-point pass, in both product modes (IEEE FP64 keeps the gate-by-gate form)."""
    from quest_gb300._lib import lib
    amps = qc.random_statevector(nq, nq + 3)
    want, wres, _ = qc.oracle().run(text, nq, 0, amps)
    try:
        for mode in (0, 1):
            assert lib().qg_set_fp64_products(mode) == 0
            got, res, _ = run_gpu(env, text, nq, 0, amps)
            assert np.max(np.abs(got - want)) <= TOL
            assert np.max(np.abs(res - wres), initial=0) <= TOL
    finally:
        lib().qg_set_fp64_products(0)


@pytest.mark.parametrize("nq,nb", [(10, 10), (11, 10), (13, 13), (16, 12), (20, 20), (21, 15)])
def test_reverse_low_bits_bit_exact(env, nq, nb):
    """The closing swaps of a QFT on qubits 0..nb-1 as one permutation pass: every index has
    its low nb bits reversed, bit for bit (a permutation of the amplitudes)."""
    import ctypes
    from quest_gb300._lib import lib
    amps = qc.random_statevector(nq, 7 * nq + nb)
    idx = np.arange(1 << nq, dtype=np.int64)
    low = idx & ((1 << nb) - 1)
    rev = np.zeros_like(low)
    for b in range(nb):
        rev |= ((low >> b) & 1) << (nb - 1 - b)
    want = np.empty_like(amps)
    want[(idx & ~((1 << nb) - 1)) | rev] = amps
    Q = env.Q
    q = Q.createQureg(nq)
    try:
        env.set_amps(q, amps)
        assert lib().qg_sync() == 0
        assert lib().qg_sv_reverseLowBits(ctypes.cast(q.gpuAmps, ctypes.c_void_p), nq, nb, None) == 0
        assert lib().qg_sync() == 0
        got = env.get_amps(q)
    finally:
        Q.destroyQureg(q)
    assert got.tobytes() == want.tobytes()


def test_qft_two_steps_match_single_steps(env):
    """Two QFT steps in one pass (targets T and T - 1 from qubit 0) against the two single-step
    passes, on a 26-qubit state, for T from 25 (four twiddle tables) down to 1: the same values
    to 1e-14 of the largest amplitude (the step of T on the pairs whose bit T - 1 is set takes
    its twiddle as i W, which the single step forms from its tables)."""
    import ctypes
    from quest_gb300._lib import lib
    L = lib()
    nq = 26
    nbytes = 16 << nq
    bufs = [ctypes.c_void_p(), ctypes.c_void_p()]
    for b in bufs:
        assert L.qg_alloc(ctypes.byref(b), nbytes) == 0
    try:
        for T in (25, 24, 17, 16, 9, 8, 3, 1):
            for b in bufs:
                assert L.qg_sv_initDebugState(b, nq, None) == 0
            assert L.qg_sv_qftTwoSteps(bufs[0], nq, T, None) == 0
            assert L.qg_sv_qftStep(bufs[1], nq, T, 0, T, None) == 0
            assert L.qg_sv_qftStep(bufs[1], nq, T - 1, 0, T - 1, None) == 0
            out = [np.empty(1 << nq, dtype=np.complex128) for _ in bufs]
            for o, b in zip(out, bufs):
                assert L.qg_copy_d2h(o.ctypes.data_as(ctypes.c_void_p), b, nbytes, None) == 0
            assert L.qg_sync() == 0
            scale = np.max(np.abs(out[1]))
            assert np.max(np.abs(out[0] - out[1])) <= 1e-14 * scale, T
    finally:
        for b in bufs:
            L.qg_free(b)


@pytest.mark.parametrize("T", [11, 5])
def test_qft_two_steps_special_values(env, T):
    """Two QFT steps in one pass on a 12-qubit state holding zeros, denormals, values near
    the top of the double range, Inf and NaN in some quadruples (the FP64 butterflies) next
    to ordinary ones (fixed point): against two single-step passes, the same non-finite
    outputs and every finite output within 1e-13 of its quadruple's largest input."""
    import ctypes
    from quest_gb300._lib import lib
    L = lib()
    nq = 12
    rng = np.random.default_rng(T)
    amps = (rng.standard_normal(1 << nq) + 1j * rng.standard_normal(1 << nq)) * 1e-2
    idx = rng.choice(1 << nq, 40, replace=False)
    specials = [0.0, 5e-324, 3e-310, 1.7e308, 1e300, np.inf, -np.inf, np.nan, 1e-300]
    for k, i in enumerate(idx):
        amps[i] = complex(specials[k % len(specials)], 0.0 if k % 2 else 1e-3)
    amps[:64] = 0.0                                            # all-zero quadruples
    nbytes = 16 << nq
    bufs = [ctypes.c_void_p(), ctypes.c_void_p()]
    for b in bufs:
        assert L.qg_alloc(ctypes.byref(b), nbytes) == 0
    try:
        src = np.ascontiguousarray(amps)
        for b in bufs:
            assert L.qg_copy_h2d(b, src.ctypes.data_as(ctypes.c_void_p), nbytes, None) == 0
        assert L.qg_sync() == 0
        assert L.qg_sv_qftTwoSteps(bufs[0], nq, T, None) == 0
        assert L.qg_sv_qftStep(bufs[1], nq, T, 0, T, None) == 0
        assert L.qg_sv_qftStep(bufs[1], nq, T - 1, 0, T - 1, None) == 0
        out = [np.empty(1 << nq, dtype=np.complex128) for _ in bufs]
        for o, b in zip(out, bufs):
            assert L.qg_copy_d2h(o.ctypes.data_as(ctypes.c_void_p), b, nbytes, None) == 0
        assert L.qg_sync() == 0
    finally:
        for b in bufs:
            L.qg_free(b)
    fused, single = out
    # largest input magnitude of each amplitude's quadruple (bits T and T - 1)
    i = np.arange(1 << nq)
    base = i & ~((1 << T) | (1 << (T - 1)))
    mags = np.abs(np.nan_to_num(amps, nan=0.0, posinf=1.8e308, neginf=1.8e308))
    qmax = np.zeros(1 << nq)
    for off in (0, 1 << (T - 1), 1 << T, (1 << T) | (1 << (T - 1))):
        qmax = np.maximum(qmax, mags[base | off])
    for part in (np.real, np.imag):
        a, b = part(fused), part(single)
        assert np.array_equal(np.isfinite(a), np.isfinite(b))
        fin = np.isfinite(a)
        assert np.all(np.abs(a[fin] - b[fin]) <= 1e-13 * qmax[fin])


def test_qft_three_steps_match_single_steps(env):
    """Three QFT steps in one pass (targets T, T - 1, T - 2 from qubit 0) against three
    single-step passes, on a 26-qubit state, for T from 25 (four twiddle tables) down to 2:
    the same values to 1e-14 of the largest amplitude."""
    import ctypes
    from quest_gb300._lib import lib
    L = lib()
    nq = 26
    nbytes = 16 << nq
    bufs = [ctypes.c_void_p(), ctypes.c_void_p()]
    for b in bufs:
        assert L.qg_alloc(ctypes.byref(b), nbytes) == 0
    try:
        for T in (25, 24, 18, 17, 10, 8, 5, 2):
            for b in bufs:
                assert L.qg_sv_initDebugState(b, nq, None) == 0
            assert L.qg_sv_qftThreeSteps(bufs[0], nq, T, None) == 0
            for k in range(3):
                assert L.qg_sv_qftStep(bufs[1], nq, T - k, 0, T - k, None) == 0
            out = [np.empty(1 << nq, dtype=np.complex128) for _ in bufs]
            for o, b in zip(out, bufs):
                assert L.qg_copy_d2h(o.ctypes.data_as(ctypes.c_void_p), b, nbytes, None) == 0
            assert L.qg_sync() == 0
            scale = np.max(np.abs(out[1]))
            assert np.max(np.abs(out[0] - out[1])) <= 1e-14 * scale, T
        assert L.qg_sv_qftThreeSteps(bufs[0], nq, 9, None) != 0       # 9: not a pass of three
    finally:
        for b in bufs:
            L.qg_free(b)


@pytest.mark.parametrize("T", [12, 6])
def test_qft_three_steps_special_values(env, T):
    """Three QFT steps in one pass on a 13-qubit state holding zeros, denormals, values near
    the top of the double range, Inf and NaN beside ordinary octets: against three
    single-step passes, non-finite outputs in the same places and every finite output
    within 1e-13 of its octet's largest input."""
    import ctypes
    from quest_gb300._lib import lib
    L = lib()
    nq = 13
    rng = np.random.default_rng(T + 50)
    amps = (rng.standard_normal(1 << nq) + 1j * rng.standard_normal(1 << nq)) * 1e-2
    idx = rng.choice(1 << nq, 60, replace=False)
    specials = [0.0, 5e-324, 3e-310, 1.7e308, 1e300, np.inf, -np.inf, np.nan, 1e-300]
    for k, i in enumerate(idx):
        amps[i] = complex(specials[k % len(specials)], 0.0 if k % 2 else 1e-3)
    amps[:64] = 0.0
    nbytes = 16 << nq
    bufs = [ctypes.c_void_p(), ctypes.c_void_p()]
    for b in bufs:
        assert L.qg_alloc(ctypes.byref(b), nbytes) == 0
    try:
        src = np.ascontiguousarray(amps)
        for b in bufs:
            assert L.qg_copy_h2d(b, src.ctypes.data_as(ctypes.c_void_p), nbytes, None) == 0
        assert L.qg_sync() == 0
        assert L.qg_sv_qftThreeSteps(bufs[0], nq, T, None) == 0
        for k in range(3):
            assert L.qg_sv_qftStep(bufs[1], nq, T - k, 0, T - k, None) == 0
        out = [np.empty(1 << nq, dtype=np.complex128) for _ in bufs]
        for o, b in zip(out, bufs):
            assert L.qg_copy_d2h(o.ctypes.data_as(ctypes.c_void_p), b, nbytes, None) == 0
        assert L.qg_sync() == 0
    finally:
        for b in bufs:
            L.qg_free(b)
    fused, single = out
    i = np.arange(1 << nq)
    m3 = (1 << T) | (1 << (T - 1)) | (1 << (T - 2))
    base = i & ~m3
    mags = np.abs(np.nan_to_num(amps, nan=0.0, posinf=1.8e308, neginf=1.8e308))
    omax = np.zeros(1 << nq)
    for o in range(8):
        off = ((o >> 2) & 1) << T | ((o >> 1) & 1) << (T - 1) | (o & 1) << (T - 2)
        omax = np.maximum(omax, mags[base | off])
    for part in (np.real, np.imag):
        a, b = part(fused), part(single)
        assert np.array_equal(np.isfinite(a), np.isfinite(b))
        fin = np.isfinite(a)
        assert np.all(np.abs(a[fin] - b[fin]) <= 1e-13 * omax[fin])
