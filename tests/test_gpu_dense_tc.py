"""Three- and four-target dense gates on the tensor cores as exact 8-bit slices
(quest_gb300/csrc/qg_dense_tc.cu).

* Bit for bit the host restatement of the kernel's arithmetic (tests/slices_ref.cpp over
  qg_slices.h): this shows that every digit product and digit sum on the tensor cores is
  exact, for every target placement (lowest bits included), with controls, for registers
  of less than one tile of 128 groups, and for groups that go to FP64 (Inf, NaN, denormal
  and extreme scales), which must give the FP64 path's bits.
* Within the FP64 bar (max-abs <= 1e-12) of the oracle, in the automatic mode at sizes where
  it picks the tensor cores, for state vectors and a density matrix's two-qubit Kraus map.
* The switch and the error flag: no bounded wait runs out."""
import ctypes
import os
import shutil
import subprocess

import numpy as np
import pytest

import qcircuits as qc

pytestmark = pytest.mark.gpu
TOL = 1e-12
HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "..", "quest_gb300", "csrc")


@pytest.fixture(scope="module")
def host_ref(tmp_path_factory):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not available")
    so = str(tmp_path_factory.mktemp("slices") / "libslices_ref.so")
    subprocess.run([gxx, "-O2", "-std=c++17", "-shared", "-fPIC", "-I", CSRC, os.path.join(HERE, "slices_ref.cpp"),
                    "-o", so], check=True)
    L = ctypes.CDLL(so)
    ip = ctypes.POINTER(ctypes.c_int)
    dp = ctypes.POINTER(ctypes.c_double)
    L.slices_apply_state.argtypes = [ctypes.c_int, ctypes.c_int, ip, ctypes.c_int, ip, ip, dp, dp]
    L.slices_apply_state.restype = ctypes.c_int
    return L


def _ints(v):
    a = (ctypes.c_int * max(1, len(v)))()
    for i, x in enumerate(v):
        a[i] = int(x)
    return a


def host_apply(L, nq, targs, ctrls, states, u, amps):
    a = np.ascontiguousarray(amps, dtype=np.complex128).copy()
    m = np.ascontiguousarray(u, dtype=np.complex128)
    dp = ctypes.POINTER(ctypes.c_double)
    rc = L.slices_apply_state(nq, len(targs), _ints(targs), len(ctrls), _ints(ctrls), _ints(states),
                              m.ctypes.data_as(dp), a.ctypes.data_as(dp))
    assert rc == 0
    return a


def gate_text(targs, ctrls, states, u):
    k = len(targs)
    t = " ".join(map(str, targs))
    if ctrls:
        return (f"CUK {len(ctrls)} {' '.join(map(str, ctrls))} {' '.join(map(str, states))} {k} {t} "
                f"{qc.mat_tokens(u)}\n")
    return f"UK {k} {t} {qc.mat_tokens(u)}\n"


def run_gpu(env, text, nq, amps, is_dm=False):
    from quest_gb300.circuit import run_text
    Q = env.Q
    q = Q.createDensityQureg(nq) if is_dm else Q.createQureg(nq)
    try:
        env.set_amps(q, amps)
        res, _ = run_text(text, q)
        return env.get_amps(q), res
    finally:
        Q.destroyQureg(q)


def _lib():
    from quest_gb300._lib import lib
    return lib()


def _set_slices(mode):
    assert _lib().qg_set_tensor_slices(mode) == 0


def _flag():
    f = ctypes.c_int(-1)
    assert _lib().qg_tc_get_error_flag(ctypes.byref(f)) == 0
    return f.value


def _same_bits(a, b):
    x, y = a.view(np.float64), b.view(np.float64)
    return np.array_equal(x, y) or bool(np.all((x == y) | (np.isnan(x) & np.isnan(y))))


CASES = [
    # nq, targets, controls, control states
    (12, [5, 9, 1, 11], [], []),
    (13, [0, 1, 2, 3], [], []),            # the four lowest bits: each group is 16 adjacent amplitudes
    (10, [3, 0, 8, 6], [], []),            # 64 groups: less than one tile
    (16, [15, 9, 4, 12], [2], [1]),
    (15, [7, 0, 13, 2], [5, 10], [0, 1]),
    (12, [2, 7, 0], [], []),
    (14, [13, 1, 6], [3], [0]),
    (11, [0, 1, 2], [], []),
]


@pytest.mark.parametrize("nq,targs,ctrls,states", CASES, ids=[f"{c[0]}q-{len(c[1])}t-{len(c[2])}c" for c in CASES])
def test_bits_equal_the_host_restatement(env, host_ref, nq, targs, ctrls, states):
    rng = np.random.default_rng(nq * 100 + len(targs) * 10 + len(ctrls))
    u = qc.haar_unitary(1 << len(targs), rng)
    amps = qc.random_statevector(nq, nq + 7)
    want = host_apply(host_ref, nq, targs, ctrls, states, u, amps)
    try:
        _set_slices(2)
        got, _ = run_gpu(env, gate_text(targs, ctrls, states, u), nq, amps)
    finally:
        _set_slices(1)
    assert _same_bits(got, want)
    ref, _, _ = qc.oracle().run(gate_text(targs, ctrls, states, u), nq, 0, amps)
    assert np.max(np.abs(got - ref)) <= TOL
    assert _flag() == 0


@pytest.mark.parametrize("k", [3, 4])
def test_special_groups_take_the_fp64_path(env, host_ref, k):
    """Groups holding Inf/NaN, denormals only, magnitudes from 1e-300 to 1e300, and zeros."""
    nq = 12
    rng = np.random.default_rng(40 + k)
    amps = qc.random_statevector(nq, 41) * 10.0 ** rng.integers(-300, 300, 1 << nq)
    amps[3] = complex(np.inf, 0)
    amps[100] = complex(np.nan, 1.0)
    amps[200:232] = 0
    amps[300:340] = complex(3e-312, -1e-310)
    amps[500] = complex(1e-310, 0)
    targs = [int(v) for v in rng.choice(nq, k, replace=False)]
    u = qc.haar_unitary(1 << k, rng)
    want = host_apply(host_ref, nq, targs, [], [], u, amps)
    try:
        _set_slices(2)
        got, _ = run_gpu(env, gate_text(targs, [], [], u), nq, amps)
    finally:
        _set_slices(1)
    assert _same_bits(got, want)
    assert _flag() == 0


@pytest.mark.parametrize("nq,k", [(20, 4), (21, 3), (19, 4)])
def test_automatic_mode_meets_the_fp64_bar(env, nq, k):
    """Sizes where mode 1 picks the tensor cores (at least one tile per SM); the integer
    kernels (mode 0) on the same gates for comparison."""
    rng = np.random.default_rng(nq + k)
    text = ""
    for _ in range(3):
        t = [int(v) for v in rng.choice(nq, k, replace=False)]
        text += gate_text(t, [], [], qc.haar_unitary(1 << k, rng))
    text += "TOTALPROB\n"
    amps = qc.random_statevector(nq, nq)
    want, wres, _ = qc.oracle().run(text, nq, 0, amps)
    outs = {}
    try:
        for mode in (1, 0):
            _set_slices(mode)
            outs[mode], res = run_gpu(env, text, nq, amps)
            assert np.max(np.abs(outs[mode] - want)) <= TOL
            assert np.max(np.abs(res - wres)) <= TOL
    finally:
        _set_slices(1)
    assert _flag() == 0


def test_density_matrix_kraus_map_on_the_tensor_cores(env):
    """A two-qubit Kraus map on a 10-qubit density matrix: a four-target superoperator on
    2^20 amplitudes, in the automatic mode."""
    nq = 10
    rng = np.random.default_rng(77)
    ops = qc.random_kraus(2, 4, rng)
    text = f"KRAUS 2 3 8 4 {' '.join(qc.mat_tokens(o) for o in ops)}\nPURITY\nTOTALPROB\n"
    amps = qc.random_density_matrix(nq, 78)
    want, wres, _ = qc.oracle().run(text, nq, 1, amps)
    got, res = run_gpu(env, text, nq, amps, is_dm=True)
    assert np.max(np.abs(got - want)) <= TOL
    assert np.max(np.abs(res - wres)) <= TOL
    assert _flag() == 0


def test_deferred_statevector_gates(env):
    """One-qubit dense gates on a 20-qubit statevector are deferred and applied four qubits
    per tensor-core pass; random interleavings with controlled, two-qubit, diagonal and
    Pauli gates, reductions and a measurement stay within 1e-12 of the oracle (outcomes
    bit-exact), in both product modes (IEEE FP64 defers nothing)."""
    nq = 20
    rng = np.random.default_rng(2024)
    lines = ["SEED 7"]
    for layer in range(6):
        for t in rng.permutation(nq)[: int(rng.integers(5, nq + 1))]:
            lines.append(f"U1 {int(t)} {qc.mat_tokens(qc.haar_unitary(2, rng))}")
            if rng.random() < 0.3:
                lines.append(f"H {int(rng.integers(nq))}")
        a, b, c = (int(v) for v in rng.choice(nq, 3, replace=False))
        lines.append(f"CU1 1 {a} 1 {b} {qc.mat_tokens(qc.haar_unitary(2, rng))}")
        lines.append(f"U2 {b} {c} {qc.mat_tokens(qc.haar_unitary(4, rng))}")
        lines.append(f"CPS {a} {c} {0.3 + layer}")
        lines.append(f"X {int(rng.integers(nq))}")
        if layer == 2:
            lines.append("TOTALPROB")
            lines.append(f"PROBQ {int(rng.integers(nq))} 1")
        if layer == 4:
            lines.append(f"MEAS {int(rng.integers(nq))}")
    lines.append("TOTALPROB")
    text = "\n".join(lines) + "\n"
    amps = qc.random_statevector(nq, 2025)
    want, wres, wout = qc.oracle().run(text, nq, 0, amps)
    from quest_gb300._lib import lib
    try:
        for mode in (0, 1):
            assert lib().qg_set_fp64_products(mode) == 0
            got, res = run_gpu(env, text, nq, amps)
            assert np.max(np.abs(got - want)) <= TOL
            assert np.max(np.abs(res - wres)) <= TOL
    finally:
        lib().qg_set_fp64_products(0)
    assert _flag() == 0


def test_flush_before_reading_the_device_amplitudes(env):
    """flushQuregDeferredOps applies the deferred gates without a read of the state: the
    device amplitudes, copied through the C ABI, then equal the oracle's."""
    import ctypes
    from quest_gb300._lib import lib
    nq = 20
    rng = np.random.default_rng(99)
    text = "".join(f"U1 {t} {qc.mat_tokens(qc.haar_unitary(2, rng))}\n" for t in range(nq))
    amps = qc.random_statevector(nq, 98)
    want, _, _ = qc.oracle().run(text, nq, 0, amps)
    from quest_gb300.circuit import run_text
    Q = env.Q
    q = Q.createQureg(nq)
    try:
        env.set_amps(q, amps)
        run_text(text, q)
        Q.flushQuregDeferredOps(q)
        out = np.zeros(1 << nq, dtype=np.complex128)
        assert lib().qg_sync() == 0
        assert lib().qg_copy_d2h(out.ctypes.data_as(ctypes.c_void_p), ctypes.cast(q.gpuAmps, ctypes.c_void_p), 16 << nq, None) == 0
        assert lib().qg_sync() == 0
        assert np.max(np.abs(out - want)) <= TOL
    finally:
        Q.destroyQureg(q)


@pytest.mark.parametrize("seed", [11, 12])
def test_deferred_phases_and_gates(env, seed):
    """Controlled phases (CPhase, CZ, phase shifts, S, T, Z) on a 20-qubit statevector are
    deferred as a set and applied in one pass, one-qubit gates four per pass; they
    interleave on shared qubits (a gate on a qubit with a pending phase applies the phases
    first), with more than 32 phases pending at once, a controlled gate, a QFT and
    reductions: within 1e-12 of the oracle in both product modes."""
    nq = 20
    rng = np.random.default_rng(seed)
    lines = []
    for layer in range(5):
        for t in rng.permutation(nq)[: int(rng.integers(8, nq + 1))]:
            lines.append(f"U1 {int(t)} {qc.mat_tokens(qc.haar_unitary(2, rng))}")
        for _ in range(int(rng.integers(10, 40))):
            a, b = (int(v) for v in rng.choice(nq, 2, replace=False))
            kind = int(rng.integers(6))
            lines.append([f"CPS {a} {b} {rng.uniform(-3, 3)}", f"CZ {a} {b}", f"PS {a} {rng.uniform(-3, 3)}",
                          f"S {a}", f"T {a}", f"Z {a}"][kind])
        a, b, c = (int(v) for v in rng.choice(nq, 3, replace=False))
        lines.append(f"CU1 1 {a} 1 {b} {qc.mat_tokens(qc.haar_unitary(2, rng))}")
        lines.append(f"H {c}")
        if layer == 3:
            lines.append("TOTALPROB")
            lines.append(f"PROBQ {int(rng.integers(nq))} 0")
    lines.append("FQFT")
    lines.append("TOTALPROB")
    text = "\n".join(lines) + "\n"
    amps = qc.random_statevector(nq, seed + 100)
    want, wres, _ = qc.oracle().run(text, nq, 0, amps)
    from quest_gb300._lib import lib
    try:
        for mode in (0, 1):
            assert lib().qg_set_fp64_products(mode) == 0
            got, res = run_gpu(env, text, nq, amps)
            assert np.max(np.abs(got - want)) <= TOL
            assert np.max(np.abs(res - wres)) <= TOL
    finally:
        lib().qg_set_fp64_products(0)


def _pair_layer(nq, rng, phases=True):
    lines = [f"U1 {t} {qc.mat_tokens(qc.haar_unitary(2, rng))}" for t in range(nq)]
    if phases:
        perm = rng.permutation(nq)
        lines += [f"CPS {int(perm[2 * p])} {int(perm[2 * p + 1])} {rng.uniform(-3, 3)}" for p in range(nq // 2)]
    return "\n".join(lines) + "\n"


def test_pair_layer_takes_no_phase_pass(env):
    """A one-qubit gate on every qubit of a 22-qubit statevector, then controlled phases on
    disjoint random pairs: the pairs are packed into the four-qubit passes and their phases
    folded into those passes, so the layer launches exactly as many kernels as the same
    layer without phases (no phase pass), and matches the oracle within 1e-12."""
    from quest_gb300.circuit import run_text
    nq = 22
    rng = np.random.default_rng(404)
    Q = env.Q
    q = Q.createQureg(nq)
    try:
        amps = qc.random_statevector(nq, 405)
        env.set_amps(q, amps)
        counts = {}
        text = ""
        for rep in range(2):
            for phases in (False, True):
                layer = _pair_layer(nq, rng, phases)
                text += layer
                before = ctypes.c_int64(0)
                assert _lib().qg_get_launch_count(ctypes.byref(before)) == 0
                run_text(layer, q)
                Q.flushQuregDeferredOps(q)
                after = ctypes.c_int64(0)
                assert _lib().qg_get_launch_count(ctypes.byref(after)) == 0
                counts[(rep, phases)] = after.value - before.value
        got = env.get_amps(q)
    finally:
        Q.destroyQureg(q)
    # 5 four-qubit passes + 1 two-qubit pass
    assert counts[(1, True)] == counts[(1, False)] == 6, counts
    want, _, _ = qc.oracle().run(text, nq, 0, amps)
    assert np.max(np.abs(got - want)) <= TOL
    assert _flag() == 0


@pytest.mark.parametrize("seed", [21, 22])
def test_phases_folded_into_gate_groups(env, seed):
    """Deferred phases folded into the passes of the deferred one-qubit gates, on a 22-qubit
    statevector: pair layers, three-qubit phase shifts, one-qubit phases on qubits with a
    pending gate, a chain of phases joining more than four qubits (not packed together: the
    phases left out go to the phase pass), phases on qubits with no pending gate, and layers
    on a subset of the qubits: within 1e-12 of the oracle in both product modes."""
    nq = 22
    rng = np.random.default_rng(seed)
    lines = []
    for layer in range(6):
        qubits = range(nq) if layer % 3 != 2 else sorted(int(v) for v in rng.choice(nq, 13, replace=False))
        for t in qubits:
            lines.append(f"U1 {t} {qc.mat_tokens(qc.haar_unitary(2, rng))}")
        perm = [int(v) for v in rng.permutation(nq)]
        for p in range(int(rng.integers(3, nq // 2 + 1))):
            lines.append(f"CPS {perm[2 * p]} {perm[2 * p + 1]} {rng.uniform(-3, 3)}")
        if layer == 1:
            a, b, c, d = (int(v) for v in rng.choice(nq, 4, replace=False))
            lines.append(f"MPS 3 {a} {b} {c} {rng.uniform(-3, 3)}")
            lines.append(f"PS {d} {rng.uniform(-3, 3)}")
            lines.append(f"T {a}")
            lines.append(f"CZ {b} {d}")
        if layer == 3:
            chain = [int(v) for v in rng.choice(nq, 7, replace=False)]
            for i in range(6):
                lines.append(f"CPS {chain[i]} {chain[i + 1]} {rng.uniform(-3, 3)}")
            lines.append(f"MPS 4 {chain[0]} {chain[2]} {chain[4]} {chain[6]} {rng.uniform(-3, 3)}")
        if layer == 4:
            lines.append("TOTALPROB")
    lines.append("TOTALPROB")
    text = "\n".join(lines) + "\n"
    amps = qc.random_statevector(nq, seed + 300)
    want, wres, _ = qc.oracle().run(text, nq, 0, amps)
    try:
        for mode in (0, 1):
            assert _lib().qg_set_fp64_products(mode) == 0
            got, res = run_gpu(env, text, nq, amps)
            assert np.max(np.abs(got - want)) <= TOL
            assert np.max(np.abs(res - wres)) <= TOL
    finally:
        _lib().qg_set_fp64_products(0)
    assert _flag() == 0
