"""Seeded inputs and circuit text for the parity tests.

The text format is the one parsed by the oracle's circuit runner
(oracle/qoracle.cpp, ``orc_run_circuit``), by the reference harness
(oracle/ref_harness.cpp) and by ``quest_gb300.circuit.run_text`` on the GPU:
one QuEST API call per line (``H 3``, ``U1 t m00r m00i ...``, ``DEPOL q p``,
``EXPEC XIZY`` ...).
"""
import ctypes
import os

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ORACLE_SO = os.path.join(ROOT, "oracle", "_build", "libqoracle.so")
REF_SO = os.path.join(ROOT, "oracle", "_ref", "libqref.so")


# ---------------------------------------------------------------- inputs

def random_statevector(nq, seed):
    """Complex Gaussian amplitudes (re, im ~ N(0,1)), L2-normalised."""
    rng = np.random.default_rng(seed)
    a = rng.standard_normal(1 << nq) + 1j * rng.standard_normal(1 << nq)
    return (a / np.linalg.norm(a)).astype(np.complex128)


def random_density_matrix(nq, seed, num_pure=8):
    """sum_j w_j |psi_j><psi_j| with Dirichlet(1..1) weights, as a flat
    column-major Choi vector (row = low nq bits)."""
    rng = np.random.default_rng(seed)
    w = rng.dirichlet(np.ones(num_pure))
    dim = 1 << nq
    rho = np.zeros((dim, dim), dtype=np.complex128)
    for j in range(num_pure):
        psi = rng.standard_normal(dim) + 1j * rng.standard_normal(dim)
        psi /= np.linalg.norm(psi)
        rho += w[j] * np.outer(psi, psi.conj())
    return rho.T.reshape(-1).copy()   # column-major flatten: index = row + col*dim


def haar_unitary(dim, rng):
    """Haar-random unitary: QR of a complex Gaussian matrix with the phases of
    R's diagonal fixed (the construction of tests/utils/random.cpp in QuEST)."""
    z = (rng.standard_normal((dim, dim)) + 1j * rng.standard_normal((dim, dim))) / np.sqrt(2)
    q, r = np.linalg.qr(z)
    d = np.diag(r)
    return q * (d / np.abs(d))


def random_kraus(k, num_ops, rng):
    """num_ops Kraus operators of a random CPTP map on k qubits: blocks of a
    random (num_ops*2^k) x 2^k isometry."""
    dim = 1 << k
    big = haar_unitary(num_ops * dim, rng)[:, :dim]
    return [big[i * dim:(i + 1) * dim, :] for i in range(num_ops)]


def fmt(x):
    return repr(float(x))


def mat_tokens(m):
    m = np.asarray(m, dtype=np.complex128).reshape(-1)
    out = []
    for v in m:
        out.append(fmt(v.real))
        out.append(fmt(v.imag))
    return " ".join(out)


def pauli_text(codes):
    return "".join("IXYZ"[c] for c in codes)


# ---------------------------------------------------------------- runners

class CircuitLib:
    """ctypes view of a circuit runner with the orc_run_circuit signature."""

    def __init__(self, path, fn_name):
        self.lib = ctypes.CDLL(path)
        self.fn = getattr(self.lib, fn_name)
        self.fn.restype = ctypes.c_int
        self.fn.argtypes = [ctypes.c_char_p, ctypes.c_int, ctypes.c_int, ctypes.c_void_p,
                            ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(ctypes.c_int),
                            ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(ctypes.c_int)]

    def run(self, text, nq, is_dm, amps, max_results=4096):
        amps = np.ascontiguousarray(amps, dtype=np.complex128).copy()
        res = np.zeros(max_results, dtype=np.float64)
        outs = np.zeros(max_results, dtype=np.int32)
        nres = ctypes.c_int(0)
        nout = ctypes.c_int(0)
        rc = self.fn(text.encode(), nq, int(is_dm), amps.ctypes.data, res.ctypes.data, max_results,
                     ctypes.byref(nres), outs.ctypes.data, max_results, ctypes.byref(nout))
        if rc != 0:
            raise RuntimeError(f"circuit runner failed with {rc}")
        return amps, res[:nres.value].copy(), outs[:nout.value].copy()


_oracle = None


def oracle():
    """The CPU oracle's circuit runner (builds it on first use)."""
    global _oracle
    if _oracle is None:
        if not os.path.exists(ORACLE_SO):
            import subprocess
            subprocess.check_call(["make", "-s", "-C", os.path.join(ROOT, "oracle")])
        _oracle = CircuitLib(ORACLE_SO, "orc_run_circuit")
    return _oracle


def reference():
    """The reference library's circuit runner, or None where it was not built."""
    if not os.path.exists(REF_SO):
        return None
    return CircuitLib(REF_SO, "ref_run_circuit")


# ---------------------------------------------------------------- circuits

def every_op_circuit(nq, is_dm, seed, with_measure=True):
    """A circuit that exercises every op of the text format at least once on
    random qubits, ending with every reduction."""
    rng = np.random.default_rng(seed)
    L = []
    q = lambda: int(rng.integers(nq))

    def distinct(k):
        return [int(v) for v in rng.choice(nq, size=k, replace=False)]

    ang = lambda: fmt(rng.uniform(0, 2 * np.pi))
    for t in range(nq):
        L.append(f"H {t}")
    for op in ("X", "Y", "Z", "S", "T"):
        L.append(f"{op} {q()}")
    for op in ("RX", "RY", "RZ"):
        L.append(f"{op} {q()} {ang()}")
    for op in ("CRX", "CRY", "CRZ"):
        c, t = distinct(2)
        L.append(f"{op} {c} {t} {ang()}")
    L.append(f"PS {q()} {ang()}")
    a, b = distinct(2); L.append(f"CPS {a} {b} {ang()}")
    a, b = distinct(2); L.append(f"CX {a} {b}")
    a, b = distinct(2); L.append(f"CZ {a} {b}")
    a, b = distinct(2); L.append(f"SWAP {a} {b}")
    if nq >= 4:
        c1, c2, a, b = distinct(4)
        L.append(f"CSWAP 2 {c1} {c2} {int(rng.integers(2))} {int(rng.integers(2))} {a} {b}")
    L.append(f"U1 {q()} {mat_tokens(haar_unitary(2, rng))}")
    c1, c2, t = distinct(3)
    L.append(f"CU1 2 {c1} {c2} 0 1 {t} {mat_tokens(haar_unitary(2, rng))}")
    a, b = distinct(2); L.append(f"U2 {a} {b} {mat_tokens(haar_unitary(4, rng))}")
    if nq >= 4:
        c, a, b = distinct(3); L.append(f"CU2 1 {c} 0 {a} {b} {mat_tokens(haar_unitary(4, rng))}")
    for k in (3, min(5, nq), min(6, nq)):
        if k <= nq and k >= 3:
            t = distinct(k)
            L.append(f"UK {k} {' '.join(map(str, t))} {mat_tokens(haar_unitary(1 << k, rng))}")
    if nq >= 4:
        c = distinct(4)
        L.append(f"CUK 1 {c[0]} 1 3 {c[1]} {c[2]} {c[3]} {mat_tokens(haar_unitary(8, rng))}")
    ph = lambda k: np.exp(1j * rng.uniform(0, 2 * np.pi, size=1 << k))
    L.append(f"D1 {q()} {mat_tokens(ph(1))}")
    a, b = distinct(2); L.append(f"D2 {a} {b} {mat_tokens(ph(2))}")
    t = distinct(3); L.append(f"DK 3 {' '.join(map(str, t))} {mat_tokens(ph(3))}")
    if nq >= 4:
        c = distinct(4)
        L.append(f"CDK 1 {c[0]} 0 3 {c[1]} {c[2]} {c[3]} {mat_tokens(ph(3))}")
    t = distinct(2); L.append(f"DKP 2 {' '.join(map(str, t))} {mat_tokens(ph(2))} {fmt(rng.uniform(-2, 2))} 0.0")
    codes = [int(v) for v in rng.integers(0, 4, size=nq)]
    L.append(f"PSTR {pauli_text(codes)}")
    codes = [int(v) for v in rng.integers(0, 4, size=nq)]
    L.append(f"PG {pauli_text(codes)} {ang()}")
    zonly = [int(v) * 3 for v in rng.integers(0, 2, size=nq)]
    L.append(f"PG {pauli_text(zonly)} {ang()}")
    c = q()
    codes = [int(v) for v in rng.integers(0, 4, size=nq)]
    codes[c] = 0
    if all(v == 0 for v in codes):
        codes[(c + 1) % nq] = 1
    L.append(f"CPSTR 1 {c} 1 {pauli_text(codes)}")
    L.append(f"CPG 1 {c} 0 {pauli_text(codes)} {ang()}")
    t = distinct(min(3, nq)); L.append(f"PHG {len(t)} {' '.join(map(str, t))} {ang()}")
    t = distinct(min(3, nq)); L.append(f"MPS {len(t)} {' '.join(map(str, t))} {ang()}")
    t = distinct(min(4, nq)); L.append(f"QFT {len(t)} {' '.join(map(str, t))}")
    L.append("FQFT")
    if is_dm:
        L.append(f"DEPOL {q()} {fmt(rng.uniform(0, 0.5))}")
        a, b = distinct(2); L.append(f"DEPOL2 {a} {b} {fmt(rng.uniform(0, 0.5))}")
        L.append(f"DEPHASE {q()} {fmt(rng.uniform(0, 0.4))}")
        a, b = distinct(2); L.append(f"DEPHASE2 {a} {b} {fmt(rng.uniform(0, 0.4))}")
        L.append(f"DAMP {q()} {fmt(rng.uniform(0, 0.9))}")
        px, py, pz = rng.uniform(0, 0.1, size=3)
        L.append(f"PAULIS {q()} {fmt(px)} {fmt(py)} {fmt(pz)}")
        for k in (1, 2):
            t = distinct(k)
            ops = random_kraus(k, 4, rng)
            L.append(f"KRAUS {k} {' '.join(map(str, t))} 4 " + " ".join(mat_tokens(o) for o in ops))
    L.append("TOTALPROB")
    L.append("PURITY")
    for o in (0, 1):
        L.append(f"PROBQ {q()} {o}")
    t = distinct(min(3, nq)); L.append(f"PROBMQ {len(t)} {' '.join(map(str, t))} {' '.join(str(int(v)) for v in rng.integers(0, 2, size=len(t)))}")
    for _ in range(6):
        L.append(f"EXPEC {pauli_text([int(v) for v in rng.integers(0, 4, size=nq)])}")
    L.append(f"EXPEC {pauli_text([int(v) * 3 for v in rng.integers(0, 2, size=nq)])}")
    L.append(f"EXPEC {'I' * nq}")
    t = distinct(min(3, nq)); L.append(f"PROBALL {len(t)} {' '.join(map(str, t))}")
    L.append(expsum_line(nq, 5, rng))
    if with_measure:
        L.append(f"SEED {int(rng.integers(1 << 31))} {int(rng.integers(1 << 31))}")
        m = distinct(min(nq, 4))
        L.append(f"MEAS {m[0]}")
        L.append(f"MEAS {m[1]}")
        L.append("TOTALPROB")
        if nq >= 4:
            L.append(f"FMEAS {m[3]} {int(rng.integers(2))}")
            L.append(f"MEASM 2 {m[0]} {m[2]}")
            L.append("TOTALPROB")
        # a projector on a qubit not measured keeps part of the state (unnormalised)
        L.append(f"PROJ 1 {m[2]} {int(rng.integers(2))}")
        L.append("TOTALPROB")
    return "\n".join(L) + "\n"


def expsum_line(nq, num_terms, rng):
    """calcExpecPauliStrSum over `num_terms` random strings with real Gaussian coefficients."""
    terms = " ".join(f"{fmt(rng.standard_normal())} 0.0 {pauli_text([int(v) for v in rng.integers(0, 4, size=nq)])}"
                     for _ in range(num_terms))
    return f"EXPSUM {num_terms} {terms}"


def measure_sum_circuit(nq, is_dm, seed):
    """Outcome histograms, Pauli-string sums and the multi-qubit and forced measurements,
    on a register prepared by a few gates (nq >= 4)."""
    rng = np.random.default_rng(seed)
    L = [f"H {t}" for t in range(nq)]
    for t in range(nq):
        L.append(f"U1 {t} {mat_tokens(haar_unitary(2, rng))}")
    L.append(f"U2 0 {nq - 1} {mat_tokens(haar_unitary(4, rng))}")
    if is_dm:
        L.append(f"DEPOL 1 {fmt(0.05)}")
    L.append("PROBALL 1 0")
    L.append(f"PROBALL 3 {nq - 1} 0 2")
    L.append(f"PROBALL {nq} {' '.join(str(q) for q in range(nq))}")
    L.append(expsum_line(nq, 7, rng))
    L.append(f"EXPSUM 2 1.5 0.0 {'I' * nq} -0.5 0.0 {'Z' * nq}")
    L.append(f"SEED {int(rng.integers(1 << 31))}")
    L.append(f"MEASM 3 2 0 {nq - 1}")
    L.append("TOTALPROB")
    L.append(f"FMEAS 1 {int(rng.integers(2))}")
    L.append(f"FMEASM 1 3 {int(rng.integers(2))}")
    L.append("TOTALPROB")
    L.append(f"MEASM 1 1")
    L.append(f"MEASM {nq} {' '.join(str(q) for q in reversed(range(nq)))}")
    L.append("TOTALPROB")
    return "\n".join(L) + "\n"


def config1_circuit(nq, layers, seed, num_expec=16):
    """The CPU-runnable plain method: `layers` x (H on all qubits; RX, RY, RZ on
    every qubit with angles U[0,2pi); CNOT ladder q->q+1), then calcTotalProb and
    `num_expec` Pauli expectations with I/X/Y/Z uniform per qubit."""
    rng = np.random.default_rng(seed)
    L = []
    for _ in range(layers):
        for t in range(nq):
            L.append(f"H {t}")
        for t in range(nq):
            for op in ("RX", "RY", "RZ"):
                L.append(f"{op} {t} {fmt(rng.uniform(0, 2 * np.pi))}")
        for t in range(nq - 1):
            L.append(f"CX {t} {t + 1}")
    L.append("TOTALPROB")
    for _ in range(num_expec):
        L.append(f"EXPEC {pauli_text([int(v) for v in rng.integers(0, 4, size=nq)])}")
    return "\n".join(L) + "\n"


def isometry_kraus(rng):
    """Four 4x4 Kraus operators: the 4x4 blocks of a random 16x4 isometry (QR of a
    complex Gaussian matrix), so sum_i K_i^dagger K_i = I."""
    g = rng.standard_normal((16, 4)) + 1j * rng.standard_normal((16, 4))
    q, r = np.linalg.qr(g)
    q = q * (np.diag(r) / np.abs(np.diag(r)))
    return [q[4 * i:4 * i + 4, :] for i in range(4)]


def config3_circuit(nq, layers, seed, num_expec=16):
    """The density-matrix method: `layers` x (random 1-qubit Haar unitaries on every
    qubit on even layers, random 2-qubit Haar unitaries on disjoint random pairs on odd
    layers; each layer followed by mixDepolarising(p=0.01) on every qubit and one
    random 2-qubit 4-operator CPTP mixKrausMap), then calcPurity and `num_expec`
    Pauli expectations with I/X/Y/Z uniform per qubit."""
    rng = np.random.default_rng(seed)
    L = []
    for layer in range(layers):
        if layer % 2 == 0:
            for t in range(nq):
                L.append(f"U1 {t} {mat_tokens(haar_unitary(2, rng))}")
        else:
            perm = [int(v) for v in rng.permutation(nq)]
            for i in range(0, nq - 1, 2):
                L.append(f"U2 {perm[i]} {perm[i + 1]} {mat_tokens(haar_unitary(4, rng))}")
        for t in range(nq):
            L.append(f"DEPOL {t} {fmt(0.01)}")
        a, b = (int(v) for v in rng.choice(nq, size=2, replace=False))
        L.append(f"KRAUS 2 {a} {b} 4 " + " ".join(mat_tokens(o) for o in isometry_kraus(rng)))
    L.append("PURITY")
    for _ in range(num_expec):
        L.append(f"EXPEC {pauli_text([int(v) for v in rng.integers(0, 4, size=nq)])}")
    return "\n".join(L) + "\n"


def fullstate_diag_circuit(nq, is_dm, seed):
    """FullStateDiagMatr on a register prepared by a few gates: apply (unit-modulus
    elements), apply with a real power, multiply (general elements), multiply with a
    complex power, then the four expectation forms (Hermitian, Hermitian with a real
    power of positive elements, non-Hermitian, non-Hermitian with a complex power)."""
    rng = np.random.default_rng(seed)
    dim = 1 << nq

    def elems(kind):
        if kind == "phase":
            return np.exp(1j * rng.uniform(0, 2 * np.pi, dim))
        if kind == "real+":
            return rng.uniform(0.2, 2.0, dim).astype(np.complex128)
        if kind == "real":
            return rng.uniform(-2.0, 2.0, dim).astype(np.complex128)
        return (rng.uniform(0.3, 1.5, dim) * np.exp(1j * rng.uniform(0, 2 * np.pi, dim)))

    L = [f"H {t}" for t in range(nq)]
    L.append(f"U1 0 {mat_tokens(haar_unitary(2, rng))}")
    if nq > 1:
        L.append(f"U2 0 {nq - 1} {mat_tokens(haar_unitary(4, rng))}")
    L.append(f"FSD 0 0 {mat_tokens(elems('phase'))}")
    L.append(f"FSD 0 1 {fmt(rng.uniform(-2, 2))} 0.0 {mat_tokens(elems('phase'))}")
    L.append("TOTALPROB")
    L.append(f"EXPFSD 0 {mat_tokens(elems('real'))}")
    L.append(f"EXPFSD 1 {fmt(rng.uniform(0.5, 2.5))} {mat_tokens(elems('real+'))}")
    L.append(f"EXPFSD 2 {mat_tokens(elems('general'))}")
    L.append(f"EXPFSD 3 {fmt(rng.uniform(-1, 2))} {fmt(rng.uniform(-1, 1))} {mat_tokens(elems('general'))}")
    L.append(f"EXPEC {pauli_text([int(v) for v in rng.integers(0, 4, size=nq)])}")
    # multiplying leaves a density matrix non-Hermitian: only the total probability after
    L.append(f"FSD 1 0 {mat_tokens(elems('general'))}")
    L.append(f"FSD 1 1 {fmt(rng.uniform(0.5, 1.5))} {fmt(rng.uniform(-0.5, 0.5))} {mat_tokens(elems('general'))}")
    L.append("TOTALPROB")
    return "\n".join(L) + "\n"


def benchmark_circuit_text(nq, depth, seed):
    """The 30-qubit benchmark's circuit at nq qubits: per layer a Haar 2x2 on every qubit
    and a controlled phase of random angle on 15 disjoint random pairs, then the QFT."""
    rng = np.random.default_rng(seed)
    L = []
    for _ in range(depth):
        for t in range(nq):
            L.append(f"U1 {t} {mat_tokens(haar_unitary(2, rng))}")
        perm = rng.permutation(nq)
        for p in range(min(15, nq // 2)):
            L.append(f"CPS {int(perm[2 * p])} {int(perm[2 * p + 1])} {fmt(rng.uniform(0, 2 * np.pi))}")
    L.append("FQFT")
    L.append("TOTALPROB")
    return "\n".join(L) + "\n"
