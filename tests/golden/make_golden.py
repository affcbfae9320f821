"""Generates the golden fixtures in this folder by running each circuit through
the REFERENCE QuEST library (oracle/_ref/libqref.so, built from the reference's
own sources by `make -C oracle ref REF=<QuEST sources>`).

Each fixture stores the circuit text, the input amplitudes, and the reference's
output amplitudes, reduction results and sampled measurement outcomes.

    python tests/golden/make_golden.py [case names]
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))
import qcircuits as qc  # noqa: E402

CASES = [
    # name, nq, is_dm, kind, seed
    ("sv1_every", 1, 0, "tiny", 11),
    ("sv2_every", 2, 0, "tiny", 12),
    ("sv5_every", 5, 0, "every", 13),
    ("sv6_every", 6, 0, "every", 14),
    ("sv8_every", 8, 0, "every", 15),
    ("dm1_every", 1, 1, "tiny", 21),
    ("dm3_every", 3, 1, "every", 22),
    ("dm4_every", 4, 1, "every", 23),
    ("dm5_every", 5, 1, "every", 24),
    ("sv12_config1", 12, 0, "config1", 31),
    ("dm6_config3", 6, 1, "config3", 41),
    ("sv5_fullstate_diag", 5, 0, "fsd", 51),
    ("dm3_fullstate_diag", 3, 1, "fsd", 52),
    ("sv7_measure_sum", 7, 0, "measure", 61),
    ("dm4_measure_sum", 4, 1, "measure", 62),
]


def tiny_circuit(nq, is_dm, seed):
    """Edge case: one- and two-qubit registers, every op that fits."""
    rng = np.random.default_rng(seed)
    L = [f"H 0", f"X 0", f"Y 0", f"Z 0", f"S 0", f"T 0",
         f"RX 0 {qc.fmt(rng.uniform(0, 6.28))}", f"RY 0 {qc.fmt(rng.uniform(0, 6.28))}",
         f"RZ 0 {qc.fmt(rng.uniform(0, 6.28))}", f"PS 0 {qc.fmt(rng.uniform(0, 6.28))}",
         f"U1 0 {qc.mat_tokens(qc.haar_unitary(2, rng))}",
         f"D1 0 {qc.mat_tokens(np.exp(1j * rng.uniform(0, 6.28, 2)))}",
         f"PSTR {'Y' * nq}", f"PG {'X' * nq} {qc.fmt(rng.uniform(0, 6.28))}",
         f"PG {'I' * nq} {qc.fmt(rng.uniform(0, 6.28))}"]
    if nq >= 2:
        L += [f"CX 0 1", f"CZ 1 0", f"SWAP 0 1", f"CPS 0 1 {qc.fmt(rng.uniform(0, 6.28))}",
              f"U2 1 0 {qc.mat_tokens(qc.haar_unitary(4, rng))}", "FQFT"]
    if is_dm:
        L += [f"DEPOL 0 {qc.fmt(rng.uniform(0, 0.5))}", f"DAMP 0 0.3", f"DEPHASE 0 0.2",
              f"PAULIS 0 0.05 0.02 0.07",
              f"KRAUS 1 0 3 " + " ".join(qc.mat_tokens(o) for o in qc.random_kraus(1, 3, rng))]
    L += ["TOTALPROB", "PURITY", "PROBQ 0 1", f"EXPEC {'X' * nq}", f"EXPEC {'Z' * nq}",
          f"EXPEC {'Y' * nq}", "SEED 7 8 9", "MEAS 0", "TOTALPROB"]
    return "\n".join(L) + "\n"


def config3_circuit(nq, layers, seed):
    """Density-matrix method in small: layers of random 1-/2-qubit Haar unitaries,
    each followed by depolarising p=0.01 on all qubits and one random 2-qubit
    4-operator Kraus map; then purity and 16 Pauli expectations."""
    rng = np.random.default_rng(seed)
    L = []
    for _ in range(layers):
        for t in range(nq):
            L.append(f"U1 {t} {qc.mat_tokens(qc.haar_unitary(2, rng))}")
        a, b = [int(v) for v in rng.choice(nq, 2, replace=False)]
        L.append(f"U2 {a} {b} {qc.mat_tokens(qc.haar_unitary(4, rng))}")
        for t in range(nq):
            L.append(f"DEPOL {t} 0.01")
        a, b = [int(v) for v in rng.choice(nq, 2, replace=False)]
        L.append(f"KRAUS 2 {a} {b} 4 " + " ".join(qc.mat_tokens(o) for o in qc.random_kraus(2, 4, rng)))
    L.append("PURITY")
    for _ in range(16):
        L.append(f"EXPEC {qc.pauli_text([int(v) for v in rng.integers(0, 4, size=nq)])}")
    return "\n".join(L) + "\n"


def make_case(name, nq, is_dm, kind, seed):
    if kind == "tiny":
        text = tiny_circuit(nq, is_dm, seed)
    elif kind == "every":
        text = qc.every_op_circuit(nq, is_dm, seed)
    elif kind == "config1":
        text = qc.config1_circuit(nq, 3, seed)
    elif kind == "fsd":
        text = qc.fullstate_diag_circuit(nq, is_dm, seed)
    elif kind == "measure":
        text = qc.measure_sum_circuit(nq, is_dm, seed)
    else:
        text = config3_circuit(nq, 3, seed)
    amps = qc.random_density_matrix(nq, seed) if is_dm else qc.random_statevector(nq, seed)
    return text, amps


def main():
    ref = qc.reference()
    if ref is None:
        sys.exit("the reference library is not built: make -C oracle ref REF=<QuEST sources>")
    only = set(sys.argv[1:])          # optional: names of the cases to (re)generate
    for name, nq, is_dm, kind, seed in CASES:
        if only and name not in only:
            continue
        text, amps = make_case(name, nq, is_dm, kind, seed)
        out, res, outs = ref.run(text, nq, is_dm, amps)
        np.savez_compressed(os.path.join(HERE, name + ".npz"), text=np.array(text), nq=nq, is_dm=is_dm,
                            amps_in=amps, amps_out=out, results=res, outcomes=outs)
        print(f"{name}: {len(text.splitlines())} ops, {len(res)} results, outcomes {outs.tolist()}")


if __name__ == "__main__":
    main()
