"""Host-side gate fusion (no GPU): the product of the fused blocks equals the
product of the circuit's gates, every block fits the fusion width, and fusion
reduces the number of passes."""
import numpy as np
import pytest

import qcircuits as qc


def full_operator(n, targs, m):
    """2^n x 2^n operator of matrix m on `targs` (index bit i <-> targs[i])."""
    dim = 1 << n
    k = len(targs)
    out = np.zeros((dim, dim), dtype=np.complex128)
    mask = sum(1 << t for t in targs)
    for col in range(dim):
        j = sum(((col >> t) & 1) << i for i, t in enumerate(targs))
        base = col & ~mask
        for r in range(1 << k):
            row = base | sum(((r >> i) & 1) << t for i, t in enumerate(targs))
            out[row, col] += m[r, j]
    return out


def brickwork(n, depth, rng):
    gates = []
    cz = np.diag([1, 1, 1, -1]).astype(np.complex128)
    for d in range(depth):
        for t in range(n):
            gates.append(([t], qc.haar_unitary(2, rng)))
        for t in range(d % 2, n - 1, 2):
            gates.append(([t, t + 1], cz))
    return gates


@pytest.mark.parametrize("n,depth,k", [(6, 4, 5), (7, 6, 3), (8, 5, 4), (5, 3, 2), (6, 3, 2)])
def test_fused_blocks_reproduce_the_circuit(built_lib, n, depth, k):
    from quest_gb300.fused import Circuit
    rng = np.random.default_rng(n * 100 + depth)
    gates = brickwork(n, depth, rng)
    # a few random 2-qubit unitaries on distant qubits too
    for _ in range(3):
        a, b = [int(v) for v in rng.choice(n, 2, replace=False)]
        gates.append(([a, b], qc.haar_unitary(4, rng)))
    c = Circuit(n)
    for t, m in gates:
        c.add(t, m)
    c.fuse(k)
    expect = np.eye(1 << n, dtype=np.complex128)
    for t, m in gates:
        expect = full_operator(n, t, m) @ expect
    got = np.eye(1 << n, dtype=np.complex128)
    for i in range(c.num_blocks):
        t, m = c.block(i)
        assert len(t) <= k and t == sorted(t)
        got = full_operator(n, t, m) @ got
    assert np.max(np.abs(got - expect)) < 1e-12
    if k >= 4:
        assert c.num_blocks < len(gates) / 2


def test_fusion_rejects_wide_gate(built_lib):
    from quest_gb300.fused import Circuit
    from quest_gb300._lib import BackendError
    c = Circuit(4)
    c.add([0, 1, 2], qc.haar_unitary(8, np.random.default_rng(0)))
    with pytest.raises(BackendError):
        c.fuse(2)


def test_diagonal_gates_held_back_keep_the_circuit(built_lib):
    """Diagonal gates (RZ, CZ ladder, controlled phases) that the fuser defers past
    commuting gates still give the circuit's exact product."""
    from quest_gb300.fused import Circuit
    rng = np.random.default_rng(99)
    n = 7
    cz = np.diag([1, 1, 1, -1]).astype(np.complex128)
    gates = []
    for _ in range(4):
        for t in range(n):
            th = rng.uniform(0, 2 * np.pi)
            gates.append(([t], np.array([[np.cos(th / 2), -np.sin(th / 2)], [np.sin(th / 2), np.cos(th / 2)]])))
        for t in range(n):
            gates.append(([t], np.diag(np.exp(1j * rng.uniform(0, 6.3, 2)))))
        for t in range(n - 1):
            gates.append(([t, t + 1], cz))
        a, b = [int(v) for v in rng.choice(n, 2, replace=False)]
        gates.append(([a, b], np.diag(np.exp(1j * rng.uniform(0, 6.3, 4)))))
    c = Circuit(n)
    for t, m in gates:
        c.add(t, m)
    c.fuse(5)
    expect = np.eye(1 << n, dtype=np.complex128)
    for t, m in gates:
        expect = full_operator(n, t, m) @ expect
    got = np.eye(1 << n, dtype=np.complex128)
    for i in range(c.num_blocks):
        t, m = c.block(i)
        got = full_operator(n, t, m) @ got
    assert np.max(np.abs(got - expect)) < 1e-12
    assert c.num_blocks <= len(gates) / 6
