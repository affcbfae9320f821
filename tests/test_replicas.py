"""The replica path of bench.py on CPU: world_size-2 gloo ranks run the same set-up,
barrier and max-over-ranks timing that one process per GPU runs under torchrun (the
path has no data-path collective; each rank owns its own register).  Also checks
that under torchrun only rank 0 runs the reference arm."""
import importlib.util
import os
import socket

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
BENCH = os.path.join(HERE, "..", "bench.py")


def _bench():
    spec = importlib.util.spec_from_file_location("qg_bench", BENCH)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    os.environ.update({"WORLD_SIZE": str(world), "RANK": str(rank), "LOCAL_RANK": str(rank),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    b = _bench()
    w, r, local, dist = b.dist_setup()
    assert (w, r, local) == (world, rank, rank) and dist is not None and dist.get_backend() == "gloo"
    b.barrier(dist)
    # each replica's own timing; the job's time is the slowest replica's
    t = b.max_over_ranks(dist, 1.5 + rank)
    b.barrier(dist)
    dist.destroy_process_group()
    out.put((rank, t))


def test_two_gloo_replicas_agree_on_the_slowest_time():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
    assert all(p.exitcode == 0 for p in procs), [p.exitcode for p in procs]
    got = dict(q.get(timeout=10) for _ in procs)
    assert got == {0: 2.5, 1: 2.5}


def test_single_process_needs_no_process_group():
    b = _bench()
    for k in ("WORLD_SIZE", "RANK", "LOCAL_RANK"):
        os.environ.pop(k, None)
    world, rank, local, dist = b.dist_setup()
    assert (world, rank, local, dist) == (1, 0, 0, None)
    assert b.max_over_ranks(None, 3.25) == 3.25


def test_reference_arm_runs_on_rank_zero_only(capsys):
    b = _bench()

    class Args:
        qubits, depth, warmup, steps, cpu_sample = 12, 1, 0, 1, 2

    b.run_reference(Args, 2, 1, None)        # rank 1 of 2: no work, no output
    assert capsys.readouterr().out == ""


def test_benchmark_circuits_match_the_parity_tests():
    """The circuits bench.py times are the ones the parity tests hold against the oracle:
    the plain method (c1) draws the same angles and Pauli codes as the tests' text form
    (and its CPU baseline runs that text), and the 30-qubit circuit has the stated
    1380 gates (600 Haar 2x2, 300 controlled phases on disjoint pairs, the QFT)."""
    import numpy as np
    import qcircuits as qc
    b = _bench()
    nq, layers, seed = 20, 10, 0x5155455354 + 1
    gates, codes = b.c1_gates(nq, layers, seed)
    text = qc.config1_circuit(nq, layers, seed, len(codes)).splitlines()
    ops = [l.split() for l in text]
    gate_lines = [o for o in ops if o[0] in ("H", "RX", "RY", "RZ", "CX")]
    assert len(gate_lines) == len(gates) == layers * (nq + 3 * nq + nq - 1)
    for g, o in zip(gates, gate_lines):
        assert g[0] == o[0] and g[1] == int(o[1])
        if g[0] in ("RX", "RY", "RZ"):
            assert g[2] == float(o[2])
        if g[0] == "CX":
            assert g[2] == int(o[2])
    expec = [o for o in ops if o[0] == "EXPEC"]
    assert [qc.pauli_text(c) for c in codes] == [o[1] for o in expec]
    circ = b.make_circuit(30, 20, 7)
    assert b.num_gates(circ, 30) == 1380
    us = [g for g in circ if g[0] == "U"]
    cps = [g for g in circ if g[0] == "CP"]
    assert len(us) == 600 and len(cps) == 300 and circ[-1] == ("QFT",)
    for layer in range(20):
        pairs = cps[15 * layer:15 * layer + 15]
        qubits = [q for g in pairs for q in g[1:3]]
        assert len(set(qubits)) == 30                      # disjoint pairs covering every qubit
        assert all(np.allclose(u[2] @ u[2].conj().T, np.eye(2)) for u in us[30 * layer:30 * layer + 30])
