"""The continuous-batching server on the GPU: served results (FP32 fused, small
registers in shared memory, large ones on streams) against the FP64 oracle;
each request's result is the same alone and in a mix of other requests; the
queue drains when the HBM budget cannot hold every request at once."""
import numpy as np
import pytest

import qcircuits as qc

pytestmark = pytest.mark.gpu


def _requests(sizes, seed):
    from quest_gb300.serve import hea_request
    rng = np.random.default_rng(seed)
    out = []
    for n in sizes:
        depth = int(rng.integers(3, 9))
        out.append((n, hea_request(n, depth, rng)))
    return out


def test_served_results_match_the_fp64_oracle(env):
    from quest_gb300.serve import Server, circuit_of, text_of
    reqs = _requests([5, 8, 11, 13, 14, 15, 16, 18], 1)
    server = Server(1 << 30)
    try:
        got = server.run_all([(circuit_of(n, ops), codes) for n, (ops, codes) in reqs])
    finally:
        server.close()
    for (n, (ops, codes)), vals in zip(reqs, got):
        zero = np.zeros(1 << n, dtype=np.complex128)
        zero[0] = 1
        _, want, _ = qc.oracle().run(text_of(ops, codes), n, 0, zero)
        assert np.max(np.abs(vals - want)) < 2e-5, n


def test_result_is_the_same_alone_and_in_the_mix(env):
    from quest_gb300.serve import Server, circuit_of
    probe = _requests([12, 17], 7)
    others = _requests([6, 9, 10, 12, 13, 14, 15, 16, 17, 19, 8, 11, 14, 18], 8)
    alone = []
    for n, (ops, codes) in probe:
        s = Server(1 << 30)
        try:
            alone.append(s.run_all([(circuit_of(n, ops), codes)])[0])
        finally:
            s.close()
    mix = [(circuit_of(n, ops), codes) for n, (ops, codes) in others]
    mix.insert(3, (circuit_of(probe[0][0], probe[0][1][0]), probe[0][1][1]))
    mix.insert(9, (circuit_of(probe[1][0], probe[1][1][0]), probe[1][1][1]))
    s = Server(1 << 30)
    try:
        got = s.run_all(mix)
    finally:
        s.close()
    assert np.max(np.abs(got[3] - alone[0])) <= 1e-12
    assert np.max(np.abs(got[9] - alone[1])) <= 1e-12


def test_queue_drains_under_a_tight_memory_budget(env):
    from quest_gb300.serve import Server, circuit_of
    reqs = _requests([18, 19, 18, 19, 18, 19], 3)
    # room for about one 19-qubit register (4 MiB state + circuit) at a time
    s = Server(12 << 20)
    try:
        got = s.run_all([(circuit_of(n, ops), codes) for n, (ops, codes) in reqs])
        assert s.stats()["hbm_in_use"] == 0
    finally:
        s.close()
    assert len(got) == 6 and all(np.all(np.isfinite(v)) for v in got)


@pytest.mark.parametrize("n", [4, 16])
def test_values_are_normalised_only_for_unitary_circuits(env, n):
    """<P> / <psi|psi> when every gate is unitary; <psi|P|psi> as computed otherwise."""
    from quest_gb300.fused import Circuit
    from quest_gb300.serve import Server
    h = np.array([[1, 1], [1, -1]]) / np.sqrt(2)
    damp = np.diag([1.0, 0.5])          # not unitary: shrinks the norm
    codes = [[3] + [0] * (n - 1), [1] * n, [0] * n]
    for unitary in (True, False):
        c = Circuit(n)
        for q in range(n):
            c.add([q], h)
        if not unitary:
            c.add([0], damp)
        c.fuse(5)
        psi = np.ones(1 << n) / np.sqrt(1 << n)
        if not unitary:
            psi = psi * np.where(np.arange(1 << n) & 1, 0.5, 1.0)
        sign = np.where(np.arange(1 << n) & 1, -1.0, 1.0)
        z0, xall, ident = np.vdot(psi, sign * psi).real, np.vdot(psi, psi[::-1]).real, np.vdot(psi, psi).real
        server = Server(1 << 30)
        try:
            got = server.run_all([(c, codes)])[0]
        finally:
            server.close()
        want = np.array([z0, xall, ident]) / (ident if unitary else 1.0)
        assert np.max(np.abs(got - want)) < 1e-6, (unitary, got, want)


def test_cancelled_requests_free_their_memory(env):
    """A client that goes away: one request cancelled while on the GPU, one while still
    queued.  The others complete with the right values and nothing stays held."""
    from quest_gb300.serve import Server, circuit_of, text_of
    reqs = _requests([9, 18, 18, 12, 18, 10], 5)
    circs = [circuit_of(n, ops) for n, (ops, codes) in reqs]
    server = Server(6 << 20)          # room for one 18-qubit request at a time
    try:
        ids = [server.submit(c, codes) for c, (n, (ops, codes)) in zip(circs, reqs)]
        server.poll()                 # admits and launches what fits
        st = server.stats()
        assert st["in_flight"] >= 1 and st["queued"] >= 1
        running, queued = ids[1], ids[4]
        server.cancel(running)
        server.cancel(queued)
        keep = [i for i in ids if i not in (running, queued)]
        got = {}
        for _ in range(100000):
            server.poll()
            for rid in keep:
                if rid not in got:
                    done, vals = server.result(rid)
                    if done:
                        got[rid] = vals
            if len(got) == len(keep):
                break
        assert len(got) == len(keep)
        for k, rid in enumerate(ids):
            if rid in got:
                n, (ops, codes) = reqs[k]
                zero = np.zeros(1 << n, dtype=np.complex128)
                zero[0] = 1
                _, want, _ = qc.oracle().run(text_of(ops, codes), n, 0, zero)
                assert np.max(np.abs(got[rid] - want)) < 2e-5
                server.release(rid)
        for _ in range(1000):          # the cancelled request still on the GPU retires too
            server.poll()
            if server.stats()["hbm_in_use"] == 0:
                break
        st = server.stats()
        assert st == {**st, "queued": 0, "in_flight": 0, "hbm_in_use": 0}
        with pytest.raises(Exception):
            server.result(running)
    finally:
        server.close()


def test_budget_larger_than_the_gpu_is_refused(env):
    from quest_gb300.serve import Server
    with pytest.raises(Exception):
        Server(1 << 50)               # a petabyte: the allocation fails cleanly
