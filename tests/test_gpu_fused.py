"""FP32 fused-block path on the GPU (SIMT and tcgen05 3xTF32 kernels) against the
FP64 oracle applying the same gates one by one.

Bar (precision form): fidelity |<psi32|psi64>|^2 >= 1 - 1e-6; max-abs amplitude
error <= 2e-6 x max|psi| (SIMT) or 1e-5 x max|psi| (3xTF32 tensor cores) over
whole circuits, <= 2e-6 x max|psi| for a single block."""
import ctypes

import numpy as np
import pytest

import qcircuits as qc

pytestmark = pytest.mark.gpu
CZ = np.diag([1, 1, 1, -1]).astype(np.complex128)


def run_oracle(n, amps, gates):
    lines = []
    for t, m in gates:
        if len(t) == 1:
            lines.append(f"U1 {t[0]} {qc.mat_tokens(m)}")
        elif len(t) == 2:
            lines.append(f"U2 {t[0]} {t[1]} {qc.mat_tokens(m)}")
        else:
            lines.append(f"UK {len(t)} {' '.join(map(str, t))} {qc.mat_tokens(m)}")
    out, _, _ = qc.oracle().run("\n".join(lines) + "\n", n, 0, amps)
    return out


def run_fused(env, n, amps, gates, k, impl):
    from quest_gb300.fused import Circuit, StateVector32
    c = Circuit(n)
    for t, m in gates:
        c.add(t, m)
    c.fuse(k)
    s = StateVector32(n)
    try:
        s.set(amps)
        c.apply(s, impl=impl)
        return s.get().astype(np.complex128), c.num_blocks
    finally:
        s.free()


def brickwork(n, depth, rng):
    gates = []
    for d in range(depth):
        for t in range(n):
            gates.append(([t], qc.haar_unitary(2, rng)))
        for t in range(d % 2, n - 1, 2):
            gates.append(([t, t + 1], CZ))
    return gates


def fidelity(a, b):
    return abs(np.vdot(a, b)) ** 2 / (np.vdot(a, a).real * np.vdot(b, b).real)


@pytest.mark.parametrize("n,depth", [(12, 6), (15, 8), (18, 10)])
@pytest.mark.parametrize("impl", [1, 2])
def test_fused_brickwork_vs_fp64_oracle(env, n, depth, impl):
    rng = np.random.default_rng(n * 10 + depth)
    gates = brickwork(n, depth, rng)
    amps = qc.random_statevector(n, n)
    ref = run_oracle(n, amps, gates)
    got, nblocks = run_fused(env, n, amps, gates, 5, impl)
    scale = np.max(np.abs(ref))
    assert fidelity(got, ref) >= 1 - 1e-6
    # SIMT FP32 stays within 2e-6 of max|psi|; 3xTF32 on the tensor cores (22-bit
    # split operands) within 1e-5 over these 20-60 block passes
    assert np.max(np.abs(got - ref)) <= (2e-6 if impl == 1 else 1e-5) * scale
    assert nblocks < len(gates) / 3
    from quest_gb300 import _lib
    flag = ctypes.c_int(0)
    _lib.lib().qg_tc_get_error_flag(ctypes.byref(flag))
    assert flag.value == 0


# The tensor-core kernel picks its mode from how many 128-byte lines one warp instruction
# would touch row by row: 32 lines (e.g. targets 0-4, or 0-3 and any) load and store in
# address order through shared memory, 16 lines (e.g. 1-5) load that way only, and the
# rest go row by row.  These layouts cover all three.
@pytest.mark.parametrize("n,targs", [(14, [0, 1, 2, 3, 4]), (14, [7, 8, 9, 10, 11]), (14, [11, 0, 6, 3, 9]),
                                     (14, [2, 5, 6, 10, 13]), (14, [13, 12, 1, 0, 7]), (14, [1, 2, 3, 4, 5]),
                                     (14, [4, 5, 6, 7, 8]), (14, [5, 6, 7, 8, 9]), (12, [0, 1, 2, 3, 11]),
                                     (12, [11, 10, 9, 8, 7])])
def test_single_5qubit_block_every_layout(env, n, targs):
    rng = np.random.default_rng(sum(targs))
    u = qc.haar_unitary(32, rng)
    amps = qc.random_statevector(n, 3)
    ref = run_oracle(n, amps, [(targs, u)])
    scale = np.max(np.abs(ref))
    simt, _ = run_fused(env, n, amps, [(targs, u)], 5, 1)
    tc, _ = run_fused(env, n, amps, [(targs, u)], 5, 2)
    assert np.max(np.abs(simt - ref)) <= 2e-6 * scale
    assert np.max(np.abs(tc - ref)) <= 2e-6 * scale
    assert np.max(np.abs(tc - simt)) <= 2e-6 * scale


def test_fp32_reductions_accumulate_in_fp64(env):
    from quest_gb300.fused import StateVector32
    n = 16
    amps = qc.random_statevector(n, 8).astype(np.complex64)
    s = StateVector32(n)
    try:
        s.set(amps)
        a64 = amps.astype(np.complex128)
        assert abs(s.total_prob() - np.vdot(a64, a64).real) < 1e-12
        rng = np.random.default_rng(1)
        codes = [[int(v) for v in rng.integers(0, 4, n)] for _ in range(20)]
        got = s.expec_paulis(codes)
        text = "".join(f"EXPEC {qc.pauli_text(c)}\n" for c in codes)
        _, want, _ = qc.oracle().run(text, n, 0, a64)
        assert np.max(np.abs(got - want)) < 1e-12
    finally:
        s.free()


@pytest.mark.gpu
def test_normalise_rescales_to_the_target_probability(env):
    from quest_gb300.fused import StateVector32
    n = 18
    amps = (qc.random_statevector(n, 9) * 0.93).astype(np.complex64)
    s = StateVector32(n)
    try:
        s.set(amps)
        s.normalise(0.5)
        got = s.get().astype(np.complex128)
        a64 = amps.astype(np.complex128)
        want = a64 * np.sqrt(0.5 / np.vdot(a64, a64).real)
        assert np.max(np.abs(got - want)) <= 4 * np.finfo(np.float32).eps * np.max(np.abs(want))
        assert abs(s.total_prob() - 0.5) < 1e-6
    finally:
        s.free()


def test_fp32_norm_and_rescale_on_an_8_byte_aligned_pointer(env):
    # the norm and rescale kernels move 16-byte amplitude pairs when the pointer allows
    # it; a pointer that is only 8-byte aligned takes their one-amplitude path
    from quest_gb300 import _lib
    lib = _lib.lib()
    n = 15
    amps = (qc.random_statevector(n, 21) * 1.7).astype(np.complex64)
    a64 = amps.astype(np.complex128)
    want_sum = np.vdot(a64, a64).real
    base = ctypes.c_void_p()
    _lib.check(lib.qg_alloc(ctypes.byref(base), (len(amps) + 2) * 8))
    try:
        for shift in (0, 8):
            ptr = ctypes.c_void_p(base.value + shift)
            _lib.check(lib.qg_copy_h2d(ptr, amps.ctypes.data, amps.nbytes, None))
            lib.qg_sync()
            tot = ctypes.c_double()
            _lib.check(lib.qg_sv32_calcTotalProb(ptr, n, ctypes.byref(tot), None))
            assert abs(tot.value - want_sum) < 1e-12 * want_sum
            _lib.check(lib.qg_sv32_normalise(ptr, n, 1.0, None))
            got = np.empty_like(amps)
            _lib.check(lib.qg_copy_d2h(got.ctypes.data, ptr, got.nbytes, None))
            want = a64 / np.sqrt(want_sum)
            assert np.max(np.abs(got.astype(np.complex128) - want)) <= 4 * np.finfo(np.float32).eps * np.max(np.abs(want))
    finally:
        lib.qg_free(base)


@pytest.mark.parametrize("impl", [1, 2])
def test_graph_replays_the_circuit(env, impl):
    """A CUDA graph of the block kernels gives the same bits as applying the circuit."""
    from quest_gb300.fused import Circuit, StateVector32
    n = 14
    rng = np.random.default_rng(21)
    gates = brickwork(n, 6, rng)
    amps = qc.random_statevector(n, 21)
    c = Circuit(n)
    for t, m in gates:
        c.add(t, m)
    c.fuse(5)
    direct, replay = StateVector32(n), StateVector32(n)
    try:
        direct.set(amps)
        c.apply(direct, impl=impl)
        c.apply(direct, impl=impl)
        replay.set(amps)
        g = c.graph(replay, impl=impl)
        assert g.num_kernels == c.num_blocks
        g.launch()
        g.launch()
        g.close()
        assert np.array_equal(direct.get().view(np.float32), replay.get().view(np.float32))
    finally:
        direct.free()
        replay.free()


def test_autotune_fuses_at_the_fastest_candidate(env):
    from quest_gb300.fused import Circuit, StateVector32
    n = 16
    rng = np.random.default_rng(22)
    gates = brickwork(n, 8, rng)
    amps = qc.random_statevector(n, 22)
    c = Circuit(n)
    for t, m in gates:
        c.add(t, m)
    k, impl, ms = c.autotune()
    assert (k, impl) == min(ms, key=ms.get)
    assert set(ms) == {(3, 1), (4, 1), (5, 1), (5, 2)}
    s = StateVector32(n)
    try:
        s.set(amps)
        c.apply(s)                       # automatic: the tuned kernel
        got = s.get().astype(np.complex128)
    finally:
        s.free()
    assert fidelity(got, run_oracle(n, amps, gates)) >= 1 - 1e-6


# 1024 tiles of 128 groups: every CTA runs several tiles, so both operand buffers and
# both accumulator sets are reused (the barrier phases of later tiles)
@pytest.mark.parametrize("targs", [[0, 1, 2, 3, 4], [1, 2, 3, 4, 5], [3, 9, 0, 15, 21], [5, 6, 7, 8, 9],
                                   [17, 18, 19, 20, 21]])
def test_single_block_many_tiles_per_cta(env, targs):
    n = 22
    rng = np.random.default_rng(7 + sum(targs))
    u = qc.haar_unitary(32, rng)
    amps = qc.random_statevector(n, 11)
    ref = run_oracle(n, amps, [(targs, u)])
    tc, _ = run_fused(env, n, amps, [(targs, u)], 5, 2)
    assert np.max(np.abs(tc - ref)) <= 2e-6 * np.max(np.abs(ref))
    from quest_gb300 import _lib
    flag = ctypes.c_int(0)
    _lib.lib().qg_tc_get_error_flag(ctypes.byref(flag))
    assert flag.value == 0


@pytest.mark.parametrize("targs", [[0, 1, 2, 3, 4], [1, 2, 3, 4, 5], [5, 6, 7, 8, 9]])
def test_tensor_core_wait_runs_out_cleanly(env, targs):
    # A launch in which no operand buffer is ever signalled full: the kernel's bounded
    # waits run out, it stores nothing, raises the error flag and returns.  The context
    # stays usable: a normal block right after matches the oracle.
    from quest_gb300 import _lib
    lib = _lib.lib()
    t = (ctypes.c_int * 5)(*targs)
    flag, secs, same = ctypes.c_int(0), ctypes.c_double(0), ctypes.c_int(0)
    _lib.check(lib.qg_tc_selftest_timeout(14, t, ctypes.byref(flag), ctypes.byref(secs), ctypes.byref(same)))
    assert flag.value == 1
    assert same.value == 1
    assert 1.0 < secs.value < 30.0
    cleared = ctypes.c_int(1)
    lib.qg_tc_get_error_flag(ctypes.byref(cleared))
    assert cleared.value == 0
    n = 14
    u = qc.haar_unitary(32, np.random.default_rng(5))
    amps = qc.random_statevector(n, 6)
    ref = run_oracle(n, amps, [(targs, u)])
    tc, _ = run_fused(env, n, amps, [(targs, u)], 5, 2)
    assert np.max(np.abs(tc - ref)) <= 2e-6 * np.max(np.abs(ref))
    lib.qg_tc_get_error_flag(ctypes.byref(cleared))
    assert cleared.value == 0


def test_timed_out_launch_is_reported_by_the_next_apply(env):
    # Kernel choice 3 makes every 5-qubit tensor-core launch give up its bounded waits
    # (about 2 s) and leave the register untouched.  The apply itself returns at once
    # (asynchronous); the device's flag is set once the launch ends, and the next apply
    # reports the timeout with QG_ERR_TIMEOUT and clears the flag before launching
    # anything.  The apply after that runs normally and matches the oracle.
    from quest_gb300 import _lib
    from quest_gb300.fused import Circuit, StateVector32
    lib = _lib.lib()
    n = 13
    u = qc.haar_unitary(32, np.random.default_rng(8))
    amps = qc.random_statevector(n, 9)
    c = Circuit(n)
    c.add([1, 3, 5, 7, 9], u)
    c.fuse(5)
    s = StateVector32(n)
    try:
        s.set(amps)
        _lib.check(lib.qg_sv32_apply_circuit(c.h, s.ptr, n, 3, None))
        _lib.check(lib.qg_sync())
        flag = ctypes.c_int(0)
        _lib.check(lib.qg_tc_get_error_flag(ctypes.byref(flag)))
        assert flag.value == 1
        assert np.array_equal(s.get(), amps.astype(np.complex64))       # nothing was stored
        assert lib.qg_sv32_apply_circuit(c.h, s.ptr, n, 2, None) == -4     # QG_ERR_TIMEOUT
        _lib.check(lib.qg_tc_get_error_flag(ctypes.byref(flag)))
        assert flag.value == 0
        _lib.check(lib.qg_sv32_apply_circuit(c.h, s.ptr, n, 2, None))
        got = s.get().astype(np.complex128)
    finally:
        s.free()
    ref = run_oracle(n, amps, [([1, 3, 5, 7, 9], u)])
    assert np.max(np.abs(got - ref)) <= 2e-6 * np.max(np.abs(ref))


def test_server_fails_only_the_request_that_timed_out(env):
    # A server whose large registers run with kernel choice 3: each large request's
    # tensor-core launch gives up and that request alone is failed with QG_ERR_TIMEOUT;
    # small requests (shared memory, no tensor cores) in the same server finish normally,
    # and the device's own flag is left clear.
    from quest_gb300 import _lib, serve
    lib = _lib.lib()
    rng = np.random.default_rng(12)
    from quest_gb300.fused import Circuit
    # 15 qubits: above the shared-memory path (at most 14), so the request runs as
    # whole-state passes with one tensor-core block
    big = Circuit(15).add([0, 2, 4, 6, 8], qc.haar_unitary(32, rng)).fuse(5)
    small = serve.circuit_of(8, serve.hea_request(8, 6, rng)[0])
    codes = [[1] * 15, [3] * 15]
    srv = serve.Server(1 << 28, 8, impl=3)
    try:
        rid_big = srv.submit(big, codes)
        rid_small = srv.submit(small, [[3] * 8])
        import time
        t0 = time.time()
        states = {}
        while len(states) < 2 and time.time() - t0 < 60:
            srv.poll()
            for rid in (rid_big, rid_small):
                if rid in states:
                    continue
                vals = (ctypes.c_double * 2)()
                done = ctypes.c_int(0)
                rc = lib.qg_server_result(srv.h, rid, vals, ctypes.byref(done))
                if done.value:
                    states[rid] = rc
        assert states.get(rid_big) == -4
        assert states.get(rid_small) == 0
        srv.release(rid_big)
        srv.release(rid_small)
    finally:
        srv.close()
    flag = ctypes.c_int(1)
    _lib.check(lib.qg_tc_get_error_flag(ctypes.byref(flag)))
    assert flag.value == 0
