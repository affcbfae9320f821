"""The allocation-free batched Pauli expectation entry point
(qg_sv_calcExpecPauliStrBatch_noalloc), called through the C ABI.

It exists for callers that cannot allocate during a call -- their device
memory is reserved up front by another allocator, or they cannot take
cudaMalloc's implicit synchronisation -- so it keeps its partial sums in a fixed
device array inside the library.  Its results must match the regular entry
point's within the FP64 tolerance of the other parity tests, on two calls in a
row (the shared array keeps the previous call's contents).  This file is
collected last so that a run stopping at the first failure has run every other
test already; it also passes alone in a fresh process."""
import ctypes

import numpy as np
import pytest

import qcircuits as qc

pytestmark = pytest.mark.gpu
TOL = 1e-12


def _strings(n, count, seed):
    rng = np.random.default_rng(seed)
    mxy = (ctypes.c_int64 * count)()
    myz = (ctypes.c_int64 * count)()
    ny = (ctypes.c_int * count)()
    for s in range(count):
        codes = [int(v) for v in rng.integers(0, 4, n)]
        mxy[s] = sum(1 << q for q, c in enumerate(codes) if c in (1, 2))
        myz[s] = sum(1 << q for q, c in enumerate(codes) if c in (2, 3))
        ny[s] = sum(1 for c in codes if c == 2)
    return mxy, myz, ny


def test_noalloc_matches_regular_entry_point_twice(env):
    from quest_gb300 import _lib
    L = _lib.lib()
    Q = env.Q
    n = 18
    q = Q.createQureg(n)
    try:
        for call, seed in enumerate((5, 6)):
            env.set_amps(q, qc.random_statevector(n, seed))
            count = 40   # three launches of up to 16 strings
            mxy, myz, ny = _strings(n, count, seed)
            want = (_lib.qg_cplx * count)()
            got = (_lib.qg_cplx * count)()
            _lib.check(L.qg_sv_calcExpecPauliStrBatch(q.gpuAmps, n, mxy, myz, ny, count, want, None))
            _lib.check(L.qg_sv_calcExpecPauliStrBatch_noalloc(q.gpuAmps, n, mxy, myz, ny, count, got, None))
            w = np.array([[x.re, x.im] for x in want])
            g = np.array([[x.re, x.im] for x in got])
            assert np.max(np.abs(w - g)) <= TOL, f"call {call}"
            assert np.max(np.abs(g[:, 0])) > 0
    finally:
        Q.destroyQureg(q)


def test_noalloc_rejects_too_many_strings(env):
    from quest_gb300 import _lib
    L = _lib.lib()
    Q = env.Q
    q = Q.createQureg(6)
    try:
        count = 65
        mxy, myz, ny = _strings(6, count, 1)
        out = (_lib.qg_cplx * count)()
        rc = L.qg_sv_calcExpecPauliStrBatch_noalloc(q.gpuAmps, 6, mxy, myz, ny, count, out, None)
        assert rc == -2
        assert b"at most 64" in L.qg_get_last_error()
    finally:
        Q.destroyQureg(q)
