"""General complex one- and two-target gates on FP64 states in both product modes
(qg_set_fp64_products): block-floating fixed point on the integer pipes (the
default) and IEEE FP64.  Both must meet the FP64 bar against the oracle (max-abs
<= 1e-12); the fixed-point path must hand pairs with Inf/NaN or results outside the
normal range to FP64, giving the FP64 kernel's bits there."""
import ctypes

import numpy as np
import pytest

import qcircuits as qc

pytestmark = pytest.mark.gpu
TOL = 1e-12


def _set_mode(mode):
    from quest_gb300._lib import lib
    assert lib().qg_set_fp64_products(mode) == 0


def _haar_circuit(nq, layers, seed):
    rng = np.random.default_rng(seed)
    lines = []
    for _ in range(layers):
        for t in range(nq):
            lines.append(f"U1 {t} {qc.mat_tokens(qc.haar_unitary(2, rng))}")
        c1, c2, t = (int(v) for v in rng.choice(nq, 3, replace=False))
        lines.append(f"CU1 2 {c1} {c2} 1 0 {t} {qc.mat_tokens(qc.haar_unitary(2, rng))}")
        a, b = (int(v) for v in rng.choice(nq, 2, replace=False))
        lines.append(f"U2 {a} {b} {qc.mat_tokens(qc.haar_unitary(4, rng))}")
        lines.append(f"CU2 1 {c1} 1 {t} {c2} {qc.mat_tokens(qc.haar_unitary(4, rng))}")
        for k in (3, 4):
            if nq >= k:
                tk = [int(v) for v in rng.choice(nq, k, replace=False)]
                lines.append(f"UK {k} {' '.join(map(str, tk))} {qc.mat_tokens(qc.haar_unitary(1 << k, rng))}")
    lines.append("TOTALPROB")
    return "\n".join(lines) + "\n"


def _run(env, text, nq, amps):
    from quest_gb300.circuit import run_text
    q = env.Q.createQureg(nq)
    try:
        env.set_amps(q, amps)
        res, _ = run_text(text, q)
        return env.get_amps(q), res
    finally:
        env.Q.destroyQureg(q)


@pytest.mark.parametrize("nq,layers,seed", [(5, 6, 1), (12, 4, 2), (20, 3, 3)])
def test_both_modes_meet_the_fp64_bar(env, nq, layers, seed):
    text = _haar_circuit(nq, layers, seed)
    amps = qc.random_statevector(nq, seed)
    want, wres, _ = qc.oracle().run(text, nq, 0, amps)
    try:
        got = {}
        for mode in (0, 1):
            _set_mode(mode)
            got[mode] = _run(env, text, nq, amps)
            assert np.max(np.abs(got[mode][0] - want)) <= TOL, mode
            assert np.max(np.abs(got[mode][1] - wres)) <= TOL, mode
        # the two modes agree far inside the bar
        assert np.max(np.abs(got[0][0] - got[1][0])) <= 1e-14
    finally:
        _set_mode(0)


@pytest.mark.parametrize("nq", [3, 5])
def test_density_matrix_channels_in_both_modes(env, nq):
    """Kraus maps (superoperators on 2 and 4 Choi targets), depolarising and unitaries
    on density matrices meet the FP64 bar in both product modes."""
    text = qc.config3_circuit(nq, 4, 90 + nq)
    amps = qc.random_density_matrix(nq, 90 + nq)
    want, wres, _ = qc.oracle().run(text, nq, 1, amps)
    from quest_gb300.circuit import run_text
    try:
        for mode in (0, 1):
            _set_mode(mode)
            q = env.Q.createDensityQureg(nq)
            try:
                env.set_amps(q, amps)
                res, _ = run_text(text, q)
                got = env.get_amps(q)
            finally:
                env.Q.destroyQureg(q)
            assert np.max(np.abs(got - want)) <= TOL, mode
            assert np.max(np.abs(res - wres)) <= TOL, mode
    finally:
        _set_mode(0)


def test_special_values_go_to_fp64(env):
    """Pairs holding Inf/NaN, denormal-range results and magnitudes from 1e-300 to 1e300."""
    nq = 8
    rng = np.random.default_rng(5)
    amps = qc.random_statevector(nq, 5) * 10.0 ** rng.integers(-300, 300, 1 << nq)
    amps[3] = complex(np.inf, 0)
    amps[8] = complex(np.nan, 1.0)
    amps[16] = complex(3e-312, 0)
    amps[17] = complex(1e-310, -2e-311)
    u = qc.haar_unitary(2, rng)
    text = f"U1 0 {qc.mat_tokens(u)}\n"          # pairs (2k, 2k+1)
    try:
        _set_mode(1)
        ref, _ = _run(env, text, nq, amps)
        _set_mode(0)
        got, _ = _run(env, text, nq, amps)
    finally:
        _set_mode(0)
    r = ref.view(np.float64).reshape(-1, 4)        # one row per pair: o0.re, o0.im, o1.re, o1.im
    g = got.view(np.float64).reshape(-1, 4)
    a = amps.view(np.float64).reshape(-1, 4)
    special = (~np.isfinite(r) | ((r != 0) & (np.abs(r) < 2.2250738585072014e-308))).any(axis=1)
    assert special[[1, 4, 8]].all()               # the Inf, NaN and denormal pairs
    same = ((r == g) | (np.isnan(r) & np.isnan(g))).all(axis=1)
    assert same[special].all(), "pairs sent to FP64 differ from the FP64 kernel"
    # elsewhere: both results lie within 2 x 2^-52 of the pair's largest input of the
    # exact value (the matrix is unitary), so within 2^-50 of each other
    bound = 2.0 ** -50 * np.max(np.abs(a), axis=1, keepdims=True)
    keep = ~special
    assert np.all(np.abs(g[keep] - r[keep]) <= bound[keep])


def test_every_launch_shape_gives_the_same_bits(env):
    """The autotuner's candidate shapes only change the schedule, never the result."""
    import ctypes
    from quest_gb300._lib import lib
    L = lib()
    nq = 16
    text = _haar_circuit(nq, 2, 9)
    amps = qc.random_statevector(nq, 9)
    want, _, _ = qc.oracle().run(text, nq, 0, amps)
    outs = []
    text += "".join(f"CPS {c} {t} {0.1 + 0.3 * c}\n" for c, t in [(0, 5), (3, 9), (12, 2)])
    rng = np.random.default_rng(19)
    text += "".join(f"U2 {a} {b} {qc.mat_tokens(qc.haar_unitary(4, rng))}\n" for a, b in [(0, 1), (15, 2), (4, 12), (9, 8)])
    want, _, _ = qc.oracle().run(text, nq, 0, amps)
    try:
        for ppt, thr in [(1, 256), (1, 128), (2, 256), (2, 128)]:
            for kern in (0, 1, 2):
                assert L.qg_set_kernel_shape(kern, ppt, thr) == 0
            out, _ = _run(env, text, nq, amps)
            assert np.max(np.abs(out - want)) <= TOL
            outs.append(out)
    finally:
        for kern in (0, 1, 2):
            L.qg_set_kernel_shape(kern, 1, 256)
    for o in outs[1:]:
        assert np.array_equal(o.view(np.float64), outs[0].view(np.float64))


def test_autotune_picks_the_fastest_candidate(env):
    import ctypes
    from quest_gb300._lib import lib
    L = lib()
    ms = (ctypes.c_double * 12)()
    n = ctypes.c_int()
    try:
        assert L.qg_autotune_fp64(22, ms, 12, ctypes.byref(n)) == 0
        assert n.value == 12 and all(ms[i] > 0 for i in range(12))
        cands = [(1, 256), (1, 128), (2, 256), (2, 128)]
        for kernel in (0, 1, 2):
            ppt, thr = ctypes.c_int(), ctypes.c_int()
            assert L.qg_get_kernel_shape(kernel, ctypes.byref(ppt), ctypes.byref(thr)) == 0
            best = min(range(4), key=lambda i: ms[4 * kernel + i])
            assert (ppt.value, thr.value) == cands[best]
    finally:
        for kernel in (0, 1, 2):
            L.qg_set_kernel_shape(kernel, 1, 256)
