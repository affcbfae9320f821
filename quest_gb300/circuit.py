"""Runs circuit text (one QuEST API call per line) through the GB300 API.

The text format is shared with the CPU oracle's runner and the reference
harness used to make the golden fixtures (``H 3``, ``U1 t m00r m00i ...``,
``DEPOL q p``, ``EXPEC XIZY``, ``MEAS q`` ...); each op calls the QuEST-named
function of the same meaning.
"""
import ctypes

import numpy as np

from ._lib import qg_cplx
from .api import (Q, comp_matr, comp_matr1, comp_matr2, diag_matr, diag_matr1, diag_matr2, full_state_diag, ints,
                  kraus_map, pauli_str, pauli_str_sum, seeds)


def _f(tokens, k):
    return [float(t) for t in tokens[:k]], tokens[k:]


def _cvals(vals):
    v = np.asarray(vals, dtype=np.float64)
    return v[0::2] + 1j * v[1::2]


def run_text(text, qureg):
    """Applies every op of `text` to `qureg`; returns (results, outcomes)."""
    results, outcomes = [], []
    for raw in text.splitlines():
        tok = raw.split()
        if not tok or tok[0].startswith("#"):
            continue
        op, a = tok[0], tok[1:]
        if op in ("H", "X", "Y", "Z", "S", "T"):
            fn = {"H": Q.applyHadamard, "X": Q.applyPauliX, "Y": Q.applyPauliY, "Z": Q.applyPauliZ,
                  "S": Q.applyS, "T": Q.applyT}[op]
            fn(qureg, int(a[0]))
        elif op in ("RX", "RY", "RZ"):
            getattr(Q, "applyRotate" + op[1])(qureg, int(a[0]), float(a[1]))
        elif op in ("CRX", "CRY", "CRZ"):
            getattr(Q, "applyControlledRotate" + op[2])(qureg, int(a[0]), int(a[1]), float(a[2]))
        elif op == "PS":
            Q.applyPhaseShift(qureg, int(a[0]), float(a[1]))
        elif op == "CPS":
            Q.applyTwoQubitPhaseShift(qureg, int(a[0]), int(a[1]), float(a[2]))
        elif op == "MPS":
            k = int(a[0])
            Q.applyMultiQubitPhaseShift(qureg, ints(a[1:1 + k]), k, float(a[1 + k]))
        elif op == "CX":
            Q.applyControlledPauliX(qureg, int(a[0]), int(a[1]))
        elif op == "CZ":
            Q.applyControlledPauliZ(qureg, int(a[0]), int(a[1]))
        elif op == "SWAP":
            Q.applySwap(qureg, int(a[0]), int(a[1]))
        elif op == "CSWAP":
            nc = int(a[0]); c = a[1:1 + nc]; s = a[1 + nc:1 + 2 * nc]; r = a[1 + 2 * nc:]
            Q.applyMultiStateControlledSwap(qureg, ints(c), ints(s), nc, int(r[0]), int(r[1]))
        elif op == "U1":
            Q.applyCompMatr1(qureg, int(a[0]), comp_matr1(_cvals(a[1:9])))
        elif op == "CU1":
            nc = int(a[0]); c = a[1:1 + nc]; s = a[1 + nc:1 + 2 * nc]; r = a[1 + 2 * nc:]
            Q.applyMultiStateControlledCompMatr1(qureg, ints(c), ints(s), nc, int(r[0]), comp_matr1(_cvals(r[1:9])))
        elif op == "U2":
            Q.applyCompMatr2(qureg, int(a[0]), int(a[1]), comp_matr2(_cvals(a[2:34])))
        elif op == "CU2":
            nc = int(a[0]); c = a[1:1 + nc]; s = a[1 + nc:1 + 2 * nc]; r = a[1 + 2 * nc:]
            Q.applyMultiStateControlledCompMatr2(qureg, ints(c), ints(s), nc, int(r[0]), int(r[1]), comp_matr2(_cvals(r[2:34])))
        elif op in ("UK", "CUK"):
            if op == "CUK":
                nc = int(a[0]); c = a[1:1 + nc]; s = a[1 + nc:1 + 2 * nc]; a = a[1 + 2 * nc:]
            k = int(a[0]); t = a[1:1 + k]
            m = comp_matr(_cvals(a[1 + k:1 + k + (2 << (2 * k))]).reshape(1 << k, 1 << k))
            try:
                if op == "UK":
                    Q.applyCompMatr(qureg, ints(t), k, m)
                else:
                    Q.applyMultiStateControlledCompMatr(qureg, ints(c), ints(s), nc, ints(t), k, m)
            finally:
                Q.destroyCompMatr(m)
        elif op == "D1":
            Q.applyDiagMatr1(qureg, int(a[0]), diag_matr1(_cvals(a[1:5])))
        elif op == "D2":
            Q.applyDiagMatr2(qureg, int(a[0]), int(a[1]), diag_matr2(_cvals(a[2:10])))
        elif op == "FSD":
            mult, has_pow = int(a[0]), int(a[1])
            ex = (float(a[2]), float(a[3])) if has_pow else None
            m = full_state_diag(_cvals(a[4 if has_pow else 2:]))
            try:
                if ex is None:
                    (Q.multiplyFullStateDiagMatr if mult else Q.applyFullStateDiagMatr)(qureg, m)
                else:
                    (Q.multiplyFullStateDiagMatrPower if mult else Q.applyFullStateDiagMatrPower)(qureg, m, qg_cplx(*ex))
            finally:
                Q.destroyFullStateDiagMatr(m)
        elif op == "EXPFSD":
            kind = int(a[0])
            skip = {0: 1, 1: 2, 2: 1, 3: 3}[kind]
            m = full_state_diag(_cvals(a[skip:]))
            try:
                if kind == 0:
                    results.append(Q.calcExpecFullStateDiagMatr(qureg, m))
                elif kind == 1:
                    results.append(Q.calcExpecFullStateDiagMatrPower(qureg, m, float(a[1])))
                else:
                    v = (Q.calcExpecNonHermitianFullStateDiagMatr(qureg, m) if kind == 2 else
                         Q.calcExpecNonHermitianFullStateDiagMatrPower(qureg, m, qg_cplx(float(a[1]), float(a[2]))))
                    results += [v.re, v.im]
            finally:
                Q.destroyFullStateDiagMatr(m)
        elif op in ("DK", "CDK", "DKP"):
            if op == "CDK":
                nc = int(a[0]); c = a[1:1 + nc]; s = a[1 + nc:1 + 2 * nc]; a = a[1 + 2 * nc:]
            k = int(a[0]); t = a[1:1 + k]
            d = diag_matr(_cvals(a[1 + k:1 + k + (2 << k)]))
            try:
                if op == "DK":
                    Q.applyDiagMatr(qureg, ints(t), k, d)
                elif op == "CDK":
                    Q.applyMultiStateControlledDiagMatr(qureg, ints(c), ints(s), nc, ints(t), k, d)
                else:
                    ex = a[1 + k + (2 << k):]
                    Q.applyDiagMatrPower(qureg, ints(t), k, d, qg_cplx(float(ex[0]), float(ex[1])))
            finally:
                Q.destroyDiagMatr(d)
        elif op == "PSTR":
            Q.applyPauliStr(qureg, pauli_str(a[0]))
        elif op == "CPSTR":
            nc = int(a[0]); c = a[1:1 + nc]; s = a[1 + nc:1 + 2 * nc]; r = a[1 + 2 * nc:]
            Q.applyMultiStateControlledPauliStr(qureg, ints(c), ints(s), nc, pauli_str(r[0]))
        elif op == "PG":
            Q.applyPauliGadget(qureg, pauli_str(a[0]), float(a[1]))
        elif op == "CPG":
            nc = int(a[0]); c = a[1:1 + nc]; s = a[1 + nc:1 + 2 * nc]; r = a[1 + 2 * nc:]
            Q.applyMultiStateControlledPauliGadget(qureg, ints(c), ints(s), nc, pauli_str(r[0]), float(r[1]))
        elif op == "PHG":
            k = int(a[0])
            Q.applyPhaseGadget(qureg, ints(a[1:1 + k]), k, float(a[1 + k]))
        elif op == "QFT":
            k = int(a[0])
            Q.applyQuantumFourierTransform(qureg, ints(a[1:1 + k]), k)
        elif op == "FQFT":
            Q.applyFullQuantumFourierTransform(qureg)
        elif op == "DEPOL":
            Q.mixDepolarising(qureg, int(a[0]), float(a[1]))
        elif op == "DEPOL2":
            Q.mixTwoQubitDepolarising(qureg, int(a[0]), int(a[1]), float(a[2]))
        elif op == "DEPHASE":
            Q.mixDephasing(qureg, int(a[0]), float(a[1]))
        elif op == "DEPHASE2":
            Q.mixTwoQubitDephasing(qureg, int(a[0]), int(a[1]), float(a[2]))
        elif op == "DAMP":
            Q.mixDamping(qureg, int(a[0]), float(a[1]))
        elif op == "PAULIS":
            Q.mixPaulis(qureg, int(a[0]), float(a[1]), float(a[2]), float(a[3]))
        elif op == "KRAUS":
            k = int(a[0]); t = a[1:1 + k]; nops = int(a[1 + k])
            vals = _cvals(a[2 + k:2 + k + nops * (2 << (2 * k))]).reshape(nops, 1 << k, 1 << k)
            km = kraus_map(vals)
            try:
                Q.mixKrausMap(qureg, ints(t), k, km)
            finally:
                Q.destroyKrausMap(km)
        elif op == "PROJ":
            k = int(a[0])
            Q.applyMultiQubitProjector(qureg, ints(a[1:1 + k]), ints(a[1 + k:1 + 2 * k]), k)
        elif op == "SEED":
            seeds(*[int(v) for v in a])
        elif op == "MEAS":
            outcomes.append(Q.applyQubitMeasurement(qureg, int(a[0])))
        elif op == "MEASM":
            k = int(a[0])
            p = ctypes.c_double(0)
            outcomes.append(int(Q.applyMultiQubitMeasurementAndGetProb(qureg, ints(a[1:1 + k]), k, ctypes.byref(p))))
            results.append(p.value)
        elif op == "FMEAS":
            results.append(Q.applyForcedQubitMeasurement(qureg, int(a[0]), int(a[1])))
        elif op == "FMEASM":
            k = int(a[0])
            results.append(Q.applyForcedMultiQubitMeasurement(qureg, ints(a[1:1 + k]), ints(a[1 + k:1 + 2 * k]), k))
        elif op == "PROBALL":
            k = int(a[0])
            out = (ctypes.c_double * (1 << k))()
            Q.calcProbsOfAllMultiQubitOutcomes(out, qureg, ints(a[1:1 + k]), k)
            results += list(out)
        elif op == "EXPSUM":
            T = int(a[0])
            cs = [complex(float(a[1 + 3 * t]), float(a[2 + 3 * t])) for t in range(T)]
            ps = [a[3 + 3 * t] for t in range(T)]
            sm = pauli_str_sum(cs, ps)
            try:
                results.append(Q.calcExpecPauliStrSum(qureg, sm))
            finally:
                Q.destroyPauliStrSum(sm)
        elif op == "TOTALPROB":
            results.append(Q.calcTotalProb(qureg))
        elif op == "PURITY":
            results.append(Q.calcPurity(qureg))
        elif op == "PROBQ":
            results.append(Q.calcProbOfQubitOutcome(qureg, int(a[0]), int(a[1])))
        elif op == "PROBMQ":
            k = int(a[0])
            results.append(Q.calcProbOfMultiQubitOutcome(qureg, ints(a[1:1 + k]), ints(a[1 + k:1 + 2 * k]), k))
        elif op == "EXPEC":
            results.append(Q.calcExpecPauliStr(qureg, pauli_str(a[0])))
        else:
            raise ValueError(f"unknown op {op!r}")
    return np.array(results, dtype=np.float64), np.array(outcomes, dtype=np.int32)


def default_seed_text():
    """The runners start from setSeeds({0}); the GPU side does the same before a circuit."""
    return "SEED 0\n"
