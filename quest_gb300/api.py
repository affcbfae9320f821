"""Python binding of the QuEST-named API (include/quest_gb300_api.h).

Mirrors QuEST v4's C API for the gate path: the same function names and
argument order.  Validation errors raised by the library's input-error handler
become ``QuESTError`` exceptions here, the way QuEST's own test-suite turns
them into C++ exceptions (tests/main.cpp:63-66 in the QuEST sources).
"""
import ctypes

import numpy as np

from . import _lib
from ._lib import qg_cplx

qindex = ctypes.c_longlong


class QuESTError(RuntimeError):
    pass


class Qureg(ctypes.Structure):
    _fields_ = [("isMultithreaded", ctypes.c_int), ("isGpuAccelerated", ctypes.c_int), ("isDistributed", ctypes.c_int),
                ("rank", ctypes.c_int), ("numNodes", ctypes.c_int), ("logNumNodes", ctypes.c_int),
                ("isDensityMatrix", ctypes.c_int), ("numQubits", ctypes.c_int),
                ("numAmps", qindex), ("logNumAmps", qindex), ("numAmpsPerNode", qindex),
                ("logNumAmpsPerNode", qindex), ("logNumColsPerNode", qindex),
                ("cpuAmps", ctypes.POINTER(qg_cplx)), ("gpuAmps", ctypes.POINTER(qg_cplx)),
                ("cpuCommBuffer", ctypes.POINTER(qg_cplx)), ("gpuCommBuffer", ctypes.POINTER(qg_cplx))]


class CompMatr1(ctypes.Structure):
    _fields_ = [("numQubits", ctypes.c_int), ("numRows", qindex), ("elems", (qg_cplx * 2) * 2)]


class CompMatr2(ctypes.Structure):
    _fields_ = [("numQubits", ctypes.c_int), ("numRows", qindex), ("elems", (qg_cplx * 4) * 4)]


class DiagMatr1(ctypes.Structure):
    _fields_ = [("numQubits", ctypes.c_int), ("numElems", qindex), ("elems", qg_cplx * 2)]


class DiagMatr2(ctypes.Structure):
    _fields_ = [("numQubits", ctypes.c_int), ("numElems", qindex), ("elems", qg_cplx * 4)]


_IP = ctypes.POINTER(ctypes.c_int)
_CP = ctypes.POINTER(qg_cplx)


class CompMatr(ctypes.Structure):
    _fields_ = [("numQubits", ctypes.c_int), ("numRows", qindex), ("isApproxUnitary", _IP), ("isApproxHermitian", _IP),
                ("wasGpuSynced", _IP), ("cpuElems", ctypes.POINTER(_CP)), ("cpuElemsFlat", _CP), ("gpuElemsFlat", _CP)]


class DiagMatr(ctypes.Structure):
    _fields_ = [("numQubits", ctypes.c_int), ("numElems", qindex), ("isApproxUnitary", _IP), ("isApproxHermitian", _IP),
                ("isApproxNonZero", _IP), ("isStrictlyNonNegative", _IP), ("wasGpuSynced", _IP),
                ("cpuElems", _CP), ("gpuElems", _CP)]


class FullStateDiagMatr(ctypes.Structure):
    _fields_ = [("numQubits", ctypes.c_int), ("numElems", qindex), ("isGpuAccelerated", ctypes.c_int),
                ("isMultithreaded", ctypes.c_int), ("isDistributed", ctypes.c_int), ("numElemsPerNode", qindex),
                ("isApproxUnitary", _IP), ("isApproxHermitian", _IP), ("isApproxNonZero", _IP),
                ("isStrictlyNonNegative", _IP), ("wasGpuSynced", _IP), ("cpuElems", _CP), ("gpuElems", _CP)]


class SuperOp(ctypes.Structure):
    _fields_ = [("numQubits", ctypes.c_int), ("numRows", qindex), ("cpuElems", ctypes.POINTER(_CP)),
                ("cpuElemsFlat", _CP), ("gpuElemsFlat", _CP), ("wasGpuSynced", _IP)]


class KrausMap(ctypes.Structure):
    _fields_ = [("numQubits", ctypes.c_int), ("numMatrices", ctypes.c_int), ("numRows", qindex),
                ("matrices", ctypes.POINTER(ctypes.POINTER(_CP))), ("superop", SuperOp), ("isApproxCPTP", _IP)]


class PauliStr(ctypes.Structure):
    _fields_ = [("lowPaulis", ctypes.c_ulonglong), ("highPaulis", ctypes.c_ulonglong)]


class PauliStrSum(ctypes.Structure):
    _fields_ = [("numTerms", qindex), ("strings", ctypes.POINTER(PauliStr)), ("coeffs", _CP), ("isApproxHermitian", _IP)]


_HANDLER_T = ctypes.CFUNCTYPE(None, ctypes.c_char_p, ctypes.c_char_p)
_errors = []


def _on_error(func, msg):
    _errors.append((func.decode(errors="replace"), msg.decode(errors="replace")))


_handler = _HANDLER_T(_on_error)

I, D, V = ctypes.c_int, ctypes.c_double, None
_PROTOS = {
    "initQuESTEnv": (V, []),
    "initCustomQuESTEnv": (V, [I, I, I]),
    "finalizeQuESTEnv": (V, []),
    "isQuESTEnvInit": (I, []),
    "syncQuESTEnv": (V, []),
    "setInputErrorHandler": (V, [_HANDLER_T]),
    "setSeeds": (V, [ctypes.POINTER(ctypes.c_uint), I]),
    "setValidationEpsilon": (V, [D]),
    "setValidationEpsilonToDefault": (V, []),
    "setQuESTStream": (V, [ctypes.c_void_p]),
    "createQureg": (Qureg, [I]),
    "createDensityQureg": (Qureg, [I]),
    "createCustomQureg": (Qureg, [I, I, I, I, I]),
    "createCloneQureg": (Qureg, [Qureg]),
    "destroyQureg": (V, [Qureg]),
    "syncQuregToGpu": (V, [Qureg]),
    "syncQuregFromGpu": (V, [Qureg]),
    "getQuregAmps": (V, [ctypes.c_void_p, Qureg, qindex, qindex]),
    "getQuregAmp": (qg_cplx, [Qureg, qindex]),
    "initZeroState": (V, [Qureg]),
    "initPlusState": (V, [Qureg]),
    "initClassicalState": (V, [Qureg, qindex]),
    "initDebugState": (V, [Qureg]),
    "setQuregAmps": (V, [Qureg, qindex, ctypes.c_void_p, qindex]),
    "setDensityQuregFlatAmps": (V, [Qureg, qindex, ctypes.c_void_p, qindex]),
    "createCompMatr": (CompMatr, [I]),
    "destroyCompMatr": (V, [CompMatr]),
    "setCompMatrFlat": (V, [CompMatr, ctypes.c_void_p]),
    "createDiagMatr": (DiagMatr, [I]),
    "destroyDiagMatr": (V, [DiagMatr]),
    "setDiagMatrFlat": (V, [DiagMatr, ctypes.c_void_p]),
    "createKrausMap": (KrausMap, [I, I]),
    "setKrausMapFlat": (V, [KrausMap, ctypes.c_void_p]),
    "destroyKrausMap": (V, [KrausMap]),
    "getPauliStrFromCodes": (PauliStr, [_IP, _IP, I]),
    "applyCompMatr1": (V, [Qureg, I, CompMatr1]),
    "applyControlledCompMatr1": (V, [Qureg, I, I, CompMatr1]),
    "applyMultiStateControlledCompMatr1": (V, [Qureg, _IP, _IP, I, I, CompMatr1]),
    "applyCompMatr2": (V, [Qureg, I, I, CompMatr2]),
    "applyMultiStateControlledCompMatr2": (V, [Qureg, _IP, _IP, I, I, I, CompMatr2]),
    "applyCompMatr": (V, [Qureg, _IP, I, CompMatr]),
    "applyMultiStateControlledCompMatr": (V, [Qureg, _IP, _IP, I, _IP, I, CompMatr]),
    "applyDiagMatr1": (V, [Qureg, I, DiagMatr1]),
    "applyMultiStateControlledDiagMatr1": (V, [Qureg, _IP, _IP, I, I, DiagMatr1]),
    "applyDiagMatr2": (V, [Qureg, I, I, DiagMatr2]),
    "applyDiagMatr": (V, [Qureg, _IP, I, DiagMatr]),
    "applyMultiStateControlledDiagMatr": (V, [Qureg, _IP, _IP, I, _IP, I, DiagMatr]),
    "applyDiagMatrPower": (V, [Qureg, _IP, I, DiagMatr, qg_cplx]),
    "applyS": (V, [Qureg, I]),
    "applyT": (V, [Qureg, I]),
    "applyHadamard": (V, [Qureg, I]),
    "applySwap": (V, [Qureg, I, I]),
    "applyMultiStateControlledSwap": (V, [Qureg, _IP, _IP, I, I, I]),
    "applyPauliX": (V, [Qureg, I]),
    "applyPauliY": (V, [Qureg, I]),
    "applyPauliZ": (V, [Qureg, I]),
    "applyControlledPauliX": (V, [Qureg, I, I]),
    "applyControlledPauliZ": (V, [Qureg, I, I]),
    "applyPauliStr": (V, [Qureg, PauliStr]),
    "applyMultiStateControlledPauliStr": (V, [Qureg, _IP, _IP, I, PauliStr]),
    "applyRotateX": (V, [Qureg, I, D]),
    "applyRotateY": (V, [Qureg, I, D]),
    "applyRotateZ": (V, [Qureg, I, D]),
    "applyControlledRotateX": (V, [Qureg, I, I, D]),
    "applyControlledRotateY": (V, [Qureg, I, I, D]),
    "applyControlledRotateZ": (V, [Qureg, I, I, D]),
    "applyPauliGadget": (V, [Qureg, PauliStr, D]),
    "applyMultiStateControlledPauliGadget": (V, [Qureg, _IP, _IP, I, PauliStr, D]),
    "applyPhaseGadget": (V, [Qureg, _IP, I, D]),
    "applyPhaseShift": (V, [Qureg, I, D]),
    "applyTwoQubitPhaseShift": (V, [Qureg, I, I, D]),
    "applyMultiQubitPhaseShift": (V, [Qureg, _IP, I, D]),
    "applyPhaseFlip": (V, [Qureg, I]),
    "applyTwoQubitPhaseFlip": (V, [Qureg, I, I]),
    "applyQuantumFourierTransform": (V, [Qureg, _IP, I]),
    "applyFullQuantumFourierTransform": (V, [Qureg]),
    "applyQubitProjector": (V, [Qureg, I, I]),
    "applyMultiQubitProjector": (V, [Qureg, _IP, _IP, I]),
    "applyQubitMeasurement": (I, [Qureg, I]),
    "applyQubitMeasurementAndGetProb": (I, [Qureg, I, ctypes.POINTER(D)]),
    "applyForcedQubitMeasurement": (D, [Qureg, I, I]),
    "applyMultiQubitMeasurement": (qindex, [Qureg, _IP, I]),
    "applyMultiQubitMeasurementAndGetProb": (qindex, [Qureg, _IP, I, ctypes.POINTER(D)]),
    "applyForcedMultiQubitMeasurement": (D, [Qureg, _IP, _IP, I]),
    "mixDephasing": (V, [Qureg, I, D]),
    "mixTwoQubitDephasing": (V, [Qureg, I, I, D]),
    "mixDepolarising": (V, [Qureg, I, D]),
    "mixTwoQubitDepolarising": (V, [Qureg, I, I, D]),
    "mixDamping": (V, [Qureg, I, D]),
    "mixPaulis": (V, [Qureg, I, D, D, D]),
    "mixKrausMap": (V, [Qureg, _IP, I, KrausMap]),
    "calcExpecPauliStr": (D, [Qureg, PauliStr]),
    "calcExpecPauliStrs": (V, [ctypes.POINTER(D), Qureg, ctypes.POINTER(PauliStr), I]),
    "createPauliStrSum": (PauliStrSum, [ctypes.POINTER(PauliStr), _CP, qindex]),
    "destroyPauliStrSum": (V, [PauliStrSum]),
    "calcExpecPauliStrSum": (D, [Qureg, PauliStrSum]),
    "calcProbOfQubitOutcome": (D, [Qureg, I, I]),
    "calcProbOfMultiQubitOutcome": (D, [Qureg, _IP, _IP, I]),
    "calcProbsOfAllMultiQubitOutcomes": (V, [ctypes.POINTER(D), Qureg, _IP, I]),
    "calcTotalProb": (D, [Qureg]),
    "isQuregHostMirrorPinned": (I, [Qureg]),
    "flushQuregDeferredOps": (V, [Qureg]),
    "calcPurity": (D, [Qureg]),
    "createFullStateDiagMatr": (FullStateDiagMatr, [I]),
    "destroyFullStateDiagMatr": (V, [FullStateDiagMatr]),
    "setFullStateDiagMatr": (V, [FullStateDiagMatr, qindex, ctypes.c_void_p, qindex]),
    "syncFullStateDiagMatr": (V, [FullStateDiagMatr]),
    "multiplyFullStateDiagMatr": (V, [Qureg, FullStateDiagMatr]),
    "multiplyFullStateDiagMatrPower": (V, [Qureg, FullStateDiagMatr, qg_cplx]),
    "applyFullStateDiagMatr": (V, [Qureg, FullStateDiagMatr]),
    "applyFullStateDiagMatrPower": (V, [Qureg, FullStateDiagMatr, qg_cplx]),
    "calcExpecFullStateDiagMatr": (D, [Qureg, FullStateDiagMatr]),
    "calcExpecFullStateDiagMatrPower": (D, [Qureg, FullStateDiagMatr, D]),
    "calcExpecNonHermitianFullStateDiagMatr": (qg_cplx, [Qureg, FullStateDiagMatr]),
    "calcExpecNonHermitianFullStateDiagMatrPower": (qg_cplx, [Qureg, FullStateDiagMatr, qg_cplx]),
}


class _API:
    """Attribute access to every API function, raising QuESTError on validation failure."""

    def __init__(self):
        self._fns = {}

    def _get(self, name):
        if name not in self._fns:
            L = _lib.lib()
            f = getattr(L, name)
            res, args = _PROTOS[name]
            f.restype = res
            f.argtypes = args
            self._fns[name] = f
        return self._fns[name]

    def __getattr__(self, name):
        if name.startswith("_") or name not in _PROTOS:
            raise AttributeError(name)
        f = self._get(name)

        def call(*args):
            del _errors[:]
            out = f(*args)
            if _errors:
                func, msg = _errors[0]
                del _errors[:]
                raise QuESTError(f"{func}: {msg}")
            return out
        call.__name__ = name
        return call


Q = _API()
_env_ready = False


def init_env():
    """initQuESTEnv with the raising error handler installed (idempotent)."""
    global _env_ready
    if not _env_ready:
        Q._get("setInputErrorHandler")(_handler)
        if not Q._get("isQuESTEnvInit")():
            Q.initQuESTEnv()
        _env_ready = True


# ---------------------------------------------------------------- helpers

def ints(seq):
    return _lib.ints(seq)


def comp_matr1(m):
    m = np.asarray(m, dtype=np.complex128).reshape(2, 2)
    out = CompMatr1(numQubits=1, numRows=2)
    for r in range(2):
        for c in range(2):
            out.elems[r][c].re, out.elems[r][c].im = m[r, c].real, m[r, c].imag
    return out


def comp_matr2(m):
    m = np.asarray(m, dtype=np.complex128).reshape(4, 4)
    out = CompMatr2(numQubits=2, numRows=4)
    for r in range(4):
        for c in range(4):
            out.elems[r][c].re, out.elems[r][c].im = m[r, c].real, m[r, c].imag
    return out


def diag_matr1(d):
    d = np.asarray(d, dtype=np.complex128).reshape(2)
    out = DiagMatr1(numQubits=1, numElems=2)
    for i in range(2):
        out.elems[i].re, out.elems[i].im = d[i].real, d[i].imag
    return out


def diag_matr2(d):
    d = np.asarray(d, dtype=np.complex128).reshape(4)
    out = DiagMatr2(numQubits=2, numElems=4)
    for i in range(4):
        out.elems[i].re, out.elems[i].im = d[i].real, d[i].imag
    return out


def comp_matr(m):
    """A heap CompMatr holding m (caller destroys it with Q.destroyCompMatr)."""
    m = np.ascontiguousarray(np.asarray(m, dtype=np.complex128))
    k = int(np.log2(m.shape[0]))
    out = Q.createCompMatr(k)
    Q.setCompMatrFlat(out, m.ctypes.data)
    return out


def diag_matr(d):
    d = np.ascontiguousarray(np.asarray(d, dtype=np.complex128).reshape(-1))
    k = int(np.log2(d.shape[0]))
    out = Q.createDiagMatr(k)
    Q.setDiagMatrFlat(out, d.ctypes.data)
    return out


def kraus_map(ops):
    ops = np.ascontiguousarray(np.asarray(ops, dtype=np.complex128))
    n, dim, _ = ops.shape
    k = int(np.log2(dim))
    out = Q.createKrausMap(k, n)
    Q.setKrausMapFlat(out, ops.ctypes.data)
    return out


def pauli_str(codes):
    """PauliStr from per-qubit codes (0=I, 1=X, 2=Y, 3=Z; index = qubit) or a string 'IXYZ...'."""
    if isinstance(codes, str):
        codes = ["IXYZ".index(ch) for ch in codes]
    idx = [q for q, c in enumerate(codes) if c]
    vals = [codes[q] for q in idx]
    if not idx:
        return PauliStr(0, 0)
    return Q.getPauliStrFromCodes(ints(vals), ints(idx), len(idx))


def set_amps(qureg, amps):
    a = np.ascontiguousarray(np.asarray(amps, dtype=np.complex128).reshape(-1))
    if a.size != qureg.numAmps:
        raise ValueError("amplitude count mismatch")
    Q.setQuregAmps(qureg, 0, a.ctypes.data, a.size)


def get_amps(qureg):
    out = np.empty(qureg.numAmps, dtype=np.complex128)
    Q.getQuregAmps(out.ctypes.data, qureg, 0, qureg.numAmps)
    return out


def seeds(*values):
    arr = (ctypes.c_uint * len(values))(*values)
    Q.setSeeds(arr, len(values))


def full_state_diag(elems):
    """A FullStateDiagMatr holding `elems` (2^n complex); destroy it with Q.destroyFullStateDiagMatr."""
    e = np.ascontiguousarray(np.asarray(elems, dtype=np.complex128).reshape(-1))
    n = int(e.size).bit_length() - 1
    if e.size != 1 << n:
        raise ValueError("a FullStateDiagMatr holds 2^n elements")
    m = Q.createFullStateDiagMatr(n)
    Q.setFullStateDiagMatr(m, 0, e.ctypes.data, e.size)
    return m


def pauli_str_sum(coeffs, strings):
    """createPauliStrSum from complex coefficients and Pauli strings ('IXYZ...' text or codes)."""
    n = len(strings)
    strs = (PauliStr * n)(*[pauli_str(x) for x in strings])
    cs = (qg_cplx * n)(*[qg_cplx(complex(c).real, complex(c).imag) for c in coeffs])
    return Q.createPauliStrSum(strs, cs, n)
