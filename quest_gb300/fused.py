"""Python view of the FP32 fused-block path (qg_circuit_* / qg_sv32_* in
include/quest_gb300.h): build a circuit of small unitaries, fuse it into
<=k-qubit blocks, apply it to an FP32 statevector held in device memory."""
import ctypes

import numpy as np

from . import _lib
from ._lib import check, lib, qg_cplx, qg_cplxf

IMPL_AUTO, IMPL_SIMT, IMPL_TC = 0, 1, 2


def _cplx(m):
    m = np.ascontiguousarray(np.asarray(m, dtype=np.complex128).reshape(-1))
    arr = (qg_cplx * m.size)()
    ctypes.memmove(arr, m.ctypes.data, m.nbytes)
    return arr


class Circuit:
    def __init__(self, num_qubits):
        self.num_qubits = num_qubits
        h = ctypes.c_void_p()
        check(lib().qg_circuit_create(ctypes.byref(h), num_qubits))
        self.h = h

    def __del__(self):
        h = getattr(self, "h", None)
        if h is not None and h.value:
            try:
                lib().qg_circuit_destroy(h)
            except Exception:
                pass
            self.h = None

    def add(self, targs, matrix):
        targs = list(targs)
        check(lib().qg_circuit_add_matrix(self.h, _lib.ints(targs), len(targs), _cplx(matrix)))
        return self

    def add_many(self, num_targs, targs, mats):
        """Appends many 1-/2-qubit gates in one call: num_targs (G,), targs (G, 2),
        mats (G, 16) complex with each gate's row-major matrix in its first 4^k entries."""
        num_targs = np.ascontiguousarray(num_targs, dtype=np.int32)
        targs = np.ascontiguousarray(targs, dtype=np.int32)
        mats = np.ascontiguousarray(mats, dtype=np.complex128)
        check(lib().qg_circuit_add_matrices(self.h, len(num_targs), num_targs.ctypes.data_as(_lib.c_int_p),
                                            targs.ctypes.data_as(_lib.c_int_p), mats.ctypes.data_as(_lib.c_cplx_p)))
        return self

    def fuse(self, k=5):
        check(lib().qg_circuit_fuse(self.h, k))
        return self

    @property
    def num_gates(self):
        n = ctypes.c_int()
        check(lib().qg_circuit_get_num_gates(self.h, ctypes.byref(n)))
        return n.value

    @property
    def num_blocks(self):
        n = ctypes.c_int()
        check(lib().qg_circuit_get_num_blocks(self.h, ctypes.byref(n)))
        return n.value

    def block(self, i):
        targs = (ctypes.c_int * 8)()
        k = ctypes.c_int()
        m = (qg_cplx * 1024)()
        check(lib().qg_circuit_get_block(self.h, i, targs, ctypes.byref(k), m))
        d = 1 << k.value
        arr = np.frombuffer(m, dtype=np.complex128, count=d * d).reshape(d, d).copy()
        return [targs[j] for j in range(k.value)], arr

    def apply(self, state, impl=IMPL_AUTO, stream=None):
        check(lib().qg_sv32_apply_circuit(self.h, state.ptr, state.num_qubits, impl, stream))

    def autotune(self):
        """Fuses at the fastest width with the fastest kernel (timed on this GPU);
        returns (k, impl, {(k, impl): ms per circuit})."""
        k, impl, n = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        ck, ci, ms = (ctypes.c_int * 8)(), (ctypes.c_int * 8)(), (ctypes.c_double * 8)()
        check(lib().qg_circuit_autotune(self.h, ctypes.byref(k), ctypes.byref(impl), ck, ci, ms, 8, ctypes.byref(n)))
        return k.value, impl.value, {(ck[i], ci[i]): ms[i] for i in range(min(n.value, 8))}

    def graph(self, state, impl=IMPL_AUTO):
        """A CUDA graph of one application of this circuit to `state`."""
        return Graph(self, state, impl)


class Graph:
    def __init__(self, circuit, state, impl=IMPL_AUTO):
        h = ctypes.c_void_p()
        check(lib().qg_circuit_graph_create(circuit.h, state.ptr, state.num_qubits, impl, ctypes.byref(h)))
        self.h = h
        self._keep = (circuit, state)

    @property
    def num_kernels(self):
        n = ctypes.c_int()
        check(lib().qg_graph_get_num_kernels(self.h, ctypes.byref(n)))
        return n.value

    def launch(self, stream=None):
        check(lib().qg_graph_launch(self.h, stream))

    def close(self):
        if self.h is not None and self.h.value:
            lib().qg_graph_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class StateVector32:
    """An FP32 (complex64) statevector in device memory."""

    def __init__(self, num_qubits):
        self.num_qubits = num_qubits
        self.num_amps = 1 << num_qubits
        p = ctypes.c_void_p()
        check(lib().qg_alloc(ctypes.byref(p), self.num_amps * 8))
        self.ptr = p

    def free(self):
        if self.ptr is not None and self.ptr.value:
            lib().qg_free(self.ptr)
            self.ptr = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass

    def set(self, amps):
        a = np.ascontiguousarray(np.asarray(amps).astype(np.complex64).reshape(-1))
        check(lib().qg_copy_h2d(self.ptr, a.ctypes.data, a.nbytes, None))
        lib().qg_sync()

    def get(self):
        out = np.empty(self.num_amps, dtype=np.complex64)
        check(lib().qg_copy_d2h(out.ctypes.data, self.ptr, out.nbytes, None))
        return out

    def init_zero(self):
        check(lib().qg_sv32_initClassicalState(self.ptr, self.num_qubits, 0, None))

    def total_prob(self):
        v = ctypes.c_double()
        check(lib().qg_sv32_calcTotalProb(self.ptr, self.num_qubits, ctypes.byref(v), None))
        return v.value

    def normalise(self, target=1.0):
        """Rescales the state to total probability `target` (FP64-summed norm)."""
        check(lib().qg_sv32_normalise(self.ptr, self.num_qubits, float(target), None))

    def expec_paulis(self, codes_list):
        """Expectation values of Pauli strings given as per-qubit codes (0=I,1=X,2=Y,3=Z)."""
        n = len(codes_list)
        mxy = (ctypes.c_int64 * n)()
        myz = (ctypes.c_int64 * n)()
        ny = (ctypes.c_int * n)()
        for s, codes in enumerate(codes_list):
            a = b = 0
            for q, c in enumerate(codes):
                if c in (1, 2):
                    a |= 1 << q
                if c in (2, 3):
                    b |= 1 << q
            mxy[s], myz[s], ny[s] = a, b, sum(1 for c in codes if c == 2)
        out = (qg_cplx * n)()
        check(lib().qg_sv32_calcExpecPauliStrBatch(self.ptr, self.num_qubits, mxy, myz, ny, n, out, None))
        return np.array([out[s].re for s in range(n)])
