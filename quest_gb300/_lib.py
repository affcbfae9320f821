"""Loads the in-tree backend library and declares its C ABI for ctypes.

The library is built by ``quest_gb300.build`` (``__graft_entry__.build()``);
loading fails loudly if it is missing -- there is no fallback path.
"""
import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libquest_gb300.so")

_lib = None


class BackendError(RuntimeError):
    """A qg_* call returned a QG_ERR_* code."""


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(
                f"the GB300 backend library is not built ({LIB_PATH} missing); "
                "run `python -m quest_gb300.build` (or __graft_entry__.build())")
        _lib = ctypes.CDLL(LIB_PATH)
        _declare(_lib)
    return _lib


class qg_cplx(ctypes.Structure):
    _fields_ = [("re", ctypes.c_double), ("im", ctypes.c_double)]


class qg_cplxf(ctypes.Structure):
    _fields_ = [("re", ctypes.c_float), ("im", ctypes.c_float)]


c_int_p = ctypes.POINTER(ctypes.c_int)
c_dbl_p = ctypes.POINTER(ctypes.c_double)
c_i64_p = ctypes.POINTER(ctypes.c_int64)
c_cplx_p = ctypes.POINTER(qg_cplx)
vp = ctypes.c_void_p
I = ctypes.c_int
D = ctypes.c_double
I64 = ctypes.c_int64

# name -> argtypes (all return int status)
ABI = {
    "qg_init": [I],
    "qg_get_num_devices": [c_int_p],
    "qg_get_device_info": [c_int_p, c_i64_p, c_i64_p, c_int_p, c_int_p],
    "qg_set_l2_fetch_granularity": [I],
    "qg_get_l2_fetch_granularity": [c_int_p],
    "qg_restore_l2_fetch_granularity": [],
    "qg_alloc": [ctypes.POINTER(vp), I64],
    "qg_free": [vp],
    "qg_copy_h2d": [vp, vp, I64, vp],
    "qg_copy_d2h": [vp, vp, I64, vp],
    "qg_copy_d2d": [vp, vp, I64, vp],
    "qg_sync": [],
    "qg_stream_sync": [vp],
    "qg_get_cache_size": [c_i64_p],
    "qg_clear_cache": [],
    "qg_get_launch_count": [c_i64_p],
    "qg_stream_create": [ctypes.POINTER(vp)],
    "qg_stream_destroy": [vp],
    "qg_stream_wait_event": [vp, vp],
    "qg_event_create": [ctypes.POINTER(vp)],
    "qg_event_destroy": [vp],
    "qg_event_record": [vp, vp],
    "qg_event_elapsed_ms": [vp, vp, ctypes.POINTER(ctypes.c_float)],
    "qg_measure_fp64_fma_rate": [c_dbl_p],
    "qg_sv_initUniformState": [vp, I, qg_cplx, vp],
    "qg_sv_initClassicalState": [vp, I, I64, vp],
    "qg_sv_initDebugState": [vp, I, vp],
    "qg_sv_anyCtrlSwap": [vp, I, c_int_p, c_int_p, I, I, I, vp],
    "qg_sv_anyCtrlOneTargDenseMatr": [vp, I, c_int_p, c_int_p, I, I, c_cplx_p, vp],
    "qg_sv_anyCtrlTwoTargDenseMatr": [vp, I, c_int_p, c_int_p, I, I, I, c_cplx_p, vp],
    "qg_sv_anyCtrlAnyTargDenseMatr": [vp, I, c_int_p, c_int_p, I, c_int_p, I, c_cplx_p, I, vp],
    "qg_sv_qftStep": [vp, I, I, I, I, vp],
    "qg_sv_reverseLowBits": [vp, I, I, vp],
    "qg_sv_qftTwoSteps": [vp, I, I, vp],
    "qg_sv_qftThreeSteps": [vp, I, I, vp],
    "qg_sv_phaseSet": [vp, I, ctypes.POINTER(ctypes.c_int64), c_cplx_p, I, vp],
    "qg_sv_anyCtrlOneTargDiagMatr": [vp, I, c_int_p, c_int_p, I, I, c_cplx_p, vp],
    "qg_sv_anyCtrlTwoTargDiagMatr": [vp, I, c_int_p, c_int_p, I, I, I, c_cplx_p, vp],
    "qg_sv_anyCtrlAnyTargDiagMatr": [vp, I, c_int_p, c_int_p, I, c_int_p, I, c_cplx_p, I, c_cplx_p, vp],
    "qg_sv_anyCtrlPauliTensorOrGadget": [vp, I, c_int_p, c_int_p, I, c_int_p, I, c_int_p, I, c_int_p, I, qg_cplx, qg_cplx, vp],
    "qg_sv_anyCtrlAnyTargZOrPhaseGadget": [vp, I, c_int_p, c_int_p, I, c_int_p, I, qg_cplx, qg_cplx, vp],
    "qg_sv_multiQubitProjector": [vp, I, c_int_p, c_int_p, I, D, vp],
    "qg_dm_multiQubitProjector": [vp, I, c_int_p, c_int_p, I, D, vp],
    "qg_dm_oneQubitDepolarising": [vp, I, I, D, vp],
    "qg_dm_twoQubitDepolarising": [vp, I, I, I, D, vp],
    "qg_dm_oneQubitDephasing": [vp, I, I, D, vp],
    "qg_dm_twoQubitDephasing": [vp, I, I, I, D, vp],
    "qg_dm_oneQubitDamping": [vp, I, I, D, vp],
    "qg_dm_oneQubitPauliChannel": [vp, I, I, D, D, D, vp],
    "qg_sv_calcTotalProb": [vp, I, c_dbl_p, vp],
    "qg_dm_calcTotalProb": [vp, I, c_dbl_p, vp],
    "qg_sv_calcProbOfMultiQubitOutcome": [vp, I, c_int_p, c_int_p, I, c_dbl_p, vp],
    "qg_dm_calcProbOfMultiQubitOutcome": [vp, I, c_int_p, c_int_p, I, c_dbl_p, vp],
    "qg_sv_calcProbsOfAllMultiQubitOutcomes": [c_dbl_p, vp, I, c_int_p, I, vp],
    "qg_dm_calcProbsOfAllMultiQubitOutcomes": [c_dbl_p, vp, I, c_int_p, I, vp],
    "qg_sv_calcExpecAnyTargZ": [vp, I, c_int_p, I, c_dbl_p, vp],
    "qg_dm_calcExpecAnyTargZ": [vp, I, c_int_p, I, c_cplx_p, vp],
    "qg_sv_calcExpecPauliStr": [vp, I, c_int_p, I, c_int_p, I, c_int_p, I, c_cplx_p, vp],
    "qg_dm_calcExpecPauliStr": [vp, I, c_int_p, I, c_int_p, I, c_int_p, I, c_cplx_p, vp],
    "qg_sv_calcExpecPauliStrBatch": [vp, I, c_i64_p, c_i64_p, c_int_p, I, c_cplx_p, vp],
    "qg_dm_calcExpecPauliStrBatch": [vp, I, c_i64_p, c_i64_p, c_int_p, I, c_cplx_p, vp],
    "qg_sv_calcExpecPauliStrBatch_noalloc": [vp, I, c_i64_p, c_i64_p, c_int_p, I, c_cplx_p, vp],
    "qg_circuit_create": [ctypes.POINTER(vp), I],
    "qg_circuit_destroy": [vp],
    "qg_circuit_add_matrix": [vp, c_int_p, I, c_cplx_p],
    "qg_circuit_add_matrices": [vp, I, c_int_p, c_int_p, c_cplx_p],
    "qg_circuit_fuse": [vp, I],
    "qg_circuit_get_num_gates": [vp, c_int_p],
    "qg_circuit_get_num_blocks": [vp, c_int_p],
    "qg_circuit_get_block": [vp, I, c_int_p, c_int_p, c_cplx_p],
    "qg_sv32_apply_circuit": [vp, vp, I, I, vp],
    "qg_tc_get_error_flag": [c_int_p],
    "qg_tc_clear_error_flag": [],
    "qg_tc_selftest_timeout": [I, c_int_p, c_int_p, ctypes.POINTER(ctypes.c_double), c_int_p],
    "qg_circuit_autotune": [vp, c_int_p, c_int_p, c_int_p, c_int_p, c_dbl_p, I, c_int_p],
    "qg_circuit_graph_create": [vp, vp, I, I, ctypes.POINTER(vp)],
    "qg_graph_launch": [vp, vp],
    "qg_graph_get_num_kernels": [vp, c_int_p],
    "qg_graph_destroy": [vp],
    "qg_sv32_initUniformState": [vp, I, qg_cplxf, vp],
    "qg_sv32_initClassicalState": [vp, I, I64, vp],
    "qg_sv_convert_f64_to_f32": [vp, vp, I, vp],
    "qg_sv_convert_f32_to_f64": [vp, vp, I, vp],
    "qg_sv32_calcTotalProb": [vp, I, c_dbl_p, vp],
    "qg_sv32_normalise": [vp, I, D, vp],
    "qg_sv_allTargDiagMatr": [vp, I, vp, qg_cplx, I, vp],
    "qg_dm_allTargDiagMatr": [vp, I, vp, qg_cplx, I, I, vp],
    "qg_sv_calcExpecFullStateDiagMatr": [vp, I, vp, qg_cplx, I, I, c_cplx_p, vp],
    "qg_dm_calcExpecFullStateDiagMatr": [vp, I, vp, qg_cplx, I, I, c_cplx_p, vp],
    "qg_set_fp64_products": [I],
    "qg_get_fp64_products": [c_int_p],
    "qg_set_tensor_slices": [I],
    "qg_get_tensor_slices": [c_int_p],
    "qg_dense_tc_timing": [I],
    "qg_dense_tc_timing_read": [ctypes.POINTER(ctypes.c_float), I, c_int_p],
    "qg_set_kernel_shape": [I, I, I],
    "qg_get_kernel_shape": [I, c_int_p, c_int_p],
    "qg_autotune_fp64": [I, c_dbl_p, I, c_int_p],
    "qg_tune_save": [ctypes.c_char_p],
    "qg_tune_load": [ctypes.c_char_p, c_int_p],
    "qg_sv32_calcExpecPauliStrBatch": [vp, I, c_i64_p, c_i64_p, c_int_p, I, c_cplx_p, vp],
    "qg_server_create": [ctypes.POINTER(vp), I64, I, I],
    "qg_server_destroy": [vp],
    "qg_server_submit": [vp, vp, c_i64_p, c_i64_p, c_int_p, I, c_i64_p],
    "qg_server_poll": [vp, c_int_p],
    "qg_server_result": [vp, I64, c_dbl_p, c_int_p],
    "qg_server_release": [vp, I64],
    "qg_server_cancel": [vp, I64],
    "qg_server_stats": [vp, c_i64_p, c_i64_p, c_i64_p, c_i64_p],
}


def _declare(L):
    for name, args in ABI.items():
        f = getattr(L, name)
        f.argtypes = args
        f.restype = ctypes.c_int
    L.qg_get_last_error.restype = ctypes.c_char_p
    L.qg_get_last_error.argtypes = []
    L.qg_get_error_string.restype = ctypes.c_char_p
    L.qg_get_error_string.argtypes = [ctypes.c_int]
    L.qg_get_version.restype = ctypes.c_int


def check(rc):
    if rc != 0:
        msg = lib().qg_get_last_error().decode(errors="replace")
        raise BackendError(f"backend error {rc}: {msg}")
    return rc


def ints(seq):
    """A ctypes int array (or None for an empty sequence)."""
    seq = list(seq)
    if not seq:
        return None
    return (ctypes.c_int * len(seq))(*[int(v) for v in seq])


def cplx_array(values):
    values = list(values)
    arr = (qg_cplx * len(values))()
    for i, v in enumerate(values):
        v = complex(v)
        arr[i].re = v.real
        arr[i].im = v.imag
    return arr
