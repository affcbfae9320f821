"""Python view of the continuous-batching server (qg_server_* in
include/quest_gb300.h) and the hardware-efficient-ansatz requests it serves."""
import ctypes

import numpy as np

from . import _lib
from ._lib import check, lib
from .fused import Circuit


def ry(theta):
    c, s = np.cos(theta / 2), np.sin(theta / 2)
    return np.array([[c, -s], [s, c]], dtype=np.complex128)


def rz(phi):
    return np.diag([np.exp(-0.5j * phi), np.exp(0.5j * phi)]).astype(np.complex128)


CZ = np.diag([1, 1, 1, -1]).astype(np.complex128)


def hea_request(nq, depth, rng, num_strings=16):
    """A hardware-efficient ansatz: `depth` layers of RY and RZ (angles U[0, 2pi)) on
    every qubit and a CZ ladder (q, q+1); plus `num_strings` random Pauli strings
    (I/X/Y/Z uniform per qubit).  Returns (ops, codes): ops are ("RY"|"RZ", t, angle)
    and ("CZ", a, b)."""
    ops = []
    for _ in range(depth):
        for t in range(nq):
            ops.append(("RY", t, float(rng.uniform(0, 2 * np.pi))))
        for t in range(nq):
            ops.append(("RZ", t, float(rng.uniform(0, 2 * np.pi))))
        for t in range(nq - 1):
            ops.append(("CZ", t, t + 1))
    codes = [[int(v) for v in rng.integers(0, 4, nq)] for _ in range(num_strings)]
    return ops, codes


def circuit_of(nq, ops, k=5):
    """The fused FP32 circuit of an op list (one library call for the whole gate list)."""
    g = len(ops)
    kind = np.array([0 if o[0] == "RY" else 1 if o[0] == "RZ" else 2 for o in ops], dtype=np.int32)
    ang = np.array([o[2] if o[0] != "CZ" else 0.0 for o in ops], dtype=np.float64)
    q1 = np.array([o[1] for o in ops], dtype=np.int32)
    q2 = np.array([o[2] if o[0] == "CZ" else 0 for o in ops], dtype=np.int32)
    mats = np.zeros((g, 16), dtype=np.complex128)
    c, s = np.cos(ang / 2), np.sin(ang / 2)
    isy, isz, iscz = kind == 0, kind == 1, kind == 2
    mats[isy, 0], mats[isy, 1], mats[isy, 2], mats[isy, 3] = c[isy], -s[isy], s[isy], c[isy]
    mats[isz, 0], mats[isz, 3] = np.exp(-0.5j * ang[isz]), np.exp(0.5j * ang[isz])
    mats[iscz, 0], mats[iscz, 5], mats[iscz, 10], mats[iscz, 15] = 1, 1, 1, -1
    num_targs = np.where(iscz, 2, 1).astype(np.int32)
    targs = np.stack([q1, q2], axis=1)
    return Circuit(nq).add_many(num_targs, targs, mats).fuse(k)


def text_of(ops, codes):
    """The same request as circuit text for the CPU oracle (RY/RZ/CZ, EXPEC)."""
    lines = []
    for op in ops:
        if op[0] in ("RY", "RZ"):
            lines.append(f"{op[0]} {op[1]} {op[2]!r}")
        else:
            lines.append(f"CZ {op[1]} {op[2]}")
    for c in codes:
        lines.append("EXPEC " + "".join("IXYZ"[v] for v in c))
    return "\n".join(lines) + "\n"


def masks_of(codes):
    n = len(codes)
    mxy = (ctypes.c_int64 * n)()
    myz = (ctypes.c_int64 * n)()
    ny = (ctypes.c_int * n)()
    for s, cs in enumerate(codes):
        mxy[s] = sum(1 << q for q, c in enumerate(cs) if c in (1, 2))
        myz[s] = sum(1 << q for q, c in enumerate(cs) if c in (2, 3))
        ny[s] = sum(1 for c in cs if c == 2)
    return mxy, myz, ny


class Server:
    def __init__(self, hbm_budget_bytes, max_in_flight=512, impl=0):
        h = ctypes.c_void_p()
        check(lib().qg_server_create(ctypes.byref(h), int(hbm_budget_bytes), max_in_flight, impl))
        self.h = h
        self._circuits = {}

    def close(self):
        if self.h is not None and self.h.value:
            lib().qg_server_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def submit(self, circuit, codes):
        mxy, myz, ny = masks_of(codes)
        rid = ctypes.c_int64()
        check(lib().qg_server_submit(self.h, circuit.h, mxy, myz, ny, len(codes), ctypes.byref(rid)))
        self._circuits[rid.value] = (circuit, len(codes))   # keeps the circuit alive until released
        return rid.value

    def poll(self):
        n = ctypes.c_int()
        check(lib().qg_server_poll(self.h, ctypes.byref(n)))
        return n.value

    def result(self, rid):
        _, ns = self._circuits[rid]
        vals = (ctypes.c_double * max(ns, 1))()
        done = ctypes.c_int()
        check(lib().qg_server_result(self.h, rid, vals, ctypes.byref(done)))
        return bool(done.value), np.array(vals[:ns])

    def release(self, rid):
        check(lib().qg_server_release(self.h, rid))
        self._circuits.pop(rid, None)

    def cancel(self, rid):
        """Drops a request whose client went away (queued: at once; running: when it completes)."""
        check(lib().qg_server_cancel(self.h, rid))
        self._circuits.pop(rid, None)

    def stats(self):
        q, f, m, d = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int64()
        check(lib().qg_server_stats(self.h, ctypes.byref(q), ctypes.byref(f), ctypes.byref(m), ctypes.byref(d)))
        return {"queued": q.value, "in_flight": f.value, "hbm_in_use": m.value, "finished": d.value}

    def run_all(self, requests):
        """Submits (circuit, codes) pairs at once and polls until all finish; returns values per request."""
        ids = [self.submit(c, codes) for c, codes in requests]
        out = {}
        while len(out) < len(ids):
            self.poll()
            for rid in ids:
                if rid not in out:
                    done, vals = self.result(rid)
                    if done:
                        out[rid] = vals
        res = [out[rid] for rid in ids]
        for rid in ids:
            self.release(rid)
        return res
