"""Times the oracle port (oracle/_build/libqoracle.so) beside the reference library built
from its own sources (oracle/_ref/libqref.so) on the same circuit sample, the same state
and the same thread count, so that the CPU arm of the benchmark (which times the port,
since the reference library is built for this container's architecture only) can be
compared with QuEST's own CPU build.

Sample: the first `--gates` gates (Haar 2x2 unitaries and controlled phases) of the
benchmark circuit on an n-qubit FP64 statevector.  Each runner's time is the median over
`--reps` runs, timed by each runner around its ops only (the reference runner creates a
Qureg and copies the state in and out on every call, which is not gate work); the two
runners alternate.

    python oracle/compare_port_speed.py [--qubits 28] [--gates 45] [--threads N] [--reps 3]
"""
import argparse
import ctypes
import os
import statistics
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests"))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--qubits", type=int, default=28)
    ap.add_argument("--gates", type=int, default=45)
    ap.add_argument("--threads", type=int, default=os.cpu_count())
    ap.add_argument("--reps", type=int, default=3)
    a = ap.parse_args()
    os.environ["OMP_NUM_THREADS"] = str(a.threads)     # the reference library reads it at its first parallel region
    import bench
    import qcircuits as qc
    ref = qc.reference()
    if ref is None:
        sys.exit("the reference library is not built: make -C oracle ref REF=<QuEST sources>")
    orc = qc.oracle()
    orc.lib.orc_set_num_threads(a.threads)
    n = a.qubits
    gates = bench.make_circuit(n, 20, seed=0x5155455354 + 2)
    lines, nbytes = [], 0
    for g in gates[:a.gates]:
        if g[0] == "U":
            lines.append(f"U1 {g[1]} {qc.mat_tokens(g[2])}")
        elif g[0] == "CP":
            lines.append(f"CPS {g[1]} {g[2]} {qc.fmt(g[3])}")
        else:
            continue
        nbytes += bench.gate_bytes(g, n)
    text = "\n".join(lines) + "\n"
    state = bench.random_state(n, seed=0x5155455354 + 2)
    res = np.zeros(8)
    outs = np.zeros(8, dtype=np.int32)

    seconds = {id(orc): orc.lib.orc_last_run_seconds, id(ref): ref.lib.ref_last_run_seconds}
    for f in seconds.values():
        f.restype = ctypes.c_double

    # both runners work on memory allocated the way QuEST allocates a Qureg (calloc), so
    # that page sizes do not differ between them (numpy asks for transparent huge pages)
    libc = ctypes.CDLL(None)
    libc.calloc.restype = ctypes.c_void_p
    libc.calloc.argtypes = [ctypes.c_size_t, ctypes.c_size_t]
    raw = libc.calloc(1, state.nbytes)
    work = np.ctypeslib.as_array(ctypes.cast(raw, ctypes.POINTER(ctypes.c_double)), shape=(2 * state.size,)).view(np.complex128)

    def timed(runner, body):
        amps = work
        amps[:] = state
        nr, no = ctypes.c_int(0), ctypes.c_int(0)
        rc = runner.fn(body.encode(), n, 0, amps.ctypes.data, res.ctypes.data, 8, ctypes.byref(nr), outs.ctypes.data, 8,
                       ctypes.byref(no))
        if rc != 0:
            raise RuntimeError("runner failed")
        return seconds[id(runner)](), amps

    runners = (("port", orc), ("reference", ref))
    for _, runner in runners:
        timed(runner, text)                                        # warm-up (first-touch, thread pool)
    # the two runners alternate, so that a change in the machine's load falls on both
    times = {name: [] for name, _ in runners}
    for _ in range(a.reps):
        for name, runner in runners:
            times[name].append(timed(runner, text)[0])
    out = {}
    for name, _ in runners:
        secs = statistics.median(times[name])
        out[name] = (secs, nbytes / secs / 1e9)
    a_port = timed(orc, text)[1].copy()
    a_ref = timed(ref, text)[1].copy()
    diff = float(np.max(np.abs(a_port - a_ref)))
    print(f"{n}-qubit FP64 statevector, first {len(lines)} gates of the benchmark circuit, {a.threads} threads, "
          f"median of {a.reps}")
    for name, (secs, gbs) in out.items():
        print(f"  {name:9s}: {secs:8.3f} s of gate work, {gbs:7.2f} GB/s algorithmic")
    print(f"  port / reference speed: {out['port'][1] / out['reference'][1]:.3f}; max-abs difference of the states {diff:.2e}")


if __name__ == "__main__":
    main()
