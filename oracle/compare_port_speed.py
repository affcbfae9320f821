"""Times the oracle port (oracle/_build/libqoracle.so) beside the reference library built
from its own sources (oracle/_ref/libqref.so) on the same circuit sample, the same state
and the same thread count, so that the CPU arm of the benchmark (which times the port,
since the reference library is built for this container's architecture only) can be
compared with QuEST's own CPU build.

Sample: the first `--gates` gates (Haar 2x2 unitaries and controlled phases) of the
benchmark circuit on an n-qubit FP64 statevector.  Each runner's time is the median over
`--reps` runs of the sample minus the median of an empty circuit (the runners' own
copies of the state in and out are not gate work).

    python oracle/compare_port_speed.py [--qubits 28] [--gates 45] [--threads N] [--reps 3]
"""
import argparse
import ctypes
import os
import statistics
import sys
import time

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

    def timed(runner, body):
        amps = state.copy()
        nr, no = ctypes.c_int(0), ctypes.c_int(0)
        t0 = time.perf_counter()
        rc = runner.fn(body.encode(), n, 0, amps.ctypes.data, res.ctypes.data, 8, ctypes.byref(nr), outs.ctypes.data, 8,
                       ctypes.byref(no))
        dt = time.perf_counter() - t0
        if rc != 0:
            raise RuntimeError("runner failed")
        return dt, amps

    out = {}
    for name, runner in (("port", orc), ("reference", ref)):
        timed(runner, text)                                        # warm-up (first-touch, thread pool)
        full = statistics.median(timed(runner, text)[0] for _ in range(a.reps))
        empty = statistics.median(timed(runner, "\n")[0] for _ in range(a.reps))
        out[name] = (full - empty, nbytes / (full - empty) / 1e9)
    _, a_port = timed(orc, text)
    _, a_ref = timed(ref, text)
    diff = float(np.max(np.abs(a_port - a_ref)))
    print(f"{n}-qubit FP64 statevector, first {len(lines)} gates of the benchmark circuit, {a.threads} threads, "
          f"median of {a.reps}")
    for name, (secs, gbs) in out.items():
        print(f"  {name:9s}: {secs:8.3f} s of gate work, {gbs:7.2f} GB/s algorithmic")
    print(f"  port / reference speed: {out['port'][1] / out['reference'][1]:.3f}; max-abs difference of the states {diff:.2e}")


if __name__ == "__main__":
    main()
