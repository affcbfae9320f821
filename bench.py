"""Benchmark of the gate-application path: 30-qubit FP64 statevector circuit.

Workload (one step): a seeded random 30-qubit pure state (16 GiB), a depth-20
circuit of Haar-random 2x2 unitaries (QR of a complex Gaussian, phase-fixed) on
every qubit plus a controlled phase of random angle on 15 random disjoint qubit
pairs per layer, then the full QFT (30 H + 435 controlled phases + 15 swaps):
1380 gates, each one QuEST API call (applyCompMatr1, applyTwoQubitPhaseShift,
applyFullQuantumFourierTransform).

Metric: whole-job algorithmic HBM throughput of the gates (GB/s), with the
per-gate algorithmic bytes 2*16*2^(n-c) for a dense gate and 2*16*2^(n-2) for a
controlled phase or a swap (the amplitudes each gate must read and write).
`value` is timed with the state resident in HBM; `e2e` adds the host->device
copy of the input state (pinned) and the device->host copy of the final state
to every step.  The 16 GiB state exceeds L2 (129 MB), so no flush is needed.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference] [--qubits n]
"""
import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

AMP_BYTES = 16


# ------------------------------------------------------------------ workload

def haar_2x2(rng):
    z = (rng.standard_normal((2, 2)) + 1j * rng.standard_normal((2, 2))) / np.sqrt(2)
    q, r = np.linalg.qr(z)
    d = np.diag(r)
    return q * (d / np.abs(d))


def make_circuit(nq, depth, seed):
    """Gate list: ("U", t, 2x2) / ("CP", t1, t2, angle) / ("QFT",)."""
    rng = np.random.default_rng(seed)
    gates = []
    for _ in range(depth):
        for t in range(nq):
            gates.append(("U", t, haar_2x2(rng)))
        perm = rng.permutation(nq)
        for p in range(min(15, nq // 2)):
            gates.append(("CP", int(perm[2 * p]), int(perm[2 * p + 1]), float(rng.uniform(0, 2 * np.pi))))
    gates.append(("QFT",))
    return gates


def gate_bytes(g, nq):
    """Algorithmic bytes (read + write of every amplitude the gate changes)."""
    if g[0] == "U":
        return 2 * AMP_BYTES * (1 << nq)
    if g[0] == "CP":
        return 2 * AMP_BYTES * (1 << (nq - 2))
    # QFT: nq Hadamards, nq(nq-1)/2 controlled phases, nq//2 swaps (a swap moves the
    # |01> and |10> subspaces: 2^(n-1) amplitudes)
    return (nq * 2 * AMP_BYTES * (1 << nq) + (nq * (nq - 1) // 2) * 2 * AMP_BYTES * (1 << (nq - 2))
            + (nq // 2) * 2 * AMP_BYTES * (1 << (nq - 1)))


def num_gates(gates, nq):
    n = 0
    for g in gates:
        n += (nq + nq * (nq - 1) // 2 + nq // 2) if g[0] == "QFT" else 1
    return n


def random_state(nq, seed):
    """Complex Gaussian amplitudes, L2-normalised (generated in chunks)."""
    rng = np.random.default_rng(seed)
    n = 1 << nq
    out = np.empty(n, dtype=np.complex128)
    chunk = 1 << 24
    for s in range(0, n, chunk):
        e = min(n, s + chunk)
        out.real[s:e] = rng.standard_normal(e - s)
        out.imag[s:e] = rng.standard_normal(e - s)
    out /= np.linalg.norm(out)
    return out


# ------------------------------------------------------------------ clocks

class ClockSampler:
    """nvidia-smi clock and throttle-reason samples every 200 ms during a region."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.path = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.QUERY}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if not self.path or not os.path.exists(self.path):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"]}
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax = float(f[2])
            except ValueError:
                continue
            for i, nm in enumerate(names):
                if f[5 + i].lower().startswith("active"):
                    reasons.add(nm)
        os.unlink(self.path)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}


# ------------------------------------------------------------------ distributed plumbing (replicas)

def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch
        import torch.distributed as td
        torch.cuda.set_device(local)
        td.init_process_group("nccl")
        dist = td
    return world, rank, local, dist


def barrier(dist):
    if dist is not None:
        dist.barrier()


def max_over_ranks(dist, value):
    if dist is None:
        return value
    import torch
    t = torch.tensor([value], dtype=torch.float64, device="cuda")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


# ------------------------------------------------------------------ CPU baseline (oracle port)

def cpu_sample(nq, gates, state, num_gates_sample, threads):
    """Runs the first `num_gates_sample` gates of the circuit on the host with the
    CPU oracle (OpenMP restatement of the reference's CPU backend) and returns
    (GB/s, seconds, gates)."""
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import qcircuits as qc
    lines = []
    nbytes = 0
    for g in gates[:num_gates_sample]:
        if g[0] == "U":
            lines.append(f"U1 {g[1]} {qc.mat_tokens(g[2])}")
        elif g[0] == "CP":
            lines.append(f"CPS {g[1]} {g[2]} {qc.fmt(g[3])}")
        else:
            continue
        nbytes += gate_bytes(g, nq)
    orc = qc.oracle()
    orc.lib.orc_set_num_threads(threads)
    amps = np.array(state, copy=True)
    res = np.zeros(8)
    outs = np.zeros(8, dtype=np.int32)
    nres, nout = ctypes.c_int(0), ctypes.c_int(0)
    text = ("\n".join(lines) + "\n").encode()
    t0 = time.perf_counter()
    rc = orc.fn(text, nq, 0, amps.ctypes.data, res.ctypes.data, 8, ctypes.byref(nres), outs.ctypes.data, 8, ctypes.byref(nout))
    dt = time.perf_counter() - t0
    if rc != 0:
        raise RuntimeError("oracle sample failed")
    return nbytes / dt / 1e9, dt, len(lines)


def host_threads():
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


# ------------------------------------------------------------------ GPU arm

def run_gb300(args, world, rank, local, dist):
    from quest_gb300 import _lib, api
    from quest_gb300.api import Q, comp_matr1

    L = _lib.lib()
    import ctypes as C
    dev_count = C.c_int(0)
    L.qg_get_num_devices(C.byref(dev_count))
    if dev_count.value < 1:
        raise SystemExit("no CUDA device visible: the GB300 arm needs a GPU")
    os.environ.setdefault("CUDA_DEVICE_ORDER", "PCI_BUS_ID")
    _lib.check(L.qg_init(local if dev_count.value > local else 0))
    api.init_env()

    nq = args.qubits
    gates = make_circuit(nq, args.depth, seed=0x5155455354 + 2)
    step_bytes = sum(gate_bytes(g, nq) for g in gates)
    step_gates = num_gates(gates, nq)
    state = random_state(nq, seed=0x5155455354 + 2 + rank)

    q = Q.createQureg(nq)
    nbytes = (1 << nq) * AMP_BYTES
    host_in = np.ctypeslib.as_array(C.cast(q.cpuAmps, C.POINTER(C.c_double)), shape=(2 << nq,))
    host_in[:] = state.view(np.float64)       # the pinned host mirror holds the input
    host_out = np.empty(1 << nq, dtype=np.complex128)
    api.set_amps(q, state)

    mats = [comp_matr1(g[2]) if g[0] == "U" else None for g in gates]
    ev = []

    def new_event():
        e = C.c_void_p()
        _lib.check(L.qg_event_create(C.byref(e)))
        return e

    timed_dense = []   # (start, stop) events around every Haar-gate kernel in the timed region

    def run_step(record_dense=False):
        for g, m in zip(gates, mats):
            if g[0] == "U":
                if record_dense:
                    a, b = new_event(), new_event()
                    L.qg_event_record(a, None)
                    Q.applyCompMatr1(q, g[1], m)
                    L.qg_event_record(b, None)
                    timed_dense.append((a, b))
                else:
                    Q.applyCompMatr1(q, g[1], m)
            elif g[0] == "CP":
                Q.applyTwoQubitPhaseShift(q, g[1], g[2], g[3])
            else:
                Q.applyFullQuantumFourierTransform(q)

    for _ in range(args.warmup):
        run_step()
    L.qg_sync()

    # ---- device-resident timing
    launches0 = C.c_int64(0)
    L.qg_get_launch_count(C.byref(launches0))
    start, stop = new_event(), new_event()
    with ClockSampler(local) as clocks:
        barrier(dist)
        L.qg_sync()
        L.qg_event_record(start, None)
        for _ in range(args.steps):
            run_step(record_dense=True)
        L.qg_event_record(stop, None)
        L.qg_sync()
        barrier(dist)
    launches1 = C.c_int64(0)
    L.qg_get_launch_count(C.byref(launches1))
    ms = C.c_float(0)
    L.qg_event_elapsed_ms(start, stop, C.byref(ms))
    t_dev = max_over_ranks(dist, ms.value / 1e3)
    dense_ms = []
    for a, b in timed_dense:
        x = C.c_float(0)
        L.qg_event_elapsed_ms(a, b, C.byref(x))
        dense_ms.append(x.value)
        L.qg_event_destroy(a)
        L.qg_event_destroy(b)
    clk = clocks.summary()

    # ---- end to end through the API with host buffers: H2D input, circuit, D2H result
    e2e_steps = max(1, args.steps)
    barrier(dist)
    L.qg_sync()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        Q.syncQuregToGpu(q)                                  # pinned host -> HBM (16 GiB)
        run_step()
        Q.getQuregAmps(host_out.ctypes.data, q, 0, 1 << nq)  # HBM -> host (16 GiB)
    L.qg_sync()
    t_e2e = max_over_ranks(dist, time.perf_counter() - t0)
    barrier(dist)

    norm = Q.calcTotalProb(q)
    Q.destroyQureg(q)

    value = world * args.steps * step_bytes / t_dev / 1e9
    e2e_value = world * e2e_steps * step_bytes / t_e2e / 1e9
    avg_dense = statistics.mean(dense_ms) / 1e3
    dense_bytes = 2 * AMP_BYTES * (1 << nq)
    peaks = {}
    pk = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(pk):
        peaks = json.load(open(pk))
    peak = peaks.get("hbm_gbs")
    peak_src = "measured" if peak else "fallback"
    peak = peak or 6800.0
    achieved = dense_bytes / avg_dense / 1e9
    # the general complex 2x2 gate needs 16 FP64 FMAs per amplitude pair (64 B): its
    # FP64 issue ceiling in bandwidth terms, from a live probe of the FMA rate
    fma_rate = C.c_double(0)
    _lib.check(L.qg_measure_fp64_fma_rate(C.byref(fma_rate)))
    fp64_ceiling_gbs = fma_rate.value / 16 * 64 / 1e9
    roofline = {"bound": "hbm", "kernel": "k_dense1 (applyCompMatr1, general complex 2x2, FP64)",
                "achieved": round(achieved, 1), "peak": peak, "peak_source": peak_src, "unit": "GB/s",
                "frac": round(achieved / peak, 4), "traffic": args.traffic,
                "launches_timed": len(dense_ms), "avg_launch_ms": round(avg_dense * 1e3, 4),
                "fp64_fma_per_s": round(fma_rate.value, -8), "fp64_ceiling_gbs": round(fp64_ceiling_gbs, 1),
                "fp64_ceiling_frac": round(achieved / fp64_ceiling_gbs, 4)}

    cpu = None
    if rank == 0 and args.cpu_sample > 0:
        threads = host_threads()
        gbps, secs, ng = cpu_sample(nq, gates, state, args.cpu_sample, threads)
        cpu = {"value": round(gbps, 3), "unit": "GB/s", "cores": threads, "kind": "port",
               "sample": f"first {ng} gates of the circuit ({args.qubits}-qubit FP64 statevector) in {secs:.1f} s "
                         f"on {threads} host threads with the OpenMP oracle"}

    line = {
        "metric": "30q gate GB/s vs HBM peak (FP64 statevector, depth-20 Haar 1q + 15 CPhase/layer + QFT)",
        "value": round(value, 2), "unit": "GB/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(t_dev / args.steps * 1e3, 3), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded Gaussian state, seeded Haar gates)",
        "config": {"workload": f"{nq}-qubit FP64 statevector (16 GiB at 30 qubits), depth {args.depth} Haar 1q "
                               f"+ 15 CPhase per layer, then full QFT", "qubits": nq, "depth": args.depth,
                   "gates_per_step": step_gates, "algorithmic_bytes_per_step": step_bytes,
                   "l2": "state (16 GiB) larger than L2; no flush", "parallelism": f"replicas x{world}"},
        "e2e": {"value": round(e2e_value, 2), "unit": "GB/s", "h2d_bytes_per_step": nbytes, "d2h_bytes_per_step": nbytes},
        "gpu_launches": int(launches1.value - launches0.value),
        "roofline": roofline,
        "cpu_baseline": cpu,
        "clocks": clk,
        "final_total_prob": norm,
    }
    if rank == 0:
        print(json.dumps(line), flush=True)


# ------------------------------------------------------------------ reference arm

def run_reference(args, world, rank, dist):
    """The reference's CPU algorithm (the OpenMP oracle port; the reference library
    itself is x86-built here and does not travel to the Arm machine) on all host cores."""
    if rank != 0:
        return
    nq = args.qubits
    gates = make_circuit(nq, args.depth, seed=0x5155455354 + 2)
    state = random_state(nq, seed=0x5155455354 + 2)
    threads = host_threads()
    for _ in range(args.warmup):
        cpu_sample(nq, gates, state, min(2, args.cpu_sample), threads)
    vals, secs = [], 0.0
    for _ in range(args.steps):
        gbps, s, ng = cpu_sample(nq, gates, state, args.cpu_sample, threads)
        vals.append(gbps)
        secs += s
    v = statistics.mean(vals)
    sample = (f"first {ng} gates of the circuit per step ({nq}-qubit FP64 statevector), "
              f"OpenMP oracle port of the reference CPU backend, {threads} threads")
    line = {"impl": "reference",
            "metric": "30q gate GB/s vs HBM peak (FP64 statevector, depth-20 Haar 1q + 15 CPhase/layer + QFT)",
            "value": round(v, 3), "unit": "GB/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": round(secs / args.steps * 1e3, 1), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded Gaussian state, seeded Haar gates)",
            "config": {"workload": f"{nq}-qubit FP64 statevector, depth {args.depth} Haar 1q + 15 CPhase per layer, "
                                   f"then full QFT", "qubits": nq, "depth": args.depth},
            "cpu_baseline": {"value": round(v, 3), "unit": "GB/s", "cores": threads, "kind": "port", "sample": sample},
            "e2e": {"value": round(v, 3), "unit": "GB/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--qubits", type=int, default=30)
    ap.add_argument("--depth", type=int, default=20)
    ap.add_argument("--cpu-sample", type=int, default=45, help="gates of the circuit timed on the host CPU")
    ap.add_argument("--traffic", type=float, default=None, help="ncu DRAM bytes per dense launch, if captured")
    args = ap.parse_args()
    world, rank, local, dist = dist_setup()
    if args.impl == "reference":
        run_reference(args, world, rank, dist)
    else:
        run_gb300(args, world, rank, local, dist)
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
