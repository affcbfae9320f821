"""Benchmark of the gate-application path: 30-qubit FP64 statevector circuit.

Workload (one step): a seeded random 30-qubit pure state (16 GiB), a depth-20
circuit of Haar-random 2x2 unitaries (QR of a complex Gaussian, phase-fixed) on
every qubit plus a controlled phase of random angle on 15 random disjoint qubit
pairs per layer, then the full QFT (30 H + 435 controlled phases + 15 swaps):
1380 gates, each one QuEST API call (applyCompMatr1, applyTwoQubitPhaseShift,
applyFullQuantumFourierTransform).

Metric: whole-job algorithmic HBM throughput of the gates (GB/s), with the
per-gate algorithmic bytes 2*16*2^(n-c) for a dense gate, 2*16*2^(n-2) for a
controlled phase and 2*16*2^(n-1) for a swap (the amplitudes each gate must read and
write).  `value` is timed with the state resident in HBM; `e2e` adds, to every step,
the host->device copy of the input state and the device->host copy of the final
state, both through the register's pinned host mirror (syncQuregToGpu /
syncQuregFromGpu).  The 16 GiB state exceeds L2 (129 MB), so no flush is needed.

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

def haar(dim, rng):
    """A Haar-random dim x dim unitary (QR of a complex Gaussian matrix, R's diagonal phase-fixed)."""
    z = (rng.standard_normal((dim, dim)) + 1j * rng.standard_normal((dim, dim))) / np.sqrt(2)
    q, r = np.linalg.qr(z)
    d = np.diag(r)
    return q * (d / np.abs(d))


def haar_2x2(rng):
    return haar(2, rng)


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
    """Replicas: one process per GPU under torchrun (NCCL), or gloo where no GPU is
    visible (the replica logic's CPU tests).  No data-path collective: only a barrier
    around the timed region and the max of the ranks' times."""
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch
        import torch.distributed as td
        if torch.cuda.is_available():
            torch.cuda.set_device(local)
            td.init_process_group("nccl")
        else:
            td.init_process_group("gloo")
        dist = td
    return world, rank, local, dist


def barrier(dist):
    if dist is not None:
        dist.barrier()


def max_over_ranks(dist, value):
    if dist is None:
        return value
    import torch
    device = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([value], dtype=torch.float64, device=device)
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
    _lib.check(L.qg_set_fp64_products(0 if args.fp64_products == "fixed" else 1))
    # the library's launch-shape autotuner, on a 28-qubit scratch register (4 GiB), before any timing
    tune_ms = (C.c_double * 12)()
    tune_n = C.c_int(0)
    _lib.check(L.qg_autotune_fp64(min(28, args.qubits), tune_ms, 12, C.byref(tune_n)))
    shapes = []
    for kern in (0, 1, 2):
        tppt, tthr = C.c_int(), C.c_int()
        _lib.check(L.qg_get_kernel_shape(kern, C.byref(tppt), C.byref(tthr)))
        shapes.append([tppt.value, tthr.value])
    tuning = {"dense1_fx_shape": shapes[0], "diag1_fx_shape": shapes[1], "dense2_fx_shape": shapes[2],
              "candidates_ms": [round(tune_ms[i], 4) for i in range(tune_n.value)]}

    nq = args.qubits
    gates = make_circuit(nq, args.depth, seed=0x5155455354 + 2)
    step_bytes = sum(gate_bytes(g, nq) for g in gates)
    step_gates = num_gates(gates, nq)
    state = random_state(nq, seed=0x5155455354 + 2 + rank)

    q = Q.createQureg(nq)
    nbytes = (1 << nq) * AMP_BYTES
    host_in = np.ctypeslib.as_array(C.cast(q.cpuAmps, C.POINTER(C.c_double)), shape=(2 << nq,))
    host_in[:] = state.view(np.float64)       # the pinned host mirror holds the input
    api.set_amps(q, state)

    mats = [comp_matr1(g[2]) if g[0] == "U" else None for g in gates]
    ev = []

    def new_event():
        e = C.c_void_p()
        _lib.check(L.qg_event_create(C.byref(e)))
        return e

    timed_dense = []   # (start, stop) events around every Haar-gate kernel in the timed region

    def run_step(record_dense=False, reg=None):
        r = q if reg is None else reg
        for g, m in zip(gates, mats):
            if g[0] == "U":
                if record_dense:
                    a, b = new_event(), new_event()
                    L.qg_event_record(a, None)
                    Q.applyCompMatr1(r, g[1], m)
                    L.qg_event_record(b, None)
                    timed_dense.append((a, b))
                else:
                    Q.applyCompMatr1(r, g[1], m)
            elif g[0] == "CP":
                Q.applyTwoQubitPhaseShift(r, g[1], g[2], g[3])
            else:
                Q.applyFullQuantumFourierTransform(r)
        # one-qubit gates deferred by the API (applied four qubits per tensor-core pass)
        # are applied now, on this step's stream, so the step's result is complete
        Q.flushQuregDeferredOps(r)

    def tc_times():
        # durations of the tensor-core dense launches recorded since qg_dense_tc_timing(1)
        n = C.c_int(0)
        _lib.check(L.qg_dense_tc_timing_read(None, 0, C.byref(n)))
        buf = (C.c_float * max(1, n.value))()
        _lib.check(L.qg_dense_tc_timing_read(buf, n.value, C.byref(n)))
        _lib.check(L.qg_dense_tc_timing(0))
        return [buf[i] for i in range(n.value)]

    for _ in range(args.warmup):
        run_step()
    L.qg_sync()

    # ---- device-resident timing
    launches0 = C.c_int64(0)
    L.qg_get_launch_count(C.byref(launches0))
    start, stop = new_event(), new_event()
    _lib.check(L.qg_dense_tc_timing(1))
    with ClockSampler(local) as clocks:
        barrier(dist)
        L.qg_sync()
        L.qg_event_record(start, None)
        for _ in range(args.steps):
            run_step(record_dense=True)
        L.qg_event_record(stop, None)
        L.qg_sync()
        barrier(dist)
    tc_ms = tc_times()
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

    # ---- end to end through the API with host buffers, double-buffered.  Step i runs its
    # gates on register regs[i % 2] (compute stream) while the copy stream reads step
    # i-1's result out of the other register and then writes step i+1's input into it.
    # Every step's input (16 GiB, from q's pinned host mirror) and result (16 GiB, into
    # q2's pinned host mirror) cross the host link inside the timed region; events on the
    # two streams order each copy against the gates of its register.
    q2 = Q.createQureg(nq)
    regs = [q, q2]
    namps = 1 << nq
    in_ptr = C.cast(q.cpuAmps, C.c_void_p)
    out_ptr = C.cast(q2.cpuAmps, C.c_void_p)
    mirrors = ["pinned" if Q.isQuregHostMirrorPinned(r) else "pageable" for r in regs]
    sc, sx = C.c_void_p(), C.c_void_p()
    _lib.check(L.qg_stream_create(C.byref(sc)))
    _lib.check(L.qg_stream_create(C.byref(sx)))
    # the host link alone: one 16 GiB copy each way on the copy stream
    a, b = new_event(), new_event()
    Q.setQuESTStream(sx)
    L.qg_event_record(a, sx)
    Q.setQuregAmps(q2, 0, in_ptr, namps)
    L.qg_event_record(b, sx)
    h2d_ms = C.c_float(0)
    L.qg_event_elapsed_ms(a, b, C.byref(h2d_ms))
    L.qg_event_record(a, sx)
    Q.getQuregAmps(out_ptr, q2, 0, namps)
    L.qg_event_record(b, sx)
    d2h_ms = C.c_float(0)
    L.qg_event_elapsed_ms(a, b, C.byref(d2h_ms))
    Q.setQuESTStream(None)
    e2e_steps = max(1, args.steps)
    ev_up = [new_event() for _ in range(e2e_steps)]
    ev_done = [new_event() for _ in range(e2e_steps)]
    barrier(dist)
    L.qg_sync()
    t0 = time.perf_counter()
    Q.setQuESTStream(sx)
    Q.setQuregAmps(regs[0], 0, in_ptr, namps)           # step 0's input
    L.qg_event_record(ev_up[0], sx)
    for i in range(e2e_steps):
        L.qg_stream_wait_event(sc, ev_up[i])
        Q.setQuESTStream(sc)
        run_step(reg=regs[i % 2])
        L.qg_event_record(ev_done[i], sc)
        Q.setQuESTStream(sx)
        if i >= 1:
            L.qg_stream_wait_event(sx, ev_done[i - 1])
            Q.getQuregAmps(out_ptr, regs[(i - 1) % 2], 0, namps)     # step i-1's result
        if i + 1 < e2e_steps:
            Q.setQuregAmps(regs[(i + 1) % 2], 0, in_ptr, namps)      # step i+1's input
            L.qg_event_record(ev_up[i + 1], sx)
    L.qg_stream_wait_event(sx, ev_done[e2e_steps - 1])
    Q.getQuregAmps(out_ptr, regs[(e2e_steps - 1) % 2], 0, namps)     # the last step's result
    L.qg_sync()
    t_e2e = max_over_ranks(dist, time.perf_counter() - t0)
    Q.setQuESTStream(None)
    barrier(dist)
    for e in ev_up + ev_done + [a, b]:
        L.qg_event_destroy(e)
    L.qg_stream_destroy(sc)
    L.qg_stream_destroy(sx)

    # ---- both product modes on one step from the same input: final total probabilities,
    # and the IEEE-FP64 dense kernel's launch time beside the fixed-point one
    modes = {}
    for mode_name, mode_val, reg in (("fixed", 0, q), ("fp64", 1, q2)):
        _lib.check(L.qg_set_fp64_products(mode_val))
        Q.setQuregAmps(reg, 0, in_ptr, namps)
        timed_dense.clear()
        _lib.check(L.qg_dense_tc_timing(1))
        run_step(record_dense=True, reg=reg)
        L.qg_sync()
        mode_tc = tc_times()
        ms_list = []
        for x, y in timed_dense:
            v = C.c_float(0)
            L.qg_event_elapsed_ms(x, y, C.byref(v))
            ms_list.append(v.value)
            L.qg_event_destroy(x)
            L.qg_event_destroy(y)
        timed_dense.clear()
        modes[mode_name] = {"final_total_prob": Q.calcTotalProb(reg)}
        if mode_tc:
            modes[mode_name]["fused_pass_ms"] = round(statistics.mean(mode_tc), 4)
            modes[mode_name]["fused_passes"] = len(mode_tc)
        else:
            modes[mode_name]["dense_kernel_ms"] = round(statistics.mean(ms_list), 4)
    _lib.check(L.qg_set_fp64_products(0 if args.fp64_products == "fixed" else 1))
    norm = Q.calcTotalProb(q)
    Q.destroyQureg(q2)
    Q.destroyQureg(q)

    value = world * args.steps * step_bytes / t_dev / 1e9
    e2e_value = world * e2e_steps * step_bytes / t_e2e / 1e9
    # the dominant kernel: the tensor-core passes of deferred one-qubit gates (four per
    # pass) when the API defers them, else the per-gate dense kernel; either streams the
    # state once per launch
    fused = len(tc_ms) > 0
    avg_dense = statistics.mean(tc_ms if fused else dense_ms) / 1e3
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
    # DRAM bytes per dense launch: given on the command line, else scaled from the ncu
    # capture of the same kernel at 28 qubits (dram__bytes_read.sum + dram__bytes_write.sum
    # = 8.530e9 B for 2^27 pairs: 63.55 B per pair; the FP64-FMA kernel's capture: 8.53e9 B too)
    if args.traffic is not None:
        traffic, traffic_src = args.traffic, "command line"
    elif fused:
        # the 26-qubit capture of the four-target kernel: 1.0739e9 + 1.0131e9 B for 2^26
        # amplitudes (31.10 B per amplitude), profiles/k_dense_tc_26q_ncu.md
        traffic = round(31.10 * (1 << nq))
        traffic_src = "ncu capture of k_dense_tc at 26 qubits (31.10 B per amplitude) scaled to this size"
    else:
        traffic = round(63.55 * (1 << (nq - 1)))
        traffic_src = "ncu capture at 28 qubits (63.55 B per amplitude pair) scaled to this size"
    if fused:
        kname = ("k_dense_tc (deferred one-qubit gates, four per pass, as one 16x16 operator with the layer's "
                 "controlled phases on those qubits folded in: exact 8-bit slices on the fp16 tensor cores)")
    elif args.fp64_products == "fixed":
        kname = "k_dense1_fx (applyCompMatr1, general complex 2x2, FP64 storage, fixed-point products)"
    else:
        kname = "k_dense1 (applyCompMatr1, general complex 2x2, FP64)"
    roofline = {"bound": "hbm", "kernel": kname,
                "achieved": round(achieved, 1), "peak": peak, "peak_source": peak_src, "unit": "GB/s",
                "frac": round(achieved / peak, 4), "traffic": traffic, "traffic_source": traffic_src,
                "launches_timed": len(tc_ms) if fused else len(dense_ms), "avg_launch_ms": round(avg_dense * 1e3, 4),
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
        "vs_baseline": None,
        "dtype": "f64" if args.fp64_products == "fp64" else
                 "f64 (storage and all other ops; general 2x2 products in 60-bit block-floating fixed point, "
                 "deferred one-qubit gates four per pass, with the controlled phases among them folded in, as "
                 "exact 8-bit slices on the fp16 tensor cores)",
        "data": "synthetic (seeded Gaussian state, seeded Haar gates)",
        "config": {"workload": f"{nq}-qubit FP64 statevector (16 GiB at 30 qubits), depth {args.depth} Haar 1q "
                               f"+ 15 CPhase per layer, then full QFT", "qubits": nq, "depth": args.depth,
                   "gates_per_step": step_gates, "algorithmic_bytes_per_step": step_bytes,
                   "l2": "state (16 GiB) larger than L2; no flush", "parallelism": f"replicas x{world}",
                   "fp64_products": args.fp64_products, "autotune": tuning},
        "e2e": {"value": round(e2e_value, 2), "unit": "GB/s", "h2d_bytes_per_step": nbytes, "d2h_bytes_per_step": nbytes,
                "steps": e2e_steps, "ms_per_step": round(t_e2e / e2e_steps * 1e3, 3),
                "frac_of_value": round(e2e_value / value, 4),
                "schedule": "double-buffered: two registers, gates on one stream, host copies on another",
                "host_mirror": mirrors[0] if mirrors[0] == mirrors[1] else ",".join(mirrors),
                "h2d_gbs": round(nbytes / (h2d_ms.value / 1e3) / 1e9, 1),
                "d2h_gbs": round(nbytes / (d2h_ms.value / 1e3) / 1e9, 1)},
        "product_modes": {**modes, "note": "one step of the circuit from the same input in each mode; "
                                            "fused_pass_ms = mean CUDA-event time of the tensor-core passes of "
                                            "deferred one-qubit gates (fixed point); dense_kernel_ms = mean time of "
                                            "the per-gate Haar launches (IEEE FP64, not deferred)"},
        "gpu_launches": int(launches1.value - launches0.value),
        "roofline": roofline,
        "cpu_baseline": cpu,
        "clocks": clk,
        "final_total_prob": norm,
    }
    if world == 1 and not args.no_extras:
        line["precision_form"], line["serving"], line["density_matrix"] = extras_summary(args, world, rank, local, dist)
    if rank == 0:
        print(json.dumps(line), flush=True)


def extras_summary(args, world, rank, local, dist):
    """The precision form (32-qubit FP32 fused blocks on the tensor cores, accuracy at 28
    qubits), the serving form (a short request set, served vs plain) and the
    density-matrix method (14 qubits, 30 layers, one step) in small, so the default line
    records them beside the FP64 circuit.  A failure here is reported in the line and does
    not lose the headline."""
    precision = serving = None
    try:
        pa = argparse.Namespace(**vars(args))
        pa.qubits, pa.acc_qubits, pa.depth, pa.steps, pa.warmup, pa.fused_impl = 32, 28, 40, 2, 1, "tc"
        pl = run_precision(pa, world, rank, local, dist, emit=False)
        precision = {"workload": pl["config"]["workload"], "blocks": pl["config"]["blocks"], "steps": pa.steps,
                     "value_gbs": pl["value"], "frac_of_hbm": pl["roofline"]["frac"],
                     "ms_per_block_pass": pl["ms_per_block_pass"], "tensor_tflops": pl["roofline"]["tensor_tflops"],
                     "accuracy": pl["accuracy"], "tc_error_flag": pl["tc_error_flag"]}
    except Exception as e:          # noqa: BLE001 -- recorded in the line
        precision = {"error": f"{type(e).__name__}: {e}"}
    try:
        sa = argparse.Namespace(**vars(args))
        sa.requests, sa.min_qubits, sa.max_qubits, sa.load = 12, 8, 26, 0.8
        sl = run_serve(sa, world, rank, local, dist, emit=False)
        serving = {"requests": sa.requests, "data": sl["data"], "saturation": sl["saturation"],
                   "poisson": sl["poisson"], "max_abs_expec_err_served_vs_fp64": sl["max_abs_expec_err_served_vs_fp64"],
                   "plain_registers": sl["plain_registers"], "plain_path": sl["plain_path"]}
    except Exception as e:          # noqa: BLE001
        serving = {"error": f"{type(e).__name__}: {e}"}
    try:
        da = argparse.Namespace(**vars(args))
        da.steps, da.warmup, da.cpu_sample, da.dm_qubits, da.dm_layers = 1, 1, 1, 14, 30
        dl = run_dm(da, world, rank, local, dist, emit=False)
        dm = {"workload": dl["config"]["workload"], "steps": 1, "value_gbs": dl["value"], "frac_of_hbm": dl["frac_of_hbm"],
              "ms_per_step": dl["ms_per_step"], "ms_per_layer": dl["ms_per_layer"], "per_op": dl["per_op"],
              "final_purity": dl["final_purity"], "cpu_baseline": dl["cpu_baseline"]}
    except Exception as e:          # noqa: BLE001
        dm = {"error": f"{type(e).__name__}: {e}"}
    return precision, serving, dm


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


# ------------------------------------------------------------------ precision form (FP32 fused blocks)

def brickwork_gates(nq, depth, seed):
    """Haar 1q on every qubit + CZ on alternating neighbour pairs, per layer."""
    rng = np.random.default_rng(seed)
    cz = np.diag([1, 1, 1, -1]).astype(np.complex128)
    gates = []
    for d in range(depth):
        for t in range(nq):
            gates.append(([t], haar_2x2(rng)))
        for t in range(d % 2, nq - 1, 2):
            gates.append(([t, t + 1], cz))
    return gates


def precision_accuracy(na, depth, impl):
    """Fidelity, max-abs amplitude error and Pauli-expectation error of the fused FP32
    path against the FP64 per-gate path on the same seeded state and circuit."""
    import ctypes as C
    from quest_gb300 import api
    from quest_gb300.api import Q, comp_matr1
    from quest_gb300.fused import Circuit, StateVector32
    gates = brickwork_gates(na, depth, seed=0x5155455354 + 4)
    psi0 = random_state(na, seed=0x5155455354 + 4)
    q = Q.createQureg(na)
    api.set_amps(q, psi0)
    for t, m in gates:
        if len(t) == 1:
            Q.applyCompMatr1(q, t[0], comp_matr1(m))
        else:
            Q.applyControlledPauliZ(q, t[0], t[1])
    psi64 = api.get_amps(q)
    rng = np.random.default_rng(7)
    codes = [[int(v) for v in rng.integers(0, 4, na)] for _ in range(16)]
    strs = (api.PauliStr * 16)(*[api.pauli_str(c) for c in codes])
    e64 = (C.c_double * 16)()
    Q.calcExpecPauliStrs(e64, q, strs, 16)
    Q.destroyQureg(q)
    circ = Circuit(na)
    for t, m in gates:
        circ.add(t, m)
    circ.fuse(5)
    s = StateVector32(na)
    s.set(psi0)
    circ.apply(s, impl=impl)
    norm_drift = s.total_prob() - 1.0
    s.normalise(1.0)        # the circuit is unitary and psi0 has norm 1
    e32 = s.expec_paulis(codes)
    psi32 = s.get().astype(np.complex128)
    s.free()
    fid = float(abs(np.vdot(psi32, psi64)) ** 2 / (np.vdot(psi32, psi32).real * np.vdot(psi64, psi64).real))
    maxabs = float(np.max(np.abs(psi32 - psi64)))
    experr = float(np.max(np.abs(np.array(e32) - np.array(list(e64)))))
    return fid, maxabs, experr, norm_drift


def run_precision(args, world, rank, local, dist, emit=True):
    """FP32 statevector, brickwork circuit fused into 5-qubit blocks applied as 3xTF32
    tensor-core GEMM tiles, then an FP64-summed renormalisation (the circuit is unitary).
    Accuracy against the FP64 per-gate path (which is pinned to the FP64 oracle) at
    `--acc-qubits`; throughput at `--qubits`."""
    import ctypes as C
    from quest_gb300 import _lib, api
    from quest_gb300.api import Q, comp_matr1
    from quest_gb300.fused import Circuit, StateVector32, IMPL_TC, IMPL_SIMT
    L = _lib.lib()
    _lib.check(L.qg_init(local))
    api.init_env()
    nq, na, depth = args.qubits, args.acc_qubits, args.depth
    impl = {"simt": IMPL_SIMT, "tc": IMPL_TC}[args.fused_impl]

    # ---- accuracy at na qubits (0: skipped)
    fid = maxabs = experr = drift = None
    if na > 0:
        fid, maxabs, experr, drift = precision_accuracy(na, depth, impl)
    accuracy = {"qubits": na, "fidelity": fid, "one_minus_fidelity": None if fid is None else 1 - fid,
                "max_abs_amp_err": maxabs, "max_pauli_expec_err": experr,
                "norm_drift_before_normalise": drift,
                "reference": "FP64 per-gate GPU path (parity-pinned to the oracle)"}

    # ---- throughput at nq qubits
    gates = brickwork_gates(nq, depth, seed=0x5155455354 + 4)
    circ = Circuit(nq)
    for t, m in gates:
        circ.add(t, m)
    circ.fuse(5)
    nblocks = circ.num_blocks
    s = StateVector32(nq)
    s.init_zero()
    for _ in range(args.warmup):
        circ.apply(s, impl=impl)
        s.normalise(1.0)
    L.qg_sync()
    ev0, ev1 = C.c_void_p(), C.c_void_p()
    L.qg_event_create(C.byref(ev0))
    L.qg_event_create(C.byref(ev1))
    launches0 = C.c_int64(0)
    L.qg_get_launch_count(C.byref(launches0))
    with ClockSampler(local) as clocks:
        barrier(dist)
        L.qg_event_record(ev0, None)
        for _ in range(args.steps):
            circ.apply(s, impl=impl)
            s.normalise(1.0)
        L.qg_event_record(ev1, None)
        L.qg_sync()
        barrier(dist)
    launches1 = C.c_int64(0)
    L.qg_get_launch_count(C.byref(launches1))
    ms = C.c_float(0)
    L.qg_event_elapsed_ms(ev0, ev1, C.byref(ms))
    t = max_over_ranks(dist, ms.value / 1e3)
    norm = s.total_prob()
    flag = C.c_int(0)
    L.qg_tc_get_error_flag(C.byref(flag))
    s.free()
    pass_bytes = 2 * 8 * (1 << nq)
    norm_bytes = 3 * 8 * (1 << nq)     # FP64-summed norm (read) + rescale (read + write)
    eff = world * args.steps * (nblocks * pass_bytes + norm_bytes) / t / 1e9
    per_pass_ms = t / (args.steps * nblocks) * 1e3
    peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json"))) if os.path.exists(os.path.join(ROOT, "MEASURED_PEAKS.json")) else {}
    peak = peaks.get("hbm_gbs", 6800.0)
    tensor_flops = nblocks * 3 * 2 * (1 << (nq - 5)) * 64 * 64   # 3 real 64x64 products per 32-amplitude group
    line = {"metric": "precision form: FP32 fused-block circuit throughput (effective HBM GB/s) and fidelity vs FP64",
            "value": round(eff, 1), "unit": "GB/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": round(t / args.steps * 1e3, 2), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32 (3xTF32 tensor-core products)" if impl != IMPL_SIMT else "f32 (SIMT FFMA)",
            "data": "synthetic (|0> start for throughput; seeded Gaussian state for accuracy)",
            "config": {"workload": f"{nq}-qubit FP32 statevector, depth-{depth} Haar 1q + CZ brickwork fused into "
                                   f"<=5-qubit blocks", "qubits": nq, "depth": depth, "gates": len(gates),
                       "blocks": nblocks, "impl": args.fused_impl},
            "circuits_per_s": round(world * args.steps / t, 3), "ms_per_block_pass": round(per_pass_ms, 3),
            "roofline": {"bound": "hbm", "kernel": "k32_fused_tc" if impl == IMPL_TC else "k32_fused",
                         "achieved": round(eff / world, 1), "peak": peak, "unit": "GB/s",
                         "frac": round(eff / world / peak, 4), "traffic": None,
                         "tensor_tflops": round(tensor_flops * args.steps / t / 1e12, 1)},
            "accuracy": accuracy,
            "gpu_launches": int(launches1.value - launches0.value), "tc_error_flag": flag.value,
            "final_total_prob": norm, "clocks": clocks.summary()}
    if rank == 0 and emit:
        print(json.dumps(line), flush=True)
    return line


# ------------------------------------------------------------------ serving form

def log(msg):
    print(f"[bench {time.strftime('%H:%M:%S')}] {msg}", file=sys.stderr, flush=True)

def run_serve(args, world, rank, local, dist, emit=True):
    """Poisson stream of hardware-efficient-ansatz requests (8-26 qubits, depth 10-100,
    16 Pauli expectations each).  Served: FP32 fused blocks through the continuous-
    batching server (circuits fused on a host thread pool as they arrive).  Plain:
    QuEST's per-gate FP64 path through the API, one request at a time in arrival order."""
    import concurrent.futures as cf
    import ctypes as C
    from quest_gb300 import _lib, api
    from quest_gb300.api import Q
    from quest_gb300.serve import Server, circuit_of, hea_request
    L = _lib.lib()
    _lib.check(L.qg_init(local))
    api.init_env()
    rng = np.random.default_rng(0x5155455354 + 5 + rank)
    reqs = []
    for _ in range(args.requests):
        n = int(rng.integers(args.min_qubits, args.max_qubits + 1))
        depth = int(rng.integers(10, 101))
        ops, codes = hea_request(n, depth, rng)
        reqs.append((n, depth, ops, codes))
    ngates = sum(len(r[2]) for r in reqs)

    # one register per qubit count, made before any timing: the plain arm then times gate
    # work and reductions, not allocation (the served arm carves its registers out of a
    # pre-allocated arena the same way)
    plain_regs = {}
    for n in sorted({r[0] for r in reqs} | {10}):
        plain_regs[n] = Q.createQureg(n)

    def plain_one(n, ops, codes):
        # per gate: the API's deferral of one-qubit gates into tensor-core passes is off
        # for this arm (it follows the tensor-slice switch), so every gate is one pass
        _lib.check(L.qg_set_tensor_slices(0))
        try:
            return plain_gates(n, ops, codes)
        finally:
            _lib.check(L.qg_set_tensor_slices(1))

    def plain_gates(n, ops, codes):
        q = plain_regs[n]
        Q.initZeroState(q)
        for op in ops:
            if op[0] == "RY":
                Q.applyRotateY(q, op[1], op[2])
            elif op[0] == "RZ":
                Q.applyRotateZ(q, op[1], op[2])
            else:
                Q.applyControlledPauliZ(q, op[1], op[2])
        strs = (api.PauliStr * len(codes))(*[api.pauli_str(c) for c in codes])
        vals = (C.c_double * len(codes))()
        Q.calcExpecPauliStrs(vals, q, strs, len(codes))
        return np.array(list(vals))

    def run_plain(arrivals):
        t0 = time.perf_counter()
        lat, vals = [], []
        for (n, depth, ops, codes), ta in zip(reqs, arrivals):
            while time.perf_counter() - t0 < ta:
                time.sleep(1e-4)
            t1 = time.perf_counter()
            vals.append(plain_one(n, ops, codes))
            lat.append(time.perf_counter() - t0 - ta)
            log(f"plain  n={n:2d} depth={depth:3d} gates={len(ops):5d} {1e3 * (time.perf_counter() - t1):9.1f} ms")
        return time.perf_counter() - t0, lat, vals

    def run_served(arrivals):
        server = Server(args.hbm_budget_gib << 30, max_in_flight=max(64, len(reqs)))
        pool = cf.ThreadPoolExecutor(max_workers=args.fuse_threads)
        t0 = time.perf_counter()
        nxt, futs, live, lat, vals = 0, {}, {}, [None] * len(reqs), [None] * len(reqs)
        done = 0
        last_progress = time.perf_counter()
        while done < len(reqs):
            now = time.perf_counter() - t0
            if time.perf_counter() - last_progress > args.stall_s:
                raise RuntimeError(f"served path made no progress for {args.stall_s} s: {server.stats()}, "
                                   f"{len(futs)} circuits being fused, {len(live)} in the server, {done} done")
            while nxt < len(reqs) and arrivals[nxt] <= now:
                n, depth, ops, codes = reqs[nxt]
                futs[nxt] = pool.submit(circuit_of, n, ops)
                nxt += 1
            progressed = False
            for i in [i for i, f in futs.items() if f.done()]:
                live[server.submit(futs.pop(i).result(), reqs[i][3])] = i
                progressed = True
            progressed |= server.poll() > 0
            for rid in list(live):
                ok, v = server.result(rid)
                if ok:
                    i = live.pop(rid)
                    lat[i] = time.perf_counter() - t0 - arrivals[i]
                    vals[i] = v
                    server.release(rid)
                    done += 1
                    last_progress = time.perf_counter()
                    log(f"served n={reqs[i][0]:2d} depth={reqs[i][1]:3d} latency {1e3 * lat[i]:9.1f} ms")
            if not futs and not live and nxt < len(reqs):
                time.sleep(max(0.0, min(1e-3, arrivals[nxt] - (time.perf_counter() - t0))))
            elif not progressed:
                time.sleep(5e-5)   # leaves the interpreter lock to the fusing threads
        makespan = time.perf_counter() - t0
        pool.shutdown()
        server.close()
        return makespan, lat, vals

    # warm-up: compile kernels, create contexts
    small = [(10, 5, *hea_request(10, 5, np.random.default_rng(1)))]
    run_served_small = Server(1 << 30)
    run_served_small.run_all([(circuit_of(10, small[0][2]), small[0][3])])
    run_served_small.close()
    plain_one(10, small[0][2], small[0][3])

    zero = [0.0] * len(reqs)
    # saturation: every request queued at t = 0
    log("phase: plain, saturation")
    ms_plain, lat_p0, vals_plain = run_plain(zero)
    log(f"phase: served, saturation (plain took {ms_plain:.1f} s)")
    ms_served, lat_s0, vals_served = run_served(zero)
    log(f"served took {ms_served:.1f} s")
    err = max(float(np.max(np.abs(a - b))) for a, b in zip(vals_plain, vals_served))
    cps_plain = len(reqs) / ms_plain
    cps_served = len(reqs) / ms_served
    # Poisson arrivals at `load` x the plain path's capacity, the same stream for both
    lam = args.load * cps_plain
    arrivals = list(np.cumsum(np.random.default_rng(11).exponential(1.0 / lam, len(reqs))))
    log(f"phase: Poisson at {lam:.2f}/s, plain")
    _, lat_p, _ = run_plain(arrivals)
    log("phase: Poisson, served")
    _, lat_s, _ = run_served(arrivals)
    pct = lambda xs, q: float(np.percentile(np.array(xs) * 1e3, q))
    line = {"metric": "serving: circuits/s and p50/p99 latency, served FP32 fused batched vs plain per-gate FP64",
            "value": round(world * cps_served, 3), "unit": "circuits/s", "n_gpus": world,
            "steps": 1, "warmup": args.warmup, "ms_per_step": round(ms_served * 1e3, 1), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32 served / f64 plain",
            "data": f"synthetic: {len(reqs)} hardware-efficient ansatz requests, {args.min_qubits}-{args.max_qubits} qubits, "
                    f"depth 10-100, 16 Pauli strings each ({ngates} gates)",
            "config": {"workload": "Poisson stream of HEA circuits (RY/RZ + CZ ladder), 16 Pauli expectations each",
                       "requests": len(reqs), "hbm_budget_gib": args.hbm_budget_gib, "fuse_threads": args.fuse_threads},
            "saturation": {"served_circuits_per_s": round(cps_served, 3), "plain_circuits_per_s": round(cps_plain, 3),
                           "speedup": round(cps_served / cps_plain, 2),
                           "served_makespan_s": round(ms_served, 3), "plain_makespan_s": round(ms_plain, 3)},
            "poisson": {"rate_per_s": round(lam, 3), "load_vs_plain_capacity": args.load,
                        "served_p50_ms": round(pct(lat_s, 50), 2), "served_p99_ms": round(pct(lat_s, 99), 2),
                        "plain_p50_ms": round(pct(lat_p, 50), 2), "plain_p99_ms": round(pct(lat_p, 99), 2)},
            "max_abs_expec_err_served_vs_fp64": err,
            "plain_registers": "one pre-created register per qubit count, reset to |0> per request",
            "plain_path": "one pass per gate (fixed-point FP64 products; the API's deferral of one-qubit gates off)"}
    for r in plain_regs.values():
        Q.destroyQureg(r)
    if rank == 0 and emit:
        print(json.dumps(line), flush=True)
    return line


def run_gates(args, world, rank, local, dist):
    """Per-gate-kind timing on one FP64 register: 1- to 4-target dense unitaries, a
    controlled phase and a swap, in both product modes (fixed point, FP64 FMAs), after
    the launch-shape autotuner, and the API's fused passes (a set of controlled phases,
    one, two and three QFT steps, the QFT's closing swaps); then density-matrix channels on a
    register of half the qubits (the same bytes).  ms per call from CUDA events over
    `--steps` calls."""
    import ctypes as C
    from quest_gb300 import _lib, api
    from quest_gb300._lib import qg_cplx
    L = _lib.lib()
    _lib.check(L.qg_init(local))
    api.init_env()
    n = args.qubits if "--qubits" in sys.argv else 28
    ms_buf, cnt = (C.c_double * 12)(), C.c_int(0)
    _lib.check(L.qg_autotune_fp64(min(28, n), ms_buf, 12, C.byref(cnt)))
    tuned = {}
    for kern, name in ((0, "dense1_fx"), (1, "diag1_fx"), (2, "dense2_fx")):
        tppt, tthr = C.c_int(), C.c_int()
        _lib.check(L.qg_get_kernel_shape(kern, C.byref(tppt), C.byref(tthr)))
        tuned[name] = {"shape": [tppt.value, tthr.value],
                       "candidates_ms": [round(ms_buf[4 * kern + i], 4) for i in range(4)]}
    p = C.c_void_p()
    _lib.check(L.qg_alloc(C.byref(p), 16 << n))
    _lib.check(L.qg_sv_initUniformState(p, n, qg_cplx(1 / np.sqrt(2.0 ** n), 0), None))
    rng = np.random.default_rng(0x5155455354 + 6)
    e0, e1 = C.c_void_p(), C.c_void_p()
    L.qg_event_create(C.byref(e0))
    L.qg_event_create(C.byref(e1))
    state_bytes = 16 << n
    phase = (qg_cplx * 2)(qg_cplx(1, 0), qg_cplx(np.cos(0.3), np.sin(0.3)))

    def timed(fn):
        for _ in range(max(1, args.warmup)):
            fn()
        L.qg_sync()
        L.qg_event_record(e0, None)
        for _ in range(args.steps):
            fn()
        L.qg_event_record(e1, None)
        ms = C.c_float()
        L.qg_event_elapsed_ms(e0, e1, C.byref(ms))
        return ms.value / args.steps

    rows = []
    for mode in ("fixed", "fp64"):
        _lib.check(L.qg_set_fp64_products(0 if mode == "fixed" else 1))
        for k in (1, 2, 3, 4):
            D = 1 << k
            u = haar(D, rng).reshape(-1)
            m = (qg_cplx * (D * D))(*[qg_cplx(v.real, v.imag) for v in u])
            t = (C.c_int * k)(*range(3, 3 + k))
            ms = timed(lambda: _lib.check(L.qg_sv_anyCtrlAnyTargDenseMatr(p, n, None, None, 0, t, k, m, 0, None)))
            label = "fixed (tensor-core slices)" if mode == "fixed" and k >= 3 else mode
            rows.append({"gate": f"dense, {k} target(s)", "products": label, "ms": round(ms, 4),
                         "gbs": round(2 * state_bytes / ms / 1e6, 1)})
            if mode == "fixed" and k >= 3:
                # the same gate on the lowest qubits, and through the integer-pipe kernels
                t0 = (C.c_int * k)(*range(k))
                ms = timed(lambda: _lib.check(L.qg_sv_anyCtrlAnyTargDenseMatr(p, n, None, None, 0, t0, k, m, 0, None)))
                rows.append({"gate": f"dense, {k} target(s) on qubits 0..{k - 1}", "products": label, "ms": round(ms, 4),
                             "gbs": round(2 * state_bytes / ms / 1e6, 1)})
                _lib.check(L.qg_set_tensor_slices(0))
                ms = timed(lambda: _lib.check(L.qg_sv_anyCtrlAnyTargDenseMatr(p, n, None, None, 0, t, k, m, 0, None)))
                _lib.check(L.qg_set_tensor_slices(1))
                rows.append({"gate": f"dense, {k} target(s)", "products": "fixed (integer pipes)", "ms": round(ms, 4),
                             "gbs": round(2 * state_bytes / ms / 1e6, 1)})
        ctrl = C.c_int(2)
        ms = timed(lambda: _lib.check(L.qg_sv_anyCtrlOneTargDiagMatr(p, n, C.byref(ctrl), None, 1, 7, phase, None)))
        rows.append({"gate": "controlled phase (quarter of the amplitudes)", "products": mode, "ms": round(ms, 4),
                     "gbs": round(2 * state_bytes / 4 / ms / 1e6, 1)})
    _lib.check(L.qg_set_fp64_products(0))
    ms = timed(lambda: _lib.check(L.qg_sv_anyCtrlSwap(p, n, None, None, 0, 4, 9, None)))
    rows.append({"gate": "swap (half of the amplitudes)", "products": "none", "ms": round(ms, 4),
                 "gbs": round(2 * state_bytes / 2 / ms / 1e6, 1)})
    # the fused passes of the API (fixed point): a set of 15 controlled phases, one QFT step
    # (Hadamard and its controlled phases), two and three QFT steps, the QFT's closing swaps;
    # GB/s of one read and one write of the whole state
    npairs = min(15, n // 2)
    pairs = rng.permutation(n)[:2 * npairs].reshape(npairs, 2)
    masks = (C.c_int64 * npairs)(*[(1 << int(a)) | (1 << int(b)) for a, b in pairs])
    th = rng.uniform(0, 2 * np.pi, npairs)
    fs = (qg_cplx * npairs)(*[qg_cplx(np.cos(x), np.sin(x)) for x in th])
    T = n - 8
    for name, fn in ((f"phase set: {npairs} controlled phases in one pass",
                      lambda: _lib.check(L.qg_sv_phaseSet(p, n, masks, fs, npairs, None))),
                     (f"QFT step of qubit {T} (Hadamard + {T} controlled phases) in one pass",
                      lambda: _lib.check(L.qg_sv_qftStep(p, n, T, 0, T, None))),
                     (f"QFT steps of qubits {T} and {T - 1} in one pass",
                      lambda: _lib.check(L.qg_sv_qftTwoSteps(p, n, T, None))),
                     (f"QFT steps of qubits {T}, {T - 1} and {T - 2} in one pass",
                      lambda: _lib.check(L.qg_sv_qftThreeSteps(p, n, T, None))),
                     (f"QFT closing swaps ({n // 2} swaps) as one bit-reversal pass",
                      lambda: _lib.check(L.qg_sv_reverseLowBits(p, n, n, None)))):
        ms = timed(fn)
        rows.append({"gate": name, "products": "fixed" if "swaps" not in name else "none", "ms": round(ms, 4),
                     "gbs": round(2 * state_bytes / ms / 1e6, 1)})
    L.qg_free(p)

    # density-matrix channels on an N-qubit density matrix (its 2N-qubit Choi vector has
    # the same bytes as the statevector above); every channel below streams the whole
    # Choi vector once
    from quest_gb300.api import Q, comp_matr1, kraus_map
    nd = n // 2
    dm = Q.createDensityQureg(nd)
    Q.initPlusState(dm)
    pass_bytes = 2 * state_bytes
    u1 = comp_matr1(haar(2, rng))
    k1 = kraus_map([np.sqrt(0.7) * np.eye(2), np.sqrt(0.3) * haar(2, rng)])
    iso = haar(16, rng)[:, :4]                                    # a 16x4 isometry: four 4x4 Kraus operators
    k2 = kraus_map([iso[4 * i:4 * i + 4, :] for i in range(4)])
    # one-qubit unitaries and channels on a density matrix are deferred (multiplied into a
    # pending superoperator per qubit); syncQuESTEnv applies them, one pass each
    def now(fn):
        def run():
            fn()
            Q.syncQuESTEnv()
        return run
    dm_gates = [("applyCompMatr1 on the density matrix (one pass of conj(U) x U)", 1, now(lambda: Q.applyCompMatr1(dm, 3, u1))),
                ("mixDepolarising", 1, now(lambda: Q.mixDepolarising(dm, 3, 0.01))),
                ("mixTwoQubitDepolarising", 1, lambda: Q.mixTwoQubitDepolarising(dm, 3, 8, 0.01)),
                ("mixDephasing (the off-diagonal half)", 0.5, now(lambda: Q.mixDephasing(dm, 3, 0.05))),
                ("mixDamping", 1, now(lambda: Q.mixDamping(dm, 3, 0.05))),
                ("mixKrausMap, 1 qubit (2-target superoperator)", 1, now(lambda: Q.mixKrausMap(dm, (C.c_int * 1)(3), 1, k1))),
                ("mixKrausMap, 2 qubits (4-target superoperator)", 1,
                 lambda: Q.mixKrausMap(dm, (C.c_int * 2)(3, 8), 2, k2))]
    for mode in ("fixed", "fp64"):
        _lib.check(L.qg_set_fp64_products(0 if mode == "fixed" else 1))
        for name, passes, fn in dm_gates:
            ms = timed(fn)
            four = "2 qubits" in name
            rows.append({"gate": f"DM {nd}q: {name}", "products": "fixed (tensor-core slices)" if mode == "fixed" and four else mode,
                         "ms": round(ms, 4), "gbs": round(passes * pass_bytes / ms / 1e6, 1)})
            if mode == "fixed" and four:
                _lib.check(L.qg_set_tensor_slices(0))
                ms = timed(fn)
                _lib.check(L.qg_set_tensor_slices(1))
                rows.append({"gate": f"DM {nd}q: {name}", "products": "fixed (integer pipes)", "ms": round(ms, 4),
                             "gbs": round(passes * pass_bytes / ms / 1e6, 1)})
    _lib.check(L.qg_set_fp64_products(0))
    Q.destroyQureg(dm)
    peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json"))) if os.path.exists(os.path.join(ROOT, "MEASURED_PEAKS.json")) else {}
    peak = peaks.get("hbm_gbs", 6800.0)
    for r in rows:
        r["frac_of_hbm"] = round(r["gbs"] / peak, 3)
    line = {"metric": "per-gate GB/s on an FP64 statevector, by gate kind and product mode", "value": rows[0]["gbs"],
            "unit": "GB/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64 storage", "data": "synthetic (uniform state, seeded Haar gates)",
            "config": {"workload": f"{n}-qubit FP64 statevector, one gate per launch", "qubits": n,
                       "l2": "state larger than L2; no flush"},
            "gates": rows, "hbm_peak_gbs": peak,
            "autotune": {"candidates": "(1,256), (1,128), (2,256), (2,128)", **tuned}}
    if rank == 0:
        print(json.dumps(line), flush=True)


def run_expec(args, world, rank, local, dist):
    """Batched Pauli expectation values on one FP64 statevector (`--qubits`, default 28):
    16 random strings (I/X/Y/Z uniform per qubit) through the batched entry point, one
    launch per call, beside the same strings one per call.  ms per call from CUDA events
    over `--steps` calls after `--warmup`; GB/s counts one read of the state (16 B per
    amplitude) per call, the bytes one pass must move."""
    import ctypes as C
    from quest_gb300 import _lib, api
    from quest_gb300._lib import qg_cplx
    L = _lib.lib()
    _lib.check(L.qg_init(local))
    api.init_env()
    n = args.qubits if "--qubits" in sys.argv else 28
    ns = 16
    rng = np.random.default_rng(0x5155455354 + 8)
    codes = [[int(v) for v in rng.integers(0, 4, n)] for _ in range(ns)]
    mxy = (C.c_int64 * ns)(*[sum(1 << q for q, c in enumerate(cs) if c in (1, 2)) for cs in codes])
    myz = (C.c_int64 * ns)(*[sum(1 << q for q, c in enumerate(cs) if c in (2, 3)) for cs in codes])
    ny = (C.c_int * ns)(*[sum(1 for c in cs if c == 2) for cs in codes])
    p = C.c_void_p()
    _lib.check(L.qg_alloc(C.byref(p), 16 << n))
    state = random_state(n, seed=0x5155455354 + 8)
    _lib.check(L.qg_copy_h2d(p, state.ctypes.data, 16 << n, None))
    out = (qg_cplx * ns)()
    e0, e1 = C.c_void_p(), C.c_void_p()
    L.qg_event_create(C.byref(e0))
    L.qg_event_create(C.byref(e1))

    def timed(fn):
        for _ in range(max(1, args.warmup)):
            fn()
        L.qg_sync()
        L.qg_event_record(e0, None)
        for _ in range(args.steps):
            fn()
        L.qg_event_record(e1, None)
        ms = C.c_float()
        L.qg_event_elapsed_ms(e0, e1, C.byref(ms))
        return ms.value / args.steps

    ms_batch = timed(lambda: _lib.check(L.qg_sv_calcExpecPauliStrBatch(p, n, mxy, myz, ny, ns, out, None)))
    batch_vals = [out[i].re for i in range(ns)]
    one = (qg_cplx * 1)()

    def per_string():
        for s in range(ns):
            x = [q for q, c in enumerate(codes[s]) if c == 1]
            y = [q for q, c in enumerate(codes[s]) if c == 2]
            z = [q for q, c in enumerate(codes[s]) if c == 3]
            _lib.check(L.qg_sv_calcExpecPauliStr(p, n, _lib.ints(x), len(x), _lib.ints(y), len(y),
                                                 _lib.ints(z), len(z), one, None))
    ms_single = timed(per_string)
    L.qg_free(p)
    state_bytes = 16 << n
    peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json"))) if os.path.exists(os.path.join(ROOT, "MEASURED_PEAKS.json")) else {}
    peak = peaks.get("hbm_gbs", 6800.0)
    line = {"metric": "batched Pauli expectation values: ms per 16 strings on an FP64 statevector",
            "value": round(ms_batch, 4), "unit": "ms", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded Gaussian state, 16 random I/X/Y/Z strings)",
            "config": {"workload": f"{n}-qubit FP64 statevector, 16 Pauli strings per call", "qubits": n,
                       "l2": "state larger than L2; no flush"},
            "batch_ms": round(ms_batch, 4), "per_string_calls_ms": round(ms_single, 4),
            "batch_one_pass_gbs": round(state_bytes / ms_batch / 1e6, 1),
            "batch_one_pass_frac_of_hbm": round(state_bytes / ms_batch / 1e6 / peak, 3),
            "values": batch_vals, "hbm_peak_gbs": peak}
    if rank == 0:
        print(json.dumps(line), flush=True)


def dm_layers(nq, layers, seed):
    """The density-matrix method's circuit: per layer, Haar 2x2 unitaries on every qubit
    (even layers) or Haar 4x4 unitaries on disjoint random pairs (odd layers), then
    mixDepolarising(0.01) on every qubit and one 2-qubit 4-operator Kraus map (the 4x4
    blocks of a random 16x4 isometry) on a random pair.  Returns a list of ops:
    ("U1", t, m) / ("U2", a, b, m) / ("DEPOL", t, p) / ("KRAUS", a, b, [K0..K3])."""
    rng = np.random.default_rng(seed)
    ops = []
    for layer in range(layers):
        if layer % 2 == 0:
            for t in range(nq):
                ops.append(("U1", t, haar(2, rng)))
        else:
            perm = rng.permutation(nq)
            for i in range(0, nq - 1, 2):
                ops.append(("U2", int(perm[i]), int(perm[i + 1]), haar(4, rng)))
        for t in range(nq):
            ops.append(("DEPOL", t, 0.01))
        a, b = (int(v) for v in rng.choice(nq, size=2, replace=False))
        g = rng.standard_normal((16, 4)) + 1j * rng.standard_normal((16, 4))
        qm, r = np.linalg.qr(g)
        qm = qm * (np.diag(r) / np.abs(np.diag(r)))
        ops.append(("KRAUS", a, b, [qm[4 * i:4 * i + 4, :] for i in range(4)]))
    return ops


def random_mixed_state(nq, seed, num_pure=8):
    """sum_j w_j |psi_j><psi_j| (Dirichlet weights, Gaussian states) as a column-major flat
    Choi vector (row = low bits)."""
    rng = np.random.default_rng(seed)
    w = rng.dirichlet(np.ones(num_pure))
    dim = 1 << nq
    psi = rng.standard_normal((dim, num_pure)) + 1j * rng.standard_normal((dim, num_pure))
    psi /= np.linalg.norm(psi, axis=0)
    rho = (psi * w) @ psi.conj().T
    return np.ascontiguousarray(rho.T).reshape(-1)


def run_dm(args, world, rank, local, dist, emit=True):
    """The density-matrix method (14-qubit density matrix: a 28-qubit Choi vector, 4 GiB)
    through the QuEST-named API: 30 layers of unitaries, depolarising on every qubit and a
    2-qubit Kraus map, then calcPurity and 16 Pauli expectation values.  One step is the
    whole circuit from the same input state.  Also the time of each kind of operation on
    its own (per call, from CUDA events), and the CPU oracle on the first layer."""
    import ctypes as C
    from quest_gb300 import _lib, api
    from quest_gb300.api import Q, comp_matr1, comp_matr2, kraus_map
    L = _lib.lib()
    _lib.check(L.qg_init(local))
    api.init_env()
    ms_buf, cnt = (C.c_double * 12)(), C.c_int(0)
    _lib.check(L.qg_autotune_fp64(28, ms_buf, 12, C.byref(cnt)))
    nq, layers = args.dm_qubits, args.dm_layers
    ops = dm_layers(nq, layers, seed=0x5155455354 + 3)
    rng = np.random.default_rng(0x5155455354 + 3)
    codes = [[int(v) for v in rng.integers(0, 4, nq)] for _ in range(16)]
    state = random_mixed_state(nq, seed=0x5155455354 + 3)
    nbytes = 16 << (2 * nq)
    prepared = []
    for op in ops:
        if op[0] == "U1":
            prepared.append((0, op[1], comp_matr1(op[2])))
        elif op[0] == "U2":
            prepared.append((1, (op[1], op[2]), comp_matr2(op[3])))
        elif op[0] == "DEPOL":
            prepared.append((2, op[1], op[2]))
        else:
            prepared.append((3, (C.c_int * 2)(op[1], op[2]), kraus_map(op[3])))
    strs = (api.PauliStr * 16)(*[api.pauli_str(c) for c in codes])
    vals = (C.c_double * 16)()
    q = Q.createDensityQureg(nq)
    api.set_amps(q, state)
    # the input stays on the device: each step starts from a device-to-device copy of it
    src = C.c_void_p()
    _lib.check(L.qg_alloc(C.byref(src), nbytes))
    _lib.check(L.qg_copy_d2d(src, C.cast(q.gpuAmps, C.c_void_p), nbytes, None))

    def apply(op):
        k = op[0]
        if k == 0:
            Q.applyCompMatr1(q, op[1], op[2])
        elif k == 1:
            Q.applyCompMatr2(q, op[1][0], op[1][1], op[2])
        elif k == 2:
            Q.mixDepolarising(q, op[1], op[2])
        else:
            Q.mixKrausMap(q, op[1], 2, op[2])

    def step():
        # nothing is pending here: the previous step ended with reductions, which apply
        # every deferred operation first
        _lib.check(L.qg_copy_d2d(C.cast(q.gpuAmps, C.c_void_p), src, nbytes, None))
        for op in prepared:
            apply(op)
        purity = Q.calcPurity(q)
        Q.calcExpecPauliStrs(vals, q, strs, 16)
        return purity

    for _ in range(args.warmup):
        step()
    L.qg_sync()
    e0, e1 = C.c_void_p(), C.c_void_p()
    L.qg_event_create(C.byref(e0))
    L.qg_event_create(C.byref(e1))
    launches0 = C.c_int64(0)
    L.qg_get_launch_count(C.byref(launches0))
    with ClockSampler(local) as clocks:
        barrier(dist)
        L.qg_sync()
        L.qg_event_record(e0, None)
        for _ in range(args.steps):
            purity = step()
        L.qg_event_record(e1, None)
        L.qg_sync()
        barrier(dist)
    launches1 = C.c_int64(0)
    L.qg_get_launch_count(C.byref(launches1))
    ms = C.c_float(0)
    L.qg_event_elapsed_ms(e0, e1, C.byref(ms))
    t = max_over_ranks(dist, ms.value / 1e3)
    # each kind of operation alone, per call (a deferred one-qubit op is applied by the sync)
    per_op = {}
    kinds = {0: "applyCompMatr1 (one-qubit unitary)", 1: "applyCompMatr2 (two-qubit unitary, ket and bra passes)",
             2: "mixDepolarising", 3: "mixKrausMap (2 qubits, 4 operators: a 4-target superoperator)"}
    for k, name in kinds.items():
        sample = [op for op in prepared if op[0] == k][:8]
        L.qg_sync()
        L.qg_event_record(e0, None)
        for op in sample:
            apply(op)
            if k in (0, 2):
                Q.syncQuESTEnv()        # applies the op now (it is deferred otherwise)
        L.qg_event_record(e1, None)
        L.qg_event_elapsed_ms(e0, e1, C.byref(ms))
        per = ms.value / len(sample)
        passes = 2 if k == 1 else 1
        per_op[name] = {"ms": round(per, 4), "gbs": round(passes * 2 * nbytes / per / 1e6, 1)}
    # the fused pair the circuit produces most: a one-qubit unitary followed by depolarising
    L.qg_sync()
    L.qg_event_record(e0, None)
    for t_ in range(8):
        Q.applyCompMatr1(q, t_ % nq, prepared[0][2])
        Q.mixDepolarising(q, t_ % nq, 0.01)
        Q.syncQuESTEnv()
    L.qg_event_record(e1, None)
    L.qg_event_elapsed_ms(e0, e1, C.byref(ms))
    per_op["applyCompMatr1 + mixDepolarising on one qubit (one fused pass)"] = {
        "ms": round(ms.value / 8, 4), "gbs": round(2 * nbytes / (ms.value / 8) / 1e6, 1)}
    Q.destroyQureg(q)
    L.qg_free(src)
    ops_count = {name: sum(1 for op in prepared if op[0] == k) for k, name in kinds.items()}
    alg_bytes = sum((2 if op[0] == 1 else 1) * 2 * nbytes for op in prepared) + nbytes * 3   # + purity and the state reset
    cpu = None
    if rank == 0 and args.cpu_sample > 0:
        sys.path.insert(0, os.path.join(ROOT, "tests"))
        import qcircuits as qc
        lines = []
        first = [op for op in ops][:2 * nq + 1] if ops[0][0] == "U1" else ops[:nq]
        cbytes = 0
        for op in first:
            if op[0] == "U1":
                lines.append(f"U1 {op[1]} {qc.mat_tokens(op[2])}"); cbytes += 2 * 2 * nbytes
            elif op[0] == "DEPOL":
                lines.append(f"DEPOL {op[1]} {qc.fmt(op[2])}"); cbytes += 2 * nbytes
            elif op[0] == "U2":
                lines.append(f"U2 {op[1]} {op[2]} {qc.mat_tokens(op[3])}"); cbytes += 2 * 2 * nbytes
            else:
                lines.append(f"KRAUS 2 {op[1]} {op[2]} 4 " + " ".join(qc.mat_tokens(m) for m in op[3])); cbytes += 2 * nbytes
        orc = qc.oracle()
        threads = host_threads()
        orc.lib.orc_set_num_threads(threads)
        amps = state.copy()
        res, outs = np.zeros(8), np.zeros(8, dtype=np.int32)
        nr, no = C.c_int(0), C.c_int(0)
        t0 = time.perf_counter()
        orc.fn(("\n".join(lines) + "\n").encode(), nq, 1, amps.ctypes.data, res.ctypes.data, 8, C.byref(nr),
               outs.ctypes.data, 8, C.byref(no))
        secs = time.perf_counter() - t0
        cpu = {"value": round(cbytes / secs / 1e9, 3), "unit": "GB/s", "cores": threads, "kind": "port",
               "sample": f"the first {len(lines)} operations (unitaries and depolarising of layer 1, the reference's "
                         f"two passes per unitary) in {secs:.1f} s on {threads} host threads with the OpenMP oracle"}
    peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json"))) if os.path.exists(os.path.join(ROOT, "MEASURED_PEAKS.json")) else {}
    peak = peaks.get("hbm_gbs", 6800.0)
    gbs = world * args.steps * alg_bytes / t / 1e9
    line = {"metric": "density-matrix method: GB/s of the whole circuit (algorithmic bytes of the reference's passes) and ms per layer",
            "value": round(gbs, 1), "unit": "GB/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": round(t / args.steps * 1e3, 2), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64 (storage; products in block-floating fixed point)",
            "data": "synthetic (seeded mixed state of 8 Gaussian pure states, Dirichlet weights; seeded Haar gates and Kraus maps)",
            "config": {"workload": f"{nq}-qubit FP64 density matrix ({2 * nq}-qubit Choi vector), {layers} layers of "
                                   f"unitaries + mixDepolarising(0.01) on every qubit + a 2-qubit 4-operator Kraus map, then "
                                   f"calcPurity and 16 Pauli expectations", "qubits": nq, "layers": layers,
                       "ops": ops_count, "l2": "state larger than L2; no flush",
                       "bytes": "per op 2 x 16 B x 4^N (the reference's passes: two for a unitary) + the state reset (a device copy) + purity",
                       "start": "each step from a device copy of the input state"},
            "ms_per_layer": round(t / args.steps / layers * 1e3, 3),
            "frac_of_hbm": round(gbs / world / peak, 4), "per_op": per_op,
            "final_purity": purity, "expec": list(vals), "gpu_launches": int(launches1.value - launches0.value),
            "cpu_baseline": cpu, "clocks": clocks.summary()}
    if rank == 0 and emit:
        print(json.dumps(line), flush=True)
    return line


def c1_gates(nq, layers, seed, num_expec=16):
    """The plain method (C1): `layers` x (H on every qubit; RX, RY, RZ on every qubit with
    angles uniform in [0, 2 pi); a CNOT ladder q -> q + 1), then the total probability and
    `num_expec` Pauli expectation values, the codes I/X/Y/Z uniform per qubit.  The same
    draws as the parity tests' text form of this circuit."""
    rng = np.random.default_rng(seed)
    gates = []
    for _ in range(layers):
        gates += [("H", t) for t in range(nq)]
        for t in range(nq):
            for op in ("RX", "RY", "RZ"):
                gates.append((op, t, float(rng.uniform(0, 2 * np.pi))))
        gates += [("CX", t, t + 1) for t in range(nq - 1)]
    codes = [[int(v) for v in rng.integers(0, 4, size=nq)] for _ in range(num_expec)]
    return gates, codes


def run_c1(args, world, rank, local, dist):
    """The plain method (C1) at 20 qubits (16 MiB: the state fits in L2) through the
    QuEST-named API: 10 layers of H, RX/RY/RZ on every qubit and a CNOT ladder, then
    calcTotalProb and 16 Pauli expectation values; one step is the whole circuit from the
    same input (a device copy), ending with the reductions (a host read).  Reports the wall
    time per circuit, the time of each gate kind alone, and the CPU oracle on the whole
    circuit with its results beside the GPU's."""
    import ctypes as C
    from quest_gb300 import _lib, api
    from quest_gb300.api import Q
    L = _lib.lib()
    _lib.check(L.qg_init(local))
    api.init_env()
    nq = args.qubits if "--qubits" in sys.argv else 20
    layers = args.depth if "--depth" in sys.argv else 10
    seed = 0x5155455354 + 1
    gates, codes = c1_gates(nq, layers, seed)
    state = random_state(nq, seed)
    strs = (api.PauliStr * len(codes))(*[api.pauli_str(c) for c in codes])
    vals = (C.c_double * len(codes))()
    nbytes = 16 << nq
    q = Q.createQureg(nq)
    api.set_amps(q, state)
    src = C.c_void_p()
    _lib.check(L.qg_alloc(C.byref(src), nbytes))
    _lib.check(L.qg_copy_d2d(src, C.cast(q.gpuAmps, C.c_void_p), nbytes, None))

    def apply(g):
        if g[0] == "H":
            Q.applyHadamard(q, g[1])
        elif g[0] == "RX":
            Q.applyRotateX(q, g[1], g[2])
        elif g[0] == "RY":
            Q.applyRotateY(q, g[1], g[2])
        elif g[0] == "RZ":
            Q.applyRotateZ(q, g[1], g[2])
        else:
            Q.applyControlledPauliX(q, g[1], g[2])

    def step():
        _lib.check(L.qg_copy_d2d(C.cast(q.gpuAmps, C.c_void_p), src, nbytes, None))
        for g in gates:
            apply(g)
        prob = Q.calcTotalProb(q)
        Q.calcExpecPauliStrs(vals, q, strs, len(codes))
        return prob

    for _ in range(args.warmup):
        step()
    L.qg_sync()
    launches0 = C.c_int64(0)
    L.qg_get_launch_count(C.byref(launches0))
    with ClockSampler(local) as clocks:
        barrier(dist)
        L.qg_sync()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            prob = step()
        L.qg_sync()
        wall = max_over_ranks(dist, time.perf_counter() - t0)
        barrier(dist)
    launches1 = C.c_int64(0)
    L.qg_get_launch_count(C.byref(launches1))
    got = [prob] + list(vals)
    # each gate kind alone: 20 calls, then flushQuregDeferredOps (deferred kinds are applied there)
    e0, e1, ms = C.c_void_p(), C.c_void_p(), C.c_float(0)
    L.qg_event_create(C.byref(e0))
    L.qg_event_create(C.byref(e1))
    per_kind = {}
    amp_bytes = {"H": 2 * nbytes, "RX": 2 * nbytes, "RY": 2 * nbytes, "RZ": 2 * nbytes, "CX": nbytes}
    for kind in ("H", "RX", "RY", "RZ", "CX"):
        sample = [g for g in gates if g[0] == kind][:20]
        L.qg_sync()
        L.qg_event_record(e0, None)
        for g in sample:
            apply(g)
        Q.flushQuregDeferredOps(q)
        L.qg_event_record(e1, None)
        L.qg_event_elapsed_ms(e0, e1, C.byref(ms))
        per = ms.value / len(sample)
        per_kind[kind] = {"ms_per_gate": round(per, 5), "gbs": round(amp_bytes[kind] / per / 1e6, 1)}
    Q.destroyQureg(q)
    L.qg_free(src)
    alg_bytes = sum(amp_bytes[g[0]] for g in gates) + nbytes * (1 + len(codes))
    cpu = None
    if rank == 0 and args.cpu_sample > 0:
        sys.path.insert(0, os.path.join(ROOT, "tests"))
        import qcircuits as qc
        text = qc.config1_circuit(nq, layers, seed, len(codes))
        orc = qc.oracle()
        threads = host_threads()
        orc.lib.orc_set_num_threads(threads)
        t0 = time.perf_counter()
        _, want, _ = orc.run(text, nq, 0, state)
        secs = time.perf_counter() - t0
        cpu = {"value": round(secs * 1e3, 2), "unit": "ms per circuit", "cores": threads, "kind": "port",
               "sample": f"the whole circuit ({len(gates)} gates and {1 + len(codes)} reductions) on {threads} host "
                         f"threads with the OpenMP oracle",
               "max_abs_diff_of_results": float(np.max(np.abs(np.array(got) - np.array(want[:len(got)]))))}
    line = {"metric": "plain method (C1): wall time per 20-qubit circuit", "value": round(wall / args.steps * 1e3, 3),
            "unit": "ms per circuit", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": round(wall / args.steps * 1e3, 3), "higher_is_better": False, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64 (storage; products in block-floating fixed point, one-qubit gates deferred)",
            "data": "synthetic (seeded Gaussian state, seeded angles and Pauli codes)",
            "config": {"workload": f"{nq}-qubit FP64 statevector, {layers} x (H on every qubit, RX/RY/RZ on every "
                                   f"qubit, CNOT ladder), then calcTotalProb and {len(codes)} Pauli expectations",
                       "qubits": nq, "layers": layers, "gates": len(gates),
                       "l2": "the 16 MiB state fits in L2 (no flush: the reference's own size)",
                       "start": "each step from a device copy of the input state; wall time includes the host reads of the results"},
            "algorithmic_gbs": round(alg_bytes * args.steps / wall / 1e9, 1), "per_gate_kind": per_kind,
            "gpu_launches": int(launches1.value - launches0.value), "results": got[:3],
            "cpu_baseline": cpu, "clocks": clocks.summary()}
    if rank == 0:
        print(json.dumps(line), flush=True)


def run_blocks(args, world, rank, local, dist):
    """Per-target-set timing of one fused 5-qubit block on an FP32 register through the
    tensor-core kernel (`Circuit` API, impl = tc): ms per apply from CUDA events over
    `--steps` applies after `--warmup`.  `lines` is how many 128-byte lines one warp
    instruction would touch loading 32 groups row by row; the kernel stages its loads
    (16 lines) or its loads and stores (32 lines) through shared memory."""
    import ctypes as C
    from quest_gb300 import _lib
    from quest_gb300.fused import Circuit, StateVector32, IMPL_TC
    L = _lib.lib()
    _lib.check(L.qg_init(local))
    n = args.qubits
    if args.block_targets:
        sets = [[int(v) for v in ts.split(",")] for ts in args.block_targets.split(";")]
    else:
        sets = [[0, 1, 2, 3, 4], [1, 2, 3, 4, 5], [2, 3, 4, 5, 6], [0, 1, 7, 13, 19], [5, 6, 7, 8, 9],
                list(range(n - 5, n))]
    rng = np.random.default_rng(0x5155455354 + 7)
    s = StateVector32(n)
    s.init_zero()
    e0, e1 = C.c_void_p(), C.c_void_p()
    L.qg_event_create(C.byref(e0))
    L.qg_event_create(C.byref(e1))
    peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json"))) if os.path.exists(os.path.join(ROOT, "MEASURED_PEAKS.json")) else {}
    peak = peaks.get("hbm_gbs", 6800.0)
    rows = []
    for targs in sets:
        c = Circuit(n)
        c.add(targs, haar(32, rng))
        c.fuse(5)
        for _ in range(max(1, args.warmup)):
            c.apply(s, impl=IMPL_TC)
        L.qg_sync()
        L.qg_event_record(e0, None)
        for _ in range(args.steps):
            c.apply(s, impl=IMPL_TC)
        L.qg_event_record(e1, None)
        L.qg_sync()
        ms = C.c_float()
        L.qg_event_elapsed_ms(e0, e1, C.byref(ms))
        per = ms.value / args.steps
        ts = sorted(targs)

        def ins(v):
            for t in ts:
                lo = v & ((1 << t) - 1)
                v = ((v ^ lo) << 1) | lo
            return v
        lines = len({ins(r) >> 4 for r in range(32)})
        gbs = 2 * 8 * (1 << n) / per / 1e6
        rows.append({"targets": targs, "lines": lines, "ms": round(per, 4), "gbs": round(gbs, 1),
                     "frac_of_hbm": round(gbs / peak, 3)})
    flag = C.c_int(0)
    L.qg_tc_get_error_flag(C.byref(flag))
    s.free()
    line = {"metric": "per-block GB/s of the FP32 tensor-core block kernel, by target set", "value": rows[-1]["gbs"],
            "unit": "GB/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32 (3xTF32 tensor-core products)",
            "data": "synthetic (|0> state, seeded Haar 32x32 unitaries)",
            "config": {"workload": f"{n}-qubit FP32 statevector, one 5-qubit block per launch", "qubits": n,
                       "l2": "state larger than L2; no flush"},
            "blocks": rows, "tc_error_flag": flag.value, "hbm_peak_gbs": peak}
    if rank == 0:
        print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--qubits", type=int, default=30)
    ap.add_argument("--depth", type=int, default=20)
    ap.add_argument("--cpu-sample", type=int, default=45, help="gates of the circuit timed on the host CPU")
    ap.add_argument("--traffic", type=float, default=None, help="ncu DRAM bytes per dense launch, if captured")
    ap.add_argument("--config", default="plain", choices=["plain", "precision", "serve", "gates", "blocks", "expec", "dm", "c1"],
                    help="plain: the 30-qubit FP64 per-gate circuit (default); precision: FP32 fused blocks; "
                         "serve: request stream, served vs plain; gates: per-gate-kind timing (28 qubits); "
                         "blocks: one FP32 5-qubit block per target set; expec: 16 Pauli strings per call (28 qubits); "
                         "dm: the density-matrix method (14-qubit density matrix, 30 layers); "
                         "c1: the plain method (20 qubits, 10 layers, reductions) as wall time per circuit")
    ap.add_argument("--block-targets", default="", help="blocks: target sets, e.g. '0,1,2,3,4;5,6,7,8,9'")
    ap.add_argument("--requests", type=int, default=48)
    ap.add_argument("--min-qubits", type=int, default=8)
    ap.add_argument("--max-qubits", type=int, default=26)
    ap.add_argument("--hbm-budget-gib", type=int, default=64)
    ap.add_argument("--fuse-threads", type=int, default=8)
    ap.add_argument("--load", type=float, default=0.8, help="Poisson rate as a fraction of the plain path's capacity")
    ap.add_argument("--stall-s", type=float, default=120.0, help="serve: abort if no request finishes for this long")
    ap.add_argument("--fp64-products", default="fixed", choices=["fixed", "fp64"],
                    help="plain: general complex 2x2 products in block-floating fixed point (default) or IEEE FP64")
    ap.add_argument("--acc-qubits", type=int, default=28, help="precision form: qubits of the accuracy check (0 skips it)")
    ap.add_argument("--fused-impl", default="tc", choices=["tc", "simt"])
    ap.add_argument("--no-extras", action="store_true",
                    help="plain: leave out the short precision-form and serving summaries of the default line")
    args = ap.parse_args()
    world, rank, local, dist = dist_setup()
    if args.config == "serve":
        run_serve(args, world, rank, local, dist)
    elif args.config == "gates":
        run_gates(args, world, rank, local, dist)
    elif args.config == "blocks":
        run_blocks(args, world, rank, local, dist)
    elif args.config == "expec":
        run_expec(args, world, rank, local, dist)
    elif args.config == "c1":
        run_c1(args, world, rank, local, dist)
    elif args.config == "dm":
        args.dm_qubits = args.qubits if "--qubits" in sys.argv else 14
        args.dm_layers = args.depth if "--depth" in sys.argv else 30
        run_dm(args, world, rank, local, dist)
    elif args.config == "precision":
        if args.qubits == 30 and "--qubits" not in sys.argv:
            args.qubits = 32
        if "--depth" not in sys.argv:
            args.depth = 40
        run_precision(args, world, rank, local, dist)
    elif args.impl == "reference":
        run_reference(args, world, rank, dist)
    else:
        run_gb300(args, world, rank, local, dist)
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
