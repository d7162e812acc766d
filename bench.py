#!/usr/bin/env python
"""Benchmark of the distillation contraction engine on one GB300.

Workload (one step): the rho two-point at production size, Nev=100, Lt=64,
7 momenta |p|^2 <= 1, 3 polarisations (gamma_i (x) Phi at both ends), every
(t_src, t_sink) pair: 64*64*3*7 = 86,016 spin-summed correlator entries
("diagrams"), each a sum of 16 spin terms coef*Tr[(Phi(tf) tau_ab)^dag tau_cd Phi(ti)].
Inputs are seeded synthetic perambulators / elementals of those shapes, resident
in HBM for `value`; `e2e` re-copies them from pinned host memory every step.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--engine split|fp64]
  python bench.py --impl reference ...   # the oracle (CPU FP64, all host threads)
"""

import argparse
import ctypes
import json
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

NT, NEV, MAXP2, SEED = 64, 100, 1, 1001
METRIC = "diagrams/s @Nev=100,Lt=64: split-TC batched vs plain FP64, rel err ≤1e-9"
WORKLOAD = "rho two-point, Nev=100, Lt=64, 7 momenta |p|^2<=1, 3 polarisations, all 64x64 (t_src,t_sink)"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--engine", default="auto", choices=["auto", "split", "fp64"])
    ap.add_argument("--fp64-steps", type=int, default=1, help="timed steps of the plain FP64 engine (0 = skip)")
    ap.add_argument("--e2e-steps", type=int, default=8)
    ap.add_argument("--e2e-repeats", type=int, default=3, help="timed e2e sequences; the value is their median")
    ap.add_argument("--graph", type=int, default=1, help="time replays of the step recorded as a CUDA graph "
                    "(the eager calls are timed beside them); 0 = eager calls only")
    ap.add_argument("--tune", type=int, default=1, help="autotune the knobs on the first warm-up step")
    ap.add_argument("--tune-force", action="append", default=[], metavar="KNOB=VALUE",
                    help="pin an autotuner knob (e.g. trace_rows=1), repeatable")
    ap.add_argument("--cpu-seconds", type=float, default=12.0, help="target CPU-baseline sample time")
    ap.add_argument("--nt", type=int, default=None, help="time extent (default: the workload's; a smaller value "
                                                              "gives a small case of the same kernels, e.g. for ncu)")
    ap.add_argument("--nev", type=int, default=NEV)
    ap.add_argument("--configs", type=int, default=1, help="append one timed step of the pi pi (19 pairs), mixed "
                    "(Nev=128), profile-adjoint and reference-kernel workloads to the headline line (0 = skip)")
    ap.add_argument("--mixed-form", default="sets", choices=["sets", "pairs"],
                    help="mixed workload: one ctr_rhopi_sigmapi_sets call for the 27 pairs, or calls per pair")
    ap.add_argument("--pipi-form", default="sets", choices=["sets", "pairs"],
                    help="pi pi workload: one ctr_pipi_sets call for the 19 momentum sets, or one ctr_pipi per pair")
    ap.add_argument("--workload", default="rho", choices=["rho", "rho_small", "pipi", "mixed", "adjoint", "legacy_gpu", "elementals",
                             "fp64_peak", "mma_probe"],
                    help="rho: the headline rho two-point (Nev=100, Lt=64); rho_small: Nev=32, Lt=16 FP64; "
                         "pipi: pi pi I=0 diagram set, 19 momentum pairs; mixed: rho-pipi / sigma-pipi / "
                         "sigma loops at Nev=128, Lt=48, 27 momenta; adjoint: profile objective and gradient; "
                         "legacy_gpu: the reference's own rho kernel built for sm_103a beside both engines; "
                         "fp64_peak: cuBLAS DGEMM/ZGEMM rates; mma_probe: the split GEMMs' MMA schedules alone")
    return ap.parse_args()


# ----------------------------------------------------------------- helpers
def dist_setup():
    """Replicas: one process per GPU (torchrun env), NCCL on GPUs, gloo without
    them (the host-side logic is tested that way).  No collective touches the
    data path; the ranks only meet at barriers and in the max-over-ranks time."""
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if ws > 1:
        import torch.distributed as dist
        import torch
        if torch.cuda.is_available():
            torch.cuda.set_device(local)
            dist.init_process_group("nccl")
        else:
            dist.init_process_group("gloo")
    return ws, rank, local


def barrier(ws):
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()


def allmax(ws, x):
    """The largest x over the ranks (the slowest replica's time)."""
    if ws == 1:
        return x
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_value(ws, units_per_rank, seconds_max):
    """Whole-job throughput of ws replicas: every rank processed units_per_rank
    units, and the job took the slowest rank's time."""
    return ws * units_per_rank / seconds_max


class ClockSampler:
    """nvidia-smi sampling of SM clocks and throttle reasons during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (OSError, FileNotFoundError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"], "samples": 0}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 7:
                continue
            try:
                sm.append(float(parts[0]))
                mx.append(float(parts[1]))
            except ValueError:
                continue
            for n, v in zip(names, parts[3:7]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        sm.sort()
        return {"sm_mhz": sm[len(sm) // 2] if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks():
    try:
        return json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except (OSError, ValueError):
        return {}


def fp64_peak_tflops():
    """Measured FP64 peak on this GPU: cuBLAS DGEMM 8192^3 (best of 3), TFLOP/s."""
    import torch
    n = 8192
    a = torch.randn(n, n, dtype=torch.float64, device="cuda")
    b = torch.randn(n, n, dtype=torch.float64, device="cuda")
    torch.matmul(a, b)
    torch.cuda.synchronize()
    best = 1e9
    for _ in range(3):
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s.record()
        torch.matmul(a, b)
        e.record()
        e.synchronize()
        best = min(best, s.elapsed_time(e) / 1e3)
    del a, b
    return 2.0 * n ** 3 / best / 1e12


def workload(nt, nev):
    from contractions_code_scattering_gb300 import api, synth
    moms = synth.momenta(MAXP2)
    rows, coef, oi = api.rho_rows_for_momenta(len(moms))
    return moms, rows, coef, oi, 3 * len(moms)


def make_inputs(nt, nev, moms):
    import torch
    from contractions_code_scattering_gb300 import synth
    tau = synth.make_prop(nt, nev, seed=SEED, decay=0.35, backend="torch")
    phi = synth.make_phi_momenta_torch(nt, nev, moms, seed=SEED + 1)
    torch.cuda.synchronize()
    return tau, phi


def cpu_sample(tau, phi, rows, coef, nout, target_s, max_ti):
    """Time the oracle (reference chain order, every row recomputing its two
    products) on t_sink = 0 and the first k source times; returns
    (diagrams/s, cores, sample description, sample values [k, nout])."""
    import numpy as np
    from oracle import pyoracle as O
    k_probe = 1
    tau_row = tau[0].cpu().numpy()
    phi_h = phi.cpu().numpy()
    t0 = time.perf_counter()
    O.twosided_rows(tau_row, phi_h, rows, coef, 0, 0, k_probe)
    dt1 = time.perf_counter() - t0
    k = int(max(1, min(max_ti, target_s / max(dt1, 1e-3))))
    t0 = time.perf_counter()
    vals = O.twosided_rows(tau_row, phi_h, rows, coef, 0, 0, k)
    dt = time.perf_counter() - t0
    diag = k * nout
    cores = os.cpu_count() or 1
    return diag / dt, cores, "t_sink=0, t_src=0..%d, %d rows each (%d diagrams), %.1f s" % (k - 1, len(rows), diag, dt), vals, k


def rows_to_out(vals, oi, nout):
    import numpy as np
    out = np.zeros(vals.shape[:-1] + (nout,), np.complex128)
    for r, o in enumerate(oi):
        out[..., o] += vals[..., r]
    return out


# -------------------------------------------------------------- reference
def oracle_rho_rows(nmom, ico=0):
    """The workload's two-sided rows (op pair `ico`, one elemental per momentum,
    out index = momentum*3 + polarisation) from the oracle's own restatement of
    the reference tables (devTools/comb_rho.cpp), so that the reference arm
    loads nothing of the product library."""
    import numpy as np
    from oracle import tables as TB
    spin, _, coef = TB.rho_tables()
    rows, cf, oi = [], [], []
    for p in range(nmom):
        for r in range(ico * 48, ico * 48 + 48):
            s = spin[r]
            rows.append((s[0], s[1], s[2], s[3], p, p))
            cf.append(coef[r])
            oi.append(p * 3 + (r % 48) // 16)
    return np.array(rows, np.int16), np.array(cf, np.float32), np.array(oi, np.int32)


def host_sink_row(nt, nev, seed, decay=0.35):
    """tau(0, t) for t < nt on the host, with the workload's distribution: complex
    Gaussian N(0,1/Nev) blocks times exp(-decay*t), the t = 0 block
    gamma5-symmetrised.  [Nt, 4, 4, N, N] complex128."""
    import numpy as np
    from contractions_code_scattering_gb300 import synth
    rng = np.random.default_rng(seed)
    sd = np.sqrt(0.5 / nev)
    row = np.empty((nt, 4, 4, nev, nev), np.complex128)
    for t in range(nt):
        x = rng.normal(0.0, sd, (4, 4, nev, nev)) + 1j * rng.normal(0.0, sd, (4, 4, nev, nev))
        x *= np.exp(-decay * t)
        if t == 0:
            x = 0.5 * (x + synth._gamma5_adjoint_np(x))
        row[t] = x
    return row


def run_reference(args):
    """--impl reference: the reference's contraction algorithm on the host cores
    (the oracle's OpenMP FP64 restatement in the reference's chain order; the
    reference's own kernels are GPU-only).  Each step is one whole t_sink row of
    the workload: t_sink = 0 against all Nt source times, every one of the 21
    outputs (7 momenta x 3 polarisations), 16 spin rows each recomputing both of
    its products, as lib/calculate_rho_core.h does."""
    ws, rank = int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    from contractions_code_scattering_gb300 import synth
    from oracle import pyoracle as O
    nt, nev = args.nt or NT, args.nev
    moms = synth.momenta(MAXP2)
    rows, coef, oi = oracle_rho_rows(len(moms))
    nout = 3 * len(moms)
    row = host_sink_row(nt, nev, SEED)
    phi = synth.mom_stack(synth.make_phi_momenta(nt, nev, moms, seed=SEED + 1), moms)
    for _ in range(args.warmup):
        O.twosided_rows(row, phi, rows, coef, 0, 0, 1)
    times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        O.twosided_rows(row, phi, rows, coef, 0, 0, nt)
        times.append(time.perf_counter() - t0)
    ms = 1e3 * sum(times) / len(times)
    diag = nt * nout
    val = diag / (ms / 1e3)
    cores = os.cpu_count() or 1
    sample = ("t_sink=0 against all %d t_src, %d outputs x 16 spin rows each (%d diagrams) per step; the work is "
              "uniform per t_sink row" % (nt, nout, diag))
    print(json.dumps({
        "impl": "reference", "metric": METRIC, "value": val, "unit": "diagrams/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": WORKLOAD, "sample": sample, "l2": "inputs larger than L2"},
        "cpu_baseline": {"value": val, "unit": "diagrams/s", "cores": cores, "kind": "port", "sample": sample},
        "e2e": {"value": val, "unit": "diagrams/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }))


# -------------------------------------------------------------------- ours
def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
        return
    if args.tune_force:
        from contractions_code_scattering_gb300 import api as _api
        for kv in args.tune_force:
            knob, val = kv.split("=")
            _api.tune_force(knob, int(val))
    if args.workload != "rho":
        WORKLOADS[args.workload](args)
        return
    import numpy as np
    import torch
    from contractions_code_scattering_gb300 import _lib, api

    ws, rank, local = dist_setup()
    torch.cuda.set_device(local)
    api.device_init(local)
    nt, nev = args.nt or NT, args.nev
    moms, rows, coef, oi, nout = workload(nt, nev)
    diagrams = nt * nt * nout
    engine = args.engine
    if engine == "auto":
        engine = "split" if _split_available() else "fp64"

    tau, phi = make_inputs(nt, nev, moms)
    out = torch.empty((nt, nt, nout), dtype=torch.complex128, device="cuda")
    # a created stream (graphs cannot be recorded on the legacy default stream)
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)

    def step(eng, o=out):
        api.twosided(tau, phi, rows, coef, oi, nout, engine=eng, out=o)

    for w in range(args.warmup):
        if w == 0 and args.tune:
            api.tune_set_mode(1)  # the autotuner measures its knobs on this step's live data
        step(engine)
        if w == 0 and args.tune:
            torch.cuda.synchronize()
            api.tune_set_mode(0)
    torch.cuda.synchronize()
    barrier(ws)

    def timed(fn, k):
        torch.cuda.synchronize()
        barrier(ws)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        n0 = _lib.launch_count()
        e0.record(stream)
        for _ in range(k):
            fn()
        e1.record(stream)
        torch.cuda.synchronize()
        barrier(ws)
        return allmax(ws, e0.elapsed_time(e1) / 1e3), _lib.launch_count() - n0

    clocks = ClockSampler(local)
    clocks.start()
    # eager calls, with per-kernel CUDA-event timing (the roofline's source)
    _lib.timing_enable(True)
    t_eager, launches_eager = timed(lambda: step(engine), args.steps)
    report = _lib.timing_report()
    _lib.timing_enable(False)
    eager = {"ms_per_step": 1e3 * t_eager / args.steps, "value": replica_value(ws, diagrams * args.steps, t_eager),
             "gpu_launches": int(launches_eager)}
    graph_info = None
    if args.graph:
        # the same step recorded once as a CUDA graph and replayed
        with api.Graph(stream) as g:
            step(engine)
        g.launch(stream)
        nseg, nker, nbytes = g.info()
        elapsed, launches = timed(lambda: g.launch(stream), args.steps)
        graph_info = {"segments": nseg, "kernels_per_replay": nker, "device_bytes": nbytes,
                      "speedup_vs_eager": t_eager / elapsed}
        g.close()
    else:
        elapsed, launches = t_eager, launches_eager
    refined = int(_lib.lib().ctr_split_refined()) if engine == "split" else 0
    clk = clocks.stop()
    ms_per_step = 1e3 * elapsed / args.steps
    value = replica_value(ws, diagrams * args.steps, elapsed)
    tuned = api.tune_report()

    res_main = out.cpu().numpy()

    # Roofline of the dominant kernel.
    roof = roofline(engine, report, args.steps, nt, nev, len(moms))

    # End to end: every step copies its inputs (tau, Phi) from pinned host memory
    # and reads its correlators back.  The copies of step i+1 run on a copy
    # stream into a second device buffer while step i computes.  The first
    # step's inputs (inside the timed region too) arrive in t_sink row chunks,
    # and that step runs as row-range calls that each wait for their own rows
    # only, so its copy overlaps its compute as well (the reference stages tau
    # row by row, lib/contract.cpp:541-547, but synchronously).
    e2e = None
    if args.e2e_steps > 0:
        K = args.e2e_steps
        h_tau = torch.empty(tau.shape, dtype=tau.dtype, pin_memory=True)
        h_tau.copy_(tau)
        h_phi = torch.empty(phi.shape, dtype=phi.dtype, pin_memory=True)
        h_phi.copy_(phi)
        h_out = torch.empty((K,) + tuple(out.shape), dtype=out.dtype, pin_memory=True)
        buf_tau, buf_phi = [tau, torch.empty_like(tau)], [phi, torch.empty_like(phi)]
        cs = torch.cuda.Stream()
        copied = [torch.cuda.Event() for _ in range(2)]
        freed = [torch.cuda.Event() for _ in range(2)]
        # the copy alone, for reference (untimed by the e2e figure)
        c0, c1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        c0.record(cs)
        with torch.cuda.stream(cs):
            buf_tau[1].copy_(h_tau, non_blocking=True)
        c1.record(cs)
        torch.cuda.synchronize()
        h2d_alone = c0.elapsed_time(c1) / 1e3
        # copy-stream events around each step's input copy: how long the copies
        # take while the previous step computes
        copy_ev = []

        def load(b):
            with torch.cuda.stream(cs):
                ca, cb = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                ca.record(cs)
                buf_tau[b].copy_(h_tau, non_blocking=True)
                buf_phi[b].copy_(h_phi, non_blocking=True)
                copied[b].record(cs)
                cb.record(cs)
                copy_ev.append((ca, cb))

        graphs = None
        if args.graph:
            # one recorded step per input buffer (recorded before the timed region)
            graphs = []
            for b in range(2):
                with api.Graph(stream) as gb:
                    api.twosided(buf_tau[b], buf_phi[b], rows, coef, oi, nout, engine=engine, out=out)
                graphs.append(gb)

        def e2e_run():
            """K pipelined steps from host inputs to host results; seconds per step."""
            torch.cuda.synchronize()
            barrier(ws)
            copy_ev.clear()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            cs.wait_event(e0)
            # step 0: Phi, then tau in chunks of RC t_sink rows, each with its event
            RC = 2
            chunk_ev = []
            with torch.cuda.stream(cs):
                buf_phi[0].copy_(h_phi, non_blocking=True)
                for r0 in range(0, nt, RC):
                    buf_tau[0][r0:r0 + RC].copy_(h_tau[r0:r0 + RC], non_blocking=True)
                    ev = torch.cuda.Event()
                    ev.record(cs)
                    chunk_ev.append(ev)
            if K > 1:
                load(1)
            for c, r0 in enumerate(range(0, nt, RC)):
                r1 = min(nt, r0 + RC)
                stream.wait_event(chunk_ev[c])
                api.twosided(buf_tau[0][r0:r1], buf_phi[0], rows, coef, oi, nout, engine=engine,
                             tf_range=(r0, r1), out=out[r0:r1])
            freed[0].record(stream)
            h_out[0].copy_(out, non_blocking=True)
            for i in range(1, K):
                b = i % 2
                if i + 1 < K:
                    cs.wait_event(freed[1 - b])
                    load(1 - b)
                stream.wait_event(copied[b])
                if graphs:
                    graphs[b].launch(stream)
                else:
                    api.twosided(buf_tau[b], buf_phi[b], rows, coef, oi, nout, engine=engine, out=out)
                freed[b].record(stream)
                h_out[i].copy_(out, non_blocking=True)
            e1.record(stream)
            torch.cuda.synchronize()
            return allmax(ws, e0.elapsed_time(e1) / 1e3) / K

        runs, copies = [], []
        for _ in range(max(1, args.e2e_repeats)):
            runs.append(e2e_run())
            copies.append([round(ca.elapsed_time(cb), 1) for ca, cb in copy_ev])
        te = sorted(runs)[len(runs) // 2]
        # every e2e step (row-range calls for step 0, replays after) gives the timed step's result
        e2e_same = bool(all(np.array_equal(h_out[i].numpy(), res_main) for i in range(K)))
        e2e = {"value": replica_value(ws, diagrams, te), "unit": "diagrams/s",
               "h2d_bytes_per_step": int(h_tau.numel() * 16 + h_phi.numel() * 16),
               "d2h_bytes_per_step": int(out.numel() * 16), "ms_per_step": 1e3 * te,
               "pipelining": "inputs of step i+1 copied on a second stream while step i computes; step 0's "
                             "tau in 2-row chunks, each row range computed once its rows arrived", "steps": K,
               "graph": bool(args.graph), "bitwise_equal_to_value_step": e2e_same,
               "repeats": len(runs), "value_is": "median of the repeats",
               "ms_per_step_runs": [round(1e3 * r, 2) for r in runs], "worst_ms_per_step": 1e3 * max(runs),
               "h2d_tau_alone_ms": 1e3 * h2d_alone, "h2d_tau_alone_gbs": h_tau.numel() * 16 / h2d_alone / 1e9,
               "h2d_overlapped_ms": copies}
        if graphs:
            for gb in graphs:
                gb.close()
        del h_tau, h_phi, h_out, buf_tau, buf_phi

    # Plain FP64 engine on the same workload (the metric's comparison arm), after the
    # e2e leg, so that its long full-power run does not precede that measurement.
    fp64 = None
    if engine == "split" and args.fp64_steps > 0:
        out64 = torch.empty_like(out)
        step("fp64", out64)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(args.fp64_steps):
            step("fp64", out64)
        e1.record(stream)
        torch.cuda.synchronize()
        t64 = e0.elapsed_time(e1) / 1e3 / args.fp64_steps
        r64 = out64.cpu().numpy()
        err = np.abs(res_main - r64) / np.maximum(np.abs(r64), 1e-300)
        fp64 = {"value": diagrams / t64, "unit": "diagrams/s", "ms_per_step": 1e3 * t64,
                "split_speedup": (diagrams / t64 and value / ws / (diagrams / t64)),
                "split_vs_fp64_rel_err": {"max": float(err.max()), "median": float(np.median(err)),
                                          "p99": float(np.quantile(err, 0.99)),
                                          "max_over_maxabs": float(np.abs(res_main - r64).max() / np.abs(r64).max())}}
        del out64

    # CPU baseline (the oracle, reference chain order) on a bounded sample; the
    # same sample also checks the GPU result at full size.
    cpu = None
    parity = None
    if rank == 0 and args.cpu_seconds > 0:
        rate, cores, sample, vals, k = cpu_sample(tau, phi, rows, coef, nout, args.cpu_seconds, nt)
        ref = rows_to_out(vals, oi, nout)
        got = res_main[0, :k]
        rel = np.abs(got - ref) / np.maximum(np.abs(ref), 1e-300)
        parity = {"entries": int(ref.size), "max_rel_err": float(rel.max()), "median_rel_err": float(np.median(rel)),
                  "max_err_over_maxabs": float(np.abs(got - ref).max() / np.abs(ref).max())}
        cpu = {"value": rate, "unit": "diagrams/s", "cores": cores, "kind": "port", "sample": sample}

    if rank != 0:
        return
    line = {
        "metric": METRIC, "value": value, "unit": "diagrams/s", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64" if engine == "fp64" else "f64-equivalent (bf16 x5 balanced 9-bit slices, fp32 acc)",
        "data": "synthetic (seeded tau/Phi: complex Gaussian N(0,1/Nev) x exp(-0.35|dt|), gamma5-hermitian; Phi(-p)=Phi(p)^dagger)",
        "config": {"workload": WORKLOAD, "engine": engine, "nev": nev, "lt": nt, "momenta": len(moms),
                   "diagrams_per_step": diagrams, "l2": "inputs larger than L2 (tau 10.5 GB)",
                   "parallelism": "replicas" if ws > 1 else "single GPU"},
        "roofline": roof, "cpu_baseline": cpu, "e2e": e2e, "clocks": clk, "gpu_launches": int(launches),
        "graph": graph_info, "eager": eager, "autotune": tuned,
        "kernels": {k: {"launches": v[0], "ms": v[2]} for k, v in report.items()},
        "fp64_engine": fp64, "parity_vs_oracle_sample": parity,
        "split_refined_entries_per_step": refined,
    }
    if args.configs and ws == 1:
        # the other chain configurations, each one timed step of its full workload
        del tau, phi, out
        torch.cuda.synchronize()
        line["configs"] = {}
        for name, fn in (("pipi", pipi_block), ("mixed", mixed_block), ("adjoint", adjoint_block),
                         ("legacy_gpu", legacy_block)):
            try:
                line["configs"][name] = fn(args)
            except Exception as e:  # recorded, so that the headline line still prints
                line["configs"][name] = {"error": "%s: %s" % (type(e).__name__, str(e)[:300])}
            torch.cuda.set_stream(stream)
    print(json.dumps(line))


def _split_available():
    try:
        from contractions_code_scattering_gb300 import _lib
        return bool(_lib.lib().ctr_split_available())
    except Exception:
        return False


def roofline(engine, report, steps, nt, nev, nmom):
    """Dominant kernel's achieved rate against its pipe's measured peak."""
    n3 = float(nev) ** 3
    prods = nt * nt * nmom * 32  # 16 source-side + 16 sink-side block products per (tf, ti, p)
    if engine == "fp64":
        launches, _, ms = report.get("zgemm_f64", (0, 0, 0.0))
        if not launches or ms <= 0:
            return None
        flops = steps * prods * 8.0 * n3
        per_launch_flops = flops / launches
        achieved = per_launch_flops / (ms / launches / 1e3) / 1e12
        peak = fp64_peak_tflops()
        return {"kernel": "zgemm_f64", "bound": "fp64 pipe", "achieved": achieved, "peak": peak,
                "unit": "TFLOP/s", "frac": achieved / peak, "traffic": None,
                "peak_source": "measured in bench.py: cuBLAS DGEMM 8192^3 (MEASURED_PEAKS.json has no FP64 figure)",
                "algorithmic": "8*Nev^3 flops per block product, 32 products per (t_sink, t_src, momentum)"}
    launches, _, ms = report.get("split_gemm", (0, 0, 0.0))
    if not launches or ms <= 0:
        return None
    pk = measured_peaks()
    peak = pk.get("bf16_tflops", 1924.8)
    mma_flops = steps * prods * 8.0 * n3 * 15 * (112.0 / 100.0)
    achieved = mma_flops / launches / (ms / launches / 1e3) / 1e12
    # DRAM traffic per launch: the ncu capture of one launch at Nt=8 (64 pairs, 7 momenta, Nev=100)
    # read 0.390 GB and wrote 1.093 GB, i.e. 23.2 MB per (t_sink, t_src) pair; scaled by the
    # pairs one launch processes here (both GEMMs of a batch have the same output size)
    pairs_per_launch = steps * nt * nt * 2.0 / launches
    traffic = 23.17e6 * pairs_per_launch * (nmom / 7.0) if nev == 100 else None
    return {"kernel": "split_gemm", "bound": "tensor", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
            "frac": achieved / peak, "traffic": traffic,
            "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum of one launch at Nt=8, scaled "
                              "by pairs per launch (the split_gemm rho Nt=8 ncu summary under profiles/)",
            "peak_source": "MEASURED_PEAKS.json bf16_tflops (burst)" if "bf16_tflops" in pk else "fallback 1924.8",
            "fp64_equivalent_tflops": achieved / 15 / 1.12,
            "algorithmic": "15 bf16 slice-pair products x 8*Nev^3 flops (K padded 100->112) per block product"}


# ------------------------------------------------------- other workloads
# The configurations other than the headline: each prints one JSON line with
# its own metric; the plain FP64 engine is timed on a stated subset where a
# full FP64 step would take minutes, and the per-entry errors of the split
# engine are measured against it there.
def _timed(fn, steps, warmup):
    import torch
    from contractions_code_scattering_gb300 import _lib
    for _ in range(warmup):
        fn()
    torch.cuda.synchronize()
    _lib.timing_enable(True)
    _lib.split_flops(reset=True)
    _lib.gram_flops(reset=True)
    n0 = _lib.launch_count()
    stream = torch.cuda.current_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(steps):
        fn()
    e1.record(stream)
    torch.cuda.synchronize()
    launches = _lib.launch_count() - n0
    rep = _lib.timing_report()
    _lib.timing_enable(False)
    kern = {k: {"launches": v[0], "ms": v[2]} for k, v in rep.items()}
    mma, prods = _lib.split_flops()
    kern["_split_work"] = {"mma_flops": mma / steps, "block_products": prods / steps, "steps": steps}
    gmma, gtr = _lib.gram_flops()
    kern["_gram_work"] = {"mma_flops": gmma / steps, "traces": gtr / steps, "steps": steps}
    return e0.elapsed_time(e1) / 1e3 / steps, launches, kern


def chain_roofline(kern, nev):
    """split_gemm_hp (the chain engine's block GEMMs) against the measured BF16 peak:
    executed BF16 MMA flops (the library's count, padding included) and the
    FP64-equivalent rate of the block products (8 Nev^3 each), per step."""
    w = kern.get("_split_work", {})
    g = kern.get("split_gemm_hp")
    if not g or not w.get("mma_flops"):
        return None
    t = g["ms"] / 1e3 / max(1, w.get("steps", 1))
    pk = measured_peaks()
    peak = pk.get("bf16_tflops", 1924.8)
    achieved = w["mma_flops"] / t / 1e12
    return {"kernel": "split_gemm_hp", "bound": "tensor", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
            "frac": achieved / peak, "fp64_equivalent_tflops": w["block_products"] * 8.0 * nev ** 3 / t / 1e12,
            "gemm_ms_per_step": 1e3 * t, "traffic": None,
            "peak_source": "MEASURED_PEAKS.json bf16_tflops (burst)" if "bf16_tflops" in pk else "fallback 1924.8",
            "algorithmic": "executed: 21 bf16 slice-pair products x 8 M N K per tile (the library's launch count); "
                           "FP64-equivalent: 8 Nev^3 per complex block product"}


def gram_roofline(kern, nev):
    """gram_gemm (the closing traces of the momentum-set calls as Gram products)
    against the measured BF16 peak: executed BF16 MMA flops (the library's count,
    padding included) and the FP64-equivalent rate of the traces (8 Nev^2 each)."""
    w = kern.get("_gram_work", {})
    g = kern.get("gram_gemm")
    if not g or not w.get("mma_flops"):
        return None
    t = g["ms"] / 1e3 / max(1, w.get("steps", 1))
    pk = measured_peaks()
    peak = pk.get("bf16_tflops", 1924.8)
    achieved = w["mma_flops"] / t / 1e12
    return {"kernel": "gram_gemm", "bound": "tensor", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
            "frac": achieved / peak, "fp64_equivalent_tflops": w["traces"] * 8.0 * nev ** 2 / t / 1e12,
            "gemm_ms_per_step": 1e3 * t, "traces_per_step": w["traces"],
            "peak_source": "MEASURED_PEAKS.json bf16_tflops (burst)" if "bf16_tflops" in pk else "fallback 1924.8",
            "algorithmic": "executed: 21 bf16 slice-pair products x 8 M N K per tile (the library's launch count); "
                           "FP64-equivalent: 8 Nev^2 per closing trace"}


def _errs(a, b):
    import numpy as np
    rel = np.abs(a - b) / np.maximum(np.abs(b), 1e-300)
    return {"max": float(rel.max()), "median": float(np.median(rel)), "p99": float(np.quantile(rel, 0.99)),
            "max_over_maxabs": float(np.abs(a - b).max() / np.abs(b).max()), "entries": int(rel.size)}


def _neg(p):
    return tuple(-c for c in p)


def run_rho_small(args):
    """Nev=32, Lt=16 rho two-point at p=0 (gamma_i x Phi at both ends), FP64 engine,
    against the oracle in full (16 x 16 x 3 = 768 diagrams)."""
    import numpy as np
    import torch
    from contractions_code_scattering_gb300 import api, synth
    from oracle import pyoracle as O
    api.device_init(0)
    nt, nev = 16, 32
    prop = synth.make_prop(nt, nev, seed=SEED, decay=0.35)
    rng = np.random.default_rng(SEED + 1)
    mom5 = np.ascontiguousarray(np.stack([synth.make_phi_hermitian(nt, nev, SEED + 2)] +
                                         [synth.make_phi_random(nt, nev, rng) for _ in range(4)], axis=1))
    dp, dm = torch.from_numpy(prop).cuda(), torch.from_numpy(mom5).cuda()
    stream = torch.cuda.Stream()  # a created stream, so that the step can be recorded as a graph
    torch.cuda.set_stream(stream)
    res = {}
    for eng in ("fp64", "split"):
        out = torch.empty((nt, nt, 16, 3), dtype=torch.complex128, device="cuda")
        if args.tune:
            api.tune_set_mode(1)
            api.run_contract_rho(dp, dm, engine=eng, out=out)
            torch.cuda.synchronize()
            api.tune_set_mode(0)
        t, launches, kern = _timed(lambda: api.run_contract_rho(dp, dm, engine=eng, out=out), args.steps, args.warmup)
        got = out.cpu().numpy()
        res[eng] = {"value": nt * nt * 3 / t, "ms_per_step": 1e3 * t, "gpu_launches": launches}
        if args.graph:
            with api.Graph(stream) as g:
                api.run_contract_rho(dp, dm, engine=eng, out=out)
            tg, lg, _ = _timed(lambda: g.launch(stream), args.steps, args.warmup)
            same = bool(np.array_equal(out.cpu().numpy(), got))
            res[eng]["graph"] = {"value": nt * nt * 3 / tg, "ms_per_step": 1e3 * tg, "gpu_launches": lg,
                                 "speedup_vs_eager": t / tg, "segments": g.info()[0], "bitwise_equal_to_eager": same}
            g.close()
        res[eng]["out"] = got[:, :, 0, :]
    t0 = time.perf_counter()
    ref = O.rho(prop, mom5)[:, :, 0, :]
    tcpu = time.perf_counter() - t0
    line = {"workload": "rho_small", "metric": "diagrams/s @Nev=32,Lt=16 (rho, p=0, 3 polarisations)",
            "unit": "diagrams/s", "diagrams_per_step": nt * nt * 3,
            "fp64": {k: v for k, v in res["fp64"].items() if k != "out"},
            "split": {k: v for k, v in res["split"].items() if k != "out"},
            "fp64_vs_oracle": _errs(res["fp64"]["out"], ref), "split_vs_oracle": _errs(res["split"]["out"], ref),
            "cpu_baseline": {"value": nt * nt * 768 / 16 / tcpu, "unit": "diagrams/s", "cores": os.cpu_count(),
                             "kind": "port", "sample": "all 16 x 16 pairs, all 48 outputs (768 spin rows)"},
            "autotune": api.tune_report()}
    print(json.dumps(line))


def run_pipi(args):
    """pi pi I=0 diagram set (square, double triangle, horizontal double triangle, star,
    fish) for the 19 momentum pairs (p, -p), |p|^2 <= 2, all 64 x 64 pairs, Nev=100.
    --pipi-form sets (default): all 19 sets in one ctr_pipi_sets call per step;
    pairs: one ctr_pipi call per momentum pair."""
    print(json.dumps(pipi_block(args, full=True)))


def _entry_gate(got, ref, rows_abs, tol):
    """Per-entry errors of got against ref, and how many entries miss
    |err| <= tol |ref| + 2^-44 (sum of the magnitudes of the entry's rows)."""
    import numpy as np
    err = np.abs(got - ref)
    rel = err / np.maximum(np.abs(ref), 1e-300)
    bound = tol * np.abs(ref) + 2.0 ** -44 * rows_abs
    return {"entries": int(ref.size), "max_rel": float(rel.max()), "median_rel": float(np.median(rel)),
            "outside_gate": int(np.count_nonzero(err > bound)), "gate": "%.0e |ref| + 2^-44 rows_abs" % tol}


def _pipi_rows_abs(d):
    """Row magnitudes of the oracle's I=0 pi pi entries (weights of lib/contract_kernels_pipi.cu:463-478)."""
    import numpy as np
    a = lambda x: np.abs(x).sum(-1)
    return np.stack([a(d["square"]) / 3, a(d["dtri"]) / 3, a(d["star"][0]) * a(d["star"][1]),
                     a(d["fish"][0]) * a(d["fish"][1]), 5 * a(d["dtri_hor"]) / 3], axis=-1)


def pipi_block(args, full=False):
    """The pi pi I=0 set over 19 momentum pairs at Nev=100, Lt=64 (one ctr_pipi_sets call
    per step, or one ctr_pipi call per pair with --pipi-form pairs): eager step with
    per-kernel times, the step recorded as a CUDA graph and replayed, the block GEMM's
    roofline, the FP64 engine on a subset, and an oracle sample that is also the CPU
    baseline of this configuration."""
    import numpy as np
    import torch
    from contractions_code_scattering_gb300 import _lib, api, synth
    api.device_init(0)
    nt, nev = args.nt or 64, 100
    moms = synth.momenta(2)
    idx = {p: k for k, p in enumerate(moms)}
    tau = synth.make_prop(nt, nev, seed=SEED, decay=0.35, backend="torch")
    diag = api.prop_diag(tau)
    phi_all = synth.make_phi_momenta_torch(nt, nev, moms, seed=SEED + 1).contiguous()
    P = {p: phi_all[:, idx[p]].contiguous() for p in moms}
    pairs = [(p, _neg(p)) for p in moms]
    sets = [(idx[a], idx[b], idx[a], idx[b]) for a, b in pairs]
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    form = args.pipi_form
    refined = [0]

    def step(engine, rows=None, plist=None, out=None):
        tr = rows if rows is not None else (0, nt)
        tb = tau[tr[0]:tr[1]]
        refined[0] = 0
        if form == "sets":
            sl = sets if plist is None else [sets[pairs.index(p)] for p in plist]
            o = api.run_contract_pipi_sets(tb, diag, phi_all, sl, 0, engine=engine, tf_range=tr, out=out)
            refined[0] += int(_lib.lib().ctr_split_refined()) if engine == "split" else 0
            return o
        res = []
        for a, b in (pairs if plist is None else plist):
            res.append(api.run_contract_pipi(tb, diag, P[a], P[b], P[a], P[b], 0, engine=engine, tf_range=tr))
            refined[0] += int(_lib.lib().ctr_split_refined()) if engine == "split" else 0
        return torch.stack(res)

    steps, warm = (args.steps, args.warmup) if full else (1, 1)
    out = torch.empty((len(sets), nt, nt, 5), dtype=torch.complex128, device="cuda")
    if args.tune:  # the autotuner measures the GEMM tile walks on one untimed step
        api.tune_set_mode(1)
        step("split", out=out if form == "sets" else None)
        torch.cuda.synchronize()
        api.tune_set_mode(0)
    t, launches, kern = _timed(lambda: step("split", out=out if form == "sets" else None), steps, warm)
    refined_step = refined[0]
    diagrams = nt * nt * len(pairs) * 5
    res = {"workload": "pipi I=0 set, Nev=100, Lt=64, 19 momentum pairs (p,-p) |p|^2<=2, all 64x64 (t_src,t_sink)",
           "metric": "diagrams/s @Nev=100,Lt=64: pi pi I=0 set, 19 momentum pairs, split-TC",
           "value": diagrams / t, "unit": "diagrams/s", "ms_per_step": 1e3 * t, "steps": steps, "warmup": warm,
           "form": form, "diagrams_per_step": diagrams, "gpu_launches": launches,
           "split_refined_entries_per_step": refined_step, "roofline": chain_roofline(kern, nev),
           "kernels": {k: v for k, v in kern.items() if not k.startswith("_")},
           "autotune": {k: v for k, v in api.tune_report().items() if k.startswith("split_gemm.order|hp")}}
    got = (out if form == "sets" else step("split")).cpu().numpy()
    if form == "sets":
        # the same step recorded once as a CUDA graph and replayed
        with api.Graph(stream) as g:
            step("split", out=out)
        g.launch(stream)
        torch.cuda.synchronize()
        nseg, nker, nbytes = g.info()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        g.launch(stream)
        e1.record(stream)
        torch.cuda.synchronize()
        tg = e0.elapsed_time(e1) / 1e3
        same = bool(np.array_equal(out.cpu().numpy(), got))
        g.close()
        res["graph"] = {"value": diagrams / tg, "ms_per_step": 1e3 * tg, "segments": nseg, "kernels_per_replay": nker,
                        "device_bytes": nbytes, "speedup_vs_eager": t / tg, "bitwise_equal_to_eager": same}
    # the plain FP64 engine and per-entry errors on a subset: one momentum pair, t_sink 0..3
    sub_pairs, sub_rows = [((1, 0, 0), (-1, 0, 0))], (0, 4)
    sub_diag = (sub_rows[1] - sub_rows[0]) * nt * len(sub_pairs) * 5
    t64, _, _ = _timed(lambda: step("fp64", sub_rows, plist=sub_pairs), 1, 1)
    b = step("fp64", sub_rows, plist=sub_pairs).cpu().numpy()[0]
    a = got[sets.index(sets[pairs.index(sub_pairs[0])])][sub_rows[0]:sub_rows[1]]
    res["fp64_subset"] = {"sample": "momentum pair (1,0,0)/(-1,0,0), t_sink 0..3, all t_src (%d diagrams)" % sub_diag,
                          "fp64_diagrams_per_s": sub_diag / t64,
                          "split_speedup": (sub_diag / t64) and (diagrams / t) / (sub_diag / t64),
                          "split_vs_fp64_rel_err": _errs(a, b)}
    # oracle sample (also this configuration's CPU baseline): the same pair, t_sink 0, t_src 0..7;
    # these entries involve only time slices below 8, so the oracle runs on that sub-lattice
    try:
        from oracle import pyoracle as O
        k8 = min(8, nt)
        p1, p2 = sub_pairs[0]
        sub_prop = tau[:k8, :k8].cpu().numpy()
        ph = {p: P[p][:k8].cpu().numpy() for p in (p1, p2)}
        t0 = time.perf_counter()
        d = O.pipi_row(sub_prop, ph[p1], ph[p2], ph[p1], ph[p2], 0, 0)
        tcpu = time.perf_counter() - t0
        k = pairs.index(sub_pairs[0])
        res["vs_oracle"] = {"sample": "pair (1,0,0)/(-1,0,0), t_sink 0, t_src 0..%d" % (k8 - 1),
                            "split": _entry_gate(got[k][0, :k8], d["corr"], _pipi_rows_abs(d), 1e-9),
                            "fp64": _entry_gate(b[0, :k8], d["corr"], _pipi_rows_abs(d), 1e-12)}
        res["cpu_baseline"] = {"value": k8 * 5 / tcpu, "unit": "diagrams/s", "cores": os.cpu_count(), "kind": "port",
                               "sample": "the oracle sample above (%d entries, reference chain order)" % (k8 * 5)}
    except Exception as e:  # the oracle library is not built
        res["vs_oracle"] = {"unavailable": str(e)[:200]}
    del tau, diag, phi_all, P, out
    torch.cuda.synchronize()
    return res


def run_mixed(args):
    """Mixed cross-correlator batch at Nev=128, Lt=48, decay 0.25: for each of the 27
    momenta |p|^2 <= 3, rho -> pi pi (3 polarisations x 4 operators) and sigma -> pi pi
    (triangle x 2 operators, horizontal fish) with the pion pair (p, -p), plus the
    sigma one-fish loops; split engine.  --mixed-form sets (default): one
    ctr_rhopi_sigmapi_sets call for the 27 pairs; pairs: per-pair ctr_rhopi / ctr_sigmapi."""
    print(json.dumps(mixed_block(args, full=True)))


def mixed_block(args, full=False):
    import numpy as np
    import torch
    from contractions_code_scattering_gb300 import _lib, api, synth
    api.device_init(0)
    nt, nev = args.nt or 48, 128
    moms = synth.momenta(3)
    idx = {p: k for k, p in enumerate(moms)}
    tau = synth.make_prop(nt, nev, seed=SEED, decay=0.25, backend="torch")
    diag = api.prop_diag(tau)
    phi_all = synth.make_phi_momenta_torch(nt, nev, moms, seed=SEED + 1).contiguous()
    P = {p: phi_all[:, idx[p]].contiguous() for p in moms}
    g = torch.Generator(device="cuda")
    g.manual_seed(SEED + 2)
    sd = float(np.sqrt(0.5 / nev))
    ops = torch.complex(torch.randn((nt, 5, nev, nev), generator=g, device="cuda", dtype=torch.float64) * sd,
                        torch.randn((nt, 5, nev, nev), generator=g, device="cuda", dtype=torch.float64) * sd)
    mom5 = ops.contiguous()
    mom2 = ops[:, :2].contiguous()
    sets = [(idx[p], idx[_neg(p)]) for p in moms]
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    form = args.mixed_form
    refined = [0]

    def step(engine, plist=moms, rows=None):
        """[rhopi (set, idir, rows, Nt, 4), triangle (set, rows, Nt, 2), hor_fish (set, Nt)], loops (2, Nt)"""
        tr = rows if rows is not None else (0, nt)
        tb = tau[tr[0]:tr[1]]
        refined[0] = 0
        if form == "sets":
            sl = [sets[moms.index(p)] for p in plist]
            o = api.run_contract_rhopi_sigmapi_sets(tb, diag, phi_all, sl, mom5, mom2, engine=engine, tf_range=tr)
            refined[0] += int(_lib.lib().ctr_split_refined()) if engine == "split" else 0
            res = [o["rhopi"], o["triangle"], o["hor_fish"]]
        else:
            rp, tri, hf = [], [], []
            for p in plist:
                rp.append(torch.stack([api.run_contract_rhopi(tb, diag, P[p], P[_neg(p)], mom5, idir, engine=engine,
                                                              tf_range=tr) for idir in range(3)]))
                refined[0] += int(_lib.lib().ctr_split_refined()) if engine == "split" else 0
                h, t = api.run_contract_sigmapi(tb, diag, P[p], P[_neg(p)], mom2, engine=engine, tf_range=tr)
                refined[0] += int(_lib.lib().ctr_split_refined()) if engine == "split" else 0
                tri.append(t)
                hf.append(h)
            res = [torch.stack(rp), torch.stack(tri), torch.stack(hf)]
        loops = torch.stack([api.run_contract_loop_unity(diag, mom2[:, k].contiguous(), engine=engine)
                             for k in range(2)])
        return res + [loops]

    steps, warm = (args.steps, args.warmup) if full else (1, 1)
    holder = {}
    if args.tune:  # the autotuner measures the GEMM tile walks on one untimed step
        api.tune_set_mode(1)
        step("split")
        torch.cuda.synchronize()
        api.tune_set_mode(0)
    t, launches, kern = _timed(lambda: holder.__setitem__("r", step("split")), steps, warm)
    refined_step = refined[0]
    diagrams = nt * nt * len(moms) * (12 + 2) + nt * len(moms) + 2 * nt
    res = {"workload": "mixed: rho->pipi (3 polarisations x 4 operators) + sigma->pipi (triangle x 2, horizontal "
                       "fish) for 27 pion pairs (p,-p) |p|^2<=3, + 2 sigma loops; Nev=128, Lt=48",
           "metric": "diagrams/s @Nev=128,Lt=48: rho-pipi + sigma-pipi + sigma loops, 27 momenta, split-TC",
           "value": diagrams / t, "unit": "diagrams/s", "ms_per_step": 1e3 * t, "steps": steps, "warmup": warm,
           "form": form, "diagrams_per_step": diagrams, "gpu_launches": launches,
           "split_refined_entries_per_step": refined_step, "roofline": chain_roofline(kern, nev),
           "gram_roofline": gram_roofline(kern, nev),
           "kernels": {k: v for k, v in kern.items() if not k.startswith("_")},
           "autotune": {k: v for k, v in api.tune_report().items()
                        if k.startswith("split_gemm.order|hp") or k.startswith("chains.trace_form")}}
    got = [x.cpu().numpy() for x in holder["r"]]
    if form == "sets":
        with api.Graph(stream) as gr:
            holder["g"] = step("split")
        gr.launch(stream)
        torch.cuda.synchronize()
        nseg, nker, nbytes = gr.info()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        gr.launch(stream)
        e1.record(stream)
        torch.cuda.synchronize()
        tg = e0.elapsed_time(e1) / 1e3
        same = all(np.array_equal(a.cpu().numpy(), b) for a, b in zip(holder["g"], got))
        gr.close()
        res["graph"] = {"value": diagrams / tg, "ms_per_step": 1e3 * tg, "segments": nseg, "kernels_per_replay": nker,
                        "device_bytes": nbytes, "speedup_vs_eager": t / tg, "bitwise_equal_to_eager": same}
    # FP64 engine on a subset: momentum (1,1,1), t_sink 0..3, all t_src
    sub, rows = [(1, 1, 1)], (0, 4)
    k1 = moms.index(sub[0])
    sub_diag = (rows[1] - rows[0]) * nt * 14 + nt + 2 * nt
    t64, _, _ = _timed(lambda: holder.__setitem__("f", step("fp64", sub, rows)), 1, 1)
    f = [x.cpu().numpy() for x in holder["f"]]
    a = np.concatenate([got[0][k1][:, rows[0]:rows[1]].ravel(), got[1][k1][rows[0]:rows[1]].ravel(),
                        got[2][k1].ravel(), got[3].ravel()])
    b = np.concatenate([f[0][0].ravel(), f[1][0].ravel(), f[2][0].ravel(), f[3].ravel()])
    res["fp64_subset"] = {"sample": "momentum (1,1,1), t_sink 0..3, all t_src (%d diagrams)" % sub_diag,
                          "fp64_diagrams_per_s": sub_diag / t64,
                          "split_speedup": (diagrams / t) / (sub_diag / t64), "split_vs_fp64_rel_err": _errs(a, b)}
    # oracle sample (also this configuration's CPU baseline): rho -> pi pi idir 0 and the
    # triangle for (1,1,1), t_sink 0, t_src 0..3 (sub-lattice t < 4)
    try:
        from oracle import pyoracle as O
        k4 = min(4, nt)
        p1, p2 = P[sub[0]][:k4].cpu().numpy(), P[_neg(sub[0])][:k4].cpu().numpy()
        sp = tau[:k4, :k4].cpu().numpy()
        m5, m2 = mom5[:k4].cpu().numpy(), mom2[:k4].cpu().numpy()
        t0 = time.perf_counter()
        r1, c1 = O.rhopi_row(sp, p1, p2, m5, 0, 0)
        r2, c2 = O.sigmapi_triangle_row(sp, p1, p2, m2, 0)
        tcpu = time.perf_counter() - t0
        ab1 = np.abs(r1).reshape(k4, 4, 64).sum(-1)
        ab2 = np.abs(r2).reshape(k4, 2, 64).sum(-1)
        res["vs_oracle"] = {"sample": "(1,1,1): rho->pipi idir 0 and triangle, t_sink 0, t_src 0..%d" % (k4 - 1),
                            "split": _entry_gate(np.concatenate([got[0][k1][0, 0, :k4].ravel(), got[1][k1][0, :k4].ravel()]),
                                                 np.concatenate([c1.ravel(), c2.ravel()]),
                                                 np.concatenate([ab1.ravel(), ab2.ravel()]), 1e-9),
                            "fp64": _entry_gate(np.concatenate([f[0][0][0, 0, :k4].ravel(), f[1][0][0, :k4].ravel()]),
                                                np.concatenate([c1.ravel(), c2.ravel()]),
                                                np.concatenate([ab1.ravel(), ab2.ravel()]), 1e-12)}
        res["cpu_baseline"] = {"value": k4 * 6 / tcpu, "unit": "diagrams/s", "cores": os.cpu_count(), "kind": "port",
                               "sample": "the oracle sample above (%d entries, reference chain order)" % (k4 * 6)}
    except Exception as e:
        res["vs_oracle"] = {"unavailable": str(e)[:200]}
    del tau, diag, phi_all, P, ops, mom5, mom2, holder
    torch.cuda.synchronize()
    return res


def run_adjoint(args):
    print(json.dumps(adjoint_block(args, full=True)))


def adjoint_block(args, full=False):
    """Distillation-profile objective and its gradient at Nev=100, Lt=64: rho (p=0) for
    t = 2..9 and the pi pi I=0 set at dt = 4, f_k = exp(-lambda_k/0.3); forward plus
    backward per evaluation, and FP64 central differences (h = 1e-6) on a few f_k."""
    import numpy as np
    import torch
    from contractions_code_scattering_gb300 import adjoint, api, synth
    api.device_init(0)
    nt, nev = args.nt or 64, 100
    tau = synth.make_prop(nt, nev, seed=SEED, decay=0.35, backend="torch")
    moms = [(0, 0, 0), (1, 0, 0), (-1, 0, 0)]
    phis = synth.make_phi_momenta_torch(nt, nev, moms, seed=SEED + 1)
    g = torch.Generator(device="cuda")
    g.manual_seed(SEED + 2)
    sd = float(np.sqrt(0.5 / nev))
    extra = torch.complex(torch.randn((nt, 4, nev, nev), generator=g, device="cuda", dtype=torch.float64) * sd,
                          torch.randn((nt, 4, nev, nev), generator=g, device="cuda", dtype=torch.float64) * sd)
    mom5 = torch.cat([phis[:, :1], extra], dim=1).contiguous()
    p, m = phis[:, 1].contiguous(), phis[:, 2].contiguous()
    pipi = (p, m, p, m)
    f0 = adjoint.default_profile(nev)
    kw = dict(rho_ts=(2, 8), pipi_dt=4, isospin=0, engine=args.engine if args.engine != "auto" else "split")

    def evaluate():
        f = torch.tensor(f0, device="cuda", requires_grad=True)
        L = adjoint.objective(f, tau, mom5, pipi, **kw)
        L.backward()
        return L.item(), f.grad

    steps, warm = (args.steps, args.warmup) if full else (1, 1)
    t, launches, kern = _timed(evaluate, steps, warm)
    L, grad = evaluate()
    grad = grad.cpu().numpy()
    kw64 = dict(kw, engine="fp64")  # the differences are taken on the FP64 forward
    h = 1e-6
    fd = {}
    for k in (0, 37, 99):
        fp, fm = f0.copy(), f0.copy()
        fp[k] += h
        fm[k] -= h
        with torch.no_grad():
            lp = adjoint.objective(torch.tensor(fp, device="cuda"), tau, mom5, pipi, **kw64).item()
            lm = adjoint.objective(torch.tensor(fm, device="cuda"), tau, mom5, pipi, **kw64).item()
        fd[k] = (lp - lm) / (2 * h)
    worst = max(abs(fd[k] - grad[k]) for k in fd) / np.abs(grad).max()
    line = {"workload": "adjoint", "metric": "profile objective + gradient evaluations/s @Nev=100,Lt=64",
            "value": 1.0 / t, "unit": "evaluations/s", "ms_per_evaluation": 1e3 * t, "steps": steps,
            "engine": kw["engine"],
            "warmup": warm, "objective": L, "grad_norm": float(np.linalg.norm(grad)),
            "fd_check": {"h": h, "forward": "fp64 engine", "components": {str(k): [fd[k], float(grad[k])] for k in fd},
                         "max_abs_diff_over_max_grad": worst},
            "gpu_launches": launches, "kernels": {k: v for k, v in kern.items() if not k.startswith("_")}}
    del tau, phis, extra, mom5
    torch.cuda.synchronize()
    return line


def run_legacy_gpu(args):
    print(json.dumps(legacy_block(args)))


def legacy_block(args):
    """The reference's own rho kernel (lib/contract_kernels_rho.cu built unmodified for
    sm_103a: CUDA-core FP64, 25x25 tiles, one launch of 768 spin-row blocks per
    (t_sink, t_src)) against both engines on the same workload: Nev=100, Lt=64, one
    momentum, all 48 operator/polarisation outputs (16 op pairs x 3 polarisations) of
    every (t_sink, t_src).  The reference is timed on the first t_sink rows."""
    import numpy as np
    import torch
    from contractions_code_scattering_gb300 import api, synth
    from oracle import refkernels as RK
    from oracle import tables as TB
    if not os.path.exists(RK.cubin("rho")):
        return {"workload": "legacy_gpu", "unavailable": "reference cubins not built (oracle/build_ref.sh)"}
    api.device_init(0)
    # the reference kernels launch on the legacy default stream: time there
    torch.cuda.set_stream(torch.cuda.default_stream())
    nt, nev = 64, 100
    tau = synth.make_prop(nt, nev, seed=SEED, decay=0.35, backend="torch")
    g = torch.Generator(device="cuda")
    g.manual_seed(SEED + 3)
    sd = float(np.sqrt(0.5 / nev))
    mom5 = torch.complex(torch.randn((nt, 5, nev, nev), generator=g, device="cuda", dtype=torch.float64) * sd,
                         torch.randn((nt, 5, nev, nev), generator=g, device="cuda", dtype=torch.float64) * sd)
    mom5 = mom5.contiguous()
    m = RK.RefModule(RK.cubin("rho"))
    spin, lprp, coef = TB.rho_tables()
    m.set_constant("c_spinIndices_rho", RK._i16(spin))
    m.set_constant("c_lp_rp_rho", RK._i16(lprp))
    m.set_constant("c_coef_rho", RK._f32(coef))
    k = m.kernel("calculate_rho_kernel_double")
    tmom = RK.texture(mom5)
    tmp1 = torch.zeros(768 * nev * nev, dtype=torch.complex128, device="cuda")
    tmp2 = torch.zeros_like(tmp1)
    out = torch.zeros(nt * 768, dtype=torch.complex128, device="cuda")
    rows = 2
    texs = [RK.texture(tau[tf]) for tf in range(rows)]
    m.launch(k, 768, [RK._p(out), texs[0], tmom, ctypes.c_int(0), ctypes.c_int(0), RK._p(tmp1), RK._p(tmp2)])
    m.sync()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for tf in range(rows):
        for ti in range(nt):
            m.launch(k, 768, [RK._p(out), texs[tf], tmom, ctypes.c_int(ti), ctypes.c_int(tf), RK._p(tmp1),
                              RK._p(tmp2)])
    e1.record()
    m.sync()
    t_ref = e0.elapsed_time(e1) / 1e3
    for t in texs:
        RK.destroy_texture(t)
    RK.destroy_texture(tmom)
    ref_rate = rows * nt * 48 / t_ref
    res = {}
    for eng in ("fp64", "split"):
        t, launches, kern = _timed(lambda: api.run_contract_rho(tau, mom5, engine=eng), 1, 1)
        res[eng] = {"diagrams_per_s": nt * nt * 48 / t, "ms_per_step": 1e3 * t}
    line = {"workload": "legacy_gpu", "metric": "diagrams/s @Nev=100,Lt=64: rho, 48 outputs per pair, one momentum",
            "unit": "diagrams/s", "reference_kernel": {"diagrams_per_s": ref_rate, "sample": "t_sink 0..%d, all t_src"
                                                      % (rows - 1), "ms": 1e3 * t_ref},
            "fp64_engine": res["fp64"], "split_engine": res["split"],
            "split_vs_reference_kernel": res["split"]["diagrams_per_s"] / ref_rate,
            "fp64_vs_reference_kernel": res["fp64"]["diagrams_per_s"] / ref_rate}
    del tau, mom5, tmp1, tmp2, out
    torch.cuda.synchronize()
    return line


def run_elementals(args):
    """Elementals from Laplacian eigenvectors, as the reference drivers build them
    before calculateRho (tests/compute_rho.cpp:116-223): a 16^3 x Lt=64 lattice,
    Nev=100, the 7 momenta |p|^2 <= 1, all five rho operators (plain, smeared,
    three commutators with covariant derivatives).  Seeded synthetic eigenvectors
    (orthonormal per time slice) and SU(3) links stand in for the lattice files."""
    import numpy as np
    import torch
    from contractions_code_scattering_gb300 import api, synth
    from oracle import elementals as E
    api.device_init(0)
    nt, nev, L = args.nt or 64, 100, 16
    moms = synth.momenta(MAXP2)
    V = synth.make_eigvecs(nt, nev, L, L, L, seed=SEED, backend="torch")
    U = synth.make_links(nt, L, L, L, seed=SEED + 1, backend="torch")
    out = torch.empty((len(moms), 5, nt, nev, nev), dtype=torch.complex128, device="cuda")
    step = lambda: api.elementals(V, moms, links=U, out=out)
    t, launches, kern = _timed(step, args.steps, args.warmup)
    K = 3 * L ** 3
    # 10 products X^dag diag(phase) Y of nev x nev over K per (t, p): 8 nev^2 K flops each
    flops = 10 * 8.0 * nev * nev * K * nt * len(moms)
    peak = fp64_peak_tflops()
    achieved = flops / (kern["el_gemm"]["ms"] / 1e3 / args.steps) / 1e12
    # parity on a sample: t = 0, two momenta, against the numpy restatement; and the
    # same restatement timed on the host cores (numpy einsum, its own threads)
    Vh, Uh = V[:1].cpu().numpy(), U[:1].cpu().numpy()
    sample = [moms[0], moms[1]]
    t0 = time.perf_counter()
    ref = E.elementals(Vh, sample, Uh)
    tcpu = time.perf_counter() - t0
    got = out[:2, :, :1].cpu().numpy()
    n_el = len(moms) * 5 * nt
    line = {"workload": "elementals", "metric": "elementals/s @Nev=100,16^3x64: 7 momenta x 5 operators, FP64",
            "value": n_el / t, "unit": "elementals/s", "ms_per_step": 1e3 * t, "steps": args.steps,
            "warmup": args.warmup, "elementals_per_step": n_el, "gpu_launches": launches, "kernels": kern,
            "roofline": {"kernel": "el_gemm", "bound": "fp64 pipe", "achieved": achieved, "peak": peak,
                         "unit": "TFLOP/s", "frac": achieved / peak,
                         "peak_source": "measured in bench.py: cuBLAS DGEMM 8192^3",
                         "algorithmic": "10 products of 8 nev^2 (3 L^3) flops per (t, p)"},
            "vs_restatement": _errs(got, ref),
            "cpu_baseline": {"value": 2 * 5 / tcpu, "unit": "elementals/s", "cores": os.cpu_count(), "kind": "port",
                             "sample": "t = 0, 2 momenta, 5 operators (numpy restatement)"}}
    print(json.dumps(line))


def run_fp64_peak(args):
    """cuBLAS FP64 reference rates on this GPU (torch.matmul): DGEMM and ZGEMM at
    4096^3, best of 3 after one untimed call; the FP64 engine's block GEMM is
    compared with these."""
    import torch
    n = 4096
    res = {}
    for name, dt, fl in (("dgemm", torch.float64, 2.0), ("zgemm", torch.complex128, 8.0)):
        a = torch.randn(n, n, dtype=dt, device="cuda")
        b = torch.randn(n, n, dtype=dt, device="cuda")
        torch.matmul(a, b)
        torch.cuda.synchronize()
        best = 1e9
        for _ in range(3):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            torch.matmul(a, b)
            e1.record()
            e1.synchronize()
            best = min(best, e0.elapsed_time(e1) / 1e3)
        res[name] = {"tflops": fl * n ** 3 / best / 1e12, "ms": 1e3 * best}
        del a, b
    print(json.dumps({"workload": "fp64_peak", "n": n, **res}))


def run_mma_probe(args):
    """The split GEMMs' per-chunk MMA schedules by themselves on every SM
    (include/ctr.h: ctr_mma_schedule_probe): no operand copies, no epilogue,
    operands that stay in shared memory.  Short runs (0.3 ms) show the issue rate;
    long ones (~100 ms) run under the power limit like the GEMMs do."""
    from contractions_code_scattering_gb300 import api
    api.device_init(0)
    pk = measured_peaks() or {}
    peak = pk.get("bf16_tflops")
    res = {}
    for name, hp in (("standard", False), ("high_precision", True)):
        for nchunk in (300, 100000):
            api.mma_schedule_probe(hp, 50)  # module load, TMEM and shared-memory set-up
            cpm, tf = api.mma_schedule_probe(hp, nchunk)
            res["%s_nchunk%d" % (name, nchunk)] = {"clocks_per_mma": cpm, "tflops": tf,
                                                   "frac_of_measured_bf16": tf / peak if peak else None}
    print(json.dumps({"workload": "mma_probe", "mma": {"standard": "M128 N128 K16 bf16, 30 a chunk",
                                                       "high_precision": "M128 N96 K16 bf16, 42 a chunk"},
                      "nominal_clocks_per_mma": {"standard": 64, "high_precision": 48}, **res}))


WORKLOADS = {"fp64_peak": run_fp64_peak, "rho_small": run_rho_small, "pipi": run_pipi, "mixed": run_mixed, "adjoint": run_adjoint,
             "legacy_gpu": run_legacy_gpu, "elementals": run_elementals, "mma_probe": run_mma_probe}


if __name__ == "__main__":
    main()
