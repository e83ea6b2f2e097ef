"""Benchmark of the GB300 RQA engine on the Lorenz workload.

Workload (one "step"): the x-component of the Lorenz system, N = 200,000
samples, float32, z-scored; tau in {1,2,4,8} x emb in {3,5,8}; 16 thresholds
0.05..0.8 (in units of the series' std); Euclidean norm; RR, DET (lmin=2) and
LAM (vmin=2) for every (tau, emb).  Metric: recurrence-matrix cells per
second per threshold, sum over measures of nc^2 * nthr / time.

  value : device-resident passes through the engine's C ABI
          (accrqa_gb300_*_dev), inputs already in HBM, outputs zeroed inside
          the step; CUDA events on the launching stream.
  e2e   : the reference-facing calls RR / DET / LAM (py_accrqa_* on host
          numpy buffers): H2D of the series, kernels, D2H, post-processing.
  --impl reference : the reference algorithm's CPU implementation (the
          oracle port, OpenMP on all host cores) on a bounded sample of the
          same workload, extrapolated to the full workload.

Multi-GPU: replicas only -- every rank runs the whole workload on its own GPU
(weak scaling); value = cells of all ranks / max time over ranks.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

TAUS = [1, 2, 4, 8]
EMBS = [3, 5, 8]
NTHR = 16
N = 200_000
SEED = 2024
METRIC = "RM cells/s per threshold (RR+DET+LAM)"
WORKLOAD = ("lorenz-x N=200000 fp32 z-scored, tau{1,2,4,8} x emb{3,5,8}, 16 thresholds "
            "0.05-0.8 std, Euclidean, RR+DET(lmin=2)+LAM(vmin=2)")


def series():
    from accrqa_gb300 import workloads
    x = workloads.lorenz_x(N, SEED).astype(np.float32)
    thr = (np.linspace(0.05, 0.8, NTHR) * float(np.std(x.astype(np.float64)))).astype(np.float32)
    return x, thr


def combos():
    return [(t, e) for t in TAUS for e in EMBS]


def cells_per_step(measures=3):
    tot = 0
    for t, e in combos():
        nc = N - (e - 1) * t
        tot += nc * nc * NTHR
    return tot * measures


# DRAM bytes (read + write) per pass of the dominant pass, LAM (tile_levels +
# lam_levels), on this workload: the mean over the 12 passes of one step in an
# ncu capture (dram__bytes_read.sum + dram__bytes_write.sum of both kernels).
# tile_levels writes the level planes of the upper-triangle tiles (12.44 GB),
# lam_levels reads them twice (24.87 GB) and writes the chunk records (0.33
# GB).  5.5 ms of HBM time in a 39 ms pass: HBM is not the bound.
LAM_TRAFFIC_PER_PASS = 37_662_000_000


def algo_ops(nc, emb, nthr):
    """FP32 operations one pass performs by the algorithm's count:
    U * (3*emb + 1 + nthr), U = nc(nc+1)/2 unique pairs (sub, mul, add per
    dimension, one sqrt, one compare per threshold)."""
    u = nc * (nc + 1) // 2
    return u * (3 * emb + 1 + nthr)


class ClockSampler:
    """nvidia-smi clock/throttle samples during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.thread.join(timeout=2)
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            p = [v.strip() for v in ln.split(",")]
            if len(p) < 7:
                continue
            try:
                sm.append(float(p[0]))
                mx.append(float(p[1]))
            except ValueError:
                continue
            for nm, v in zip(names, p[3:7]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


_T0 = time.perf_counter()


def log(msg):
    """Progress line on stderr (the JSON result goes to stdout)."""
    print(f"[bench {time.perf_counter() - _T0:7.1f}s] {msg}", file=sys.stderr, flush=True)


def dist_setup():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def reduce_max(value, device=None):
    """Max of a per-rank float over the initialised process group (identity
    without one).  Replicas only: this is the one cross-rank exchange."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_rate(cells_per_rank_step, steps, world_size, max_seconds):
    """Whole-job throughput of independent replicas: every rank's cells over
    the slowest rank's time."""
    return cells_per_rank_step * steps * world_size / max_seconds


# ---------------------------------------------------------------------------
# our arm
# ---------------------------------------------------------------------------
def run_ours(args):
    import torch
    import torch.distributed as dist

    import accrqa_gb300
    from accrqa_gb300 import _lib, engine

    ws, rank, local = dist_setup()
    torch.cuda.set_device(local)
    if ws > 1:
        dist.init_process_group("nccl")
    lib = _lib.handle()
    dev = torch.device("cuda", local)
    x, thr = series()
    stream = torch.cuda.current_stream(dev)
    sp = stream.cuda_stream

    # device-resident inputs and outputs
    dx = torch.zeros(N + 128, dtype=torch.float32, device=dev)
    dx[:N].copy_(torch.from_numpy(x))
    layout, off = [], 0
    for t, e in combos():
        nc = N - (e - 1) * t
        layout.append((t, e, nc, off))
        off += NTHR * (nc + 1)
    d_det = torch.zeros(off, dtype=torch.int64, device=dev)
    d_lam = torch.zeros(off, dtype=torch.int64, device=dev)
    d_cnt = torch.zeros(len(layout) * NTHR, dtype=torch.int64, device=dev)
    d_max = torch.zeros(2 * len(layout) * NTHR, dtype=torch.int32, device=dev)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)   # > 129 MB L2

    kinds = ("rr", "det", "lam")
    ev = {k: [] for k in kinds}

    def step(record):
        d_det.zero_()
        d_lam.zero_()
        d_cnt.zero_()
        d_max.zero_()
        for ci, (t, e, nc, o) in enumerate(layout):
            for kind in kinds:
                if record:
                    s0 = torch.cuda.Event(enable_timing=True)
                    s0.record(stream)
                if kind == "rr":
                    engine.rr_counts_dev(d_cnt.data_ptr() + ci * NTHR * 8, dx.data_ptr(),
                                         engine.F32, N, t, e, thr, 1, sp)
                elif kind == "det":
                    engine.det_hist_dev(d_det.data_ptr() + o * 8, nc + 1,
                                        d_max.data_ptr() + ci * NTHR * 4, dx.data_ptr(),
                                        engine.F32, N, t, e, thr, 1, sp)
                else:
                    engine.lam_hist_dev(d_lam.data_ptr() + o * 8, nc + 1,
                                        d_max.data_ptr() + (len(layout) + ci) * NTHR * 4,
                                        dx.data_ptr(), engine.F32, N, t, e, thr, 1, sp)
                if record:
                    s1 = torch.cuda.Event(enable_timing=True)
                    s1.record(stream)
                    ev[kind].append((s0, s1, nc, e))

    # the chunk granularity of the balanced walks, measured on this GPU
    # (about a second, before the warm-up and outside every timed region)
    if args.no_autotune:
        tuned = "off (built-in chunk granularity)"
    else:
        tuned = engine.autotune()
    log(f"autotune: {tuned}")
    log("inputs ready; warm-up")
    for _ in range(args.warmup):
        step(False)
        torch.cuda.synchronize()
        log("warm-up step done")
    torch.cuda.synchronize()
    if ws > 1:
        dist.barrier()
    torch.cuda.synchronize()
    clocks = ClockSampler(local)
    clocks.start()
    launches0 = lib.accrqa_gb300_kernel_launches()
    step_ms = []
    for _ in range(args.steps):
        flush.fill_(1)
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record(stream)
        step(True)
        b.record(stream)
        b.synchronize()
        step_ms.append(a.elapsed_time(b))
        log(f"timed step {step_ms[-1]:.1f} ms")
    torch.cuda.synchronize()
    launches = lib.accrqa_gb300_kernel_launches() - launches0
    clk = clocks.stop()
    total_ms = reduce_max(float(sum(step_ms)), dev)
    if ws > 1:
        dist.barrier()

    # per-kernel totals and the dominant kernel's roofline
    per_kind = {}
    for kind in kinds:
        ms = sum(s0.elapsed_time(s1) for s0, s1, _, _ in ev[kind])
        ops = sum(algo_ops(nc, e, NTHR) for _, _, nc, e in ev[kind])
        per_kind[kind] = {"ms": ms, "ops": ops, "launches": len(ev[kind])}
    dom = max(per_kind, key=lambda k: per_kind[k]["ms"])
    props = torch.cuda.get_device_properties(dev)
    sm_mhz = clk.get("sm_mhz") or 1462.0
    derived_ops = props.multi_processor_count * 128 * sm_mhz * 1e6   # 128 FP32 lanes per SM
    # measured ceiling: separately rounded FP32 multiply/add chains, scalar
    # and packed f32x2 (the kernels use both); the faster one is the peak
    probe = {"scalar": engine.probe_fp32(0), "f32x2": engine.probe_fp32(1),
             "fp64": engine.probe_fp32(2)}
    peak_ops = max(probe["scalar"], probe["f32x2"])
    achieved = per_kind[dom]["ops"] / (per_kind[dom]["ms"] * 1e-3)

    # end to end through the reference-facing API (host buffers)
    taus = np.array(TAUS, dtype=np.intc)
    embs = np.array(EMBS, dtype=np.intc)
    lm = np.array([2], dtype=np.intc)
    D = accrqa_gb300.accrqaDistance("euclidean")
    e2e_steps = max(1, min(args.steps, 3))

    def e2e_step():
        accrqa_gb300.RR(x, taus, embs, thr, D, tidy_data=False)
        accrqa_gb300.DET(x, taus, embs, lm, thr, D, tidy_data=False)
        accrqa_gb300.LAM(x, taus, embs, lm, thr, D, tidy_data=False)

    log("clocks stopped; e2e warm-up")
    e2e_step()   # warm-up
    torch.cuda.synchronize()
    log("e2e warm-up done")
    if ws > 1:
        dist.barrier()
    lib.accrqa_gb300_transfer_stats(None, None, 1)
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        flush.fill_(1)
        torch.cuda.synchronize()
        e2e_step()
    e2e_s = time.perf_counter() - t0
    log(f"e2e {e2e_s / e2e_steps:.2f} s per step")
    import ctypes
    h2d, d2h = ctypes.c_uint64(), ctypes.c_uint64()
    lib.accrqa_gb300_transfer_stats(ctypes.byref(h2d), ctypes.byref(d2h), 0)
    e2e_s = reduce_max(e2e_s, dev)

    value = replica_rate(cells_per_step(), args.steps, ws, total_ms * 1e-3)
    e2e_value = replica_rate(cells_per_step(), e2e_steps, ws, e2e_s)

    line = {
        "metric": METRIC, "value": value, "unit": "cells/s",
        "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": total_ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": WORKLOAD, "parallelism": f"replicas{ws}",
                   "l2": "flushed by a 256 MB write before every timed step",
                   "inputs_in_hbm": True},
        "e2e": {"value": e2e_value, "unit": "cells/s",
                "h2d_bytes_per_step": int(h2d.value // e2e_steps),
                "d2h_bytes_per_step": int(d2h.value // e2e_steps),
                "path": "accrqa_gb300.RR/DET/LAM -> py_accrqa_* (host numpy buffers)"},
        "gpu_launches": int(launches),
        "autotune": tuned,
        "roofline": {"bound": "fp32", "kernel": dom,
                     "pass_kernels": {"rr": "rr_rows", "det": "det_diags + line_stitch",
                                      "lam": "tile_levels + lam_levels + line_stitch"}[dom],
                     "achieved": achieved / 1e12,
                     "peak": peak_ops / 1e12, "unit": "TFLOP/s",
                     "frac": achieved / peak_ops,
                     "traffic": LAM_TRAFFIC_PER_PASS if dom == "lam" else None,
                     "peak_source": "measured: multiply/add chain probe "
                                    "(accrqa_gb300_probe_fp32), best of FP32 scalar and f32x2",
                     "probe_tflops": {k: v / 1e12 for k, v in probe.items()},
                     "derived_tflops": derived_ops / 1e12,
                     "ops_per_launch": "U*(3*emb+1+nthr), U=nc(nc+1)/2"},
        "kernels": {k: {"ms_total": v["ms"], "launches": v["launches"],
                        "tflops_algorithmic": v["ops"] / (v["ms"] * 1e-3) / 1e12}
                    for k, v in per_kind.items()},
        "clocks": clk,
    }
    if rank == 0 and not args.skip_roofline_1m:
        line["roofline_1m"] = roofline_1m_section(args, peak_ops, probe["fp64"])
    if rank == 0 and not args.skip_batched:
        line["batched"] = batched_section(args)
    if rank == 0 and not args.skip_served:
        line["served"] = [served_section(args, r) for r in args.serve_rates]
    if rank == 0 and not args.no_cpu_baseline:
        log("cpu baseline")
        line["cpu_baseline"] = cpu_baseline(args.cpu_seconds)
        log("cpu baseline done")
    if rank == 0:
        print(json.dumps(line), flush=True)
    if ws > 1:
        dist.destroy_process_group()


# ---------------------------------------------------------------------------
# Batched uneven workload: one submission vs one plain call per series
# ---------------------------------------------------------------------------
def batched_section(args):
    """512 series of log-uniform length in [1000, 64000] (seeded mixes of
    logistic, Lorenz-x and AR(1)), random tau/emb/norm, 8 thresholds, RR +
    DET + LAM with lmin = vmin = 2: the batched entry point against 512
    triples of plain public-API calls, both on host buffers end to end, and a
    check that every output is identical."""
    import accrqa_gb300 as A
    from accrqa_gb300 import engine, workloads

    log("batched: generating the uneven workload")
    jobs = workloads.uneven_batch(args.batch_series)
    cells = 0
    for j in jobs:
        nc = len(j["x"]) - (j["emb"] - 1) * j["tau"]
        cells += nc * nc * len(j["thresholds"]) * 3
    engine.batch(jobs[:8])   # warm-up of the kernel shapes
    times = []
    for _ in range(2):
        t0 = time.perf_counter()
        outs = engine.batch(jobs)
        times.append(time.perf_counter() - t0)
    t_batch = min(times)
    log(f"batched: {t_batch:.3f} s")

    def plain(j):
        D = A.accrqaDistance("euclidean" if j["norm"] == 1 else "maximal")
        t = np.array([j["tau"]], np.intc)
        e = np.array([j["emb"]], np.intc)
        lm = np.array([2], np.intc)
        return (A.RR(j["x"], t, e, j["thresholds"], D, tidy_data=False).reshape(-1),
                A.DET(j["x"], t, e, lm, j["thresholds"], D, tidy_data=False).reshape(-1, 5),
                A.LAM(j["x"], t, e, lm, j["thresholds"], D, tidy_data=False).reshape(-1, 5))

    for j in jobs[:8]:
        plain(j)
    t0 = time.perf_counter()
    ref = [plain(j) for j in jobs]
    t_plain = time.perf_counter() - t0
    log(f"plain: {t_plain:.3f} s")
    same = all(np.array_equal(o["rr"], r[0]) and np.array_equal(o["det"], r[1], equal_nan=True)
               and np.array_equal(o["lam"], r[2], equal_nan=True) for o, r in zip(outs, ref))

    # per measure: each measure batched alone and as plain calls
    per_measure = {}
    one = cells // 3
    for idx, meas in enumerate(("rr", "det", "lam")):
        t0 = time.perf_counter()
        engine.batch(jobs, measures=(meas,))
        tb = time.perf_counter() - t0
        fn = (A.RR, A.DET, A.LAM)[idx]
        t0 = time.perf_counter()
        for j in jobs:
            D = A.accrqaDistance("euclidean" if j["norm"] == 1 else "maximal")
            t = np.array([j["tau"]], np.intc)
            e = np.array([j["emb"]], np.intc)
            if meas == "rr":
                fn(j["x"], t, e, j["thresholds"], D, tidy_data=False)
            else:
                fn(j["x"], t, e, np.array([2], np.intc), j["thresholds"], D, tidy_data=False)
        tp = time.perf_counter() - t0
        per_measure[meas] = {"batched_cells_per_s": one / tb, "plain_cells_per_s": one / tp,
                             "speedup_vs_plain": tp / tb}
    log("batched: per measure done")
    return {"workload": f"{len(jobs)} uneven series (1e3..6.4e4 log-uniform, mixed generators), "
                        "tau 1..4, emb 2..8, E/M norm, 8 thresholds, RR+DET+LAM, fp32",
            "value": cells / t_batch, "unit": "cells/s", "seconds": t_batch,
            "plain_value": cells / t_plain, "plain_seconds": t_plain,
            "speedup_vs_plain": t_plain / t_batch, "identical_results": bool(same),
            "cells": cells, "per_measure": per_measure}


# ---------------------------------------------------------------------------
# Served stream: Poisson arrivals, continuous batching vs sequential calls
# ---------------------------------------------------------------------------
_SERVED = {}


def served_requests(count, seed=5):
    """Requests of the served stream: length log-uniform in [2000, 256000],
    float32 (float64 with probability 0.2), one measure of RR/DET/LAM, 1-16
    thresholds (0.05-1.0 std), tau 1..4, emb 2..8, E/M norm.  Generated once
    per (count, seed); every rate serves the same requests."""
    if (count, seed) not in _SERVED:
        _SERVED[(count, seed)] = _make_served(count, seed)
    return _SERVED[(count, seed)]


def _make_served(count, seed):
    from accrqa_gb300 import workloads
    rng = np.random.default_rng(seed)
    gens = [workloads.logistic, workloads.ar1, workloads.white]
    reqs = []
    for i in range(count):
        n = int(np.exp(rng.uniform(np.log(2000), np.log(256000))))
        dt = np.float64 if rng.uniform() < 0.2 else np.float32
        x = gens[i % 3](n, int(rng.integers(1 << 30)))
        x = ((x - x.mean()) / x.std()).astype(dt)
        nthr = int(rng.integers(1, 17))
        reqs.append(dict(x=x, tau=int(rng.integers(1, 5)), emb=int(rng.integers(2, 9)),
                         norm=int(rng.integers(1, 3)),
                         thresholds=np.linspace(0.05, 1.0, nthr).astype(dt),
                         measures=(str(rng.choice(["rr", "det", "lam"])),)))
    return reqs


def served_section(args, rate):
    """Serve a Poisson stream through the continuous-batching server and
    through sequential plain calls (one FIFO worker), same requests, same
    arrival times; report throughput and latency percentiles of both."""
    import threading

    import accrqa_gb300 as A
    from accrqa_gb300 import engine

    rate = float(rate)
    reqs = served_requests(args.serve_requests)
    rng = np.random.default_rng(6)
    arrivals = np.cumsum(rng.exponential(1.0 / rate, len(reqs)))
    cells = 0
    for r in reqs:
        nc = len(r["x"]) - (r["emb"] - 1) * r["tau"]
        cells += nc * nc * len(r["thresholds"])

    def plain(r):
        D = A.accrqaDistance("euclidean" if r["norm"] == 1 else "maximal")
        t = np.array([r["tau"]], np.intc)
        e = np.array([r["emb"]], np.intc)
        m = r["measures"][0]
        if m == "rr":
            return A.RR(r["x"], t, e, r["thresholds"], D, tidy_data=False)
        f = A.DET if m == "det" else A.LAM
        return f(r["x"], t, e, np.array([2], np.intc), r["thresholds"], D, tidy_data=False)

    # warm the kernel shapes of both paths
    for r in reqs[:6]:
        plain(r)
    with engine.Server(workers=args.serve_workers) as srv:
        for r in reqs[:6]:
            srv.wait(srv.submit(r))
        log(f"served: {len(reqs)} requests at {rate} req/s")
        lat = [0.0] * len(reqs)
        tickets = [None] * len(reqs)
        t0 = time.perf_counter()

        def producer():
            for i, r in enumerate(reqs):
                dt = t0 + arrivals[i] - time.perf_counter()
                if dt > 0:
                    time.sleep(dt)
                tickets[i] = srv.submit(r)

        th = threading.Thread(target=producer)
        th.start()
        done = 0
        while done < len(reqs):
            if tickets[done] is None:
                time.sleep(0.0005)
                continue
            _, lat[done] = srv.wait(tickets[done])
            done += 1
        th.join()
        t_served = time.perf_counter() - t0   # first arrival to last completion
        batches, served = srv.stats()
        peak = srv.peak_bytes()
    # sequential plain calls, FIFO, same arrival times
    log("served: sequential plain calls")
    seq_lat = []
    t_free = 0.0
    busy = 0.0
    t0 = time.perf_counter()
    for i, r in enumerate(reqs):
        now = time.perf_counter() - t0
        if now < arrivals[i]:
            time.sleep(arrivals[i] - now)
        start = time.perf_counter() - t0
        plain(r)
        end = time.perf_counter() - t0
        seq_lat.append((end - arrivals[i]) * 1e3)
        busy += end - start
        t_free = end
    t_seq = t_free
    p = lambda v, q: float(np.percentile(np.asarray(v), q))
    return {"workload": f"{len(reqs)} requests, Poisson {rate} req/s, n log-uniform "
                        "2e3..2.56e5, 20% fp64, one of RR/DET/LAM, 1-16 thresholds",
            "rate_req_s": rate, "workers": args.serve_workers, "batches": batches,
            "arrival_span_s": float(arrivals[-1]),
            "overloaded": bool(busy > arrivals[-1]),
            "peak_admitted_bytes": int(peak),
            "value": cells / t_served, "unit": "cells/s",
            "throughput": "cells over the makespan (first arrival to last completion)",
            "p50_ms": p(lat, 50), "p99_ms": p(lat, 99),
            "sequential_value": cells / t_seq, "sequential_p50_ms": p(seq_lat, 50),
            "sequential_p99_ms": p(seq_lat, 99), "seconds": t_served, "sequential_seconds": t_seq,
            "sequential_busy_seconds": busy}


# ---------------------------------------------------------------------------
# CPU baseline (the oracle port, test infrastructure; timed, never shipped)
# ---------------------------------------------------------------------------
def cpu_sample(budget_s):
    """Time RR, DET and LAM of the reference algorithm (one threshold, tau=1)
    for each emb of the workload, each on a bounded slice at full N (rows of
    the full matrix for RR and LAM, diagonals for DET), and extrapolate the
    measured cost per cell to every (tau, emb, threshold, measure)."""
    from oracle import oracle
    x, thr = series()
    t = float(thr[NTHR // 2])
    per = budget_s / (3.0 * len(EMBS))
    rate = {}
    cells_done = 0
    for emb in EMBS:
        nc = N - (emb - 1)
        for kind in ("rr", "lam", "det"):
            span, pos, spent, cells = 16, 1 if kind == "det" else 0, 0.0, 0
            while spent < per:
                t0 = time.perf_counter()
                if kind == "rr":
                    _, c = oracle.rr_sample(x, 1, emb, t, 1, pos, pos + span)
                elif kind == "lam":
                    _, _, c = oracle.lam_sample(x, 1, emb, t, 1, pos, pos + span)
                else:
                    _, c = oracle.det_sample(x, 1, emb, t, 1, pos, pos + span)
                dt = time.perf_counter() - t0
                spent += dt
                cells += c
                pos += span
                if dt < per / 4:
                    span *= 2
            rate[(kind, emb)] = cells / spent
            cells_done += cells
    est = 0.0
    for tt, e in combos():
        ncc = N - (e - 1) * tt
        est += NTHR * (ncc * ncc / rate[("rr", e)] + ncc * ncc / rate[("lam", e)]
                       + ncc * (ncc - 1) / 2 / rate[("det", e)])
    return cells_per_step() / est, cells_done, oracle.num_threads()


def cpu_baseline(budget_s):
    t0 = time.perf_counter()
    value, cells, cores = cpu_sample(budget_s)
    return {"value": value, "unit": "cells/s", "cores": cores, "kind": "port",
            "estimate": "extrapolated",
            "sample": f"{cells:.3g} cells in {time.perf_counter() - t0:.1f}s: full N, tau=1, "
                      "1 threshold, row slices (RR, LAM) and diagonal slices (DET) for each "
                      "emb in {3,5,8}; cost per cell extrapolated to every (tau, emb, "
                      "threshold, measure) of the workload"}


def run_reference(args):
    ws, rank, _ = dist_setup()
    if rank != 0:
        return
    from oracle import oracle
    oracle.build()
    vals, ms = [], []
    budget = args.cpu_seconds
    for i in range(args.warmup + args.steps):
        t0 = time.perf_counter()
        v, _, cores = cpu_sample(budget / 2 if i < args.warmup else budget)
        if i >= args.warmup:
            vals.append(v)
            ms.append((time.perf_counter() - t0) * 1e3)
    value = statistics.median(vals)
    line = {
        "metric": METRIC, "value": value, "unit": "cells/s", "impl": "reference",
        "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": statistics.mean(ms), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": WORKLOAD, "parallelism": "cpu"},
        "cpu_baseline": {"value": value, "unit": "cells/s", "cores": cores, "kind": "port",
                         "estimate": "extrapolated",
                         "sample": "per step: tau=1, emb in {3,5,8}, full N, 1 threshold, "
                                   "bounded row (RR, LAM) and diagonal (DET) slices; the "
                                   "measured cost per cell extrapolated to every (tau, emb, "
                                   "threshold, measure) of the workload"},
        "e2e": {"value": value, "unit": "cells/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def roofline_1m_section(args, peak_f32, peak_f64):
    """The N = 1,000,000 roofline workload: white noise and AR(1) (phi 0.95),
    tau = 1, emb = 5, Euclidean, thresholds {0.1, 0.2, 0.5, 1.0} x std, RR and
    DET (lmin 2), one pass each: float32 device-resident (CUDA events),
    float64 through the host entry points (wall time; they take the float
    filter).  Reports seconds, cells/s and algorithmic TFLOP/s against the
    measured FP32 multiply/add peak (the filter computes in FP32).""" 
    import torch

    from accrqa_gb300 import engine, workloads
    n, tau, emb = 1_000_000, 1, 5
    nc = n - (emb - 1) * tau
    dev = torch.device("cuda", torch.cuda.current_device())
    stream = torch.cuda.current_stream(dev)
    sp = stream.cuda_stream
    out = []
    dtypes = [np.float32, np.float64]
    for name, gen in (("white", workloads.white), ("ar1", workloads.ar1)):
        base = gen(n, SEED + 7)
        base = (base - base.mean()) / base.std()
        for dt in dtypes:
            x = base.astype(dt)
            tdt = torch.float32 if dt == np.float32 else torch.float64
            code = engine.F32 if dt == np.float32 else engine.F64
            std = float(np.std(x.astype(np.float64)))
            thr = (np.array([0.1, 0.2, 0.5, 1.0]) * std).astype(dt)
            dx = torch.zeros(n + 128, dtype=tdt, device=dev)
            dx[:n].copy_(torch.from_numpy(x))
            hist = torch.zeros(len(thr) * (nc + 1), dtype=torch.int64, device=dev)
            cnt = torch.zeros(len(thr), dtype=torch.int64, device=dev)
            mx = torch.zeros(len(thr), dtype=torch.int32, device=dev)
            if dt == np.float64:
                # float64 through the engine's host entry points, which split
                # the series for the float filter (wall time incl. copies)
                engine.rr_counts(x[:4096], tau, emb, thr, 1)
                engine.det_histograms(x[:4096], tau, emb, thr, 1)
                for kind in ("rr", "det"):
                    torch.cuda.synchronize()
                    t0 = time.perf_counter()
                    if kind == "rr":
                        res = engine.rr_counts(x, tau, emb, thr, 1)
                    else:
                        res = engine.det_histograms(x, tau, emb, thr, 1)
                    sec = time.perf_counter() - t0
                    ops = algo_ops(nc, emb, len(thr))
                    out.append({"series": name, "dtype": "float64", "measure": kind,
                                "path": "host entry point, float filter + exact float64 fallback",
                                "seconds": sec, "cells_per_s": nc * nc * len(thr) / sec,
                                "tflops_algorithmic": ops / sec / 1e12,
                                "frac_of_measured_peak": ops / sec / peak_f32,
                                "recurrent_cells": int(np.sum(res)) if kind == "rr" else None})
                    log(f"1M {name} float64 {kind}: {sec:.3f} s")
                del dx, hist
                continue
            # warm the same kernels on a short prefix
            engine.rr_counts_dev(cnt.data_ptr(), dx.data_ptr(), code, 4096, tau, emb, thr, 1, sp)
            engine.det_hist_dev(hist.data_ptr(), nc + 1, mx.data_ptr(), dx.data_ptr(), code,
                                4096, tau, emb, thr, 1, sp)
            for kind in ("rr", "det"):
                hist.zero_()
                cnt.zero_()
                mx.zero_()
                torch.cuda.synchronize()
                a = torch.cuda.Event(enable_timing=True)
                b = torch.cuda.Event(enable_timing=True)
                a.record(stream)
                if kind == "rr":
                    engine.rr_counts_dev(cnt.data_ptr(), dx.data_ptr(), code, n, tau, emb, thr,
                                         1, sp)
                else:
                    engine.det_hist_dev(hist.data_ptr(), nc + 1, mx.data_ptr(), dx.data_ptr(),
                                        code, n, tau, emb, thr, 1, sp)
                b.record(stream)
                b.synchronize()
                sec = a.elapsed_time(b) * 1e-3
                ops = algo_ops(nc, emb, len(thr))
                rr_cells = int(cnt.sum().item()) if kind == "rr" else None
                out.append({"series": name, "dtype": np.dtype(dt).name, "measure": kind,
                            "seconds": sec, "cells_per_s": nc * nc * len(thr) / sec,
                            "tflops_algorithmic": ops / sec / 1e12,
                            "frac_of_measured_peak": ops / sec / peak_f32,
                            "recurrent_cells": rr_cells})
                log(f"1M {name} {np.dtype(dt).name} {kind}: {sec:.3f} s")
            del dx, hist
    return {"workload": "N=1e6 white and AR(1) phi=0.95, tau 1, emb 5, Euclidean, thresholds "
                        "{0.1,0.2,0.5,1.0} x std, RR and DET(lmin 2), one pass each",
            "ops_per_pass": "U*(3*emb+1+nthr), U=nc(nc+1)/2", "passes": out}


def run_case(args):
    """One pass of one kernel on a smaller series (for profiler captures):
    --case rr|det|lam, --n samples, tau=1, emb=5.  --series lorenz: the bench
    series with its 16 thresholds; --series white|ar1: the N = 1e6 roofline
    shapes (same generator, seed and standardisation) with thresholds
    {0.1, 0.2, 0.5, 1.0} x std.  --dtype f64 goes through the host entry
    points (float filter) instead of the device-resident ones.  --case batch
    runs the batched uneven workload (--batch-series series, RR+DET+LAM)
    warmup + steps times."""
    import torch

    from accrqa_gb300 import engine
    from accrqa_gb300 import workloads
    if args.case == "batch":
        jobs = workloads.uneven_batch(args.batch_series)
        for _ in range(args.warmup + args.steps):
            engine.batch(jobs)
        torch.cuda.synchronize()
        print(json.dumps({"case": "batch", "series": len(jobs), "done": True}))
        return
    n = args.n
    tau, emb = 1, 5
    if args.series == "lorenz":
        x = workloads.lorenz_x(n, SEED).astype(np.float32)
        thr = (np.linspace(0.05, 0.8, NTHR) * float(np.std(x.astype(np.float64)))).astype(np.float32)
    else:
        gen = workloads.white if args.series == "white" else workloads.ar1
        base = gen(n, SEED + 7)
        base = (base - base.mean()) / base.std()
        dt = np.float64 if args.dtype == "f64" else np.float32
        x = base.astype(dt)
        thr = (np.array([0.1, 0.2, 0.5, 1.0]) * float(np.std(x.astype(np.float64)))).astype(dt)
        if args.dtype == "f64":
            fn = {"rr": engine.rr_counts, "det": engine.det_histograms,
                  "lam": engine.lam_histograms}[args.case]
            for _ in range(args.warmup + args.steps):
                fn(x, tau, emb, thr, 1)
            torch.cuda.synchronize()
            print(json.dumps({"case": args.case, "series": args.series, "dtype": "f64",
                              "n": n, "done": True}))
            return
    nthr = len(thr)
    dev = torch.device("cuda", 0)
    sp = torch.cuda.current_stream(dev).cuda_stream
    dx = torch.zeros(n + 128, dtype=torch.float32, device=dev)
    dx[:n].copy_(torch.from_numpy(x))
    nc = n - (emb - 1) * tau
    hist = torch.zeros(nthr * (nc + 1), dtype=torch.int64, device=dev)
    cnt = torch.zeros(nthr, dtype=torch.int64, device=dev)
    mx = torch.zeros(nthr, dtype=torch.int32, device=dev)
    for _ in range(args.warmup + args.steps):
        hist.zero_()
        cnt.zero_()
        if args.case == "rr":
            engine.rr_counts_dev(cnt.data_ptr(), dx.data_ptr(), engine.F32, n, tau, emb, thr,
                                 1, sp)
        elif args.case == "det":
            engine.det_hist_dev(hist.data_ptr(), nc + 1, mx.data_ptr(), dx.data_ptr(),
                                engine.F32, n, tau, emb, thr, 1, sp)
        else:
            engine.lam_hist_dev(hist.data_ptr(), nc + 1, mx.data_ptr(), dx.data_ptr(),
                                engine.F32, n, tau, emb, thr, 1, sp)
    torch.cuda.synchronize()
    print(json.dumps({"case": args.case, "series": args.series, "n": n, "done": True}))


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--case", choices=["rr", "det", "lam", "batch"], default=None,
                    help="run a single pass of one kernel (profiling)")
    ap.add_argument("--n", type=int, default=50_000)
    ap.add_argument("--series", choices=["lorenz", "white", "ar1"], default="lorenz",
                    help="--case series (see run_case)")
    ap.add_argument("--dtype", choices=["f32", "f64"], default="f32",
                    help="--case series dtype (white/ar1 only)")
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-autotune", action="store_true",
                    help="keep the built-in chunk granularity (profiler launch lists)")
    ap.add_argument("--skip-batched", action="store_true")
    ap.add_argument("--skip-roofline-1m", action="store_true")

    ap.add_argument("--batch-series", type=int, default=512)
    ap.add_argument("--skip-served", action="store_true")
    ap.add_argument("--serve-rates", type=lambda s: [float(v) for v in s.split(",")],
                    default=[50.0, 200.0, 500.0, 2000.0])
    ap.add_argument("--serve-requests", type=int, default=1000)
    ap.add_argument("--serve-workers", type=int, default=4)
    args = ap.parse_args(argv)
    if args.warmup < 3 and args.impl == "ours":
        args.warmup = 3
    if args.case:
        run_case(args)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
