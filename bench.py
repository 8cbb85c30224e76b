#!/usr/bin/env python3
"""Benchmark: BRMerge SpGEMM GFLOP/s and HBM-roofline fraction on one GB300.

Workload (default): C = A*A, A = R-MAT(a,b,c,d = .57,.19,.19,.05) with n = 2^18
and 2.35*n samples (duplicates removed: ~607k nnz, ~9.0e7 intermediate
products), float64, BRMerge-Precise, plain per-call GPU path.  A "step" is
one SpGEMM call.  GFLOP/s = 2 * intermediate products / time, the
reference's definition (BRMerge-SpGEMM/src/brmerge_precise.cpp:65-69).

* value   -- device-resident inputs: one brm_precise_device call (C ABI)
             timed with CUDA events on the call's stream, L2 flushed between
             steps (the inputs fit in L2).
* e2e     -- the reference-facing host call brm_precise: pinned host inputs
             copied in, C copied back to host memory, wall clock per call.
* roofline -- the whole call: algorithmic bytes bytes(A) + bytes(B) +
             bytes(C) over its CUDA-event duration, against the measured HBM
             copy bandwidth in MEASURED_PEAKS.json.
* cpu_baseline -- the oracle restatement of BRMerge-Precise (OpenMP, all
             host cores) on the same input.

--impl reference times the reference algorithm on the host cores instead
(oracle/_ref when it was built here, else the oracle restatement).
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
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

RMAT_SCALE = 18
RMAT_EDGE_FACTOR = 2.35


def csr_bytes(M: int, nnz: int, vbytes: int) -> int:
    return 4 * (M + 1) + nnz * (4 + vbytes)


def make_workload(name: str, stencil_n: int = 128):
    import brmerge_gb300 as brm
    if name == "rmat":
        n = 1 << RMAT_SCALE
        A = brm.gen_rmat(RMAT_SCALE, int(RMAT_EDGE_FACTOR * n), seed=0)
        desc = {"workload": "rmat_n2^18_ef2.35_AxA", "n": n, "a": 0.57, "b": 0.19, "c": 0.19,
                "seed": 0}
    elif name == "er":
        A = brm.gen_er(16384, 8, seed=0)
        desc = {"workload": "er_n16384_8perrow_AxA", "n": 16384, "seed": 0}
    elif name == "stencil":
        A = brm.gen_stencil27(stencil_n)
        desc = {"workload": f"stencil27_{stencil_n}^3_AxA", "n": stencil_n ** 3}
    else:
        raise SystemExit(f"unknown workload {name}")
    return A, desc


def measured_traffic():
    """DRAM bytes of one Precise call on the R-MAT workload, from the committed
    ncu launch-list summary (a capture of this bench's own command)."""
    p = ROOT / "profiles" / "rmat18_precise_launches.md"
    if p.exists():
        for line in p.read_text().splitlines():
            if line.startswith("traffic_bytes_per_step:"):
                return int(line.split(":")[1])
    return None


def peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """Samples nvidia-smi clocks and throttle reasons during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.idx = gpu_index
        self.proc = None
        self.lines = []
        self.pre = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.idx), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
            # wait for the first sample: nvidia-smi's start-up (NVML
            # initialisation) then lies before the timed region, not in it
            t_end = time.time() + 5.0
            while not self.lines and self.proc.poll() is None and time.time() < t_end:
                time.sleep(0.01)
            self.pre = list(self.lines)  # the sample taken just before the region
            self.lines.clear()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, smax, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        # samples inside the timed region; a region shorter than the sampling
        # period falls back to the one taken just before it
        for ln in (self.lines or self.pre):
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                smax = max(smax, float(parts[1]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[4:8]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def max_over_ranks(x: float, ws: int) -> float:
    if ws == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device="cuda")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(ws):
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()


def cpu_baseline(A, budget_s: float = 20.0):
    """The oracle restatement on all host cores: 1 warm-up + timed calls,
    bounded by budget_s (BRMerge-SpGEMM/src/brmerge_precise.cpp:68-82)."""
    import oracle
    oracle.build(with_ref=False)
    nt = oracle.max_threads()
    flop = oracle.compute_flop(A, A)
    t0 = time.perf_counter()
    oracle.precise(A, A, nt)
    one = time.perf_counter() - t0
    reps = max(1, min(10, int(budget_s / max(one, 1e-3))))
    t0 = time.perf_counter()
    for _ in range(reps):
        oracle.precise(A, A, nt)
    dt = (time.perf_counter() - t0) / reps
    return {"value": round(2 * flop / dt / 1e9, 4), "unit": "GFLOP/s", "cores": nt,
            "kind": "port",
            "sample": f"full workload, 1 warm-up + mean of {reps} calls, {dt * 1e3:.1f} ms/call"}


def run_reference(args):
    """--impl reference: the reference algorithm on the host cores."""
    ws, rank, _ = dist_env()
    if rank != 0:
        return
    import oracle
    oracle.build(with_ref=False)
    A, desc = make_workload(args.workload, args.stencil_n)
    use_ref = oracle.ref_available()
    nt = oracle.max_threads()
    flop = oracle.compute_flop(A, A)

    def call():
        if use_ref:
            oracle.ref_precise(A, A, nt)
        else:
            oracle.precise(A, A, nt)

    for _ in range(args.warmup):
        call()
    times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        call()
        times.append(time.perf_counter() - t0)
    tot = sum(times)
    value = 2 * flop * args.steps / tot / 1e9
    kind = "reference" if use_ref else "port"
    line = {
        "metric": "SpGEMM GFLOP/s (BRMerge-Precise, C=A*A)", "value": round(value, 4),
        "unit": "GFLOP/s", "impl": "reference", "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(tot / args.steps * 1e3, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic", "config": desc,
        "cpu_baseline": {"value": round(value, 4), "unit": "GFLOP/s", "cores": nt, "kind": kind,
                         "sample": "full workload per step"},
        "e2e": {"value": round(value, 4), "unit": "GFLOP/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


BATCH_PAIRS = 4096


def make_batch(npairs: int, seed: int, dtype=np.float64):
    """Uneven batch: C_i = A_i * B_i, n_i ~ U[256, 8192], rows lognormal(ln 6,
    0.8) capped at 256, uniform random columns, values U[-1, 1]."""
    import brmerge_gb300 as brm
    rng = np.random.default_rng(seed)
    ns = rng.integers(256, 8193, npairs)
    pairs = []
    for i, n in enumerate(ns):
        A = brm.gen_lognormal(int(n), int(n), seed=seed * 100003 + 2 * i)
        B = brm.gen_lognormal(int(n), int(n), seed=seed * 100003 + 2 * i + 1)
        pairs.append((A.astype(dtype), B.astype(dtype)))
    return pairs


def upload_pairs(pairs, dev):
    """All matrices in three device arrays; DeviceCSR views per matrix."""
    import torch
    import brmerge_gb300 as brm
    mats = [m for ab in pairs for m in ab]
    rpt = torch.from_numpy(np.concatenate([m.rpt for m in mats])).to(dev)
    col = torch.from_numpy(np.concatenate([m.col for m in mats])).to(dev)
    val = torch.from_numpy(np.concatenate([m.val for m in mats])).to(dev)
    views, r, e = [], 0, 0
    for m in mats:
        views.append(brm.DeviceCSR(m.M, m.N, rpt[r:r + m.M + 1], col[e:e + m.nnz],
                                   val[e:e + m.nnz]))
        r += m.M + 1
        e += m.nnz
    return [(views[2 * i], views[2 * i + 1]) for i in range(len(pairs))], (rpt, col, val)


def device_steps(call, dev, stream, flush, steps: int, warmup: int = 2):
    """Median CUDA-event time (ms) of `call()` on `stream`, L2 flushed before
    every timed call; returns (ms, last result).  The side sections report the
    median, so that one stalled call (seen now and then on the shared boxes)
    does not move them; the headline step keeps the mean of its K steps."""
    import torch
    out = None
    for _ in range(warmup):
        out = call()
        del out
    torch.cuda.synchronize(dev)
    ts = []
    for i in range(steps):
        flush.fill_(float(i))
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        out = call()
        e1.record(stream)
        torch.cuda.synchronize(dev)
        ts.append(e0.elapsed_time(e1))
        if i + 1 < steps:
            del out
    return statistics.median(ts), out


def method_entry(ms: float, products: int, alg_bytes: int, peak: float) -> dict:
    ach = alg_bytes / (ms / 1e3) / 1e9
    return {"ms": round(ms, 4), "gflops": round(2 * products / (ms / 1e3) / 1e9, 3),
            "achieved_gbs": round(ach, 1), "frac": round(ach / peak, 4)}


def stencil_section(ctx, dev, stream, flush, steps: int, peak: float):
    """27-point stencil on 128^3 (C = A*A, a 125-point stencil): Precise and
    Upper through the one-call device forms."""
    import brmerge_gb300 as brm
    S = brm.gen_stencil27(128)
    products = brm.compute_flop_host(S, S)
    dS = brm.DeviceCSR.from_host(S, dev)
    res = {"workload": "stencil27_128^3_AxA", "n": S.M, "nnz_A": int(S.nnz),
           "products": int(products)}
    ms, C = device_steps(lambda: ctx.precise_device(dS, dS), dev, stream, flush, steps)
    res["nnz_C"] = int(C.nnz)
    alg = 2 * csr_bytes(S.M, S.nnz, 8) + csr_bytes(S.M, C.nnz, 8)
    del C
    res["precise"] = method_entry(ms, products, alg, peak)
    ms, C = device_steps(lambda: ctx.upper(dS, dS), dev, stream, flush, steps)
    del C
    res["upper"] = method_entry(ms, products, alg, peak)
    ms, C = device_steps(lambda: ctx.hash_device(dS, dS), dev, stream, flush, steps)
    del C
    res["hash_comparator"] = method_entry(ms, products, alg, peak)
    return res


def reader_section(ctx, A, steps: int):
    """The workload's A written as a MatrixMarket file (real general, 17
    significant digits) and read back by brm_read_mtx_device; the oracle's
    reader (numpy restatement of CSR::construct) timed on the same file."""
    import tempfile
    import torch
    import brmerge_gb300 as brm
    rows = np.repeat(np.arange(A.M, dtype=np.int64), np.diff(A.rpt)) + 1
    with tempfile.TemporaryDirectory() as td:
        path = Path(td) / "a.mtx"
        body = "\n".join(f"{r} {c} {v!r}" for r, c, v in
                         zip(rows.tolist(), (A.col + 1).tolist(), A.val.tolist()))
        path.write_text(f"%%MatrixMarket matrix coordinate real general\n{A.M} {A.N} {A.nnz}\n"
                        f"{body}\n")
        size = path.stat().st_size
        ts, tms = [], []
        X = None
        for i in range(steps + 1):
            tm = brm.MtxTiming()
            t0 = time.perf_counter()
            X = ctx.read_mtx_device(path, timing=tm)
            torch.cuda.synchronize()
            if i:
                ts.append(time.perf_counter() - t0)
                tms.append(tm)
        ok = (X.nnz == A.nnz and np.array_equal(X.col.cpu().numpy(), A.col)
              and np.array_equal(X.val.cpu().numpy().view(np.int64), A.val.view(np.int64)))
        sec = statistics.mean(ts)
        t0 = time.perf_counter()
        from oracle import mtx as omtx
        omtx.read(path)
        cpu_s = time.perf_counter() - t0
    return {
        "file": "A as real general .mtx, %r values", "bytes": int(size), "entries": int(A.nnz),
        "ms": round(sec * 1e3, 3), "mb_per_s": round(size / sec / 1e6, 1),
        "phases_ms": {k: round(statistics.mean(getattr(t, k) for t in tms) * 1e3, 3)
                      for k in ("read", "parse", "build")},
        "matches_input": bool(ok),
        "cpu_port_ms": round(cpu_s * 1e3, 1),
        "cpu_port": "oracle/mtx.py (numpy restatement of CSR::construct), 1 core",
    }


def batched_section(ctx, dev, stream, steps: int):
    """The uneven batch through brm_batch_precise (one pipeline for every
    pair) against a loop of plain per-pair brm_precise_device calls."""
    import torch
    import brmerge_gb300 as brm
    L = brm._native.lib()
    pairs = make_batch(BATCH_PAIRS, seed=7)
    products = sum(brm.compute_flop_host(A, B) for A, B in pairs)
    dpairs, keep = upload_pairs(pairs, dev)
    del pairs
    out = ctx.batch_precise_raw(dpairs)  # warm-up (pools, workspaces)
    nnz = int(out[1].numel())
    del out
    torch.cuda.synchronize(dev)

    def timed():
        ts = []
        l0 = L.brm_kernel_launches()
        for _ in range(steps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            out = ctx.batch_precise_raw(dpairs)
            e1.record(stream)
            torch.cuda.synchronize(dev)
            ts.append(e0.elapsed_time(e1))
            del out
        return statistics.mean(ts), (L.brm_kernel_launches() - l0) / steps

    default_ms, _ = timed()
    t0 = time.perf_counter()
    tuning = ctx.autotune(dpairs)  # bin thresholds chosen on this batch
    tune_s = time.perf_counter() - t0
    b_ms, launches = timed()
    # fixed structure, new values: one CUDA-graph launch per recomputation
    g = ctx.batch_graph(dpairs)
    gts = []
    for _ in range(steps + 1):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        g.launch(stream)
        e1.record(stream)
        torch.cuda.synchronize(dev)
        gts.append(e0.elapsed_time(e1))
    g.close()
    graph_ms = statistics.mean(gts[1:])
    ctx.set_tuning()  # the plain loop below runs with the defaults
    # plain per-call loop over the same pairs (one pass, results released)
    for a, b in dpairs[:16]:
        ctx.precise_device(a, b)
    torch.cuda.synchronize(dev)
    t0 = time.perf_counter()
    for a, b in dpairs:
        C = ctx.precise_device(a, b)
        del C
    torch.cuda.synchronize(dev)
    plain_s = time.perf_counter() - t0
    return {
        "tuning": tuning, "default_tuning_ms": round(default_ms, 3),
        "autotune_s": round(tune_s, 2),
        "graph_replay_ms": round(graph_ms, 3),
        "graph_replay_gflops": round(2 * products / (graph_ms / 1e3) / 1e9, 3),
        "workload": f"{BATCH_PAIRS} pairs, n_i~U[256,8192], rows lognormal(ln6,0.8) cap 256, f64",
        "pairs": BATCH_PAIRS, "products": int(products), "nnz_C": nnz,
        "ms": round(b_ms, 3), "gflops": round(2 * products / (b_ms / 1e3) / 1e9, 3),
        "plain_loop_ms": round(plain_s * 1e3, 2),
        "plain_gflops": round(2 * products / plain_s / 1e9, 3),
        "speedup_vs_plain": round(plain_s * 1e3 / b_ms, 2),
        "launches_per_batch": launches, "steps": steps,
    }


def served_section(dev, rate: float, nreq: int, seed: int = 11):
    """Poisson request stream into brm_server (continuous batching under a
    60 GiB cap): 70% uneven-batch sizes, 25% R-MAT n=2^16 degree 8, 5% R-MAT
    n=2^20 degree 16; float64 and float32 mixed.  Latency = submit -> result
    ready; the isolated latency of each class is one call on an idle GPU."""
    import queue as q
    import torch
    import brmerge_gb300 as brm
    rng = np.random.default_rng(seed)
    up = lambda X: brm.DeviceCSR.from_host(X, dev)
    small = [(up(A), up(B)) for A, B in make_batch(64, seed=seed)]
    small32 = [(up(A.astype(np.float32)), up(B.astype(np.float32)))
               for A, B in make_batch(16, seed=seed + 1)]
    r16h = [brm.gen_rmat(16, 8 << 16, seed=seed + 10 + i) for i in range(4)]
    r16 = [(up(A), up(A)) for A in r16h]
    r16_32 = [(up(A.astype(np.float32)),) * 2 for A in r16h[:2]]
    big = brm.gen_rmat(20, 16 << 20, seed=seed + 20)
    r20 = [(up(big), up(big))]
    r20_32 = [(up(big.astype(np.float32)),) * 2]
    del big
    classes = {"batch_size": (small, small32), "rmat16": (r16, r16_32), "rmat20": (r20, r20_32)}
    prob = [("batch_size", 0.70), ("rmat16", 0.25), ("rmat20", 0.05)]
    flops = {}
    ctx = brm.Context()
    iso = {}
    for name, (p64, _) in classes.items():
        a, b = p64[0]
        flops[name] = 2 * ctx.compute_flop(a, b)
        _, bound = ctx.upper_bound(a, b)
        if bound > (60 << 30):
            iso[name] = f"rejected: upper bound {bound / 2**30:.0f} GiB > 60 GiB cap"
            continue
        ts = []
        for _ in range(3):
            torch.cuda.synchronize(dev)
            t0 = time.perf_counter()
            try:
                C = ctx.precise_device(a, b)
                torch.cuda.synchronize(dev)
                ts.append(time.perf_counter() - t0)
                del C
            except brm.BrmError as e:  # nnz(C) beyond int32 CSR
                iso[name] = f"rejected: {e}"
                break
        if name not in iso:
            iso[name] = round(statistics.median(ts) * 1e3, 3)
    ctx.close()
    # the stream
    names = [p[0] for p in prob]
    kinds = rng.choice(len(names), size=nreq, p=[p[1] for p in prob])
    f32 = rng.random(nreq) < 0.5
    arrivals = np.cumsum(rng.exponential(1.0 / rate, nreq))
    srv = brm.Server(mem_cap_bytes=60 << 30, workers=2)
    tickets = q.Queue()
    rejected = {n: 0 for n in names}
    t_start = time.perf_counter()

    def submitter():
        for i in range(nreq):
            now = time.perf_counter() - t_start
            if arrivals[i] > now:
                time.sleep(arrivals[i] - now)
            name = names[kinds[i]]
            pool = classes[name][1 if f32[i] else 0]
            a, b = pool[int(rng.integers(len(pool)))]
            try:
                tickets.put((i, name, srv.submit(a, b)))
            except brm.BrmError:
                rejected[name] += 1
        tickets.put(None)

    lat = {n: [] for n in names}
    batch_sizes = []
    done_flop = 0
    th = threading.Thread(target=submitter)
    th.start()
    while True:
        item = tickets.get()
        if item is None:
            break
        i, name, t = item
        C, st = srv.wait(t, timeout=600.0)
        lat[name].append(st["latency_s"] * 1e3)
        batch_sizes.append(st["batch_size"])
        done_flop += flops[name]
        del C
    th.join()
    wall = time.perf_counter() - t_start
    srv.close()
    allv = [x for v in lat.values() for x in v]
    pct = lambda v, p: round(float(np.percentile(v, p)), 3) if v else None
    per_class = {n: {"n": len(v), "p50_ms": pct(v, 50), "p99_ms": pct(v, 99),
                     "isolated_ms": iso[n], "rejected": rejected[n]} for n, v in lat.items()}
    return {
        "offered_rate_per_s": rate, "requests": nreq, "completed": len(allv),
        "wall_s": round(wall, 3), "throughput_req_per_s": round(len(allv) / wall, 1),
        "gflops": round(done_flop / wall / 1e9, 3),
        "p50_ms": pct(allv, 50), "p99_ms": pct(allv, 99),
        "mean_batch": round(float(np.mean(batch_sizes)), 2) if batch_sizes else None,
        "classes": per_class, "mem_cap_gib": 60, "workers": 2,
    }


def run_ours(args):
    import torch
    import brmerge_gb300 as brm
    ws, rank, local = dist_env()
    if ws > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    dev = torch.device("cuda", local if ws > 1 else 0)
    torch.cuda.set_device(dev)
    A, desc = make_workload(args.workload, args.stencil_n)
    products = brm.compute_flop_host(A, A)
    stream = torch.cuda.current_stream(dev)
    ctx = brm.Context(stream=stream)
    dA = brm.DeviceCSR.from_host(A, dev)
    # the configured workload is C = A*A: B is the same device matrix
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)

    def step(timed_events=None):
        # one BRMerge-Precise call (brm_precise_device): symbolic and numeric
        # phases, callee-allocated C; the PreciseTiming fields split it
        if timed_events:
            timed_events[0].record(stream)
        C = ctx.precise_device(dA, dA, timing=timed_events[1] if timed_events else None)
        if timed_events:
            timed_events[2].record(stream)
        return C, C.nnz

    for _ in range(args.warmup):
        C, cnnz = step()
    torch.cuda.synchronize(dev)
    ev = [[torch.cuda.Event(enable_timing=True), brm.PreciseTiming(),
           torch.cuda.Event(enable_timing=True)] for _ in range(args.steps)]
    L = brm._native.lib()
    barrier(ws)
    torch.cuda.synchronize(dev)
    launches0 = L.brm_kernel_launches()
    with ClockSampler(dev.index if dev.index is not None else 0) as clk:
        for i in range(args.steps):
            flush.fill_(float(i))  # write 512 MB (> 129 MB L2) between steps
            C, cnnz = step(ev[i])
        torch.cuda.synchronize(dev)
    launches = L.brm_kernel_launches() - launches0
    barrier(ws)
    step_ms = [e[0].elapsed_time(e[2]) for e in ev]
    total_s = max_over_ranks(sum(step_ms) / 1e3, ws)
    value = 2 * products * args.steps * ws / total_s / 1e9
    sym_ms = statistics.mean((e[1].compute_flop + e[1].symbolic + e[1].prefix_sum_nnz) * 1e3
                             for e in ev)
    num_ms = statistics.mean(e[1].compute * 1e3 for e in ev)

    # roofline of the whole call (every kernel of the step, one stream):
    # compulsory bytes = read A and B once, write C once
    vb = 8
    alg_bytes = csr_bytes(A.M, A.nnz, vb) * 2 + csr_bytes(A.M, cnnz, vb)
    peak, peak_kind = peaks()
    achieved = alg_bytes / (statistics.mean(step_ms) / 1e3) / 1e9

    # e2e through the host drop-in (brm_precise): pinned inputs, host outputs
    pin = lambda a: torch.from_numpy(np.ascontiguousarray(a)).pin_memory().numpy()
    hA = brm.CSR(A.M, A.N, pin(A.rpt), pin(A.col), pin(A.val))
    for _ in range(max(1, args.warmup)):
        brm.brmerge_precise(hA, hA)
    e2e_t = []
    d2h = 0
    for _ in range(args.steps):
        t0 = time.perf_counter()
        Ch = brm.brmerge_precise(hA, hA)
        e2e_t.append(time.perf_counter() - t0)
        d2h = csr_bytes(A.M, len(Ch.col), vb)
        # the reference's driver releases C between calls, outside its timing
        # (BRMerge-SpGEMM/src/brmerge_precise.cpp:73-79)
        del Ch
    e2e_s = max_over_ranks(sum(e2e_t), ws)
    e2e_val = 2 * products * args.steps * ws / e2e_s / 1e9
    h2d = csr_bytes(A.M, A.nnz, vb)  # A and B are the same host arrays: copied once

    # BRMerge-Upper on the same workload (one call: C_bar, nnz scan, compaction)
    del C
    up_ms, Cu = device_steps(lambda: ctx.upper(dA, dA), dev, stream, flush, args.steps)
    del Cu
    upper = method_entry(up_ms, products, alg_bytes, peak)
    # the hash SpGEMM comparator: same structure, values in hardware order
    h_ms, Ch = device_steps(lambda: ctx.hash_device(dA, dA), dev, stream, flush, args.steps)
    del Ch
    hashc = method_entry(h_ms, products, alg_bytes, peak)

    batched = served = stencil = reader = None
    if not args.no_batch:
        reader = reader_section(ctx, A, max(1, min(args.steps, 3)))
        stencil = stencil_section(ctx, dev, stream, flush, max(1, min(args.steps, 5)), peak)
        batched = batched_section(ctx, dev, stream, steps=max(1, min(args.steps, 3)))
        served = [served_section(dev, rate, args.serve_requests) for rate in (2000.0, 400.0, 150.0)]
    if rank != 0:
        return
    cpu = cpu_baseline(A, budget_s=args.cpu_budget) if not args.no_cpu else None
    line = {
        "metric": "SpGEMM GFLOP/s (BRMerge-Precise, C=A*A)",
        "value": round(value, 3), "unit": "GFLOP/s", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(statistics.mean(step_ms), 4),
        "step_ms": {"min": round(min(step_ms), 4), "median": round(statistics.median(step_ms), 4),
                    "max": round(max(step_ms), 4)},
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic",
        "config": dict(desc, products=int(products), nnz_A=int(A.nnz), nnz_C=int(cnnz),
                       method="precise", call="brm_precise_device (one call)",
                       l2="flushed (512 MB write) between steps",
                       parallelism="replicas" if ws > 1 else "single_gpu",
                       symbolic_ms=round(sym_ms, 4), numeric_ms=round(num_ms, 4)),
        "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak,
                     "unit": "GB/s", "frac": round(achieved / peak, 4),
                     "traffic": measured_traffic() if args.workload == "rmat" else None,
                     "traffic_source": "profiles/rmat18_precise_launches.md (ncu DRAM bytes "
                                       "of every kernel of one call)",
                     "kernel": "whole Precise call (all kernels of a step)",
                     "peak_kind": peak_kind, "algorithmic_bytes": int(alg_bytes)},
        "e2e": {"value": round(e2e_val, 3), "unit": "GFLOP/s", "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h)},
        "clocks": clk.summary(),
        "gpu_launches": int(launches),
    }
    line["upper"] = dict(upper, call="brm_upper_device (one call)")
    line["hash_comparator"] = dict(hashc, call="brm_hash_device (values not in merge order)")
    if cpu is not None:
        line["cpu_baseline"] = cpu
    if stencil is not None:
        line["stencil"] = stencil
    if reader is not None:
        line["mtx_reader"] = reader
    if batched is not None:
        line["batched"] = batched
    if served is not None:
        line["served"] = served
    print(json.dumps(line), flush=True)
    if ws > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", choices=["rmat", "er", "stencil"], default="rmat")
    ap.add_argument("--stencil-n", type=int, default=128,
                    help="grid side of the stencil workload (profiling uses a smaller one)")
    ap.add_argument("--cpu-budget", type=float, default=15.0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-batch", action="store_true",
                    help="skip the uneven-batch and served-stream sections")
    ap.add_argument("--serve-requests", type=int, default=600)
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
