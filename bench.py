#!/usr/bin/env python3
"""Benchmark: BRMerge SpGEMM GFLOP/s and HBM-roofline fraction on one GB300.

Workload (default): C = A*A, A = R-MAT(a,b,c,d = .57,.19,.19,.05) with n = 2^18
and 2.35*n samples (duplicates removed: ~607k nnz, ~9e7 intermediate
products), float64, BRMerge-Precise, plain per-call GPU path.  A "step" is
one SpGEMM call.  GFLOP/s = 2 * intermediate products / time, the
reference's definition (BRMerge-SpGEMM/src/brmerge_precise.cpp:65-69).  The
matrices are generated here with numpy, so both arms multiply the same
inputs and the reference arm loads nothing of this library.

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
* side sections (--sections): ER n=16384 (the reference's CPU case) and the
             27-point stencil, each with its CPU baseline; the MatrixMarket
             reader; the 4096-pair uneven batch in float64 and float32 with
             its graph replay; the served request stream.
* checks  -- every timed result is compared with the oracle or with a
             result that is: the headline step bit for bit against the
             oracle, e2e / Upper against it, the hash comparator within the
             reference's 1e-9 compare, the stencil on three row blocks against
             the oracle, every pair of the batches against its plain call and
             sixteen against the oracle, every served result against its
             isolated call.  "verified" is true when all of them hold.

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
from types import SimpleNamespace

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

RMAT_SCALE = 18
RMAT_EDGE_FACTOR = 2.35


def csr_bytes(M: int, nnz: int, vbytes: int) -> int:
    return 4 * (M + 1) + nnz * (4 + vbytes)


# ---------------------------------------------------------------------------
# Workloads, generated here with numpy (seeded PCG64) so that both arms --
# this library and the reference algorithm on the host cores -- multiply the
# same matrices and the reference arm loads nothing of the library.
# ---------------------------------------------------------------------------
def host_csr(M, N, rpt, col, val):
    return SimpleNamespace(M=int(M), N=int(N), rpt=np.ascontiguousarray(rpt, np.int32),
                           col=np.ascontiguousarray(col, np.int32),
                           val=np.ascontiguousarray(val), nnz=int(len(col)))


def gen_rmat_np(scale: int, edges: int, a: float, b: float, c: float, seed: int):
    """R-MAT(a, b, c, d = 1-a-b-c) on 2^scale x 2^scale: `edges` samples, one
    quadrant draw per bit, duplicates removed, values U[-1, 1)."""
    rng = np.random.default_rng(seed)
    n = 1 << scale
    r = np.zeros(edges, np.int64)
    cc = np.zeros(edges, np.int64)
    ab, abc = a + b, a + b + c
    for bit in range(scale - 1, -1, -1):
        u = rng.random(edges)
        r |= (u >= ab).astype(np.int64) << bit
        cc |= (((u >= a) & (u < ab)) | (u >= abc)).astype(np.int64) << bit
    keys = np.unique((r << 32) | cc)
    rows = keys >> 32
    rpt = np.zeros(n + 1, np.int64)
    np.cumsum(np.bincount(rows, minlength=n), out=rpt[1:])
    return host_csr(n, n, rpt, keys & 0xFFFFFFFF, rng.uniform(-1.0, 1.0, len(keys)))


def gen_er_np(n: int, per_row: int, seed: int):
    """Erdos-Renyi: exactly per_row distinct uniform columns per row (sorted),
    values U[-1, 1)."""
    rng = np.random.default_rng(seed)
    cols = np.empty((n, per_row), np.int64)
    for i in range(n):
        cols[i] = np.sort(rng.choice(n, per_row, replace=False))
    rpt = np.arange(n + 1, dtype=np.int64) * per_row
    return host_csr(n, n, rpt, cols.ravel(), rng.uniform(-1.0, 1.0, n * per_row))


def gen_stencil27_np(m: int, seed: int, jitter: float = 1e-3):
    """27-point stencil on an m^3 grid: 26 on the diagonal, -1 off it, each
    entry plus U[-jitter, jitter); columns sorted within each row."""
    rng = np.random.default_rng(seed)
    n = m ** 3
    idx = np.arange(n, dtype=np.int64)
    x, y, z = idx % m, (idx // m) % m, idx // (m * m)
    cols = np.empty((n, 27), np.int32)
    ok = np.empty((n, 27), bool)
    j = 0
    for dz in (-1, 0, 1):
        for dy in (-1, 0, 1):
            for dx in (-1, 0, 1):
                ok[:, j] = ((x + dx >= 0) & (x + dx < m) & (y + dy >= 0) & (y + dy < m)
                            & (z + dz >= 0) & (z + dz < m))
                cols[:, j] = idx + (dz * m + dy) * m + dx
                j += 1
    rpt = np.zeros(n + 1, np.int64)
    np.cumsum(ok.sum(axis=1), out=rpt[1:])
    col = cols[ok]
    rows = np.repeat(idx, np.diff(rpt))
    val = np.where(col == rows, 26.0, -1.0) + rng.uniform(-jitter, jitter, len(col))
    return host_csr(n, n, rpt, col, val)


def make_workload(name: str, stencil_n: int = 128):
    if name == "rmat":
        n = 1 << RMAT_SCALE
        A = gen_rmat_np(RMAT_SCALE, int(RMAT_EDGE_FACTOR * n), 0.57, 0.19, 0.19, seed=0)
        desc = {"workload": "rmat_n2^18_ef2.35_AxA", "n": n, "a": 0.57, "b": 0.19, "c": 0.19,
                "seed": 0, "generator": "numpy PCG64"}
    elif name == "er":
        A = gen_er_np(16384, 8, seed=0)
        desc = {"workload": "er_n16384_8perrow_AxA", "n": 16384, "seed": 0,
                "generator": "numpy PCG64"}
    elif name == "stencil":
        A = gen_stencil27_np(stencil_n, seed=0)
        desc = {"workload": f"stencil27_{stencil_n}^3_AxA", "n": stencil_n ** 3, "seed": 0,
                "generator": "numpy PCG64"}
    else:
        raise SystemExit(f"unknown workload {name}")
    return A, desc


def products_of(A, B) -> int:
    """Intermediate products of A*B (2x this is the reference's flop count)."""
    return int(np.diff(B.rpt.astype(np.int64))[A.col].sum()) if A.nnz else 0


def row_block(A, r0: int, r1: int):
    """Rows [r0, r1) of A as a CSR of their own (the same per-row work)."""
    a0, a1 = int(A.rpt[r0]), int(A.rpt[r1])
    return host_csr(r1 - r0, A.N, A.rpt[r0:r1 + 1].astype(np.int64) - a0, A.col[a0:a1],
                    A.val[a0:a1])


# ---------------------------------------------------------------------------
# Result checks: structure bit-exact, values bit-exact unless a tolerance is
# given (the hash comparator sums in hardware order).
# ---------------------------------------------------------------------------
def same_csr(X, R, tol: float | None = None) -> bool:
    if not (np.array_equal(np.asarray(X.rpt), np.asarray(R.rpt))
            and np.array_equal(np.asarray(X.col), np.asarray(R.col))):
        return False
    xv, rv = np.asarray(X.val), np.asarray(R.val)
    if tol is None:
        return xv.dtype == rv.dtype and np.array_equal(xv.view(np.uint8), rv.view(np.uint8))
    d = np.abs(xv.astype(np.float64) - rv.astype(np.float64))
    return bool(np.all((d <= tol) | (d <= tol * np.abs(rv.astype(np.float64)))))


def rows_of(C, r0: int, r1: int):
    """Rows [r0, r1) of a host CSR result, row pointers from 0."""
    e0, e1 = int(C.rpt[r0]), int(C.rpt[r1])
    return SimpleNamespace(rpt=np.asarray(C.rpt[r0:r1 + 1], np.int64) - e0,
                           col=C.col[e0:e1], val=C.val[e0:e1])


def dev_equal(x, y) -> bool:
    """Bit equality of two device tensors (values compared as raw bits)."""
    import torch
    if x.shape != y.shape or x.dtype != y.dtype:
        return False
    if x.dtype == torch.float64:
        x, y = x.view(torch.int64), y.view(torch.int64)
    elif x.dtype == torch.float32:
        x, y = x.view(torch.int32), y.view(torch.int32)
    return bool(torch.equal(x, y))


def dev_same_csr(X, Y) -> bool:
    return dev_equal(X.rpt, Y.rpt) and dev_equal(X.col, Y.col) and dev_equal(X.val, Y.val)


def dev_digest(X):
    """Position-weighted sums of a device CSR's row pointers, columns and raw
    value bits (int64, wrapping), enqueued without a host synchronisation:
    a result that differs in any entry, or in the order of two, changes it
    with overwhelming probability."""
    import torch
    bits = X.val.view(torch.int64) if X.val.dtype == torch.float64 else \
        X.val.view(torch.int32).long()

    def wsum(x):
        w = torch.arange(1, x.numel() + 1, device=x.device, dtype=torch.int64)
        return (x.long() * w).sum()

    return torch.stack([wsum(X.rpt), wsum(X.col), wsum(bits)])


def traffic_record():
    """DRAM bytes of one Precise call on the R-MAT workload as recorded by an
    ncu capture of this bench (profiles/rmat18_precise_traffic.json); it is
    a recorded profile value, not a measurement of this run."""
    p = ROOT / "profiles" / "rmat18_precise_traffic.json"
    if p.exists():
        d = json.loads(p.read_text())
        return int(d["dram_bytes_per_call"]), {k: d[k] for k in ("captured", "commit", "command")
                                               if k in d}
    return None, None


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
    """The largest x over the ranks (a device tensor under NCCL, a host one
    under gloo)."""
    if ws == 1:
        return x
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(ws):
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()


def oracle_precise_timed(A, B, budget_s: float):
    """The oracle restatement of BRMerge-Precise on all host cores, timed the
    way the reference's driver times it (BRMerge-SpGEMM/src/
    brmerge_precise.cpp:68-82): one warm-up call, then the mean of up to ten
    calls within budget_s.  Returns (seconds per call, calls timed, threads,
    the warm-up call's result)."""
    import oracle
    oracle.build(with_ref=False)
    nt = oracle.max_threads()
    t0 = time.perf_counter()
    R = oracle.precise(A, B, nt)
    one = time.perf_counter() - t0
    reps = max(1, min(10, int(budget_s / max(one, 1e-3))))
    t0 = time.perf_counter()
    for _ in range(reps):
        oracle.precise(A, B, nt)
    return (time.perf_counter() - t0) / reps, reps, nt, R


def cpu_baseline_entry(products: int, sec: float, reps: int, nt: int, sample: str) -> dict:
    return {"value": round(2 * products / sec / 1e9, 4), "unit": "GFLOP/s", "cores": nt,
            "kind": "port",
            "sample": f"{sample}, 1 warm-up + mean of {reps} calls, {sec * 1e3:.1f} ms/call"}


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
    flop = products_of(A, A)

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


_BATCH_CACHE = {}


def make_batch(npairs: int, seed: int, dtype=np.float64):
    """Uneven batch: C_i = A_i * B_i, n_i ~ U[256, 8192], rows lognormal(ln 6,
    0.8) capped at 256, uniform random columns, values U[-1, 1].  The float32
    variant is the float64 batch with its values rounded to float32."""
    import brmerge_gb300 as brm
    key = (npairs, seed)
    if key not in _BATCH_CACHE:
        rng = np.random.default_rng(seed)
        ns = rng.integers(256, 8193, npairs)
        pairs = []
        for i, n in enumerate(ns):
            A = brm.gen_lognormal(int(n), int(n), seed=seed * 100003 + 2 * i)
            B = brm.gen_lognormal(int(n), int(n), seed=seed * 100003 + 2 * i + 1)
            pairs.append((A, B))
        _BATCH_CACHE[key] = pairs
    return [(A.astype(dtype), B.astype(dtype)) for A, B in _BATCH_CACHE[key]]


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


def stencil_section(ctx, dev, stream, flush, steps: int, peak: float, cpu_budget: float,
                    m: int = 128):
    """27-point stencil on m^3 (C = A*A, a 125-point stencil): Precise and
    Upper through the one-call device forms, the hash comparator beside them.
    Checked on three row blocks (first, middle, last 1/32 of the rows) against
    the oracle, which is also the CPU baseline on those blocks."""
    import brmerge_gb300 as brm
    S, _ = make_workload("stencil", m)
    products = products_of(S, S)
    dS = brm.DeviceCSR.from_host(S, dev)
    res = {"workload": f"stencil27_{m}^3_AxA", "n": S.M, "nnz_A": int(S.nnz),
           "products": int(products)}
    ms, C = device_steps(lambda: ctx.precise_device(dS, dS), dev, stream, flush, steps)
    res["nnz_C"] = int(C.nnz)
    alg = 2 * csr_bytes(S.M, S.nnz, 8) + csr_bytes(S.M, C.nnz, 8)
    Cp = C.to_host()
    del C
    res["precise"] = method_entry(ms, products, alg, peak)
    ms, C = device_steps(lambda: ctx.upper(dS, dS), dev, stream, flush, steps)
    res["upper"] = method_entry(ms, products, alg, peak)
    res["upper"]["verified_vs_precise"] = same_csr(C.to_host(), Cp)
    del C
    ms, C = device_steps(lambda: ctx.hash_device(dS, dS), dev, stream, flush, steps)
    res["hash_comparator"] = method_entry(ms, products, alg, peak)
    res["hash_comparator"]["verified_vs_precise_1e-9"] = same_csr(C.to_host(), Cp, tol=1e-9)
    del C, dS
    # oracle on sampled row blocks: the check of the Precise result and the
    # CPU baseline on the same blocks
    blk = max(1, S.M // 32)
    starts = [0, (S.M // 2) // blk * blk, S.M - blk]
    ok, sec_tot, prod_tot, reps_min, nt = True, 0.0, 0, 10, 1
    for r0 in starts:
        Sb = row_block(S, r0, r0 + blk)
        sec, reps, nt, R = oracle_precise_timed(Sb, S, cpu_budget / len(starts))
        ok &= same_csr(rows_of(Cp, r0, r0 + blk), R)
        sec_tot += sec
        prod_tot += products_of(Sb, S)
        reps_min = min(reps_min, reps)
    res["precise"]["verified_vs_oracle"] = bool(ok)
    res["verified"] = bool(ok and res["upper"]["verified_vs_precise"]
                           and res["hash_comparator"]["verified_vs_precise_1e-9"])
    res["cpu_baseline"] = cpu_baseline_entry(
        prod_tot, sec_tot, reps_min, nt,
        f"rows [0,{blk}), [{starts[1]},{starts[1] + blk}), [{starts[2]},{S.M}) of C (3/32 of "
        f"the rows, {prod_tot} products)")
    return res


def er_section(ctx, dev, stream, flush, steps: int, peak: float, cpu_budget: float):
    """Config 1, the reference's CPU case: Erdos-Renyi n=16384, exactly 8
    columns per row, C = A*A; one-call Precise on the GPU, the oracle on the
    host cores as its baseline and its check."""
    import brmerge_gb300 as brm
    A, desc = make_workload("er")
    products = products_of(A, A)
    dA = brm.DeviceCSR.from_host(A, dev)
    ms, C = device_steps(lambda: ctx.precise_device(dA, dA), dev, stream, flush, steps)
    Ch = C.to_host()
    del C
    alg = 2 * csr_bytes(A.M, A.nnz, 8) + csr_bytes(A.M, len(Ch.col), 8)
    sec, reps, nt, R = oracle_precise_timed(A, A, cpu_budget)
    res = dict(desc, products=int(products), nnz_C=int(len(Ch.col)))
    res["precise"] = method_entry(ms, products, alg, peak)
    res["verified"] = same_csr(Ch, R)
    res["cpu_baseline"] = cpu_baseline_entry(products, sec, reps, nt, "full workload")
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


def batch_views(out, pairs):
    """Per-pair views (rpt from 0, col, val) of a brm_batch_precise result."""
    crpt, ccol, cval, row_off, nnz_off, rpt_local = out
    views = []
    for i in range(len(pairs)):
        r0, r1 = int(row_off[i]), int(row_off[i + 1])
        n0, n1 = int(nnz_off[i]), int(nnz_off[i + 1])
        views.append(SimpleNamespace(rpt=rpt_local[r0 + i:r1 + i + 1], col=ccol[n0:n1],
                                     val=cval[n0:n1]))
    return views


def batched_section(ctx, dev, stream, steps: int, dtype=np.float64, tune: bool = True,
                    n_oracle: int = 16):
    """The uneven batch through brm_batch_precise (one pipeline for every
    pair) against a loop of plain per-pair brm_precise_device calls.  Every
    C_i of the batch (and of its graph replay) is checked bit for bit against
    the plain call on the same pair, and n_oracle pairs against the oracle."""
    import torch
    import brmerge_gb300 as brm
    import oracle
    L = brm._native.lib()
    pairs = make_batch(BATCH_PAIRS, seed=7, dtype=dtype)
    products = sum(products_of(A, B) for A, B in pairs)
    dpairs, keep = upload_pairs(pairs, dev)
    host_sample = pairs[:n_oracle]
    del pairs
    out = ctx.batch_precise_raw(dpairs)  # warm-up (pools, workspaces)
    nnz = int(out[1].numel())
    del out
    torch.cuda.synchronize(dev)

    def timed():
        ts = []
        l0 = L.brm_kernel_launches()
        out = None
        for _ in range(steps):
            del out
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            out = ctx.batch_precise_raw(dpairs)
            e1.record(stream)
            torch.cuda.synchronize(dev)
            ts.append(e0.elapsed_time(e1))
        return statistics.mean(ts), (L.brm_kernel_launches() - l0) / steps, out

    res = {}
    default_ms, _, out = timed()
    del out
    if tune:
        t0 = time.perf_counter()
        res["tuning"] = ctx.autotune(dpairs)  # bin thresholds chosen on this batch
        res["autotune_s"] = round(time.perf_counter() - t0, 2)
    b_ms, launches, out = timed()
    bviews = batch_views(out, dpairs)
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
    graph_ms = statistics.mean(gts[1:])
    graph_ok = all(dev_same_csr(x, y) for x, y in zip(g.results, bviews))
    g.close()
    # a new batch every launch: the pipeline captured once (capacities from
    # this batch + 25 %), run alternately on the pairs and on the pairs in
    # reverse order (another stacked structure), one graph launch per batch
    pipe = ctx.batch_pipe(dpairs, headroom=1.25)
    orders = [list(range(len(dpairs))), list(range(len(dpairs)))[::-1]]
    pts, pwall = [], []
    l0 = L.brm_kernel_launches()
    for i in range(steps + 1):
        batch = [dpairs[j] for j in orders[i % 2]]
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        t0 = time.perf_counter()
        e0.record(stream)
        pipe_out = pipe.run_raw(batch, stream)
        e1.record(stream)
        torch.cuda.synchronize(dev)
        pwall.append(time.perf_counter() - t0)
        pts.append(e0.elapsed_time(e1))
    pipe_launches = (L.brm_kernel_launches() - l0) / (steps + 1)
    pipe_ms = statistics.mean(pts[1:])
    pipe_order = orders[steps % 2]
    ctx.set_tuning()  # the plain loop below runs with the defaults
    # plain per-call loop over the same pairs (one pass; results kept for the check)
    for a, b in dpairs[:16]:
        ctx.precise_device(a, b)
    torch.cuda.synchronize(dev)
    plain = []
    t0 = time.perf_counter()
    for a, b in dpairs:
        plain.append(ctx.precise_device(a, b))
    torch.cuda.synchronize(dev)
    plain_s = time.perf_counter() - t0
    batch_ok = all(dev_same_csr(x, y) for x, y in zip(bviews, plain))
    pviews = batch_views((None,) + pipe_out[:1] + pipe_out[1:2] + pipe_out[2:5],
                         [dpairs[j] for j in pipe_order])
    pipe_ok = all(dev_same_csr(v, plain[j]) for v, j in zip(pviews, pipe_order))
    del pviews, pipe_out
    pipe.close()
    oracle.build(with_ref=False)
    nt = oracle.max_threads()
    oracle_ok = all(same_csr(SimpleNamespace(rpt=v.rpt.cpu().numpy(), col=v.col.cpu().numpy(),
                                             val=v.val.cpu().numpy()), oracle.precise(A, B, nt))
                    for v, (A, B) in zip(bviews, host_sample))
    del plain, bviews, out
    vt = "f64" if dtype == np.float64 else "f32"
    res.update({
        "default_tuning_ms": round(default_ms, 3),
        "graph_replay_ms": round(graph_ms, 3),
        "graph_replay_gflops": round(2 * products / (graph_ms / 1e3) / 1e9, 3),
        "workload": f"{BATCH_PAIRS} pairs, n_i~U[256,8192], rows lognormal(ln6,0.8) cap 256, "
                    f"{vt}",
        "pairs": BATCH_PAIRS, "products": int(products), "nnz_C": nnz,
        "ms": round(b_ms, 3), "gflops": round(2 * products / (b_ms / 1e3) / 1e9, 3),
        "plain_loop_ms": round(plain_s * 1e3, 2),
        "plain_gflops": round(2 * products / plain_s / 1e9, 3),
        "speedup_vs_plain": round(plain_s * 1e3 / b_ms, 2),
        "launches_per_batch": launches, "steps": steps,
        "pipeline": {"call": "brm_batch_pipe_run (one graph launch per new batch)",
                     "ms": round(pipe_ms, 3),
                     "gflops": round(2 * products / (pipe_ms / 1e3) / 1e9, 3),
                     "host_wall_ms": round(statistics.mean(pwall[1:]) * 1e3, 3),
                     "speedup_vs_plain": round(plain_s * 1e3 / pipe_ms, 2),
                     "graph_launches_per_batch": 1,
                     "kernels_per_batch": pipe_launches,
                     "batches": "pairs in order and reversed, alternately (a new structure "
                                "every launch)"},
        "verified": bool(batch_ok and graph_ok and oracle_ok and pipe_ok),
        "checks": {"every_pair_vs_plain_call": bool(batch_ok),
                   "graph_replay_vs_batch": bool(graph_ok),
                   "pipeline_every_pair_vs_plain_call": bool(pipe_ok),
                   f"first_{n_oracle}_pairs_vs_oracle": bool(oracle_ok)},
    })
    return res


def served_pools(dev, seed: int = 11):
    """Request pools of the served stream (70% uneven-batch sizes, 25% R-MAT
    n=2^16 degree 8, 5% R-MAT n=2^20 degree 16; float64 and float32), the
    isolated latency of each class (one call on an idle GPU) and the digest
    of every pool entry's isolated result."""
    import torch
    import brmerge_gb300 as brm
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
    flops, iso, alone = {}, {}, {}
    ctx = brm.Context()
    for name, pools in classes.items():
        _, bound = ctx.upper_bound(*pools[0][0])
        if bound > (60 << 30):
            continue
        for f32, pool in enumerate(pools):
            for j, (a, b) in enumerate(pool):
                try:
                    alone[(name, f32, j)] = dev_digest(ctx.precise_device(a, b))
                except brm.BrmError:
                    pass
    torch.cuda.synchronize(dev)
    for name, (p64, _) in classes.items():
        a, b = p64[0]
        flops[name] = 2 * ctx.compute_flop(a, b)
        _, bound = ctx.upper_bound(a, b)
        if bound > (60 << 30):
            iso[name] = f"rejected: upper bound {bound / 2**30:.0f} GiB > 60 GiB cap"
            continue
        ts = []
        for _ in range(5):
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
    return SimpleNamespace(classes=classes, flops=flops, iso=iso, alone=alone)


def served_run(dev, pools, rate: float, nreq: int, seed: int = 11, workers: int = 2,
               express: int = 1, express_sms: int = 0,
               mix=(("batch_size", 0.70), ("rmat16", 0.25), ("rmat20", 0.05))):
    """A Poisson request stream at `rate` into brm_server (continuous
    batching under a 60 GiB cap, `workers` general and `express` small-request
    workers).  Latency = submit -> result ready.  Every served result is
    checked against the same pair's isolated brm_precise_device result
    through on-device digests (dev_digest), compared after the stream so that
    the checks never stall the submitter or hold results."""
    import queue as q
    import torch
    import brmerge_gb300 as brm
    rng = np.random.default_rng(seed)
    classes, flops, iso, alone = pools.classes, pools.flops, pools.iso, pools.alone
    prob = list(mix)
    names = [p[0] for p in prob]
    kinds = rng.choice(len(names), size=nreq, p=[p[1] for p in prob])
    f32 = rng.random(nreq) < 0.5
    arrivals = np.cumsum(rng.exponential(1.0 / rate, nreq))
    srv = brm.Server(mem_cap_bytes=60 << 30, workers=workers, express_workers=express,
                     express_sms=express_sms)
    sm_split = srv.sms()
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
            j = int(rng.integers(len(pool)))
            a, b = pool[j]
            tickets.put((i, name, (name, int(f32[i]), j), srv.submit(a, b)))
        tickets.put(None)

    lat = {n: [] for n in names}
    batch_sizes = []
    done_flop = 0
    digests = []
    held = []  # (event, result): a result is released once its digest has run
    th = threading.Thread(target=submitter)
    th.start()
    while True:
        item = tickets.get()
        if item is None:
            break
        i, name, key, t = item
        try:
            C, st = srv.wait(t, timeout=600.0)
        except brm.BrmError:  # refused at admission (bound above the cap)
            rejected[name] += 1
            continue
        digests.append((key, dev_digest(C), st["batch_size"], C.nnz))
        ev = torch.cuda.Event()
        ev.record()
        held.append((ev, C))
        while held and held[0][0].query():
            held.pop(0)
        lat[name].append(st["latency_s"] * 1e3)
        batch_sizes.append(st["batch_size"])
        done_flop += flops[name]
        del C
    torch.cuda.synchronize(dev)
    held.clear()
    th.join()
    wall = time.perf_counter() - t_start
    srv.close()
    bad = [(key, bs, nnz) for key, d, bs, nnz in digests
           if key not in alone or not torch.equal(d, alone[key])]
    mismatches = len(bad)
    allv = [x for v in lat.values() for x in v]
    pct = lambda v, p: round(float(np.percentile(v, p)), 3) if v else None
    per_class = {n: {"n": len(v), "p50_ms": pct(v, 50), "p99_ms": pct(v, 99),
                     "isolated_ms": iso[n], "rejected": rejected[n]} for n, v in lat.items()}
    for n, c in per_class.items():
        if c["p99_ms"] is not None and isinstance(c["isolated_ms"], float):
            c["p99_over_isolated"] = round(c["p99_ms"] / c["isolated_ms"], 2)
    return {
        "offered_rate_per_s": rate, "requests": nreq, "completed": len(allv),
        "wall_s": round(wall, 3), "throughput_req_per_s": round(len(allv) / wall, 1),
        "gflops": round(done_flop / wall / 1e9, 3),
        "p50_ms": pct(allv, 50), "p99_ms": pct(allv, 99),
        "mean_batch": round(float(np.mean(batch_sizes)), 2) if batch_sizes else None,
        "classes": per_class, "mem_cap_gib": 60, "workers": workers, "express_workers": express,
        "sm_partition": {"express_sms": sm_split[0], "other_sms": sm_split[1]},
        "verified": mismatches == 0,
        "checks": {"served_results_vs_isolated_call_mismatches": mismatches,
                   "first_mismatches (class, f32, pool index, batch size, nnz)":
                       [list(k) + [bs, nnz] for k, bs, nnz in bad[:8]]},
    }


def served_section(dev, nreq: int, rates=(2000.0, 1000.0, 600.0, 400.0, 250.0, 150.0)):
    """The served stream at several offered rates, and the largest rate at
    which the small class (uneven-batch sizes) keeps p99 within 2x its
    isolated latency; the same for a stream of small requests alone (no
    R-MAT requests beside them)."""
    pools = served_pools(dev)
    runs = [served_run(dev, pools, r, nreq) for r in rates]
    ok = [r["offered_rate_per_s"] for r in runs
          if r["classes"]["batch_size"].get("p99_over_isolated", 1e9) <= 2.0]
    small = [served_run(dev, pools, r, nreq, mix=(("batch_size", 1.0),))
             for r in (2000.0, 1000.0, 400.0)]
    ok_small = [r["offered_rate_per_s"] for r in small
                if r["classes"]["batch_size"].get("p99_over_isolated", 1e9) <= 2.0]
    return {"runs": runs,
            "small_class_max_rate_p99_within_2x_isolated": max(ok) if ok else None,
            "small_only_runs": small,
            "small_only_max_rate_p99_within_2x_isolated": max(ok_small) if ok_small else None,
            "verified": all(r["verified"] for r in runs + small)}


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
    sections = set(args.sections.split(",")) if args.sections else set(ALL_SECTIONS)
    if args.no_batch:
        sections -= {"reader", "stencil", "er", "batch", "batch32", "served"}
    if args.no_cpu:
        sections.discard("cpu")
    A, desc = make_workload(args.workload, args.stencil_n)
    products = products_of(A, A)
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
    phase_ms = {k: round(statistics.mean(getattr(e[1], k) for e in ev) * 1e3, 4)
                for k in ("compute_flop", "prefix_sum_flop", "load_balance", "symbolic",
                          "prefix_sum_nnz", "compute")}
    Cref = C.to_host()  # the last timed step's result, checked below
    del C

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
    e2e_ok = True
    for i in range(args.steps):
        t0 = time.perf_counter()
        Ch = brm.brmerge_precise(hA, hA)
        e2e_t.append(time.perf_counter() - t0)
        d2h = csr_bytes(A.M, len(Ch.col), vb)
        if i + 1 == args.steps:
            e2e_ok = same_csr(Ch, Cref)
        # the reference's driver releases C between calls, outside its timing
        # (BRMerge-SpGEMM/src/brmerge_precise.cpp:73-79)
        del Ch
    e2e_s = max_over_ranks(sum(e2e_t), ws)
    e2e_val = 2 * products * args.steps * ws / e2e_s / 1e9
    h2d = csr_bytes(A.M, A.nnz, vb)  # A and B are the same host arrays: copied once

    # BRMerge-Upper on the same workload (one call: C_bar, nnz scan, compaction)
    up_ms, Cu = device_steps(lambda: ctx.upper(dA, dA), dev, stream, flush, args.steps)
    upper = method_entry(up_ms, products, alg_bytes, peak)
    upper["verified_vs_precise"] = same_csr(Cu.to_host(), Cref)
    del Cu
    # the split path (brm_symbolic + brm_numeric): a structure-only symbolic
    # pass, then the values written straight into C -- the A/B of the
    # one-call form, which computes the mid rows during planning and moves
    # them into C afterwards
    sp_ms, Csp = device_steps(lambda: ctx.precise(dA, dA), dev, stream, flush, args.steps)
    split = method_entry(sp_ms, products, alg_bytes, peak)
    split["verified_vs_precise"] = same_csr(Csp.to_host(), Cref)
    del Csp
    # the hash SpGEMM comparator: same structure, values in hardware order
    h_ms, Chs = device_steps(lambda: ctx.hash_device(dA, dA), dev, stream, flush, args.steps)
    hashc = method_entry(h_ms, products, alg_bytes, peak)
    hashc["verified_vs_precise_1e-9"] = same_csr(Chs.to_host(), Cref, tol=1e-9)
    del Chs

    side = {}
    if "reader" in sections:
        side["mtx_reader"] = reader_section(ctx, A, max(1, min(args.steps, 3)))
    if "er" in sections:
        side["er"] = er_section(ctx, dev, stream, flush, max(1, min(args.steps, 5)), peak,
                                args.cpu_budget)
    if "stencil" in sections:
        side["stencil"] = stencil_section(ctx, dev, stream, flush, max(1, min(args.steps, 5)),
                                          peak, args.cpu_budget, args.stencil_n)
    if "batch" in sections:
        side["batched"] = batched_section(ctx, dev, stream, steps=max(1, min(args.steps, 3)))
    if "batch32" in sections:
        side["batched_f32"] = batched_section(ctx, dev, stream, steps=max(1, min(args.steps, 3)),
                                              dtype=np.float32, tune=False)
    if "served" in sections:
        side["served"] = served_section(dev, args.serve_requests)
    if rank != 0:
        return
    # the oracle on the host cores: the check of the headline result and,
    # timed, the CPU baseline
    cpu = None
    import oracle
    if "cpu" in sections:
        sec, reps, nt, R = oracle_precise_timed(A, A, args.cpu_budget)
        cpu = cpu_baseline_entry(products, sec, reps, nt, "full workload")
    else:
        oracle.build(with_ref=False)
        R = oracle.precise(A, A, oracle.max_threads())
    precise_ok = same_csr(Cref, R)
    del R
    traffic, traffic_src = traffic_record() if args.workload == "rmat" else (None, None)
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
                       phase_ms=phase_ms),
        "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak,
                     "unit": "GB/s", "frac": round(achieved / peak, 4),
                     "traffic": traffic,
                     "traffic_recorded": traffic_src,
                     "kernel": "whole Precise call (all kernels of a step)",
                     "peak_kind": peak_kind, "algorithmic_bytes": int(alg_bytes)},
        "e2e": {"value": round(e2e_val, 3), "unit": "GFLOP/s", "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h)},
        "clocks": clk.summary(),
        "gpu_launches": int(launches),
    }
    line["upper"] = dict(upper, call="brm_upper_device (one call)")
    line["split_path"] = dict(split, call="brm_symbolic + brm_numeric (no mid-row scratch)")
    line["hash_comparator"] = dict(hashc, call="brm_hash_device (values not in merge order)")
    if cpu is not None:
        line["cpu_baseline"] = cpu
    line.update(side)
    checks = {"precise_vs_oracle": precise_ok, "e2e_vs_precise": e2e_ok,
              "upper_vs_precise": upper["verified_vs_precise"],
              "split_vs_precise": split["verified_vs_precise"],
              "hash_vs_precise_1e-9": hashc["verified_vs_precise_1e-9"]}
    for k, v in side.items():
        if isinstance(v, dict) and "verified" in v:
            checks[k] = v["verified"]
        elif isinstance(v, list):
            checks[k] = all(x.get("verified", False) for x in v)
    line["checks"] = checks
    line["verified"] = all(checks.values())
    print(json.dumps(line), flush=True)
    if ws > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


ALL_SECTIONS = ("cpu", "reader", "er", "stencil", "batch", "batch32", "served")


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
    ap.add_argument("--sections", default="",
                    help="comma list of side sections to run (default all: "
                         + ",".join(ALL_SECTIONS) + "); the headline step, e2e, Upper and "
                         "hash legs always run")
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
