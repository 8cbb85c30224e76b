"""Times the oracle restatement against the reference's own compiled
BRMerge-Precise (oracle/_ref) on the bench's workloads, on all host cores,
alternating the two so that both see the same machine state.  Prints the
minimum and median of `runs` calls each and their ratio.  Test
infrastructure: it shows that the restatement, which stands in for the
reference on hosts without the reference tree, is no faster than the
reference itself.

    python oracle/time_port_vs_ref.py [runs]
"""
from __future__ import annotations

import statistics
import sys
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(ROOT))


def main(runs: int = 7) -> None:
    import bench
    import oracle
    oracle.build(with_ref=True)
    if not oracle.ref_available():
        raise SystemExit("the reference library is not built (needs the reference tree)")
    nt = oracle.max_threads()
    for name in ("rmat", "er"):
        A, desc = bench.make_workload(name)
        calls = {"port": lambda: oracle.precise(A, A, nt),
                 "reference": lambda: oracle.ref_precise(A, A, nt)[0]}
        outs = {k: f() for k, f in calls.items()}  # warm-up; results must agree
        assert bench.same_csr(outs["port"], outs["reference"]), name
        ts = {k: [] for k in calls}
        for _ in range(runs):
            for k, f in calls.items():
                t0 = time.perf_counter()
                f()
                ts[k].append(time.perf_counter() - t0)
        mn = {k: min(v) for k, v in ts.items()}
        md = {k: statistics.median(v) for k, v in ts.items()}
        print(f"{desc['workload']}: {nt} threads, {runs} calls each | "
              f"port min {mn['port'] * 1e3:.1f} ms median {md['port'] * 1e3:.1f} ms | "
              f"reference min {mn['reference'] * 1e3:.1f} ms median {md['reference'] * 1e3:.1f} ms"
              f" | port/reference (min) {mn['port'] / mn['reference']:.3f}")


if __name__ == "__main__":
    main(int(sys.argv[1]) if len(sys.argv) > 1 else 7)
