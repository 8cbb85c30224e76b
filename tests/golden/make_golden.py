"""Generate the golden SpGEMM fixtures from the reference itself.

Runs the reference's own brmerge_precise and brmerge_upper
(BRMerge-SpGEMM/inc/spgemm.h, compiled unmodified into oracle/_ref by
oracle/build_ref.sh) on small seeded inputs and stores inputs and outputs as
.npz files in this directory.  Needs the reference sources (present where the
fixtures are generated, not on the GPU host); the fixtures are committed.

    python tests/golden/make_golden.py
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT))

import oracle  # noqa: E402
from brmerge_gb300 import csr as gen  # noqa: E402
from brmerge_gb300.csr import CSR  # noqa: E402


def from_rows(rows, ncols, seed):
    """CSR from a list of sorted column lists, values U[-1,1] from `seed`."""
    rng = np.random.default_rng(seed)
    rpt = np.zeros(len(rows) + 1, np.int32)
    for i, r in enumerate(rows):
        rpt[i + 1] = rpt[i] + len(r)
    col = np.array([c for r in rows for c in r], np.int32)
    val = rng.uniform(-1, 1, len(col))
    return CSR(len(rows), ncols, rpt, col, val)


def edge_case():
    """Empty rows, empty B rows inside non-empty A rows, a single list,
    odd list counts, exact cancellation, signed zeros."""
    B_rows = [[0, 3, 5], [], [1, 3], [0, 1, 2, 3, 4, 5], [5], [], [2, 4], [3]]
    B = from_rows(B_rows, 6, 11)
    B.val[B.rpt[2]] = 0.5     # B(2,1)
    B.val[B.rpt[3] + 1] = 0.5  # B(3,1)
    B.val[B.rpt[4]] = -0.0    # B(4,5) = -0
    A_rows = [[], [1], [0, 1, 2], [1, 5], [0, 2, 3, 4, 6, 7, 1 + 0], [4], [2, 3],
              [0, 1, 2, 3, 4, 5, 6, 7], [6, 7], []]
    A_rows = [sorted(set(r)) for r in A_rows]
    A = from_rows(A_rows, 8, 12)
    # row 6: A(6,2)*B(2,1) + A(6,3)*B(3,1) cancels exactly
    A.val[A.rpt[6]] = 1.0
    A.val[A.rpt[6] + 1] = -1.0
    return A, B


def cases():
    yield "er64", gen.gen_er(64, 4, seed=1), None
    r = gen.gen_rmat(10, int(2.35 * 1024), seed=2)
    yield "rmat10", r, None
    yield "stencil_6x5x4", gen.gen_stencil27(6, 5, 4, seed=3), None
    yield "lognormal_nonsquare", gen.gen_lognormal(200, 300, seed=4), gen.gen_lognormal(300, 250, seed=5)
    A, B = edge_case()
    yield "edge", A, B
    yield "wide_cols", gen.gen_uniform(40, 3000, 30, seed=6), gen.gen_uniform(3000, 300000, 12, seed=7)


def main():
    oracle.build()
    if not oracle.ref_available():
        raise SystemExit("reference library unavailable; cannot generate fixtures")
    for name, A, B in cases():
        B = A if B is None else B
        A.check()
        B.check()
        Cp, _ = oracle.ref_precise(A, B, nthreads=2)
        Cu, _ = oracle.ref_upper(A, B, nthreads=2)
        assert np.array_equal(Cp.rpt, Cu.rpt) and np.array_equal(Cp.col, Cu.col)
        assert np.array_equal(Cp.val.view(np.int64), Cu.val.view(np.int64))
        np.savez_compressed(
            HERE / f"{name}.npz",
            M=A.M, K=A.N, N=B.N,
            A_rpt=A.rpt, A_col=A.col, A_val=A.val,
            B_rpt=B.rpt, B_col=B.col, B_val=B.val,
            C_rpt=Cp.rpt, C_col=Cp.col, C_val=Cp.val)
        print(f"{name}: M={A.M} K={A.N} N={B.N} nnzA={A.nnz} nnzB={B.nnz} nnzC={len(Cp.col)}")


if __name__ == "__main__":
    main()
