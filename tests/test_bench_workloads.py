"""The bench's numpy workload generators (both bench arms multiply these
matrices): valid CSR, the configured shapes and statistics, and the helpers
the bench uses to check its results.  CPU only."""
import numpy as np
import pytest

import bench
import brmerge_gb300 as brm


def _valid(X):
    brm.CSR(X.M, X.N, X.rpt, X.col, X.val).check()


def test_rmat_workload_shape_and_stats():
    A, desc = bench.make_workload("rmat")
    _valid(A)
    assert A.M == A.N == 1 << 18 and desc["n"] == A.M
    # ~2.35 n samples with duplicates removed: about 6.0-6.3e5 nnz
    assert 590_000 < A.nnz < 630_000
    prod = bench.products_of(A, A)
    assert 7e7 < prod < 1.2e8
    assert np.all(np.abs(A.val) <= 1.0)
    # seeded: the same matrix every time
    B, _ = bench.make_workload("rmat")
    assert bench.same_csr(A, B)


def test_er_workload_exact_row_length():
    A, _ = bench.make_workload("er")
    _valid(A)
    assert A.M == 16384 and np.all(np.diff(A.rpt) == 8)
    assert bench.products_of(A, A) == 16384 * 64


@pytest.mark.parametrize("m", [3, 6, 16])
def test_stencil_workload_matches_closed_forms(m):
    S = bench.gen_stencil27_np(m, seed=0)
    _valid(S)
    lo = 3 * m - 2  # entries per grid axis: 3 per point, one fewer at each end
    assert S.nnz == lo ** 3
    assert bench.products_of(S, S) == (3 * lo - 4) ** 3  # 1142^3 at m = 128
    # structure identical to the library's own generator (values differ: PRNG)
    G = brm.gen_stencil27(m)
    assert np.array_equal(S.rpt, G.rpt) and np.array_equal(S.col, G.col)
    diag = S.col == np.repeat(np.arange(S.M), np.diff(S.rpt))
    assert np.all(np.abs(S.val[diag] - 26.0) <= 1e-3)
    assert np.all(np.abs(S.val[~diag] + 1.0) <= 1e-3)


def test_row_block_and_checks():
    A = bench.gen_stencil27_np(5, seed=1)
    blk = bench.row_block(A, 10, 40)
    _valid(blk)
    assert blk.M == 30 and np.array_equal(blk.col, A.col[A.rpt[10]:A.rpt[40]])
    assert bench.same_csr(A, A)
    B = bench.host_csr(A.M, A.N, A.rpt, A.col, A.val.copy())
    B.val[3] = np.nextafter(B.val[3], 1.0)
    assert not bench.same_csr(A, B)            # bit-exact compare sees one ulp
    assert bench.same_csr(A, B, tol=1e-9)      # the reference's compare does not
    r = bench.rows_of(A, 10, 40)
    assert np.array_equal(r.col, blk.col) and r.rpt[0] == 0
