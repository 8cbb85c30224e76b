"""Synthetic generators: determinism, invariants and the configured shapes (CPU)."""
import numpy as np

import brmerge_gb300 as brm


def test_er_config_shape():
    A = brm.gen_er(16384, 8, seed=0)
    A.check()
    assert A.nnz == 16384 * 8
    assert brm.compute_flop_host(A, A) == 16384 * 8 * 8
    B = brm.gen_er(16384, 8, seed=0)
    assert np.array_equal(A.col, B.col) and np.array_equal(A.val, B.val)
    assert np.abs(A.val).max() <= 1.0


def test_rmat_config_shape():
    n = 1 << 18
    A = brm.gen_rmat(18, int(2.35 * n), seed=0)
    A.check()
    assert 5.5e5 < A.nnz < 6.5e5            # ~600k nnz, avg ~2.3 per row
    lens = np.diff(A.rpt)
    assert lens.max() > 1000                 # heavy tail
    f = brm.compute_flop_host(A, A)
    assert 8e7 < f < 1.1e8


def test_stencil_closed_form():
    for n in (3, 5, 8):
        A = brm.gen_stencil27(n)
        A.check()
        assert A.nnz == (3 * n - 2) ** 3
        d = A.val[A.col == np.repeat(np.arange(A.M), np.diff(A.rpt))]
        assert np.all(np.abs(d - 26) <= 1e-3)


def test_stencil_products_closed_form():
    # per dimension: sum over x of (neighbours of x) * (neighbours of neighbours)
    n = 6
    A = brm.gen_stencil27(n)
    per = sum(
        sum(len([z for z in (y - 1, y, y + 1) if 0 <= z < n]) for y in (x - 1, x, x + 1) if 0 <= y < n)
        for x in range(n))
    assert brm.compute_flop_host(A, A) == per ** 3


def test_lognormal_and_uniform():
    L = brm.gen_lognormal(4096, 3000, seed=1)
    L.check()
    lens = np.diff(L.rpt)
    assert lens.max() <= 256 and 5.0 < lens.mean() < 12.0
    U = brm.gen_uniform(100, 50, 50, seed=2)
    U.check()
    assert np.diff(U.rpt).max() <= 50
