"""The hash SpGEMM comparator (brm_hash_device) against the oracle.

Structure (row pointers, columns) must be bit-exact.  Values are sums in an
order the hardware picks, so they are compared with the reference's own
tolerance for SpGEMM results, |d| < 1e-9 or |d| < 1e-9 |v|
(BRMerge-SpGEMM/src/CSR.cpp:214-253); float32 runs within 1e-5 relative of
the float64 oracle.
"""
import numpy as np
import pytest

import brmerge_gb300 as brm
from conftest import GOLDEN_NAMES, load_golden

pytestmark = pytest.mark.gpu

EPS = 1e-9      # CSR.cpp:223
F32_RTOL = 1e-5


@pytest.fixture(scope="module")
def ctx():
    import torch  # noqa: F401
    c = brm.Context()
    yield c
    c.close()


def gpu_hash(ctx, A, B):
    return ctx.hash_device(brm.DeviceCSR.from_host(A), brm.DeviceCSR.from_host(B)).to_host()


def assert_hash_close(C, R, what, f32=False):
    assert C.M == R.M and C.N == R.N, what
    assert np.array_equal(np.asarray(C.rpt), np.asarray(R.rpt)), f"{what}: rpt"
    assert np.array_equal(np.asarray(C.col), np.asarray(R.col)), f"{what}: col"
    got = np.asarray(C.val, np.float64)
    ref = np.asarray(R.val, np.float64)
    d = np.abs(got - ref)
    if f32:
        ok = d <= F32_RTOL * np.maximum(1.0, np.abs(ref))
    else:
        ok = (d < EPS) | (d < EPS * np.abs(got))
    assert ok.all(), f"{what}: {int((~ok).sum())} values differ, max |d| {float(d.max())}"


@pytest.mark.parametrize("name", GOLDEN_NAMES)
def test_hash_golden(ctx, name):
    A, B, C = load_golden(name)
    assert_hash_close(gpu_hash(ctx, A, B), C, name)


def _cases():
    yield "er2048", brm.gen_er(2048, 8, seed=3), None
    yield "rmat12", brm.gen_rmat(12, int(2.35 * 4096), seed=4), None
    yield "rmat15", brm.gen_rmat(15, int(2.35 * 32768), seed=5), None  # dense-accumulator rows
    yield "stencil10", brm.gen_stencil27(10, seed=6), None
    yield "lognormal", brm.gen_lognormal(3000, 2500, seed=7), brm.gen_lognormal(2500, 4000, seed=8)
    yield "uniform_dense", brm.gen_uniform(64, 400, 300, seed=9), brm.gen_uniform(400, 500, 200, seed=10)
    yield "wide_span", brm.gen_uniform(50, 2000, 80, seed=11), brm.gen_uniform(2000, 1_500_000, 60, seed=12)


CASES = list(_cases())


@pytest.mark.parametrize("name,A,B", CASES, ids=[c[0] for c in CASES])
def test_hash_matches_oracle(ctx, oracle_mod, name, A, B):
    B = A if B is None else B
    R = oracle_mod.precise(A, B)
    assert_hash_close(gpu_hash(ctx, A, B), R, name)


@pytest.mark.parametrize("name,A,B", CASES[:5], ids=[c[0] for c in CASES[:5]])
def test_hash_f32(ctx, oracle_mod, name, A, B):
    B = A if B is None else B
    R = oracle_mod.precise(A, B)
    C = gpu_hash(ctx, A.astype(np.float32), B.astype(np.float32))
    assert C.val.dtype == np.float32
    assert_hash_close(C, R, name + " f32", f32=True)


def test_hash_bins_at_their_edges(ctx, oracle_mod):
    """Rows of exactly 0, 1, 32, 33, 512, 513, 4096 and 4097 products (every
    bin boundary) and a row whose lists are all empty."""
    rng = np.random.default_rng(31)
    K, N = 9000, 9000
    blen = np.where(np.arange(K) % 3 != 0, 1, rng.integers(0, 4, K)).astype(np.int64)
    Brows = [sorted(rng.choice(N, int(n), replace=False)) for n in blen]
    Bm = brm.CSR(K, N, np.concatenate([[0], np.cumsum(blen)]).astype(np.int32),
                 np.array([c for r in Brows for c in r], np.int32), rng.uniform(-1, 1, int(blen.sum())))
    ones = np.nonzero(blen == 1)[0]
    Arows = []
    for target in (0, 1, 32, 33, 512, 513, 4096, 4097):
        Arows.append(sorted(rng.choice(ones, target, replace=False)) if target else [])
    Arows.append(list(np.nonzero(blen == 0)[0][:50]))  # only empty B rows
    A = brm.CSR(len(Arows), K, np.concatenate([[0], np.cumsum([len(r) for r in Arows])]).astype(np.int32),
                np.array([c for r in Arows for c in r], np.int32),
                rng.uniform(-1, 1, sum(len(r) for r in Arows)))
    R = oracle_mod.precise(A, Bm)
    assert_hash_close(gpu_hash(ctx, A, Bm), R, "bin edges")


def test_hash_single_column(ctx, oracle_mod):
    K = 5000
    B = brm.CSR(K, 10, np.arange(K + 1, dtype=np.int32), np.full(K, 5, np.int32),
                np.random.default_rng(1).uniform(-1, 1, K))
    for n in (20, 300, 3000, 5000):
        A = brm.CSR(1, K, np.array([0, n], np.int32), np.arange(n, dtype=np.int32),
                    np.random.default_rng(n).uniform(-1, 1, n))
        R = oracle_mod.precise(A, B)
        assert_hash_close(gpu_hash(ctx, A, B), R, f"one column, {n} products")


def test_hash_empty(ctx):
    A = brm.CSR(3, 4, np.zeros(4, np.int32), np.zeros(0, np.int32), np.zeros(0))
    B = brm.CSR(4, 5, np.array([0, 1, 1, 2, 2], np.int32), np.array([0, 3], np.int32), np.ones(2))
    C = gpu_hash(ctx, A, B)
    assert list(C.rpt) == [0, 0, 0, 0] and len(C.col) == 0
