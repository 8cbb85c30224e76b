"""Batches: many independent C_i = A_i * B_i in one pipeline (brm_batch_precise).

Every C_i of a batch must be bit-identical to the oracle's BRMerge-Precise
of its own pair and to a separate brm_precise_device call, whatever else is
in the batch (uneven sizes, empty matrices, rectangular pairs, float32).
"""
import numpy as np
import pytest

import brmerge_gb300 as brm
from conftest import assert_same_csr

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    import torch  # noqa: F401
    c = brm.Context()
    yield c
    c.close()


def _empty(M, N):
    return brm.CSR(M, N, np.zeros(M + 1, np.int32), np.zeros(0, np.int32), np.zeros(0))


def _pairs(seed=0, n=40):
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        kind = i % 6
        if kind == 0:
            m = int(rng.integers(256, 2048))
            A = brm.gen_lognormal(m, m, seed=seed * 1000 + i)
            B = brm.gen_lognormal(m, m, seed=seed * 1000 + i + 500)
        elif kind == 1:
            A = brm.gen_rmat(10, int(2.35 * 1024), seed=seed * 1000 + i)
            B = A
        elif kind == 2:  # rectangular
            m, k, nn = (int(x) for x in rng.integers(50, 900, 3))
            A = brm.gen_uniform(m, k, 12, seed=seed * 1000 + i)
            B = brm.gen_uniform(k, nn, 30, seed=seed * 1000 + i + 500)
        elif kind == 3:  # empty A rows / empty matrices
            A = _empty(int(rng.integers(0, 5)), 17)
            B = brm.gen_uniform(17, 40, 5, seed=seed * 1000 + i)
        elif kind == 4:  # heavy rows inside a batch
            A = brm.gen_uniform(40, 3000, 400, seed=seed * 1000 + i)
            B = brm.gen_uniform(3000, 5000, 60, seed=seed * 1000 + i + 500)
        else:
            A = brm.gen_er(512, 8, seed=seed * 1000 + i)
            B = _empty(512, 300) if i % 12 == 5 else brm.gen_er(512, 8, seed=seed * 1000 + i + 1)
        out.append((A, B))
    return out


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_batch_matches_oracle_and_single_calls(ctx, oracle_mod, dtype):
    pairs = [(A.astype(dtype), B.astype(dtype)) for A, B in _pairs(seed=1)]
    dpairs = [(brm.DeviceCSR.from_host(A), brm.DeviceCSR.from_host(B)) for A, B in pairs]
    Cs = ctx.batch_precise(dpairs)
    assert len(Cs) == len(pairs)
    for i, ((A, B), (dA, dB), C) in enumerate(zip(pairs, dpairs, Cs)):
        got = C.to_host()
        assert got.M == A.M and got.N == B.N
        assert_same_csr(got, oracle_mod.precise(A, B), f"pair {i}")
        assert_same_csr(got, ctx.precise_device(dA, dB).to_host(), f"pair {i} single call")


def test_batch_same_alone_and_in_mix(ctx, oracle_mod):
    """A pair gives the same C alone, first, last and in the middle of a batch."""
    pairs = _pairs(seed=2, n=24)
    dpairs = [(brm.DeviceCSR.from_host(A), brm.DeviceCSR.from_host(B)) for A, B in pairs]
    probe = dpairs[6]
    alone = ctx.batch_precise([probe])[0].to_host()
    for order in ([probe] + dpairs, dpairs + [probe], dpairs[:10] + [probe] + dpairs[10:]):
        Cs = ctx.batch_precise(order)
        k = next(j for j, p in enumerate(order) if p is probe)
        assert_same_csr(Cs[k].to_host(), alone, "probe in mix")


def test_batch_empty_and_rejects_mismatch(ctx):
    assert ctx.batch_precise([]) == []
    A = brm.DeviceCSR.from_host(brm.gen_er(64, 4, seed=1))
    B = brm.DeviceCSR.from_host(brm.gen_uniform(65, 10, 3, seed=2))
    with pytest.raises(brm.BrmError):
        ctx.batch_precise([(A, B)])


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_batch_graph_replays_new_values(ctx, oracle_mod, dtype):
    """Fixed structure, new values: every graph launch gives what a fresh
    batch call gives on the current values, bit for bit."""
    import torch
    pairs = [(A.astype(dtype), B.astype(dtype)) for A, B in _pairs(seed=3, n=18)]
    dpairs = [(brm.DeviceCSR.from_host(A), brm.DeviceCSR.from_host(B)) for A, B in pairs]
    g = ctx.batch_graph(dpairs)
    for i, (A, B) in enumerate(pairs):
        assert_same_csr(g.results[i].to_host(), oracle_mod.precise(A, B), f"graph pair {i}")
    rng = np.random.default_rng(5)
    for it in range(2):
        for (A, B), (dA, dB) in zip(pairs, dpairs):
            A.val = rng.uniform(-1, 1, A.nnz).astype(dtype)
            B.val = rng.uniform(-1, 1, B.nnz).astype(dtype)
            dA.val.copy_(torch.from_numpy(A.val))
            dB.val.copy_(torch.from_numpy(B.val))
        torch.cuda.synchronize()
        g.launch()
        fresh = ctx.batch_precise(dpairs)
        for i, (A, B) in enumerate(pairs):
            got = g.results[i].to_host()
            assert_same_csr(got, oracle_mod.precise(A, B), f"replay {it} pair {i}")
            assert_same_csr(got, fresh[i].to_host(), f"replay {it} pair {i} vs fresh")
    g.close()


def _dev_equal(x, y):
    import torch
    if x.shape != y.shape or x.dtype != y.dtype:
        return False
    if x.dtype == torch.float64:
        x, y = x.view(torch.int64), y.view(torch.int64)
    return bool(torch.equal(x, y))


def test_batch_with_more_than_2_pow_24_long_columns(ctx):
    """Sixteen R-MAT n=2^16 degree-8 products in one batch (about 2e9
    products) hand more than 2^24 columns of heavy-row segments to the column
    reducers; every C_i must still equal its single call bit for bit
    (compared on the device)."""
    import torch
    mats = [brm.gen_rmat(16, 8 << 16, seed=21 + i) for i in range(4)]
    dev = [brm.DeviceCSR.from_host(A) for A in mats]
    alone = [ctx.precise_device(d, d) for d in dev]
    res = ctx.batch_precise([(dev[i % 4], dev[i % 4]) for i in range(16)])
    for i, C in enumerate(res):
        R = alone[i % 4]
        assert C.nnz == R.nnz, i
        assert (_dev_equal(C.rpt, R.rpt) and _dev_equal(C.col, R.col)
                and _dev_equal(C.val, R.val)), f"pair {i}"
    del res, alone
    torch.cuda.synchronize()
