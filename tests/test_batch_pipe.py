"""Batch pipeline (brm_batch_pipe_*): brm_batch_precise captured once as a
CUDA graph with fixed capacities and launched once per new batch.

Batches of different structure (other pairs, fewer pairs, another order,
heavy rows, rectangular and empty pairs) run through one captured graph;
every C_i must be bit-identical to brm_precise_device on its own pair, and
sampled pairs to the oracle (BRMerge-SpGEMM/inc/spgemm.h:468-735).  A batch
beyond the capacities is refused -- by the host for the pair count and the
stacked sizes, by the device for the products -- and the next batch runs.
"""
import numpy as np
import pytest

import brmerge_gb300 as brm
from conftest import assert_same_csr
from test_batch import _pairs

pytestmark = pytest.mark.gpu

BRM_ERR_CAPACITY = 10


@pytest.fixture(scope="module")
def ctx():
    import torch  # noqa: F401
    c = brm.Context()
    yield c
    c.close()


def _dev(pairs):
    return [(brm.DeviceCSR.from_host(A), brm.DeviceCSR.from_host(B)) for A, B in pairs]


def _check_batch(ctx, oracle_mod, pipe, pairs, n_oracle=4):
    dpairs = _dev(pairs)
    res = pipe.run(dpairs)
    assert len(res) == len(pairs)
    for i, ((a, b), C) in enumerate(zip(dpairs, res)):
        single = ctx.precise_device(a, b).to_host()
        assert_same_csr(C.to_host(), single, f"pair {i} vs a single call")
    for i in range(min(n_oracle, len(pairs))):
        A, B = pairs[i]
        assert_same_csr(res[i].to_host(), oracle_mod.precise(A, B), f"pair {i} vs oracle")


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_pipe_runs_new_batches(ctx, oracle_mod, dtype):
    sample = [(A.astype(dtype), B.astype(dtype)) for A, B in _pairs(seed=3, n=24)]
    pipe = ctx.batch_pipe(_dev(sample), headroom=2.0)
    caps = pipe.caps()
    assert caps["pairs"] >= 24 and caps["products"] > 0
    batches = [
        sample,                                                       # the sample itself
        [(A.astype(dtype), B.astype(dtype)) for A, B in _pairs(seed=4, n=24)],  # other pairs
        sample[::-1],                                                 # another order
        sample[5:17],                                                 # fewer pairs
        [(A.astype(dtype), B.astype(dtype)) for A, B in _pairs(seed=5, n=30)],
    ]
    for k, pairs in enumerate(batches):
        _check_batch(ctx, oracle_mod, pipe, pairs)
    pipe.close()


def test_pipe_heavy_rows_and_rmat(ctx, oracle_mod):
    """Heavy (segmented) rows and power-law pairs inside the captured graph."""
    big = [(brm.gen_rmat(13, int(2.35 * 8192), seed=70 + i),) * 2 for i in range(3)]
    dense = [(brm.gen_uniform(60, 3000, 500, seed=80 + i), brm.gen_uniform(3000, 4000, 80, seed=90 + i))
             for i in range(3)]
    sample = big + dense + _pairs(seed=6, n=12)
    pipe = ctx.batch_pipe(_dev(sample), headroom=1.5)
    _check_batch(ctx, oracle_mod, pipe, sample, n_oracle=6)
    other = [(brm.gen_rmat(13, int(2.35 * 8192), seed=170 + i),) * 2 for i in range(3)] + dense[::-1]
    _check_batch(ctx, oracle_mod, pipe, other, n_oracle=6)
    pipe.close()


def _csr(rows, N):
    rpt = np.zeros(len(rows) + 1, np.int32)
    rpt[1:] = np.cumsum([len(r) for r in rows])
    col = np.array([c for r in rows for c in r], np.int32)
    val = np.linspace(-1.0, 1.0, len(col)) if len(col) else np.zeros(0)
    return brm.CSR(len(rows), N, rpt, col, val)


def test_pipe_refuses_batches_beyond_its_capacities(ctx, oracle_mod):
    import torch
    # sample: 64 x 64, A's rows point at B rows of two entries each
    B_short = _csr([[j, (j + 1) % 64] if j + 1 < 64 else [0, j] for j in range(64)], 64)
    A = _csr([[i % 64] for i in range(64)], 64)
    sample = [(A, B_short)] * 4
    caps = {"pairs": 4, "rows": 4 * 64, "nnz_a": 4 * 64, "b_rows": 4 * 64, "nnz_b": 4 * 128,
            "cols": 64, "products": 4 * 128, "seg_slots": 1024, "table": 65536,
            "spill_bytes": 1 << 20}
    pipe = ctx.batch_pipe(caps=caps, dtype=np.float64)
    _check_batch(ctx, oracle_mod, pipe, sample)
    # too many pairs: refused by the host
    with pytest.raises(brm.BrmError) as e:
        pipe.run(_dev(sample * 2))
    assert e.value.status == BRM_ERR_CAPACITY
    # same sizes, more products: B's first row holds every entry and every A
    # row names it, so the products exceed the capacity -- refused by the device
    B_long = _csr([list(range(64)), list(range(64))] + [[] for _ in range(62)], 64)
    A0 = _csr([[0] for _ in range(64)], 64)
    with pytest.raises(brm.BrmError) as e:
        pipe.run(_dev([(A0, B_long)] * 4))
    assert e.value.status == BRM_ERR_CAPACITY
    torch.cuda.synchronize()
    # the pipe still runs batches that fit
    _check_batch(ctx, oracle_mod, pipe, sample[:3])
    pipe.close()
