"""Full-size parity of every configuration bench.py times, on the bench's
own inputs (its numpy generators and its 4096-pair batch):

* R-MAT n=2^18 and ER n=16384 (C = A*A): one-call Precise, Upper and the
  host drop-in bit for bit against the oracle (BRMerge-SpGEMM/inc/
  spgemm.h:468-735).
* 27-point stencil 128^3: one-call Precise and Upper identical to each other,
  exact structure by closed form, four row blocks of 3000 rows against the
  oracle (rows of C are independent).
* the 4096-pair uneven batch, float64 and float32: every C_i of
  brm_batch_precise and of its graph replay identical to brm_precise_device
  on that pair, and sixteen pairs against the oracle.
"""
import numpy as np
import pytest

import bench
import brmerge_gb300 as brm

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    c = brm.Context()
    yield c
    c.close()


def _host(X):
    return X.to_host()


@pytest.mark.parametrize("name", ["rmat", "er"])
def test_bench_workload_every_form_vs_oracle(ctx, oracle_mod, name):
    A, _ = bench.make_workload(name)
    R = oracle_mod.precise(A, A)
    dA = brm.DeviceCSR.from_host(A)
    assert bench.same_csr(_host(ctx.precise_device(dA, dA)), R)
    assert bench.same_csr(_host(ctx.upper(dA, dA)), R)
    hA = brm.CSR(A.M, A.N, A.rpt, A.col, A.val)
    assert bench.same_csr(brm.brmerge_precise(hA, hA), R)


def test_bench_stencil_one_call_precise_and_upper(ctx, oracle_mod):
    import torch
    m = 128
    S, _ = bench.make_workload("stencil", m)
    dS = brm.DeviceCSR.from_host(S)
    Cp = ctx.precise_device(dS, dS)
    assert Cp.nnz == (5 * m - 6) ** 3  # 634^3: a 5x5x5 box clipped at the faces
    w = np.array([min(x + 2, m - 1) - max(x - 2, 0) + 1 for x in range(m)], np.int64)
    lens = (w[None, None, :] * w[None, :, None] * w[:, None, None]).reshape(-1)
    rpt = Cp.rpt.cpu().numpy()
    assert np.array_equal(np.diff(rpt.astype(np.int64)), lens)
    Cu = ctx.upper(dS, dS)
    assert bench.dev_same_csr(Cp, Cu)
    del Cu
    for r0 in (0, 70000, m ** 3 // 2, m ** 3 - 3000):
        R = oracle_mod.precise(bench.row_block(S, r0, r0 + 3000), S)
        s, e = int(rpt[r0]), int(rpt[r0 + 3000])
        got = bench.host_csr(3000, S.N, rpt[r0:r0 + 3001].astype(np.int64) - s,
                             Cp.col[s:e].cpu().numpy(), Cp.val[s:e].cpu().numpy())
        assert bench.same_csr(got, R), r0
    del Cp, dS
    torch.cuda.synchronize()


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_bench_batch_every_pair_and_graph_replay(ctx, oracle_mod, dtype):
    import torch
    pairs = bench.make_batch(bench.BATCH_PAIRS, seed=7, dtype=dtype)
    dpairs, keep = bench.upload_pairs(pairs, "cuda")
    out = ctx.batch_precise_raw(dpairs)
    views = bench.batch_views(out, dpairs)
    bad = [i for i, ((a, b), v) in enumerate(zip(dpairs, views))
           if not bench.dev_same_csr(v, ctx.precise_device(a, b))]
    assert not bad, f"{len(bad)} pairs differ from the plain call, first {bad[:5]}"
    for v, (A, B) in zip(views[:16], pairs[:16]):
        got = bench.host_csr(A.M, B.N, v.rpt.cpu().numpy(), v.col.cpu().numpy(),
                             v.val.cpu().numpy())
        assert bench.same_csr(got, oracle_mod.precise(A, B))
    g = ctx.batch_graph(dpairs)
    for _ in range(2):  # the structure is planned once; each launch recomputes the values
        g.launch()
        torch.cuda.synchronize()
        assert all(bench.dev_same_csr(x, y) for x, y in zip(g.results, views))
    g.close()
    del out, views, keep
    torch.cuda.synchronize()
