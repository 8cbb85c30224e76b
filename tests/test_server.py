"""Serving: requests from several threads, batched by the server's workers.

Each result must be the same alone and in the mix: bit-identical to the
oracle and to a single brm_precise_device call on its own pair, whatever
batch it landed in.  Admission under a small memory cap must still finish
every request, and a request larger than the cap is rejected.
"""
import threading

import numpy as np
import pytest

import brmerge_gb300 as brm
from conftest import assert_same_csr

pytestmark = pytest.mark.gpu


def _requests(seed, n):
    rng = np.random.default_rng(seed)
    reqs = []
    for i in range(n):
        k = i % 4
        if k == 0:
            m = int(rng.integers(256, 2048))
            A, B = brm.gen_lognormal(m, m, seed=seed + 3 * i), brm.gen_lognormal(m, m, seed=seed + 3 * i + 1)
        elif k == 1:
            A = brm.gen_rmat(11, int(8 * 2048), seed=seed + i)
            B = A
        elif k == 2:
            A = brm.gen_uniform(300, 700, 20, seed=seed + i)
            B = brm.gen_uniform(700, 900, 25, seed=seed + i + 1)
        else:
            A = brm.gen_er(1024, 8, seed=seed + i)
            B = A
        if i % 5 == 3:
            A, B = A.astype(np.float32), B.astype(np.float32)
        reqs.append((A, B))
    return reqs


def test_server_results_same_alone_and_in_mix(oracle_mod):
    import torch
    reqs = _requests(11, 48)
    dev = [(brm.DeviceCSR.from_host(A), brm.DeviceCSR.from_host(B)) for A, B in reqs]
    ctx = brm.Context()
    alone = [ctx.precise_device(a, b).to_host() for a, b in dev]
    srv = brm.Server(workers=2)
    results = [None] * len(dev)

    def client(idx):
        tickets = [(i, srv.submit(*dev[i])) for i in idx]
        for i, t in tickets:
            C, st = srv.wait(t, timeout=120.0)
            results[i] = (C.to_host(), st)

    threads = [threading.Thread(target=client, args=(list(range(j, len(dev), 4)),))
               for j in range(4)]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    torch.cuda.synchronize()
    batched = 0
    for i, ((A, B), (C, st)) in enumerate(zip(reqs, results)):
        assert_same_csr(C, alone[i], f"request {i} vs alone")
        assert_same_csr(C, oracle_mod.precise(A, B), f"request {i} vs oracle")
        batched += st["batch_size"] > 1
    assert batched > 0  # some requests shared a batch
    srv.close()
    ctx.close()


def test_server_admission_under_small_cap():
    reqs = _requests(23, 12)
    dev = [(brm.DeviceCSR.from_host(A), brm.DeviceCSR.from_host(B)) for A, B in reqs]
    ctx = brm.Context()
    alone = [ctx.precise_device(a, b).to_host() for a, b in dev]
    # a cap that admits only a few requests at a time: later ones wait for
    # earlier results to be released
    srv = brm.Server(mem_cap_bytes=256 << 20, workers=2)
    tickets = [srv.submit(a, b) for a, b in dev]
    for i, t in enumerate(tickets):
        C, st = srv.wait(t, timeout=120.0)
        assert_same_csr(C.to_host(), alone[i], f"capped request {i}")
        del C  # releases the result and its share of the cap
    srv.close()
    ctx.close()


def test_server_rejects_request_above_cap():
    """Admission is asynchronous: the submit returns, the wait reports
    BRM_ERR_CAPACITY, and a request that fits still runs afterwards."""
    A = brm.DeviceCSR.from_host(brm.gen_rmat(12, 8 * 4096, seed=5))
    small = brm.gen_er(256, 4, seed=6)
    S = brm.DeviceCSR.from_host(small)
    srv = brm.Server(mem_cap_bytes=1 << 20, workers=1)
    t = srv.submit(A, A)
    with pytest.raises(brm.BrmError) as e:
        srv.wait(t, timeout=60.0)
    assert e.value.status == 10  # BRM_ERR_CAPACITY
    C, _ = srv.wait(srv.submit(S, S), timeout=60.0)
    ctx = brm.Context()
    assert_same_csr(C.to_host(), ctx.precise_device(S, S).to_host(), "after a rejection")
    del C
    srv.close()
    ctx.close()


def test_server_rejects_invalid_columns_at_admission():
    """A column of A outside B's rows is found by the admission kernel (it
    checks every column before it reads B's row pointers): the request fails
    with BRM_ERR_INVALID_CSR and the server keeps serving."""
    import torch
    B = brm.gen_er(64, 4, seed=7)
    dB = brm.DeviceCSR.from_host(B)
    rpt = torch.tensor([0, 2, 3], dtype=torch.int32, device="cuda")
    col = torch.tensor([1, 64, 5], dtype=torch.int32, device="cuda")  # 64 >= K = 64
    val = torch.ones(3, dtype=torch.float64, device="cuda")
    bad = brm.DeviceCSR(2, 64, rpt, col, val)
    srv = brm.Server(workers=1, express_workers=1)
    t = srv.submit(bad, dB)
    with pytest.raises(brm.BrmError) as e:
        srv.wait(t, timeout=60.0)
    assert e.value.status == 2  # BRM_ERR_INVALID_CSR
    C, _ = srv.wait(srv.submit(dB, dB), timeout=60.0)
    ctx = brm.Context()
    assert_same_csr(C.to_host(), ctx.precise_device(dB, dB).to_host(), "after invalid input")
    del C
    srv.close()
    ctx.close()


@pytest.mark.parametrize("express,sms", [(0, 0), (2, 0), (1, -1), (1, 32)])
def test_server_express_workers_same_results(oracle_mod, express, sms):
    """With no express workers, with two beside one general worker (on an SM
    partition of their own where the driver offers one), with an express
    worker on shared SMs, and with a 32-SM express partition: every result
    is the same as alone; small and large requests are mixed."""
    import torch
    reqs = _requests(31, 24)
    dev = [(brm.DeviceCSR.from_host(A), brm.DeviceCSR.from_host(B)) for A, B in reqs]
    ctx = brm.Context()
    alone = [ctx.precise_device(a, b).to_host() for a, b in dev]
    srv = brm.Server(workers=1, express_workers=express, express_bytes=8 << 20, express_sms=sms)
    tickets = [srv.submit(a, b) for a, b in dev]
    for i, t in enumerate(tickets):
        C, _ = srv.wait(t, timeout=120.0)
        assert_same_csr(C.to_host(), alone[i], f"request {i}")
        del C
    torch.cuda.synchronize()
    srv.close()
    ctx.close()
