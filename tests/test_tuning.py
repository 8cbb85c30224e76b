"""Row-class knobs and the autotuner.

Moving the heavy-row cut target or the mid-row weight limit changes only
where rows and segments are cut, never the result: every setting must give
the oracle's C bit for bit.  The autotuner must pick one of its candidates
and leave it in the context.
"""
import numpy as np
import pytest

import brmerge_gb300 as brm
from conftest import assert_same_csr

pytestmark = pytest.mark.gpu


# the largest heavy-row cut target accepted: seven eighths of the 3072
# products a segment holds
MAX_CUT = 2688


def _defaults():
    """The context defaults: cut target and the largest mid-row weight."""
    c = brm.Context()
    t = c.tuning()
    c.close()
    return t["seg_cut"], t["mid_flop"]


def _settings():
    cut, mid = _defaults()
    return [(cut, mid), (MAX_CUT, mid // 2), (cut * 2 // 3, mid // 2), (cut // 2, mid // 4),
            (cut // 3, mid), (256, 128)]


@pytest.fixture(scope="module")
def ctx():
    import torch  # noqa: F401
    c = brm.Context()
    yield c
    c.close()


@pytest.mark.parametrize("name,A,B", [
    ("rmat14", brm.gen_rmat(14, 8 << 14, seed=41), None),
    ("lognormal", brm.gen_lognormal(3000, 2500, seed=42), brm.gen_lognormal(2500, 4000, seed=43)),
    ("dense_rows", brm.gen_uniform(60, 3000, 500, seed=44), brm.gen_uniform(3000, 4000, 80, seed=45)),
])
def test_every_setting_gives_the_same_result(ctx, oracle_mod, name, A, B):
    B = A if B is None else B
    R = oracle_mod.precise(A, B)
    dA, dB = brm.DeviceCSR.from_host(A), brm.DeviceCSR.from_host(B)
    for cut, mid in _settings():
        ctx.set_tuning(seg_cut=cut, mid_flop=mid)
        assert ctx.tuning() == {"seg_cut": cut, "mid_flop": mid, "long_scratch": 0}
        assert_same_csr(ctx.precise_device(dA, dB).to_host(), R, f"{name} precise {cut}/{mid}")
        assert_same_csr(ctx.precise(dA, dB).to_host(), R, f"{name} split {cut}/{mid}")
        assert_same_csr(ctx.upper(dA, dB).to_host(), R, f"{name} upper {cut}/{mid}")
    ctx.set_tuning()
    cut, mid = _defaults()
    assert ctx.tuning() == {"seg_cut": cut, "mid_flop": mid, "long_scratch": 0}


def test_out_of_range_rejected(ctx):
    cut, mid = _defaults()
    for c, m in [(100, mid), (MAX_CUT + 1, mid), (cut, 2 * mid), (cut, 64)]:
        with pytest.raises(brm.BrmError):
            ctx.set_tuning(seg_cut=c, mid_flop=m)
    assert ctx.tuning() == {"seg_cut": cut, "mid_flop": mid, "long_scratch": 0}


def test_autotune_single_and_batch(ctx, oracle_mod):
    A = brm.gen_rmat(14, 8 << 14, seed=46)
    dA = brm.DeviceCSR.from_host(A)
    t = ctx.autotune([(dA, dA)])
    cut, mid = _defaults()
    assert t["seg_cut"] in (cut, cut * 2 // 3, cut // 2, cut // 3)
    assert t["mid_flop"] in (mid, mid // 2, mid // 4)
    assert ctx.tuning() == t
    assert_same_csr(ctx.precise_device(dA, dA).to_host(), oracle_mod.precise(A, A), "tuned")
    pairs = [(brm.gen_lognormal(m, m, seed=50 + m), brm.gen_lognormal(m, m, seed=60 + m))
             for m in (300, 900, 2000, 4000)]
    dp = [(brm.DeviceCSR.from_host(a), brm.DeviceCSR.from_host(b)) for a, b in pairs]
    t2 = ctx.autotune(dp)
    assert ctx.tuning() == t2
    for (a, b), C in zip(pairs, ctx.batch_precise(dp)):
        assert_same_csr(C.to_host(), oracle_mod.precise(a, b), "tuned batch")
    ctx.set_tuning()


@pytest.mark.parametrize("long_scratch", [1, 64, 4096])
def test_long_column_scratch_overflow_gives_the_same_result(ctx, oracle_mod, long_scratch):
    """Heavy-row segments hand their columns of more than eight products to
    separate reducers through a scratch of bounded size; columns beyond it are
    reduced inside the segment kernel.  A tiny scratch forces that path for
    almost every long column: the result must not change."""
    cases = [brm.gen_rmat(14, 8 << 14, seed=47),
             brm.gen_uniform(60, 3000, 500, seed=48)]
    for A in cases:
        B = A if A.M == A.N else brm.gen_uniform(3000, 4000, 80, seed=49)
        R = oracle_mod.precise(A, B)
        dA, dB = brm.DeviceCSR.from_host(A), brm.DeviceCSR.from_host(B)
        ctx.set_tuning(long_scratch=long_scratch)
        assert_same_csr(ctx.precise_device(dA, dB).to_host(), R, f"long scratch {long_scratch}")
        assert_same_csr(ctx.upper(dA, dB).to_host(), R, f"upper, long scratch {long_scratch}")
    ctx.set_tuning()
