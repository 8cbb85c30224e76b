"""The checked device build (-DBRM_CHECKED, brmerge_gb300/build.py
checked=True or BRM_CHECKED=1): every data-dependent index is checked
against its bound, a failing access is skipped and the call returns
BRM_ERR_INTERNAL, with the first failure's source line, index and bound
reported by brm_last_check_failure.  The whole -m gpu suite is run under that
build as well; here the representative paths (every row class, segments with
long columns handed to the reducers or reduced in the segment kernel, Upper,
a batch) must report no failed check in either build."""
import ctypes as C

import numpy as np
import pytest

import brmerge_gb300 as brm
from brmerge_gb300 import _native
from conftest import assert_same_csr

pytestmark = pytest.mark.gpu


def _failure(ctx):
    line, idx, bound = C.c_int(-1), C.c_longlong(-1), C.c_longlong(-1)
    assert _native.lib().brm_last_check_failure(ctx._h, C.byref(line), C.byref(idx),
                                                C.byref(bound)) == 0
    return line.value, idx.value, bound.value


def test_no_failed_check(oracle_mod):
    ctx = brm.Context()
    mode = "checked" if _native.lib().brm_checked_build() else "normal"
    cases = [("rmat", brm.gen_rmat(14, 8 << 14, seed=3), None),
             ("dense", brm.gen_uniform(60, 3000, 500, seed=4), brm.gen_uniform(3000, 4000, 80, seed=5)),
             ("stencil", brm.gen_stencil27(12), None),
             ("lognormal", brm.gen_lognormal(2000, 2000, seed=6), brm.gen_lognormal(2000, 3000, seed=7))]
    for long_scratch in (0, 16):
        ctx.set_tuning(long_scratch=long_scratch) if long_scratch else ctx.set_tuning()
        for name, A, B in cases:
            B = A if B is None else B
            R = oracle_mod.precise(A, B)
            dA, dB = brm.DeviceCSR.from_host(A), brm.DeviceCSR.from_host(B)
            for form in ("precise", "split", "upper"):
                C_ = {"precise": ctx.precise_device, "split": ctx.precise,
                      "upper": ctx.upper}[form](dA, dB)
                assert _failure(ctx) == (0, 0, 0), (mode, name, form)
                assert_same_csr(C_.to_host(), R, f"{mode} {name} {form}")
    pairs = [(brm.DeviceCSR.from_host(A), brm.DeviceCSR.from_host(B if B is not None else A))
             for _, A, B in cases]
    for C_, (a, b) in zip(ctx.batch_precise(pairs), pairs):
        assert_same_csr(C_.to_host(), ctx.precise_device(a, b).to_host(), f"{mode} batch")
    assert _failure(ctx) == (0, 0, 0)
    ctx.set_tuning()
    ctx.close()
