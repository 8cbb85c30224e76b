"""Allocation-free product count, checked against the allocating entry point.

brm_compute_flop_noalloc is for callers that may not allocate device memory
at the moment they need the count, such as an admission controller that
sizes a request before it reserves anything.  Its reduction scratch is a
fixed device array shared by every call.  This test calls it twice in a row
through the C ABI and checks each result, bit for bit, against
brm_compute_flop (which allocates its own workspace) and against per-row
counts computed on the host.
"""
import ctypes as C

import numpy as np
import pytest

import brmerge_gb300 as brm
from brmerge_gb300 import _native

pytestmark = pytest.mark.gpu

BRM_ERR_INVALID_CSR = 2
BRM_ERR_OVERFLOW = 5
BRM_ERR_CAPACITY = 10
MAX_ROWS = 65536 * 64


def _noalloc(lib, dA, dB, row_flop_ptr):
    fn = lib.brm_compute_flop_noalloc
    fn.restype = C.c_int
    fn.argtypes = [C.POINTER(_native.CsrC), C.POINTER(_native.CsrC), C.c_void_p,
                   C.POINTER(C.c_longlong), C.c_void_p]
    a, b = dA.c(), dB.c()
    out = C.c_longlong(-1)
    st = fn(C.byref(a), C.byref(b), row_flop_ptr, C.byref(out), None)
    return st, out.value


def _host_row_flops(A, B):
    blen = np.diff(B.rpt.astype(np.int64))
    per = blen[A.col] if A.nnz else np.zeros(0, np.int64)
    rows = np.repeat(np.arange(A.M), np.diff(A.rpt))
    return np.bincount(rows, weights=per, minlength=A.M).astype(np.int64)


def test_noalloc_flop_matches_allocating_entry_point():
    import torch
    lib = _native.lib()
    ctx = brm.Context()
    cases = [
        (brm.gen_rmat(14, int(2.35 * (1 << 14)), seed=31), None),
        (brm.gen_lognormal(3000, 2000, seed=32), brm.gen_lognormal(2000, 2500, seed=33)),
    ]
    for A, B in cases:  # two calls in a row on the shared scratch
        B = A if B is None else B
        dA, dB = brm.DeviceCSR.from_host(A), brm.DeviceCSR.from_host(B)
        expected = ctx.compute_flop(dA, dB)
        row_flop = torch.full((A.M,), -1, dtype=torch.int32, device="cuda")
        st, total = _noalloc(lib, dA, dB, row_flop.data_ptr())
        assert st == 0, _native.lib().brm_status_string(st)
        assert total == expected
        assert np.array_equal(row_flop.cpu().numpy().astype(np.int64), _host_row_flops(A, B))
        # the per-row buffer is optional
        st2, total2 = _noalloc(lib, dA, dB, None)
        assert st2 == 0 and total2 == expected
    ctx.close()


def test_noalloc_rejects_too_many_rows():
    import torch
    lib = _native.lib()
    M = MAX_ROWS + 1
    rpt = torch.zeros(M + 1, dtype=torch.int32, device="cuda")
    col = torch.zeros(1, dtype=torch.int32, device="cuda")
    val = torch.zeros(1, dtype=torch.float64, device="cuda")
    A = brm.DeviceCSR(M, 4, rpt, col[:0], val[:0])
    B = brm.DeviceCSR(4, 4, torch.zeros(5, dtype=torch.int32, device="cuda"), col[:0], val[:0])
    st, _ = _noalloc(lib, A, B, None)
    assert st == BRM_ERR_CAPACITY


def _dev_csr(M, N, rpt, col, dtype=np.float64):
    """A device CSR from raw arrays (no validation: the cases below are
    deliberately not valid CSR).  The value array is never read by the count."""
    import torch
    rpt_t = torch.tensor(np.asarray(rpt, dtype=np.int32), device="cuda")
    col_t = torch.tensor(np.asarray(col if len(col) else [0], dtype=np.int32), device="cuda")
    val_t = torch.zeros(max(1, len(col)), dtype=torch.float64, device="cuda")
    return brm.DeviceCSR(M, N, rpt_t, col_t[:len(col)], val_t[:len(col)])


def test_noalloc_reports_invalid_input_and_clears_the_error_word():
    """A column of A out of range, then B.rpt decreasing: each call returns
    BRM_ERR_INVALID_CSR (the kernel checks every column before it reads
    B.rpt, so nothing is read out of bounds).  A valid call right after each
    failure succeeds, so the shared error word is cleared per call."""
    lib = _native.lib()
    good_A = _dev_csr(2, 3, [0, 2, 3], [0, 2, 1])
    good_B = _dev_csr(3, 4, [0, 1, 3, 4], [0, 1, 3, 2])
    # out-of-range column (3 >= K = 3) in row 1
    bad_A = _dev_csr(2, 3, [0, 2, 3], [0, 2, 3])
    st, total = _noalloc(lib, bad_A, good_B, None)
    assert st == BRM_ERR_INVALID_CSR and total == 0
    st, total = _noalloc(lib, good_A, good_B, None)
    assert st == 0 and total == (1 + 1) + 2
    # B.rpt decreasing at row 1: a negative row length
    bad_B = _dev_csr(3, 4, [0, 3, 2, 4], [0, 1, 3, 2])
    st, total = _noalloc(lib, good_A, bad_B, None)
    assert st == BRM_ERR_INVALID_CSR and total == 0
    st, total = _noalloc(lib, good_A, good_B, None)
    assert st == 0 and total == 4


def test_noalloc_reports_row_count_overflow():
    """With valid CSR a row's count is at most nnz(B) <= INT_MAX.  An A row
    that repeats a column can exceed it: the call returns BRM_ERR_OVERFLOW
    instead of clamping the row's count.  Only B.rpt is read (never B.col),
    so B's row pointers can describe long rows without holding them."""
    import torch
    lib = _native.lib()
    A = _dev_csr(1, 1, [0, 3], [0, 0, 0])
    B = _dev_csr(1, 1, [0, 1 << 30], [0])
    row_flop = torch.full((1,), -7, dtype=torch.int32, device="cuda")
    st, total = _noalloc(lib, A, B, row_flop.data_ptr())
    assert st == BRM_ERR_OVERFLOW and total == 0
    assert int(row_flop.item()) == -7  # left unwritten, not clamped
    good_A = _dev_csr(2, 3, [0, 2, 3], [0, 2, 1])
    good_B = _dev_csr(3, 4, [0, 1, 3, 4], [0, 1, 3, 2])
    st, total = _noalloc(lib, good_A, good_B, None)
    assert st == 0 and total == 4
