"""CSR containers mirroring the reference's CSR class (BRMerge-SpGEMM/inc/CSR.h:7-28)."""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _native


@dataclass
class CSR:
    """Host CSR matrix: M x N, int32 row pointers and column indices,
    float64 (or float32) values; columns sorted and unique within each row."""
    M: int
    N: int
    rpt: np.ndarray
    col: np.ndarray
    val: np.ndarray

    @property
    def nnz(self) -> int:
        return int(self.rpt[self.M]) if self.M >= 0 and len(self.rpt) else 0

    def astype(self, dtype) -> "CSR":
        return CSR(self.M, self.N, self.rpt, self.col, np.ascontiguousarray(self.val, dtype=dtype))

    def copy(self) -> "CSR":
        return CSR(self.M, self.N, self.rpt.copy(), self.col.copy(), self.val.copy())

    def check(self) -> None:
        """Raise ValueError unless the invariants of CSR.cpp:454-477 hold."""
        r, c = self.rpt, self.col
        if len(r) != self.M + 1 or r[0] != 0 or np.any(np.diff(r) < 0) or r[-1] != len(c):
            raise ValueError("csr row_pointer wrong")
        if len(c) and (c.min() < 0 or c.max() >= self.N):
            raise ValueError("csr col_index out of range")
        if len(c) > 1:
            same_row = np.repeat(np.arange(self.M), np.diff(r))
            bad = (np.diff(c) <= 0) & (same_row[1:] == same_row[:-1])
            if bad.any():
                raise ValueError("csr col_index not in assending order")

    def to_scipy(self):
        import scipy.sparse as sp
        return sp.csr_matrix((self.val, self.col, self.rpt), shape=(self.M, self.N))


def _from_host_csr(h: _native.HostCsrC) -> CSR:
    M, nnz = h.M, h.nnz
    rpt = np.ctypeslib.as_array(h.rpt, shape=(M + 1,)).copy()
    if nnz > 0:
        col = np.ctypeslib.as_array(h.col, shape=(nnz,)).copy()
        val = np.ctypeslib.as_array(h.val, shape=(nnz,)).copy()
    else:
        col = np.zeros(0, np.int32)
        val = np.zeros(0, np.float64)
    out = CSR(M, h.N, rpt.astype(np.int32, copy=False), col.astype(np.int32, copy=False),
              val.astype(np.float64, copy=False))
    _native.host().brm_host_csr_free(C.byref(h))
    return out


def _gen(fn, *args) -> CSR:
    h = _native.HostCsrC()
    st = fn(*args, C.byref(h))
    if st != 0:
        raise RuntimeError(f"generator failed with status {st}")
    return _from_host_csr(h)


def gen_er(n: int, per_row: int = 8, seed: int = 0) -> CSR:
    """Erdos-Renyi n x n with exactly per_row distinct uniform columns per row."""
    return _gen(_native.host().brm_gen_er, n, per_row, seed)


def gen_rmat(scale: int, edges: int, a=0.57, b=0.19, c=0.19, seed: int = 0) -> CSR:
    """R-MAT 2^scale square with `edges` samples, duplicates removed."""
    return _gen(_native.host().brm_gen_rmat, scale, edges, a, b, c, seed)


def gen_stencil27(nx: int, ny: int | None = None, nz: int | None = None, jitter: float = 1e-3,
                  seed: int = 0) -> CSR:
    """27-point stencil: 26 on the diagonal, -1 off it, plus U[-jitter, jitter]."""
    ny = nx if ny is None else ny
    nz = nx if nz is None else nz
    return _gen(_native.host().brm_gen_stencil27, nx, ny, nz, jitter, seed)


def gen_lognormal(M: int, N: int, mu: float = float(np.log(6.0)), sigma: float = 0.8,
                  cap: int = 256, seed: int = 0) -> CSR:
    """Row lengths round(lognormal(mu, sigma)) capped at cap, uniform columns."""
    return _gen(_native.host().brm_gen_lognormal, M, N, mu, sigma, cap, seed)


def gen_uniform(M: int, N: int, max_per_row: int, seed: int = 0) -> CSR:
    """Row lengths uniform in [0, max_per_row], uniform distinct columns."""
    return _gen(_native.host().brm_gen_uniform, M, N, max_per_row, seed)
