"""CPU oracle for BRMerge SpGEMM -- TEST INFRASTRUCTURE ONLY.

Only tests/, __graft_entry__.smoke() and bench.py's CPU legs may import this
package, and only as the checker or the timed CPU baseline; the product
package brmerge_gb300 never imports it.

* ``precise`` / ``upper``: the C restatement (brm_oracle.c, built here and on
  the GPU host by ``build()``), bit-for-bit pinned against the reference.
* ``mtx``: the MatrixMarket reader (CSR::construct) restated with numpy.
* ``ref_precise`` / ``ref_upper`` / ``ref_read_mtx``: the reference's own
  brmerge_precise / brmerge_upper / MatrixMarket reader compiled from its
  sources by build_ref.sh into _ref/ when the reference tree is present (not
  on the GPU host).
"""
from __future__ import annotations

import ctypes as C
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
_LIB = HERE / "libbrm_oracle.so"
_REF = HERE / "_ref" / "libbrm_ref.so"

_lib = None
_ref = None


def build(with_ref: bool = True) -> None:
    """Compile the restatement (and the reference, when its sources exist)."""
    r = subprocess.run(["make", "-s", "-C", str(HERE)], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + r.stdout + r.stderr)
    if with_ref and not _REF.exists():
        # build_ref.sh finds the reference tree (BRM_REFERENCE_DIR) and exits
        # 3 when its sources are absent, as on hosts that only run the tests
        r = subprocess.run(["bash", str(HERE / "build_ref.sh")], capture_output=True, text=True)
        if r.returncode not in (0, 3):
            raise RuntimeError("reference build failed:\n" + r.stdout + r.stderr)


def _sig(f, args):
    f.restype = C.c_int
    f.argtypes = args


def lib():
    global _lib
    if _lib is None:
        if not _LIB.exists():
            build(with_ref=False)
        L = C.CDLL(str(_LIB))
        vp = C.c_void_p
        pp = C.POINTER(C.c_void_p)
        for n in ("brmo_precise_f64", "brmo_upper_f64", "brmo_precise_f32", "brmo_upper_f32"):
            _sig(getattr(L, n), [vp, vp, vp, vp, vp, vp, C.c_int, C.c_int, C.c_int, pp, pp, pp,
                                 C.POINTER(C.c_int), C.c_int])
        L.brmo_compute_flop.restype = C.c_longlong
        L.brmo_compute_flop.argtypes = [vp, vp, vp, C.c_int]
        L.brmo_row_flops.restype = None
        L.brmo_row_flops.argtypes = [vp, vp, vp, C.c_int, vp]
        L.brmo_free.restype = None
        L.brmo_free.argtypes = [vp]
        L.brmo_max_threads.restype = C.c_int
        _lib = L
    return _lib


def ref_available() -> bool:
    return _REF.exists()


def ref():
    global _ref
    if _ref is None:
        if not _REF.exists():
            raise RuntimeError("reference library not built (needs the reference sources)")
        R = C.CDLL(str(_REF))
        vp = C.c_void_p
        pp = C.POINTER(C.c_void_p)
        for n in ("ref_precise_f64", "ref_upper_f64"):
            _sig(getattr(R, n), [vp, vp, vp, vp, vp, vp, C.c_int, C.c_int, C.c_int, pp, pp, pp,
                                 C.POINTER(C.c_int), C.c_int, C.POINTER(C.c_double)])
        R.ref_free_int.restype = None
        R.ref_free_int.argtypes = [vp]
        R.ref_free_double.restype = None
        R.ref_free_double.argtypes = [vp]
        ip = C.POINTER(C.c_int)
        _sig(R.ref_read_mtx, [C.c_char_p, ip, ip, ip, pp, pp, pp, C.c_char_p, C.c_int])
        _ref = R
    return _ref


def ref_read_mtx(path):
    """The reference's own MatrixMarket reader (CSR::construct); returns the
    CSR or raises ValueError with the reader's message.  Only for inputs the
    reference reads without reaching an assert or undefined behaviour."""
    R = ref()
    M, N, nnz = C.c_int(), C.c_int(), C.c_int()
    pr, pc, pv = C.c_void_p(), C.c_void_p(), C.c_void_p()
    msg = C.create_string_buffer(256)
    st = R.ref_read_mtx(str(path).encode(), C.byref(M), C.byref(N), C.byref(nnz), C.byref(pr),
                        C.byref(pc), C.byref(pv), msg, 256)
    if st != 0:
        raise ValueError(msg.value.decode(errors="replace"))
    return _unpack(M.value, N.value, pr, pc, pv, nnz.value, np.float64, R.ref_free_int,
                   R.ref_free_double)


def _arrays(A, B):
    arrs = [np.ascontiguousarray(x) for x in (A.rpt, A.col, A.val, B.rpt, B.col, B.val)]
    return arrs, [a.ctypes.data_as(C.c_void_p) for a in arrs]


def _unpack(M, N, pr, pc, pv, n, vdt, free_i, free_v):
    from types import SimpleNamespace
    rpt = np.ctypeslib.as_array(C.cast(pr, C.POINTER(C.c_int)), shape=(M + 1,)).copy()
    if n:
        col = np.ctypeslib.as_array(C.cast(pc, C.POINTER(C.c_int)), shape=(n,)).copy()
        ct = C.c_double if vdt == np.float64 else C.c_float
        val = np.ctypeslib.as_array(C.cast(pv, C.POINTER(ct)), shape=(n,)).copy()
    else:
        col = np.zeros(0, np.int32)
        val = np.zeros(0, vdt)
    free_i(pr)
    free_i(pc)
    free_v(pv)
    return SimpleNamespace(M=M, N=N, rpt=rpt, col=col, val=val)


def _call(fname, A, B, nthreads):
    L = lib()
    vdt = np.dtype(A.val.dtype)
    keep, ptrs = _arrays(A, B)
    pr, pc, pv = C.c_void_p(), C.c_void_p(), C.c_void_p()
    cnnz = C.c_int(0)
    st = getattr(L, fname)(*ptrs, A.M, A.N, B.N, C.byref(pr), C.byref(pc), C.byref(pv),
                           C.byref(cnnz), nthreads)
    del keep
    if st != 0:
        raise RuntimeError(f"{fname} failed with status {st}")
    return _unpack(A.M, B.N, pr, pc, pv, cnnz.value, vdt.type, L.brmo_free, L.brmo_free)


def precise(A, B, nthreads: int = 0):
    """Oracle C = A*B (BRMerge-Precise restated); value type follows A.val."""
    sfx = "f64" if np.dtype(A.val.dtype) == np.float64 else "f32"
    return _call("brmo_precise_" + sfx, A, B, nthreads)


def upper(A, B, nthreads: int = 0):
    """Oracle C = A*B (BRMerge-Upper restated)."""
    sfx = "f64" if np.dtype(A.val.dtype) == np.float64 else "f32"
    return _call("brmo_upper_" + sfx, A, B, nthreads)


def _ref_call(fname, A, B, nthreads):
    R = ref()
    keep, ptrs = _arrays(A, B)
    pr, pc, pv = C.c_void_p(), C.c_void_p(), C.c_void_p()
    cnnz = C.c_int(0)
    sec = C.c_double(0)
    getattr(R, fname)(*ptrs, A.M, A.N, B.N, C.byref(pr), C.byref(pc), C.byref(pv), C.byref(cnnz),
                      nthreads, C.byref(sec))
    del keep
    out = _unpack(A.M, B.N, pr, pc, pv, cnnz.value, np.float64, R.ref_free_int,
                  R.ref_free_double)
    return out, sec.value


def ref_precise(A, B, nthreads: int = 0):
    """The reference's own brmerge_precise; returns (C, seconds)."""
    return _ref_call("ref_precise_f64", A, B, nthreads)


def ref_upper(A, B, nthreads: int = 0):
    """The reference's own brmerge_upper; returns (C, seconds)."""
    return _ref_call("ref_upper_f64", A, B, nthreads)


def compute_flop(A, B) -> int:
    keep, ptrs = _arrays(A, B)
    return int(lib().brmo_compute_flop(ptrs[0], ptrs[1], ptrs[3], A.M))


def max_threads() -> int:
    return int(lib().brmo_max_threads())
