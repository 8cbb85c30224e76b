"""ctypes bindings of the in-tree native libraries.

libbrmerge.so (CUDA, include/brmerge.h) and libbrm_host.so (host generators,
include/brm_gen.h) are built in-tree by brmerge_gb300.build.  Loading fails
loudly when a library is missing: there is no CPU fallback for the SpGEMM.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

_PKG = Path(__file__).resolve().parent

c_int_p = C.POINTER(C.c_int)
c_double_p = C.POINTER(C.c_double)
c_float_p = C.POINTER(C.c_float)


class PreciseTimingC(C.Structure):
    """Mirror of brm_precise_timing (Precise_Timing, Timings.h:26-46)."""
    _fields_ = [(n, C.c_double) for n in (
        "pre_allocate", "compute_flop", "prefix_sum_flop", "load_balance", "symbolic",
        "prefix_sum_nnz", "allocate_C", "compute", "cleanup", "total")]


class UpperTimingC(C.Structure):
    """Mirror of brm_upper_timing (Upper_Timing, Timings.h:4-24)."""
    _fields_ = [(n, C.c_double) for n in (
        "thread", "pre_allocate", "compute_flop", "prefix_sum_flop", "load_balance",
        "allocate_hook", "compute", "prefix_sum_nnz", "allocate_C", "copy", "cleanup", "total")]


class CsrC(C.Structure):
    """Mirror of brm_csr (device CSR view)."""
    _fields_ = [("M", C.c_int), ("N", C.c_int), ("nnz", C.c_int),
                ("rpt", C.c_void_p), ("col", C.c_void_p), ("val", C.c_void_p)]


class TuningC(C.Structure):
    """Mirror of brm_tuning."""
    _fields_ = [("seg_cut", C.c_int), ("mid_flop", C.c_int), ("long_scratch", C.c_longlong)]


class BatchC(C.Structure):
    """Mirror of brm_batch."""
    _fields_ = [("n", C.c_int), ("rows", C.c_longlong), ("nnz", C.c_longlong),
                ("row_off", C.POINTER(C.c_longlong)), ("nnz_off", C.POINTER(C.c_longlong)),
                ("crpt", C.c_void_p), ("ccol", C.c_void_p), ("cval", C.c_void_p),
                ("rpt_local", C.c_void_p)]


class BatchCapsC(C.Structure):
    """Mirror of brm_batch_caps."""
    _fields_ = [("pairs", C.c_int), ("rows", C.c_longlong), ("nnz_a", C.c_longlong),
                ("b_rows", C.c_longlong), ("nnz_b", C.c_longlong), ("cols", C.c_int),
                ("products", C.c_longlong), ("seg_slots", C.c_longlong), ("table", C.c_longlong),
                ("spill_bytes", C.c_longlong)]


class ServerConfigC(C.Structure):
    """Mirror of brm_server_config."""
    _fields_ = [("mem_cap_bytes", C.c_longlong), ("max_batch", C.c_int), ("workers", C.c_int),
                ("express_workers", C.c_int), ("express_bytes", C.c_longlong),
                ("express_sms", C.c_int)]


class ServerResultC(C.Structure):
    """Mirror of brm_server_result."""
    _fields_ = [("status", C.c_int), ("M", C.c_int), ("N", C.c_int), ("nnz", C.c_int),
                ("rpt", C.c_void_p), ("col", C.c_void_p), ("val", C.c_void_p),
                ("queued_s", C.c_double), ("latency_s", C.c_double), ("batch_size", C.c_int)]


class MtxTimingC(C.Structure):
    """Mirror of brm_mtx_timing."""
    _fields_ = [(n, C.c_double) for n in ("read", "parse", "build", "total")]


class HostCsrC(C.Structure):
    """Mirror of brm_host_csr (generator output)."""
    _fields_ = [("M", C.c_int), ("N", C.c_int), ("nnz", C.c_int),
                ("rpt", c_int_p), ("col", c_int_p), ("val", c_double_p)]


_lib = None
_host = None


def lib_path() -> Path:
    return _PKG / "libbrmerge.so"


def host_lib_path() -> Path:
    return _PKG / "libbrm_host.so"


def _decl(f, res, args):
    f.restype = res
    f.argtypes = args


def lib() -> C.CDLL:
    """The CUDA library; raises if it has not been built."""
    global _lib
    if _lib is None:
        p = lib_path()
        if not p.exists():
            raise RuntimeError(
                f"{p} is missing: build it with `python -m brmerge_gb300.build` "
                "(the SpGEMM has no CPU fallback)")
        L = C.CDLL(str(p))
        vp = C.c_void_p
        ctxp = C.POINTER(vp)
        csrp = C.POINTER(CsrC)
        _decl(L.brm_status_string, C.c_char_p, [C.c_int])
        _decl(L.brm_create, C.c_int, [ctxp])
        _decl(L.brm_destroy, C.c_int, [vp])
        _decl(L.brm_set_stream, C.c_int, [vp, vp])
        _decl(L.brm_set_validate, C.c_int, [vp, C.c_int])
        _decl(L.brm_last_device_error, C.c_int, [vp])
        _decl(L.brm_device_code_version, C.c_int, [c_int_p])
        _decl(L.brm_checked_build, C.c_int, [])
        _decl(L.brm_last_check_failure, C.c_int,
              [vp, c_int_p, C.POINTER(C.c_longlong), C.POINTER(C.c_longlong)])
        _decl(L.brm_symbolic, C.c_int, [vp, csrp, csrp, vp, c_int_p])
        _decl(L.brm_numeric, C.c_int, [vp, C.c_int, csrp, csrp, vp, vp, vp])
        _decl(L.brm_precise_device, C.c_int,
              [vp, C.c_int, csrp, csrp, ctxp, ctxp, ctxp, c_int_p, C.POINTER(PreciseTimingC)])
        _decl(L.brm_upper_device, C.c_int,
              [vp, C.c_int, csrp, csrp, ctxp, ctxp, ctxp, c_int_p, C.POINTER(UpperTimingC)])
        _decl(L.brm_device_free, C.c_int, [vp, vp])
        for name, vt, tt in (("brm_precise", c_double_p, PreciseTimingC),
                             ("brm_upper", c_double_p, UpperTimingC),
                             ("brm_precise_f32", c_float_p, PreciseTimingC),
                             ("brm_upper_f32", c_float_p, UpperTimingC)):
            _decl(getattr(L, name), C.c_int,
                  [vp, vp, vp, vp, vp, vp, C.POINTER(c_int_p), C.POINTER(c_int_p),
                   C.POINTER(vt), C.c_int, C.c_int, C.c_int, c_int_p, C.POINTER(tt)])
        _decl(L.brm_free, None, [vp])
        _decl(L.brm_host_cache_release, None, [])
        _decl(L.brm_kernel_launches, C.c_longlong, [])
        _decl(L.brm_batch_graph_create, C.c_int,
              [vp, C.c_int, C.c_int, csrp, csrp, ctxp, C.POINTER(BatchC)])
        _decl(L.brm_batch_graph_launch, C.c_int, [vp, vp])
        _decl(L.brm_batch_graph_destroy, C.c_int, [vp])
        capsp = C.POINTER(BatchCapsC)
        _decl(L.brm_batch_caps_for, C.c_int,
              [vp, C.c_int, C.c_int, csrp, csrp, C.c_double, capsp])
        _decl(L.brm_batch_pipe_create, C.c_int, [vp, C.c_int, capsp, ctxp])
        _decl(L.brm_batch_pipe_caps, C.c_int, [vp, capsp])
        _decl(L.brm_batch_pipe_run, C.c_int, [vp, C.c_int, csrp, csrp, vp, C.POINTER(BatchC)])
        _decl(L.brm_batch_pipe_destroy, C.c_int, [vp])
        _decl(L.brm_set_tuning, C.c_int, [vp, C.POINTER(TuningC)])
        _decl(L.brm_get_tuning, C.c_int, [vp, C.POINTER(TuningC)])
        _decl(L.brm_autotune, C.c_int, [vp, C.c_int, C.c_int, csrp, csrp, C.POINTER(TuningC)])
        _decl(L.brm_batch_precise, C.c_int, [vp, C.c_int, C.c_int, csrp, csrp, C.POINTER(BatchC)])
        _decl(L.brm_batch_free, C.c_int, [vp, C.POINTER(BatchC)])
        _decl(L.brm_server_create, C.c_int, [C.POINTER(ServerConfigC), ctxp])
        _decl(L.brm_server_sms, C.c_int, [vp, c_int_p, c_int_p])
        _decl(L.brm_server_submit, C.c_int, [vp, C.c_int, csrp, csrp, C.POINTER(C.c_longlong)])
        _decl(L.brm_server_wait, C.c_int,
              [vp, C.c_longlong, C.c_double, C.POINTER(ServerResultC)])
        _decl(L.brm_server_release, C.c_int, [vp, C.c_longlong])
        _decl(L.brm_server_destroy, C.c_int, [vp])
        _decl(L.brm_compute_flop, C.c_int, [vp, csrp, csrp, C.POINTER(C.c_longlong)])
        _decl(L.brm_upper_bound, C.c_int,
              [vp, C.c_int, csrp, csrp, C.POINTER(C.c_longlong), C.POINTER(C.c_longlong)])
        _decl(L.brm_validate, C.c_int, [vp, csrp, C.c_int, c_int_p])
        _decl(L.brm_hash_device, C.c_int,
              [vp, C.c_int, csrp, csrp, ctxp, ctxp, ctxp, c_int_p])
        _decl(L.brm_read_mtx_device, C.c_int,
              [vp, C.c_int, C.c_char_p, c_int_p, c_int_p, c_int_p, ctxp, ctxp, ctxp,
               C.POINTER(MtxTimingC)])
        _decl(L.brm_read_mtx, C.c_int,
              [C.c_char_p, C.c_int, c_int_p, c_int_p, c_int_p, ctxp, ctxp, ctxp,
               C.POINTER(MtxTimingC)])
        _lib = L
    return _lib


def host() -> C.CDLL:
    """The host helper library (generators)."""
    global _host
    if _host is None:
        p = host_lib_path()
        if not p.exists():
            raise RuntimeError(f"{p} is missing: build it with `python -m brmerge_gb300.build`")
        H = C.CDLL(str(p))
        hp = C.POINTER(HostCsrC)
        _decl(H.brm_host_csr_free, None, [hp])
        _decl(H.brm_gen_er, C.c_int, [C.c_int, C.c_int, C.c_ulonglong, hp])
        _decl(H.brm_gen_rmat, C.c_int, [C.c_int, C.c_longlong, C.c_double, C.c_double,
                                         C.c_double, C.c_ulonglong, hp])
        _decl(H.brm_gen_stencil27, C.c_int, [C.c_int, C.c_int, C.c_int, C.c_double,
                                              C.c_ulonglong, hp])
        _decl(H.brm_gen_lognormal, C.c_int, [C.c_int, C.c_int, C.c_double, C.c_double,
                                              C.c_int, C.c_ulonglong, hp])
        _decl(H.brm_gen_uniform, C.c_int, [C.c_int, C.c_int, C.c_int, C.c_ulonglong, hp])
        _decl(H.brm_parse_int_token, C.c_int, [C.c_char_p, C.c_int, C.POINTER(C.c_longlong)])
        _decl(H.brm_parse_real_token, C.c_int, [C.c_char_p, C.c_int, c_double_p])
        _decl(H.brm_parse_real_tokens, None,
              [C.c_void_p, C.c_void_p, C.c_void_p, C.c_longlong, C.c_void_p, C.c_void_p])
        _host = H
    return _host


class BrmError(RuntimeError):
    """A non-zero brm_status from the native library."""

    def __init__(self, status: int, where: str = ""):
        msg = lib().brm_status_string(status).decode()
        super().__init__(f"{where}: {msg} (status {status})" if where else f"{msg} (status {status})")
        self.status = status


def check(status: int, where: str = "") -> None:
    if status != 0:
        raise BrmError(status, where)
