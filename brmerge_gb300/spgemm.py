"""BRMerge SpGEMM entry points, mirroring the reference's interface.

Host forms (reference signatures, BRMerge-SpGEMM/inc/spgemm.h:460-464,
:737-741): ``brmerge_precise(A, B, C, timing)`` and ``brmerge_upper(A, B, C,
timing)`` take host CSR matrices and fill C.  They call the C ABI's host
drop-ins (brm_precise / brm_upper), which run every phase on the GPU.

Device forms: ``Context`` wraps a brm_context and works on ``DeviceCSR``
matrices whose arrays are torch CUDA tensors (torch is used only for device
memory and streams).
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, fields

import numpy as np

from . import _native
from .csr import CSR

F64, F32 = 0, 1


def _dtype_code(val_dtype) -> int:
    dt = np.dtype(val_dtype)
    if dt == np.float64:
        return F64
    if dt == np.float32:
        return F32
    raise TypeError(f"unsupported value type {dt}; use float64 or float32")


class _Timing:
    _c = None

    def __init__(self):
        for f in self._names():
            setattr(self, f, 0.0)

    @classmethod
    def _names(cls):
        return [n for n, _ in cls._c._fields_]

    def _load(self, c):
        for n in self._names():
            setattr(self, n, float(getattr(c, n)))

    def __iadd__(self, other):
        for n in self._names():
            setattr(self, n, getattr(self, n) + getattr(other, n))
        return self

    def __itruediv__(self, k: float):
        for n in self._names():
            setattr(self, n, getattr(self, n) / k)
        return self

    def as_dict(self):
        return {n: getattr(self, n) for n in self._names()}

    def reg_print(self, total_flop: float) -> str:
        """GFLOPS line as the reference's reg_print (Timings.cpp:162-165)."""
        return f"{total_flop / self.total / 1e9 if self.total else 0.0:f}"


class PreciseTiming(_Timing):
    """Phase times in seconds (Precise_Timing, Timings.h:26-46)."""
    _c = _native.PreciseTimingC


class UpperTiming(_Timing):
    """Phase times in seconds (Upper_Timing, Timings.h:4-24)."""
    _c = _native.UpperTimingC


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(C.c_void_p)


class _HostBlock:
    """Owner of one array returned by a host drop-in; releases it with brm_free."""
    __slots__ = ("_L", "_p")

    def __init__(self, L, p):
        self._L, self._p = L, p

    def __del__(self):
        if self._p:
            self._L.brm_free(self._p)
            self._p = None


def _owned(L, ptr, n: int, ctype, dtype) -> np.ndarray:
    """A numpy view of n elements at ptr that frees the block when collected."""
    addr = C.cast(ptr, C.c_void_p).value
    if not addr:
        return np.zeros(n, dtype)
    if n == 0:
        L.brm_free(addr)
        return np.zeros(0, dtype)
    buf = (ctype * n).from_address(addr)
    buf._owner = _HostBlock(L, addr)
    return np.frombuffer(buf, dtype=dtype, count=n)


def _host_call(name_f64: str, name_f32: str, A: CSR, B: CSR, C_out: CSR | None, timing, tcls):
    if A.N != B.M:
        raise ValueError(f"A.N ({A.N}) != B.M ({B.M})")
    code = _dtype_code(A.val.dtype)
    if _dtype_code(B.val.dtype) != code:
        raise TypeError("A and B must have the same value type")
    L = _native.lib()
    fn = getattr(L, name_f64 if code == F64 else name_f32)
    vt = C.c_double if code == F64 else C.c_float
    arrs = [np.ascontiguousarray(x) for x in (A.rpt, A.col, A.val, B.rpt, B.col, B.val)]
    for a, dt in zip(arrs, (np.int32, np.int32, None, np.int32, np.int32, None)):
        if dt is not None and a.dtype != dt:
            raise TypeError("row pointers and columns must be int32")
    crpt = _native.c_int_p()
    ccol = _native.c_int_p()
    cval = C.POINTER(vt)()
    cnnz = C.c_int(0)
    tc = tcls._c()
    st = fn(*[_ptr(a) for a in arrs], C.byref(crpt), C.byref(ccol), C.byref(cval),
            A.M, A.N, B.N, C.byref(cnnz), C.byref(tc))
    _native.check(st, name_f64)
    n = cnnz.value
    # the result arrays stay where the library put them (page-locked host
    # blocks); numpy views own them and hand them back through brm_free
    rpt = _owned(L, crpt, A.M + 1, C.c_int, np.int32)
    col = _owned(L, ccol, n, C.c_int, np.int32)
    val = _owned(L, cval, n, vt, np.float64 if code == F64 else np.float32)
    if timing is not None:
        timing._load(tc)
    out = C_out if C_out is not None else CSR(0, 0, np.zeros(1, np.int32), np.zeros(0, np.int32),
                                              np.zeros(0))
    out.M, out.N, out.rpt, out.col, out.val = A.M, B.N, rpt, col, val
    return out


def brmerge_precise(A: CSR, B: CSR, C_out: CSR | None = None,
                    timing: PreciseTiming | None = None) -> CSR:
    """C = A*B by BRMerge-Precise (spgemm.h:737-741) on the GPU."""
    return _host_call("brm_precise", "brm_precise_f32", A, B, C_out, timing, PreciseTiming)


def brmerge_upper(A: CSR, B: CSR, C_out: CSR | None = None,
                  timing: UpperTiming | None = None) -> CSR:
    """C = A*B by BRMerge-Upper (spgemm.h:460-464) on the GPU."""
    return _host_call("brm_upper", "brm_upper_f32", A, B, C_out, timing, UpperTiming)


class MtxTiming(_Timing):
    """Phase times (seconds) of a MatrixMarket read (brm_mtx_timing)."""
    _c = _native.MtxTimingC


def read_mtx(path, dtype=np.float64, timing: MtxTiming | None = None) -> CSR:
    """Reads a MatrixMarket coordinate file into a host CSR (brm_read_mtx;
    the reference's CSR::construct, CSR.cpp:259-479), parsing it on the GPU.
    Raises BrmError (BRM_ERR_FORMAT / BRM_ERR_IO) on a bad file."""
    code = _dtype_code(dtype)
    L = _native.lib()
    M, N, n = C.c_int(), C.c_int(), C.c_int()
    pr, pc, pv = C.c_void_p(), C.c_void_p(), C.c_void_p()
    tc = _native.MtxTimingC()
    _native.check(L.brm_read_mtx(str(path).encode(), code, C.byref(M), C.byref(N), C.byref(n),
                                 C.byref(pr), C.byref(pc), C.byref(pv), C.byref(tc)),
                  "brm_read_mtx")
    vt = C.c_double if code == F64 else C.c_float
    rpt = _owned(L, pr.value, M.value + 1, C.c_int, np.int32)
    col = _owned(L, pc.value, n.value, C.c_int, np.int32)
    val = _owned(L, pv.value, n.value, vt, np.float64 if code == F64 else np.float32)
    if timing is not None:
        timing._load(tc)
    return CSR(M.value, N.value, rpt, col, val)


# ---------------------------------------------------------------------------
# device-resident form
# ---------------------------------------------------------------------------

@dataclass
class DeviceCSR:
    """CSR on the GPU: rpt/col int32 and val float64/float32 torch CUDA tensors."""
    M: int
    N: int
    rpt: object
    col: object
    val: object

    @property
    def nnz(self) -> int:
        return int(self.col.numel())

    @staticmethod
    def from_host(X: CSR, device="cuda", non_blocking=False) -> "DeviceCSR":
        import torch
        t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(device, non_blocking=non_blocking)
        return DeviceCSR(X.M, X.N, t(X.rpt), t(X.col), t(X.val))

    def to_host(self) -> CSR:
        return CSR(self.M, self.N, self.rpt.cpu().numpy(), self.col.cpu().numpy(),
                   self.val.cpu().numpy())

    def c(self) -> _native.CsrC:
        return _native.CsrC(self.M, self.N, self.nnz, self.rpt.data_ptr(),
                            self.col.data_ptr() if self.col.numel() else None,
                            self.val.data_ptr() if self.val.numel() else None)


class Context:
    """A brm_context bound to the current CUDA device and a stream."""

    def __init__(self, stream=None, validate: bool = False):
        self._L = _native.lib()
        self._h = C.c_void_p()
        _native.check(self._L.brm_create(C.byref(self._h)), "brm_create")
        self.set_stream(stream)
        self.set_validate(validate)

    def close(self):
        if self._h:
            self._L.brm_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_stream(self, stream=None):
        ptr = None
        if stream is not None:
            ptr = stream.cuda_stream if hasattr(stream, "cuda_stream") else int(stream)
        _native.check(self._L.brm_set_stream(self._h, ptr), "brm_set_stream")

    def set_validate(self, on: bool):
        _native.check(self._L.brm_set_validate(self._h, 1 if on else 0), "brm_set_validate")

    def set_tuning(self, seg_cut: int | None = None, mid_flop: int | None = None,
                   long_scratch: int | None = None):
        """brm_set_tuning; no arguments restores the defaults."""
        if seg_cut is None and mid_flop is None and long_scratch is None:
            _native.check(self._L.brm_set_tuning(self._h, None), "brm_set_tuning")
            return
        cur = self.tuning()
        t = _native.TuningC(seg_cut if seg_cut is not None else cur["seg_cut"],
                            mid_flop if mid_flop is not None else cur["mid_flop"],
                            long_scratch if long_scratch is not None else cur["long_scratch"])
        _native.check(self._L.brm_set_tuning(self._h, C.byref(t)), "brm_set_tuning")

    def tuning(self) -> dict:
        t = _native.TuningC()
        _native.check(self._L.brm_get_tuning(self._h, C.byref(t)), "brm_get_tuning")
        return {"seg_cut": t.seg_cut, "mid_flop": t.mid_flop, "long_scratch": t.long_scratch}

    def autotune(self, pairs) -> dict:
        """brm_autotune on a list of (A, B) DeviceCSR pairs (one pair: the
        single-product form; several: the batched form); keeps and returns
        the fastest setting."""
        import torch
        n = len(pairs)
        code = _dtype_code(np.float64 if pairs[0][0].val.dtype == torch.float64 else np.float32)
        As = (_native.CsrC * n)(*[a.c() for a, _ in pairs])
        Bs = (_native.CsrC * n)(*[b.c() for _, b in pairs])
        t = _native.TuningC()
        _native.check(self._L.brm_autotune(self._h, code, n, As, Bs, C.byref(t)), "brm_autotune")
        return {"seg_cut": t.seg_cut, "mid_flop": t.mid_flop, "long_scratch": t.long_scratch}

    @property
    def last_device_error(self) -> int:
        return self._L.brm_last_device_error(self._h)

    def symbolic(self, A: DeviceCSR, B: DeviceCSR):
        """Returns (crpt tensor [M+1], nnz(C))."""
        import torch
        crpt = torch.empty(A.M + 1, dtype=torch.int32, device=A.rpt.device)
        cnnz = C.c_int(0)
        a, b = A.c(), B.c()
        _native.check(self._L.brm_symbolic(self._h, C.byref(a), C.byref(b), crpt.data_ptr(),
                                           C.byref(cnnz)), "brm_symbolic")
        return crpt, cnnz.value

    def numeric(self, A: DeviceCSR, B: DeviceCSR, crpt, cnnz: int, out=None) -> DeviceCSR:
        import torch
        code = _dtype_code(np.float64 if A.val.dtype == torch.float64 else np.float32)
        if out is None:
            ccol = torch.empty(max(cnnz, 0), dtype=torch.int32, device=A.rpt.device)
            cval = torch.empty(max(cnnz, 0), dtype=A.val.dtype, device=A.rpt.device)
        else:
            ccol, cval = out
        a, b = A.c(), B.c()
        _native.check(self._L.brm_numeric(self._h, code, C.byref(a), C.byref(b), crpt.data_ptr(),
                                          ccol.data_ptr() if cnnz else None,
                                          cval.data_ptr() if cnnz else None), "brm_numeric")
        return DeviceCSR(A.M, B.N, crpt, ccol[:cnnz], cval[:cnnz])

    def precise(self, A: DeviceCSR, B: DeviceCSR) -> DeviceCSR:
        crpt, cnnz = self.symbolic(A, B)
        return self.numeric(A, B, crpt, cnnz)

    def _device_call(self, upper: bool, A: DeviceCSR, B: DeviceCSR, timing=None) -> DeviceCSR:
        import torch
        code = _dtype_code(np.float64 if A.val.dtype == torch.float64 else np.float32)
        pr, pc, pv = C.c_void_p(), C.c_void_p(), C.c_void_p()
        cnnz = C.c_int(0)
        a, b = A.c(), B.c()
        tcls = UpperTiming if upper else PreciseTiming
        tc = tcls._c()
        fn = self._L.brm_upper_device if upper else self._L.brm_precise_device
        _native.check(fn(self._h, code, C.byref(a), C.byref(b), C.byref(pr), C.byref(pc),
                         C.byref(pv), C.byref(cnnz), C.byref(tc)),
                      "brm_upper_device" if upper else "brm_precise_device")
        n = cnnz.value
        dev = A.rpt.device
        vt = "<f8" if A.val.dtype == torch.float64 else "<f4"
        # the callee-allocated buffers become the tensors' storage; each is
        # released with brm_device_free when its tensor is collected
        crpt = _device_tensor(self._L, pr.value, A.M + 1, "<i4", dev)
        ccol = _device_tensor(self._L, pc.value, n, "<i4", dev)
        cval = _device_tensor(self._L, pv.value, n, vt, dev)
        if timing is not None:
            timing._load(tc)
        return DeviceCSR(A.M, B.N, crpt, ccol, cval)

    def precise_device(self, A: DeviceCSR, B: DeviceCSR, timing=None) -> DeviceCSR:
        """brm_precise_device: one call, callee-allocated outputs (no copy)."""
        return self._device_call(False, A, B, timing)

    def batch_precise_raw(self, pairs):
        """brm_batch_precise on a list of (A_i, B_i) DeviceCSR pairs of one
        value type.  Returns (crpt, ccol, cval, row_off, nnz_off, rpt_local):
        the concatenated C_i as device tensors (crpt holds offsets into
        ccol/cval, columns are each C_i's own), the host offsets of every pair,
        and every pair's own row pointers (pair i at row_off[i] + i)."""
        import torch
        n = len(pairs)
        dt = pairs[0][0].val.dtype
        if any(a.val.dtype != dt or b.val.dtype != dt for a, b in pairs):
            raise TypeError("all pairs of a batch must have the same value type")
        code = _dtype_code(np.float64 if dt == torch.float64 else np.float32)
        As = (_native.CsrC * n)(*[a.c() for a, _ in pairs])
        Bs = (_native.CsrC * n)(*[b.c() for _, b in pairs])
        out = _native.BatchC()
        _native.check(self._L.brm_batch_precise(self._h, code, n, As, Bs, C.byref(out)),
                      "brm_batch_precise")
        dev = pairs[0][0].rpt.device
        vt = "<f8" if dt == torch.float64 else "<f4"
        crpt = _device_tensor(self._L, out.crpt, out.rows + 1, "<i4", dev)
        ccol = _device_tensor(self._L, out.ccol, out.nnz, "<i4", dev)
        cval = _device_tensor(self._L, out.cval, out.nnz, vt, dev)
        lrpt = _device_tensor(self._L, out.rpt_local, out.rows + n, "<i4", dev)
        roff = np.ctypeslib.as_array(out.row_off, shape=(n + 1,)).copy()
        noff = np.ctypeslib.as_array(out.nnz_off, shape=(n + 1,)).copy()
        out.crpt = out.ccol = out.cval = out.rpt_local = None  # owned by the tensors now
        self._L.brm_batch_free(self._h, C.byref(out))
        return crpt, ccol, cval, roff, noff, lrpt

    def batch_graph(self, pairs) -> "BatchGraph":
        """brm_batch_graph_create: a batch of fixed structure whose values can
        be recomputed with one CUDA-graph launch (BatchGraph.launch)."""
        return BatchGraph(self, pairs)

    def batch_pipe(self, pairs=None, headroom: float = 1.25, caps: dict | None = None,
                   dtype=None) -> "BatchPipe":
        """brm_batch_pipe_create: a batch pipeline captured once and run once
        per new batch (BatchPipe.run).  Capacities from `caps` (a dict of
        brm_batch_caps fields) or from a sample list of pairs scaled by
        headroom."""
        return BatchPipe(self, pairs, headroom, caps, dtype)

    def batch_precise(self, pairs) -> list:
        """brm_batch_precise: C_i = A_i * B_i for a list of (A_i, B_i)
        DeviceCSR pairs of one value type, in one pipeline.  Returns the C_i
        as DeviceCSR views into the batch's concatenated arrays."""
        import torch
        if len(pairs) == 0:
            return []
        _, ccol, cval, roff, noff, lrpt = self.batch_precise_raw(pairs)
        res = []
        for i, (a, b) in enumerate(pairs):
            r0, r1, n0, n1 = int(roff[i]), int(roff[i + 1]), int(noff[i]), int(noff[i + 1])
            res.append(DeviceCSR(a.M, b.N, lrpt[r0 + i:r1 + i + 1], ccol[n0:n1], cval[n0:n1]))
        return res

    def hash_device(self, A: DeviceCSR, B: DeviceCSR) -> DeviceCSR:
        """brm_hash_device: the hash SpGEMM comparator (same structure as
        Precise, values summed in hardware order)."""
        import torch
        code = _dtype_code(np.float64 if A.val.dtype == torch.float64 else np.float32)
        pr, pc, pv = C.c_void_p(), C.c_void_p(), C.c_void_p()
        cnnz = C.c_int(0)
        a, b = A.c(), B.c()
        _native.check(self._L.brm_hash_device(self._h, code, C.byref(a), C.byref(b), C.byref(pr),
                                              C.byref(pc), C.byref(pv), C.byref(cnnz)),
                      "brm_hash_device")
        n = cnnz.value
        dev = A.rpt.device
        vt = "<f8" if A.val.dtype == torch.float64 else "<f4"
        return DeviceCSR(A.M, B.N, _device_tensor(self._L, pr.value, A.M + 1, "<i4", dev),
                         _device_tensor(self._L, pc.value, n, "<i4", dev),
                         _device_tensor(self._L, pv.value, n, vt, dev))

    def read_mtx_device(self, path, dtype=np.float64, timing: MtxTiming | None = None,
                        device="cuda") -> DeviceCSR:
        """brm_read_mtx_device: a MatrixMarket file straight into device CSR."""
        code = _dtype_code(dtype)
        M, N, n = C.c_int(), C.c_int(), C.c_int()
        pr, pc, pv = C.c_void_p(), C.c_void_p(), C.c_void_p()
        tc = _native.MtxTimingC()
        _native.check(self._L.brm_read_mtx_device(self._h, code, str(path).encode(), C.byref(M),
                                                  C.byref(N), C.byref(n), C.byref(pr),
                                                  C.byref(pc), C.byref(pv), C.byref(tc)),
                      "brm_read_mtx_device")
        vt = "<f8" if code == F64 else "<f4"
        rpt = _device_tensor(self._L, pr.value, M.value + 1, "<i4", device)
        col = _device_tensor(self._L, pc.value, n.value, "<i4", device)
        val = _device_tensor(self._L, pv.value, n.value, vt, device)
        if timing is not None:
            timing._load(tc)
        return DeviceCSR(M.value, N.value, rpt, col, val)

    def upper(self, A: DeviceCSR, B: DeviceCSR, timing=None) -> DeviceCSR:
        """brm_upper_device: one call, callee-allocated outputs (no copy)."""
        return self._device_call(True, A, B, timing)

    def compute_flop(self, A: DeviceCSR, B: DeviceCSR) -> int:
        out = C.c_longlong(0)
        a, b = A.c(), B.c()
        _native.check(self._L.brm_compute_flop(self._h, C.byref(a), C.byref(b), C.byref(out)),
                      "brm_compute_flop")
        return out.value

    def upper_bound(self, A: DeviceCSR, B: DeviceCSR, dtype=np.float64):
        prod, nbytes = C.c_longlong(0), C.c_longlong(0)
        a, b = A.c(), B.c()
        _native.check(self._L.brm_upper_bound(self._h, _dtype_code(dtype), C.byref(a), C.byref(b),
                                              C.byref(prod), C.byref(nbytes)), "brm_upper_bound")
        return prod.value, nbytes.value

    def validate(self, X: DeviceCSR, ncols: int | None = None) -> int:
        """-1 if X is valid CSR, else the first offending row."""
        bad = C.c_int(-1)
        x = X.c()
        st = self._L.brm_validate(self._h, C.byref(x), X.N if ncols is None else ncols,
                                  C.byref(bad))
        if st not in (0, 2):
            _native.check(st, "brm_validate")
        return bad.value


class _RawDevice:
    """A raw device allocation exposed through __cuda_array_interface__."""

    def __init__(self, ptr: int, n: int, typestr: str):
        self.__cuda_array_interface__ = {
            "shape": (n,), "typestr": typestr, "data": (ptr, False), "version": 2, "strides": None}


class BatchGraph:
    """A batch of fixed structure (brm_batch_graph_*).  `results` are views
    of C_i owned by the graph (valid until close); `launch` recomputes them
    from the pairs' current values with one graph launch."""

    def __init__(self, ctx: "Context", pairs):
        import torch
        self._L = _native.lib()
        self._h = C.c_void_p()
        self._pairs = list(pairs)  # the graph reads their arrays at every launch
        n = len(self._pairs)
        dt = self._pairs[0][0].val.dtype
        code = _dtype_code(np.float64 if dt == torch.float64 else np.float32)
        As = (_native.CsrC * n)(*[a.c() for a, _ in self._pairs])
        Bs = (_native.CsrC * n)(*[b.c() for _, b in self._pairs])
        out = _native.BatchC()
        _native.check(self._L.brm_batch_graph_create(ctx._h, code, n, As, Bs, C.byref(self._h),
                                                     C.byref(out)), "brm_batch_graph_create")
        dev = self._pairs[0][0].rpt.device
        vt = "<f8" if dt == torch.float64 else "<f4"

        def view(ptr, m, ts, tdt):
            if m == 0 or not ptr:
                return torch.empty(m, dtype=tdt, device=dev)
            return torch.as_tensor(_RawDevice(ptr, m, ts), device=dev)

        ccol = view(out.ccol, out.nnz, "<i4", torch.int32)
        cval = view(out.cval, out.nnz, vt, dt)
        lrpt = view(out.rpt_local, out.rows + n, "<i4", torch.int32)
        roff = np.ctypeslib.as_array(out.row_off, shape=(n + 1,)).copy()
        noff = np.ctypeslib.as_array(out.nnz_off, shape=(n + 1,)).copy()
        self.results = []
        for i, (a, b) in enumerate(self._pairs):
            r0, r1, n0, n1 = int(roff[i]), int(roff[i + 1]), int(noff[i]), int(noff[i + 1])
            self.results.append(DeviceCSR(a.M, b.N, lrpt[r0 + i:r1 + i + 1], ccol[n0:n1],
                                          cval[n0:n1]))

    def launch(self, stream=None):
        ptr = None
        if stream is not None:
            ptr = stream.cuda_stream if hasattr(stream, "cuda_stream") else int(stream)
        _native.check(self._L.brm_batch_graph_launch(self._h, ptr), "brm_batch_graph_launch")

    def close(self):
        if self._h:
            self.results = []
            self._L.brm_batch_graph_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class BatchPipe:
    """A captured batch pipeline (brm_batch_pipe_*).  `run(pairs)` computes a
    new batch with one graph launch and returns the C_i as DeviceCSR views of
    the pipe's own arrays, valid until the next run or close."""

    def __init__(self, ctx: "Context", pairs, headroom: float, caps: dict | None, dtype):
        import torch
        self._L = _native.lib()
        self._h = C.c_void_p()
        if caps is None:
            n = len(pairs)
            dt = pairs[0][0].val.dtype
            self._code = _dtype_code(np.float64 if dt == torch.float64 else np.float32)
            As = (_native.CsrC * n)(*[a.c() for a, _ in pairs])
            Bs = (_native.CsrC * n)(*[b.c() for _, b in pairs])
            cc = _native.BatchCapsC()
            _native.check(self._L.brm_batch_caps_for(ctx._h, self._code, n, As, Bs,
                                                     float(headroom), C.byref(cc)),
                          "brm_batch_caps_for")
        else:
            self._code = _dtype_code(dtype or np.float64)
            cc = _native.BatchCapsC(**caps)
        _native.check(self._L.brm_batch_pipe_create(ctx._h, self._code, C.byref(cc),
                                                    C.byref(self._h)), "brm_batch_pipe_create")

    def caps(self) -> dict:
        cc = _native.BatchCapsC()
        _native.check(self._L.brm_batch_pipe_caps(self._h, C.byref(cc)), "brm_batch_pipe_caps")
        return {f: getattr(cc, f) for f, _ in cc._fields_}

    def run_raw(self, pairs, stream=None):
        """(ccol, cval, row_off, nnz_off, rpt_local, nnz) of the batch, views
        of the pipe's arrays (valid until the next run)."""
        import torch
        n = len(pairs)
        dt = pairs[0][0].val.dtype
        As = (_native.CsrC * n)(*[a.c() for a, _ in pairs])
        Bs = (_native.CsrC * n)(*[b.c() for _, b in pairs])
        ptr = None
        if stream is not None:
            ptr = stream.cuda_stream if hasattr(stream, "cuda_stream") else int(stream)
        out = _native.BatchC()
        _native.check(self._L.brm_batch_pipe_run(self._h, n, As, Bs, ptr, C.byref(out)),
                      "brm_batch_pipe_run")
        dev = pairs[0][0].rpt.device
        vt = "<f8" if dt == torch.float64 else "<f4"

        def view(p, m, ts, tdt):
            if m == 0 or not p:
                return torch.empty(m, dtype=tdt, device=dev)
            return torch.as_tensor(_RawDevice(p, m, ts), device=dev)

        ccol = view(out.ccol, out.nnz, "<i4", torch.int32)
        cval = view(out.cval, out.nnz, vt, dt)
        lrpt = view(out.rpt_local, out.rows + n, "<i4", torch.int32)
        roff = np.ctypeslib.as_array(out.row_off, shape=(n + 1,)).copy()
        noff = np.ctypeslib.as_array(out.nnz_off, shape=(n + 1,)).copy()
        return ccol, cval, roff, noff, lrpt, int(out.nnz)

    def run(self, pairs, stream=None) -> list:
        ccol, cval, roff, noff, lrpt, _ = self.run_raw(pairs, stream)
        res = []
        for i, (a, b) in enumerate(pairs):
            r0, r1, n0, n1 = int(roff[i]), int(roff[i + 1]), int(noff[i]), int(noff[i + 1])
            res.append(DeviceCSR(a.M, b.N, lrpt[r0 + i:r1 + i + 1], ccol[n0:n1], cval[n0:n1]))
        return res

    def close(self):
        if self._h:
            self._L.brm_batch_pipe_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class _Ticket:
    """A finished server request; released when its last view is collected."""

    def __init__(self, server, ticket: int):
        self._srv, self.ticket = server, ticket

    def __del__(self):
        self._srv._release(self.ticket)


class _ServerBlock(_RawDevice):
    def __init__(self, owner: _Ticket, ptr: int, n: int, typestr: str):
        super().__init__(ptr, n, typestr)
        self._owner = owner


class Server:
    """brm_server: C = A * B requests from any thread, admitted in rounds on
    the device and batched by worker threads under a memory cap (one
    stacked-operand pipeline per batch); express workers take the small
    requests on high-priority streams.  A rejected request raises from
    wait()."""

    def __init__(self, mem_cap_bytes: int = 0, max_batch: int = 0, workers: int = 0,
                 express_workers: int = 1, express_bytes: int = 0, express_sms: int = 0):
        self._L = _native.lib()
        self._h = C.c_void_p()
        cfg = _native.ServerConfigC(mem_cap_bytes, max_batch, workers,
                                    express_workers if express_workers > 0 else -1, express_bytes,
                                    express_sms)
        _native.check(self._L.brm_server_create(C.byref(cfg), C.byref(self._h)),
                      "brm_server_create")
        self._inputs = {}  # ticket -> (A, B): kept alive until the result is waited for

    def sms(self) -> tuple:
        """(express partition SMs, other workers' SMs); (0, 0) without partitions."""
        x, o = C.c_int(0), C.c_int(0)
        _native.check(self._L.brm_server_sms(self._h, C.byref(x), C.byref(o)), "brm_server_sms")
        return x.value, o.value

    def submit(self, A: "DeviceCSR", B: "DeviceCSR") -> int:
        import torch
        code = _dtype_code(np.float64 if A.val.dtype == torch.float64 else np.float32)
        t = C.c_longlong(0)
        a, b = A.c(), B.c()
        _native.check(self._L.brm_server_submit(self._h, code, C.byref(a), C.byref(b),
                                                C.byref(t)), "brm_server_submit")
        self._inputs[t.value] = (A, B)
        return t.value

    def wait(self, ticket: int, timeout: float = -1.0):
        """Returns (C as DeviceCSR views, stats); the views keep the result
        alive, and it is released when the last of them is collected."""
        import torch
        r = _native.ServerResultC()
        st = self._L.brm_server_wait(self._h, ticket, timeout, C.byref(r))
        if st == 8:  # BRM_ERR_TIMEOUT
            raise TimeoutError(f"request {ticket} not done after {timeout} s")
        A, B = self._inputs.pop(ticket)
        owner = _Ticket(self, ticket)
        _native.check(st, "brm_server_wait")
        dev = A.rpt.device
        vt = "<f8" if A.val.dtype == torch.float64 else "<f4"

        def view(ptr, n, ts, dt):
            if n == 0 or not ptr:
                return torch.empty(n, dtype=dt, device=dev)
            return torch.as_tensor(_ServerBlock(owner, ptr, n, ts), device=dev)

        rpt = view(r.rpt, r.M + 1, "<i4", torch.int32)
        col = view(r.col, r.nnz, "<i4", torch.int32)
        val = view(r.val, r.nnz, vt, A.val.dtype)
        stats = {"queued_s": r.queued_s, "latency_s": r.latency_s, "batch_size": r.batch_size}
        return DeviceCSR(r.M, r.N, rpt, col, val), stats

    def _release(self, ticket: int):
        if self._h:
            self._L.brm_server_release(self._h, ticket)

    def close(self):
        if self._h:
            self._L.brm_server_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class _DeviceBlock(_RawDevice):
    """A callee-allocated device buffer that brm_device_free releases when
    the last tensor viewing it is gone (stream-ordered on the legacy stream)."""

    def __init__(self, L, ptr: int, n: int, typestr: str):
        super().__init__(ptr, n, typestr)
        self._L, self._p = L, ptr

    def __del__(self):
        if self._p:
            self._L.brm_device_free(None, self._p)
            self._p = None


def _device_tensor(L, ptr, n: int, typestr: str, device):
    import torch
    dt = {"<i4": torch.int32, "<f8": torch.float64, "<f4": torch.float32}[typestr]
    if not ptr:
        return torch.empty(n, dtype=dt, device=device)
    if n == 0:
        L.brm_device_free(None, ptr)
        return torch.empty(0, dtype=dt, device=device)
    return torch.as_tensor(_DeviceBlock(L, ptr, n, typestr), device=device)


def compute_flop_host(A: CSR, B: CSR) -> int:
    """Intermediate products of A*B from host arrays (numpy; no GPU needed)."""
    blen = np.diff(B.rpt.astype(np.int64))
    return int(blen[A.col].sum()) if A.nnz else 0
