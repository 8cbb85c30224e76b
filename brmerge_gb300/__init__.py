"""brmerge_gb300 -- BRMerge SpGEMM (C = A*B, CSR) on one NVIDIA GB300 GPU.

The hot path is hand-written sm_103a CUDA behind the C ABI in include/brmerge.h
(libbrmerge.so, built in-tree by ``python -m brmerge_gb300.build``).  This
package mirrors the reference's interface: ``CSR``, ``brmerge_precise``,
``brmerge_upper``, ``PreciseTiming`` / ``UpperTiming``, plus a device-resident
``Context`` over torch CUDA tensors (single products and batches), a request
``Server``, the MatrixMarket reader ``read_mtx`` (parsed on the GPU) and
seeded synthetic generators.
"""
from .csr import (CSR, gen_er, gen_lognormal, gen_rmat, gen_stencil27, gen_uniform)
from .spgemm import (Context, DeviceCSR, MtxTiming, PreciseTiming, Server, UpperTiming,
                     brmerge_precise, brmerge_upper, compute_flop_host, read_mtx)
from ._native import BrmError, lib_path, host_lib_path

__all__ = [
    "CSR", "DeviceCSR", "Context", "Server", "PreciseTiming", "UpperTiming", "brmerge_precise",
    "brmerge_upper", "compute_flop_host", "gen_er", "gen_rmat", "gen_stencil27",
    "gen_lognormal", "gen_uniform", "BrmError", "lib_path", "host_lib_path", "read_mtx",
    "MtxTiming",
]
