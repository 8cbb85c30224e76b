"""Build recipe for the native parts of brmerge_gb300 (no cmake).

* libbrmerge.so   -- the CUDA library behind include/brmerge.h, compiled for
                     sm_103a only (-gencode arch=compute_103a,code=sm_103a);
* libbrm_host.so  -- host-only helpers (synthetic generators, include/brm_gen.h).

Translation units are compiled in parallel into _build/ and linked in-tree
next to this file.  Output is only rebuilt when a source is newer.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
INCLUDE = ROOT / "include"
BUILD = PKG / "_build"

CUDA_SOURCES = [
    "brm_api.cu",
    "brm_analyze.cu",
    "brm_symbolic.cu",
    "brm_numeric_f64.cu",
    "brm_numeric_f32.cu",
    "brm_noalloc.cu",
    "brm_hostpool.cu",
    "brm_batch.cu",
    "brm_server.cu",
    "brm_mtx.cu",
    "brm_hash.cu",
]
HOST_SOURCES = ["host/gen.cpp", "host/numparse.cpp"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(cand).exists():
        raise RuntimeError("nvcc not found; the CUDA 13 toolkit is required to build libbrmerge.so")
    return cand


def _newer(target: Path, deps: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def _run(cmd: list[str]) -> str:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r.stdout + r.stderr


def build_cuda(verbose: bool = False, extra: list[str] | None = None) -> Path:
    """Compiles libbrmerge.so; `extra` (or the BRM_NVCC_FLAGS environment
    variable) adds nvcc flags, and a change of flags rebuilds every object."""
    nvcc = _nvcc()
    BUILD.mkdir(exist_ok=True)
    out = PKG / "libbrmerge.so"
    headers = list(CSRC.glob("*.cuh")) + list(CSRC.glob("*.h")) + [INCLUDE / "brmerge.h"]
    extra = list(extra or []) + os.environ.get("BRM_NVCC_FLAGS", "").split()
    flags = ARCH + [
        "-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-Wall",
        "-I", str(INCLUDE), "-I", str(CSRC),
    ] + extra
    if verbose:
        flags += ["-Xptxas", "-v"]
    stamp = BUILD / "flags.txt"
    same_flags = stamp.exists() and stamp.read_text() == " ".join(flags)
    objs = []
    jobs = []
    for src in CUDA_SOURCES:
        s = CSRC / src
        o = BUILD / (Path(src).stem + ".o")
        objs.append(o)
        if not same_flags or _newer(o, [s] + headers):
            jobs.append([nvcc] + flags + ["-c", str(s), "-o", str(o)])
    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        for log in ex.map(_run, jobs):
            if verbose:
                print(log)
    if jobs or _newer(out, objs):
        tmp = out.with_suffix(".so.tmp")
        _run([nvcc] + ARCH + ["-shared", "-cudart", "static", "-o", str(tmp)] + [str(o) for o in objs])
        os.replace(tmp, out)
    stamp.write_text(" ".join(flags))
    return out


def build_host() -> Path:
    cxx = shutil.which("g++") or "g++"
    out = PKG / "libbrm_host.so"
    srcs = [CSRC / s for s in HOST_SOURCES]
    if _newer(out, srcs + [INCLUDE / "brm_gen.h", CSRC / "brm_numparse.h", CSRC / "brm_pow5.h"]):
        tmp = out.with_suffix(".so.tmp")
        _run([cxx, "-O2", "-std=c++17", "-fPIC", "-shared", "-Wall", "-ffp-contract=off",
              "-I", str(INCLUDE), "-I", str(CSRC)]
             + [str(s) for s in srcs] + ["-o", str(tmp)])
        os.replace(tmp, out)
    return out


def build(verbose: bool = False, checked: bool | None = None) -> None:
    """Builds both libraries.  checked (default: the BRM_CHECKED environment
    variable) compiles the device code with -DBRM_CHECKED: every
    data-dependent index is checked against its bound, a failing access is
    skipped and reported through the device error word (brm_checked_build,
    brm_last_check_failure); a change of mode rebuilds every object."""
    if checked is None:
        checked = os.environ.get("BRM_CHECKED", "") not in ("", "0")
    with cf.ThreadPoolExecutor(max_workers=2) as ex:
        f1 = ex.submit(build_cuda, verbose, ["-DBRM_CHECKED"] if checked else None)
        f2 = ex.submit(build_host)
        f1.result()
        f2.result()


if __name__ == "__main__":
    build(verbose="-v" in sys.argv, checked=True if "--checked" in sys.argv else None)
    print("built", PKG / "libbrmerge.so", PKG / "libbrm_host.so")
