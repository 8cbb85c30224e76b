"""The C-ABI libraries load and export every declared entry point (CPU only)."""
import ctypes
import re
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


def declared(header):
    text = (ROOT / "include" / header).read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(brm_[a-z0-9_]+)\s*\(", text)))


@pytest.fixture(scope="module")
def built():
    from brmerge_gb300 import build
    build.build()
    return True


def test_brmerge_exports_all_declared(built):
    from brmerge_gb300 import _native
    lib = ctypes.CDLL(str(_native.lib_path()))
    names = declared("brmerge.h")
    assert "brm_precise" in names and "brm_symbolic" in names and "brm_numeric" in names
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, f"not exported: {missing}"


def test_gen_exports_all_declared(built):
    from brmerge_gb300 import _native
    lib = ctypes.CDLL(str(_native.host_lib_path()))
    missing = [n for n in declared("brm_gen.h") if not hasattr(lib, n)]
    assert not missing, f"not exported: {missing}"


def test_status_strings(built):
    from brmerge_gb300 import _native
    L = _native.lib()
    for s in range(13):
        assert L.brm_status_string(s)
    assert L.brm_status_string(0) == b"success"


@pytest.mark.gpu
def test_cuda_library_runs_sm103a_code(built):
    """The device code the library runs is the sm_103a build (the runtime's
    cudaFuncAttributes.binaryVersion of one of its kernels)."""
    import ctypes as C
    from brmerge_gb300 import _native
    sm = C.c_int(0)
    assert _native.lib().brm_device_code_version(C.byref(sm)) == 0
    assert sm.value == 103, sm.value


def test_product_package_does_not_import_oracle():
    pkg = ROOT / "brmerge_gb300"
    for p in pkg.rglob("*.py"):
        src = p.read_text()
        assert "import oracle" not in src and "from oracle" not in src, p
    for p in (pkg / "csrc").rglob("*"):
        if p.is_file():
            assert "brm_oracle" not in p.read_text(errors="ignore"), p


def test_no_cpu_fallback_without_library(tmp_path, monkeypatch):
    """Loading fails loudly when libbrmerge.so is absent."""
    from brmerge_gb300 import _native
    monkeypatch.setattr(_native, "_lib", None)
    monkeypatch.setattr(_native, "lib_path", lambda: tmp_path / "missing.so")
    with pytest.raises(RuntimeError, match="no CPU fallback"):
        _native.lib()
