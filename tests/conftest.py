import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

GOLDEN = ROOT / "tests" / "golden"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); run with -m gpu")


def pytest_collection_modifyitems(config, items):
    try:
        import torch
        has_gpu = torch.cuda.is_available()
    except Exception:
        has_gpu = False
    if has_gpu:
        return
    skip = pytest.mark.skip(reason="no CUDA GPU in this environment")
    for it in items:
        if "gpu" in it.keywords:
            it.add_marker(skip)


def load_golden(name):
    """(A, B, C) of a golden fixture as CSR objects."""
    from brmerge_gb300.csr import CSR
    z = np.load(GOLDEN / f"{name}.npz")
    M, K, N = int(z["M"]), int(z["K"]), int(z["N"])
    A = CSR(M, K, z["A_rpt"], z["A_col"], z["A_val"])
    B = CSR(K, N, z["B_rpt"], z["B_col"], z["B_val"])
    C = CSR(M, N, z["C_rpt"], z["C_col"], z["C_val"])
    return A, B, C


# SpGEMM fixtures (mtx_cases.npz holds the MatrixMarket reader's cases)
GOLDEN_NAMES = sorted(p.stem for p in GOLDEN.glob("*.npz") if not p.stem.startswith("mtx_"))


def assert_same_csr(C, R, what=""):
    """Bit-exact structure and values."""
    assert np.array_equal(np.asarray(C.rpt), np.asarray(R.rpt)), f"{what}: rpt differs"
    assert np.array_equal(np.asarray(C.col), np.asarray(R.col)), f"{what}: col differs"
    cv, rv = np.asarray(C.val), np.asarray(R.val)
    assert cv.dtype == rv.dtype, f"{what}: dtype {cv.dtype} vs {rv.dtype}"
    iv = np.int64 if cv.dtype == np.float64 else np.int32
    if not np.array_equal(cv.view(iv), rv.view(iv)):
        bad = np.nonzero(cv.view(iv) != rv.view(iv))[0]
        raise AssertionError(f"{what}: {len(bad)} values differ, first at {bad[:5]}: "
                             f"{cv[bad[:5]]} vs {rv[bad[:5]]}")


@pytest.fixture(scope="session")
def oracle_mod():
    import oracle
    oracle.build()
    return oracle
