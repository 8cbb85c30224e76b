"""The oracle restatement against the reference (CPU only).

The restatement (oracle/brm_oracle.c) is pinned to the reference in two ways:
against the committed golden fixtures, which the reference itself produced
(tests/golden/make_golden.py), and, where the reference sources are present,
against the reference compiled by oracle/build_ref.sh on fresh seeded inputs.
"""
import numpy as np
import pytest

from conftest import GOLDEN_NAMES, assert_same_csr, load_golden


@pytest.mark.parametrize("name", GOLDEN_NAMES)
def test_oracle_precise_matches_golden(oracle_mod, name):
    A, B, C = load_golden(name)
    assert_same_csr(oracle_mod.precise(A, B), C, name)


@pytest.mark.parametrize("name", GOLDEN_NAMES)
def test_oracle_upper_matches_golden(oracle_mod, name):
    A, B, C = load_golden(name)
    assert_same_csr(oracle_mod.upper(A, B), C, name)


@pytest.mark.parametrize("nthreads", [1, 3, 8])
def test_oracle_thread_count_independent(oracle_mod, nthreads):
    from brmerge_gb300 import gen_rmat
    A = gen_rmat(11, int(2.35 * 2048), seed=5)
    assert_same_csr(oracle_mod.precise(A, A, nthreads), oracle_mod.precise(A, A, 1), "threads")


def _ref_or_skip(oracle_mod):
    if not oracle_mod.ref_available():
        pytest.skip("reference sources not present on this host")


@pytest.mark.parametrize("seed", range(4))
def test_oracle_matches_reference_random(oracle_mod, seed):
    _ref_or_skip(oracle_mod)
    from brmerge_gb300 import gen_lognormal, gen_rmat, gen_uniform
    cases = [
        (gen_rmat(12, int(2.35 * 4096), seed=seed), None),
        (gen_uniform(300, 500, 40, seed=seed), gen_uniform(500, 700, 60, seed=seed + 10)),
        (gen_lognormal(400, 400, seed=seed + 20), None),
    ]
    for A, B in cases:
        B = A if B is None else B
        R, _ = oracle_mod.ref_precise(A, B, 4)
        assert_same_csr(oracle_mod.precise(A, B), R, "precise")
        U, _ = oracle_mod.ref_upper(A, B, 4)
        assert_same_csr(oracle_mod.upper(A, B), U, "upper")
        assert_same_csr(U, R, "reference upper vs precise")


def test_oracle_matches_reference_er_config(oracle_mod):
    """The CPU configuration: ER n=16384, 8 per row, seed 0, C = A*A."""
    _ref_or_skip(oracle_mod)
    from brmerge_gb300 import gen_er
    A = gen_er(16384, 8, seed=0)
    R, _ = oracle_mod.ref_precise(A, A, 8)
    assert_same_csr(oracle_mod.precise(A, A), R, "er16384")


def test_golden_fixtures_are_valid_csr():
    for name in GOLDEN_NAMES:
        A, B, C = load_golden(name)
        A.check()
        B.check()
        C.check()


def test_oracle_f32_close_to_f64(oracle_mod):
    A, B, C = load_golden("rmat10")
    C32 = oracle_mod.precise(A.astype(np.float32), B.astype(np.float32))
    assert np.array_equal(C32.rpt, C.rpt) and np.array_equal(C32.col, C.col)
    err = np.abs(C32.val.astype(np.float64) - C.val)
    assert np.all(err <= 1e-5 * np.maximum(1.0, np.abs(C.val)))
