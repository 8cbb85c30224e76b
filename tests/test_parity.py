"""GPU parity: the CUDA path against the oracle and the reference's golden output.

Integer structure (row pointers, columns) must be bit-exact, and so must
double values, because the kernels add partial products in the reference's
merge-tree order.  float32 runs are bit-exact against the float32 oracle
(same order, same rounding) and within 1e-5 relative of the float64 oracle.
"""
import numpy as np
import pytest

import brmerge_gb300 as brm
from conftest import GOLDEN_NAMES, assert_same_csr, load_golden

pytestmark = pytest.mark.gpu

F32_RTOL = 1e-5


@pytest.fixture(scope="module")
def ctx():
    import torch  # noqa: F401
    c = brm.Context()
    yield c
    c.close()


def dev(X):
    return brm.DeviceCSR.from_host(X)


def gpu_precise(ctx, A, B):
    return ctx.precise(dev(A), dev(B)).to_host()


def gpu_upper(ctx, A, B):
    return ctx.upper(dev(A), dev(B)).to_host()


def gpu_precise_one_call(ctx, A, B):
    """brm_precise_device: mid rows computed during the plan, moved after."""
    return ctx.precise_device(dev(A), dev(B)).to_host()


def assert_f32_close(C32, R64):
    assert np.array_equal(C32.rpt, R64.rpt) and np.array_equal(C32.col, R64.col)
    ref = np.asarray(R64.val, np.float64)
    err = np.abs(np.asarray(C32.val, np.float64) - ref)
    # |error| <= 1e-5 * max(1, |ref|): values are sums of products of U[-1,1] entries
    assert np.all(err <= F32_RTOL * np.maximum(1.0, np.abs(ref))), float(err.max())


# ---------------------------------------------------------------------------
# golden fixtures (produced by the reference itself)
# ---------------------------------------------------------------------------

@pytest.mark.parametrize("name", GOLDEN_NAMES)
def test_golden_host_precise(name):
    A, B, C = load_golden(name)
    assert_same_csr(brm.brmerge_precise(A, B), C, name)


@pytest.mark.parametrize("name", GOLDEN_NAMES)
def test_golden_host_upper(name):
    A, B, C = load_golden(name)
    assert_same_csr(brm.brmerge_upper(A, B), C, name)


@pytest.mark.parametrize("name", GOLDEN_NAMES)
def test_golden_device_split(ctx, name):
    A, B, C = load_golden(name)
    assert_same_csr(gpu_precise(ctx, A, B), C, name)
    assert_same_csr(gpu_upper(ctx, A, B), C, name)


# ---------------------------------------------------------------------------
# seeded inputs against the oracle
# ---------------------------------------------------------------------------

def _cases():
    yield "er2048", brm.gen_er(2048, 8, seed=3), None
    yield "rmat12", brm.gen_rmat(12, int(2.35 * 4096), seed=4), None
    yield "rmat14", brm.gen_rmat(14, int(2.35 * 16384), seed=5), None
    yield "stencil10", brm.gen_stencil27(10, seed=6), None
    yield "lognormal", brm.gen_lognormal(3000, 2500, seed=7), brm.gen_lognormal(2500, 4000, seed=8)
    yield "uniform_dense", brm.gen_uniform(64, 400, 300, seed=9), brm.gen_uniform(400, 500, 200, seed=10)
    yield "wide_span", brm.gen_uniform(50, 2000, 80, seed=11), brm.gen_uniform(2000, 1_500_000, 60, seed=12)


CASES = list(_cases())


@pytest.mark.parametrize("name,A,B", CASES, ids=[c[0] for c in CASES])
def test_precise_matches_oracle(ctx, oracle_mod, name, A, B):
    B = A if B is None else B
    assert_same_csr(gpu_precise(ctx, A, B), oracle_mod.precise(A, B), name)


@pytest.mark.parametrize("name,A,B", CASES, ids=[c[0] for c in CASES])
def test_precise_one_call_matches_oracle(ctx, oracle_mod, name, A, B):
    B = A if B is None else B
    assert_same_csr(gpu_precise_one_call(ctx, A, B), oracle_mod.precise(A, B), name)


@pytest.mark.parametrize("name,A,B", CASES, ids=[c[0] for c in CASES])
def test_upper_matches_oracle(ctx, oracle_mod, name, A, B):
    B = A if B is None else B
    assert_same_csr(gpu_upper(ctx, A, B), oracle_mod.precise(A, B), name)


@pytest.mark.parametrize("name,A,B", CASES[:5], ids=[c[0] for c in CASES[:5]])
def test_f32(ctx, oracle_mod, name, A, B):
    B = A if B is None else B
    A32, B32 = A.astype(np.float32), B.astype(np.float32)
    C32 = gpu_precise(ctx, A32, B32)
    assert_same_csr(C32, oracle_mod.precise(A32, B32), name + " f32 order-exact")
    assert_f32_close(C32, oracle_mod.precise(A, B))
    assert_same_csr(gpu_upper(ctx, A32, B32), C32, name + " f32 upper")
    assert_same_csr(gpu_precise_one_call(ctx, A32, B32), C32, name + " f32 one call")


def test_host_drop_in_matches_device(ctx):
    A = brm.gen_rmat(13, int(2.35 * 8192), seed=13)
    t = brm.PreciseTiming()
    C1 = brm.brmerge_precise(A, A, timing=t)
    assert t.total > 0
    assert_same_csr(C1, gpu_precise(ctx, A, A), "host vs device")


PRECISE_PHASES = ("pre_allocate", "compute_flop", "prefix_sum_flop", "load_balance", "symbolic",
                  "prefix_sum_nnz", "allocate_C", "compute", "cleanup")
UPPER_PHASES = ("pre_allocate", "compute_flop", "prefix_sum_flop", "load_balance",
                "allocate_hook", "compute", "prefix_sum_nnz", "allocate_C", "copy", "cleanup")


def _check_phases(t, names, must_be_positive):
    vals = {n: getattr(t, n) for n in names}
    assert all(v >= 0 for v in vals.values()), vals
    for n in must_be_positive:
        assert vals[n] > 0, (n, vals)
    # the phases are disjoint intervals of one call (1 us of slack for the
    # rounding of event and wall-clock times)
    assert sum(vals.values()) <= t.total + 1e-6, (sum(vals.values()), t.total, vals)


def test_timing_fields(ctx):
    """Every form fills the reference's phase fields (Timings.h:4-46) from
    CUDA events, and the phases sum to at most the call's total time
    (spgemm.h:476-503 times compute_flop, prefix_sum_flop, load_balance and
    the rest as consecutive phases)."""
    A = brm.gen_rmat(14, int(2.35 * (1 << 14)), seed=17)
    gpu_phases = ("compute_flop", "prefix_sum_flop", "symbolic", "prefix_sum_nnz", "compute")
    for _ in range(2):  # the second call runs with grown workspaces
        t = brm.PreciseTiming()
        brm.brmerge_precise(A, A, timing=t)
        _check_phases(t, PRECISE_PHASES, gpu_phases + ("pre_allocate", "load_balance"))
        u = brm.UpperTiming()
        brm.brmerge_upper(A, A, timing=u)
        _check_phases(u, UPPER_PHASES, ("pre_allocate", "compute_flop", "prefix_sum_flop",
                                        "load_balance", "compute", "prefix_sum_nnz", "copy"))
        dA = brm.DeviceCSR.from_host(A)
        t = brm.PreciseTiming()
        ctx.precise_device(dA, dA, timing=t)
        _check_phases(t, PRECISE_PHASES, gpu_phases + ("load_balance",))
        u = brm.UpperTiming()
        ctx.upper(dA, dA, timing=u)
        _check_phases(u, UPPER_PHASES, ("compute_flop", "prefix_sum_flop", "load_balance",
                                        "compute", "prefix_sum_nnz", "copy"))


def test_host_results_are_independent_blocks(oracle_mod):
    """Results held at the same time never share a cached host block, and a
    released block is reused only after its result is gone."""
    import gc
    from brmerge_gb300 import _native
    A = brm.gen_rmat(12, int(2.35 * 4096), seed=21)
    B = brm.gen_lognormal(4096, 4096, seed=22)
    R1, R2 = oracle_mod.precise(A, A), oracle_mod.precise(A, B)
    held = [brm.brmerge_precise(A, A), brm.brmerge_precise(A, B), brm.brmerge_precise(A, A)]
    ptrs = {a.ctypes.data for C in held for a in (C.rpt, C.col, C.val)}
    assert len(ptrs) == 9
    assert_same_csr(held[0], R1, "held 0")
    assert_same_csr(held[1], R2, "held 1")
    assert_same_csr(held[2], R1, "held 2")
    view = held[1].val[5:50]  # a slice keeps its block alive
    expect = view.copy()
    del held
    gc.collect()
    again = [brm.brmerge_precise(A, B) for _ in range(2)]
    assert np.array_equal(view, expect)
    for C in again:
        assert_same_csr(C, R2, "after release")
    del again, view
    gc.collect()
    _native.lib().brm_host_cache_release()
    assert_same_csr(brm.brmerge_precise(A, A), R1, "after cache release")


# ---------------------------------------------------------------------------
# edge cases
# ---------------------------------------------------------------------------

def _csr(rows, ncols, seed=0):
    rng = np.random.default_rng(seed)
    rpt = np.zeros(len(rows) + 1, np.int32)
    for i, r in enumerate(rows):
        rpt[i + 1] = rpt[i] + len(r)
    col = np.array([c for r in rows for c in sorted(r)], np.int32)
    return brm.CSR(len(rows), ncols, rpt, col, rng.uniform(-1, 1, len(col)))


def test_empty_matrices(ctx, oracle_mod):
    A = _csr([[], [], []], 4)
    B = _csr([[0], [], [1, 2], []], 5)
    for C in (brm.brmerge_precise(A, B), gpu_precise(ctx, A, B), gpu_upper(ctx, A, B)):
        assert C.M == 3 and C.N == 5 and list(C.rpt) == [0, 0, 0, 0] and len(C.col) == 0
    A2 = _csr([[0, 1], [1, 3]], 4)
    B2 = _csr([[], [], [], []], 7)
    C2 = gpu_precise(ctx, A2, B2)
    assert list(C2.rpt) == [0, 0, 0]


def test_single_and_pass_through_lists(ctx, oracle_mod):
    # rows with exactly one nonempty list among many empty ones (copy rows),
    # odd list counts, and exact cancellation kept as an explicit zero
    Brows = [[], [0, 2, 4], [], [1, 2], [2], [], [0, 1, 2, 3, 4]]
    B = _csr(Brows, 5, 1)
    Arows = [[0, 1, 2], [1], [0, 2, 5], [1, 3, 4], [0, 1, 3, 4, 6], [3, 4], [6], []]
    A = _csr(Arows, 7, 2)
    B.val[B.rpt[3] + 1] = 0.25   # B(3,2)
    B.val[B.rpt[4]] = 0.25       # B(4,2)
    A.val[A.rpt[5]] = 1.0        # A(5,3)
    A.val[A.rpt[5] + 1] = -1.0   # A(5,4)
    R = oracle_mod.precise(A, B)
    assert_same_csr(gpu_precise(ctx, A, B), R, "edge")
    assert_same_csr(gpu_upper(ctx, A, B), R, "edge upper")
    assert 0.0 in list(R.val)


def test_signed_zero_pass_through(ctx, oracle_mod):
    A = _csr([[0, 1]], 2)
    B = _csr([[0], [1]], 2)
    A.val[:] = [1.0, 1.0]
    B.val[:] = [-0.0, 0.5]
    C = gpu_precise(ctx, A, B)
    assert np.signbit(C.val[0]) and C.val[0] == 0.0
    assert_same_csr(C, oracle_mod.precise(A, B), "-0")


def test_long_rows_many_windows(ctx, oracle_mod):
    # a few very long rows: many lists, thousands of products per row, many
    # shared columns (windows cut inside one chunk)
    rng = np.random.default_rng(21)
    K, N = 3000, 20000
    Brows = [sorted(rng.choice(N, rng.integers(5, 120), replace=False)) for _ in range(K)]
    Arows = [sorted(rng.choice(K, k, replace=False)) for k in (2500, 1800, 900, 64, 7)]
    A, B = _csr(Arows, K, 3), _csr(Brows, N, 4)
    R = oracle_mod.precise(A, B)
    assert_same_csr(gpu_precise(ctx, A, B), R, "long rows")
    assert_same_csr(gpu_upper(ctx, A, B), R, "long rows upper")


def test_spill_many_lists(ctx, oracle_mod):
    # an A row with more lists than the shared-memory list table holds
    rng = np.random.default_rng(22)
    K, N = 6000, 5000
    Brows = [sorted(rng.choice(N, rng.integers(0, 6), replace=False)) for _ in range(K)]
    Arows = [list(range(0, K, 1)), list(range(0, K, 3)), [5, 9]]
    A, B = _csr(Arows, K, 5), _csr(Brows, N, 6)
    R = oracle_mod.precise(A, B)
    assert_same_csr(gpu_precise(ctx, A, B), R, "spill lists")
    assert_same_csr(gpu_upper(ctx, A, B), R, "spill lists upper")


def test_spill_dense_word(ctx, oracle_mod):
    # more products inside one 32-column word than a window holds
    K, N = 400, 64
    Brows = [list(range(32)) for _ in range(K)]
    Arows = [list(range(K)), list(range(0, K, 2)), [3]]
    A, B = _csr(Arows, K, 7), _csr(Brows, N, 8)
    R = oracle_mod.precise(A, B)
    assert_same_csr(gpu_precise(ctx, A, B), R, "dense word")
    assert_same_csr(gpu_upper(ctx, A, B), R, "dense word upper")


def test_spill_dense_column(ctx, oracle_mod):
    # one column shared by more lists than a column segment holds (the
    # global-memory spill path), next to ordinary segmented rows
    rng = np.random.default_rng(23)
    K, N = 4000, 3000
    Brows = [sorted(set([7] + list(rng.choice(N, rng.integers(0, 5), replace=False))))
             for _ in range(K)]
    Arows = [list(range(K)), list(range(0, K, 7)), [1, 2, 3]]
    A, B = _csr(Arows, K, 9), _csr(Brows, N, 10)
    R = oracle_mod.precise(A, B)
    assert_same_csr(gpu_precise(ctx, A, B), R, "dense column")
    assert_same_csr(gpu_upper(ctx, A, B), R, "dense column upper")


def test_invalid_input_rejected():
    A = _csr([[0, 1], [2], [1]], 3)
    bad = A.copy()
    bad.col[0], bad.col[1] = bad.col[1], bad.col[0]  # unsorted row
    with pytest.raises(brm.BrmError) as ei:
        brm.brmerge_precise(bad, A.copy())
    assert ei.value.status == 2
    oob = A.copy()
    oob.col[2] = 7  # column out of range
    with pytest.raises(brm.BrmError) as ei:
        brm.brmerge_precise(A, oob)
    assert ei.value.status == 2
    with pytest.raises(ValueError):
        brm.brmerge_precise(A, _csr([[0]], 1))  # A.N != B.M


def test_device_validate(ctx):
    A = _csr([[0, 1], [2], []], 3)
    assert ctx.validate(dev(A)) == -1
    bad = A.copy()
    bad.col[1] = 0
    assert ctx.validate(dev(bad)) == 0


def test_numeric_requires_plan(ctx):
    A = brm.gen_er(256, 4, seed=1)
    dA = dev(A)
    crpt, n = ctx.symbolic(dA, dA)
    other = dev(brm.gen_er(256, 4, seed=2))
    with pytest.raises(brm.BrmError) as ei:
        ctx.numeric(other, other, crpt, n)
    assert ei.value.status == 6


def test_compute_flop_and_bound(ctx, oracle_mod):
    A = brm.gen_rmat(12, int(2.35 * 4096), seed=4)
    dA = dev(A)
    f = ctx.compute_flop(dA, dA)
    assert f == oracle_mod.compute_flop(A, A) == brm.compute_flop_host(A, A)
    p, nbytes = ctx.upper_bound(dA, dA)
    assert p == f and nbytes >= 24 * f


# ---------------------------------------------------------------------------
# full-size configurations
# ---------------------------------------------------------------------------

def test_er_config_full(ctx, oracle_mod):
    """ER n=16384, exactly 8 per row, seed 0 (the CPU configuration)."""
    A = brm.gen_er(16384, 8, seed=0)
    assert_same_csr(gpu_precise(ctx, A, A), oracle_mod.precise(A, A), "er16384")


def test_rmat_config_full(ctx, oracle_mod):
    """Power-law R-MAT n=2^18, ~600k nnz, Precise and Upper, bit-exact."""
    A = brm.gen_rmat(18, int(2.35 * (1 << 18)), seed=0)
    R = oracle_mod.precise(A, A)
    assert_same_csr(gpu_precise(ctx, A, A), R, "rmat18 precise")
    assert_same_csr(gpu_precise_one_call(ctx, A, A), R, "rmat18 precise one call")
    assert_same_csr(gpu_upper(ctx, A, A), R, "rmat18 upper")


def test_stencil_config_full_properties(ctx, oracle_mod):
    """27-point stencil on 128^3: exact structure by closed form, values of
    sampled row blocks against the oracle (rows of C are independent)."""
    import torch
    n = 128
    A = brm.gen_stencil27(n)
    dA = dev(A)
    crpt, cnnz = ctx.symbolic(dA, dA)
    assert cnnz == (5 * n - 6) ** 3  # 634^3: every row reaches a 5x5x5 box clipped at faces
    C = ctx.numeric(dA, dA, crpt, cnnz)
    # row lengths: product over dimensions of the clipped box widths
    w = np.array([min(x + 2, n - 1) - max(x - 2, 0) + 1 for x in range(n)], np.int64)
    lens = (w[None, None, :] * w[None, :, None] * w[:, None, None]).reshape(-1)
    assert np.array_equal(np.diff(crpt.cpu().numpy().astype(np.int64)), lens)
    rpt = crpt.cpu().numpy()
    for r0 in (0, 70000, n ** 3 // 2, n ** 3 - 3000):
        rows = np.arange(r0, r0 + 3000)
        sub = brm.CSR(len(rows), A.N, np.concatenate([[0], np.cumsum(np.diff(A.rpt)[rows])]).astype(np.int32),
                      np.concatenate([A.col[A.rpt[i]:A.rpt[i + 1]] for i in rows]),
                      np.concatenate([A.val[A.rpt[i]:A.rpt[i + 1]] for i in rows]))
        R = oracle_mod.precise(sub, A)
        s, e = int(rpt[r0]), int(rpt[r0 + 3000])
        got = brm.CSR(len(rows), A.N, (rpt[r0:r0 + 3001] - rpt[r0]).astype(np.int32),
                      C.col[s:e].cpu().numpy(), C.val[s:e].cpu().numpy())
        assert_same_csr(got, R, f"stencil rows {r0}")
    torch.cuda.synchronize()


def test_repeat_calls_identical(ctx):
    A = brm.gen_rmat(15, int(2.35 * 32768), seed=9)
    dA = dev(A)
    C1 = ctx.precise(dA, dA).to_host()
    C2 = ctx.precise(dA, dA).to_host()
    assert_same_csr(C1, C2, "repeat")


# ---------------------------------------------------------------------------
# warp and four-warp mid rows: class boundaries and fallbacks
# ---------------------------------------------------------------------------

def _rows_with_products(rng, targets, K, N, blen_lo=1, blen_hi=6, span=None):
    """B with K rows of blen_lo..blen_hi columns (within [0, span) when given)
    and one A row per target product count (A rows pick B rows greedily,
    longest first, so the short rows fill the remainder exactly)."""
    span = N if span is None else span
    blens = rng.integers(blen_lo, blen_hi + 1, K)
    Brows = [sorted(rng.choice(span, int(b), replace=False)) for b in blens]
    Arows = []
    for t in targets:
        order = rng.permutation(K)
        order = order[np.argsort(-blens[order], kind="stable")]
        row, f = [], 0
        for b in order:
            if f + blens[b] <= t:
                row.append(int(b))
                f += int(blens[b])
            if f == t:
                break
        Arows.append(sorted(row))
    return _csr(Arows, K, 1), _csr(Brows, N, 2)


def test_mid_row_class_boundaries(ctx, oracle_mod):
    """Rows on either side of every class boundary: 33, 64 / 65 and 128 / 129
    (half-warp tiles), 768 / 769 (warp), 3072 / 3073 (four-warp groups) and
    5888 / 5889 (longer four-warp groups, then segmented)."""
    rng = np.random.default_rng(41)
    A, B = _rows_with_products(rng, [33, 64, 65, 128, 129, 767, 768, 769, 1500, 3071, 3072, 3073,
                                     5000, 5888, 5889],
                               K=3000, N=20000, blen_lo=1, blen_hi=30)
    R = oracle_mod.precise(A, B)
    assert_same_csr(gpu_precise(ctx, A, B), R, "boundaries split")
    assert_same_csr(gpu_precise_one_call(ctx, A, B), R, "boundaries one call")
    assert_same_csr(gpu_upper(ctx, A, B), R, "boundaries upper")


def test_mid_rows_long_groups(ctx, oracle_mod):
    """Rows around the long four-warp group limit (5888 / 5889 products) and
    longer rows of at most 255 lists (segmented), built from long B rows."""
    rng = np.random.default_rng(44)
    A, B = _rows_with_products(rng, [5888, 5889, 8000, 11776, 11777], K=3000, N=20000,
                               blen_lo=40, blen_hi=60)
    assert np.diff(A.rpt).max() <= 255
    R = oracle_mod.precise(A, B)
    assert_same_csr(gpu_precise(ctx, A, B), R, "long groups split")
    assert_same_csr(gpu_precise_one_call(ctx, A, B), R, "long groups one call")
    assert_same_csr(gpu_upper(ctx, A, B), R, "long groups upper")


def test_mid_rows_wide_column_range(ctx, oracle_mod):
    """Mid-size rows whose columns span more than 2^19 .. 2^22 columns take
    the batched or segmented paths instead of the warp kernels."""
    rng = np.random.default_rng(42)
    N = 6_000_000
    A, B = _rows_with_products(rng, [100, 700, 2000, 3000, 5000, 7000], K=2000, N=N, blen_lo=1,
                               blen_hi=40)
    R = oracle_mod.precise(A, B)
    assert_same_csr(gpu_precise(ctx, A, B), R, "wide split")
    assert_same_csr(gpu_precise_one_call(ctx, A, B), R, "wide one call")
    assert_same_csr(gpu_upper(ctx, A, B), R, "wide upper")


@pytest.mark.parametrize("blen,ks", [
    # warp rows (at most 768 products) with 31, 32, 33 lists (register stack
    # of 6 or 7 levels) and 63, 64 lists; 65, 100 and 255 lists go to the
    # longer four-warp rows (stack of 9 levels)
    ((4, 8), (31, 32, 33, 63, 64, 65, 100, 255)),
    # four-warp rows (769 .. 3072 products) with 64 lists, and with 65 and 200
    # lists (longer four-warp rows)
    ((14, 20), (64, 65, 200)),
])
def test_mid_rows_list_counts(ctx, oracle_mod, blen, ks):
    """Mid rows around the list limits of the warp and four-warp classes, many
    repeated columns so that long runs are reduced."""
    rng = np.random.default_rng(43)
    K, N = 400, 60 * blen[1]
    Brows = [sorted(rng.choice(N, int(rng.integers(blen[0], blen[1] + 1)), replace=False))
             for _ in range(K)]
    Arows = [sorted(rng.choice(K, k, replace=False)) for k in ks]
    A, B = _csr(Arows, K, 3), _csr(Brows, N, 4)
    R = oracle_mod.precise(A, B)
    assert_same_csr(gpu_precise(ctx, A, B), R, "list counts")
    assert_same_csr(gpu_precise_one_call(ctx, A, B), R, "list counts one call")
    assert_same_csr(gpu_upper(ctx, A, B), R, "list counts upper")
    C32 = gpu_precise(ctx, A.astype(np.float32), B.astype(np.float32))
    assert_same_csr(C32, oracle_mod.precise(A.astype(np.float32), B.astype(np.float32)), "f32")


def test_heavy_segments_list_counts(ctx, oracle_mod):
    """Heavy-row segments done by four-warp groups: about 400 sub-lists per
    segment with long runs (stack of 13 levels), 200 lists (9 levels), and
    100 nonempty lists at leaves above 4900 of a 5000-entry row (17 levels);
    and segments of about 1000 short sub-lists, left to the segment kernel."""
    rng = np.random.default_rng(45)
    N = 400
    # B rows: 0..4999 empty, 5000..5599 long (30..60 columns), 5600..6999 short
    Brows = ([[] for _ in range(5000)]
             + [sorted(rng.choice(N, int(rng.integers(30, 61)), replace=False)) for _ in range(600)]
             + [sorted(rng.choice(N, int(rng.integers(1, 4)), replace=False)) for _ in range(1400)])
    K = len(Brows)
    longs, shorts = np.arange(5000, 5600), np.arange(5600, 7000)
    Arows = [sorted(rng.choice(longs, 400, replace=False)),
             sorted(rng.choice(shorts, 1000, replace=False)),
             sorted(list(rng.choice(5000, 4900, replace=False)) + list(rng.choice(longs, 100, replace=False))),
             sorted(rng.choice(longs, 200, replace=False)),
             [5000, 5001, 5600]]
    A, B = _csr(Arows, K, 11), _csr(Brows, N, 12)
    R = oracle_mod.precise(A, B)
    assert_same_csr(gpu_precise(ctx, A, B), R, "segment lists split")
    assert_same_csr(gpu_precise_one_call(ctx, A, B), R, "segment lists one call")
    assert_same_csr(gpu_upper(ctx, A, B), R, "segment lists upper")
    C32 = gpu_precise(ctx, A.astype(np.float32), B.astype(np.float32))
    assert_same_csr(C32, oracle_mod.precise(A.astype(np.float32), B.astype(np.float32)), "f32")


def test_empty_row_classes_are_not_launched(ctx, oracle_mod):
    """Kernels of row classes without rows are skipped: a product whose rows
    all have at most 64 products (one tile class) launches far fewer kernels
    than one with rows of every class, and both stay bit-exact."""
    from brmerge_gb300 import _native
    L = _native.lib()
    small = brm.gen_er(4096, 8, seed=5)
    mixed = brm.gen_rmat(13, 8 << 13, seed=6)
    counts = {}
    for name, A in (("small", small), ("mixed", mixed)):
        dA = brm.DeviceCSR.from_host(A)
        R = oracle_mod.precise(A, A)
        assert_same_csr(ctx.precise_device(dA, dA).to_host(), R, name)  # warm-up
        l0 = L.brm_kernel_launches()
        C = ctx.precise_device(dA, dA)
        counts[name] = L.brm_kernel_launches() - l0
        assert_same_csr(C.to_host(), R, name)
        assert_same_csr(ctx.upper(dA, dA).to_host(), R, name + " upper")
    assert counts["small"] + 8 <= counts["mixed"], counts
