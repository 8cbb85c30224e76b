"""MatrixMarket reader: the oracle against the reference's own reader
(golden fixtures), the token conversion against an exact one (CPU), and the
device reader against both (GPU).

The reference reads with CSR::construct (BRMerge-SpGEMM/src/CSR.cpp:259-479);
tests/golden/mtx_cases.npz holds its output on each case text
(tests/golden/make_mtx_golden.py).
"""
from __future__ import annotations

import ctypes as C
import json

import numpy as np
import pytest

from conftest import GOLDEN, assert_same_csr

from oracle import mtx as omtx


def golden_cases():
    z = np.load(GOLDEN / "mtx_cases.npz")
    index = json.loads(bytes(z["index"]).decode())
    out = []
    for ent in index:
        name = ent["name"]
        text = bytes(z[f"{name}__text"])
        exp = None
        if ent["error"] is None:
            M, N = (int(x) for x in z[f"{name}__dims"])
            exp = (M, N, z[f"{name}__rpt"], z[f"{name}__col"], z[f"{name}__val"])
        out.append((name, text, exp))
    return out


CASES = golden_cases()
CASE_IDS = [c[0] for c in CASES]


def _csr(M, N, rpt, col, val):
    from types import SimpleNamespace
    return SimpleNamespace(M=M, N=N, rpt=rpt, col=col, val=val)


B = "%%MatrixMarket matrix coordinate"
# inputs the reference mishandles (undefined behaviour or a silently wrong
# matrix): the oracle and the library reject them
EXTRA_ERRORS = {
    "row_out_of_range": f"{B} real general\n3 3 2\n1 1 1.0\n4 1 2.0\n",
    "row_zero": f"{B} real general\n3 3 1\n0 1 1.0\n",
    "col_out_of_range": f"{B} real general\n3 3 2\n1 1 1.0\n2 4 2.0\n",
    "fewer_entries": f"{B} real general\n3 3 3\n1 1 1.0\n2 2 2.0\n",
    "bad_int_token": f"{B} real general\n3 3 1\n1.0 1 1.0\n",
    "bad_real_token": f"{B} real general\n3 3 1\n1 1 1.0x\n",
    "nan_token": f"{B} real general\n3 3 1\n1 1 nan\n",
    "hex_token": f"{B} real general\n3 3 1\n1 1 0x1p3\n",
    "overflow": f"{B} real general\n3 3 1\n1 1 1e400\n",
    "bad_imag": f"{B} complex general\n3 3 1\n1 1 1.0 i\n",
    "nnz_zero": f"{B} real general\n3 3 0\n",
    "mirror_outside": f"{B} real symmetric\n2 5 1\n1 4 1.0\n",
    "blank_before_size": f"{B} real general\n%c\n\n3 3 1\n1 1 1.0\n",
    "int_overflow": f"{B} real general\n3 3 1\n4294967297 1 1.0\n",
}


# ---------------------------------------------------------------------------
# CPU: the oracle, pinned to the reference's reader
# ---------------------------------------------------------------------------

@pytest.mark.parametrize("name,text,exp", CASES, ids=CASE_IDS)
def test_oracle_matches_reference_reader(name, text, exp):
    if exp is None:
        with pytest.raises(omtx.MtxError):
            omtx.parse(text)
        return
    got = omtx.parse(text)
    assert (got.M, got.N) == exp[:2]
    assert_same_csr(got, _csr(*exp), name)


@pytest.mark.parametrize("name", sorted(EXTRA_ERRORS))
def test_oracle_rejects_malformed(name):
    with pytest.raises(omtx.MtxError):
        omtx.parse(EXTRA_ERRORS[name].encode())


def test_oracle_reads_with_reference_when_available(tmp_path):
    """Where the reference was compiled here, re-check a random file."""
    import oracle
    if not oracle.ref_available():
        pytest.skip("reference reader not built on this host")
    text = random_mtx_text(np.random.default_rng(5), 500, 400, 3000, "real", "general", "%.17g")
    p = tmp_path / "r.mtx"
    p.write_bytes(text)
    R = oracle.ref_read_mtx(p)
    assert_same_csr(omtx.parse(text), R, "random general")


# ---------------------------------------------------------------------------
# CPU: the token conversion (host build of the device parser)
# ---------------------------------------------------------------------------

def _host():
    from brmerge_gb300 import _native
    return _native.host()


def parse_tokens(tokens: list[bytes]):
    H = _host()
    buf = b"".join(tokens)
    lens = np.array([len(t) for t in tokens], np.int32)
    off = np.zeros(len(tokens), np.int64)
    off[1:] = np.cumsum(lens[:-1])
    out = np.zeros(len(tokens), np.float64)
    st = np.zeros(len(tokens), np.int32)
    cbuf = C.create_string_buffer(buf, len(buf) + 1)
    H.brm_parse_real_tokens(cbuf, off.ctypes.data, lens.ctypes.data, len(tokens),
                            out.ctypes.data, st.ctypes.data)
    return out, st


def random_real_tokens(rng, n: int) -> list[bytes]:
    """Spellings of doubles across the range: shortest round trip, 17 and
    16+ significant digits, few digits, huge and tiny exponents, long
    mantissas, near-halfway decimal expansions, subnormals."""
    toks = []
    bits = rng.integers(0, 0x7FF0000000000000, n // 4, dtype=np.int64)
    d = bits.view(np.float64)
    d = np.where(rng.random(len(d)) < 0.5, -d, d)
    toks += [repr(float(x)).encode() for x in d]
    toks += [(b"%.17g" % x) for x in d[: n // 8]]
    u = rng.uniform(-1e3, 1e3, n // 8)
    toks += [(b"%.16e" % x) for x in u]
    toks += [(b"%.6g" % x) for x in u]
    # near-halfway: the exact midpoint of two neighbours, rounded to 19..25 digits
    from decimal import Decimal, getcontext
    getcontext().prec = 800
    for x in rng.uniform(1e-5, 1e5, n // 16):
        a = float(x)
        b = np.nextafter(a, np.inf)
        mid = (Decimal(a) + Decimal(float(b))) / 2
        for p in (19, 20, 25):
            s = format(mid, f".{p}e").encode()
            toks.append(s)
    # exact midpoints (ties): small integers + 0.5 ulp, all digits
    for x in rng.integers(2 ** 53, 2 ** 54, n // 32, dtype=np.int64):
        if x % 2:
            toks.append(str(int(x)).encode())  # odd integer above 2^53: a tie
    # subnormals and extremes
    sub = rng.integers(1, 2 ** 52, n // 32, dtype=np.int64).view(np.float64)
    toks += [repr(float(x)).encode() for x in sub]
    toks += [b"1e-400", b"-1e-400", b"0e999999", b"1e308", b"1.7976931348623157e308",
             b"1.7976931348623158e308", b"2.2250738585072012e-308", b"9007199254740993",
             b"0.000000000000000000000000000000000000000001234567890123456789012345",
             b"123456789012345678901234567890123456789e-20", b"-0.0", b"+0", b".5", b"5."]
    return toks


def test_real_token_conversion_is_correctly_rounded():
    rng = np.random.default_rng(2024)
    toks = random_real_tokens(rng, 200_000)
    out, st = parse_tokens(toks)
    assert not np.any(st == -1), [toks[i] for i in np.nonzero(st == -1)[0][:5]]
    ok = np.nonzero(st == 0)[0]
    ref = np.array([float(t) for t in toks])
    mism = ok[out[ok].view(np.int64) != ref[ok].view(np.int64)]
    assert len(mism) == 0, [(toks[i], out[i], ref[i]) for i in mism[:5]]
    # the device decides almost everything itself (deferred: ties, >19-digit
    # near-halfway spellings, subnormals, out-of-range exponents)
    typical = len(toks) // 2
    assert np.mean(st[:typical] == 1) < 0.01


def test_real_token_grammar():
    good = [b"1", b"-1", b"+1", b"1.", b".5", b"-.5e-3", b"1E5", b"1e+05", b"00012.5000",
            b"0", b"-0"]
    bad = [b"", b"+", b"-", b".", b"e5", b"1e", b"1e+", b"1.2.3", b"1e5.0", b"nan", b"inf",
           b"0x10", b"1,5", b"--1", b"1-", b" 1"]
    out, st = parse_tokens(good + bad)
    assert np.all(st[: len(good)] >= 0)
    assert np.all(st[len(good):] == -1)
    assert np.array_equal(out[: len(good)], np.array([float(t) for t in good]))
    assert np.signbit(out[good.index(b"-0")])


def test_int_token_grammar():
    H = _host()
    v = C.c_longlong()
    for t, exp in ((b"1", 1), (b"+7", 7), (b"-3", -3), (b"0001", 1), (b"2147483647", 2 ** 31 - 1),
                   (b"-2147483648", -2 ** 31)):
        assert H.brm_parse_int_token(t, len(t), C.byref(v)) == 0 and v.value == exp, t
    for t in (b"", b"+", b"1.0", b"1e3", b"2147483648", b"-2147483649", b"12a", b"0x1"):
        assert H.brm_parse_int_token(t, len(t), C.byref(v)) == -1, t


# ---------------------------------------------------------------------------
# GPU: the device reader
# ---------------------------------------------------------------------------

def random_mtx_text(rng, M, N, n, field, symmetry, fmt, newline="\n", shuffle=True) -> bytes:
    if symmetry == "general":
        cells = rng.choice(M * N, n, replace=False)
        I, J = cells // N + 1, cells % N + 1
    else:
        r = rng.integers(1, M + 1, 2 * n)
        c = rng.integers(1, M + 1, 2 * n)
        keep = r > c if symmetry == "skew-symmetric" else r >= c
        lo = np.unique(np.stack([r[keep], c[keep]], 1), axis=0)[:n]
        if shuffle:
            rng.shuffle(lo)
        I, J = lo[:, 0], lo[:, 1]
    V = rng.standard_normal(len(I)) * 10.0 ** rng.integers(-5, 6, len(I))
    lines = [f"{B} {field} {symmetry}", "% generated", f"{M} {N} {len(I)}"]
    for i in range(len(I)):
        if field == "pattern":
            lines.append(f"{I[i]} {J[i]}")
        elif field == "integer":
            lines.append(f"{I[i]} {J[i]} {int(V[i] * 100)}")
        elif field == "complex":
            lines.append(f"{I[i]} {J[i]} {fmt % V[i]} {fmt % -V[i]}")
        else:
            lines.append(f"{I[i]} {J[i]} {fmt % V[i]}")
    return (newline.join(lines) + newline).encode()


@pytest.fixture(scope="module")
def gctx():
    import brmerge_gb300 as brm
    c = brm.Context()
    yield c
    c.close()


def _host_read(path, dtype=np.float64):
    import brmerge_gb300 as brm
    return brm.read_mtx(path, dtype=dtype)


def _dev_read(ctx, path, dtype=np.float64):
    X = ctx.read_mtx_device(path, dtype=dtype)
    return X.to_host()


@pytest.mark.gpu
@pytest.mark.parametrize("name,text,exp", CASES, ids=CASE_IDS)
def test_device_reader_matches_reference_reader(tmp_path, gctx, name, text, exp):
    import brmerge_gb300 as brm
    p = tmp_path / f"{name}.mtx"
    p.write_bytes(text)
    if exp is None:
        with pytest.raises(brm.BrmError) as ei:
            _host_read(p)
        assert ei.value.status == 11
        with pytest.raises(brm.BrmError):
            _dev_read(gctx, p)
        return
    R = _csr(*exp)
    for got in (_host_read(p), _dev_read(gctx, p)):
        assert (got.M, got.N) == exp[:2]
        assert_same_csr(got, R, name)
    g32 = _host_read(p, np.float32)
    with np.errstate(over="ignore"):  # 1.8e308 rounds to float32 infinity
        v32 = exp[4].astype(np.float32)
    assert_same_csr(g32, _csr(exp[0], exp[1], exp[2], exp[3], v32), name + " f32")


@pytest.mark.gpu
@pytest.mark.parametrize("name", sorted(EXTRA_ERRORS))
def test_device_reader_rejects_malformed(tmp_path, name):
    import brmerge_gb300 as brm
    p = tmp_path / f"{name}.mtx"
    p.write_text(EXTRA_ERRORS[name])
    with pytest.raises(brm.BrmError) as ei:
        _host_read(p)
    assert ei.value.status == 11, name


@pytest.mark.gpu
def test_device_reader_missing_file(tmp_path):
    import brmerge_gb300 as brm
    with pytest.raises(brm.BrmError) as ei:
        _host_read(tmp_path / "absent.mtx")
    assert ei.value.status == 12


KINDS = [
    ("real", "general", "%.17g", "\n"),
    ("real", "general", "%.16e", "\r\n"),
    ("real", "symmetric", "%.6g", "\n"),
    ("real", "skew-symmetric", "%.17g", "\n"),
    ("integer", "general", "", "\n"),
    ("pattern", "symmetric", "", "\n"),
    ("complex", "general", "%.12e", "\n"),
]


@pytest.mark.gpu
@pytest.mark.parametrize("kind", KINDS, ids=["-".join(k[:2]) + k[2] for k in KINDS])
def test_device_reader_random_files(tmp_path, gctx, kind):
    field, sym, fmt, nl = kind
    rng = np.random.default_rng(hash(kind) % 2 ** 32)
    M = 3000 if sym != "general" else 2500
    N = M if sym != "general" else 4000
    text = random_mtx_text(rng, M, N, 120_000, field, sym, fmt or "%g", nl)
    p = tmp_path / "r.mtx"
    p.write_bytes(text)
    R = omtx.parse(text)
    assert_same_csr(_host_read(p), R, "host form")
    assert_same_csr(_dev_read(gctx, p), R, "device form")


@pytest.mark.gpu
def test_device_reader_large_body_many_blocks(tmp_path, gctx):
    """A body of tens of MB (many staging blocks and text blocks), tokens
    spread over irregular whitespace."""
    rng = np.random.default_rng(77)
    M, N, n = 200_000, 150_000, 1_500_000
    cells = rng.choice(M * N, n, replace=False)
    I, J = cells // N + 1, cells % N + 1
    V = rng.standard_normal(n)
    seps = np.array([" ", "  ", "\t", " \t "])
    sep = seps[rng.integers(0, 4, n)]
    body = "".join(f"{i}{s}{j}{s}{float(v)!r}\n" for i, j, v, s in zip(I, J, V, sep))
    text = f"{B} real general\n{M} {N} {n}\n{body}".encode()
    p = tmp_path / "big.mtx"
    p.write_bytes(text)
    R = omtx.parse(text)
    assert_same_csr(_dev_read(gctx, p), R, "large")


@pytest.mark.gpu
def test_read_then_multiply(tmp_path, gctx, oracle_mod):
    """The reader's CSR feeds the SpGEMM directly (C = A*A, bit-exact)."""
    import brmerge_gb300 as brm
    rng = np.random.default_rng(3)
    text = random_mtx_text(rng, 2000, 2000, 30_000, "real", "symmetric", "%.17g")
    p = tmp_path / "a.mtx"
    p.write_bytes(text)
    dA = gctx.read_mtx_device(p)
    C = gctx.precise_device(dA, dA).to_host()
    A = brm.read_mtx(p)
    R = oracle_mod.precise(A, A)
    assert_same_csr(C, R, "read then multiply")
