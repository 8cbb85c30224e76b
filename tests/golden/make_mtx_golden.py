"""Generate the golden MatrixMarket fixtures from the reference's own reader.

Writes small MatrixMarket texts that cover the reader's formats (real,
integer, pattern, complex; general, symmetric, skew-symmetric; comments,
CRLF line ends, entries split across lines, surplus tokens, values that need
correct rounding) and reads each with the reference's CSR::construct
(BRMerge-SpGEMM/src/CSR.cpp:259-479, compiled unmodified into oracle/_ref by
oracle/build_ref.sh).  The texts and the reference's CSR (or the fact that it
threw) are stored in mtx_cases.npz; the restatement in oracle/mtx.py must
agree on every case before the fixture is written.  Needs the reference
sources; the fixture is committed.

    python tests/golden/make_mtx_golden.py
"""
from __future__ import annotations

import json
import sys
import tempfile
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT))

import oracle  # noqa: E402
from oracle import mtx  # noqa: E402

B = "%%MatrixMarket matrix coordinate"


def text_cases():
    rng = np.random.default_rng(21)
    # general real, unsorted entries, 17 significant digits, empty rows
    I = [3, 1, 6, 1, 2, 6, 4]
    J = [2, 5, 1, 1, 4, 5, 3]
    V = rng.uniform(-1, 1, len(I))
    body = "".join(f"{i} {j} {v:.17g}\n" for i, j, v in zip(I, J, V))
    yield "general_real", f"{B} real general\n% a comment\n%\n7 5 {len(I)}\n{body}"
    # symmetric with diagonal entries, comments, CRLF line ends
    ent = [(1, 1, 2.5), (3, 1, -1.25), (4, 2, 0.5), (4, 4, 1e-3), (5, 3, 7.0)]
    body = "".join(f"{i} {j} {v!r}\r\n" for i, j, v in ent)
    yield "symmetric_crlf", f"{B} real symmetric\r\n%c1\r\n%c2\r\n5 5 {len(ent)}\r\n{body}"
    # skew-symmetric (mirror negated), one signed zero
    ent = [(2, 1, 3.0), (4, 1, -0.0), (4, 3, 1.5), (5, 2, -2.25)]
    body = "".join(f"{i} {j} {v!r}\n" for i, j, v in ent)
    yield "skew", f"{B} real skew-symmetric\n5 5 {len(ent)}\n{body}"
    # pattern, rectangular
    ent = [(1, 7), (3, 1), (2, 2), (3, 6), (1, 1)]
    body = "".join(f"{i} {j}\n" for i, j in ent)
    yield "pattern_rect", f"{B} pattern general\n3 7 {len(ent)}\n{body}"
    # integer symmetric
    ent = [(1, 1, 4), (2, 1, -3), (3, 2, 12), (3, 3, 0)]
    body = "".join(f"{i} {j} {v}\n" for i, j, v in ent)
    yield "integer_symmetric", f"{B} integer symmetric\n3 3 {len(ent)}\n{body}"
    # complex: the real part is kept
    ent = [(1, 2, 1.5, -9.0), (2, 1, -0.25, 3.0), (2, 2, 8.0, 0.0)]
    body = "".join(f"{i} {j} {a!r} {b!r}\n" for i, j, a, b in ent)
    yield "complex", f"{B} complex general\n2 2 {len(ent)}\n{body}"
    # tokens split across lines, tabs and blanks, surplus tokens at the end
    yield "ragged_tokens", (f"{B} real general\n4 4 3\n1\t1  0.5 2\n 3 -1.5\n\n4 4\n  2.0e1 "
                            f"9 9 9\n")
    # value spellings that need a correctly rounded conversion
    vals = ["1e-300", "-0", "+.5", "5.", "1E+10", "123456789012345678901234567890",
            "4.9406564584124654e-324", "2.2250738585072011e-308", "0.1",
            "1.7976931348623157e308", "9007199254740993", "0.30000000000000004",
            "-1.0000000000000002", "3.141592653589793238462643383279", "1e22", "1e23",
            "8.98846567431158e307", "2.47032822920623272e-324", "00012.5000", "-.75e-2"]
    body = "".join(f"{k + 1} {k % 3 + 1} {v}\n" for k, v in enumerate(vals))
    yield "value_spellings", f"{B} real general\n{len(vals)} 3 {len(vals)}\n{body}"
    # larger random symmetric matrix (general spelling of its lower half)
    n = 300
    r = rng.integers(1, n + 1, 3000)
    c = rng.integers(1, n + 1, 3000)
    lo = np.unique(np.stack([np.maximum(r, c), np.minimum(r, c)], 1), axis=0)
    rng.shuffle(lo)
    v = rng.standard_normal(len(lo))
    body = "".join(f"{a} {b} {x:.16e}\n" for (a, b), x in zip(lo, v))
    yield "random_symmetric", f"{B} real symmetric\n{n} {n} {len(lo)}\n{body}"
    # larger random rectangular general matrix, %.6g values, rows out of order
    m, k = 200, 1000
    cells = rng.choice(m * k, 4000, replace=False)
    v = rng.uniform(-100, 100, len(cells))
    body = "".join(f"{q // k + 1} {q % k + 1} {x:.6g}\n" for q, x in zip(cells, v))
    yield "random_rect", f"{B} real general\n{m} {k} {len(cells)}\n{body}"
    # errors the reference reports by throwing
    yield "err_duplicate", f"{B} real general\n3 3 3\n1 1 1.0\n2 2 2.0\n1 1 3.0\n"
    yield "err_mirror_duplicate", f"{B} real symmetric\n3 3 2\n2 1 1.0\n1 2 2.0\n"
    yield "err_array", "%%MatrixMarket matrix array real general\n2 2\n1\n2\n3\n4\n"
    yield "err_hermitian", f"{B} complex hermitian\n2 2 1\n1 1 1.0 0.0\n"
    yield "err_banner", "%%MatrixMarket matrix coordinate real\n2 2 1\n1 1 1.0\n"
    yield "err_type", f"{B} double general\n2 2 1\n1 1 1.0\n"
    yield "err_size_line", f"{B} real general\n2 2\n1 1 1.0\n"


def main():
    oracle.build()
    if not oracle.ref_available():
        raise SystemExit("reference library unavailable; cannot generate fixtures")
    out = {}
    index = []
    with tempfile.TemporaryDirectory() as td:
        for name, text in text_cases():
            raw = text.encode()
            p = Path(td) / f"{name}.mtx"
            p.write_bytes(raw)
            try:
                R = oracle.ref_read_mtx(p)
                ref_err = None
            except ValueError as e:
                R, ref_err = None, str(e)
            try:
                O = mtx.parse(raw)
                o_err = None
            except mtx.MtxError as e:
                O, o_err = None, str(e)
            if (ref_err is None) != (o_err is None):
                raise SystemExit(f"{name}: reference error {ref_err!r}, restatement {o_err!r}")
            out[f"{name}__text"] = np.frombuffer(raw, np.uint8)
            if R is not None:
                assert (O.M, O.N) == (R.M, R.N), name
                assert np.array_equal(O.rpt, R.rpt) and np.array_equal(O.col, R.col), name
                assert np.array_equal(O.val.view(np.int64), R.val.view(np.int64)), name
                out[f"{name}__dims"] = np.array([R.M, R.N], np.int64)
                out[f"{name}__rpt"] = R.rpt
                out[f"{name}__col"] = R.col
                out[f"{name}__val"] = R.val
            index.append({"name": name, "error": ref_err})
            print(f"{name}: " + (f"reference throws: {ref_err}" if ref_err else
                                 f"M={R.M} N={R.N} nnz={len(R.col)}"))
    out["index"] = np.frombuffer(json.dumps(index).encode(), np.uint8)
    np.savez_compressed(HERE / "mtx_cases.npz", **out)


if __name__ == "__main__":
    main()
