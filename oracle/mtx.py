"""MatrixMarket reader restated on the CPU -- TEST INFRASTRUCTURE ONLY.

Restates the reference's CSR::construct (BRMerge-SpGEMM/src/CSR.cpp:259-479)
with numpy, as the checker of the library's device reader.  Only tests/ and
the golden-fixture script use it.

Semantics, step by step:

* banner (CSR.cpp:42-79): the first line splits on " \\t\\r\\n" into exactly
  five tokens ``%%MatrixMarket matrix coordinate <type> <symmetry>``; type is
  real, integer, pattern or complex, symmetry general, symmetric or
  skew-symmetric ("array" storage, "vector" and "hermitian" are rejected);
* comments (CSR.cpp:272-276): following lines are skipped while they start
  with '%'; the next line must hold exactly three tokens M N nnz, nnz > 0
  (CSR.cpp:279-288; the reference asserts nnz > 0);
* entries (CSR.cpp:297-335): the rest of the file is read as a stream of
  whitespace-separated tokens, F per entry (2 pattern, 3 real/integer, 4
  complex), ignoring line breaks; tokens after nnz entries are ignored;
  pattern values are 1, complex values their real part;
* 1-based to 0-based (CSR.cpp:355-358); symmetric formats (CSR.cpp:361-420):
  every entry followed by its mirror when off the diagonal, the mirror's
  value negated for skew-symmetric;
* sort by (row, column) and build the row pointers (CSR.cpp:426-450); the
  rows must then hold strictly ascending columns (CSR.cpp:454-477), so a
  repeated (row, column) is an error.

Where the reference's behaviour on malformed input is undefined or silently
wrong, this restatement (and the library) reports an error instead: fewer
entries than declared (the reference counts a failed extraction as read,
CSR.cpp:297-303), a token that is not a complete number (the reference's
stream extraction stops inside it), a row index outside [1, M] (the
reference writes outside its row-pointer array, CSR.cpp:442-444) and a
column index outside [1, N] (the reference's key N*I+J moves it to another
row), a value that overflows a double (the reference's extraction fails).
"""
from __future__ import annotations

import math
import re
from types import SimpleNamespace

import numpy as np


class MtxError(ValueError):
    """The file is not a MatrixMarket coordinate matrix this reader accepts."""


_INT = re.compile(rb"[+-]?[0-9]+\Z")
_REAL = re.compile(rb"[+-]?([0-9]+\.?[0-9]*|\.[0-9]+)([eE][+-]?[0-9]+)?\Z")
_FIELDS = {b"pattern": 2, b"real": 3, b"integer": 3, b"complex": 4}
_BANNER_WS = b" \t\r\n"  # tokenize() delimiters, CSR.cpp:22


def _split_banner(line: bytes) -> list[bytes]:
    return [t for t in re.split(rb"[ \t\r\n]+", line) if t]


def _int_tok(t: bytes) -> int:
    if not _INT.match(t):
        raise MtxError(f"invalid integer token {t[:32]!r}")
    v = int(t)
    if not -(2 ** 31) <= v < 2 ** 31:
        raise MtxError(f"integer token out of range {t[:32]!r}")
    return v


def _real_tok(t: bytes) -> float:
    if not _REAL.match(t):
        raise MtxError(f"invalid real token {t[:32]!r}")
    v = float(t)
    if math.isinf(v):
        # the reference's extraction fails on overflow (failbit)
        raise MtxError(f"real token overflows a double {t[:32]!r}")
    return v


def parse(text: bytes) -> SimpleNamespace:
    """Returns the reader's CSR (float64 values) or raises MtxError."""
    nl = text.find(b"\n")
    first = text if nl < 0 else text[:nl]
    tok = _split_banner(first)
    if len(tok) != 5 or tok[0] != b"%%MatrixMarket" or tok[1] != b"matrix":
        raise MtxError("invalid MatrixMarket banner")
    storage, typ, sym = tok[2], tok[3], tok[4]
    if storage != b"coordinate":
        raise MtxError("only coordinate storage is read")
    if typ not in _FIELDS:
        raise MtxError("invalid data type")
    if sym not in (b"general", b"symmetric", b"skew-symmetric"):
        raise MtxError("invalid or unsupported symmetry")
    pos = len(text) if nl < 0 else nl + 1
    # comment lines (CSR.cpp:272-276); the size line follows
    while True:
        if pos >= len(text):
            raise MtxError("missing size line")
        e = text.find(b"\n", pos)
        line = text[pos:] if e < 0 else text[pos:e]
        pos = len(text) if e < 0 else e + 1
        if not line.startswith(b"%"):
            break
    st = _split_banner(line)
    if len(st) != 3:
        raise MtxError("invalid size line")
    M, N, nnz = (_int_tok(t) for t in st)
    if M < 0 or N < 0 or nnz <= 0:
        raise MtxError("invalid sizes")
    F = _FIELDS[typ]
    body = text[pos:].split()  # C-locale whitespace, like operator>>
    if len(body) < nnz * F:
        raise MtxError("fewer entries than declared")
    body = body[: nnz * F]
    I = np.fromiter((_int_tok(t) for t in body[0::F]), np.int64, nnz) - 1
    J = np.fromiter((_int_tok(t) for t in body[1::F]), np.int64, nnz) - 1
    if F == 2:
        V = np.ones(nnz, np.float64)
    else:
        V = np.fromiter((_real_tok(t) for t in body[2::F]), np.float64, nnz)
        if F == 4:
            for t in body[3::F]:
                _real_tok(t)
    if nnz and (I.min() < 0 or I.max() >= M):
        raise MtxError("row index out of range")
    if nnz and (J.min() < 0 or J.max() >= N):
        raise MtxError("column index out of range")
    if sym != b"general":
        off = I != J
        # entry n, then its mirror (CSR.cpp:377-409): interleave
        k = np.cumsum(np.concatenate([[0], 1 + off[:-1].astype(np.int64)]))
        n2 = nnz + int(off.sum())
        I2 = np.empty(n2, np.int64)
        J2 = np.empty(n2, np.int64)
        V2 = np.empty(n2, np.float64)
        I2[k], J2[k], V2[k] = I, J, V
        km = k[off] + 1
        I2[km], J2[km] = J[off], I[off]
        V2[km] = -V[off] if sym == b"skew-symmetric" else V[off]
        I, J, V = I2, J2, V2
        if I.max() >= M or J.max() >= N:
            raise MtxError("a mirrored entry falls outside the matrix")
    order = np.lexsort((J, I))
    I, J, V = I[order], J[order], V[order]
    if len(I) > 1 and np.any((I[1:] == I[:-1]) & (J[1:] == J[:-1])):
        raise MtxError("repeated entry (columns not ascending)")
    if len(I) >= 2 ** 31:
        raise MtxError("too many entries for int32 CSR")
    rpt = np.zeros(M + 1, np.int64)
    np.add.at(rpt, I + 1, 1)
    rpt = np.cumsum(rpt).astype(np.int32)
    return SimpleNamespace(M=M, N=N, rpt=rpt, col=J.astype(np.int32), val=V)


def read(path) -> SimpleNamespace:
    with open(path, "rb") as f:
        return parse(f.read())


def write(path, M: int, N: int, I, J, V=None, field: str = "real", symmetry: str = "general",
          comments: tuple[str, ...] = (), fmt: str = "%.17g", newline: str = "\n") -> None:
    """Writes a coordinate file from 1-based I, J (test input generation)."""
    nl = newline
    with open(path, "w", newline="") as f:
        f.write(f"%%MatrixMarket matrix coordinate {field} {symmetry}{nl}")
        for c in comments:
            f.write(f"%{c}{nl}")
        f.write(f"{M} {N} {len(I)}{nl}")
        for n in range(len(I)):
            if field == "pattern":
                f.write(f"{I[n]} {J[n]}{nl}")
            elif field == "integer":
                f.write(f"{I[n]} {J[n]} {int(V[n])}{nl}")
            elif field == "complex":
                f.write(f"{I[n]} {J[n]} {fmt % V[n]} {fmt % (0.5 * V[n])}{nl}")
            else:
                f.write(f"{I[n]} {J[n]} {fmt % V[n]}{nl}")
