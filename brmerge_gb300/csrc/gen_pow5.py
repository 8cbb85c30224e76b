"""Writes brm_pow5.h: 128-bit truncations of 5^q, q in [-342, 308].

Entry q holds T(q) = floor(5^q * 2^s) with s chosen so that
2^127 <= T(q) < 2^128 (for q >= 0 the top 128 bits of 5^q; for q < 0 the
top 128 bits of 2^b / 5^-q, rounded down).  Then 5^q = T(q) * 2^(f5(q) - 127)
up to the truncation, with f5(q) = floor(q * log2 5); the decimal-to-binary
conversion of brm_numparse.h (Eisel-Lemire: D. Lemire, "Number parsing at a
gigabyte per second", Software: Practice and Experience 51(8), 2021) needs
only these and floor(q * log2 10) = q + f5(q) = (217706 * q) >> 16, which
this script checks for every q of the table.

    python brmerge_gb300/csrc/gen_pow5.py
"""
from pathlib import Path

QMIN, QMAX = -342, 308


def table():
    rows = []
    for q in range(QMIN, QMAX + 1):
        if q >= 0:
            p = 5 ** q
            L = p.bit_length()
            t = p << (128 - L) if L <= 128 else p >> (L - 128)
            f5 = L - 1
        else:
            p = 5 ** (-q)
            L = p.bit_length()
            b = L + 127
            t = (1 << b) // p
            f5 = -L
        assert (1 << 127) <= t < (1 << 128), q
        # floor(q log2 10) = q + floor(q log2 5): the shift formula must agree
        assert (217706 * q) >> 16 == q + f5, q
        rows.append((q, t >> 64, t & ((1 << 64) - 1)))
    return rows


def main():
    out = Path(__file__).resolve().parent / "brm_pow5.h"
    lines = [
        "// brm_pow5.h -- generated by gen_pow5.py; do not edit.",
        "// 128-bit truncations of 5^q (normalised: top bit set), q in [-342, 308].",
        "#pragma once",
        "",
        "#include <cstdint>",
        "",
        "namespace brm {",
        f"constexpr int kPow5Min = {QMIN};",
        f"constexpr int kPow5Max = {QMAX};",
        f"constexpr int kPow5Rows = {QMAX - QMIN + 1};",
        "}  // namespace brm",
        "",
        "// The rows {high 64 bits, low 64 bits} of T(q), q = kPow5Min.. in order;",
        "// a translation unit instantiates them in host or device memory:",
        "//   const uint64_t table[brm::kPow5Rows][2] = {BRM_POW5_ROWS};",
        "#define BRM_POW5_ROWS \\",
    ]
    rows = table()
    for i, (q, hi, lo) in enumerate(rows):
        tail = "" if i == len(rows) - 1 else ", \\"
        lines.append(f"    {{0x{hi:016x}ull, 0x{lo:016x}ull}}{tail}")
    lines += [""]
    out.write_text("\n".join(lines))
    print(f"wrote {out}")


if __name__ == "__main__":
    main()
