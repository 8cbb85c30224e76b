"""The order-exact value semantics the GPU kernels rely on (CPU only).

BRMerge merges a row's k lists pairwise, adjacent pairs first, odd last list
passed through (BRMerge-SpGEMM/inc/spgemm.h:639-707).  The GPU kernels
evaluate each output column as a binary trie over the leaf index instead
(shift-reduce on the leaves in increasing order, ShiftReduce in
brm_common.cuh; level-synchronous sibling pairing in the warp kernel).  This
test restates both in Python and checks them bit-for-bit against the oracle.
"""
import numpy as np
import pytest

from brmerge_gb300.csr import CSR


def shift_reduce(leaves, vals):
    """Trie reduction over increasing leaves (mirror of ShiftReduce)."""
    st_v, st_op = [vals[0]], []
    last = leaves[0]
    for l, v in zip(leaves[1:], vals[1:]):
        s = (last ^ l).bit_length() - 1
        while len(st_v) >= 2 and st_op[-1] < s:
            b = st_v.pop()
            st_op.pop()
            st_v[-1] = np.float64(st_v[-1] + b)
        st_op.append(s)
        st_v.append(v)
        last = l
    while len(st_v) >= 2:
        b = st_v.pop()
        st_v[-1] = np.float64(st_v[-1] + b)
    return st_v[0]


def level_pairs(leaves, vals):
    """Level-synchronous sibling pairing (mirror of the warp kernel)."""
    nodes = list(zip(leaves, vals))
    while len(nodes) > 1:
        out, i = [], 0
        while i < len(nodes):
            n, v = nodes[i]
            if i + 1 < len(nodes) and n % 2 == 0 and nodes[i + 1][0] == n + 1:
                out.append((n >> 1, np.float64(v + nodes[i + 1][1])))
                i += 2
            else:
                out.append((n >> 1, v))
                i += 1
        nodes = out
    return nodes[0][1]


def aligned_ranges(leaves, vals):
    """Mirror of the long-column warp reducer (k_long_warp): the leaves are cut
    into the 32 aligned ranges of 2^s leaves (s = bits of the largest leaf - 5),
    each range is one subtree of the trie and is reduced on its own, and the
    range values are joined by the trie over the range indices."""
    s = max((leaves[-1] | 1).bit_length() - 5, 0)
    ranges = {}
    for l, v in zip(leaves, vals):
        ranges.setdefault(l >> s, []).append((l, v))
    idx = sorted(ranges)
    sub = [shift_reduce([x[0] for x in ranges[j]], [x[1] for x in ranges[j]]) for j in idx]
    return shift_reduce(idx, sub)


def trie_product(A, B, reducer):
    rows, cols, vals = [], [], []
    for i in range(A.M):
        contrib = {}
        for l, j in enumerate(range(A.rpt[i], A.rpt[i + 1])):
            b = A.col[j]
            for q in range(B.rpt[b], B.rpt[b + 1]):
                contrib.setdefault(int(B.col[q]), []).append((l, np.float64(A.val[j] * B.val[q])))
        for c in sorted(contrib):
            ls = contrib[c]
            rows.append(i)
            cols.append(c)
            vals.append(reducer([x[0] for x in ls], [x[1] for x in ls]))
    rpt = np.zeros(A.M + 1, np.int32)
    np.add.at(rpt, np.array(rows, np.int64) + 1, 1)
    return CSR(A.M, B.N, np.cumsum(rpt).astype(np.int32), np.array(cols, np.int32),
               np.array(vals, np.float64))


@pytest.mark.parametrize("reducer", [shift_reduce, level_pairs, aligned_ranges])
@pytest.mark.parametrize("seed", range(3))
def test_trie_forms_match_oracle(oracle_mod, reducer, seed):
    from brmerge_gb300 import gen_uniform
    from conftest import assert_same_csr
    A = gen_uniform(25, 40, 23, seed=seed)
    B = gen_uniform(40, 30, 12, seed=seed + 100)
    assert_same_csr(trie_product(A, B, reducer), oracle_mod.precise(A, B), reducer.__name__)


def test_trie_order_differs_from_sequential_sum():
    """The merge order is observable: a left-to-right sum differs in general."""
    rng = np.random.default_rng(0)
    diffs = 0
    for _ in range(200):
        v = rng.uniform(-1, 1, 7) * 10.0 ** rng.integers(-8, 8, 7)
        seq = np.float64(0)
        for x in v:
            seq = np.float64(seq + x)
        diffs += shift_reduce(list(range(7)), list(v)) != seq
    assert diffs > 0


@pytest.mark.parametrize("reducer", [shift_reduce, aligned_ranges])
@pytest.mark.parametrize("seed", range(2))
def test_trie_forms_wide_rows(oracle_mod, reducer, seed):
    """Rows of 200 lists: columns with many products at leaves up to 199, so
    the aligned ranges of the warp reducer span 8 leaves each."""
    from brmerge_gb300 import gen_uniform
    from conftest import assert_same_csr
    A = gen_uniform(6, 600, 200, seed=seed)
    B = gen_uniform(600, 40, 10, seed=seed + 100)
    assert_same_csr(trie_product(A, B, reducer), oracle_mod.precise(A, B), reducer.__name__)
