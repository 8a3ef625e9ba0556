"""The parallel topology construction used by the CUDA kernel (k_topology in
bhut_gb300/csrc/build.cu), restated here in Python, against the reference's
LIFO-stack build (bhut/tree/build.py:110-212) as restated by the oracle.

Each BFS slot (depth d, index j) follows the path bits of j from the root;
the node id comes from the parent's internal-node rank k (children 2k+1,
2k+2); right children have rank k+1, left children k+1+I(right subtree).
"""
import numpy as np
import pytest


def closed_form(n, L):
    # host tables (make_topo_tables)
    depth = 0
    while -(-n // (1 << depth)) > L:
        depth += 1
    lo = [n >> d for d in range(depth + 2)]
    internal = [[0, 0] for _ in range(depth + 2)]
    for d in range(depth + 1, -1, -1):
        for v in range(2):
            c = lo[d] + v
            if c <= L:
                internal[d][v] = 0
                continue
            h, r = c // 2, c - c // 2
            internal[d][v] = 1 + internal[d + 1][h - lo[d + 1]] + internal[d + 1][r - lo[d + 1]]
    M = 1 + 2 * internal[0][0]
    fc = np.full(M, -2, np.int64)
    st = np.full(M, -2, np.int64)
    ct = np.full(M, -2, np.int64)
    for slot in range((2 << depth) - 1):
        d = (slot + 1).bit_length() - 1
        j = slot + 1 - (1 << d)
        c, s, k, node, ok = n, 0, 0, 0, True
        for t in range(d):
            if c <= L:
                ok = False
                break
            bit = (j >> (d - 1 - t)) & 1
            half, rc = c // 2, c - c // 2
            if bit == 0:
                node = 2 * k + 1
                k = k + 1 + internal[t + 1][rc - lo[t + 1]]
                c = half
            else:
                node = 2 * k + 2
                k = k + 1
                s += half
                c = rc
        if not ok:
            continue
        st[node], ct[node] = s, c
        fc[node] = -1 if c <= L else 2 * k + 1
    return fc, st, ct


@pytest.mark.parametrize("n,L", [(1, 1), (1, 32), (2, 1), (3, 1), (7, 2), (31, 32), (33, 32),
                                 (65, 32), (100, 4), (257, 8), (1000, 1), (1023, 16),
                                 (4097, 32), (10000, 32), (12345, 7), (65537, 64)])
def test_closed_form_matches_stack_build(oracle_mod, n, L):
    fc, cc, st, ct, il = oracle_mod.topology(n, L)
    gfc, gst, gct = closed_form(n, L)
    assert len(gfc) == len(fc)
    assert np.array_equal(gfc, fc)
    assert np.array_equal(gst, st)
    assert np.array_equal(gct, ct)
    assert np.array_equal(gfc == -1, il)
