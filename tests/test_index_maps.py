"""Index maps of the batched gradient update, restated on the CPU.

The compact-WY step of the gradient (G <- G + V Z'^T - Z' V^T on the rows i >= r0,
columns j < i, mirrored) deals (row strip, column block) items to warps.  Strip si
holds rows [n - 32(si+1), n - 32 si) restricted to i >= r0, and its column blocks of
32 cover the columns before its last row.  The test walks the same item numbering
as the kernel, for every block of 8 reflectors of many sizes. It checks that every
element (i, j) with r0 <= i < n and j < i is updated exactly once, and nothing else.
"""
import numpy as np
import pytest

GNB = 8


def g6_elements(n, r0):
    m = n - r0
    S = (m + 31) >> 5
    total = sum((n - 32 * si - 1 + 31) // 32 for si in range(S))
    hits = np.zeros((n, n), dtype=np.int32)
    for item in range(total):
        si, rem = 0, item
        while True:
            nbk = (n - 32 * si - 1 + 31) // 32
            if rem < nbk:
                break
            rem -= nbk
            si += 1
        jb = rem * 32
        je = min(jb + 32, n - 32 * si - 1)
        for lane in range(32):
            i = n - 32 * (si + 1) + lane
            if i < r0:
                continue
            for j in range(jb, je):
                if j >= i:
                    break
                hits[i, j] += 1
    return hits


@pytest.mark.parametrize("n", [3, 4, 9, 16, 31, 32, 33, 40, 64, 65, 97, 130, 170, 256])
def test_gradient_update_covers_each_element_once(n):
    nref = n - 2
    kend = nref
    while kend > 0:
        k0 = max(0, kend - GNB)
        r0 = k0 + 1
        hits = g6_elements(n, r0)
        want = np.zeros((n, n), dtype=np.int32)
        for i in range(r0, n):
            want[i, :i] = 1
        np.testing.assert_array_equal(hits, want, err_msg=f"n={n} r0={r0}")
        kend -= GNB
