"""The oracle's two sort paths agree: the packed-key parallel merge sort it
uses from 2^20 nonzeros up (full-size parity of the device sorts) and the
comparison merge sort pinned to the reference's own sorts by the golden
fixtures.  Inputs with repeated coordinates, skewed and wide coordinates,
orders 2-8 (lexicographic, any mode order) and 3-4 (HiCOO order)."""
import numpy as np
import pytest

import oracle as O


def _inds(rng, ndims, n, zipf=False, dup=0.1):
    cols = []
    for d in ndims:
        if zipf:
            c = np.minimum(rng.zipf(1.3, n) - 1, d - 1)
        else:
            c = rng.integers(0, d, n)
        cols.append(c)
    a = np.stack(cols).astype(np.uint32)
    k = int(n * dup)
    if k:
        a[:, rng.integers(0, n, k)] = a[:, rng.integers(0, n, k)]   # repeated coordinates (ties)
    return a


@pytest.mark.parametrize("ndims", [[5, 7], [4_000_000, 2_000_000, 25_000], [10_000, 5_000, 2_000, 500],
                                   [2**32 - 1, 3, 2**31], [9, 8, 7, 6, 5, 4, 3, 2]])
def test_lex_keyed_matches_comparison_sort(ndims):
    rng = np.random.default_rng(len(ndims))
    a = _inds(rng, ndims, 50_000, zipf=len(ndims) == 3)
    N = len(ndims)
    for order in (list(range(N)), list(range(N))[::-1], [N - 1] + list(range(N - 1))):
        assert O.sort_keyed_check(a, order=order)


@pytest.mark.parametrize("ndims,sk", [([4_000_000, 2_000_000, 25_000], 17), ([300, 200, 100], 4),
                                      ([2**24 + 5, 70_000, 1_000], 7), ([10_000, 5_000, 2_000, 500], 9)])
def test_hicoo_keyed_matches_comparison_sort(ndims, sk):
    rng = np.random.default_rng(sk)
    a = _inds(rng, ndims, 50_000, zipf=True)
    assert O.sort_keyed_check(a, sk_bits=sk)
