"""The Morton sort on the device against std::sort with the reference's comparator.

BuildTree sorts keys with a comparator that ignores the index bits (src/tree.hpp:2269-2273,
2831), so for repeated keys the order is libstdc++'s. The device reproduces that order;
these inputs stress it: heavy repetition, presorted and reversed inputs, and organ-pipe
inputs that exhaust the introsort depth budget and take its heap-sort path.
"""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def finder(built):
    f = built.Finder(0)
    yield f
    f.close()


def _cases():
    rng = np.random.default_rng(7)
    out = []
    for n, nd in ((17, 3), (100, 5), (3000, 40), (20000, 200), (200000, 1500), (200000, 200000)):
        base = rng.integers(0, 2**32, size=(nd, 3), dtype=np.uint64).astype(np.uint32)
        out.append((f"rand{n}_{nd}", base[rng.integers(0, nd, size=n)]))
    k = out[3][1]
    out.append(("presorted", k[np.lexsort((k[:, 0], k[:, 1], k[:, 2]))]))
    out.append(("reversed", out[-1][1][::-1].copy()))
    for n in (4000, 100000):
        x = np.concatenate([np.arange(n // 2), np.arange(n // 2)[::-1]]).astype(np.uint32)
        out.append((f"organ{n}", np.stack([x, np.zeros_like(x), np.zeros_like(x)], 1)))
    return out


@pytest.mark.parametrize("name,keys", _cases(), ids=[c[0] for c in _cases()])
def test_morton_order_matches_std_sort(name, keys, finder):
    import oracle

    np.testing.assert_array_equal(finder.morton_order(keys), oracle.morton_order(keys))
