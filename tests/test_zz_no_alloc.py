"""plan_morton_order_noalloc: the Morton sort with its keys and scratch in the library's fixed
device array (no allocation). Collected last; it must also pass on its own."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def finder(built):
    f = built.Finder(0)
    yield f
    f.close()


def _keys(n: int, distinct: int, seed: int) -> np.ndarray:
    rng = np.random.default_rng(seed)
    base = rng.integers(0, 2**32, size=(distinct, 3), dtype=np.uint64).astype(np.uint32)
    return base[rng.integers(0, distinct, size=n)]


@pytest.mark.parametrize("n,distinct", [(1, 1), (17, 3), (5000, 40), (65536, 900), (65536, 65536)])
def test_noalloc_matches_allocating_entry_point(n, distinct, finder):
    """Two calls in a row give the same order as plan_morton_order (the array is reused)."""
    keys = _keys(n, distinct, seed=n + distinct)
    want = finder.morton_order(keys)
    first = finder.morton_order_noalloc(keys)
    second = finder.morton_order_noalloc(keys)
    np.testing.assert_array_equal(first, want)
    np.testing.assert_array_equal(second, want)


def test_noalloc_after_other_input(finder):
    """A different input after a large one: no state is carried over in the array."""
    big = _keys(60000, 500, seed=1)
    finder.morton_order_noalloc(big)
    small = _keys(300, 7, seed=2)
    np.testing.assert_array_equal(finder.morton_order_noalloc(small), finder.morton_order(small))


def test_noalloc_rejects_more_than_the_limit(built, finder):
    keys = _keys(built.PLAN_NOALLOC_SORT_MAX + 1, 100, seed=3)
    with pytest.raises(built.PlanError) as e:
        finder.morton_order_noalloc(keys)
    assert e.value.status == 6
    assert "limit" in finder.error()
