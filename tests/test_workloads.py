"""CPU tests of the seeded workload generators: the sort-based dedup equals
numpy's unique, the R-MAT quadrant draw by comparisons equals the binary
search it replaced, and the graphs are symmetric CSRs the engine accepts."""
import numpy as np

from scs_gb300 import workloads as W


def test_sorted_unique_equals_numpy_unique():
    rng = np.random.default_rng(3)
    for size in (0, 1, 2, 17, 1000, 100000):
        a = rng.integers(-50, 50 if size < 1000 else 1 << 40, size=size, dtype=np.int64)
        assert np.array_equal(W._sorted_unique(a), np.unique(a))


def test_quadrant_by_comparisons_equals_searchsorted():
    rng = np.random.default_rng(4)
    cum = np.cumsum(np.array([0.57, 0.19, 0.19, 1.0 - 0.57 - 0.19 - 0.19]))
    x = rng.random(200000)
    x[:4] = [0.0, cum[0], cum[1], cum[2]]  # the bounds themselves
    want = np.minimum(np.searchsorted(cum, x, side="right"), 3)
    got = (x >= cum[0]).astype(np.int64) + (x >= cum[1]) + (x >= cum[2])
    assert np.array_equal(got, want)


def test_rmat_graph_is_a_symmetric_csr():
    n, u, v = W.rmat(10, 16 << 10)
    assert len(u) == 16 << 10
    assert np.all(u < v)  # canonical pairs: no self-loops
    keys = u.astype(np.int64) * (1 << 32) + v
    assert np.unique(keys).size == keys.size
    off, adj = W.to_csr(n, u, v)
    from scs_gb300 import engine as E
    core = E.core_numbers(n, off, adj)  # refused unless symmetric and ascending
    assert core.size == n
