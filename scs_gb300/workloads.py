"""Seeded synthetic graphs and query sets for the SCS workloads.

The reference measures on SNAP graphs that are not shipped; seeded synthetic
graphs with the stated shapes stand in for them:

* ``chung_lu``  -- power-law expected degrees, endpoints drawn in proportion to
  weight, self-loops and duplicates dropped, topped up to exactly ``m`` edges.
* ``rmat``      -- recursive-matrix edges (a, b, c, d), ids permuted with the
  same seed, self-loops and duplicates dropped, topped up to exactly ``m``.

Edge lists use the reference's file format (src/Graph.h:5-67): a header line
``<n> <m>`` then one ``u<TAB>v`` line per undirected edge; ``m`` is the exact
deduplicated undirected edge count because the reference sizes its adjacency
array from the header.
"""
import os

import numpy as np

GRAPH_SEED = 1234
QUERY_SEED = 42


def _sorted_unique(a):
    """np.unique of an int64 array (ascending, no repeats) by one sort."""
    a = np.sort(a, kind="stable")
    keep = np.ones(a.size, dtype=bool)
    np.not_equal(a[1:], a[:-1], out=keep[1:])
    return a[keep]


def _dedup_pairs(u, v):
    """Canonical (min, max) pairs without self-loops, unique, as int64 keys."""
    keep = u != v
    u, v = u[keep], v[keep]
    lo = np.minimum(u, v).astype(np.int64)
    hi = np.maximum(u, v).astype(np.int64)
    return _sorted_unique(lo * (1 << 32) + hi)


def _top_up(sampler, m, rng, batch):
    """Draw batches of endpoint pairs until exactly m unique edges exist;
    edges are kept in first-drawn order so the result is prefix-stable."""
    keys = np.empty(0, dtype=np.int64)
    rounds = 0
    while keys.size < m:
        u, v = sampler(rng, batch)
        new = _dedup_pairs(u, v)
        # union of two ascending runs: the stable sort merges them
        keys = _sorted_unique(np.concatenate([keys, new])) if keys.size else new
        rounds += 1
        if rounds > 10000:
            raise RuntimeError("generator cannot reach the requested edge count")
    if keys.size > m:
        # drop a seeded random subset of the surplus to land on exactly m
        keep = rng.choice(keys.size, size=m, replace=False)
        keys = np.sort(keys[keep])
    return keys


def chung_lu(n, m, exponent, seed=GRAPH_SEED):
    """Undirected Chung-Lu graph with power-law weights w_i ~ (i+i0)^(-1/(g-1)),
    i0 chosen so the largest expected degree is sqrt(2m).  Returns (n, u, v)."""
    rng = np.random.default_rng(seed)
    alpha = 1.0 / (exponent - 1.0)
    target_max = np.sqrt(2.0 * m)
    mean = 2.0 * m / n
    idx = np.arange(n, dtype=np.float64)

    def shape(i0):
        w = (idx + i0) ** (-alpha)
        return w / w.mean() * mean

    lo, hi = 1e-3, float(n)
    for _ in range(200):  # bisection on i0: max weight decreases with i0
        mid = np.sqrt(lo * hi)
        if shape(mid)[0] > target_max:
            lo = mid
        else:
            hi = mid
    w = shape(hi)
    p = w / w.sum()
    cdf = np.cumsum(p)
    cdf[-1] = 1.0

    def sampler(r, batch):
        a = np.searchsorted(cdf, r.random(batch), side="right")
        b = np.searchsorted(cdf, r.random(batch), side="right")
        return np.minimum(a, n - 1), np.minimum(b, n - 1)

    keys = _top_up(sampler, m, rng, max(m // 2, 1024))
    return n, (keys >> 32).astype(np.uint32), (keys & 0xffffffff).astype(np.uint32)


def rmat(scale, m, a=0.57, b=0.19, c=0.19, seed=GRAPH_SEED):
    """Undirected R-MAT graph on 2^scale vertices with exactly m edges."""
    rng = np.random.default_rng(seed)
    n = 1 << scale
    perm = rng.permutation(n).astype(np.int64)
    probs = np.array([a, b, c, 1.0 - a - b - c])
    cum = np.cumsum(probs)

    def sampler(r, batch):
        u = np.zeros(batch, dtype=np.int64)
        v = np.zeros(batch, dtype=np.int64)
        for bit in range(scale):
            x = r.random(batch)
            # quadrant = number of cumulative bounds <= x, at most 3
            q = (x >= cum[0]).astype(np.int64) + (x >= cum[1]) + (x >= cum[2])
            u |= ((q >> 1) & 1).astype(np.int64) << bit
            v |= (q & 1).astype(np.int64) << bit
        return perm[u], perm[v]

    keys = _top_up(sampler, m, rng, max(m // 2, 1024))
    return n, (keys >> 32).astype(np.uint32), (keys & 0xffffffff).astype(np.uint32)


def write_edgelist(path, n, u, v):
    """Write the reference edge-list format (one line per undirected edge)."""
    os.makedirs(os.path.dirname(os.path.abspath(path)), exist_ok=True)
    arr = np.stack([u.astype(np.int64), v.astype(np.int64)], axis=1)
    with open(path, "w") as f:
        f.write("%d\t%d\n" % (n, len(u)))
        np.savetxt(f, arr, fmt="%d", delimiter="\t")
    return path


def to_csr(n, u, v):
    """Symmetric CSR with ascending neighbour lists (uint32)."""
    src = np.concatenate([u, v]).astype(np.int64)
    dst = np.concatenate([v, u]).astype(np.int64)
    order = np.lexsort((dst, src))
    src, dst = src[order], dst[order]
    off = np.zeros(n + 1, dtype=np.int64)
    np.add.at(off, src + 1, 1)
    off = np.cumsum(off)
    return off.astype(np.uint32), dst.astype(np.uint32)


# ---------------------------------------------------------------------------
# query sets: rows of (l, h, q, heuristic_flag, limit_dominating_set), the
# message fields of the reference server (main.cu:92-119)
# ---------------------------------------------------------------------------

def queries_small(core, count=50, seed=QUERY_SEED):
    """Plain method, small: q uniform over core >= 5, l = 3, h ~ U[5, 15]."""
    rng = np.random.default_rng(seed)
    cand = np.flatnonzero(core >= 5)
    q = rng.choice(cand, size=count)
    h = rng.integers(5, 16, size=count)
    l = np.full(count, 3)
    return np.stack([l, h, q, np.ones(count, int), np.full(count, 10)], 1).astype(np.uint32)


def queries_mid(core, count=1000, seed=QUERY_SEED):
    """Plain GPU method, mid size: q over core >= 8, l ~ U[3, 10],
    h = l + U[5, 30], heuristic on, dominating limit 10."""
    rng = np.random.default_rng(seed)
    cand = np.flatnonzero(core >= 8)
    q = rng.choice(cand, size=count)
    l = rng.integers(3, 11, size=count)
    h = l + rng.integers(5, 31, size=count)
    return np.stack([l, h, q, np.ones(count, int), np.full(count, 10)], 1).astype(np.uint32)


def queries_uneven(core, count=10000, seed=QUERY_SEED):
    """Uneven sizes: h log-uniform in [10, 100], l ~ U[3, h/2], q over
    core >= 10."""
    rng = np.random.default_rng(seed)
    cand = np.flatnonzero(core >= 10)
    q = rng.choice(cand, size=count)
    h = np.floor(np.exp(rng.uniform(np.log(10), np.log(100.999), size=count))).astype(int)
    l = np.array([rng.integers(3, max(3, hh // 2) + 1) for hh in h])
    return np.stack([l, h, q, np.ones(count, int), np.full(count, 10)], 1).astype(np.uint32)


def queries_serve(core, count=10000, seed=QUERY_SEED):
    """Serving: h ~ U[10, 200], l ~ U[3, h/2], q over core >= 12."""
    rng = np.random.default_rng(seed)
    cand = np.flatnonzero(core >= 12)
    q = rng.choice(cand, size=count)
    h = rng.integers(10, 201, size=count)
    l = np.array([rng.integers(3, max(3, hh // 2) + 1) for hh in h])
    return np.stack([l, h, q, np.ones(count, int), np.full(count, 10)], 1).astype(np.uint32)


WORKLOADS = {
    # name: (graph builder, query builder)
    "chunglu_n4000": (lambda: chung_lu(4000, 88000, 2.5), queries_small),
    "rmat_s15_ef16": (lambda: rmat(15, 16 << 15), queries_mid),
    "chunglu_n1m": (lambda: chung_lu(1000000, 20000000, 2.3), queries_uneven),
    "rmat_s22_ef16": (lambda: rmat(22, 16 << 22), queries_serve),
}
