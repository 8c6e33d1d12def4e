"""Core numbers on the GPU (core.cu) against the host bin-sort peeling, which
the oracle pins against the reference's own loader (src/Graph.h:82-109).
Core numbers are unique, so the two must agree exactly."""
import numpy as np
import pytest

from scs_gb300 import build as B
from scs_gb300 import engine as E
from scs_gb300 import workloads as W


def _csr(n, edges):
    u = np.array([a for a, b in edges], dtype=np.int64)
    v = np.array([b for a, b in edges], dtype=np.int64)
    return W.to_csr(n, u, v)


def test_gpu_core_rejects_bad_csr_without_a_gpu():
    B.build()
    off = np.array([0, 2, 1], dtype=np.uint32)  # not monotone
    adj = np.array([1, 0], dtype=np.uint32)
    core = np.zeros(2, dtype=np.uint32)
    assert E.lib().scs_core_decompose_gpu(2, E._p(off), E._p(adj), E._p(core), 0) < 0
    off = np.array([0, 1, 2], dtype=np.uint32)
    adj = np.array([1, 5], dtype=np.uint32)  # neighbour id out of range
    assert E.lib().scs_core_decompose_gpu(2, E._p(off), E._p(adj), E._p(core), 0) < 0


def _shapes():
    yield "isolated", 5, []
    yield "single", 1, []
    yield "path", 6, [(i, i + 1) for i in range(5)]
    yield "star", 9, [(0, i) for i in range(1, 9)]
    yield "clique", 7, [(i, j) for i in range(7) for j in range(i + 1, 7)]
    yield "clique+tail", 9, [(i, j) for i in range(5) for j in range(i + 1, 5)] + [(4, 5), (5, 6)]
    rng = np.random.default_rng(11)
    for t in range(4):
        n = int(rng.integers(20, 300))
        m = int(rng.integers(n, 8 * n))
        e = set()
        while len(e) < m:
            a, b = (int(x) for x in rng.integers(0, n, size=2))
            if a != b:
                e.add((min(a, b), max(a, b)))
        yield "random%d" % t, n, sorted(e)


@pytest.mark.gpu
@pytest.mark.parametrize("name,n,edges", list(_shapes()), ids=[s[0] for s in _shapes()])
def test_gpu_core_matches_host_small(name, n, edges):
    off, adj = _csr(n, edges)
    assert np.array_equal(E.core_numbers_gpu(n, off, adj), E.core_numbers(n, off, adj))


@pytest.mark.gpu
@pytest.mark.parametrize("gen", ["chunglu_n4000", "rmat_s15_ef16"])
def test_gpu_core_matches_host_workloads(gen):
    make, _ = W.WORKLOADS[gen]
    n, u, v = make()
    off, adj = W.to_csr(n, u, v)
    host = E.core_numbers(n, off, adj)
    assert np.array_equal(E.core_numbers_gpu(n, off, adj), host)


@pytest.mark.gpu
def test_engine_core_numbers_come_from_gpu_and_match_host(rmat15):
    n, off, adj = E.read_edge_list(rmat15)
    eng = E.Engine(graph=rmat15, limit_queries=4)
    try:
        assert np.array_equal(eng.core_numbers(), E.core_numbers(n, off, adj))
    finally:
        eng.close()


@pytest.mark.parametrize("name,n,edges", list(_shapes()), ids=[s[0] for s in _shapes()])
def test_host_core_matches_oracle_small(name, n, edges, oracle_lib):
    """The host peeling (the GPU's reference above) equals the oracle's core
    numbers, which are pinned to the reference's own loader and peeling."""
    B.build()
    off, adj = _csr(n, edges)
    og = oracle_lib.OracleGraph(n, off, adj)
    assert np.array_equal(E.core_numbers(n, off, adj), np.asarray(og.core, dtype=np.uint32))


@pytest.mark.parametrize("gen", ["chunglu_n4000", "rmat_s15_ef16"])
def test_host_core_matches_oracle_workloads(gen, oracle_lib):
    B.build()
    make, _ = W.WORKLOADS[gen]
    n, u, v = make()
    off, adj = W.to_csr(n, u, v)
    og = oracle_lib.OracleGraph(n, off, adj)
    assert np.array_equal(E.core_numbers(n, off, adj), np.asarray(og.core, dtype=np.uint32))
