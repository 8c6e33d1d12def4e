"""CPU tests: the oracle pinned against the reference's own CPU code and
exhaustive search, and the engine's host code (loader, core numbers, greedy
incumbent, distance bound) against the oracle.  No GPU needed."""
import json
import os

import numpy as np
import pytest

from conftest import ROOT, random_graph

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _ref_dir():
    from oracle.build_ref import ref_dir
    return ref_dir()


def _golden_graph(name):
    from scs_gb300 import workloads as W
    gb, _ = W.WORKLOADS[name]
    n, u, v = gb()
    off, adj = W.to_csr(n, u, v)
    return n, off, adj


@pytest.mark.parametrize("name", ["chunglu_n4000", "rmat_s15_ef16"])
def test_oracle_heuristics_match_reference_golden(oracle_lib, name):
    """heu2/heu3/heu4/CSSC of the oracle equal the reference's own code's
    outputs recorded in tests/golden (inc/heuristic.h)."""
    import sys
    sys.path.insert(0, os.path.join(GOLD))
    from make_golden import graph_sum
    gold = json.load(open(os.path.join(GOLD, "heuristic_%s.json" % name)))
    n, off, adj = _golden_graph(name)
    assert graph_sum(off, adj) == gold["checksum"], "generator drift"
    g = oracle_lib.OracleGraph(n, off, adj)
    assert g.dmax == gold["dmax"]
    assert int(g.core.max()) == gold["core_max"]
    assert int(g.core.astype(np.int64).sum()) == gold["core_sum"]
    for rec in gold["queries"][:60]:
        for k in (2, 3, 4, 0):
            kl, H = g.heuristic(k, rec["l"], rec["h"], rec["q"])
            assert kl == rec["kl%d" % k], (rec["q"], k)
            assert H.tolist() == rec["H%d" % k], (rec["q"], k)


@pytest.mark.parametrize("name", ["chunglu_n4000", "rmat_s15_ef16"])
def test_engine_host_heuristic_matches_golden(name):
    """The engine's own host incumbent (libscs.so) equals the reference's."""
    from scs_gb300 import engine as E
    gold = json.load(open(os.path.join(GOLD, "heuristic_%s.json" % name)))
    n, off, adj = _golden_graph(name)
    core = E.core_numbers(n, off, adj)
    assert int(core.max()) == gold["core_max"]
    assert int(core.astype(np.int64).sum()) == gold["core_sum"]
    for rec in gold["queries"][:60]:
        kl, H = E.greedy_incumbent(n, off, adj, rec["l"], rec["h"], rec["q"])
        assert kl == rec["kl0"]
        assert H.tolist() == rec["H0"]


def test_engine_host_heuristic_matches_oracle_with_hubs(oracle_lib):
    """The engine's heu2/heu3 keep their counts and member lists up to date
    instead of rescanning neighbour rows; kl and H still equal the oracle's
    rescanning restatement, on random graphs of several densities and on an
    R-MAT graph with hubs under serving-size h (up to 200)."""
    from scs_gb300 import engine as E
    from scs_gb300 import workloads as W
    rng = np.random.default_rng(7)
    cases = [random_graph(rng, n, p) for n, p in ((30, .2), (60, .1), (120, .05), (200, .15))]
    n, u, v = W.rmat(12, 16 << 12, seed=5)
    cases.append((n,) + tuple(W.to_csr(n, u, v)))
    checked = 0
    for n, off, adj in cases:
        og = oracle_lib.OracleGraph(n, off, adj)
        deg = np.diff(off.astype(np.int64))
        cand = np.flatnonzero(deg > 0)
        for q in rng.choice(cand, size=min(40, cand.size), replace=False):
            h = int(rng.integers(3, min(200, n - 1) + 1))
            l = int(rng.integers(2, h + 1))
            kl, H = E.greedy_incumbent(n, off, adj, l, h, int(q))
            kl0, H0 = og.heuristic(0, l, h, int(q))
            assert (kl, H.tolist()) == (kl0, H0.tolist()), (n, int(q), l, h)
            checked += 1
    assert checked >= 150


def test_asymmetric_csr_is_rejected():
    """A CSR that lists an edge in only one of its rows is refused."""
    from scs_gb300 import engine as E
    off = np.array([0, 1, 1, 1], np.uint32)
    adj = np.array([1], np.uint32)
    with pytest.raises(E.SCSError):
        E.greedy_incumbent(3, off, adj, 1, 2, 0)
    with pytest.raises(E.SCSError):
        E.core_numbers(3, off, adj)


def test_distance_bound_forms_agree(oracle_lib):
    """Host ubD (main.cu:154-172), device ubD (src/helpers.cc:974-990, u32
    wrap for kl < 2) and the engine's host form agree everywhere used."""
    from scs_gb300 import engine as E
    L = oracle_lib.lib()
    for kl in range(0, 200):
        for h in range(1, 260):
            a = L.orc_ubd_host(kl, h)
            b = L.orc_ubd_dev(kl, h)
            assert a == b, (kl, h, a, b)
            if h % 7 == 0:
                assert E.distance_bound(kl, h) == a


def test_oracle_matches_bruteforce(oracle_lib):
    """The oracle's branch-and-bound is exact on small graphs, for every rule
    subset, with the heuristic off; with it on the answer is max(opt, kl)."""
    from scs_gb300 import workloads as W
    cases = json.load(open(os.path.join(GOLD, "bruteforce_small.json")))
    checked = 0
    for c in cases[:20]:
        off, adj = W.to_csr(c["n"], np.array(c["u"], np.uint32), np.array(c["v"], np.uint32))
        g = oracle_lib.OracleGraph(c["n"], off, adj)
        for qq in c["queries"]:
            for rules in (31, 1 | 8, 4 | 16, 2 | 8, 0):
                r, H = g.solve(qq["l"], qq["h"], qq["q"], 0, 10, rules)
                assert r.degree == qq["degree"], (qq, rules)
                checked += 1
            r, H = g.solve(qq["l"], qq["h"], qq["q"], 1, 10)
            assert r.degree == max(qq["degree"], r.kl_heu)
            if r.degree == qq["degree"] and r.degree > 0:
                from oracle import verify_community
                conn, hq, sz, md = verify_community(g, H, qq["q"], qq["l"], qq["h"])
                assert conn and hq and sz and md == r.degree
    assert checked > 1000


def test_oracle_random_bruteforce_fresh(oracle_lib):
    """Fresh random graphs (not the fixture): oracle == exhaustive search."""
    rng = np.random.default_rng(99)
    for _ in range(30):
        n, off, adj = random_graph(rng, int(rng.integers(6, 13)), float(rng.uniform(0.2, 0.7)))
        g = oracle_lib.OracleGraph(n, off, adj)
        for q in range(n):
            for (l, h) in ((1, 3), (3, 5), (2, 8)):
                assert g.solve(l, h, q, 0, 3)[0].degree == g.bruteforce(l, h, q)


def test_oracle_golden_answers_reproduce(oracle_lib, chunglu_small):
    """A few cheap config-1 answers recomputed from scratch."""
    gold = json.load(open(os.path.join(GOLD, "answers_chunglu_n4000.json")))
    g = oracle_lib.OracleGraph.from_file(chunglu_small)
    cheap = [q for q in gold["queries"] if q["finished"] and q["nodes"] < 3000][:6]
    assert cheap
    for qq in cheap:
        r, _ = g.solve(qq["l"], qq["h"], qq["q"], qq["heur"], qq["limit_doms"])
        assert r.degree == qq["degree"] and r.nodes == qq["nodes"]


def test_loader_semantics(tmp_path, oracle_lib):
    """Self-loops dropped, duplicates and reversed duplicates merged, rows
    ascending (src/Graph.h:5-67); engine and oracle loaders agree."""
    from scs_gb300 import engine as E
    p = tmp_path / "g.txt"
    p.write_text("6 7\n0\t1\n1\t0\n2 2\n3 1\n1 3\n4 5\n5 4\n0 3\n")
    n, off, adj = E.read_edge_list(str(p))
    g = oracle_lib.OracleGraph.from_file(str(p))
    assert n == g.n == 6
    assert off.tolist() == g.off.tolist() == [0, 2, 4, 4, 6, 7, 8]
    assert adj.tolist() == g.adj.tolist() == [1, 3, 0, 3, 0, 1, 5, 4]


def test_library_exports_all_declared_symbols():
    """libscs.so loads without a GPU and exports every scs_* entry point that
    include/scs.h declares."""
    import ctypes
    from scs_gb300 import build as B
    from scs_gb300 import engine as E
    B.build()
    lib = ctypes.CDLL(B.lib_path())
    names = E.exported_symbols()
    assert len(names) >= 15
    missing = [s for s in names if not hasattr(lib, s)]
    assert not missing, missing


def test_engine_without_gpu_fails_loudly():
    """No silent CPU fallback: creating an engine without a GPU raises."""
    import torch
    if torch.cuda.is_available():
        pytest.skip("GPU present")
    from scs_gb300 import workloads as W
    from scs_gb300.engine import Engine, SCSError
    n, u, v = W.chung_lu(200, 1000, 2.5, seed=3)
    off, adj = W.to_csr(n, u, v)
    with pytest.raises(SCSError):
        Engine(csr=(n, off, adj), limit_queries=2)


@pytest.mark.skipif(_ref_dir() is None, reason="reference tree absent (set SCS_REF_DIR)")
def test_reference_sample_graphs_live(oracle_lib):
    """On the reference's own sample graphs and query files, the reference's
    compiled CPU code and the oracle agree (loader, cores, BFS, heuristics)."""
    import subprocess
    import sys
    from oracle import build_ref
    if not build_ref.build_ref():
        pytest.skip("reference CPU build unavailable")
    code = r'''
import sys, json, numpy as np
sys.path.insert(0, %r)
import oracle as O
path, qfile = sys.argv[1], sys.argv[2]
R = O.RefLib(); R.load(path)
g = O.OracleGraph.from_file(path)
assert np.array_equal(R.off, g.off) and np.array_equal(R.adj, g.adj)
assert np.array_equal(R.core, g.core) and R.dmax == g.dmax
n = 0
for line in open(qfile):
    p = line.split()
    if len(p) != 5: continue
    l, h, q = int(p[0]), int(p[1]), int(p[2])
    if q >= g.n: continue
    assert np.array_equal(R.bfs(q), g.bfs(q))
    for k in (2, 3, 4, 0):
        a, b = R.heuristic(k, l, h, q), g.heuristic(k, l, h, q)
        assert a[0] == b[0] and np.array_equal(a[1], b[1]), (k, l, h, q)
    n += 1
print(n)
''' % ROOT
    for graph, qf in (("data/graph.txt", "client/query/exp1_2/100"),
                      ("data/100.txt", "client/query/exp1_2/100"),
                      ("data/hepPH_SCS", "client/query/exp1_2/hepPh")):
        out = subprocess.run([sys.executable, "-c", code, os.path.join(_ref_dir(), graph),
                              os.path.join(_ref_dir(), qf)], capture_output=True, text=True)
        assert out.returncode == 0, out.stderr[-2000:]


def test_binding_structs_match_the_compiled_abi():
    """The ctypes mirrors of scs_config / scs_query / scs_result have the
    sizes and field offsets the library was compiled with."""
    import ctypes as C
    import numpy as np
    from scs_gb300 import build as B
    from scs_gb300 import engine as E
    B.build()
    out = np.zeros(8, dtype=np.uint64)
    assert E.lib().scs_abi_layout(out.ctypes.data_as(C.POINTER(C.c_uint64)), 8) == 8
    want = [C.sizeof(E.Config), E.Config.node_budget.offset, E.Config.device.offset,
            E.Config.active_queries.offset, C.sizeof(E.Query), C.sizeof(E.Result),
            E.Result.nodes.offset, E.Result.search_ns.offset]
    assert out.tolist() == want


def test_oracle_answers_match_reference_gpu_rows():
    """The oracle's exact answers equal the reference's own GPU search
    (its main.cu built unchanged, one query per server process, rows
    recorded by tests/golden/make_ref_gpu.py) on every query of the
    4000-vertex workload that the reference answered (Overtime = 0)."""
    ref = json.load(open(os.path.join(GOLD, "ref_gpu_chunglu_n4000.json")))
    gold = json.load(open(os.path.join(GOLD, "answers_chunglu_n4000.json")))
    assert ref["checksum"] == gold["checksum"]
    by_q = {(g["l"], g["h"], g["q"]): g for g in gold["queries"]}
    compared = 0
    for rq in ref["queries"]:
        g = by_q[(rq["l"], rq["h"], rq["q"])]
        for run in rq["runs"]:
            if run.get("degree") is None or run.get("overtime") != 0:
                continue
            assert g["finished"]
            assert run["degree"] == g["degree"], (rq, g)
            compared += 1
    assert compared >= 5
