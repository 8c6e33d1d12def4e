"""The learned branching path on the GPU: the trace the exact solver emits,
answers that do not depend on the network (any network, trained or not),
and what the trained network gains over the plain method on held-out
queries."""
import json
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
MODEL = os.path.join(ROOT, "scs_gb300", "weights", "rmat_s15_ef16.mlp")


def _gold_c1():
    g = json.load(open(os.path.join(GOLD, "answers_chunglu_n4000.json")))["queries"]
    return [q for q in g if q["finished"]]


@pytest.fixture(scope="module")
def og_c1_learned(chunglu_small, oracle_lib):
    return oracle_lib.OracleGraph.from_file(chunglu_small)


@pytest.fixture(scope="module")
def eng_c1_learned(chunglu_small):
    e = _engine(chunglu_small, limit_queries=32)
    yield e
    e.close()


def _engine(graph, **kw):
    from scs_gb300.engine import Engine
    kw.setdefault("pool_words", 1 << 26)
    kw.setdefault("stack_words", 1 << 22)
    kw.setdefault("slice_us", 50000)
    return Engine(graph=graph, **kw)


def test_trace_records_shortlisted_candidates(chunglu_small):
    """With the trace on, sampled steps record up to 16 candidates each: 16
    finite features in their stated ranges, keyed by the query's tag (its
    ticket) and a global vertex id of the graph."""
    gold = _gold_c1()[:8]
    rows = [(g["l"], g["h"], g["q"], g["heur"], g["limit_doms"]) for g in gold]
    e = _engine(chunglu_small, limit_queries=16)
    try:
        e.trace_enable(200000, 0)
        tickets = e.submit_many(rows)
        e.run()
        res = {r["ticket"]: r for r in e.poll()}
        X, keys, produced = e.trace_read()
    finally:
        e.close()
    assert len(X) > 0 and produced >= len(X)
    assert np.isfinite(X).all()
    tags = {t & 0xFFFFFFFF for t in tickets}
    assert set(keys[:, 0].tolist()) <= tags
    assert (keys[:, 1] < 4000).all()
    assert (X[:, 0] >= 0).all() and (X[:, 0] <= 1).all()   # dC / |C|
    assert set(np.unique(X[:, 8]).tolist()) <= {0.0, 1.0}   # rule's u* flag
    assert (X[:, 7] <= 1.0 + 1e-6).all()                    # score / best score
    # every traced step holds the rule's own u*
    assert X[:, 8].sum() > 0
    for t in tickets:
        assert res[t]["status"] in (0, 1)


def test_any_network_keeps_the_answers(chunglu_small, tmp_path):
    """The network only picks u* among the candidates the reference's rule
    accepts, so even an untrained network leaves every answer equal to the
    exact one (the oracle's, recorded in tests/golden)."""
    from oracle import mlp_ref as R
    from scs_gb300.engine import save_model
    path = str(tmp_path / "random.mlp")
    save_model(path, R.init_params(21))
    gold = _gold_c1()
    rows = [(g["l"], g["h"], g["q"], g["heur"], g["limit_doms"]) for g in gold]
    e = _engine(chunglu_small, limit_queries=64)
    try:
        e.load_model(path)
        res = e.solve(rows)
        e.load_model(None)
        plain = e.solve(rows[:6])
    finally:
        e.close()
    for g, r in zip(gold, res):
        assert r["status"] in (0, 1), r
        assert r["degree"] == g["degree"], (g, r)
        if r["status"] == 0 and r["degree"] > g["kl_heu"]:
            assert r["h_verified"] == 1
    for g, r in zip(gold, plain):
        assert r["degree"] == g["degree"]


def test_bad_model_files_are_rejected(chunglu_small, tmp_path):
    from scs_gb300.engine import SCSError
    bad = tmp_path / "bad.mlp"
    bad.write_bytes(b"SCSMLP01" + np.array([16, 64, 64, 1], np.uint32).tobytes())
    e = _engine(chunglu_small, limit_queries=4)
    try:
        with pytest.raises(SCSError):
            e.load_model(str(bad))
        with pytest.raises(SCSError):
            e.load_model(str(tmp_path / "missing.mlp"))
        assert e.solve([(3, 6, 10, 1, 1)])[0]["status"] in (0, 1)
    finally:
        e.close()


@pytest.mark.skipif(not os.path.exists(MODEL), reason="trained model not present")
def test_trained_network_gain_on_heldout_queries():
    """The trained network (scs_gb300/weights, trained by scs_gb300.train on
    the exact solver's traces) against the plain method on 200 held-out
    queries of the mid-size R-MAT workload (query seed 200), same 100k-task
    budget: every query both solve exactly gets the same degree, and the
    gain (exact answers, search tasks) is printed.  On the 1,000 held-out
    queries scs_gb300.train evaluates, the committed network answered 237
    exactly against the plain method's 236, with 0.3 % fewer search tasks:
    it does not shorten the searches on this workload."""
    from scs_gb300 import workloads as W
    from scs_gb300.engine import Engine, core_numbers
    from scs_gb300.train import HELDOUT_SEED, evaluate
    n, u, v = W.rmat(15, 16 << 15)
    off, adj = W.to_csr(n, u, v)
    core = core_numbers(n, off, adj)
    rows = [tuple(int(x) for x in r) for r in W.queries_mid(core, 200, seed=HELDOUT_SEED)]
    e = Engine(csr=(n, off, adj), limit_queries=200, node_budget=100000)
    try:
        ev = evaluate(e, rows, MODEL)
    finally:
        e.close()
    p, l = ev["plain"], ev["learned"]
    print("plain exact %d tasks %d %.2fs | learned exact %d tasks %d %.2fs"
          % (p["exact"], p["nodes"], p["seconds"], l["exact"], l["nodes"], l["seconds"]))
    assert ev["agree_where_both_exact"] == ev["both_exact"]
    # the network must not cost exact answers (within 2 % of the queries:
    # the two searches cut different trees at the same task budget)
    assert l["exact"] >= p["exact"] - 4


def test_forced_rule_choice_and_lookahead(eng_c1_learned, og_c1_learned, oracle_lib):
    """The one-step test kernel's forced u*: forcing the rule's own choice
    reproduces the unforced step, the shortlist holds the rule's u*, and the
    strong-branching lookahead counts that step's children."""
    from scs_gb300 import workloads as W
    og = og_c1_learned
    cases = []
    for (l, h, q, hf, ld) in W.queries_small(og.core).tolist():
        kl, _ = og.heuristic(0, l, h, q)
        if kl < min(int(og.core[q]), h - 1):
            cases.append((l, h, q, ld, kl, int(oracle_lib.lib().orc_ubd_host(kl, h))))
        if len(cases) == 4:
            break
    eng = eng_c1_learned
    eng.debug_prepare([(l, h, q, 0, ld) for (l, h, q, ld, kl, ubd) in cases],
                      [c[4] for c in cases], [c[5] for c in cases])
    tasks = []
    for i, (l, h, q, ld, kl, ubd) in enumerate(cases):
        ctx = oracle_lib.OracleCtx(og, l, h, q, kl, ubd, ld)
        tasks += [(i, k, e) for e, k in ctx.collect_tasks(kl, 10)]
    base = eng.debug_step(tasks, shortlist=True)
    branching = [j for j, g in enumerate(base) if int(g["hdr"][0]) == 0]
    assert branching
    force = [int(base[j]["hdr"][7]) for j in branching]
    sub = [tasks[j] for j in branching]
    forced = eng.debug_step(sub, force=force)
    for j, g in zip(branching, forced):
        b = base[j]
        assert int(b["hdr"][7]) in set(int(x) for x in b["sl_ids"])
        assert np.array_equal(g["hdr"][:12], b["hdr"][:12])
        assert len(g["kids"]) == len(b["kids"])
        for k1, k2 in zip(g["kids"], b["kids"]):
            assert np.array_equal(k1[2], k2[2])
        assert b["sl_feat"].shape == (len(b["sl_ids"]), 16)
        assert np.isfinite(b["sl_feat"]).all()
    hdr, nk, br, cost = eng.debug_lookahead(sub, force)
    for j, i in enumerate(branching):
        assert int(nk[j]) == len(base[i]["kids"])
        assert int(br[j]) <= int(nk[j])
        assert (int(cost[j]) == 0) == (int(br[j]) == 0)
    # another shortlisted candidate as u*: still a valid branching step
    alt = []
    for j in branching:
        ids = [int(x) for x in base[j]["sl_ids"]]
        alt.append(ids[-1])
    hdr2, nk2, br2, cost2 = eng.debug_lookahead(sub, alt)
    for j in range(len(sub)):
        assert int(hdr2[j][0]) == 0 and int(hdr2[j][7]) == alt[j]
