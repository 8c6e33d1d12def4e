"""Failure paths, driven from the host (no GPU fault, trap or hang): the
search budget (the reference's level cap, Overtime=1), task-store overflow
(the reference's buffer overflow, Overtime=2) and malformed queries."""
import json
import os

import pytest

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _gold_hard(k):
    g = json.load(open(os.path.join(GOLD, "answers_chunglu_n4000.json")))["queries"]
    return [q for q in g if not q["heu_hit"]][:k]


def test_search_budget_reports_timeout(chunglu_small):
    from scs_gb300.engine import TIMEOUT, DONE, Engine
    eng = Engine(graph=chunglu_small, limit_queries=8, node_budget=40,
                 stack_words=1 << 22, pool_words=1 << 24)
    rows = [(g["l"], g["h"], g["q"], g["heur"], g["limit_doms"]) for g in _gold_hard(4)]
    res = eng.solve(rows)
    assert any(r["status"] == TIMEOUT for r in res)
    for g, r in zip(_gold_hard(4), res):
        assert r["status"] in (TIMEOUT, DONE)
        assert r["kl_heuristic"] <= r["degree"] <= max(g["degree"], r["kl_heuristic"])
        assert r["nodes"] >= 1
    # the engine keeps working after stopped queries
    again = eng.solve(rows[:1])
    assert again[0]["status"] in (TIMEOUT, DONE)
    eng.close()


def test_task_store_overflow_reports_capacity(chunglu_small):
    from scs_gb300.engine import CAPACITY, DONE, Engine
    # stacks and pool too small for the 4000-vertex root task records
    eng = Engine(graph=chunglu_small, limit_queries=4, stack_words=4096, pool_words=1 << 14)
    rows = [(g["l"], g["h"], g["q"], g["heur"], g["limit_doms"]) for g in _gold_hard(2)]
    res = eng.solve(rows)
    assert all(r["status"] in (CAPACITY, DONE) for r in res)
    assert any(r["status"] == CAPACITY for r in res)
    for r in res:
        assert r["degree"] >= r["kl_heuristic"]
    eng.close()


def test_bad_queries_are_rejected_not_fatal(chunglu_small):
    from scs_gb300.engine import BAD_QUERY, Engine
    eng = Engine(graph=chunglu_small, limit_queries=4, stack_words=1 << 22, pool_words=1 << 24)
    res = eng.solve([(3, 8, 10 ** 7, 1, 1), (9, 5, 10, 1, 1), (3, 600, 10, 1, 1)])
    assert [r["status"] for r in res] == [BAD_QUERY] * 3
    ok = eng.solve([(3, 6, 10, 1, 1)])[0]
    assert ok["status"] in (0, 1)
    eng.close()


def test_small_task_store_answers_match_golden(chunglu_small):
    """A task store far smaller than the default (16k-word stacks per CTA,
    two of the largest task records; a 512 MB pool) on the
    4000-vertex workload's queries the oracle solved exactly: records spill
    from the stacks to the pool, the bottom records are donated to idle CTAs
    and stolen, stacks slide down over the room the donations left, and
    every answer still equals the golden one (the reference's overflow
    store, src/helpers.cc:1393-1618)."""
    from scs_gb300.engine import DONE, HEURISTIC, Engine
    g = json.load(open(os.path.join(GOLD, "answers_chunglu_n4000.json")))["queries"]
    gold = [q for q in g if q["finished"] and not q["heu_hit"]]
    assert len(gold) >= 20
    rows = [(q["l"], q["h"], q["q"], q["heur"], q["limit_doms"]) for q in gold]
    eng = Engine(graph=chunglu_small, limit_queries=16, stack_words=1 << 14,
                 pool_words=1 << 27, slice_us=50000, active_queries=4)
    try:
        res = eng.solve(rows)
        st = eng.stats()
    finally:
        eng.close()
    print("small store:", {k: st[k] for k in ("spills", "donations", "steals", "slides")})
    for q, r in zip(gold, res):
        assert r["status"] in (DONE, HEURISTIC), (q, r)
        assert r["degree"] == q["degree"], (q, r)
    assert st["spills"] > 0 and st["donations"] > 0 and st["steals"] > 0, st
    assert st["slides"] > 0, st


def test_release_waits_for_pool_room(chunglu_small):
    """Admission by free task-store memory: with a pool that holds only a
    few root-sized records, prepared queries wait for room (release_headroom
    records of their root's size each) instead of all starting at once, and
    every answer still equals the golden one."""
    from scs_gb300.engine import DONE, HEURISTIC, Engine
    g = json.load(open(os.path.join(GOLD, "answers_chunglu_n4000.json")))["queries"]
    gold = [q for q in g if q["finished"] and not q["heu_hit"]][:16]
    rows = [(q["l"], q["h"], q["q"], q["heur"], q["limit_doms"]) for q in gold]
    eng = Engine(graph=chunglu_small, limit_queries=32, stack_words=1 << 22,
                 pool_words=1 << 17, slice_us=20000, release_headroom=4)
    try:
        res = eng.solve(rows)
        st = eng.stats()
    finally:
        eng.close()
    for q, r in zip(gold, res):
        assert r["status"] in (DONE, HEURISTIC), (q, r)
        assert r["degree"] == q["degree"], (q, r)
    assert st["held_memory"] > 0, st
    assert st["releases"] == sum(1 for r in res if r["nodes"] > 0)


def test_local_graph_limit_reports_too_large(chunglu_small):
    """scs_config.max_local bounds the local graph a query may search: with a
    limit of 64 vertices the 4000-vertex workload's searched queries report
    SCS_TOO_LARGE (their incumbent as the degree), the others keep their
    exact answers, and the engine goes on working."""
    from scs_gb300.engine import DONE, HEURISTIC, TOO_LARGE, Engine
    g = json.load(open(os.path.join(GOLD, "answers_chunglu_n4000.json")))["queries"]
    gold = [q for q in g if q["finished"]][:12]
    rows = [(q["l"], q["h"], q["q"], q["heur"], q["limit_doms"]) for q in gold]
    eng = Engine(graph=chunglu_small, limit_queries=16, stack_words=1 << 20,
                 pool_words=1 << 24, max_local=64)
    try:
        res = eng.solve(rows)
    finally:
        eng.close()
    assert any(r["status"] == TOO_LARGE for r in res)
    for q, r in zip(gold, res):
        if r["status"] == TOO_LARGE:
            assert r["degree"] == r["kl_heuristic"] <= q["degree"]
        else:
            assert r["status"] in (DONE, HEURISTIC) and r["degree"] == q["degree"]


def test_invalid_prep_cluster_is_refused(chunglu_small):
    """A preparation cluster size other than 1, 2, 4, 8 or 16 is refused at
    creation with an error, and a valid one on the same graph works."""
    from scs_gb300.engine import Engine, SCSError
    with pytest.raises(SCSError):
        Engine(graph=chunglu_small, limit_queries=4, stack_words=1 << 20, pool_words=1 << 24,
               prep_ctas=3)
    eng = Engine(graph=chunglu_small, limit_queries=4, stack_words=1 << 20, pool_words=1 << 24,
                 prep_ctas=2)
    try:
        assert eng.solve([(3, 6, 10, 1, 1)])[0]["status"] in (0, 1)
    finally:
        eng.close()
