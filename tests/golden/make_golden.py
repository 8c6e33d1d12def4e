"""Generate the golden fixtures in tests/golden/ (run from the repo root).

* ``heuristic_<graph>.json`` -- the reference's OWN greedy incumbent
  (inc/heuristic.h, compiled from its sources into oracle/_ref) for the first
  queries of each workload: kl and H per heu2/heu3/heu4/CSSC.  Pins the
  oracle's and the engine's heuristic restatements.
* ``answers_<graph>.json`` -- exact answers (max min degree) of the CPU
  oracle's branch-and-bound for the workload queries, with the oracle's node
  count; only queries finishing within the node limit are recorded.
* ``bruteforce_small.json`` -- exhaustive answers on small random graphs.
Each file records a checksum of the graph it was computed on, so a change in
the generators is detected instead of silently comparing different graphs.

Usage: python tests/golden/make_golden.py [heuristic|answers|brute|all]
       python tests/golden/make_golden.py answers_rmat <count> <node_limit>
           (answers_rmat_s15_ef16.json: the mid-size workload's first
           <count> queries; committed with 120 and 200000, about
           2.5 hours on 8 cores)
"""
import hashlib
import json
import multiprocessing as mp
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
OUT = os.path.dirname(os.path.abspath(__file__))


def graph_sum(off, adj):
    h = hashlib.sha256()
    h.update(np.asarray(off, dtype=np.uint32).tobytes())
    h.update(np.asarray(adj, dtype=np.uint32).tobytes())
    return h.hexdigest()[:16]


def workload(name, tmpdir):
    from scs_gb300 import workloads as W
    gb, qb = W.WORKLOADS[name]
    n, u, v = gb()
    path = os.path.join(tmpdir, name + ".txt")
    if not os.path.exists(path):
        W.write_edgelist(path, n, u, v)
    return path, qb


def _heu_child(args):
    path, name, count = args
    import oracle as O
    R = O.RefLib()
    R.load(path)
    from scs_gb300 import workloads as W
    qb = W.WORKLOADS[name][1]
    Q = qb(R.core)
    rows = []
    for (l, h, q, hf, ld) in Q[:count].tolist():
        rec = {"l": l, "h": h, "q": q}
        for k in (2, 3, 4, 0):
            kl, H = R.heuristic(k, l, h, q)
            rec["kl%d" % k] = kl
            rec["H%d" % k] = H.tolist()
        rows.append(rec)
    return {"graph": name, "checksum": graph_sum(R.off, R.adj), "n": R.n,
            "dmax": R.dmax, "core_max": int(R.core.max()),
            "core_sum": int(R.core.astype(np.int64).sum()), "queries": rows}


def make_heuristic(tmpdir):
    jobs = [("chunglu_n4000", 50), ("rmat_s15_ef16", 200)]
    for name, count in jobs:
        path, _ = workload(name, tmpdir)
        # the reference library keeps one graph per process: one child each
        with mp.get_context("spawn").Pool(1) as p:
            res = p.map(_heu_child, [(path, name, count)])[0]
        with open(os.path.join(OUT, "heuristic_%s.json" % name), "w") as f:
            json.dump(res, f)
        print("heuristic", name, len(res["queries"]))


def _solve_child(args):
    path, name, idx, limit = args
    import oracle as O
    from scs_gb300 import workloads as W
    g = O.OracleGraph.from_file(path)
    Q = W.WORKLOADS[name][1](g.core)
    l, h, q, hf, ld = [int(x) for x in Q[idx]]
    r, H = g.solve(l, h, q, hf, ld, node_limit=limit)
    return dict(i=idx, l=l, h=h, q=q, heur=hf, limit_doms=ld, degree=int(r.degree),
                kl_heu=int(r.kl_heu), heu_hit=int(r.heu_hit), nodes=int(r.nodes),
                finished=int(r.status == 0), n_local=int(r.n_local))


def make_answers(tmpdir, name, count, limit, procs):
    path, _ = workload(name, tmpdir)
    import oracle as O
    g = O.OracleGraph.from_file(path)
    with mp.get_context("spawn").Pool(procs) as p:
        rows = p.map(_solve_child, [(path, name, i, limit) for i in range(count)])
    res = {"graph": name, "checksum": graph_sum(g.off, g.adj), "node_limit": limit,
           "queries": rows}
    with open(os.path.join(OUT, "answers_%s.json" % name), "w") as f:
        json.dump(res, f)
    print("answers", name, sum(r["finished"] for r in rows), "of", len(rows))


def make_brute():
    import oracle as O
    from scs_gb300 import workloads as W
    rng = np.random.default_rng(20261203)
    cases = []
    for trial in range(40):
        n = int(rng.integers(7, 15))
        p = float(rng.uniform(0.25, 0.6))
        iu = np.triu_indices(n, 1)
        mask = rng.random(len(iu[0])) < p
        u, v = iu[0][mask].astype(np.uint32), iu[1][mask].astype(np.uint32)
        off, adj = W.to_csr(n, u, v)
        g = O.OracleGraph(n, off, adj)
        qs = []
        for q in range(n):
            for (l, h) in [(2, 4), (3, 6), (4, 8), (2, 10)]:
                qs.append(dict(l=l, h=h, q=q, degree=g.bruteforce(l, h, q)))
        cases.append(dict(n=n, u=u.tolist(), v=v.tolist(), queries=qs))
    with open(os.path.join(OUT, "bruteforce_small.json"), "w") as f:
        json.dump(cases, f)
    print("brute", len(cases))


if __name__ == "__main__":
    what = sys.argv[1] if len(sys.argv) > 1 else "all"
    import tempfile
    tmp = tempfile.mkdtemp(prefix="scs_golden_")
    from oracle import build_ref
    build_ref.build_oracle()
    if what in ("heuristic", "all"):
        build_ref.build_ref()
        make_heuristic(tmp)
    if what in ("brute", "all"):
        make_brute()
    if what in ("answers", "all"):
        make_answers(tmp, "chunglu_n4000", 50, 300000, 8)
    if what == "answers_rmat":
        make_answers(tmp, "rmat_s15_ef16", int(sys.argv[2]), int(sys.argv[3]), 8)
