"""Train the learned branching scorer from the exact solver's own traces.

    python -m scs_gb300.train [--queries 5000] [--label membership|lookahead]
                              [--out scs_gb300/weights/rmat_s15_ef16.mlp]

1. The plain engine solves the training queries of the mid-size R-MAT
   workload (scale 15, edge factor 16; query seed 100, disjoint from the
   benchmark's seeds 42/43 and the held-out seed 200) with the trace on:
   sampled search steps record their shortlisted candidates' 16 features
   (mlp.cuh: d_C, d_R, q_dist, core, degree, task size, bounds, ...) and the
   candidate's global id.
2. Labels come from the solver's answers: for each query it solved exactly
   (status done), a candidate is positive when it lies in the returned
   optimal community.  Records of queries stopped by the budget are dropped.
3. The network is trained on the GPU by the engine's own kernels
   (scs_mlp_train), positives weighted up to balance the classes, and
   written as a model file for scs_load_model.

With --label lookahead, step 1-2 are replaced by strong-branching labels
from the engine's one-step test kernel (see lookahead()).

The file written here is the one the benchmark's learned arm loads.
"""
import argparse
import json
import os
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

DEFAULT_OUT = os.path.join(ROOT, "scs_gb300", "weights", "rmat_s15_ef16.mlp")
TRAIN_SEED = 100
HELDOUT_SEED = 200


def init_params(seed=0):
    """He-uniform weights, zero biases, in file order."""
    rng = np.random.default_rng(seed)
    parts = []
    for fan_in, fan_out in ((16, 128), (128, 128), (128, 1)):
        lim = np.sqrt(6.0 / fan_in)
        parts.append(rng.uniform(-lim, lim, size=fan_in * fan_out))
        parts.append(np.zeros(fan_out))
    return np.concatenate(parts).astype(np.float32)


def collect(eng, rows, max_records=8_000_000, sample_shift=2):
    """Solve rows with the trace on; returns (X, y, per-query info)."""
    eng.trace_enable(max_records, sample_shift)
    t0 = time.time()
    tickets = eng.submit_many(rows)
    eng.run()
    res = {}
    while True:
        rs = eng.poll()
        if not rs:
            break
        for r in rs:
            res[r["ticket"]] = r
    X, keys, produced = eng.trace_read()
    eng.trace_enable(0)
    by_tag = {t & 0xFFFFFFFF: res[t] for t in tickets}
    keep = np.zeros(len(keys), dtype=bool)
    y = np.zeros(len(keys), dtype=np.float32)
    members = {}
    for tag, r in by_tag.items():
        if r["status"] == 0 and r["h_verified"]:
            members[tag] = set(int(v) for v in r["H"])
    for i, (tag, gid) in enumerate(keys.tolist()):
        m = members.get(tag)
        if m is not None:
            keep[i] = True
            y[i] = 1.0 if gid in m else 0.0
    info = {"queries": len(rows), "exact": len(members), "records": int(len(keys)),
            "records_produced": int(produced), "labelled": int(keep.sum()),
            "positives": int(y[keep].sum()), "seconds": round(time.time() - t0, 1)}
    return X[keep], y[keep], info


def lookahead(eng, n, off, adj, rows, max_len=8000, per_level=3, levels=3, batch=24,
              seed=0, log=None):
    """Strong-branching labels from the engine's own one-step test kernel.

    For each training query: its local graph is prepared, the root task and
    a few sampled descendants (up to `levels` deep, `per_level` children of
    each) are stepped with the shortlist on, and every shortlisted candidate
    is then forced as u* (scs_debug_lookahead): the forced step's children
    get one step each, and the candidate's cost is the summed live size of
    the children that still branch -- the work left one level below that
    choice.  Candidates of least cost are the positives; tasks whose
    candidates all cost the same carry no preference and are dropped.
    Returns (X, y, info)."""
    from .engine import distance_bound, greedy_incumbent
    rng = np.random.default_rng(seed)
    X, Y = [], []
    stat = {"queries": 0, "tasks": 0, "tasks_labelled": 0}
    t0 = time.time()
    core = eng.core_numbers()
    for b0 in range(0, len(rows), batch):
        kls, ubds, keep = [], [], []
        for (l, h, q, hf, ld) in rows[b0:b0 + batch]:
            kl, _ = greedy_incumbent(n, off, adj, l, h, q)
            if kl >= min(int(core[q]), h - 1):
                continue  # answered by the incumbent: never searched
            keep.append((l, h, q, 0, ld))
            kls.append(kl)
            ubds.append(distance_bound(kl, h))
        if not keep:
            continue
        nl, ql = eng.debug_prepare(keep, kls, ubds)
        level = []
        for i in range(len(keep)):
            if 0 < int(nl[i]) <= max_len:
                ent = np.arange(int(nl[i]), dtype=np.uint32) << 1
                ent[int(ql[i])] |= 1
                level.append((i, kls[i], ent))
        stat["queries"] += len(level)
        for _ in range(levels):
            if not level:
                break
            got = eng.debug_step(level, shortlist=True)
            nxt, lt, lf, pend = [], [], [], []
            for task, g in zip(level, got):
                if int(g["hdr"][0]) != 0:
                    continue  # pruned: no branching decision here
                kids = [k for k in g["kids"] if len(k[2]) <= max_len]
                for j in rng.permutation(len(kids))[:per_level]:
                    nxt.append((task[0], int(g["hdr"][1]), kids[j][2]))
                ids = g["sl_ids"]
                if len(ids) < 2:
                    continue
                lt += [task] * len(ids)
                lf += [int(c) for c in ids]
                pend.append((g["sl_feat"], len(ids)))
            stat["tasks"] += len(pend)
            if lt:
                _, _, _, cost = eng.debug_lookahead(lt, lf)
                k = 0
                for feat, m in pend:
                    c = cost[k:k + m].astype(np.float64)
                    k += m
                    if c.max() > c.min():
                        X.append(feat)
                        Y.append((c == c.min()).astype(np.float32))
            level = nxt
        if log:
            log("lookahead: %d queries, %d tasks, %d labelled, %.0f s"
                % (stat["queries"], stat["tasks"], len(Y), time.time() - t0))
    stat["tasks_labelled"] = len(Y)
    stat["seconds"] = round(time.time() - t0, 1)
    if not X:
        return np.zeros((0, 16), np.float32), np.zeros(0, np.float32), stat
    return np.concatenate(X).astype(np.float32), np.concatenate(Y), stat


def evaluate(eng, rows, model_path):
    """Plain vs learned on the same queries: answers, exact counts, tasks."""
    out = {}
    for name, path in (("plain", None), ("learned", model_path)):
        eng.load_model(path)
        t0 = time.time()
        res = eng.solve(rows)
        dt = time.time() - t0
        out[name] = {"seconds": dt, "exact": sum(1 for r in res if r["status"] in (0, 1)),
                     "nodes": int(sum(r["nodes"] for r in res)),
                     "degrees": [int(r["degree"]) for r in res],
                     "status": [int(r["status"]) for r in res]}
    eng.load_model(None)
    p, l = out["plain"], out["learned"]
    both = [i for i in range(len(rows)) if p["status"][i] in (0, 1) and l["status"][i] in (0, 1)]
    out["agree_where_both_exact"] = sum(1 for i in both if p["degrees"][i] == l["degrees"][i])
    out["both_exact"] = len(both)
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--queries", type=int, default=5000)
    ap.add_argument("--heldout", type=int, default=1000)
    ap.add_argument("--node-budget", type=int, default=100000,
                    help="task budget of the trace run and the held-out evaluation "
                         "(the committed model: 100000)")
    ap.add_argument("--epochs", type=int, default=30)
    ap.add_argument("--max-samples", type=int, default=400000)
    ap.add_argument("--sample-shift", type=int, default=2)
    ap.add_argument("--label", default="membership", choices=["membership", "lookahead"],
                    help="lookahead: strong-branching labels from forced one-step "
                         "lookahead; membership: candidate in the returned optimum")
    ap.add_argument("--lookahead-queries", type=int, default=400)
    ap.add_argument("--out", default=DEFAULT_OUT)
    ap.add_argument("--device", type=int, default=0)
    a = ap.parse_args()
    from scs_gb300 import workloads as W
    from scs_gb300.engine import Engine, core_numbers, mlp_train, save_model
    n, u, v = W.rmat(15, 16 << 15)
    off, adj = W.to_csr(n, u, v)
    core = core_numbers(n, off, adj)
    rows = [tuple(int(x) for x in r) for r in W.queries_mid(core, a.queries, seed=TRAIN_SEED)]
    eng = Engine(csr=(n, off, adj), limit_queries=1000, node_budget=a.node_budget,
                 device=a.device)
    if a.label == "lookahead":
        X, y, info = lookahead(eng, n, off, adj, rows[: a.lookahead_queries],
                               log=lambda m: print(m, flush=True))
    else:
        X, y, info = collect(eng, rows, sample_shift=a.sample_shift)
    info["label"] = a.label
    rng = np.random.default_rng(0)
    if len(y) > a.max_samples:
        idx = rng.choice(len(y), a.max_samples, replace=False)
        X, y = X[idx], y[idx]
    pos = max(float(y.sum()), 1.0)
    w = np.where(y > 0.5, (len(y) - pos) / pos, 1.0).astype(np.float32)
    t0 = time.time()
    params, losses = mlp_train(X, y, init_params(1), w=w, epochs=a.epochs, batch=4096,
                               lr=1e-3, seed=2, device=a.device)
    info["train_seconds"] = round(time.time() - t0, 2)
    info["samples"] = int(len(y))
    info["epoch_loss"] = [round(float(x), 5) for x in losses]
    os.makedirs(os.path.dirname(os.path.abspath(a.out)), exist_ok=True)
    save_model(a.out, params)
    if a.heldout:
        held = [tuple(int(x) for x in r)
                for r in W.queries_mid(core, a.heldout, seed=HELDOUT_SEED)]
        ev = evaluate(eng, held, a.out)
        info["heldout"] = {k: (v if not isinstance(v, dict) else
                               {kk: vv for kk, vv in v.items() if kk not in ("degrees", "status")})
                           for k, v in ev.items()}
    eng.close()
    print(json.dumps(info))
    with open(os.path.splitext(a.out)[0] + ".json", "w") as f:
        json.dump(info, f, indent=1)
    return 0


if __name__ == "__main__":
    sys.exit(main())
