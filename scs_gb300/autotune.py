"""Autotuner: picks the search launch shape per graph and query-size range.

Swept parameters (the engine's counterparts of the reference's compile-time
BLK_NUMS/BLK_DIM and its partition/limitTasks arguments, inc/Intialize.h:26-31,
src/gpuMemoryAllocation.cc:73-78, main.cu:484-497):

* ``ctas_per_sm``    -- search CTAs per SM (the reference's blocks); it also
  sets how many per-vertex state words fit in shared memory (the
  shared-memory staging threshold: local graphs above it keep their state in
  L2-resident global memory);
* ``active_queries`` -- queries searched at once (the others wait prepared):
  the engine's counterpart of the reference's concurrent partitions;
* ``slice_us``       -- length of one persistent search launch;
* ``stack_words``    -- task-stack words per CTA (the reference's partition
  size pSize; 0 sizes the stacks from device memory).

The CTA width (256 threads) is fixed at compile time: 128-, 384- and
512-thread builds were measured slower on the mid-size workload.

Each candidate runs the same sample of queries under the same node budget;
the one with the most exact answers per second wins (ties: all answers per
second).  Results are cached as JSON keyed by a checksum of the graph and the
sample's h range.
"""
import hashlib
import json
import os
import time

import numpy as np

CACHE_DIR = os.environ.get("SCS_TUNE_DIR", os.path.join(os.path.expanduser("~"), ".cache", "scs_gb300"))
# (ctas_per_sm, active_queries, slice_us, stack_words)
DEFAULT_GRID = [(3, 32, 80000, 0), (2, 32, 80000, 0), (3, 16, 80000, 0), (3, 64, 80000, 0),
                (3, 128, 80000, 0), (3, 32, 40000, 0), (3, 32, 160000, 0),
                (3, 32, 80000, 1 << 21)]


def graph_key(off, adj, rows):
    h = hashlib.sha256()
    h.update(np.asarray(off, dtype=np.uint32).tobytes())
    h.update(np.asarray(adj, dtype=np.uint32).tobytes())
    hs = [int(r[1]) for r in rows]
    return "%s_h%d-%d" % (h.hexdigest()[:16], min(hs), max(hs))


def autotune(n, off, adj, rows, node_budget, grid=DEFAULT_GRID, use_cache=True,
             verbose=False, device=0):
    """Return (best_config_dict, trials).  rows: list of query tuples."""
    from .engine import Engine
    key = graph_key(off, adj, rows)
    path = os.path.join(CACHE_DIR, key + ".json")
    if use_cache and os.path.exists(path):
        try:
            d = json.load(open(path))
            return d["best"], d["trials"]
        except Exception:
            pass
    trials = []
    for cps, active, slice_us, stack_words in grid:
        # task store sized from device memory unless the trial sets the stacks
        eng = Engine(csr=(n, off, adj), limit_queries=len(rows), ctas_per_sm=cps,
                     slice_us=slice_us, node_budget=node_budget, device=device,
                     active_queries=active, stack_words=stack_words)
        t0 = time.perf_counter()
        res = eng.solve(rows)
        dt = time.perf_counter() - t0
        st = eng.stats()
        eng.close()
        exact = sum(1 for r in res if r["status"] in (0, 1))
        trial = {"ctas_per_sm": cps, "active_queries": active, "slice_us": slice_us,
                 "stack_words": stack_words, "seconds": dt, "qps": len(rows) / dt,
                 "exact_qps": exact / dt, "nodes": st["nodes"], "exact": exact}
        trials.append(trial)
        if verbose:
            print("autotune", trial, flush=True)
    best = max(trials, key=lambda t: (t["exact_qps"], t["qps"]))
    best = {k: best[k] for k in ("ctas_per_sm", "active_queries", "slice_us", "stack_words")}
    try:
        os.makedirs(CACHE_DIR, exist_ok=True)
        json.dump({"best": best, "trials": trials}, open(path, "w"))
    except OSError:
        pass
    return best, trials
