"""Benchmark: exact size-bounded community search queries/sec on one GB300.

Workload (one per GPU): the mid-size plain-GPU workload -- R-MAT scale 15
(n = 32,768), exactly 16 * 2^15 unique undirected edges, (a, b, c) =
(.57, .19, .19), graph seed 1234; 1,000 queries (seed 42): q uniform over
vertices with core >= 8, l ~ U[3, 10], h = l + U[5, 30], heuristic on,
dominating limit 10.  Warm-up steps use extra queries from seed 43.

A step is one batch of `--batch` queries submitted at once and run to
completion (default: the whole 1,000-query workload in one step, as the
workload defines it, so the engine batches continuously across all of them);
warm-up steps run `--warmup-batch` other queries each.  Every query
carries the same search budget (`--node-budget` tasks, the stand-in for the
reference's level cap, main.cu:444-463); a query that hits it reports the
best degree found with status "timeout" (the reference's Overtime=1) and
does not count as exact.

value  = exact answers (status done or heuristic) / device time of the
         timed steps (CUDA events recorded around submit, run and poll; the
         engine's own stream is synchronized before the call returns; graph
         resident).  Budget-stopped answers are not counted; all answers per
         second are reported beside it in config.  Default budget: 20,000
         search tasks per query.
e2e    = exact answers / host-clock time of the same calls through the C
         ABI from host buffers (submit, run, poll of results and
         communities).  The engine is host-driven between slices, so the two
         agree.
--impl reference times the reference's CPU path (the oracle port of its
branch-and-bound on the reference's heuristics) on all host cores, on a
sample of each step's queries under the same node budget, no wall cap.
--serve RATES runs Poisson arrivals at each rate (queries/s) instead and
prints one line per rate with latency from arrival (see run_serve).
--arm plain|learned picks the integer rules alone (default) or the trained
network's branching and incumbent proposal; the other arm is run on the
first step's queries after the timed region and reported in config.compare.
--workload chunglu_n1m / rmat_s22 selects the 1M-vertex Chung-Lu workload or
the scale-22 R-MAT serving workload instead of the mid-size one.
"""
import argparse
import json
import os
import subprocess
import sys
import tempfile
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "exact queries/sec + p50/p99 latency"
UNIT = "queries/s"
# --workload: graph name in scs_gb300.workloads, workload name, description
WORKLOADS = {
    "rmat_s15": ("rmat_s15_ef16", "rmat_s15_ef16_q1000", "R-MAT scale 15, 524288 edges"),
    "chunglu_n1m": ("chunglu_n1m", "chunglu_n1m_q10000_uneven",
                    "Chung-Lu n=1,000,000, m=20,000,000, exponent 2.3"),
    "rmat_s22": ("rmat_s22_ef16", "rmat_s22_ef16_serving", "R-MAT scale 22, edge factor 16"),
}
_WL = ["rmat_s15"]
MODEL = os.path.join(ROOT, "scs_gb300", "weights", "rmat_s15_ef16.mlp")


def env_rank():
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")),
            int(os.environ.get("LOCAL_RANK", "0")))


def build_workload(batch, warmup, steps):
    from scs_gb300 import workloads as W
    gb, _ = W.WORKLOADS[WORKLOADS[_WL[0]][0]]
    n, u, v = gb()
    off, adj = W.to_csr(n, u, v)
    return n, off, adj


def queries_for(core, count, seed):
    from scs_gb300 import workloads as W
    _, qb = W.WORKLOADS[WORKLOADS[_WL[0]][0]]
    return qb(core, count=count, seed=seed)


class Clocks:
    """nvidia-smi samples during the timed region."""

    def __init__(self, path):
        self.path = path
        self.proc = None

    def start(self):
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", "--query-gpu=index,clocks.sm,clocks.max.sm,power.draw,"
                 "clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
                 "clocks_event_reasons.hw_thermal_slowdown,"
                 "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self, gpu_index=0):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.f.close()
        sms, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            p = [x.strip() for x in line.split(",")]
            if len(p) < 9 or p[0] != str(gpu_index):
                continue
            try:
                sms.append(float(p[1]))
                mx = float(p[2])
            except ValueError:
                continue
            for nm, val in zip(names, p[5:9]):
                if val.lower() == "active":
                    reasons.add(nm)
        if not sms:
            return None
        return {"sm_mhz": float(np.median(sms)), "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sms)}


def reduce_over_ranks(dist, torch, t_dev, wall, queries, device):
    """Replicas: whole-job time is the slowest rank's, throughput counts the
    queries of every rank."""
    if dist is None:
        return t_dev, wall, queries
    t = torch.tensor([t_dev, wall], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    q = torch.tensor([float(queries)], dtype=torch.float64, device=device)
    dist.all_reduce(q)
    return float(t[0]), float(t[1]), int(q[0])


def flush_l2(torch, buf):
    # write a buffer larger than L2 (129 MB) between timed steps
    buf.fill_(1.0)


def measured_peak_gbs():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        try:
            return float(json.load(open(p))["hbm_gbs"]), "measured"
        except Exception:
            pass
    return 6800.0, "fallback"


def host_cpu_info():
    """Host cores and CPU model of the machine the CPU arm runs on."""
    model = ""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.startswith("Model name"):
                model = line.split(":", 1)[1].strip()
                break
    except Exception:
        pass
    return {"nproc": os.cpu_count() or 1, "lscpu_model": model}


def cpu_baseline(n, off, adj, rows, budget, procs=None, cap_s=0.0):
    """The reference's CPU path (the oracle port of its branch-and-bound on
    the reference's own heuristics, oracle.c) on the host cores: the sampled
    queries go to a pool of single-threaded processes, one query at a time
    each, under the same per-query node budget as the GPU (no wall-clock cap
    unless cap_s > 0).  Returns a dict: the makespan of the sample, exact
    answers (status done/heuristic) and all answers, per-query times (each
    is the single-thread time of that query), tasks."""
    import multiprocessing as mp
    procs = max(1, min(procs or (os.cpu_count() or 1), len(rows)))
    ctx = mp.get_context("spawn")
    args = [(tuple(int(x) for x in r), budget) for r in rows]
    with ctx.Pool(procs, initializer=_cpu_init, initargs=(n, off, adj, cap_s)) as pool:
        pool.map(_cpu_noop, range(procs))  # processes up and the graph loaded
        t0 = time.perf_counter()
        out = list(pool.imap_unordered(_cpu_solve, args, chunksize=1))
        span = time.perf_counter() - t0
    times = [o[0] for o in out]
    exact = sum(1 for o in out if o[2] == 0)
    return {"span_s": span, "queries": len(rows), "exact": exact, "procs": procs,
            "times": times, "tasks": sum(o[1] for o in out),
            "budget_stopped": sum(1 for o in out if o[2] == 1),
            "capped": sum(1 for o in out if o[2] == 2)}


def _cpu_desc(r, budget):
    t = np.array(r["times"]) if r["times"] else np.zeros(1)
    return ("%d queries (the first of each step), one per process on %d host cores, "
            "node budget %d per query, no wall-clock cap; makespan %.1f s; %d exact, %d stopped "
            "by the budget; single-thread %.2f s per query (mean), %.0f tasks/s per core"
            % (r["queries"], r["procs"], budget, r["span_s"], r["exact"], r["budget_stopped"],
               float(t.mean()), r["tasks"] / max(float(t.sum()), 1e-9)))


_CPU_G = None


def _cpu_init(n, off, adj, cap_s):
    global _CPU_G
    import oracle as O
    _CPU_G = O.OracleGraph(n, off, adj)
    O.lib().orc_set_time_limit(cap_s)


def _cpu_noop(_):
    return 0


def _cpu_solve(args):
    """One query on one core.  Status as the engine reports it: 0 exact
    (search finished, or the incumbent is optimal), 1 stopped by the node
    budget, 2 stopped by a wall-clock cap."""
    row, budget = args
    l, h, q, hf, ld = row
    t0 = time.perf_counter()
    r, _ = _CPU_G.solve(l, h, q, hf, ld, node_limit=budget)
    return time.perf_counter() - t0, int(r.nodes), int(r.status)


def run_reference(args):
    """--impl reference: the reference's CPU path on the host cores, on the
    same workload, metric and node budget as the GPU arm.  Each of the K
    timed steps contributes a sample of its own queries (its first
    --ref-sample); the K samples run together on all host cores, one query
    per process at a time, and the timed region is their makespan, so
    ms_per_step = makespan / K and value = exact answers / makespan.
    Warm-up steps run a few other queries (seed 43) under a small budget,
    only to start the processes."""
    rank, world, _ = env_rank()
    if rank != 0:
        return 0
    n, off, adj = build_workload(args.batch, args.warmup, args.steps)
    import oracle as O
    og = O.OracleGraph(n, off, adj)
    rows = queries_for(og.core, args.batch * args.steps, 42)
    procs = os.cpu_count() or 1
    if args.warmup:
        warm = queries_for(og.core, 2 * args.warmup, 43)
        cpu_baseline(n, off, adj, warm, 1000, procs=procs)
    sample = [r for i in range(args.steps)
              for r in rows[i * args.batch:(i + 1) * args.batch][: args.ref_sample]]
    r = cpu_baseline(n, off, adj, sample, args.node_budget, procs=procs)
    span = r["span_s"]
    v = r["exact"] / span if span > 0 else 0.0
    t = np.array(r["times"])
    info = host_cpu_info()
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 * span / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u32",
            "data": "synthetic",
            "config": {"workload": WORKLOADS[_WL[0]][1], "batch": args.batch, "sample_per_step": args.ref_sample,
                       "sampled_queries": len(sample), "node_budget": args.node_budget,
                       "wall_cap": None,
                       "timed_region": "the K steps' samples run together on all host cores "
                                       "(makespan); ms_per_step = makespan / K",
                       "all_answers_per_s": len(sample) / span if span > 0 else 0.0,
                       "exact_fraction": r["exact"] / max(len(sample), 1),
                       "single_thread_s_per_query": float(t.mean()) if len(t) else None,
                       "single_thread_exact_per_s": r["exact"] / max(float(t.sum()), 1e-9),
                       **info},
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": r["procs"], "kind": "port",
                             "sample": _cpu_desc(r, args.node_budget)},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


def run_serve(args):
    """Serving mode: queries arrive as a Poisson process at each rate for
    --serve-seconds and are submitted at their arrival times while the engine
    steps (admission between slices; the engine's 80 ms slices unless
    --slice-us says otherwise: a slice ends early once nothing is left to
    search, so long slices cost no latency at low load and save slice
    boundaries under load).  Latency runs from arrival to the result;
    throughput is the completed queries over the time to the last result.
    One GPU, rank 0."""
    rank, world, local = env_rank()
    if rank != 0:
        return 0
    from scs_gb300.engine import Engine, core_numbers
    n, off, adj = build_workload(args.batch, args.warmup, args.steps)
    core = core_numbers(n, off, adj)
    for rate in [float(x) for x in args.serve.split(",") if x]:
        count = max(1, int(rate * args.serve_seconds))
        rows = [tuple(int(x) for x in r) for r in queries_for(core, count, 44)]
        rng = np.random.default_rng(45)
        arrive = np.cumsum(rng.exponential(1.0 / rate, count))
        eng = Engine(csr=(n, off, adj), limit_queries=args.slots or 256,
                     slice_us=args.slice_us,
                     ctas_per_sm=args.ctas_per_sm, node_budget=args.node_budget,
                     stack_words=args.stack_words, pool_words=args.pool_words, device=local,
                     active_queries=args.active_queries, max_local=args.max_local,
                     prep_ctas=args.prep_ctas)
        if args.arm == "learned":
            eng.load_model(args.model)
        eng.solve([tuple(int(x) for x in r) for r in queries_for(core, 8, 46)])  # warm-up
        pending, lat, res = {}, [], []
        i = 0
        t0 = time.perf_counter()
        cap = args.serve_seconds * 20 + 60
        while len(res) < count:
            now = time.perf_counter() - t0
            if now > cap:
                break
            while i < count and arrive[i] <= now:
                pending[eng.submit(*rows[i])] = (arrive[i], now)
                i += 1
            busy = eng.step()
            for r in eng.poll():
                a, s = pending.pop(r["ticket"])
                lat.append((s - a) + r["latency_ns"] / 1e9)
                res.append(r)
            if not busy and i < count:
                time.sleep(max(0.0, min(arrive[i] - (time.perf_counter() - t0), 0.002)))
        span = time.perf_counter() - t0
        st = eng.stats()
        eng.close()
        lat_ms = np.array(lat) * 1e3 if lat else np.zeros(1)
        line = {"mode": "serve", "metric": METRIC, "unit": UNIT, "n_gpus": 1,
                "offered_qps": rate, "arrivals": count, "completed": len(res),
                "throughput_qps": len(res) / span if span > 0 else None,
                "p50_ms": float(np.percentile(lat_ms, 50)),
                "p99_ms": float(np.percentile(lat_ms, 99)),
                "exact_fraction": sum(1 for r in res if r["status"] in (0, 1)) / max(len(res), 1),
                "verified_fraction": sum(1 for r in res if r["h_verified"]) / max(len(res), 1),
                "data": "synthetic",
                "config": {"workload": WORKLOADS[_WL[0]][1], "arrival_window_s": args.serve_seconds,
                           "node_budget": args.node_budget, "slice_us": args.slice_us or 80000,
                           "active_queries": st["active"], "slots": args.slots or 256,
                           "arm": args.arm if args.arm != "auto" else "plain",
                           "held_by_memory": st["held_memory"],
                           "status_counts": {nm: sum(1 for r in res if r["status"] == k)
                                             for k, nm in ((0, "done"), (1, "heuristic"),
                                                           (2, "capacity"), (3, "timeout"),
                                                           (5, "too_large"))},
                           "engine": {k: st[k] for k in ("nodes", "slices", "prep_ns",
                                                         "search_ns", "heur_ns",
                                                         "device_releases")}}}
        print(json.dumps(line), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=1)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--batch", type=int, default=1000)
    ap.add_argument("--warmup-batch", type=int, default=48)
    ap.add_argument("--node-budget", type=int, default=20000,
                    help="search tasks per query (both arms); the stand-in for the "
                         "reference's level cap")
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="rmat_s15", choices=sorted(WORKLOADS),
                    help="rmat_s15: the mid-size workload (default, the measured one); "
                         "chunglu_n1m: uneven queries on the 1M-vertex Chung-Lu graph; "
                         "rmat_s22: the scale-22 R-MAT serving workload")
    ap.add_argument("--slots", type=int, default=0,
                    help="query slots (0: the batch size, at most 1000)")
    ap.add_argument("--max-local", type=int, default=0,
                    help="largest local graph searched (0: the engine default)")
    ap.add_argument("--arm", default="plain", choices=["auto", "plain", "learned"],
                    help="plain (default, the faster arm on this workload): the integer rules "
                         "alone; learned: u* and an incumbent proposal from the trained "
                         "network; auto: learned when the model exists")
    ap.add_argument("--host-release-only", action="store_true",
                    help="release prepared queries only between slices (no device release)")
    ap.add_argument("--model", default=MODEL, help="model file of the learned arm")
    ap.add_argument("--no-compare", action="store_true",
                    help="skip the other arm's run on the first step's queries")
    ap.add_argument("--ref-sample", type=int, default=4,
                    help="--impl reference: queries of each step timed on the host cores "
                         "(all steps' samples run together)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--ctas-per-sm", type=int, default=0,
                    help="search CTAs per SM (0: autotuned on the warm-up queries)")
    ap.add_argument("--slice-us", type=int, default=0)
    ap.add_argument("--active-queries", type=int, default=0,
                    help="queries searched at once (0: the engine default)")
    ap.add_argument("--release-order", type=int, default=0,
                    help="next prepared query to search: 0 smallest local graph, 1 admission order")
    ap.add_argument("--stack-words", type=int, default=0,
                    help="task-stack words per CTA (0: sized from device memory)")
    ap.add_argument("--pool-words", type=int, default=0)
    ap.add_argument("--prep-ctas", type=int, default=0,
                    help="CTAs per query in preparation (one cluster; 0: the engine's choice)")
    ap.add_argument("--clocks-csv", default=os.path.join(tempfile.gettempdir(), "scs_clocks_r%d.csv"),
                    help="where the nvidia-smi clock samples of the timed region go (%%d: rank)")
    ap.add_argument("--serve", default="",
                    help="serving mode: Poisson arrival rates in queries/s, comma-separated "
                         "(one JSON line per rate, latency measured from arrival)")
    ap.add_argument("--serve-seconds", type=float, default=20.0,
                    help="serving mode: arrival window per rate (seconds)")
    args = ap.parse_args()
    _WL[0] = args.workload
    if args.impl == "reference":
        return run_reference(args)
    if args.serve:
        return run_serve(args)

    import torch
    rank, world, local = env_rank()
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)
    from scs_gb300.engine import Engine

    n, off, adj = build_workload(args.batch, args.warmup, args.steps)
    from scs_gb300.engine import core_numbers
    core = core_numbers(n, off, adj)
    warm = queries_for(core, args.warmup_batch * args.warmup, 43 + 1000 * rank)
    tune = {"ctas_per_sm": args.ctas_per_sm, "slice_us": args.slice_us or 80000,
            "active_queries": args.active_queries, "stack_words": args.stack_words}
    trials = None
    if not args.ctas_per_sm:
        # launch shape chosen by the autotuner on warm-up queries (not timed)
        from scs_gb300.autotune import autotune
        sample = [tuple(int(x) for x in r) for r in warm[: min(len(warm), 64)]]
        tune, trials = autotune(n, off, adj, sample, args.node_budget, device=local)
    eng = Engine(csr=(n, off, adj), limit_queries=args.slots or max(min(args.batch, 1000), 1),
                 slice_us=tune["slice_us"], ctas_per_sm=tune["ctas_per_sm"],
                 node_budget=args.node_budget, stack_words=tune["stack_words"],
                 pool_words=args.pool_words, device=local,
                 active_queries=tune["active_queries"], release_order=args.release_order,
                 max_local=args.max_local, host_release_only=int(args.host_release_only),
                 prep_ctas=args.prep_ctas)
    arm = args.arm
    if arm == "auto":  # the model is trained on the mid-size workload
        arm = "learned" if os.path.exists(args.model) and args.workload == "rmat_s15" else "plain"
    if arm == "learned":
        eng.load_model(args.model)
    # weak scaling: every rank runs the full 1,000-query workload of its own
    # query seed (rank 0 uses the workload's seed 42)
    rows = queries_for(core, args.batch * args.steps, 42 + 1000 * rank)
    flush = torch.empty(64 << 20, dtype=torch.float32, device="cuda")  # 256 MB > L2

    def barrier():
        torch.cuda.synchronize()
        if dist is not None:
            dist.barrier()

    wb = args.warmup_batch
    for i in range(args.warmup):
        eng.solve([tuple(int(x) for x in r) for r in warm[i * wb:(i + 1) * wb]])
    st0 = eng.stats()
    clocks = Clocks(args.clocks_csv % rank if "%d" in args.clocks_csv else args.clocks_csv)
    results, dev_ms, wall = [], 0.0, 0.0
    h2d = d2h = 0
    barrier()
    clocks.start()
    for i in range(args.steps):
        batch = [tuple(int(x) for x in r) for r in rows[i * args.batch:(i + 1) * args.batch]]
        flush_l2(torch, flush)
        barrier()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        t0 = time.perf_counter()
        e0.record()
        res = eng.solve(batch)  # submit from host buffers, run, poll results
        e1.record()
        torch.cuda.synchronize()
        wall += time.perf_counter() - t0
        dev_ms += e0.elapsed_time(e1)
        results += res
    barrier()
    ck = clocks.stop(local)
    st1 = eng.stats()
    compare = None
    if not args.no_compare and (arm == "learned" or os.path.exists(args.model)):
        # the other arm on the first step's queries (after the timed region)
        other = "plain" if arm == "learned" else "learned"
        eng.load_model(args.model if other == "learned" else None)
        batch = [tuple(int(x) for x in r) for r in rows[: args.batch]]
        flush_l2(torch, flush)
        torch.cuda.synchronize()
        s0 = eng.stats()
        t0 = time.perf_counter()
        oth = eng.solve(batch)
        dt = time.perf_counter() - t0
        s1 = eng.stats()
        mine = results[: args.batch]
        ex = lambda r: r["status"] in (0, 1)
        both = [(a, b) for a, b in zip(mine, oth) if ex(a) and ex(b)]
        lat_o = np.array([r["latency_ns"] for r in oth]) / 1e6
        compare = {"arm": other, "queries": len(oth), "seconds": dt,
                   "exact_per_s": sum(1 for r in oth if ex(r)) / dt,
                   "all_answers_per_s": len(oth) / dt,
                   "exact_fraction": sum(1 for r in oth if ex(r)) / max(len(oth), 1),
                   "p50_ms": float(np.percentile(lat_o, 50)),
                   "p99_ms": float(np.percentile(lat_o, 99)),
                   "nodes": s1["nodes"] - s0["nodes"],
                   "this_arm_exact_on_these": sum(1 for r in mine if ex(r)),
                   "both_exact": len(both),
                   "same_degree_where_both_exact": sum(1 for a, b in both
                                                       if a["degree"] == b["degree"]),
                   "degree_differs_anywhere_exact": sum(
                       1 for a, b in zip(mine, oth) if ex(a) and ex(b) and a["degree"] != b["degree"])}
    # max of the times over ranks, sum of the queries
    t_dev, wall, total_q = reduce_over_ranks(dist, torch, dev_ms / 1e3, wall, len(results),
                                             "cuda")
    lat = np.array([r["latency_ns"] for r in results]) / 1e6
    exact = sum(1 for r in results if r["status"] in (0, 1))
    exact_all = exact
    if dist is not None:
        ex = torch.tensor([float(exact)], dtype=torch.float64, device="cuda")
        dist.all_reduce(ex)
        exact_all = int(ex[0])
    verified = sum(1 for r in results if r["h_verified"])
    search_ns = st1["search_ns"] - st0["search_ns"]
    nbytes = st1["bytes"] - st0["bytes"]
    launches = st1["launches"] - st0["launches"]
    slices = st1["slices"] - st0["slices"]
    peak, peak_kind = measured_peak_gbs()
    achieved = (nbytes / (search_ns / 1e9) / 1e9) if search_ns else 0.0
    # DRAM bytes per search launch: the DRAM rate an ncu capture measured on
    # search slices of this same configuration (workload, budget, launch
    # shape, task store, release mode, arm), times this run's mean launch
    # time.  No capture of the configuration: null.
    traffic, traffic_src = None, None
    tp = os.path.join(ROOT, "profiles", "search_traffic_%s.json" % args.workload)
    if os.path.exists(tp) and slices:
        try:
            prof = json.load(open(tp))
            # the slice length only scales the launch; the DRAM rate per ms is
            # what the capture measured, so it is not matched
            want = {"node_budget": args.node_budget, "ctas_per_sm": tune["ctas_per_sm"],
                    "active_queries": st1["active"], "arm": arm,
                    "stack_words": tune["stack_words"], "pool_words": args.pool_words,
                    "host_release_only": bool(args.host_release_only)}
            if all(prof["config"].get(k) == v for k, v in want.items()):
                traffic = float(prof["dram_bytes_per_ms"]) * (search_ns / 1e6) / slices
                traffic_src = os.path.relpath(tp, ROOT)
        except Exception:
            traffic = None
    line = {
        "metric": METRIC, "value": exact_all / t_dev, "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 * t_dev / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u32",
        "data": "synthetic",
        "config": {"workload": WORKLOADS[_WL[0]][1], "graph": WORKLOADS[_WL[0]][2],
                   "queries": total_q, "exact_answers": exact_all,
                   "all_answers_per_s": total_q / t_dev,
                   "batch": args.batch, "node_budget": args.node_budget,
                   "l2": "flushed between steps (256 MB write)",
                   "exact_fraction": exact / max(len(results), 1),
                   "verified_fraction": verified / max(len(results), 1),
                   "status_counts": {nm: sum(1 for r in results if r["status"] == st)
                                     for st, nm in ((0, "done"), (1, "heuristic"), (2, "capacity"),
                                                    (3, "timeout"), (4, "bad_query"),
                                                    (5, "too_large"))},
                   "p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
                   "nodes": st1["nodes"] - st0["nodes"], "parallelism": "replicas" if world > 1 else "1 GPU",
                   "ctas_per_sm": tune["ctas_per_sm"],
                   "resident_ctas": st1["ctas"], "smem_state_words": st1["smem_words"],
                   "active_queries": st1["active"],
                   "slice_us": tune["slice_us"], "stack_words": tune["stack_words"],
                   "autotune_trials": trials,
                   "arm": arm, "model": os.path.relpath(args.model, ROOT) if arm == "learned" else None,
                   "proposals_better": st1["proposals_better"] - st0["proposals_better"],
                   "device_releases": st1["device_releases"] - st0["device_releases"],
                   "host_release_only": bool(args.host_release_only),
                   # engine time over the timed steps: preparation launches,
                   # search slices, and admission waiting on host incumbents
                   # with nothing searching
                   "engine_ms": {k: (st1[k + "_ns"] - st0[k + "_ns"]) / 1e6
                                 for k in ("prep", "search", "heur")},
                   "compare": compare},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak if peak else None, "traffic": traffic,
                     "traffic_source": traffic_src,
                     "peak_kind": peak_kind, "kernel": "search_kernel",
                     "launches": slices,
                     "algorithmic_bytes_per_launch": nbytes / max(slices, 1),
                     "mean_launch_ms": search_ns / 1e6 / max(slices, 1)},
        "e2e": {"value": exact_all / wall, "unit": UNIT, "all_answers_per_s": total_q / wall,
                "h2d_bytes_per_step": (st1["h2d_bytes"] - st0["h2d_bytes"]) // max(args.steps, 1)
                + 20 * args.batch,
                "d2h_bytes_per_step": (st1["d2h_bytes"] - st0["d2h_bytes"]) // max(args.steps, 1)},
        "gpu_launches": launches,
        "clocks": ck,
    }
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        # one query per host core from the start of the step, same budget,
        # no wall-clock cap (one wave: about a budget-stopped query's time)
        procs = os.cpu_count() or 1
        r = cpu_baseline(n, off, adj, rows[: min(procs, len(rows))], args.node_budget, procs=procs)
        line["cpu_baseline"] = {"value": r["exact"] / r["span_s"] if r["span_s"] > 0 else 0.0,
                                "unit": UNIT, "cores": r["procs"], "kind": "port",
                                "sample": _cpu_desc(r, args.node_budget), **host_cpu_info()}
    eng.close()
    if rank == 0:
        print(json.dumps(line))
    if dist is not None:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
