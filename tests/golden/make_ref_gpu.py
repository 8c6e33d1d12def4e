"""Record the reference's own GPU answers as golden fixtures (run on a GPU
machine from the repo root; test-fixture generator, not product code).

The reference server (``oracle/_ref/scs_ref_server``: the reference's
``main.cu`` compiled unchanged by ``oracle/build_ref.py``) is started once
per query and per repeat, with one query slot (``limitQueries = 1``), so its
global level counter (``main.cu:15,421,444``: never reset, 4000 levels in all)
and its stop-on-overflow (``main.cu:340-360``) apply to that query alone.
The query and ``server_exit`` go through the reference's own SysV queue
(key ``ftok("/tmp", 'g')``, mtype 1, ``ipc/msgtool.h``); its answer is the
row it appends to ``results/results_<graph file>`` (``main.cu:124-128,
328-333, 348-352, 451-454``).  Each run gets its own working folder and, when
``unshare --ipc`` is available, its own IPC namespace, so several servers can
share the GPU at once; otherwise the runs go one after another.

Every run has a wall-clock limit; a server still running at the limit is
killed and its query recorded without an answer.

Output: ``ref_gpu_<workload>.json`` with, per query, the rows of all repeats
(degree, Overtime, Heu, time in microseconds).  The reference is not
deterministic (task layouts follow atomic order; its dominance test depends
on row order, src/helpers.cc:615-621), so the fixture keeps every repeat.

Usage: python tests/golden/make_ref_gpu.py <workload> <count> <repeats>
           [--jobs J] [--timeout S] [--out DIR] [--server PATH]
"""
import argparse
import ctypes as C
import json
import os
import shutil
import signal
import subprocess
import sys
import tempfile
import threading
import time

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
HERE = os.path.dirname(os.path.abspath(__file__))

# Server arguments (main.cu:476-502): partition size per warp, buffer size,
# copy limit, read limit, query slots, factor, red1 red2 red3 prun1 prun2.
# The README's run line with one query slot, a partition large enough for any
# filtered graph of the mid-size workload (n = 32,768) and a larger overflow
# buffer.
SERVER_ARGS = ["40000", "20000000", "0.5", "1", "1", "100", "1", "1", "1", "1", "1"]

IPC_CREAT = 0o1000
IPC_RMID = 0


class _Msg(C.Structure):
    _fields_ = [("mtype", C.c_long), ("mtext", C.c_char * 80)]


def _libc():
    lc = C.CDLL(None, use_errno=True)
    lc.ftok.argtypes = [C.c_char_p, C.c_int]
    lc.ftok.restype = C.c_int
    lc.msgget.argtypes = [C.c_int, C.c_int]
    lc.msgsnd.argtypes = [C.c_int, C.c_void_p, C.c_size_t, C.c_int]
    lc.msgctl.argtypes = [C.c_int, C.c_int, C.c_void_p]
    return lc


def _send(lc, qid, text):
    m = _Msg()
    m.mtype = 1
    m.mtext = text.encode()
    if lc.msgsnd(qid, C.byref(m), len(text) + 1, 0) != 0:
        raise OSError(C.get_errno(), "msgsnd failed")


def _parse_rows(path):
    rows = []
    if not os.path.exists(path):
        return rows
    for line in open(path):
        p = line.strip().split("|")
        if len(p) < 7 or p[0] in ("N1", "-1"):
            continue
        rows.append({"l": int(p[0]), "h": int(p[1]), "q": int(p[2]),
                     "time_us": int(p[3].replace(",", "")), "degree": int(p[4]),
                     "overtime": int(p[5]), "heu": int(p[6])})
    return rows


def run_one(server, graph, row, timeout):
    """One query on a fresh server in a fresh working folder (this process's
    IPC namespace).  Returns the run record."""
    l, h, q, hf, ld = row
    lc = _libc()
    work = tempfile.mkdtemp(prefix="scs_refrun_")
    try:
        os.makedirs(os.path.join(work, "results"))
        gname = os.path.basename(graph)
        os.symlink(os.path.abspath(graph), os.path.join(work, gname))
        key = lc.ftok(b"/tmp", ord("g"))
        old = lc.msgget(key, 0)
        if old >= 0:  # a queue left by an earlier server in this namespace
            lc.msgctl(old, IPC_RMID, None)
        log = open(os.path.join(work, "server.log"), "w")
        t0 = time.time()
        proc = subprocess.Popen([server, gname] + SERVER_ARGS, cwd=work, stdout=log,
                                stderr=subprocess.STDOUT, start_new_session=True)
        qid = lc.msgget(key, IPC_CREAT | 0o660)
        if qid < 0:
            raise OSError(C.get_errno(), "msgget failed")
        _send(lc, qid, "%d %d %d %d %d" % (l, h, q, hf, ld))
        _send(lc, qid, "server_exit")
        status = "exited"
        try:
            rc = proc.wait(timeout=timeout)
        except subprocess.TimeoutExpired:
            os.killpg(proc.pid, signal.SIGTERM)
            try:
                rc = proc.wait(timeout=30)
            except subprocess.TimeoutExpired:
                os.killpg(proc.pid, signal.SIGKILL)
                rc = proc.wait()
            status = "killed at the wall-clock limit"
        wall = time.time() - t0
        log.close()
        got = [r for r in _parse_rows(os.path.join(work, "results", "results_" + gname))
               if r["q"] == q]
        tail = open(os.path.join(work, "server.log"), errors="replace").read()[-400:]
        rec = {"rc": rc, "status": status, "wall_s": round(wall, 3)}
        if got:
            rec.update({k: got[-1][k] for k in ("degree", "overtime", "heu", "time_us")})
        else:
            rec["degree"] = None
            rec["log_tail"] = tail
        return rec
    finally:
        shutil.rmtree(work, ignore_errors=True)


def _have_unshare():
    try:
        return subprocess.run(["unshare", "--ipc", "true"], capture_output=True,
                              timeout=30).returncode == 0
    except Exception:
        return False


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("workload", nargs="?")
    ap.add_argument("count", nargs="?", type=int)
    ap.add_argument("repeats", nargs="?", type=int, default=3)
    ap.add_argument("--jobs", type=int, default=4)
    ap.add_argument("--timeout", type=float, default=240.0)
    ap.add_argument("--out", default=HERE)
    ap.add_argument("--server", default=os.path.join(ROOT, "oracle", "_ref", "scs_ref_server"))
    ap.add_argument("--one", default="", help=argparse.SUPPRESS)
    a = ap.parse_args()
    if a.one:  # child mode: one run, record on stdout
        spec = json.loads(a.one)
        print(json.dumps(run_one(spec["server"], spec["graph"], spec["row"], spec["timeout"])))
        return 0
    from scs_gb300 import workloads as W
    sys.path.insert(0, HERE)
    from make_golden import graph_sum
    gb, qb = W.WORKLOADS[a.workload]
    n, u, v = gb()
    off, adj = W.to_csr(n, u, v)
    from scs_gb300.engine import core_numbers
    core = core_numbers(n, off, adj)
    rows = [tuple(int(x) for x in r) for r in qb(core)[: a.count]]
    tmp = tempfile.mkdtemp(prefix="scs_refgraph_")
    graph = W.write_edgelist(os.path.join(tmp, a.workload + ".txt"), n, u, v)
    iso = _have_unshare()
    jobs = a.jobs if iso else 1
    work = [(i, r) for r in range(a.repeats) for i in range(len(rows))]
    out = [[None] * a.repeats for _ in rows]
    lock = threading.Lock()
    t_start = time.time()

    def worker():
        while True:
            with lock:
                if not work:
                    return
                i, r = work.pop(0)
            spec = json.dumps({"server": a.server, "graph": graph, "row": rows[i],
                               "timeout": a.timeout})
            cmd = ([sys.executable, os.path.abspath(__file__), "--one", spec])
            if iso:
                cmd = ["unshare", "--ipc"] + cmd
            p = subprocess.run(cmd, capture_output=True, text=True, timeout=a.timeout + 120)
            try:
                rec = json.loads(p.stdout.strip().splitlines()[-1])
            except Exception:
                rec = {"degree": None, "status": "runner failed", "stderr": p.stderr[-400:]}
            with lock:
                out[i][r] = rec
                print("query %d repeat %d: %s" % (i, r, json.dumps(rec)), flush=True)

    ths = [threading.Thread(target=worker) for _ in range(jobs)]
    for t in ths:
        t.start()
    for t in ths:
        t.join()
    doc = {"workload": a.workload, "checksum": graph_sum(off, adj), "server_args": SERVER_ARGS,
           "repeats": a.repeats, "isolated_ipc": iso, "jobs": jobs,
           "wall_s": round(time.time() - t_start, 1),
           "queries": [{"l": r[0], "h": r[1], "q": r[2], "heur": r[3], "limit_doms": r[4],
                        "runs": out[i]} for i, r in enumerate(rows)]}
    os.makedirs(a.out, exist_ok=True)
    path = os.path.join(a.out, "ref_gpu_%s.json" % a.workload)
    with open(path, "w") as f:
        json.dump(doc, f, indent=0)
    print("wrote", path)
    shutil.rmtree(tmp, ignore_errors=True)
    return 0


if __name__ == "__main__":
    sys.exit(main())
