"""ctypes binding of the engine's C ABI (include/scs.h).

The host-side mirror of the reference's server surface: queries are the
reference's message fields ``(l, h, q, heuristic_flag, limit_dominating_set)``
(main.cu:92-119) and results carry the Degree column plus the status codes
that stand in for its Heu / Overtime columns (main.cu:122-133, 317-360,
444-463).  There is no CPU fallback: every call goes to libscs.so and raises
when the library or the GPU is missing.
"""
import ctypes as C
import os

import numpy as np

from . import build as _build

_u32p = C.POINTER(C.c_uint32)
_u64p = C.POINTER(C.c_uint64)

DONE, HEURISTIC, CAPACITY, TIMEOUT, BAD_QUERY, TOO_LARGE = range(6)
STATUS_NAMES = {DONE: "done", HEURISTIC: "heuristic", CAPACITY: "capacity",
                TIMEOUT: "timeout", BAD_QUERY: "bad_query", TOO_LARGE: "too_large"}

STAT_NAMES = ["nodes", "slices", "donations", "steals", "spills", "bytes",
              "prep_bytes", "search_ns", "prep_ns", "launches", "h2d_bytes",
              "d2h_bytes", "heur_ns", "ctas", "smem_words", "errors", "active",
              "releases", "slides", "proposals_better", "held_memory", "pool_free",
              "device_releases"]


class Config(C.Structure):
    _fields_ = [("limit_queries", C.c_uint32), ("red1", C.c_uint32),
                ("red2", C.c_uint32), ("red3", C.c_uint32),
                ("prun1", C.c_uint32), ("prun2", C.c_uint32),
                ("rules_set", C.c_uint32), ("ctas_per_sm", C.c_uint32),
                ("threads_per_cta", C.c_uint32), ("stack_words", C.c_uint64),
                ("pool_words", C.c_uint64), ("slice_us", C.c_uint32),
                ("node_budget", C.c_uint64), ("host_threads", C.c_uint32),
                ("device", C.c_int32), ("active_queries", C.c_uint32),
                ("release_order", C.c_uint32), ("release_headroom", C.c_uint32),
                ("max_local", C.c_uint32), ("host_release_only", C.c_uint32),
                ("prep_ctas", C.c_uint32), ("prep_big_row", C.c_uint32)]


class Query(C.Structure):
    _fields_ = [("l", C.c_uint32), ("h", C.c_uint32), ("q", C.c_uint32),
                ("heuristic", C.c_uint32), ("limit_doms", C.c_uint32)]


class Result(C.Structure):
    _fields_ = [("ticket", C.c_uint64), ("l", C.c_uint32), ("h", C.c_uint32),
                ("q", C.c_uint32), ("degree", C.c_uint32),
                ("status", C.c_int32), ("kl_heuristic", C.c_uint32),
                ("h_size", C.c_uint32), ("h_verified", C.c_uint32),
                ("nodes", C.c_uint64), ("latency_ns", C.c_uint64),
                ("search_ns", C.c_uint64)]


class SCSError(RuntimeError):
    pass


class MlpTrainCfg(C.Structure):
    _fields_ = [("epochs", C.c_uint32), ("batch", C.c_uint32), ("lr", C.c_float),
                ("weight_decay", C.c_float), ("seed", C.c_uint64)]


MLP_NPARAM = 18817
MLP_IN = 16


def _fp(a):
    return a.ctypes.data_as(C.POINTER(C.c_float))


def _mlp_check(rc, what):
    if rc < 0:
        raise SCSError("%s failed (%d): %s" % (what, rc, lib().scs_mlp_last_error().decode()))
    return rc


def mlp_train(X, y, params, w=None, epochs=20, batch=4096, lr=1e-3, weight_decay=0.0,
              seed=0, device=0):
    """Train on the GPU with the engine's own kernels; returns (params,
    per-epoch mean loss)."""
    X = np.ascontiguousarray(X, dtype=np.float32)
    y = np.ascontiguousarray(y, dtype=np.float32)
    p = np.ascontiguousarray(params, dtype=np.float32).copy()
    assert X.shape[1] == MLP_IN and p.size == MLP_NPARAM
    wa = None if w is None else np.ascontiguousarray(w, dtype=np.float32)
    cfg = MlpTrainCfg(epochs, batch, lr, weight_decay, seed)
    losses = np.zeros(epochs, dtype=np.float32)
    _mlp_check(lib().scs_mlp_train(_fp(X), _fp(y), None if wa is None else _fp(wa), len(y),
                                   C.byref(cfg), _fp(p), _fp(losses), device), "scs_mlp_train")
    return p, losses


def mlp_grad(params, X, y, w=None, device=0):
    """(loss, gradient) of one batch computed by the GPU training kernels."""
    X = np.ascontiguousarray(X, dtype=np.float32)
    y = np.ascontiguousarray(y, dtype=np.float32)
    p = np.ascontiguousarray(params, dtype=np.float32)
    wa = None if w is None else np.ascontiguousarray(w, dtype=np.float32)
    g = np.zeros(MLP_NPARAM, dtype=np.float32)
    loss = C.c_double()
    _mlp_check(lib().scs_mlp_grad(_fp(p), _fp(X), _fp(y), None if wa is None else _fp(wa),
                                  len(y), C.byref(loss), _fp(g), device), "scs_mlp_grad")
    return loss.value, g


def mlp_infer(params, X, device=0):
    """Logits of the rows of X by the tensor-core BF16 inference path."""
    X = np.ascontiguousarray(X, dtype=np.float32)
    p = np.ascontiguousarray(params, dtype=np.float32)
    out = np.zeros(len(X), dtype=np.float32)
    _mlp_check(lib().scs_mlp_infer(_fp(p), _fp(X), len(X), _fp(out), device), "scs_mlp_infer")
    return out


def save_model(path, params):
    """Write a model file scs_load_model reads."""
    p = np.ascontiguousarray(params, dtype=np.float32)
    assert p.size == MLP_NPARAM
    with open(path, "wb") as f:
        f.write(b"SCSMLP01")
        f.write(np.array([16, 128, 128, 1], dtype=np.uint32).tobytes())
        f.write(p.tobytes())


def load_model_file(path):
    raw = open(path, "rb").read()
    assert raw[:8] == b"SCSMLP01"
    dims = np.frombuffer(raw[8:24], dtype=np.uint32)
    assert list(dims) == [16, 128, 128, 1]
    return np.frombuffer(raw[24:24 + 4 * MLP_NPARAM], dtype=np.float32).copy()


_lib = None


def lib(build_if_missing=False):
    """Load libscs.so (built in-tree).  Raises if it is missing."""
    global _lib
    if _lib is not None:
        return _lib
    path = _build.lib_path()
    if not os.path.exists(path):
        if not build_if_missing:
            raise SCSError("libscs.so is not built (run __graft_entry__.build())")
        _build.build()
    L = C.CDLL(path)
    vp = C.c_void_p
    L.scs_create.argtypes = [C.POINTER(vp), C.c_char_p, C.POINTER(Config)]
    L.scs_create_csr.argtypes = [C.POINTER(vp), C.c_uint32, _u32p, _u32p, C.POINTER(Config)]
    L.scs_graph_info.argtypes = [vp, _u32p, _u64p, _u32p]
    L.scs_core_numbers.argtypes = [vp, _u32p]
    L.scs_submit.argtypes = [vp, C.POINTER(Query), _u64p]
    L.scs_step.argtypes = [vp]
    L.scs_run.argtypes = [vp]
    L.scs_poll.argtypes = [vp, C.POINTER(Result), C.c_int, _u32p, C.c_uint32]
    L.scs_stats.argtypes = [vp, _u64p]
    L.scs_profile.argtypes = [vp, _u64p]
    L.scs_last_error.argtypes = [vp]
    L.scs_last_error.restype = C.c_char_p
    L.scs_destroy.argtypes = [vp]
    L.scs_read_edge_list.argtypes = [C.c_char_p, _u32p, _u64p, C.POINTER(_u32p), C.POINTER(_u32p)]
    L.scs_free.argtypes = [vp]
    L.scs_core_decompose.argtypes = [C.c_uint32, _u32p, _u32p, _u32p]
    L.scs_core_decompose_gpu.argtypes = [C.c_uint32, _u32p, _u32p, _u32p, C.c_int]
    L.scs_greedy_incumbent.argtypes = [C.c_uint32, _u32p, _u32p, C.c_uint32, C.c_uint32,
                                       C.c_uint32, _u32p, _u32p, _u32p]
    L.scs_distance_bound.argtypes = [C.c_uint32, C.c_uint32]
    L.scs_distance_bound.restype = C.c_uint32
    L.scs_abi_layout.argtypes = [_u64p, C.c_int]
    L.scs_check_community.argtypes = [C.c_uint32, _u32p, _u32p, _u32p, C.c_uint32, C.c_uint32,
                                      C.c_uint32, C.c_uint32, _u32p]
    L.scs_local_graph_noalloc.argtypes = [vp, vp, vp, C.c_uint32, C.c_uint32, C.c_uint32,
                                          C.c_uint32, C.c_uint32, vp, vp, vp, vp,
                                          C.c_uint64, vp, vp]
    L.scs_debug_prepare.argtypes = [vp, C.c_uint32, C.POINTER(Query), _u32p, _u32p, _u32p, _u32p]
    L.scs_debug_local_graph.argtypes = [vp, C.c_uint32, _u32p, _u32p, _u32p, _u32p]
    L.scs_debug_step.argtypes = [vp, C.c_uint32, _u32p, _u32p, _u64p, _u32p, _u32p,
                                 _u32p, _u32p, C.c_uint32, _u32p, C.c_uint64, _u32p,
                                 C.c_uint32, _u32p, _u32p, C.POINTER(C.c_float)]
    L.scs_debug_lookahead.argtypes = [vp, C.c_uint32, _u32p, _u32p, _u64p, _u32p, _u32p,
                                      _u32p, _u32p, _u32p, _u32p, _u64p]
    fp = C.POINTER(C.c_float)
    L.scs_load_model.argtypes = [vp, C.c_char_p]
    L.scs_trace_enable.argtypes = [vp, C.c_uint64, C.c_uint32]
    L.scs_trace_read.argtypes = [vp, fp, _u32p, C.c_uint64, _u64p]
    L.scs_mlp_train.argtypes = [fp, fp, fp, C.c_uint64, C.POINTER(MlpTrainCfg), fp, fp, C.c_int]
    L.scs_mlp_grad.argtypes = [fp, fp, fp, fp, C.c_uint64, C.POINTER(C.c_double), fp, C.c_int]
    L.scs_mlp_infer.argtypes = [fp, fp, C.c_uint64, fp, C.c_int]
    L.scs_mlp_last_error.restype = C.c_char_p
    _lib = L
    return L


def _p(a):
    return a.ctypes.data_as(_u32p)


def exported_symbols():
    """Names declared in include/scs.h (parsed from the header)."""
    import re
    hdr = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))),
                       "include", "scs.h")
    text = open(hdr).read()
    return sorted(set(re.findall(r"\b(scs_[a-z_]+)\s*\(", text)))


# ---------------------------------------------------------------------------
# host-only utilities
# ---------------------------------------------------------------------------

def read_edge_list(path):
    n = C.c_uint32()
    nnz = C.c_uint64()
    off = _u32p()
    adj = _u32p()
    rc = lib().scs_read_edge_list(path.encode(), C.byref(n), C.byref(nnz),
                                  C.byref(off), C.byref(adj))
    if rc:
        raise SCSError("scs_read_edge_list failed (%d)" % rc)
    o = np.ctypeslib.as_array(off, shape=(n.value + 1,)).copy()
    a = np.ctypeslib.as_array(adj, shape=(max(nnz.value, 1),))[: nnz.value].copy()
    lib().scs_free(C.cast(off, C.c_void_p))
    lib().scs_free(C.cast(adj, C.c_void_p))
    return n.value, o, a


def core_numbers(n, off, adj):
    off = np.ascontiguousarray(off, dtype=np.uint32)
    adj = np.ascontiguousarray(adj, dtype=np.uint32)
    core = np.zeros(n, dtype=np.uint32)
    rc = lib().scs_core_decompose(n, _p(off), _p(adj), _p(core))
    if rc:
        raise SCSError("scs_core_decompose failed (%d)" % rc)
    return core


def core_numbers_gpu(n, off, adj, device=0):
    """Core numbers by GPU peeling (scs_core_decompose_gpu); equal to
    core_numbers()."""
    off = np.ascontiguousarray(off, dtype=np.uint32)
    adj = np.ascontiguousarray(adj, dtype=np.uint32)
    core = np.zeros(max(n, 1), dtype=np.uint32)
    rc = lib().scs_core_decompose_gpu(n, _p(off), _p(adj) if len(adj) else None, _p(core), device)
    if rc:
        raise SCSError("scs_core_decompose_gpu failed (%d)" % rc)
    return core[:n]


def greedy_incumbent(n, off, adj, l, h, q):
    off = np.ascontiguousarray(off, dtype=np.uint32)
    adj = np.ascontiguousarray(adj, dtype=np.uint32)
    deg = int(off[q + 1] - off[q])
    H = np.zeros(max(h, deg + 1, 1), dtype=np.uint32)
    kl = C.c_uint32()
    hs = C.c_uint32()
    rc = lib().scs_greedy_incumbent(n, _p(off), _p(adj), l, h, q, C.byref(kl), _p(H), C.byref(hs))
    if rc:
        raise SCSError("scs_greedy_incumbent failed (%d)" % rc)
    return kl.value, H[: hs.value].copy()


def distance_bound(kl, h):
    return int(lib().scs_distance_bound(kl, h))


CHECK_REASONS = {0: "ok", 1: "empty", 2: "id out of range", 3: "repeated id",
                 4: "query vertex missing", 5: "size outside [l, h]", 6: "not connected"}


def check_community(n, off, adj, H, q, l, h):
    """(code, min degree) of community H for query (l, h, q); code 0 = valid
    (ids in range and distinct, q in H, l <= |H| <= h, connected)."""
    off = np.ascontiguousarray(off, dtype=np.uint32)
    adj = np.ascontiguousarray(adj, dtype=np.uint32)
    H = np.ascontiguousarray(H, dtype=np.uint32)
    md = C.c_uint32()
    rc = lib().scs_check_community(n, _p(off), _p(adj), _p(H) if len(H) else None, len(H),
                                   q, l, h, C.byref(md))
    if rc < 0:
        raise SCSError("scs_check_community failed (%d)" % rc)
    return rc, md.value


NOALLOC_MAX_N = 1 << 19


def local_graph_noalloc(d_off, d_adj, d_core, n, dmax, q, kl, ubd, d_gid, d_dist,
                        d_loc_off, d_loc_adj, loc_adj_cap, d_info, stream=0):
    """Allocation-free local-graph build (device pointers as ints); see
    scs_local_graph_noalloc in include/scs.h."""
    rc = lib().scs_local_graph_noalloc(d_off, d_adj, d_core, n, dmax, q, kl, ubd, d_gid,
                                       d_dist, d_loc_off, d_loc_adj, loc_adj_cap, d_info,
                                       stream)
    if rc:
        raise SCSError("scs_local_graph_noalloc failed (%d)" % rc)


# ---------------------------------------------------------------------------
# engine
# ---------------------------------------------------------------------------

class Engine:
    """One engine on one GPU.  Mirrors the reference server: a resident graph,
    query slots (limit_queries), rule switches red1..prun2."""

    def __init__(self, graph=None, csr=None, limit_queries=64, rules=None,
                 slice_us=0, node_budget=0, ctas_per_sm=0, stack_words=0,
                 pool_words=0, host_threads=0, device=0, active_queries=0,
                 release_order=0, release_headroom=0, max_local=0, host_release_only=0,
                 prep_ctas=0, prep_big_row=0):
        L = lib()
        cfg = Config()
        cfg.limit_queries = limit_queries
        cfg.slice_us = slice_us
        cfg.node_budget = node_budget
        cfg.ctas_per_sm = ctas_per_sm
        cfg.stack_words = stack_words
        cfg.pool_words = pool_words
        cfg.host_threads = host_threads
        cfg.device = device
        cfg.active_queries = active_queries
        cfg.release_order = release_order
        cfg.release_headroom = release_headroom
        cfg.max_local = max_local
        cfg.host_release_only = host_release_only
        cfg.prep_ctas = prep_ctas
        cfg.prep_big_row = prep_big_row
        if rules is not None:
            cfg.rules_set = 1
            cfg.red1, cfg.red2, cfg.red3, cfg.prun1, cfg.prun2 = [int(bool(r)) for r in rules]
        self._h = C.c_void_p()
        if graph is not None:
            rc = L.scs_create(C.byref(self._h), graph.encode(), C.byref(cfg))
        else:
            n, off, adj = csr
            self._off = np.ascontiguousarray(off, dtype=np.uint32)
            self._adj = np.ascontiguousarray(adj, dtype=np.uint32)
            rc = L.scs_create_csr(C.byref(self._h), n, _p(self._off), _p(self._adj), C.byref(cfg))
        if rc:
            raise SCSError("scs_create failed (%d): %s" % (rc, L.scs_last_error(None).decode()))
        n = C.c_uint32()
        nnz = C.c_uint64()
        dmax = C.c_uint32()
        L.scs_graph_info(self._h, C.byref(n), C.byref(nnz), C.byref(dmax))
        self.n, self.nnz, self.dmax = n.value, nnz.value, dmax.value

    def _check(self, rc, what):
        if rc < 0:
            raise SCSError("%s failed (%d): %s" % (what, rc, lib().scs_last_error(self._h).decode()))
        return rc

    def core_numbers(self):
        out = np.zeros(self.n, dtype=np.uint32)
        self._check(lib().scs_core_numbers(self._h, _p(out)), "scs_core_numbers")
        return out

    def submit(self, l, h, q, heuristic=1, limit_doms=10):
        qq = Query(int(l), int(h), int(q), int(heuristic), int(limit_doms))
        t = C.c_uint64()
        self._check(lib().scs_submit(self._h, C.byref(qq), C.byref(t)), "scs_submit")
        return t.value

    def submit_many(self, rows):
        return [self.submit(*r) for r in rows]

    def step(self):
        return self._check(lib().scs_step(self._h), "scs_step")

    def run(self):
        self._check(lib().scs_run(self._h), "scs_run")

    def poll(self, max_results=4096, h_stride=512):
        res = (Result * max_results)()
        hb = np.zeros(max_results * h_stride, dtype=np.uint32)
        k = self._check(lib().scs_poll(self._h, res, max_results, _p(hb), h_stride), "scs_poll")
        out = []
        for i in range(k):
            r = res[i]
            out.append(dict(ticket=r.ticket, l=r.l, h=r.h, q=r.q, degree=r.degree,
                            status=r.status, kl_heuristic=r.kl_heuristic,
                            h_verified=r.h_verified, nodes=r.nodes,
                            latency_ns=r.latency_ns, search_ns=r.search_ns,
                            H=hb[i * h_stride: i * h_stride + min(r.h_size, h_stride)].copy()))
        return out

    def solve(self, rows):
        """Submit rows of (l, h, q, heuristic, limit_doms), run to completion
        and return results ordered like the input."""
        tickets = self.submit_many(rows)
        self.run()
        got = {}
        while True:
            rs = self.poll()
            if not rs:
                break
            for r in rs:
                got[r["ticket"]] = r
        return [got[t] for t in tickets]

    def load_model(self, path):
        """Use the network in model file `path` to pick branching vertices
        (None: back to the plain method)."""
        self._check(lib().scs_load_model(self._h, None if path is None else path.encode()),
                    "scs_load_model")

    def trace_enable(self, max_records, sample_shift=0):
        self._check(lib().scs_trace_enable(self._h, max_records, sample_shift),
                    "scs_trace_enable")
        self._trace_cap = max_records

    def trace_read(self):
        """(features[k][16], keys[k][2] = (query tag, global vertex), records
        produced incl. dropped ones)."""
        cap = getattr(self, "_trace_cap", 0)
        f = np.zeros((max(cap, 1), MLP_IN), dtype=np.float32)
        k = np.zeros((max(cap, 1), 2), dtype=np.uint32)
        w = C.c_uint64()
        n = self._check(lib().scs_trace_read(self._h, _fp(f), _p(k), cap, C.byref(w)),
                        "scs_trace_read")
        return f[:n], k[:n], w.value

    def stats(self):
        arr = (C.c_uint64 * 24)()
        self._check(lib().scs_stats(self._h, arr), "scs_stats")
        return {name: int(arr[i]) for i, name in enumerate(STAT_NAMES)}

    def profile(self):
        arr = (C.c_uint64 * 16)()
        self._check(lib().scs_profile(self._h, arr), "scs_profile")
        names = ["load", "mindeg_rule3", "rules12", "bounds", "ustar", "doms", "children",
                 "other", "r12_rounds", "r3_rounds", "steps", "sub_cycles0", "sub_cycles1",
                 "sub_cycles2", "sub_count0", "sub_count1"]
        return {nm: int(arr[i]) for i, nm in enumerate(names)}

    # ---- test hooks ----
    def debug_prepare(self, queries, kls, ubds):
        nq = len(queries)
        qs = (Query * nq)(*[Query(*[int(x) for x in q]) for q in queries])
        kl = np.ascontiguousarray(kls, dtype=np.uint32)
        ub = np.ascontiguousarray(ubds, dtype=np.uint32)
        nl = np.zeros(nq, dtype=np.uint32)
        ql = np.zeros(nq, dtype=np.uint32)
        self._check(lib().scs_debug_prepare(self._h, nq, qs, _p(kl), _p(ub), _p(nl), _p(ql)),
                    "scs_debug_prepare")
        return nl, ql

    def debug_local_graph(self, slot, n_local, nnz_cap):
        gid = np.zeros(max(n_local, 1), dtype=np.uint32)
        off = np.zeros(n_local + 1, dtype=np.uint32)
        adj = np.zeros(max(nnz_cap, 1), dtype=np.uint32)
        dist = np.zeros(max(n_local, 1), dtype=np.uint32)
        self._check(lib().scs_debug_local_graph(self._h, slot, _p(gid), _p(off), _p(adj), _p(dist)),
                    "scs_debug_local_graph")
        return gid[:n_local], off, adj[: off[-1]], dist[:n_local]

    @staticmethod
    def _task_arrays(tasks):
        nt = len(tasks)
        slots = np.array([t[0] for t in tasks], dtype=np.uint32)
        kls = np.array([t[1] for t in tasks], dtype=np.uint32)
        lens = np.array([len(t[2]) for t in tasks], dtype=np.uint32)
        offs = np.zeros(nt, dtype=np.uint64)
        offs[1:] = np.cumsum(lens[:-1].astype(np.uint64))
        ent = (np.concatenate([np.asarray(t[2], dtype=np.uint32) for t in tasks])
               if nt else np.zeros(1, np.uint32))
        return nt, slots, kls, lens, offs, ent

    def debug_lookahead(self, tasks, force):
        """Strong-branching lookahead: for each task (slot, kl, entries) the
        step that branches on force[i] (a local id), then one step on each
        child.  Returns (hdr[n][16], nkids, branching, cost)."""
        nt, slots, kls, lens, offs, ent = self._task_arrays(tasks)
        f = np.ascontiguousarray(force, dtype=np.uint32)
        hdr = np.zeros(16 * nt, dtype=np.uint32)
        nk = np.zeros(nt, dtype=np.uint32)
        br = np.zeros(nt, dtype=np.uint32)
        cost = np.zeros(nt, dtype=np.uint64)
        self._check(lib().scs_debug_lookahead(self._h, nt, _p(slots), _p(kls),
                                              offs.ctypes.data_as(_u64p), _p(lens), _p(ent),
                                              _p(f), _p(hdr), _p(nk), _p(br),
                                              cost.ctypes.data_as(_u64p)),
                    "scs_debug_lookahead")
        return hdr.reshape(nt, 16), nk, br, cost

    def debug_step(self, tasks, kids_stride=None, force=None, shortlist=False):
        """tasks: list of (slot, kl, entries[uint32 (id<<1)|inC]).  Returns a
        list of dicts with hdr, doms, kids, wit (and sl_ids, sl_feat with
        shortlist=True).  force: per task a local id to branch on, or
        0xFFFFFFFF for the rule's u*."""
        nt = len(tasks)
        slots = np.array([t[0] for t in tasks], dtype=np.uint32)
        kls = np.array([t[1] for t in tasks], dtype=np.uint32)
        lens = np.array([len(t[2]) for t in tasks], dtype=np.uint32)
        offs = np.zeros(nt, dtype=np.uint64)
        offs[1:] = np.cumsum(lens[:-1].astype(np.uint64))
        ent = np.concatenate([np.asarray(t[2], dtype=np.uint32) for t in tasks]) if nt else np.zeros(1, np.uint32)
        maxlen = int(lens.max()) if nt else 1
        ks = kids_stride or (17 * (2 + 2 * maxlen))
        hdr = np.zeros(16 * nt, dtype=np.uint32)
        doms = np.zeros(16 * nt, dtype=np.uint32)
        kids = np.zeros(ks * nt, dtype=np.uint32)
        wit = np.zeros(513 * nt, dtype=np.uint32)
        fa = None if force is None else np.ascontiguousarray(force, dtype=np.uint32)
        sl = np.zeros(17 * nt, dtype=np.uint32) if shortlist else None
        slf = np.zeros(16 * 16 * nt, dtype=np.float32) if shortlist else None
        self._check(lib().scs_debug_step(self._h, nt, _p(slots), _p(kls),
                                         offs.ctypes.data_as(_u64p), _p(lens), _p(ent),
                                         _p(hdr), _p(doms), 16, _p(kids), ks, _p(wit), 513,
                                         None if fa is None else _p(fa),
                                         None if sl is None else _p(sl),
                                         None if slf is None else _fp(slf)),
                    "scs_debug_step")
        out = []
        for i in range(nt):
            h = hdr[16 * i: 16 * i + 16].copy()
            k = kids[ks * i: ks * i + ks]
            children = []
            w = 0
            for _ in range(int(h[9]) if h[0] == 0 else 0):
                s2, c2 = int(k[w]), int(k[w + 1])
                children.append((s2, c2, k[w + 2: w + 2 + s2].copy(), k[w + 2 + s2: w + 2 + 2 * s2].copy()))
                w += 2 + 2 * s2
            wn = int(wit[513 * i + 512])
            d = dict(hdr=h, doms=doms[16 * i: 16 * i + int(h[8])].copy(),
                     kids=children, wit=np.sort(wit[513 * i: 513 * i + wn].copy()))
            if shortlist:
                k_sl = int(sl[17 * i])
                d["sl_ids"] = sl[17 * i + 1: 17 * i + 1 + k_sl].copy()
                d["sl_feat"] = slf[256 * i: 256 * i + 16 * k_sl].reshape(k_sl, 16).copy()
            out.append(d)
        return out

    def close(self):
        if self._h:
            lib().scs_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
