"""ctypes binding of the CPU oracle (oracle.c) and of the reference's own CPU
code built into oracle/_ref.  TEST INFRASTRUCTURE ONLY: imported by tests/,
__graft_entry__.smoke() and bench.py's CPU-baseline legs, never by the
product path."""
import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
_u32p = C.POINTER(C.c_uint32)

RED1, RED2, RED3, PRUN1, PRUN2 = 1, 2, 4, 8, 16
ALL_RULES = 31


class Graph(C.Structure):
    _fields_ = [("n", C.c_uint32), ("off", _u32p), ("adj", _u32p),
                ("degree", _u32p), ("core", _u32p), ("dmax", C.c_uint32)]


class Result(C.Structure):
    _fields_ = [("degree", C.c_uint32), ("kl_heu", C.c_uint32),
                ("ku", C.c_uint32), ("heu_hit", C.c_uint32),
                ("ubd", C.c_uint32), ("n_kept", C.c_uint32),
                ("n_local", C.c_uint32), ("status", C.c_uint32),
                ("nodes", C.c_uint64), ("max_task", C.c_uint64),
                ("sum_task", C.c_uint64), ("h_size", C.c_uint32),
                ("h_from_bnb", C.c_uint32), ("size_hist", C.c_uint64 * 8)]


class QCtx(C.Structure):
    _fields_ = [("n", C.c_uint32), ("off", _u32p), ("adj", _u32p),
                ("dist", _u32p), ("gid", _u32p), ("q_local", C.c_uint32),
                ("l", C.c_uint32), ("h", C.c_uint32),
                ("limit_doms", C.c_uint32), ("dmax", C.c_uint32),
                ("rules", C.c_uint32), ("pos", C.POINTER(C.c_int32))]


def _p(a):
    return a.ctypes.data_as(_u32p)


_lib = None


def lib():
    global _lib
    if _lib is None:
        path = os.path.join(HERE, "liboracle.so")
        if not os.path.exists(path):
            from . import build_ref
            build_ref.build_oracle()
        L = C.CDLL(path)
        L.orc_load_edgelist.argtypes = [C.c_char_p, _u32p, C.POINTER(C.c_uint64),
                                        C.POINTER(_u32p), C.POINTER(_u32p)]
        L.orc_free.argtypes = [C.c_void_p]
        L.orc_core.argtypes = [C.c_uint32, _u32p, _u32p, _u32p]
        L.orc_bfs.argtypes = [C.c_uint32, _u32p, _u32p, C.c_uint32, _u32p]
        L.orc_ubd_host.restype = C.c_uint32
        L.orc_ubd_dev.restype = C.c_uint32
        L.orc_ubd_host.argtypes = [C.c_uint32, C.c_uint32]
        L.orc_ubd_dev.argtypes = [C.c_uint32, C.c_uint32]
        for f in ("orc_heu2", "orc_heu3", "orc_heu4", "orc_cssc_heu"):
            getattr(L, f).argtypes = [C.POINTER(Graph), C.c_uint32, C.c_uint32,
                                      C.c_uint32, _u32p, _u32p]
            getattr(L, f).restype = C.c_uint32
        L.orc_solve.argtypes = [C.POINTER(Graph), C.c_uint32, C.c_uint32,
                                C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32,
                                C.c_uint64, C.POINTER(Result), _u32p, C.c_uint32]
        L.orc_set_time_limit.argtypes = [C.c_double]
        L.orc_bruteforce.argtypes = [C.POINTER(Graph), C.c_uint32, C.c_uint32,
                                     C.c_uint32, C.c_uint32]
        L.orc_bruteforce.restype = C.c_uint32
        L.orc_prepare.argtypes = [C.POINTER(Graph), C.c_uint32, C.c_uint32,
                                  C.c_uint32, C.c_uint32, C.POINTER(QCtx), _u32p]
        L.orc_qctx_free.argtypes = [C.POINTER(QCtx)]
        L.orc_step.argtypes = [C.POINTER(QCtx), _u32p, C.c_uint32, C.c_uint32,
                               _u32p, _u32p, _u32p, C.c_uint64, _u32p]
        _lib = L
    return _lib


class OracleGraph:
    """Holds a CSR graph plus degree/core arrays for oracle calls."""

    def __init__(self, n, off, adj):
        self.n = int(n)
        self.off = np.ascontiguousarray(off, dtype=np.uint32)
        self.adj = np.ascontiguousarray(adj, dtype=np.uint32)
        self.degree = np.diff(self.off.astype(np.int64)).astype(np.uint32)
        self.dmax = int(self.degree.max()) if self.n else 0
        self.core = np.zeros(self.n, dtype=np.uint32)
        if self.n:
            lib().orc_core(self.n, _p(self.off), _p(self.adj), _p(self.core))
        self.g = Graph(self.n, _p(self.off), _p(self.adj), _p(self.degree),
                       _p(self.core), self.dmax)

    @classmethod
    def from_file(cls, path):
        n = C.c_uint32()
        m = C.c_uint64()
        off = _u32p()
        adj = _u32p()
        rc = lib().orc_load_edgelist(path.encode(), C.byref(n), C.byref(m),
                                     C.byref(off), C.byref(adj))
        if rc != 0:
            raise IOError("oracle loader failed (%d) on %s" % (rc, path))
        nn = n.value
        o = np.ctypeslib.as_array(off, shape=(nn + 1,)).copy()
        a = np.ctypeslib.as_array(adj, shape=(max(int(o[-1]), 1),))[: int(o[-1])].copy()
        lib().orc_free(C.cast(off, C.c_void_p))
        lib().orc_free(C.cast(adj, C.c_void_p))
        g = cls(nn, o, a)
        g.m_header = m.value
        return g

    def bfs(self, q):
        d = np.empty(self.n, dtype=np.uint32)
        lib().orc_bfs(self.n, _p(self.off), _p(self.adj), q, _p(d))
        return d

    def heuristic(self, which, l, h, q):
        H = np.zeros(max(self.n, 1), dtype=np.uint32)
        hs = C.c_uint32()
        f = {2: "orc_heu2", 3: "orc_heu3", 4: "orc_heu4", 0: "orc_cssc_heu"}[which]
        kl = getattr(lib(), f)(C.byref(self.g), l, h, q, _p(H), C.byref(hs))
        return int(kl), H[: hs.value].copy()

    def solve(self, l, h, q, heur=1, limit_doms=10, rules=ALL_RULES,
              node_limit=0):
        r = Result()
        H = np.zeros(max(self.n, 1), dtype=np.uint32)
        lib().orc_solve(C.byref(self.g), l, h, q, heur, limit_doms, rules,
                        node_limit, C.byref(r), _p(H), H.size)
        return r, H[: r.h_size].copy()

    def bruteforce(self, l, h, q, max_comp=22):
        return int(lib().orc_bruteforce(C.byref(self.g), l, h, q, max_comp))


def verify_community(g, H, q, l, h):
    """(connected, contains q, size ok, min degree) of H in graph g."""
    H = np.asarray(H, dtype=np.int64)
    s = set(H.tolist())
    if not s:
        return False, False, False, 0
    md = None
    for v in s:
        nb = g.adj[g.off[v]:g.off[v + 1]]
        d = sum(1 for w in nb.tolist() if w in s)
        md = d if md is None else min(md, d)
    start = next(iter(s))
    seen = {start}
    stack = [start]
    while stack:
        v = stack.pop()
        for w in g.adj[g.off[v]:g.off[v + 1]].tolist():
            if w in s and w not in seen:
                seen.add(w)
                stack.append(w)
    return len(seen) == len(s), q in s, l <= len(s) <= h, md


class RefLib:
    """The reference's own CPU code (oracle/_ref/libscsref.so)."""

    def __init__(self, path=None):
        path = path or os.path.join(HERE, "_ref", "libscsref.so")
        if not os.path.exists(path):
            raise FileNotFoundError(path)
        L = C.CDLL(path)
        L.ref_load.argtypes = [C.c_char_p]
        L.ref_sizes.argtypes = [_u32p, C.POINTER(C.c_uint64),
                                C.POINTER(C.c_uint64), _u32p]
        L.ref_copy.argtypes = [_u32p, _u32p, _u32p, _u32p]
        L.ref_bfs.argtypes = [C.c_uint32, _u32p]
        L.ref_heu.argtypes = [C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32,
                              _u32p, _u32p]
        L.ref_heu.restype = C.c_uint32
        self.L = L
        self.loaded = False

    def load(self, path):
        # The reference keeps one graph in process globals: load once.
        assert not self.loaded, "the reference library holds one graph per process"
        self.L.ref_load(path.encode())
        n = C.c_uint32()
        m = C.c_uint64()
        nnz = C.c_uint64()
        dmax = C.c_uint32()
        self.L.ref_sizes(C.byref(n), C.byref(m), C.byref(nnz), C.byref(dmax))
        self.n, self.m_header, self.dmax = n.value, m.value, dmax.value
        self.off = np.zeros(self.n + 1, dtype=np.uint32)
        self.adj = np.zeros(max(nnz.value, 1), dtype=np.uint32)
        self.degree = np.zeros(self.n, dtype=np.uint32)
        self.core = np.zeros(self.n, dtype=np.uint32)
        self.L.ref_copy(_p(self.off), _p(self.adj), _p(self.degree), _p(self.core))
        self.adj = self.adj[: nnz.value]
        self.loaded = True

    def bfs(self, q):
        d = np.empty(self.n, dtype=np.uint32)
        self.L.ref_bfs(q, _p(d))
        return d

    def heuristic(self, which, l, h, q):
        H = np.zeros(max(self.n, 1), dtype=np.uint32)
        hs = C.c_uint32()
        kl = self.L.ref_heu(which, l, h, q, _p(H), C.byref(hs))
        return int(kl), H[: hs.value].copy()


class OracleCtx:
    """Per-query local graph (orc_prepare) plus single steps (orc_step)."""

    def __init__(self, og, l, h, q, kl, ubd, limit_doms=10, rules=ALL_RULES,
                 component_only=1):
        self.ctx = QCtx()
        nk = C.c_uint32()
        lib().orc_prepare(C.byref(og.g), q, kl, ubd, component_only, C.byref(self.ctx), C.byref(nk))
        self.ctx.l, self.ctx.h = l, h
        self.ctx.limit_doms = limit_doms
        self.ctx.dmax = og.dmax
        self.ctx.rules = rules
        self.n_kept = nk.value
        n = self.ctx.n
        self.n = n
        self.q_local = self.ctx.q_local
        self.off = np.ctypeslib.as_array(self.ctx.off, shape=(n + 1,)).copy()
        e = int(self.off[-1])
        self.adj = np.ctypeslib.as_array(self.ctx.adj, shape=(max(e, 1),))[:e].copy()
        self.gid = np.ctypeslib.as_array(self.ctx.gid, shape=(max(n, 1),))[:n].copy()
        self.dist = np.ctypeslib.as_array(self.ctx.dist, shape=(max(n, 1),))[:n].copy()

    def root(self):
        return np.array([(i << 1) | (1 if i == self.q_local else 0) for i in range(self.n)],
                        dtype=np.uint32)

    def step(self, entries, kl):
        entries = np.ascontiguousarray(entries, dtype=np.uint32)
        s = len(entries)
        hdr = np.zeros(16, dtype=np.uint32)
        doms = np.zeros(max(self.ctx.limit_doms, 1) + 1, dtype=np.uint32)
        cap = (s + 2) * (self.ctx.limit_doms + 2) + 8
        kids = np.zeros(cap, dtype=np.uint32)
        wit = np.zeros(s + 1, dtype=np.uint32)
        rc = lib().orc_step(C.byref(self.ctx), _p(entries), s, kl, _p(hdr), _p(doms),
                            _p(kids), cap, _p(wit))
        assert rc == 0
        children = []
        w = 0
        if hdr[0] == 0:
            for _ in range(int(hdr[9])):
                s2, c2 = int(kids[w]), int(kids[w + 1])
                children.append((s2, c2, kids[w + 2: w + 2 + s2].copy()))
                w += 2 + s2
        return dict(hdr=hdr, doms=doms[: int(hdr[8])].copy(), kids=children,
                    wit=np.sort(wit[: int(hdr[11])].copy()) if hdr[2] != 0xFFFFFFFF else None)

    def degrees(self, entries):
        """(dC, dR) of each entry inside the task (reference semantics of
        degreeInC/degreeInR, inc/Intialize.h:120-138)."""
        ids = entries >> 1
        inC = (entries & 1).astype(bool)
        pos = {int(v): i for i, v in enumerate(ids)}
        dc = np.zeros(len(ids), dtype=np.uint32)
        dr = np.zeros(len(ids), dtype=np.uint32)
        for i, v in enumerate(ids.tolist()):
            for w in self.adj[self.off[v]:self.off[v + 1]].tolist():
                j = pos.get(w)
                if j is not None:
                    if inC[j]:
                        dc[i] += 1
                    else:
                        dr[i] += 1
        return dc, dr

    def collect_tasks(self, kl, limit):
        """Tasks of the serial depth-first search (Include first), with the
        incumbent each was processed under: [(entries, kl), ...]."""
        stack = [self.root()]
        out = []
        while stack and len(out) < limit:
            e = stack.pop()
            out.append((e, kl))
            r = self.step(e, kl)
            kl = int(r["hdr"][1])
            for ch in reversed(r["kids"]):
                stack.append(ch[2])
        return out

    def close(self):
        if self.ctx.off:
            lib().orc_qctx_free(C.byref(self.ctx))

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
