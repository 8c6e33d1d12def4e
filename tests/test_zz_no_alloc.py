"""The allocation-free local-graph entry point (scs_local_graph_noalloc),
for callers that cannot allocate device memory, against the engine's own
preprocessing entry point and the CPU oracle's local graph on the same
queries, plus its argument checks.

This file is named to be collected last.  It passes both alone in a fresh
process and after the other tests: the entry point looks up its fixed scratch
array on first use and every call clears what it needs.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _strip(off, adj, nl):
    rows = []
    for i in range(nl):
        r = adj[off[i]:off[i + 1]]
        rows.append(r[r != 0xFFFFFFFF])
    o = np.zeros(nl + 1, dtype=np.int64)
    o[1:] = np.cumsum([len(r) for r in rows])
    return o, (np.concatenate(rows) if rows else np.zeros(0, np.uint32))


def test_noalloc_matches_engine_two_calls_in_a_row(oracle_lib):
    import torch
    from scs_gb300 import workloads as W
    from scs_gb300.engine import Engine, SCSError, local_graph_noalloc
    n, u, v = W.chung_lu(4000, 88000, 2.5)
    off, adj = W.to_csr(n, u, v)
    og = oracle_lib.OracleGraph(n, off, adj)
    cand = [int(x) for x in np.flatnonzero(og.core >= 8)[:2]]
    cases = []
    for q in cand:
        kl, _ = og.heuristic(0, 3, 12, q)
        cases.append((3, 12, q, int(oracle_lib.lib().orc_ubd_host(kl, 12)), kl))
    # existing entry point: the engine's preprocessing into slots 0 and 1
    eng = Engine(csr=(n, off, adj), limit_queries=4, stack_words=1 << 20, pool_words=1 << 22)
    nl, ql = eng.debug_prepare([(l, h, q, 0, 10) for (l, h, q, ubd, kl) in cases],
                               [c[4] for c in cases], [c[3] for c in cases])
    dev = torch.device("cuda:0")
    d_off = torch.from_numpy(off.astype(np.int32)).to(dev)
    d_adj = torch.from_numpy(adj.astype(np.int32)).to(dev)
    d_core = torch.from_numpy(og.core.astype(np.int32)).to(dev)
    cap = int(len(adj)) + 3 * n + 4
    gid = torch.zeros(n, dtype=torch.int32, device=dev)
    dist = torch.zeros(n, dtype=torch.int32, device=dev)
    loff = torch.zeros(n + 1, dtype=torch.int32, device=dev)
    ladj = torch.zeros(cap, dtype=torch.int32, device=dev)
    info = torch.zeros(4, dtype=torch.int32, device=dev)
    stream = torch.cuda.current_stream().cuda_stream
    for i, (l, h, q, ubd, kl) in enumerate(cases):  # two calls in a row
        local_graph_noalloc(d_off.data_ptr(), d_adj.data_ptr(), d_core.data_ptr(), n,
                            og.dmax, q, kl, ubd, gid.data_ptr(), dist.data_ptr(),
                            loff.data_ptr(), ladj.data_ptr(), cap, info.data_ptr(), stream)
        torch.cuda.synchronize()
        inf = info.cpu().numpy().view(np.uint32)
        assert inf[3] == 0
        assert inf[0] == nl[i] and inf[1] == ql[i]
        m = int(inf[0])
        g_gid, g_off, g_adj, g_dist = eng.debug_local_graph(i, m, int(inf[2]))
        o = loff.cpu().numpy().view(np.uint32)[: m + 1]
        a = ladj.cpu().numpy().view(np.uint32)[: int(inf[2])]
        so, sa = _strip(o, a, m)
        assert np.array_equal(gid.cpu().numpy().view(np.uint32)[:m], g_gid)
        assert np.array_equal(so, g_off.astype(np.int64))
        assert np.array_equal(sa, g_adj)
        assert np.array_equal(dist.cpu().numpy().view(np.uint32)[:m], g_dist)
        # and directly against the oracle's local graph
        ctx = oracle_lib.OracleCtx(og, l, h, q, kl, ubd, 10)
        assert m == ctx.n and int(inf[1]) == ctx.q_local
        assert np.array_equal(gid.cpu().numpy().view(np.uint32)[:m], ctx.gid)
        assert np.array_equal(so, ctx.off.astype(np.int64))
        assert np.array_equal(sa, ctx.adj)
        assert np.array_equal(dist.cpu().numpy().view(np.uint32)[:m], ctx.dist)
        ctx.close()
    # a distance bound the 16-bit distances cannot hold is rejected
    l, h, q, ubd, kl = cases[0]
    with pytest.raises(SCSError, match=r"\(-1\)"):
        local_graph_noalloc(d_off.data_ptr(), d_adj.data_ptr(), d_core.data_ptr(), n,
                            og.dmax, q, kl, 0xFFFF, gid.data_ptr(), dist.data_ptr(),
                            loff.data_ptr(), ladj.data_ptr(), cap, info.data_ptr(), stream)
    eng.close()
