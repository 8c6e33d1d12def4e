"""The answer verifier (scs_check_community) and the scs_verify CLI.

The reference reports only the degree of an answer (main.cu:328-334); the
engine also returns the community, and these tests pin the checks applied to
it: valid distinct ids, q in H, l <= |H| <= h, connectivity, and the minimum
internal degree (against the oracle's verify_community)."""
import os
import subprocess

import numpy as np
import pytest

from scs_gb300 import build as B
from scs_gb300 import engine as E
from scs_gb300 import workloads as W


@pytest.fixture(scope="module")
def built():
    B.build()
    return B.exe_path("scs_verify")


def _csr(n, edges):
    u = np.array([a for a, b in edges], dtype=np.int64)
    v = np.array([b for a, b in edges], dtype=np.int64)
    return W.to_csr(n, u, v)


def test_check_community_reasons(built):
    # path 0-1-2, triangle 3-4-5, bridge 2-3, isolated 6
    n = 7
    off, adj = _csr(n, [(0, 1), (1, 2), (2, 3), (3, 4), (4, 5), (3, 5)])
    chk = lambda H, q, l, h: E.check_community(n, off, adj, H, q, l, h)
    assert chk([3, 4, 5], 3, 2, 5) == (0, 2)
    assert chk([2, 3, 4, 5], 4, 3, 4) == (0, 1)
    assert chk([], 3, 1, 5)[0] == 1
    assert chk([3, 4, 9], 3, 1, 5)[0] == 2
    assert chk([3, 4, 4], 3, 1, 5)[0] == 3
    assert chk([3, 4, 5], 0, 1, 5) == (4, 2)
    assert chk([3, 4, 5], 3, 4, 5)[0] == 5
    assert chk([3, 4, 5], 3, 1, 2)[0] == 5
    assert chk([0, 4], 0, 1, 5) == (6, 0)
    assert chk([6], 6, 1, 1) == (0, 0)


def test_check_community_matches_oracle(built, oracle_lib):
    n, u, v = W.chung_lu(300, 1500, 2.5, seed=7)
    off, adj = W.to_csr(n, u, v)
    og = oracle_lib.OracleGraph(n, off, adj)
    rng = np.random.default_rng(3)
    for _ in range(400):
        k = int(rng.integers(1, 12))
        H = rng.choice(n, size=k, replace=False)
        if rng.random() < 0.5:  # grow a connected set from a random start
            H = [int(rng.integers(n))]
            for _ in range(k - 1):
                nb = adj[off[H[-1]]:off[H[-1] + 1]]
                cand = [w for w in nb.tolist() if w not in H]
                if not cand:
                    break
                H.append(int(rng.choice(cand)))
            H = np.array(H)
        q = int(H[0]) if rng.random() < 0.8 else int(rng.integers(n))
        l, h = int(rng.integers(1, 6)), int(rng.integers(6, 14))
        code, md = E.check_community(n, off, adj, H, q, l, h)
        conn, has_q, size_ok, omd = oracle_lib.verify_community(og, H, q, l, h)
        assert md == omd
        assert (code == 0) == (conn and has_q and size_ok)


def _rows_from_heuristics(oracle_lib, path, count):
    n, off, adj = E.read_edge_list(path)
    og = oracle_lib.OracleGraph(n, off, adj)
    core = E.core_numbers(n, off, adj)
    Q = W.queries_small(core, count=count * 2)
    rows = []
    for l, h, q, _, _ in Q.tolist():
        kl, H = og.heuristic(0, l, h, q)
        if kl > 0 and len(H):
            rows.append((q, l, h, kl, 3, list(map(int, H))))
        if len(rows) == count:
            break
    return rows


def _write(path, rows, extra=()):
    with open(path, "w") as f:
        f.write("QID|N1|N2|Degree|Status|Community\n")
        for q, l, h, d, st, H in rows:
            f.write("%d|%d|%d|%d|%d|%s\n" % (q, l, h, d, st, " ".join(map(str, H))))
        for line in extra:
            f.write(line + "\n")


def test_verify_cli(built, oracle_lib, chunglu_small, tmp_path):
    rows = _rows_from_heuristics(oracle_lib, chunglu_small, 20)
    assert len(rows) >= 10
    good = tmp_path / "good.txt"
    _write(good, rows)
    r = subprocess.run([built, chunglu_small, str(good)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "verified %d of %d rows" % (len(rows), len(rows)) in r.stdout
    assert r.stdout.count("|OK") == len(rows)

    bad = list(rows)
    q, l, h, d, st, H = bad[0]
    bad[0] = (q, l, h, d + 1, st, H)                       # wrong degree
    q, l, h, d, st, H = bad[1]
    bad[1] = (q, l, h, d, st, H + [10 ** 7])               # id out of range
    q, l, h, d, st, H = bad[2]
    bad[2] = (q, l, h, d, st, [x for x in H if x != q] or [0])  # q missing
    badf = tmp_path / "bad.txt"
    _write(badf, bad)
    r = subprocess.run([built, chunglu_small, str(badf)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 1
    lines = r.stdout.splitlines()
    assert "FAIL minimum degree" in lines[0]
    assert "FAIL vertex id out of range" in lines[1]
    assert "FAIL" in lines[2]
    assert "verified %d of %d rows" % (len(rows) - 3, len(rows)) in r.stdout

    mal = tmp_path / "malformed.txt"
    _write(mal, rows[:2], extra=["1|2|x|4|0|1 2"])
    r = subprocess.run([built, chunglu_small, str(mal)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 2

    r = subprocess.run([built, chunglu_small], capture_output=True, text=True, timeout=60)
    assert r.returncode == 2 and "usage" in r.stderr
