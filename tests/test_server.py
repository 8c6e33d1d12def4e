"""The reference-compatible server surface: queue messages, result rows,
CLI, the SysV transport of scs_client, and (GPU) an end-to-end server run."""
import ctypes as C
import json
import os
import subprocess
import time

import numpy as np
import pytest

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _lib():
    from scs_gb300 import build as B
    from scs_gb300.engine import Query, Result
    B.build()
    L = C.CDLL(B.lib_path())
    L.scs_parse_message.argtypes = [C.c_char_p, C.POINTER(Query)]
    L.scs_format_result_row.argtypes = [C.POINTER(Result), C.c_char_p, C.c_uint32]
    return L, Query, Result


def test_parse_messages():
    L, Query, _ = _lib()
    q = Query()
    assert L.scs_parse_message(b"9 12 1127 1 10", C.byref(q)) == 0
    assert (q.l, q.h, q.q, q.heuristic, q.limit_doms) == (9, 12, 1127, 1, 10)
    assert L.scs_parse_message(b"  SERVER_EXIT \n", C.byref(q)) == 1
    for bad in (b"9 12 1127 1", b"9 12 1127 1 10 3", b"9 12 x 1 10", b"", b"-1 2 3 4 5"):
        assert L.scs_parse_message(bad, C.byref(q)) < 0, bad


def test_result_rows_match_reference_layout():
    """Rows for a finished search, a heuristic answer, the level cap and the
    buffer overflow (main.cu:124-128, 328-333, 348-352, 451-454)."""
    L, _, Result = _lib()
    buf = C.create_string_buffer(128)

    def row(status, degree=7, lat_us=1234567):
        r = Result(l=9, h=12, q=1127, degree=degree, status=status, latency_ns=lat_us * 1000)
        n = L.scs_format_result_row(C.byref(r), buf, 128)
        assert n > 0
        return buf.value.decode()

    assert row(0) == "9|12|1127|1,234,567|7|0|0|0"
    assert row(1) == "9|12|1127|1,234,567|7|0|1|0"
    assert row(3) == "9|12|1127|1,234,567|7|1|0"
    assert row(2) == "9|12|1127|1,234,567|7|2|0|0"
    assert row(0, lat_us=0) == "9|12|1127|0|7|0|0|0"
    assert row(0, lat_us=999) == "9|12|1127|999|7|0|0|0"
    assert row(0, lat_us=1000) == "9|12|1127|1,000|7|0|0|0"


def test_server_rejects_wrong_arguments(tmp_path):
    from scs_gb300 import build as B
    B.build()
    out = subprocess.run([B.exe_path("scs_server"), "g.txt", "1"], capture_output=True,
                         text=True, cwd=str(tmp_path), timeout=60)
    assert out.returncode == 1
    assert "Server wrong input parameters!" in out.stdout


class _MsgBuf(C.Structure):
    _fields_ = [("mtype", C.c_long), ("mtext", C.c_char * 80)]


def test_client_sends_reference_messages(tmp_path):
    """scs_client puts one mtype-1 message per line on the ftok("/tmp", p)
    queue and server_exit last; read back here with msgrcv."""
    from scs_gb300 import build as B
    B.build()
    libc = C.CDLL(None, use_errno=True)
    libc.ftok.argtypes = [C.c_char_p, C.c_int]
    libc.msgget.argtypes = [C.c_int, C.c_int]
    libc.msgrcv.argtypes = [C.c_int, C.c_void_p, C.c_size_t, C.c_long, C.c_int]
    libc.msgctl.argtypes = [C.c_int, C.c_int, C.c_void_p]
    proj = "k"
    key = libc.ftok(b"/tmp", ord(proj))
    IPC_CREAT, IPC_RMID, IPC_NOWAIT = 0o1000, 0, 0o4000
    qid = libc.msgget(key, IPC_CREAT | 0o660)
    if qid < 0:
        pytest.skip("System V message queues unavailable")
    try:
        while True:  # drain leftovers
            m = _MsgBuf()
            if libc.msgrcv(qid, C.byref(m), 80, 0, IPC_NOWAIT) < 0:
                break
        qf = tmp_path / "q.txt"
        qf.write_text("3 6 10 1 1\n6 9 54 1 1\nserver_exit\n9 12 7 1 1\n")
        env = dict(os.environ, SCS_IPC_PROJ=proj)
        out = subprocess.run([B.exe_path("scs_client"), str(qf)], env=env,
                             capture_output=True, text=True, timeout=60)
        assert out.returncode == 0, out.stderr
        got = []
        for _ in range(3):
            m = _MsgBuf()
            r = libc.msgrcv(qid, C.byref(m), 80, 1, IPC_NOWAIT)
            assert r > 0
            got.append(m.mtext.decode())
        assert got == ["3 6 10 1 1", "6 9 54 1 1", "server_exit"]
        m = _MsgBuf()
        assert libc.msgrcv(qid, C.byref(m), 80, 0, IPC_NOWAIT) < 0
    finally:
        libc.msgctl(qid, IPC_RMID, None)


@pytest.mark.gpu
def test_server_end_to_end(tmp_path, chunglu_small):
    """scs_server with the reference CLI answers queries sent by scs_client
    and writes the reference's results file; degrees equal the oracle's, and
    the communities it writes on request pass scs_verify."""
    from scs_gb300 import build as B
    B.build()
    gold = [g for g in json.load(open(os.path.join(GOLD, "answers_chunglu_n4000.json")))["queries"]
            if g["finished"]][:10]
    qf = tmp_path / "queries.txt"
    qf.write_text("".join("%d %d %d %d %d\n" % (g["l"], g["h"], g["q"], g["heur"], g["limit_doms"])
                          for g in gold) + "1 2\nserver_exit\n")
    env = dict(os.environ, SCS_IPC_PROJ="s", SCS_COMMUNITIES="1")
    srv = subprocess.Popen([B.exe_path("scs_server"), chunglu_small, "300000", "100000", "0.5",
                            "1", "8", "100", "1", "1", "1", "1", "1"],
                           cwd=str(tmp_path), env=env, stdout=subprocess.PIPE,
                           stderr=subprocess.PIPE, text=True)
    try:
        cl = subprocess.run([B.exe_path("scs_client"), str(qf)], env=env, capture_output=True,
                            text=True, timeout=120)
        assert cl.returncode == 0, cl.stderr
        out, err = srv.communicate(timeout=300)
    finally:
        if srv.poll() is None:
            srv.kill()
    assert srv.returncode == 0, err
    assert "Client wrong input parameters!" in out
    rows = (tmp_path / "results" / "results_chunglu_n4000.txt").read_text().strip().splitlines()
    assert rows[0] == "N1|N2|QID|Time|Degree|Overtime|Heu|TotalTime"
    assert rows[-1].startswith("-1|-1|-1|-1|-1|-1|-1|")
    body = [r.split("|") for r in rows[1:-1]]
    assert len(body) == len(gold)
    want = {(g["l"], g["h"], g["q"]): g for g in gold}
    for f in body:
        g = want[(int(f[0]), int(f[1]), int(f[2]))]
        assert int(f[4]) == g["degree"]
        assert f[5] == "0" and f[6] == ("1" if g["heu_hit"] else "0")
    comm = tmp_path / "results" / "communities_chunglu_n4000.txt"
    v = subprocess.run([B.exe_path("scs_verify"), chunglu_small, str(comm)],
                       capture_output=True, text=True, timeout=120)
    assert v.returncode == 0, v.stdout + v.stderr
    assert "verified %d of %d rows" % (len(gold), len(gold)) in v.stdout
