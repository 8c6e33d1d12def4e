import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300)")


def pytest_collection_modifyitems(config, items):
    try:
        import torch
        has_gpu = torch.cuda.is_available()
    except Exception:
        has_gpu = False
    if has_gpu:
        return
    skip = pytest.mark.skip(reason="no GPU")
    for it in items:
        if "gpu" in it.keywords:
            it.add_marker(skip)


@pytest.fixture(scope="session")
def oracle_lib():
    import oracle
    from oracle import build_ref
    build_ref.build_oracle()
    return oracle


@pytest.fixture(scope="session")
def graph_dir(tmp_path_factory):
    return tmp_path_factory.mktemp("graphs")


@pytest.fixture(scope="session")
def chunglu_small(graph_dir):
    """Chung-Lu n=4000, m=88000, exponent 2.5 (seed 1234) as an edge list."""
    from scs_gb300 import workloads as W
    n, u, v = W.chung_lu(4000, 88000, 2.5)
    path = str(graph_dir / "chunglu_n4000.txt")
    W.write_edgelist(path, n, u, v)
    return path


@pytest.fixture(scope="session")
def rmat15(graph_dir):
    """R-MAT scale 15, 16*2^15 edges, (.57,.19,.19) (seed 1234)."""
    from scs_gb300 import workloads as W
    n, u, v = W.rmat(15, 16 << 15)
    path = str(graph_dir / "rmat_s15.txt")
    W.write_edgelist(path, n, u, v)
    return path


def random_graph(rng, n, p):
    from scs_gb300 import workloads as W
    iu = np.triu_indices(n, 1)
    mask = rng.random(len(iu[0])) < p
    u, v = iu[0][mask].astype(np.uint32), iu[1][mask].astype(np.uint32)
    off, adj = W.to_csr(n, u, v)
    return n, off, adj
