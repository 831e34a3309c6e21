import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
GOLDEN = os.path.join(ROOT, "tests", "golden")
GOLDEN_CASES = ("3elt", "tri69", "rmat10", "wgrid40")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103a) and the built libcm.so")


def load_golden(name):
    """-> dict(threshold, nparts, graph0, seeds={seed: (maxvwgt, [graphs], [cmaps])})."""
    from oracle import oracle as O
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    g0 = O.CSR(z["xadj"], z["adjncy"], z["adjwgt"], z["vwgt"])
    seeds = {}
    for seed in (1, 2):
        p = "s%d_" % seed
        nl = int(z[p + "nlevels"])
        graphs = [g0]
        for l in range(1, nl + 1):
            q = p + "L%d_" % l
            graphs.append(O.CSR(z[q + "xadj"], z[q + "adjncy"], z[q + "adjwgt"], z[q + "vwgt"]))
        cmaps = [z[p + "L%d_cmap" % l] for l in range(nl)]
        seeds[seed] = (int(z[p + "maxvwgt"]), graphs, cmaps)
    return dict(threshold=int(z["threshold"]), nparts=int(z["nparts"]), graph0=g0, seeds=seeds)


def sorted_rows(g):
    """(xadj, adjncy, adjwgt) with rows sorted by neighbour id."""
    a, w = g.rows_sorted()
    return np.asarray(g.xadj), a, w


@pytest.fixture(scope="session")
def golden():
    return {name: load_golden(name) for name in GOLDEN_CASES}


@pytest.fixture(scope="session")
def ctx():
    import cumetis_gb300 as cm
    c = cm.Context(0)
    yield c
    c.close()
