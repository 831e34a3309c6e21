"""Initial partition (host code): bit-exact against the reference's own
cuMetis_rbbisection (cuMetis.cu:3046) outputs recorded in
tests/golden/initpart.npz, plus edge cases.  No GPU needed."""
import os

import numpy as np
import pytest

import cumetis_gb300 as cm
from conftest import GOLDEN

Z = np.load(os.path.join(GOLDEN, "initpart.npz"))
NAMES = [str(x) for x in Z["names"]]
KS = [tuple(int(v) for v in r) for r in Z["ks"]]


def _graph(name):
    return cm.Graph(Z[name + "_xadj"], Z[name + "_adjncy"], Z[name + "_adjwgt"], Z[name + "_vwgt"])


@pytest.mark.parametrize("name", NAMES)
@pytest.mark.parametrize("k,seed", KS)
def test_initial_partition_matches_reference(name, k, seed):
    g = _graph(name)
    part, obj = cm.initial_partition(g, k, seed)
    ref = Z["%s_k%d_s%d_part" % (name, k, seed)]
    assert obj == int(Z["%s_k%d_s%d_obj" % (name, k, seed)])
    np.testing.assert_array_equal(part, ref)


def test_initial_partition_properties():
    g = _graph("3elt")
    part, obj = cm.initial_partition(g, 8, 1)
    assert part.min() >= 0 and part.max() < 8
    assert len(np.unique(part)) == 8
    # the bisection objectives sum to at least the final cut
    assert obj >= g.edge_cut(part)
    pw = np.bincount(part, weights=g.vwgt, minlength=8)
    assert pw.max() / (g.vwgt.sum() / 8) < 1.10


def test_initial_partition_one_part_and_empty():
    g = _graph("tri69")
    part, obj = cm.initial_partition(g, 1, 1)
    assert (part == 0).all() and obj == 0
    e = cm.Graph(np.zeros(1, np.int32), np.zeros(0, np.int32))
    part, obj = cm.initial_partition(e, 4, 1)
    assert len(part) == 0 and obj == 0


def test_initial_partition_seed_changes_result():
    g = _graph("rgg3000")
    a, _ = cm.initial_partition(g, 8, 1)
    b, _ = cm.initial_partition(g, 8, 7)
    assert not np.array_equal(a, b)


def test_initial_partition_rejects_bad_arguments():
    g = _graph("tri69")
    with pytest.raises(cm.CMError):
        cm.initial_partition(g, 0, 1)
