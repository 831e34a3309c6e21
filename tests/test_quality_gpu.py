"""Partition quality against the reference's k-way pipeline run from its
own code (tests/golden/quality.json, made by tests/golden/make_quality.py):
edge cut and imbalance of cm_part_graph with the fixture's initial-partition
seeds (1..10; fewer where the fixture says so).  The mean cut must be within
1% of the reference pipeline's and the mean imbalance within 1.10.  The
reference pipeline matches with its CPU heavy-edge matching (its GPU
matching is racy and cannot run where the fixtures are made); its initial
partition and k-way refinement are its own code."""
import json
import os

import numpy as np
import pytest

import cumetis_gb300 as cm
from conftest import GOLDEN

pytestmark = pytest.mark.gpu

REF = json.load(open(os.path.join(GOLDEN, "quality.json")))
GEN = {
    "tri69_k8": lambda: cm.gen_tri_grid(69, 69),
    "grid725_k64": lambda: cm.gen_grid2d(725, 725),
    "rmat18_k256": lambda: cm.gen_rmat(18, 16, 0.57, 0.19, 0.19, 1, 1, 100),
    "rmat22_k256": lambda: cm.gen_rmat(22, 16, 0.57, 0.19, 0.19, 1, 1, 100),
}
GEN = {k: v for k, v in GEN.items() if k in REF}


@pytest.mark.parametrize("name", sorted(GEN))
def test_quality_against_reference_pipeline(ctx, name):
    ref = REF[name]
    k = ref["k"]
    g = GEN[name]()
    assert g.nvtxs == ref["nvtxs"] and g.nedges == ref["nedges"]
    cuts, imbs = [], []
    for s in ref["seeds"]:
        part, cut, st = ctx.part_graph(g, k, seed=s)
        ec = g.edge_cut(part)
        assert cut == ((ec + 2**31) % 2**32) - 2**31  # objval is int32 and wraps (R-MAT 22: cut > 2^31)
        cuts.append(ec)
        imbs.append(float(np.bincount(part, weights=g.vwgt, minlength=k).max() * k / g.vwgt.sum()))
    mc, mi = float(np.mean(cuts)), float(np.mean(imbs))
    print("\nquality %s: ours mean cut %.1f (imbalance %.4f)  reference-pipeline mean cut %.1f (imbalance %.4f)  "
          "ratio %.4f" % (name, mc, mi, ref["mean_cut"], ref["mean_imbalance"], mc / ref["mean_cut"]))
    assert mc <= 1.01 * ref["mean_cut"]
    assert mi <= 1.10
