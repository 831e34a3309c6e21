"""Partition quality over 10 seeds against the reference's k-way pipeline
emulated from its own code (tests/golden/quality.json, made by
tests/golden/make_quality.py): edge cut and imbalance of cm_part_graph with
initial-partition seeds 1..10.  The numbers are printed (pytest -s) and bound
loosely; the emulated reference matches with its CPU heavy-edge matching in
place of its racy GPU one."""
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
}


@pytest.mark.parametrize("name", sorted(GEN))
def test_quality_against_reference_pipeline(ctx, name):
    ref = REF[name]
    k = ref["k"]
    g = GEN[name]()
    assert g.nvtxs == ref["nvtxs"] and g.nedges == ref["nedges"]
    cuts, imbs = [], []
    for s in ref["seeds"]:
        part, cut, st = ctx.part_graph(g, k, seed=s)
        assert cut == g.edge_cut(part)
        cuts.append(cut)
        imbs.append(float(np.bincount(part, weights=g.vwgt, minlength=k).max() * k / g.vwgt.sum()))
    mc, mi = float(np.mean(cuts)), float(np.mean(imbs))
    print("\nquality %s: ours mean cut %.1f (imbalance %.4f)  reference-pipeline mean cut %.1f (imbalance %.4f)  "
          "ratio %.4f" % (name, mc, mi, ref["mean_cut"], ref["mean_imbalance"], mc / ref["mean_cut"]))
    assert mc <= 1.10 * ref["mean_cut"]
    assert mi <= 1.10
