"""Many graphs coarsened together (cm_coarsen_batch): every level of the
disjoint union is one matching and one contraction for all graphs, and each
graph's hierarchy must equal, level for level and bit for bit, the coarsening
of that graph alone."""
import numpy as np
import pytest

import cumetis_gb300 as cm

pytestmark = pytest.mark.gpu


def _batch_graphs():
    gs = [cm.gen_rgg(int(n), 8.0, seed=int(s)) for n, s in ((1000, 1), (3000, 2), (8000, 3), (20000, 4), (1500, 5))]
    gs += [cm.gen_grid2d(40, 30), cm.gen_grid3d(12, 12, 12), cm.gen_tri_grid(50, 50), cm.gen_rmat(12, 16, seed=3),
           cm.gen_rmat(10, 8, seed=9)]
    gs.append(cm.Graph(np.arange(0, 1, dtype=np.int32) * 0, [], [], []))            # no vertices
    gs.append(cm.Graph(np.zeros(31, np.int32), [], [], np.arange(1, 31)))            # no edges
    g = cm.gen_grid2d(30, 30)
    gs.append(cm.Graph(g.xadj, g.adjncy, g.adjwgt, (1 + np.arange(g.nvtxs) % 7).astype(np.int32)))  # weighted
    return gs


@pytest.mark.parametrize("mode", [0, 1])
def test_batch_hierarchies_equal_single_coarsening(ctx, mode):
    gs = _batch_graphs()
    ks = [2, 4, 8, 16, 32, 64, 2, 8, 256, 16, 4, 2, 8]
    thr = [cm.coarsen_threshold(max(g.nvtxs, 1), k) for g, k in zip(gs, ks)]
    hs = ctx.coarsen_batch(gs, thr, mode)
    assert len(hs) == len(gs)
    for i, (g, t, h) in enumerate(zip(gs, thr, hs)):
        alone = ctx.coarsen(g, t, mode)
        assert h.sizes() == alone.sizes(), i
        for l in range(len(h)):
            bg, bc, bm = h.copy_level(l)
            ag, ac, am = alone.copy_level(l)
            for f in ("xadj", "adjncy", "adjwgt", "vwgt"):
                assert np.array_equal(getattr(bg, f), getattr(ag, f)), (i, l, f)
            if ac is not None:
                assert np.array_equal(bc, ac) and np.array_equal(bm, am), (i, l)
        alone.close()
        h.close()


def test_batch_hierarchies_outlive_each_other(ctx):
    """Graphs of one batch share device allocations per level; freeing the
    hierarchies in any order leaves the others intact."""
    gs = [cm.gen_grid2d(50 + 7 * i, 40) for i in range(6)]
    hs = ctx.coarsen_batch(gs, 100, 1)
    want = [ctx.coarsen(g, 100, 1) for g in gs]
    for i in (3, 0, 5):
        hs[i].close()
    for i in (1, 2, 4):
        assert hs[i].sizes() == want[i].sizes()
        a, _, _ = hs[i].copy_level(len(hs[i]) - 1)
        b, _, _ = want[i].copy_level(len(want[i]) - 1)
        assert np.array_equal(a.adjncy, b.adjncy) and np.array_equal(a.xadj, b.xadj)
    for h in hs + want:
        h.close()
