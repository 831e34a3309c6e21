"""k-way refinement, projection and the whole partition driver on the GPU,
through the C ABI, against the oracle's restatement of the reference's
refinement (cuMetis.cu:3236-3514).

With two parts the refinement is deterministic (one part group moves per
phase), so partitions are compared bit for bit, up to the whole pipeline
(coarsening -> initial partition -> refinement and projection per level).
With more parts the part threads interleave their balance checks as in the
reference; there every move is checked against the boundary targets of the
starting partition."""
import numpy as np
import pytest

import cumetis_gb300 as cm
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _o(g):
    return O.CSR(g.xadj, g.adjncy, g.adjwgt, g.vwgt)


def _perturbed_partition(g, k, seed, frac=0.15):
    part, _ = cm.initial_partition(g, k, 1)
    rng = np.random.default_rng(seed)
    flip = rng.random(g.nvtxs) < frac
    part = part.copy()
    part[flip] = rng.integers(0, k, flip.sum())
    return part.astype(np.int32)


def _refine_gpu(ctx, g, k, where):
    import torch
    dg = g.to_device()
    w = torch.from_numpy(where.copy()).cuda()
    moves = ctx.refine_kway(dg, k, w)
    torch.cuda.synchronize()
    return w.cpu().numpy(), moves


GRAPHS = {
    "tri69": lambda: cm.gen_tri_grid(69, 69),
    "grid60x40": lambda: cm.gen_grid2d(60, 40),
    "rmat11": lambda: cm.gen_rmat(11, 16, seed=2),
    "rgg5000": lambda: cm.gen_rgg(5000, 8.0, seed=5),
}


@pytest.mark.parametrize("name", sorted(GRAPHS))
def test_refine_two_parts_exact(ctx, name):
    g = GRAPHS[name]()
    for seed in (1, 2):
        where0 = _perturbed_partition(g, 2, seed)
        got, moves = _refine_gpu(ctx, g, 2, where0)
        want, wmoves = O.refine_kway_model(_o(g), where0, 2)
        np.testing.assert_array_equal(got, want)
        assert moves == wmoves


@pytest.mark.parametrize("name", sorted(GRAPHS))
@pytest.mark.parametrize("k", [3, 8, 64])
def test_refine_kway_moves_follow_targets(ctx, name, k):
    g = GRAPHS[name]()
    where0 = _perturbed_partition(g, k, 3)
    got, moves = _refine_gpu(ctx, g, k, where0)
    flag, target = O.boundary_targets(_o(g), where0, k)
    changed = got != where0
    assert changed.sum() == moves
    assert flag[changed].all(), "only boundary vertices move"
    np.testing.assert_array_equal(got[changed], target[changed])
    assert got.min() >= 0 and got.max() < k
    # every part's weight changed only by accepted moves: totals are preserved
    assert np.bincount(got, weights=g.vwgt, minlength=k).sum() == g.vwgt.sum()


def test_refine_many_parts_global_accumulators(ctx):
    """k above the shared-memory accumulator limit (1024) uses per-warp
    global slices."""
    g = cm.gen_grid2d(120, 100)
    k = 1500
    rng = np.random.default_rng(4)
    where0 = (np.arange(g.nvtxs) // 8 % k).astype(np.int32)
    flip = rng.random(g.nvtxs) < 0.2
    where0[flip] = rng.integers(0, k, flip.sum())
    got, moves = _refine_gpu(ctx, g, k, where0)
    flag, target = O.boundary_targets(_o(g), where0, k)
    changed = got != where0
    assert changed.sum() == moves and flag[changed].all()
    np.testing.assert_array_equal(got[changed], target[changed])


def test_project(ctx):
    import torch
    rng = np.random.default_rng(1)
    n, cn = 10000, 3000
    cmap = rng.integers(0, cn, n).astype(np.int32)
    cwhere = rng.integers(0, 17, cn).astype(np.int32)
    w = torch.empty(n, dtype=torch.int32, device="cuda")
    ctx.project(torch.from_numpy(cmap).cuda(), torch.from_numpy(cwhere).cuda(), w)
    np.testing.assert_array_equal(w.cpu().numpy(), cwhere[cmap])


def _pipeline_model(g, k, seed, threshold):
    levels = O.coarsen(_o(g), threshold, mode=1)  # cm_part_graph's default: hash-ordered ties
    coarsest = levels[-1][0]
    where, _ = cm.initial_partition(cm.Graph(coarsest.xadj, coarsest.adjncy, coarsest.adjwgt, coarsest.vwgt), k, seed)
    where = np.asarray(where, np.int32)
    where, _ = O.refine_kway_model(coarsest, where, k)
    for lg, _, cmap in reversed(levels[:-1]):
        where = where[cmap]
        where, _ = O.refine_kway_model(lg, where, k)
    return where


@pytest.mark.parametrize("name", ["tri69", "rmat11"])
def test_part_graph_two_parts_matches_pipeline_model(ctx, name):
    g = GRAPHS[name]()
    thr = cm.coarsen_threshold(g.nvtxs, 2)
    part, cut, st = ctx.part_graph(g, 2, seed=1)
    want = _pipeline_model(g, 2, 1, thr)
    np.testing.assert_array_equal(part, want)
    assert cut == g.edge_cut(part)
    assert st["edge_cut"] == cut and st["levels"] >= 2


def test_blocking_waits_same_result():
    """A context that sleeps on blocking-sync events while the GPU works (the
    engine workers' setting) gives the same two-part partition as a spinning
    one, through the whole pipeline."""
    g = GRAPHS["rmat11"]()
    a, b = cm.Context(0), cm.Context(0)
    try:
        b.set_blocking_waits(True)
        pa, ca, _ = a.part_graph(g, 2, seed=3)
        pb, cb, _ = b.part_graph(g, 2, seed=3)
        np.testing.assert_array_equal(pa, pb)
        assert ca == cb
        h = b.coarsen(g, cm.coarsen_threshold(g.nvtxs, 8))
        assert len(h) >= 2
        h.close()
    finally:
        a.close()
        b.close()


@pytest.mark.parametrize("k", [4, 8, 64])
def test_part_graph_kway_quality(ctx, k):
    g = cm.gen_grid2d(200, 150)
    part, cut, st = ctx.part_graph(g, k, seed=1)
    assert part.min() >= 0 and part.max() < k and len(np.unique(part)) == k
    assert cut == g.edge_cut(part)
    pw = np.bincount(part, weights=g.vwgt, minlength=k)
    assert pw.max() * k / g.vwgt.sum() < 1.10
    # refinement does not lose to the projected initial partition by much and
    # usually wins; the initial cut is of the coarsest graph, equal weightwise
    assert cut <= st["initial_cut"] * 1.05 + 10


def test_part_graph_unit_weights_and_dropin(ctx):
    import ctypes
    g = cm.gen_tri_grid(40, 40)
    n = g.nvtxs
    part = np.zeros(n, np.int32)
    obj = np.zeros(1, np.int32)
    nv = np.array([n], np.int32)
    nparts = np.array([8], np.int32)
    L = cm.lib()
    p = lambda a: a.ctypes.data_as(ctypes.POINTER(ctypes.c_int32))
    rc = L.cuMetis_PartGraph(p(nv), p(g.xadj), p(g.adjncy), None, None, p(nparts), None, None, p(obj), p(part))
    assert rc == 1, cm.lib().cm_last_error()
    assert part.max() < 8 and part.min() >= 0
    assert obj[0] == g.edge_cut(part)
    pw = np.bincount(part, minlength=8)
    assert pw.max() * 8 / n < 1.10


def test_part_graph_trivial(ctx):
    g = cm.gen_grid2d(10, 10)
    part, cut, _ = ctx.part_graph(g, 1)
    assert (part == 0).all() and cut == 0


def test_cli_partitions_a_graph_file(tmp_path):
    import os
    import subprocess
    g = cm.gen_tri_grid(30, 30)
    path = str(tmp_path / "tri30.graph")
    cm.write_graph(path, g) if hasattr(cm, "write_graph") else None
    if not os.path.exists(path):
        with open(path, "w") as f:
            f.write("%d %d\n" % (g.nvtxs, g.nedges // 2))
            for v in range(g.nvtxs):
                f.write(" ".join(str(int(x) + 1) for x in g.adjncy[g.xadj[v]:g.xadj[v + 1]]) + "\n")
    exe = os.path.join(os.path.dirname(cm.LIB_PATH), "cuMetis")
    r = subprocess.run([exe, path, "4", "--seed", "2"], stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True,
                       timeout=120)
    assert r.returncode == 0, r.stderr
    assert "cuMetis-Partition-end" in r.stdout and "Edge-cut=" in r.stdout
    part = np.loadtxt(path + ".part.4", dtype=np.int64)
    assert len(part) == g.nvtxs and part.min() >= 0 and part.max() < 4
    cut = int(r.stdout.split("Edge-cut=")[1].split()[0])
    assert cut == g.edge_cut(part.astype(np.int32))
