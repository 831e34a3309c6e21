"""CPU tests of the oracle itself: pinned against the reference's own
outputs (tests/golden, produced by the reference's CPU coarsening) before
anything else is checked against it."""
import numpy as np
import pytest

from conftest import GOLDEN_CASES, load_golden
from oracle import oracle as O


def _rows_sorted_equal(a, b):
    assert np.array_equal(a.xadj, b.xadj)
    aa, aw = a.rows_sorted()
    ba, bw = b.rows_sorted()
    assert np.array_equal(aa, ba)
    assert np.array_equal(aw, bw)
    assert np.array_equal(a.vwgt, b.vwgt)


@pytest.mark.parametrize("name", GOLDEN_CASES)
def test_oracle_contraction_reproduces_reference(name):
    """Given the reference's matching, the oracle's cmap and coarse graph equal
    the reference's cuMetis_cpu_create_cgraph output at every level (rows
    compared as sorted sets: the reference CPU path emits first-seen order,
    its GPU path sorts by coarse id)."""
    G = load_golden(name)
    for seed, (maxvwgt, graphs, cmaps) in G["seeds"].items():
        for l, cmap in enumerate(cmaps):
            match = O.match_from_cmap(cmap)
            cg, ocmap = O.contract(graphs[l], match)
            assert np.array_equal(ocmap, cmap), (name, seed, l)
            _rows_sorted_equal(cg, graphs[l + 1])


@pytest.mark.parametrize("name", GOLDEN_CASES)
def test_restated_reference_cpu_coarsening_is_exact(name):
    """The oracle's restatement of cuMetis_cpu_match/cuMetis_cpu_create_cgraph
    (used as the timed CPU baseline) reproduces the reference bit for bit,
    including the rand() stream and first-seen row order."""
    G = load_golden(name)
    for seed, (maxvwgt, graphs, cmaps) in G["seeds"].items():
        O.srand(seed)
        for l, cmap in enumerate(cmaps):
            cg, ocmap, _ = O.ref_cpu_coarsen_level(graphs[l], maxvwgt)
            assert np.array_equal(ocmap, cmap), (name, seed, l)
            nxt = graphs[l + 1]
            assert np.array_equal(cg.xadj, nxt.xadj)
            assert np.array_equal(cg.adjncy, nxt.adjncy)
            assert np.array_equal(cg.adjwgt, nxt.adjwgt)
            assert np.array_equal(cg.vwgt, nxt.vwgt)


@pytest.mark.parametrize("name", GOLDEN_CASES)
def test_reference_matchings_are_legal(name):
    G = load_golden(name)
    for seed, (maxvwgt, graphs, cmaps) in G["seeds"].items():
        for l, cmap in enumerate(cmaps):
            code, bad, _ = O.check_matching(graphs[l], maxvwgt, O.match_from_cmap(cmap), require_light=False)
            assert code == 0, (name, seed, l, code, bad)


def _small_graphs():
    import cumetis_gb300 as cm
    out = {
        "tri30": cm.gen_tri_grid(30, 30),
        "grid2d_17x23": cm.gen_grid2d(17, 23),
        "grid3d_7": cm.gen_grid3d(7, 7, 7),
        "rmat11": cm.gen_rmat(11, 8, seed=3),
        "rgg3000": cm.gen_rgg(3000, 8.0, seed=5),
    }
    return {k: O.CSR(g.xadj, g.adjncy, g.adjwgt, g.vwgt) for k, g in out.items()}


@pytest.mark.parametrize("mode", [0, 1])
def test_greedy_equals_rounds(mode):
    """Two independent statements of the deterministic matching agree."""
    for name, g in _small_graphs().items():
        mv = O.maxvwgt_rule(int(g.vwgt.sum()), 100)
        a = O.match_greedy(g, mv, mode)
        b, rounds = O.match_rounds(g, mv, mode)
        assert np.array_equal(a, b), name
        code, bad, maximal = O.check_matching(g, mv, a)
        assert code == 0 and maximal, (name, code, bad)


def test_tie_break_lower_id():
    # path 0-1-2-3 with unit weights: greedy in (lo, hi) order pairs (0,1), (2,3)
    g = O.CSR([0, 1, 3, 5, 6], [1, 0, 2, 1, 3, 2], [1] * 6, [1] * 4)
    assert list(O.match_greedy(g, 10, 0)) == [1, 0, 3, 2]
    # heavier middle edge wins: 1-2 weight 5
    g = O.CSR([0, 1, 3, 5, 6], [1, 0, 2, 1, 3, 2], [1, 1, 5, 5, 1, 1], [1] * 4)
    assert list(O.match_greedy(g, 10, 0)) == [0, 2, 1, 3]


def test_light_rule_and_cap():
    # two heavy vertices (3*vwgt >= maxvwgt) may not pair; a light one may join a heavy one
    g = O.CSR([0, 1, 3, 4], [1, 0, 2, 1], [1, 1, 1, 1], [10, 10, 1])
    m = O.match_greedy(g, 29, 0)
    assert list(m) == [0, 2, 1]
    # cap: 10 + 25 > 29
    g = O.CSR([0, 1, 2], [1, 0], [1, 1], [10, 25])
    assert list(O.match_greedy(g, 29, 0)) == [0, 1]


def test_contract_edge_cases():
    # isolated vertices, a star, and an input self loop (dropped by the GPU contract)
    xadj = [0, 0, 3, 4, 5, 6, 6, 8]
    adj = [2, 3, 4, 1, 1, 1, 6, 6]
    # vertex 6 has a self loop twice? make it a proper self loop + nothing else
    g = O.CSR([0, 0, 3, 4, 5, 6, 6, 7], [2, 3, 4, 1, 1, 1, 6], [1, 2, 3, 1, 2, 3, 9], [1] * 7)
    match = np.array([0, 2, 1, 3, 4, 5, 6], np.int32)
    cg, cmap = O.contract(g, match)
    assert list(cmap) == [0, 1, 1, 2, 3, 4, 5]
    assert list(cg.xadj) == [0, 0, 2, 3, 4, 4, 4]
    assert list(cg.adjncy) == [2, 3, 1, 1]
    assert list(cg.adjwgt) == [2, 3, 2, 3]
    assert list(cg.vwgt) == [1, 2, 1, 1, 1, 1]


def test_contract_duplicate_merge():
    # square 0-1-2-3-0 with (0,1) and (2,3) matched: coarse edge weight = 2 edges summed
    g = O.CSR([0, 2, 4, 6, 8], [1, 3, 0, 2, 1, 3, 0, 2], [1, 2, 1, 3, 3, 4, 2, 4], [1] * 4)
    match = np.array([1, 0, 3, 2], np.int32)
    cg, _ = O.contract(g, match)
    assert list(cg.xadj) == [0, 1, 2]
    assert list(cg.adjncy) == [1, 0]
    assert list(cg.adjwgt) == [5, 5]
    assert list(cg.vwgt) == [2, 2]


def test_coarsen_loop_stop_rule():
    import cumetis_gb300 as cm
    g = cm.gen_tri_grid(69, 69)
    og = O.CSR(g.xadj, g.adjncy, g.adjwgt, g.vwgt)
    levels = O.coarsen(og, 240)
    ns = [lv[0].n for lv in levels]
    assert ns[0] == 4761 and ns[-1] <= 240 or ns[-1] >= 0.75 * ns[-2]
    for a, b in zip(ns, ns[1:]):
        assert b < a


def test_refine_model_c_equals_python():
    import cumetis_gb300 as cm
    for g, k in ((cm.gen_tri_grid(40, 40), 2), (cm.gen_tri_grid(40, 40), 8), (cm.gen_rmat(10, 16, seed=3), 16),
                 (cm.gen_grid2d(30, 50), 64)):
        og = O.CSR(g.xadj, g.adjncy, g.adjwgt, g.vwgt)
        rng = np.random.default_rng(k)
        where = rng.integers(0, k, g.nvtxs).astype(np.int32)
        a, ma = O.refine_kway_model(og, where, k)
        b, mb = O.refine_kway_c(og, where, k)
        np.testing.assert_array_equal(a, b)
        assert ma == mb


def test_oracle_generators_equal_the_library_generators():
    """The CPU arm builds its inputs with the oracle's restated generators;
    they must produce the library's graphs exactly."""
    import cumetis_gb300 as cm
    pairs = [(O.gen_rmat(12, 16, 0.57, 0.19, 0.19, 1, 1, 100), cm.gen_rmat(12, 16, 0.57, 0.19, 0.19, 1, 1, 100)),
             (O.gen_rmat(9, 8, 0.6, 0.15, 0.15, 7, 1, 5), cm.gen_rmat(9, 8, 0.6, 0.15, 0.15, 7, 1, 5)),
             (O.gen_grid2d(37, 21), cm.gen_grid2d(37, 21)), (O.gen_tri_grid(19, 23), cm.gen_tri_grid(19, 23))]
    for og, g in pairs:
        for f in ("xadj", "adjncy", "adjwgt", "vwgt"):
            assert np.array_equal(getattr(og, f), getattr(g, f)), f
