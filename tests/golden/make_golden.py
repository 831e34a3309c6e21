"""Generates tests/golden/*.npz from the reference's own CPU code: its CPU
coarsening (one file per graph) and its initial partition (initpart.npz).

Run here, where the reference tree is present (it builds the include-harness
oracle/_ref/libref.so around the unmodified reference sources):

    python tests/golden/make_golden.py

For every case the harness seeds the reference's rand() stream once
(srand(seed)) and then runs the reference's level loop (cuMetis_cpu_coarsen,
cuMetis.cu:1854-1875): cuMetis_cpu_match (cu:830), which contracts with
cuMetis_cpu_create_cgraph (cu:737), until n <= threshold, n >= 0.75 n_finer or
m <= n/2.  Each level's input graph, its cmap (the reference's coarse-vertex
numbering) and the final coarse graph are stored; the matching is the pairing
that cmap induces.  Coarse rows are stored as the reference emits them
(first-seen order).
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402
import cumetis_gb300 as cm  # noqa: E402

from oracle.build import REF_TREE  # noqa: E402  ($CM_REFERENCE_TREE, else reference/ beside the repository)


def read_mtx_symmetric(path):
    """Pattern/real symmetric or general Matrix Market -> A + A^T without the
    diagonal, unit weights, rows sorted (what the reference's mtx_to_graph
    converter produces, cu mtx_to_graph.c:110-309)."""
    with open(path) as f:
        header = f.readline()
        line = f.readline()
        while line.startswith("%"):
            line = f.readline()
        nr, nc, nnz = (int(x) for x in line.split()[:3])
        data = np.loadtxt(f, usecols=(0, 1), dtype=np.int64, ndmin=2)
    i, j = data[:, 0] - 1, data[:, 1] - 1
    keep = i != j
    i, j = i[keep], j[keep]
    lo, hi = np.minimum(i, j), np.maximum(i, j)
    keys = np.unique(lo * nr + hi)
    lo, hi = keys // nr, keys % nr
    src = np.concatenate([lo, hi])
    dst = np.concatenate([hi, lo])
    order = np.lexsort((dst, src))
    src, dst = src[order], dst[order]
    xadj = np.zeros(nr + 1, np.int64)
    np.add.at(xadj, src + 1, 1)
    xadj = np.cumsum(xadj)
    return O.CSR(xadj, dst, np.ones(len(dst)), np.ones(nr))


def weighted_grid(nx, ny):
    """5-point grid with vertex weights 1..4 and symmetric edge weights 1..9."""
    g = cm.gen_grid2d(nx, ny)
    n = g.nvtxs
    row = np.repeat(np.arange(n), np.diff(g.xadj))
    lo, hi = np.minimum(row, g.adjncy), np.maximum(row, g.adjncy)
    w = 1 + (lo * 7919 + hi * 104729) % 9
    vw = 1 + (np.arange(n) * 31) % 4
    return O.CSR(g.xadj, g.adjncy, w, vw)


def to_csr(g):
    return O.CSR(g.xadj, g.adjncy, g.adjwgt, g.vwgt)


def threshold_kway(n, k):
    return cm.coarsen_threshold(n, k)


def ref_coarsen(g, threshold, seed, max_levels=32):
    maxvwgt = O.maxvwgt_rule(int(g.vwgt.sum()), threshold)
    O.ref_harness_srand(seed)
    levels = [g]
    cmaps = []
    cur = g
    while True:
        cg, cmap = O.ref_harness_match_contract(cur, maxvwgt)
        cmaps.append(cmap)
        levels.append(cg)
        prev, cur = cur, cg
        if not (cur.n > threshold and cur.n < 0.75 * prev.n and cur.m > cur.n // 2) or len(cmaps) >= max_levels:
            break
    return levels, cmaps, maxvwgt


def two_grids():
    """Two disconnected 20x20 grids (the bisection must restart its BFS)."""
    g = cm.gen_grid2d(20, 20)
    n, m = g.nvtxs, g.nedges
    xadj = np.concatenate([g.xadj, g.xadj[1:] + m])
    adj = np.concatenate([g.adjncy, g.adjncy + n])
    return O.CSR(xadj, adj, np.ones(2 * m), np.ones(2 * n))


# Initial-partition cases: graph, then (nparts, seed) pairs.  The reference's
# cuMetis_rbbisection (cu:3046) runs with its rand() stream seeded by srand(seed).
INITPART_KS = ((2, 1), (3, 1), (5, 4), (8, 1), (8, 2), (16, 3), (64, 1))


def make_initpart(cases):
    out = {}
    for name, g in cases.items():
        out[name + "_xadj"], out[name + "_adjncy"] = g.xadj, g.adjncy
        out[name + "_adjwgt"], out[name + "_vwgt"] = g.adjwgt, g.vwgt
        for k, seed in INITPART_KS:
            part, obj = O.ref_harness_rbbisection(g, k, seed)
            out["%s_k%d_s%d_part" % (name, k, seed)] = part
            out["%s_k%d_s%d_obj" % (name, k, seed)] = np.int32(obj)
    out["names"] = np.array(sorted(cases))
    out["ks"] = np.array(INITPART_KS, np.int32)
    np.savez_compressed(os.path.join(HERE, "initpart.npz"), **out)
    print("initpart.npz", len(cases), "graphs")


def main():
    if O.ref() is None:
        sys.exit("reference tree not found; golden fixtures can only be generated where it is present")
    cases = {
        "3elt": (read_mtx_symmetric(os.path.join(REF_TREE, "mtx", "3elt.mtx")), 8),
        "tri69": (to_csr(cm.gen_tri_grid(69, 69)), 8),
        "rmat10": (to_csr(cm.gen_rmat(10, 16, seed=1)), 8),
        "wgrid40": (weighted_grid(40, 40), 4),
    }
    for name, (g, k) in cases.items():
        thr = threshold_kway(g.n, k)
        out = {"threshold": np.int32(thr), "nparts": np.int32(k)}
        for seed in (1, 2):
            levels, cmaps, maxvwgt = ref_coarsen(g, thr, seed)
            p = "s%d_" % seed
            out[p + "nlevels"] = np.int32(len(cmaps))
            out[p + "maxvwgt"] = np.int32(maxvwgt)
            for l, lg in enumerate(levels):
                if l == 0 and seed != 1:
                    continue  # level 0 is the same input for every seed
                q = "L%d_" % l if l > 0 else ""
                out[p + q + "xadj" if l > 0 else "xadj"] = lg.xadj
                out[p + q + "adjncy" if l > 0 else "adjncy"] = lg.adjncy
                out[p + q + "adjwgt" if l > 0 else "adjwgt"] = lg.adjwgt
                out[p + q + "vwgt" if l > 0 else "vwgt"] = lg.vwgt
            for l, cmap in enumerate(cmaps):
                out[p + "L%d_cmap" % l] = cmap
            print(name, "seed", seed, "levels", [lg.n for lg in levels], "maxvwgt", maxvwgt)
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)

    make_initpart({"tri69": to_csr(cm.gen_tri_grid(69, 69)), "rmat10": to_csr(cm.gen_rmat(10, 16, seed=1)),
                   "wgrid40": weighted_grid(40, 40), "rgg3000": to_csr(cm.gen_rgg(3000, 8.0, seed=3)),
                   "two_grids": two_grids(),
                   "3elt": read_mtx_symmetric(os.path.join(REF_TREE, "mtx", "3elt.mtx"))})


if __name__ == "__main__":
    main()
