"""Generates tests/golden/quality.json: edge cut and imbalance of the
reference's k-way pipeline over 10 seeds, emulated on the host from the
reference's own code, for the quality comparison in
tests/test_quality_gpu.py.

Run here, where the reference tree is present (the include-harness
oracle/_ref/libref.so is built around the unmodified sources):

    python tests/golden/make_quality.py [--cases a,b] [--jobs J] [--seeds 1,2,..]

(--jobs runs the seeds of a case in J worker processes, each holding a copy
of the graph's levels -- about 11 GB for rmat22_k256; --cases recomputes the
named cases and keeps the others of an existing quality.json.)

Per seed s: srand(s); coarsening with the reference's CPU heavy-edge matching
and contraction (cuMetis_cpu_match, cuMetis.cu:830 -- a restatement of its GPU
matching, which is racy and cannot run here) under cuMetis_coarsen's stop rule
and k-way threshold (cu:1824-1850, 3634); the reference's initial partition
cuMetis_rbbisection (cu:3046) continuing the same rand() stream; then per
level, coarsest to finest, the projection and one pass of the reference's
k-way refinement (cu:3494-3514) with its part threads run one after another
(oracle or_refine_kway).
"""
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402
import cumetis_gb300 as cm  # noqa: E402

SEEDS = list(range(1, 11))
CASES = {
    # name: (generator, k)
    "tri69_k8": (lambda: cm.gen_tri_grid(69, 69), 8),
    "grid725_k64": (lambda: cm.gen_grid2d(725, 725), 64),
    "rmat18_k256": (lambda: cm.gen_rmat(18, 16, 0.57, 0.19, 0.19, 1, 1, 100), 256),
    "rmat22_k256": (lambda: cm.gen_rmat(22, 16, 0.57, 0.19, 0.19, 1, 1, 100), 256),
}


def ref_pipeline(g, k, seed):
    thr = cm.coarsen_threshold(g.n, k)
    maxvwgt = O.maxvwgt_rule(int(g.vwgt.sum()), thr)
    O.ref_harness_srand(seed)
    levels, cmaps, cur = [g], [], g
    while True:
        cg, cmap = O.ref_harness_match_contract(cur, maxvwgt)
        cmaps.append(cmap)
        levels.append(cg)
        prev, cur = cur, cg
        if not (cur.n > thr and cur.n < 0.75 * prev.n and cur.m > cur.n // 2):
            break
    where, _ = O.ref_harness_rbbisection(levels[-1], k, None)
    where = np.asarray(where, np.int32)
    where, _ = O.refine_kway_c(levels[-1], where, k)
    for lg, cmap in zip(reversed(levels[:-1]), reversed(cmaps)):
        where = where[cmap]
        where, _ = O.refine_kway_c(lg, where, k)
    return where, len(levels), levels[-1].n


def _seed_run(args):
    name, s = args
    gen, k = CASES[name]
    hg = gen()
    g = O.CSR(hg.xadj, hg.adjncy, hg.adjwgt, hg.vwgt)
    where, nl, cn = ref_pipeline(g, k, s)
    pw = np.bincount(where, weights=g.vwgt, minlength=k)
    return int(hg.edge_cut(where)), float(pw.max() * k / g.vwgt.sum()), [nl, cn]


def main():
    import argparse
    import concurrent.futures as cf
    import multiprocessing as mp
    ap = argparse.ArgumentParser()
    ap.add_argument("--cases", default=",".join(CASES))
    ap.add_argument("--jobs", type=int, default=1)
    ap.add_argument("--seeds", default=",".join(map(str, SEEDS)),
                    help="initial-partition seeds (rmat22_k256 uses 1-4: about 2 h of host time per seed)")
    args = ap.parse_args()
    seeds = [int(x) for x in args.seeds.split(",")]
    if O.ref() is None:
        sys.exit("reference tree not found; quality fixtures can only be generated where it is present")
    path = os.path.join(HERE, "quality.json")
    out = json.load(open(path)) if os.path.exists(path) else {}
    for name in args.cases.split(","):
        gen, k = CASES[name]
        hg = gen()
        t0 = time.time()
        if args.jobs > 1:  # a worker that dies (e.g. out of memory) fails the run instead of hanging it
            with cf.ProcessPoolExecutor(args.jobs, mp_context=mp.get_context("spawn")) as ex:
                res = list(ex.map(_seed_run, [(name, s) for s in seeds]))
        else:
            res = [_seed_run((name, s)) for s in seeds]
        cuts = [r[0] for r in res]
        imbs = [r[1] for r in res]
        lv = [r[2] for r in res]
        out[name] = {"k": k, "nvtxs": hg.nvtxs, "nedges": hg.nedges, "seeds": seeds, "cut": cuts, "imbalance": imbs,
                     "levels_coarsest": lv, "mean_cut": float(np.mean(cuts)), "mean_imbalance": float(np.mean(imbs))}
        print(name, "mean cut %.1f  mean imbalance %.4f  (%.1f s)" % (np.mean(cuts), np.mean(imbs), time.time() - t0),
              flush=True)
        with open(path, "w") as f:
            json.dump(out, f, indent=1)


if __name__ == "__main__":
    main()
