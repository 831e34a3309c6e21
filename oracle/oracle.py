"""ctypes wrapper of the CPU oracle (oracle/liboracle.so) and of the
reference include-harness (oracle/_ref/libref.so, present only where the
reference tree was available at build time).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline leg as the checker; the product never imports it.
"""
import ctypes
import os

import numpy as np

from . import build as _build

_I32P = ctypes.POINTER(ctypes.c_int32)
_lib = None
_ref = None


def _p(a):
    return a.ctypes.data_as(_I32P) if a is not None else None


def lib():
    global _lib
    if _lib is None:
        _lib = ctypes.CDLL(_build.build_oracle())
        L = _lib
        L.or_match_greedy.restype = ctypes.c_int64
        L.or_match_greedy.argtypes = [ctypes.c_int32, _I32P, _I32P, _I32P, _I32P, ctypes.c_int32, ctypes.c_int32, _I32P]
        L.or_match_rounds.restype = ctypes.c_int32
        L.or_match_rounds.argtypes = [ctypes.c_int32, _I32P, _I32P, _I32P, _I32P, ctypes.c_int32, ctypes.c_int32,
                                      ctypes.c_int32, _I32P]
        L.or_check_matching.restype = ctypes.c_int32
        L.or_check_matching.argtypes = [ctypes.c_int32, _I32P, _I32P, _I32P, ctypes.c_int32, ctypes.c_int32, _I32P,
                                        _I32P, _I32P]
        L.or_build_cmap.restype = ctypes.c_int32
        L.or_build_cmap.argtypes = [ctypes.c_int32, _I32P, _I32P, _I32P, _I32P, _I32P, _I32P, _I32P]
        L.or_contract.restype = ctypes.c_int64
        L.or_contract.argtypes = [ctypes.c_int32, _I32P, _I32P, _I32P, _I32P, _I32P, ctypes.c_int32, _I32P,
                                  _I32P, _I32P, _I32P]
        L.or_ref_cpu_match.restype = ctypes.c_int32
        L.or_ref_cpu_match.argtypes = [ctypes.c_int32, _I32P, _I32P, _I32P, _I32P, ctypes.c_int32, _I32P, _I32P]
        L.or_ref_cpu_contract.restype = ctypes.c_int64
        L.or_ref_cpu_contract.argtypes = [ctypes.c_int32, _I32P, _I32P, _I32P, _I32P, _I32P, _I32P, ctypes.c_int32,
                                          _I32P, _I32P, _I32P, _I32P]
        L.or_refine_kway.restype = ctypes.c_int64
        L.or_refine_kway.argtypes = [ctypes.c_int32, _I32P, _I32P, _I32P, _I32P, ctypes.c_int32, _I32P]
        L.or_edge_hash.restype = ctypes.c_uint32
        L.or_edge_hash.argtypes = [ctypes.c_uint32, ctypes.c_uint32]
        L.srand_seed = ctypes.CDLL(None).srand
    return _lib


def ref():
    """The reference include-harness, or None if it was not built here."""
    global _ref
    if _ref is None:
        path = _build.build_ref()
        if path is None or not os.path.exists(path):
            return None
        _ref = ctypes.CDLL(path)
        for name in ("ref_cpu_match_contract", "ref_cpu_contract", "ref_rbbisection"):
            getattr(_ref, name).restype = ctypes.c_int32
    return _ref


def _i32(a):
    return np.ascontiguousarray(a, dtype=np.int32)


class CSR:
    """Plain host CSR with int32 numpy arrays."""

    def __init__(self, xadj, adjncy, adjwgt, vwgt):
        self.xadj, self.adjncy = _i32(xadj), _i32(adjncy)
        self.adjwgt, self.vwgt = _i32(adjwgt), _i32(vwgt)

    @property
    def n(self):
        return len(self.xadj) - 1

    @property
    def m(self):
        return int(self.xadj[-1])

    def rows_sorted(self):
        """(adjncy, adjwgt) with every row sorted by neighbour id."""
        row = np.repeat(np.arange(self.n, dtype=np.int64), np.diff(self.xadj))
        order = np.lexsort((self.adjncy, row))
        return self.adjncy[order], self.adjwgt[order]


def match_greedy(g, maxvwgt, mode=0):
    m = np.empty(g.n, np.int32)
    lib().or_match_greedy(g.n, _p(g.xadj), _p(g.adjncy), _p(g.adjwgt), _p(g.vwgt), int(maxvwgt), int(mode), _p(m))
    return m


def match_rounds(g, maxvwgt, mode=0, max_rounds=1 << 30):
    m = np.empty(g.n, np.int32)
    r = lib().or_match_rounds(g.n, _p(g.xadj), _p(g.adjncy), _p(g.adjwgt), _p(g.vwgt), int(maxvwgt), int(mode),
                              int(max_rounds), _p(m))
    return m, r


def check_matching(g, maxvwgt, match, require_light=True):
    """Returns (code, bad_vertex, maximal); code 0 = legal."""
    bad = np.zeros(1, np.int32)
    mx = np.zeros(1, np.int32)
    code = lib().or_check_matching(g.n, _p(g.xadj), _p(g.adjncy), _p(g.vwgt), int(maxvwgt), int(require_light),
                                   _p(_i32(match)), _p(bad), _p(mx))
    return int(code), int(bad[0]), bool(mx[0])


def build_cmap(g, match):
    n = g.n
    cmap, leader = np.empty(n, np.int32), np.empty(max(n, 1), np.int32)
    cvwgt, eoff = np.empty(max(n, 1), np.int32), np.empty(n + 1, np.int32)
    cn = lib().or_build_cmap(n, _p(g.xadj), _p(g.vwgt), _p(_i32(match)), _p(cmap), _p(leader), _p(cvwgt), _p(eoff))
    return cmap, leader[:cn].copy(), cvwgt[:cn].copy(), eoff[:cn + 1].copy()


def contract(g, match):
    """Coarse CSR (rows sorted by coarse id) and cmap for a given matching."""
    match = _i32(match)
    cmap, leader, cvwgt, _ = build_cmap(g, match)
    cn = len(leader)
    cxadj = np.empty(cn + 1, np.int32)
    cadj, cw = np.empty(max(g.m, 1), np.int32), np.empty(max(g.m, 1), np.int32)
    me = lib().or_contract(g.n, _p(g.xadj), _p(g.adjncy), _p(g.adjwgt), _p(match), _p(cmap), cn, _p(leader),
                           _p(cxadj), _p(cadj), _p(cw))
    return CSR(cxadj, cadj[:me], cw[:me], cvwgt), cmap


def maxvwgt_rule(tvwgt, threshold):
    """(int)(1.5 * tvwgt / threshold), cuMetis.cu:1828."""
    return int(1.5 * tvwgt / threshold)


def coarsen(g, threshold, mode=0, maxvwgt=None, shrink=0.75, max_levels=64):
    """Level loop of cuMetis_coarsen (cu:1824-1850) with the deterministic
    matching.  Returns [(graph, match, cmap), ..., (coarsest, None, None)]."""
    if maxvwgt is None:
        maxvwgt = maxvwgt_rule(int(g.vwgt.sum()), threshold)
    levels = []
    cur = g
    while True:
        match = match_greedy(cur, maxvwgt, mode)
        cg, cmap = contract(cur, match)
        levels.append((cur, match, cmap))
        cur = cg
        if not (cur.n > threshold and cur.n < shrink * levels[-1][0].n and cur.m > cur.n // 2) \
                or len(levels) >= max_levels:
            break
    levels.append((cur, None, None))
    return levels


def srand(seed):
    lib().srand_seed(ctypes.c_uint(seed))


def ref_cpu_coarsen_level(g, maxvwgt):
    """The restated reference CPU coarsening step (cu:830-918), continuing the
    C library rand() stream (seed it with srand()).  Returns (coarse graph with
    rows in first-seen order, cmap, match)."""
    L = lib()
    n = g.n
    match, cmap = np.empty(n, np.int32), np.empty(n, np.int32)
    cn = L.or_ref_cpu_match(n, _p(g.xadj), _p(g.adjncy), _p(g.adjwgt), _p(g.vwgt), int(maxvwgt), _p(match), _p(cmap))
    cxadj, cvwgt = np.empty(cn + 1, np.int32), np.empty(max(cn, 1), np.int32)
    cadj, cw = np.empty(max(g.m, 1), np.int32), np.empty(max(g.m, 1), np.int32)
    me = L.or_ref_cpu_contract(n, _p(g.xadj), _p(g.adjncy), _p(g.adjwgt), _p(g.vwgt), _p(match), _p(cmap), cn,
                               _p(cxadj), _p(cvwgt), _p(cadj), _p(cw))
    return CSR(cxadj, cadj[:me], cw[:me], cvwgt[:cn]), cmap, match


def ref_harness_srand(seed):
    R = ref()
    if R is None:
        raise RuntimeError("reference harness not built (reference tree absent)")
    R.ref_srand(ctypes.c_uint(seed))


def ref_harness_match_contract(g, maxvwgt):
    """The reference's own cuMetis_cpu_match + cuMetis_cpu_create_cgraph
    (continuing the rand() stream; seed it with ref_harness_srand)."""
    R = ref()
    if R is None:
        raise RuntimeError("reference harness not built (reference tree absent)")
    n = g.n
    cmap, cxadj, cvwgt = np.empty(n, np.int32), np.empty(n + 1, np.int32), np.empty(max(n, 1), np.int32)
    cadj, cw, cne = np.empty(max(g.m, 1), np.int32), np.empty(max(g.m, 1), np.int32), np.zeros(1, np.int32)
    cn = R.ref_cpu_match_contract(ctypes.c_int(n), _p(g.xadj), _p(g.adjncy), _p(g.adjwgt), _p(g.vwgt),
                                  ctypes.c_int(int(maxvwgt)), _p(cmap), _p(cxadj), _p(cvwgt),
                                  _p(cadj), _p(cw), _p(cne))
    me = int(cne[0])
    return CSR(cxadj[:cn + 1], cadj[:me], cw[:me], cvwgt[:cn]), cmap


def ref_harness_contract(g, match):
    R = ref()
    if R is None:
        raise RuntimeError("reference harness not built (reference tree absent)")
    n = g.n
    cmap, cxadj, cvwgt = np.empty(n, np.int32), np.empty(n + 1, np.int32), np.empty(max(n, 1), np.int32)
    cadj, cw, cne = np.empty(max(g.m, 1), np.int32), np.empty(max(g.m, 1), np.int32), np.zeros(1, np.int32)
    cn = R.ref_cpu_contract(ctypes.c_int(n), _p(g.xadj), _p(g.adjncy), _p(g.adjwgt), _p(g.vwgt), _p(_i32(match)),
                            _p(cmap), _p(cxadj), _p(cvwgt), _p(cadj), _p(cw), _p(cne))
    me = int(cne[0])
    return CSR(cxadj[:cn + 1], cadj[:me], cw[:me], cvwgt[:cn]), cmap


def match_from_cmap(cmap):
    """Recovers the involution match[] from a cmap whose classes have size 1 or 2."""
    cmap = np.asarray(cmap, np.int64)
    n = len(cmap)
    order = np.argsort(cmap, kind="stable")
    match = np.arange(n, dtype=np.int32)
    cs = cmap[order]
    same = np.nonzero(cs[1:] == cs[:-1])[0]
    a, b = order[same], order[same + 1]
    match[a], match[b] = b, a
    return match


def ref_harness_rbbisection(g, nparts, seed):
    """The reference's own initial partition (cuMetis_rbbisection,
    cuMetis.cu:3046) of graph g into nparts, with its rand() stream seeded by
    srand(seed) (seed None: the stream continues).  Returns (part, objval)."""
    R = ref()
    if R is None:
        raise RuntimeError("reference harness not built (reference tree absent)")
    if seed is not None:
        R.ref_srand(ctypes.c_uint(seed))
    part = np.zeros(max(g.n, 1), np.int32)
    obj = np.zeros(1, np.int32)
    R.ref_rbbisection(ctypes.c_int32(g.n), _p(g.xadj), _p(g.adjncy), _p(g.vwgt), _p(g.adjwgt),
                      ctypes.c_int32(nparts), _p(part), _p(obj))
    return part[:g.n], int(obj[0])


def _part_windows(tvwgt, k):
    """Balance window of every part as Sum_maxmin_pwgts computes it
    (cuMetis.cu:3424-3433) in single precision, tpwgts = (float)(1.0/k)."""
    tp = np.float32(1.0 / k)
    x = np.float32(tp * np.float32(tvwgt))
    return int(np.float32(x * np.float32(1.03))), int(np.float32(x / np.float32(1.03)))


def boundary_targets(g, where, k):
    """Boundary flag and target part of every vertex (Find_real_bnd_info +
    find_kayparams, cuMetis.cu:3236-3306): boundary when the weight to other
    parts exceeds the weight to the own part; target = the first part id with
    the largest connection if it beats the own part, else the own part."""
    n = g.n
    flag = np.zeros(n, bool)
    target = where.copy()
    for v in range(n):
        lo, hi = g.xadj[v], g.xadj[v + 1]
        nb = where[g.adjncy[lo:hi]]
        w = g.adjwgt[lo:hi].astype(np.int64)
        me = where[v]
        mw = int(w[nb == me].sum())
        ow = int(w[nb != me].sum())
        if ow > mw:
            flag[v] = True
            acc = np.bincount(nb, weights=w, minlength=k).astype(np.int64)
            mx = acc.max()
            if mx > acc[me]:
                target[v] = int(np.argmax(acc == mx))
    return flag, target


def refine_kway_model(g, where, k):
    """One k-way refinement pass (cuMetis_uncoarsen, cuMetis.cu:3494-3514)
    with the part groups run one after another in part order: boundary
    vertices grouped by target part in vertex order; first the moves to a
    higher part id, then to a lower one, each kept only if both parts stay in
    their windows.  With two parts the GPU's concurrent part threads cannot
    interleave (one group moves per phase), so this is exact for k = 2.
    Returns (where, moves)."""
    where = np.array(where, np.int32).copy()
    vw = g.vwgt.astype(np.int64)
    pw = np.bincount(where, weights=vw, minlength=k).astype(np.int64)
    mx, mn = _part_windows(int(vw.sum()), k)
    flag, target = boundary_targets(g, where, k)
    groups = [[] for _ in range(k)]
    for v in np.nonzero(flag)[0]:
        groups[target[v]].append(int(v))
    moves = 0
    for up in (True, False):
        for t in range(k):
            for v in groups[t]:
                me = int(where[v])
                if (me >= t) if up else (me <= t):
                    continue
                w = int(vw[v])
                if mn <= pw[t] + w <= mx and mn <= pw[me] - w <= mx:
                    pw[t] += w
                    pw[me] -= w
                    where[v] = t
                    moves += 1
    return where, moves


def refine_kway_c(g, where, k):
    """C restatement of refine_kway_model (same rules, same group order), for
    graphs too large for the Python loop.  Returns (where, moves)."""
    w = np.array(where, np.int32).copy()
    mv = lib().or_refine_kway(g.n, _p(g.xadj), _p(g.adjncy), _p(g.adjwgt), _p(g.vwgt), int(k), _p(w))
    return w, int(mv)


def gen_rmat(scale, edge_factor=16, a=0.57, b=0.19, c=0.19, seed=1, wmin=1, wmax=100):
    """The R-MAT workload generator restated in the oracle (or_gen_rmat):
    the same graph as the library's cm_gen_rmat, without loading it."""
    L = lib()
    P = ctypes.POINTER(ctypes.c_int32)
    L.or_gen_rmat.restype = ctypes.c_int64
    L.or_gen_rmat.argtypes = [ctypes.c_int32, ctypes.c_int32, ctypes.c_double, ctypes.c_double, ctypes.c_double,
                              ctypes.c_uint64, ctypes.c_int32, ctypes.c_int32, ctypes.POINTER(P),
                              ctypes.POINTER(P), ctypes.POINTER(P)]
    L.or_free.argtypes = [ctypes.c_void_p]
    px, pa, pw = P(), P(), P()
    m = L.or_gen_rmat(int(scale), int(edge_factor), a, b, c, int(seed), int(wmin), int(wmax), ctypes.byref(px),
                      ctypes.byref(pa), ctypes.byref(pw))
    if m < 0:
        raise ValueError("or_gen_rmat: bad parameters")
    n = 1 << scale
    xadj = np.ctypeslib.as_array(px, shape=(n + 1,)).copy()
    adj = np.ctypeslib.as_array(pa, shape=(max(m, 1),))[:m].copy()
    wt = np.ctypeslib.as_array(pw, shape=(max(m, 1),))[:m].copy()
    for p in (px, pa, pw):
        L.or_free(p)
    return CSR(xadj, adj, wt, np.ones(n, np.int32))


def gen_mesh(nx, ny, offsets):
    """2D mesh with unit weights: vertex (i, j) -> i * ny + j, joined to
    (i, j) +- each offset; rows sorted (the library's grid generators)."""
    n = nx * ny
    ii, jj = np.divmod(np.arange(n, dtype=np.int64), ny)
    src, dst = [], []
    for di, dj in offsets:
        for s in (-1, 1):
            a, b = ii + s * di, jj + s * dj
            ok = (a >= 0) & (a < nx) & (b >= 0) & (b < ny)
            src.append(np.nonzero(ok)[0])
            dst.append((a * ny + b)[ok])
    src, dst = np.concatenate(src), np.concatenate(dst)
    order = np.lexsort((dst, src))
    xadj = np.zeros(n + 1, np.int64)
    np.add.at(xadj, src + 1, 1)
    return CSR(np.cumsum(xadj), dst[order], np.ones(len(dst), np.int32), np.ones(n, np.int32))


def gen_grid2d(nx, ny):
    return gen_mesh(nx, ny, [(0, 1), (1, 0)])


def gen_tri_grid(nx, ny):
    return gen_mesh(nx, ny, [(0, 1), (1, 0), (1, 1)])
