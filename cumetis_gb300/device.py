"""Device side of the Python binding: a Context wraps a cm_ctx; arrays are
torch int32 CUDA tensors (torch only provides device memory and the stream).
Every call goes through libcm's C ABI; there is no fallback path."""
import ctypes

import numpy as np

from . import (CMError, Graph, DeviceGraph, cm_coarsen_params, cm_graph, lib, _check, MATCH_HEM,
               MATCH_HEM_HASH)


def _torch():
    import torch
    return torch


def _stream_ptr(stream=None):
    torch = _torch()
    s = stream if stream is not None else torch.cuda.current_stream()
    return ctypes.c_void_p(s.cuda_stream)


def _empty(n, device):
    torch = _torch()
    return torch.empty(max(int(n), 1), dtype=torch.int32, device=device)


class Context:
    """A libcm device context (workspace, status block) on one GPU."""

    def __init__(self, device=0):
        L = lib()
        if not hasattr(L, "cm_ctx_create"):
            raise CMError(6, "libcm.so was built without device entry points")
        h = ctypes.c_void_p()
        _check(L.cm_ctx_create(int(device), ctypes.byref(h)))
        self._h = h
        self.device = int(device)
        self.torch_device = "cuda:%d" % self.device

    def close(self):
        if getattr(self, "_h", None):
            lib().cm_ctx_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    @property
    def handle(self):
        return self._h

    def reserve(self, nvtxs, nedges):
        _check(lib().cm_ctx_reserve(self._h, int(nvtxs), int(nedges)))

    def launch_count(self):
        return int(lib().cm_ctx_launch_count(self._h))

    def set_stage_timing(self, enable):
        _check(lib().cm_ctx_set_stage_timing(self._h, 1 if enable else 0))

    def stage_times(self, reset=False):
        """{kernel name: accumulated ms} recorded with CUDA events."""
        n = 7
        buf = (ctypes.c_double * n)()
        _check(lib().cm_ctx_stage_times(self._h, buf, n, 1 if reset else 0))
        return {lib().cm_stage_name(i).decode(): float(buf[i]) for i in range(n)}

    def set_blocking_waits(self, enable=True):
        """Sleep instead of spinning while the library waits on the GPU."""
        _check(lib().cm_ctx_set_blocking_waits(self._h, 1 if enable else 0))

    def set_match_trace(self, max_rounds):
        _check(lib().cm_ctx_set_match_trace(self._h, int(max_rounds)))

    def match_trace(self, cap_rows=4096):
        """Rows of the last matching's trace (see cm_ctx_match_trace)."""
        buf = (ctypes.c_int64 * (8 * cap_rows))()
        rows = ctypes.c_int32(0)
        _check(lib().cm_ctx_match_trace(self._h, buf, int(cap_rows), ctypes.byref(rows)))
        a = np.frombuffer(buf, dtype=np.int64).reshape(cap_rows, 8)
        return a[:rows.value].copy()

    def sync(self, stream=None):
        _check(lib().cm_ctx_sync(self._h, _stream_ptr(stream)))

    # ---- one level -------------------------------------------------------
    def match(self, g, maxvwgt, mode=MATCH_HEM, out=None, stream=None, want_rounds=True):
        """Heavy-edge matching of DeviceGraph g -> (match tensor, rounds)."""
        out = out if out is not None else _empty(g.nvtxs, self.torch_device)
        rounds = ctypes.c_int32(-1)
        cg = g.as_cm()
        _check(lib().cm_match(self._h, ctypes.byref(cg), int(maxvwgt), int(mode), ctypes.c_void_p(out.data_ptr()),
                              ctypes.byref(rounds) if want_rounds else None, _stream_ptr(stream)))
        return out[:g.nvtxs], int(rounds.value)

    def build_cmap(self, g, match, stream=None):
        """-> (cmap, leader[:n'], cvwgt[:n'], eoff[:n'+1], n')."""
        n = g.nvtxs
        dev = self.torch_device
        cmap, leader, cvwgt, eoff = _empty(n, dev), _empty(n, dev), _empty(n, dev), _empty(n + 1, dev)
        cn = _empty(1, dev)
        _check(lib().cm_build_cmap(self._h, n, ctypes.c_void_p(g.xadj.data_ptr()), ctypes.c_void_p(g.vwgt.data_ptr()),
                                   ctypes.c_void_p(match.data_ptr()), ctypes.c_void_p(cmap.data_ptr()),
                                   ctypes.c_void_p(leader.data_ptr()), ctypes.c_void_p(cvwgt.data_ptr()),
                                   ctypes.c_void_p(eoff.data_ptr()), ctypes.c_void_p(cn.data_ptr()),
                                   _stream_ptr(stream)))
        self.sync(stream)
        c = int(cn[0].item())
        return cmap[:n], leader[:c], cvwgt[:c], eoff[:c + 1], c

    def contract(self, g, match, stream=None, sync=True):
        """Coarse DeviceGraph (trimmed to n', m' when sync) and cmap."""
        n, m = g.nvtxs, g.nedges
        dev = self.torch_device
        cx, cv, ca, cw = _empty(n + 1, dev), _empty(n, dev), _empty(m, dev), _empty(m, dev)
        cmap = _empty(n, dev)
        sizes = _empty(2, dev)
        coarse = cm_graph(0, 0, cx.data_ptr(), ca.data_ptr(), cw.data_ptr(), cv.data_ptr())
        fg = g.as_cm()
        _check(lib().cm_contract(self._h, ctypes.byref(fg), ctypes.c_void_p(match.data_ptr()),
                                 ctypes.c_void_p(cmap.data_ptr()), ctypes.byref(coarse),
                                 ctypes.c_void_p(sizes.data_ptr()), _stream_ptr(stream)))
        if not sync:
            return (cx, ca, cw, cv), cmap[:n], sizes
        self.sync(stream)
        cn, cm_ = (int(v) for v in sizes.cpu().tolist())
        return DeviceGraph(cx[:cn + 1], ca[:cm_], cw[:cm_], cv[:cn]), cmap[:n]

    # ---- multilevel -------------------------------------------------------
    def part_graph(self, g, nparts, seed=1, mode=MATCH_HEM_HASH, refine_passes=1, coarsen_to=0):
        """k-way partition of a host Graph (cm_part_graph).  Returns
        (part, edge_cut, stats dict)."""
        from . import cm_part_params, cm_part_stats, _np_p
        p = cm_part_params(int(seed), int(mode), int(refine_passes), int(coarsen_to))
        st = cm_part_stats()
        part = np.zeros(max(g.nvtxs, 1), np.int32)
        obj = np.zeros(1, np.int32)
        _check(lib().cm_part_graph(self._h, g.nvtxs, _np_p(g.xadj), _np_p(g.adjncy), _np_p(g.vwgt),
                                   _np_p(g.adjwgt), int(nparts), None, None, _np_p(obj), _np_p(part),
                                   ctypes.byref(p), ctypes.byref(st)))
        return part[:g.nvtxs], int(obj[0]), st.as_dict()

    def refine_kway(self, g_dev, nparts, d_where, stream=None):
        """One k-way refinement pass of d_where (torch int32 CUDA tensor) on a
        DeviceGraph.  Returns the number of vertices moved."""
        mv = ctypes.c_int64(0)
        cg = g_dev.as_cm()
        _check(lib().cm_refine_kway(self._h, ctypes.byref(cg), int(nparts), ctypes.c_void_p(d_where.data_ptr()),
                                    ctypes.byref(mv), _stream_ptr(stream)))
        return int(mv.value)

    def project(self, d_cmap, d_cwhere, d_where, stream=None):
        _check(lib().cm_project(self._h, int(d_where.numel()), ctypes.c_void_p(d_cmap.data_ptr()),
                                ctypes.c_void_p(d_cwhere.data_ptr()), ctypes.c_void_p(d_where.data_ptr()),
                                _stream_ptr(stream)))

    def coarsen(self, g, coarsen_to, mode=MATCH_HEM, maxvwgt=0, shrink=0.75, max_levels=64, stream=None):
        """Coarsens a host Graph (uploaded inside the call) or a DeviceGraph."""
        p = cm_coarsen_params(int(coarsen_to), int(maxvwgt), int(mode), int(max_levels), float(shrink))
        on_dev = isinstance(g, DeviceGraph)
        cg = g.as_cm()
        h = ctypes.c_void_p()
        _check(lib().cm_coarsen(self._h, ctypes.byref(cg), 1 if on_dev else 0, ctypes.byref(p), ctypes.byref(h),
                                _stream_ptr(stream)))
        return Hierarchy(h, keep=g)

    def coarsen_batch(self, graphs, coarsen_to, mode=MATCH_HEM, maxvwgt=0, shrink=0.75, max_levels=64, stream=None):
        """Coarsens host Graphs together (cm_coarsen_batch); coarsen_to is one
        threshold or one per graph.  Returns one Hierarchy per graph."""
        ng = len(graphs)
        thr = list(coarsen_to) if hasattr(coarsen_to, "__len__") else [coarsen_to] * ng
        gs = (cm_graph * max(ng, 1))(*[g.as_cm() for g in graphs])
        ps = (cm_coarsen_params * max(ng, 1))(*[cm_coarsen_params(int(t), int(maxvwgt), int(mode), int(max_levels),
                                                                   float(shrink)) for t in thr])
        hs = (ctypes.c_void_p * max(ng, 1))()
        _check(lib().cm_coarsen_batch(self._h, ng, gs, ps, hs, _stream_ptr(stream)))
        return [Hierarchy(ctypes.c_void_p(hs[i]), keep=graphs[i]) for i in range(ng)]


class Hierarchy:
    """Levels of one coarsening, resident on the device."""

    def __init__(self, h, keep=None):
        self._h = h
        self._keep = keep

    def close(self):
        if getattr(self, "_h", None):
            lib().cm_hierarchy_free(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __len__(self):
        return int(lib().cm_hierarchy_levels(self._h))

    def sizes(self):
        out = []
        for l in range(len(self)):
            g = cm_graph()
            _check(lib().cm_hierarchy_level(self._h, l, ctypes.byref(g), None, None))
            out.append((g.nvtxs, g.nedges))
        return out

    def copy_level(self, level, with_cmap=True):
        """(host Graph, cmap, match) of one level; cmap/match are None for the
        coarsest level or when with_cmap is False."""
        g = cm_graph()
        sizes = self.sizes()
        n = sizes[level][0]
        inner = with_cmap and level < len(sizes) - 1
        cmap = np.empty(max(n, 1), np.int32) if inner else None
        match = np.empty(max(n, 1), np.int32) if inner else None
        P = ctypes.POINTER(ctypes.c_int32)
        _check(lib().cm_hierarchy_copy_level(self._h, level, ctypes.byref(g),
                                             cmap.ctypes.data_as(P) if inner else None,
                                             match.ctypes.data_as(P) if inner else None))
        return Graph._from_cm(g), (cmap[:n] if inner else None), (match[:n] if inner else None)

    def read_level(self, level, xadj, adjncy, adjwgt, vwgt):
        """Copies a level into caller-owned host buffers (e.g. pinned tensors'
        data pointers); sizes from sizes()."""
        _check(lib().cm_hierarchy_read_level(self._h, int(level), ctypes.c_void_p(xadj), ctypes.c_void_p(adjncy),
                                             ctypes.c_void_p(adjwgt), ctypes.c_void_p(vwgt)))
