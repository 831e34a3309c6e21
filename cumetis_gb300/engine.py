"""Batched and served partitioning: Python side of cm_engine_* and
cm_part_batch (the scheduler and worker pool live in libcm, cm_engine.cu)."""
import ctypes

import numpy as np

from . import (cm_batch_stats, cm_graph, cm_job_info, cm_part_params, lib, _check, _np_p,
               MATCH_HEM_HASH)


def _params(seed=1, mode=MATCH_HEM_HASH, refine_passes=1, coarsen_to=0):
    return cm_part_params(int(seed), int(mode), int(refine_passes), int(coarsen_to))


class Job:
    """A submitted partition; keeps the graph arrays and the output alive."""

    def __init__(self, engine, job_id, graph, part):
        self.engine, self.id, self.graph, self.part = engine, job_id, graph, part


class Engine:
    """Worker pool on one device: submit host graphs, wait for partitions."""

    def __init__(self, device=0, workers=8, hbm_budget_bytes=0, max_queue=0, reserve_nvtxs=0, reserve_nedges=0):
        h = ctypes.c_void_p()
        _check(lib().cm_engine_create(int(device), int(workers), int(hbm_budget_bytes), int(max_queue),
                                      int(reserve_nvtxs), int(reserve_nedges), ctypes.byref(h)))
        self._h = h

    def submit(self, g, nparts, seed=1, mode=MATCH_HEM_HASH, refine_passes=1, coarsen_to=0):
        part = np.zeros(max(g.nvtxs, 1), np.int32)
        jid = ctypes.c_int64(0)
        cg = g.as_cm()
        p = _params(seed, mode, refine_passes, coarsen_to)
        _check(lib().cm_engine_submit(self._h, ctypes.byref(cg), int(nparts), ctypes.byref(p), _np_p(part),
                                      ctypes.byref(jid)))
        return Job(self, jid.value, g, part)

    def poll(self, job):
        d = np.zeros(1, np.int32)
        _check(lib().cm_engine_poll(self._h, int(job.id), _np_p(d)))
        return bool(d[0])

    def wait(self, job):
        """-> (part, edge_cut, info dict)."""
        obj = np.zeros(1, np.int32)
        info = cm_job_info()
        _check(lib().cm_engine_wait(self._h, int(job.id), _np_p(obj), ctypes.byref(info)))
        d = {"queue_ms": info.queue_ms, "run_ms": info.run_ms, "latency_ms": info.latency_ms,
             "stats": info.stats.as_dict()}
        return job.part[:job.graph.nvtxs], int(obj[0]), d

    def stats(self, reset=False):
        c = ctypes.c_int64(0)
        p50, p99 = ctypes.c_double(0), ctypes.c_double(0)
        _check(lib().cm_engine_stats(self._h, ctypes.byref(c), ctypes.byref(p50), ctypes.byref(p99),
                                     1 if reset else 0))
        return {"completed": c.value, "p50_ms": p50.value, "p99_ms": p99.value}

    def close(self):
        if getattr(self, "_h", None):
            lib().cm_engine_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()


def part_batch(graphs, nparts, device=0, workers=8, seed=1, mode=MATCH_HEM_HASH):
    """Partitions a list of host Graphs (cm_part_batch).  nparts: int or one
    per graph.  Returns (list of parts, edge cuts, stats dict)."""
    nb = len(graphs)
    ks = np.full(nb, nparts, np.int32) if np.isscalar(nparts) else np.asarray(nparts, np.int32)
    arr = (cm_graph * max(nb, 1))()
    keep = []
    for i, g in enumerate(graphs):
        cg = g.as_cm()
        keep.append(cg)
        arr[i] = cg
    parts = [np.zeros(max(g.nvtxs, 1), np.int32) for g in graphs]
    pp = (ctypes.POINTER(ctypes.c_int32) * max(nb, 1))(*[_np_p(p) for p in parts])
    objs = np.zeros(max(nb, 1), np.int32)
    st = cm_batch_stats()
    p = _params(seed, mode)
    _check(lib().cm_part_batch(int(device), int(workers), nb, arr, _np_p(ks), pp, _np_p(objs), ctypes.byref(p),
                               ctypes.byref(st)))
    return ([parts[i][:graphs[i].nvtxs] for i in range(nb)], objs[:nb].copy(),
            {"setup_ms": st.setup_ms, "run_ms": st.run_ms, "graphs": st.graphs, "sum_nedges": st.sum_nedges,
             "sum_cut": st.sum_cut, "sum_coarsen_ms": st.sum_coarsen_ms, "sum_init_ms": st.sum_init_ms,
             "sum_uncoarsen_ms": st.sum_uncoarsen_ms})
