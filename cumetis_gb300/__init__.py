"""cumetis_gb300 -- Python host binding of libcm, the GB300-native rebuild of
cuMetis's multilevel coarsening hot path (heavy-edge matching, coarse-vertex
map, contraction).

Everything goes through the C ABI declared in include/cm.h (ctypes; no torch
types cross it).  Device arrays may be torch CUDA tensors (int32, contiguous)
or raw device addresses.  There is no CPU fallback: if libcm.so is missing or
no GPU is present, the device entry points raise CMError.
"""
import ctypes
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
# CUMETIS_LIB selects another build of the library (the autotuner's variants).
LIB_PATH = os.environ.get("CUMETIS_LIB") or os.path.join(_HERE, "libcm.so")
CLI_PATH = os.path.join(_HERE, "cuMetis")

CM_OK, CM_ERR_INVALID, CM_ERR_NOMEM, CM_ERR_CUDA, CM_ERR_LIMIT, CM_ERR_IO, CM_ERR_UNSUPPORTED = range(7)
MATCH_HEM, MATCH_HEM_HASH, MATCH_RACY = 0, 1, 2
_I32P = ctypes.POINTER(ctypes.c_int32)


class CMError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("libcm error %d: %s" % (code, msg))
        self.code = code


class cm_graph(ctypes.Structure):
    _fields_ = [("nvtxs", ctypes.c_int32), ("nedges", ctypes.c_int32), ("xadj", ctypes.c_void_p),
                ("adjncy", ctypes.c_void_p), ("adjwgt", ctypes.c_void_p), ("vwgt", ctypes.c_void_p)]


class cm_coarsen_params(ctypes.Structure):
    _fields_ = [("coarsen_to", ctypes.c_int32), ("maxvwgt", ctypes.c_int32), ("match_mode", ctypes.c_int32),
                ("max_levels", ctypes.c_int32), ("shrink", ctypes.c_double)]


class cm_part_params(ctypes.Structure):
    _fields_ = [("seed", ctypes.c_int32), ("match_mode", ctypes.c_int32), ("refine_passes", ctypes.c_int32),
                ("coarsen_to", ctypes.c_int32)]


class cm_part_stats(ctypes.Structure):
    _fields_ = [("coarsen_ms", ctypes.c_double), ("init_ms", ctypes.c_double), ("uncoarsen_ms", ctypes.c_double),
                ("total_ms", ctypes.c_double), ("levels", ctypes.c_int32), ("coarsest_nvtxs", ctypes.c_int32),
                ("initial_cut", ctypes.c_int32), ("edge_cut", ctypes.c_int64), ("moves", ctypes.c_int64)]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_}


class cm_job_info(ctypes.Structure):
    _fields_ = [("queue_ms", ctypes.c_double), ("run_ms", ctypes.c_double), ("latency_ms", ctypes.c_double),
                ("stats", cm_part_stats), ("status", ctypes.c_int32)]


class cm_batch_stats(ctypes.Structure):
    _fields_ = [("setup_ms", ctypes.c_double), ("run_ms", ctypes.c_double), ("graphs", ctypes.c_int32),
                ("sum_nedges", ctypes.c_int64), ("sum_cut", ctypes.c_int64), ("sum_coarsen_ms", ctypes.c_double),
                ("sum_init_ms", ctypes.c_double), ("sum_uncoarsen_ms", ctypes.c_double)]


_lib = None


def lib():
    """Loads libcm.so (building it first if this tree has never been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            from . import build as _b
            _b.build()
        L = ctypes.CDLL(LIB_PATH)
        _declare(L)
        _lib = L
    return _lib


def _declare(L):
    c_int, c_i32, c_i64, c_vp = ctypes.c_int, ctypes.c_int32, ctypes.c_int64, ctypes.c_void_p
    G = ctypes.POINTER(cm_graph)
    sigs = {
        "cm_last_error": (ctypes.c_char_p, []),
        "cm_graph_alloc": (c_int, [c_i32, c_i32, G]),
        "cm_graph_free": (None, [G]),
        "cm_graph_validate": (c_int, [G, c_int, c_int]),
        "cm_gen_tri_grid": (c_int, [c_i32, c_i32, G]),
        "cm_gen_grid2d": (c_int, [c_i32, c_i32, G]),
        "cm_gen_grid3d": (c_int, [c_i32, c_i32, c_i32, G]),
        "cm_gen_rmat": (c_int, [c_i32, c_i32, ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_uint64,
                                c_i32, c_i32, G]),
        "cm_gen_rgg": (c_int, [c_i32, ctypes.c_double, ctypes.c_uint64, G]),
        "cm_read_graph": (c_int, [ctypes.c_char_p, G]),
        "cm_read_mtx": (c_int, [ctypes.c_char_p, G]),
        "cm_write_graph": (c_int, [ctypes.c_char_p, G]),
        "cm_write_partition": (c_int, [ctypes.c_char_p, c_i32, c_i32, _I32P]),
        "cm_edge_cut": (c_i64, [G, _I32P]),
        "cm_imbalance": (ctypes.c_double, [G, c_i32, _I32P]),
        "cm_initial_partition": (c_int, [G, c_i32, ctypes.c_uint32, _I32P, _I32P]),
    }
    optional = {
        "cm_ctx_create": (c_int, [c_int, ctypes.POINTER(c_vp)]),
        "cm_ctx_destroy": (None, [c_vp]),
        "cm_ctx_reserve": (c_int, [c_vp, c_i64, c_i64]),
        "cm_ctx_launch_count": (c_i64, [c_vp]),
        "cm_match": (c_int, [c_vp, G, c_i32, c_i32, c_vp, _I32P, c_vp]),
        "cm_build_cmap": (c_int, [c_vp, c_i32, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp]),
        "cm_contract": (c_int, [c_vp, G, c_vp, c_vp, G, c_vp, c_vp]),
        "cm_coarsen_default_params": (None, [c_i32, c_i32, ctypes.POINTER(cm_coarsen_params)]),
        "cm_coarsen": (c_int, [c_vp, G, c_int, ctypes.POINTER(cm_coarsen_params), ctypes.POINTER(c_vp), c_vp]),
        "cm_coarsen_batch": (c_int, [c_vp, c_i32, G, ctypes.POINTER(cm_coarsen_params), ctypes.POINTER(c_vp), c_vp]),
        "cm_hierarchy_free": (None, [c_vp]),
        "cm_hierarchy_levels": (c_i32, [c_vp]),
        "cm_hierarchy_level": (c_int, [c_vp, c_i32, G, ctypes.POINTER(c_vp), ctypes.POINTER(c_vp)]),
        "cm_hierarchy_copy_level": (c_int, [c_vp, c_i32, G, _I32P, _I32P]),
        "cm_ctx_sync": (c_int, [c_vp, c_vp]),
        "cm_ctx_set_stage_timing": (c_int, [c_vp, c_int]),
        "cm_ctx_stage_times": (c_int, [c_vp, ctypes.POINTER(ctypes.c_double), c_i32, c_int]),
        "cm_stage_name": (ctypes.c_char_p, [c_i32]),
        "cm_ctx_set_match_trace": (c_int, [c_vp, c_i32]),
        "cm_ctx_set_blocking_waits": (c_int, [c_vp, c_int]),
        "cm_ctx_match_trace": (c_int, [c_vp, ctypes.POINTER(ctypes.c_int64), c_i32, _I32P]),
        "cm_hierarchy_read_level": (c_int, [c_vp, c_i32, c_vp, c_vp, c_vp, c_vp]),
        "cm_refine_kway": (c_int, [c_vp, G, c_i32, c_vp, ctypes.POINTER(c_i64), c_vp]),
        "cm_project": (c_int, [c_vp, c_i32, c_vp, c_vp, c_vp, c_vp]),
        "cm_part_default_params": (None, [ctypes.POINTER(cm_part_params)]),
        "cm_part_graph": (c_int, [c_vp, c_i32, _I32P, _I32P, _I32P, _I32P, c_i32, c_vp, c_vp, _I32P, _I32P,
                                  ctypes.POINTER(cm_part_params), ctypes.POINTER(cm_part_stats)]),
        "cuMetis_PartGraph": (c_int, [_I32P, _I32P, _I32P, _I32P, _I32P, _I32P, c_vp, c_vp, _I32P, _I32P]),
        "cm_ctx_stream": (c_vp, [c_vp]),
        "cm_ctx_selftest_wait": (c_int, [c_vp, c_vp]),
        "cm_engine_create": (c_int, [c_int, c_i32, c_i64, c_i32, c_i64, c_i64, ctypes.POINTER(c_vp)]),
        "cm_engine_poll": (c_int, [c_vp, c_i64, _I32P]),
        "cm_engine_destroy": (None, [c_vp]),
        "cm_engine_submit": (c_int, [c_vp, G, c_i32, ctypes.POINTER(cm_part_params), _I32P, ctypes.POINTER(c_i64)]),
        "cm_engine_wait": (c_int, [c_vp, c_i64, _I32P, ctypes.POINTER(cm_job_info)]),
        "cm_engine_stats": (c_int, [c_vp, ctypes.POINTER(c_i64), ctypes.POINTER(ctypes.c_double),
                                    ctypes.POINTER(ctypes.c_double), c_int]),
        "cm_part_batch": (c_int, [c_int, c_i32, c_i32, G, _I32P, ctypes.POINTER(_I32P), _I32P,
                                  ctypes.POINTER(cm_part_params), ctypes.POINTER(cm_batch_stats)]),
    }
    for name, (res, args) in list(sigs.items()) + list(optional.items()):
        fn = getattr(L, name, None)
        if fn is None:
            if name in sigs:
                raise RuntimeError("libcm.so lacks %s" % name)
            continue
        fn.restype, fn.argtypes = res, args


def _check(rc):
    if rc != CM_OK:
        raise CMError(rc, lib().cm_last_error().decode(errors="replace"))


def _i32(a):
    return np.ascontiguousarray(a, dtype=np.int32)


def _np_p(a):
    return a.ctypes.data_as(_I32P)


class Graph:
    """Host CSR graph backed by int32 numpy arrays."""

    def __init__(self, xadj, adjncy, adjwgt=None, vwgt=None):
        self.xadj = _i32(xadj)
        self.adjncy = _i32(adjncy)
        self.adjwgt = _i32(adjwgt) if adjwgt is not None else np.ones(len(self.adjncy), np.int32)
        self.vwgt = _i32(vwgt) if vwgt is not None else np.ones(len(self.xadj) - 1, np.int32)

    @property
    def nvtxs(self):
        return len(self.xadj) - 1

    @property
    def nedges(self):
        return int(self.xadj[-1])

    def as_cm(self):
        g = cm_graph(self.nvtxs, self.nedges, self.xadj.ctypes.data, self.adjncy.ctypes.data,
                     self.adjwgt.ctypes.data, self.vwgt.ctypes.data)
        g._keep = self  # keep arrays alive
        return g

    @staticmethod
    def _from_cm(g):
        n, m = g.nvtxs, g.nedges

        def arr(ptr, k):
            if k == 0:
                return np.zeros(0, np.int32)
            return np.ctypeslib.as_array(ctypes.cast(ptr, _I32P), shape=(k,)).copy()

        out = Graph(arr(g.xadj, n + 1), arr(g.adjncy, m), arr(g.adjwgt, m), arr(g.vwgt, n))
        lib().cm_graph_free(ctypes.byref(g))
        return out

    def validate(self, check_symmetry=True, allow_self_loops=False):
        _check(lib().cm_graph_validate(ctypes.byref(self.as_cm()), int(check_symmetry), int(allow_self_loops)))

    def edge_cut(self, part):
        part = _i32(part)
        return int(lib().cm_edge_cut(ctypes.byref(self.as_cm()), _np_p(part)))

    def imbalance(self, nparts, part):
        part = _i32(part)
        return float(lib().cm_imbalance(ctypes.byref(self.as_cm()), int(nparts), _np_p(part)))

    def write(self, path):
        _check(lib().cm_write_graph(path.encode(), ctypes.byref(self.as_cm())))

    def to_device(self, device="cuda"):
        import torch
        return DeviceGraph(*(torch.from_numpy(a).to(device) for a in (self.xadj, self.adjncy, self.adjwgt, self.vwgt)))


class DeviceGraph:
    """CSR whose arrays are torch int32 CUDA tensors."""

    def __init__(self, xadj, adjncy, adjwgt, vwgt):
        self.xadj, self.adjncy, self.adjwgt, self.vwgt = xadj, adjncy, adjwgt, vwgt

    @property
    def nvtxs(self):
        return int(self.xadj.numel()) - 1

    @property
    def nedges(self):
        return int(self.adjncy.numel())

    def as_cm(self, nvtxs=None, nedges=None):
        return cm_graph(self.nvtxs if nvtxs is None else nvtxs, self.nedges if nedges is None else nedges,
                        self.xadj.data_ptr(), self.adjncy.data_ptr(), self.adjwgt.data_ptr(), self.vwgt.data_ptr())

    def to_host(self):
        return Graph(*(t.cpu().numpy() for t in (self.xadj, self.adjncy, self.adjwgt, self.vwgt)))


def _gen(fn, *args):
    g = cm_graph()
    _check(fn(*args, ctypes.byref(g)))
    return Graph._from_cm(g)


def gen_tri_grid(nx, ny):
    return _gen(lib().cm_gen_tri_grid, nx, ny)


def gen_grid2d(nx, ny):
    return _gen(lib().cm_gen_grid2d, nx, ny)


def gen_grid3d(nx, ny, nz):
    return _gen(lib().cm_gen_grid3d, nx, ny, nz)


def gen_rmat(scale, edge_factor=16, a=0.57, b=0.19, c=0.19, seed=1, wmin=1, wmax=100):
    return _gen(lib().cm_gen_rmat, scale, edge_factor, a, b, c, seed, wmin, wmax)


def gen_rgg(n, mean_degree=8.0, seed=1):
    return _gen(lib().cm_gen_rgg, n, mean_degree, seed)


def read_graph(path):
    return _gen(lib().cm_read_graph, path.encode())


def read_mtx(path):
    """MatrixMarket coordinate matrix -> Graph (pattern of A + A^T without the
    diagonal, unit weights; the reference's mtx_to_graph)."""
    return _gen(lib().cm_read_mtx, path.encode())


def write_partition(graph_path, nparts, part):
    part = _i32(part)
    _check(lib().cm_write_partition(graph_path.encode(), int(nparts), len(part), _np_p(part)))


def initial_partition(g, nparts, seed=1):
    """Initial partition of a host Graph by recursive bisection (host code,
    the reference's cuMetis_rbbisection restated).  Returns (part, objval)."""
    part = np.zeros(max(g.nvtxs, 1), np.int32)
    obj = np.zeros(1, np.int32)
    cg = g.as_cm()
    _check(lib().cm_initial_partition(ctypes.byref(cg), int(nparts), ctypes.c_uint32(seed), _np_p(part),
                                      _np_p(obj)))
    return part[:g.nvtxs], int(obj[0])


def coarsen_threshold(nvtxs, nparts):
    """k-way Coarsen_threshold = max(n / (20 log2 k), 30 k), cuMetis.cu:3634."""
    lg = 0
    k = nparts
    while k > 1:
        lg, k = lg + 1, k >> 1
    return max(nvtxs // (20 * lg) if lg > 0 else nvtxs, 30 * nparts)


def maxvwgt_rule(tvwgt, threshold):
    """(int)(1.5 * tvwgt / threshold), cuMetis.cu:1828."""
    return int(1.5 * tvwgt / threshold)


from .engine import Engine, part_batch  # noqa: E402,F401
from .device import Context, Hierarchy  # noqa: E402  (device side, needs libcm's CUDA entry points)
