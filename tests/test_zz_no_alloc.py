"""cm_build_cmap_noalloc: the allocation-free coarse-vertex map.

Some callers cannot allocate device memory once they are running (a host
whose memory planner owns every device allocation, or a latency-critical loop
that cannot absorb the device-wide synchronisation of a cudaMalloc).  For
them the library offers one entry point whose scratch is a fixed array inside
the library.  This file checks, through the C ABI, that it returns exactly
what cm_build_cmap returns, on two calls in a row (the calls share that
array, and a larger graph runs before smaller ones so that leftovers of a
bigger call are exercised), that an empty graph and an invalid matching are
handled (the latter reported in band through d_cnvtxs), and that it refuses
inputs beyond its fixed size.  It is collected last so that a failure here
never hides the other GPU tests.
"""
import ctypes

import pytest

import cumetis_gb300 as cm
from oracle import oracle as O

pytestmark = pytest.mark.gpu

MAX_VERTICES = 1 << 24


def _entry():
    f = cm.lib().cm_build_cmap_noalloc
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_int32] + [ctypes.c_void_p] * 9
    return f


def _call(f, dg, match, outs, stream):
    cmap, leader, cvwgt, eoff, cn = outs
    return f(dg.nvtxs, dg.xadj.data_ptr(), dg.vwgt.data_ptr(), match.data_ptr(), cmap.data_ptr(),
             leader.data_ptr(), cvwgt.data_ptr(), eoff.data_ptr(), cn.data_ptr(), stream)


def test_noalloc_cmap_equals_allocating_entry_point():
    import torch
    f = _entry()
    ctx = cm.Context(0)
    stream = torch.cuda.current_stream().cuda_stream
    # largest first: later, smaller calls find the look-back words of a bigger one
    graphs = [cm.gen_grid2d(300, 200), cm.gen_rmat(14, 16, seed=3), cm.gen_tri_grid(69, 69)]
    for g in graphs:
        og = O.CSR(g.xadj, g.adjncy, g.adjwgt, g.vwgt)
        match = O.match_greedy(og, O.maxvwgt_rule(int(g.vwgt.sum()), 100), 0)
        dg = g.to_device()
        dm = torch.from_numpy(match).cuda()
        want_cmap, want_leader, want_cvwgt, want_eoff, want_cn = ctx.build_cmap(dg, dm)
        n = g.nvtxs
        for _ in range(2):  # two calls in a row share the library's scratch array
            outs = [torch.full((n,), -7, dtype=torch.int32, device="cuda") for _ in range(3)]
            outs += [torch.full((n + 1,), -7, dtype=torch.int32, device="cuda"),
                     torch.full((1,), -7, dtype=torch.int32, device="cuda")]
            assert _call(f, dg, dm, outs, stream) == cm.CM_OK, cm.lib().cm_last_error()
            torch.cuda.synchronize()
            cn = int(outs[4].item())
            assert cn == want_cn
            assert torch.equal(outs[0], want_cmap)
            assert torch.equal(outs[1][:cn], want_leader)
            assert torch.equal(outs[2][:cn], want_cvwgt)
            assert torch.equal(outs[3][:cn + 1], want_eoff)
    ctx.close()


def test_noalloc_cmap_rejects_oversized_input():
    import torch
    f = _entry()
    buf = torch.zeros(4, dtype=torch.int32, device="cuda")
    p = buf.data_ptr()
    rc = f(MAX_VERTICES + 1, p, p, p, p, p, p, p, p, None)
    assert rc == cm.CM_ERR_INVALID
    assert b"16777216" in cm.lib().cm_last_error()


def _outs(n, fill=-7):
    import torch
    outs = [torch.full((max(n, 1),), fill, dtype=torch.int32, device="cuda") for _ in range(3)]
    outs += [torch.full((n + 1,), fill, dtype=torch.int32, device="cuda"),
             torch.full((1,), fill, dtype=torch.int32, device="cuda")]
    return outs


def test_noalloc_cmap_empty_graph():
    import torch
    f = _entry()
    stream = torch.cuda.current_stream().cuda_stream
    g = cm.Graph([0], [], [], []).to_device()
    match = torch.zeros(1, dtype=torch.int32, device="cuda")
    outs = _outs(0)
    assert _call(f, g, match, outs, stream) == cm.CM_OK, cm.lib().cm_last_error()
    torch.cuda.synchronize()
    assert int(outs[4].item()) == 0 and int(outs[3][0].item()) == 0


def test_noalloc_cmap_reports_an_invalid_matching_in_band():
    """A matching that is not an involution (host-side invalid input; nothing
    faults): d_cnvtxs comes back as -CM_ERR_INVALID, and the next call with a
    valid matching is exact again."""
    import torch
    f = _entry()
    stream = torch.cuda.current_stream().cuda_stream
    g = cm.gen_grid2d(120, 90)
    og = O.CSR(g.xadj, g.adjncy, g.adjwgt, g.vwgt)
    dg = g.to_device()
    n = g.nvtxs
    bad = O.match_greedy(og, O.maxvwgt_rule(int(g.vwgt.sum()), 100), 0).copy()
    u = int(next(v for v in range(n) if bad[v] > v))  # a matched pair (u, bad[u])
    bad[u] = u  # u leaves its pair while its partner still points at it
    outs = _outs(n)
    assert _call(f, dg, torch.from_numpy(bad).cuda(), outs, stream) == cm.CM_OK
    torch.cuda.synchronize()
    assert int(outs[4].item()) == -cm.CM_ERR_INVALID
    good = O.match_greedy(og, O.maxvwgt_rule(int(g.vwgt.sum()), 100), 0)
    ctx = cm.Context(0)
    want = ctx.build_cmap(dg, torch.from_numpy(good).cuda())
    outs = _outs(n)
    assert _call(f, dg, torch.from_numpy(good).cuda(), outs, stream) == cm.CM_OK
    torch.cuda.synchronize()
    assert int(outs[4].item()) == want[4]
    assert torch.equal(outs[0], want[0])
    ctx.close()
