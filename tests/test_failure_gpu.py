"""Failure detection without a GPU fault: a bounded device wait that runs
out is reported as a status and leaves the context usable."""
import time

import numpy as np
import pytest

import cumetis_gb300 as cm
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def test_device_wait_times_out_and_context_recovers(ctx):
    t0 = time.perf_counter()
    rc = cm.lib().cm_ctx_selftest_wait(ctx._h, None)
    dt = time.perf_counter() - t0
    assert rc == cm.CM_ERR_LIMIT, cm.lib().cm_last_error()
    assert b"look-back" in cm.lib().cm_last_error()
    assert 1.5 < dt < 30
    # the same context still matches and contracts correctly
    g = cm.gen_tri_grid(40, 40)
    og = O.CSR(g.xadj, g.adjncy, g.adjwgt, g.vwgt)
    m, _ = ctx.match(g.to_device(), 10, 0)
    np.testing.assert_array_equal(m.cpu().numpy(), O.match_greedy(og, 10, 0))
    ctx.sync()  # no error left behind
