"""Failure detection of the bounded device waits, without a GPU fault.

Every device-side wait of the persistent solvers (grid barriers, mbarrier
waits of the staged SpMV) gives up after a bounded number of polls and
reports GRMP_ERR_TIMEOUT through a status word the host reads.  These tests
make such waits run out on purpose -- a barrier one block never reaches, an
mbarrier nothing completes, and a real solve under a wait limit far too short
for its grid -- and check that the status is reported and the context stays
usable afterwards.  Nothing faults, traps or spins without a bound.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_selftest_waits_time_out_and_context_survives(G, ctx):
    from grmp_gb300 import _lib as L
    gs, ms = ctypes.c_int32(-1), ctypes.c_int32(-1)
    ctx.check(ctx.lib.grmp_selftest_wait_timeout(ctx.h, 2000, ctypes.byref(gs), ctypes.byref(ms)))
    assert gs.value == L.ERR_TIMEOUT   # blocks waiting for the block that left
    assert ms.value == L.ERR_TIMEOUT   # mbarrier that no copy completes
    # the context still runs work correctly
    from grmp_gb300 import problems as P
    prob = P.poisson2d(16)
    sysd = P.DeviceSystem(ctx, prob, mixed=False)
    st = sysd.assemble_and_solve(G.GB300PCG(mode="fp64", reltol=1e-10, abstol=0.0))
    assert st["status"] == 0


@pytest.mark.parametrize("mode,cfg", [("fp64", 408), ("mixed", 10408)])
def test_solve_reports_timeout_under_a_tiny_wait_limit(G, ctx, mode, cfg):
    """With a wait limit of one poll, blocks reaching a grid barrier ahead of
    the others give up at once: grmp_solve returns GRMP_ERR_TIMEOUT with its
    message.  The default limit restored, the same solve converges."""
    from grmp_gb300 import _lib as L
    from grmp_gb300 import problems as P
    prob = P.poisson2d(192)   # 148k DoFs: a grid of hundreds of blocks
    sysd = P.DeviceSystem(ctx, prob, mixed=(mode == "mixed"))
    solver = G.GB300PCG(mode=mode, reltol=1e-10, abstol=0.0, spmv_config=cfg)
    try:
        ctx.check(ctx.lib.grmp_context_set_wait_limit(ctx.h, 1))
        with pytest.raises(L.GrmpError) as ei:
            sysd.assemble_and_solve(solver)
        assert ei.value.code == L.ERR_TIMEOUT
        assert "timed out" in str(ei.value)
    finally:
        ctx.check(ctx.lib.grmp_context_set_wait_limit(ctx.h, 0))
    st = sysd.assemble_and_solve(solver)
    assert st["status"] == 0 and st["iterations"] > 0
    assert np.isfinite(sysd.x.entries).all()


def test_wait_limit_rejects_negative(ctx):
    from grmp_gb300 import _lib as L
    assert ctx.lib.grmp_context_set_wait_limit(ctx.h, -5) == L.ERR_INVALID_ARG
