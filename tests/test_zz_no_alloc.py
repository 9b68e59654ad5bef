"""grmp_solve_fp64_noalloc: the FP64 solve whose work arrays are a fixed
scratch area of the library instead of device allocations.

This file is named to be collected last: the entry point must give the same
result when it runs after every other GPU test in the same process (its
scratch is then reused, not fresh).  Results are compared with the ordinary
grmp_solve entry point on the same system, on two calls in a row.
"""
import ctypes
import gc

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

REL_TOL = 1e-12   # same configuration and grid as grmp_solve: agreement to rounding


def _system(G, ctx, n, order=2):
    from grmp_gb300 import problems as P
    prob = P.poisson2d(n, order=order)
    sysd = P.DeviceSystem(ctx, prob, mixed=False)
    G.assemble(sysd.A, prob.operators, G.FP64)
    sysd.b.fill(0.0)
    G.assemble(sysd.b, prob.rhs)
    G.apply_dirichlet(sysd.A, sysd.b, prob.fixed, None, G.DIRICHLET_ELIMINATE)
    return sysd


def _noalloc(ctx, sysd, solver):
    from grmp_gb300 import _lib as L
    p = solver.params()
    st = L.SolveStats()
    rc = ctx.lib.grmp_solve_fp64_noalloc(sysd.A.h, sysd.b.h, sysd.x.h, ctypes.byref(p), ctypes.byref(st))
    return rc, st


@pytest.mark.parametrize("n", [24, 160])   # 2,401 and 103,041 DoFs (the latter autotuned by grmp_solve)
def test_noalloc_matches_solve_on_two_calls(G, ctx, n):
    sysd = _system(G, ctx, n)
    solver = G.GB300PCG(mode="fp64", reltol=1e-11, abstol=0.0)
    ref_stats = solver.solve(sysd.A, sysd.b, sysd.x)
    xref = sysd.x.entries
    gc.collect()   # handles of earlier tests freed now, not during the calls below
    mem0 = ctx.memory_in_use()
    for call in range(2):
        sysd.x.fill(123.0)   # overwritten: use_initial_guess = 0
        rc, st = _noalloc(ctx, sysd, solver)
        assert rc == 0, ctx.lib.grmp_last_error(ctx.h)
        assert st.status == 0
        assert st.spmv_config == ref_stats["spmv_config"]
        assert st.grid_blocks == ref_stats["grid_blocks"]   # the tuned grid too: the same launch
        assert st.final_relres <= max(1e-10, 2.0 * ref_stats["final_relres"])
        x = sysd.x.entries
        err = np.linalg.norm(x - xref) / np.linalg.norm(xref)
        assert err <= REL_TOL, (call, err)
    gc.collect()
    assert ctx.memory_in_use() == mem0   # nothing was allocated through the context


def test_noalloc_rejects_oversize_and_mixed(G, ctx):
    from grmp_gb300 import _lib as L
    big = _system(G, ctx, 512, order=1)   # 513^2 = 263,169 rows > GRMP_NOALLOC_MAX_ROWS
    assert big.A.info()[0] > L.NOALLOC_MAX_ROWS
    rc, _ = _noalloc(ctx, big, G.GB300PCG(mode="fp64", reltol=1e-8))
    assert rc == L.ERR_INVALID_ARG
    assert b"scratch limit" in ctx.lib.grmp_last_error(ctx.h)
    small = _system(G, ctx, 8)
    rc, _ = _noalloc(ctx, small, G.GB300PCG(mode="mixed", reltol=1e-8))
    assert rc == L.ERR_UNSUPPORTED
    rc, _ = _noalloc(ctx, small, G.GB300PCG(mode="fp64", reltol=-1.0))
    assert rc == L.ERR_INVALID_ARG
    assert b"invalid tolerance" in ctx.lib.grmp_last_error(ctx.h)
