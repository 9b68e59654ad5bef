"""The persistent PCG in one thread-block cluster (spmv_config 7xxxx: row loop,
FP64 and mixed; 8xxxx: two-run 16-bit columns, mixed): hardware cluster
barriers and reductions through distributed shared memory instead of grid
barriers, for systems that sit in L2.  Tolerance: 1e-10 relative 2-norm
error against the oracle's sparse-direct FP64 solution (the same bar as the
grid-wide solvers), bitwise repeatability, and the no-allocation FP64 entry
point running the same cluster launch."""
import ctypes

import numpy as np
import pytest

from parity_helpers import oracle_system

pytestmark = pytest.mark.gpu


def _prob(which):
    from grmp_gb300 import problems as P
    return {"p2_128": lambda: P.poisson2d(128), "p1_96": lambda: P.poisson2d(96, order=1),
            "p2_3d_6": lambda: P.poisson3d(6, seed=3)}[which]()


@pytest.mark.parametrize("which,mode,cfg", [("p2_128", "fp64", 70204), ("p2_128", "fp64", 70404),
                                            ("p2_128", "mixed", 70204), ("p2_128", "mixed", 80204),
                                            ("p2_128", "mixed", 80404), ("p1_96", "mixed", 70404),
                                            ("p2_3d_6", "fp64", 70802), ("p2_3d_6", "mixed", 80404)])
def test_cluster_solve_matches_oracle(G, O, ctx, which, mode, cfg):
    from grmp_gb300 import problems as P
    prob = _prob(which)
    _, Apen, _, bpen = oracle_system(G, O, prob)
    uo = O.solve_direct(Apen, bpen)
    sysd = P.DeviceSystem(ctx, prob, mixed=mode == "mixed")
    st = sysd.assemble_and_solve(G.GB300PCG(mode=mode, reltol=1e-11, abstol=0.0, spmv_config=cfg))
    assert st["spmv_config"] == cfg
    assert st["grid_blocks"] in (8, 16)   # one cluster
    u = sysd.x.entries
    assert np.linalg.norm(u - uo) / np.linalg.norm(uo) <= 1e-10


@pytest.mark.parametrize("mode,cfg", [("fp64", 70404), ("mixed", 80204)])
def test_cluster_solve_repeatable(G, ctx, mode, cfg):
    from grmp_gb300 import problems as P
    prob = P.poisson2d(64)
    sysd = P.DeviceSystem(ctx, prob, mixed=mode == "mixed")
    solver = G.GB300PCG(mode=mode, reltol=1e-11, abstol=0.0, spmv_config=cfg)
    st1 = sysd.assemble_and_solve(solver)
    u1 = sysd.x.entries.copy()
    st2 = sysd.assemble_and_solve(solver)
    assert st1["iterations"] == st2["iterations"]
    assert np.array_equal(u1, sysd.x.entries)


def test_noalloc_runs_the_cluster_launch(G, ctx):
    from grmp_gb300 import _lib as L
    from grmp_gb300 import problems as P
    prob = P.poisson2d(48)
    sysd = P.DeviceSystem(ctx, prob, mixed=False)
    solver = G.GB300PCG(mode="fp64", reltol=1e-11, abstol=0.0, spmv_config=70404)
    ref = sysd.assemble_and_solve(solver)
    xref = sysd.x.entries.copy()
    sysd.x.fill(5.0)
    p = solver.params()
    st = L.SolveStats()
    rc = ctx.lib.grmp_solve_fp64_noalloc(sysd.A.h, sysd.b.h, sysd.x.h, ctypes.byref(p), ctypes.byref(st))
    assert rc == 0, ctx.lib.grmp_last_error(ctx.h)
    assert st.spmv_config == 70404 and st.grid_blocks == ref["grid_blocks"]
    assert np.array_equal(sysd.x.entries, xref)   # same launch, same reduction order
