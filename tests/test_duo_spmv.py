"""The mixed solver over the two-run 16-bit column copy of the FP32 matrix
(duo records, spmv_config 60xxx) on the other problem shapes: 2D P2 Poisson
at the config-1 size, P1, a vector (elasticity) pattern, a repeat run for
reproducibility, the refusal for a plain FP64 solve, and the FP32 values
refreshed after a reassembly with other coefficients.  Tolerance: 1e-10
relative 2-norm error against the oracle's sparse-direct FP64 solution."""
import numpy as np
import pytest

from parity_helpers import oracle_system

pytestmark = pytest.mark.gpu


def _solve_oracle(G, O, prob):
    _, Apen, _, bpen = oracle_system(G, O, prob)
    return O.solve_direct(Apen, bpen)


@pytest.mark.parametrize("which,cfg", [("p2_128", 60404), ("p2_128", 60208), ("p1_96", 60802),
                                       ("p1_96", 60404), ("p2_128", 64208), ("p1_96", 64404),
                                       ("p2_128", 65404), ("p1_96", 65208)])
def test_duo_2d_matches_oracle(G, O, ctx, which, cfg):
    from grmp_gb300 import problems as P
    prob = P.poisson2d(128) if which == "p2_128" else P.poisson2d(96, order=1)
    uo = _solve_oracle(G, O, prob)
    sysd = P.DeviceSystem(ctx, prob, mixed=True)
    st = sysd.assemble_and_solve(G.GB300PCG(mode="mixed", reltol=1e-11, abstol=0.0, spmv_config=cfg))
    assert st["spmv_config"] == cfg
    u = sysd.x.entries
    assert np.linalg.norm(u - uo) / np.linalg.norm(uo) <= 1e-10


def test_duo_repeatable_and_refreshed(G, O, ctx):
    """Two solves agree bit for bit; after reassembly with other cell
    coefficients the duo values follow (the solution matches the oracle of
    the new problem, not the old one)."""
    from grmp_gb300 import problems as P
    prob = P.poisson3d(6, seed=7)
    sysd = P.DeviceSystem(ctx, prob, mixed=True)
    solver = G.GB300PCG(mode="mixed", reltol=1e-11, abstol=0.0, spmv_config=60404)
    sysd.assemble_and_solve(solver)
    u1 = sysd.x.entries
    sysd.assemble_and_solve(solver)
    assert np.array_equal(u1, sysd.x.entries)
    prob2 = P.poisson3d(6, seed=8)   # same mesh and pattern, other kappa and rhs
    sysd.prob = prob2
    sysd.assemble_and_solve(solver)
    uo2 = _solve_oracle(G, O, prob2)
    u2 = sysd.x.entries
    assert np.linalg.norm(u2 - uo2) / np.linalg.norm(uo2) <= 1e-10


def test_fp64_refuses_duo(G, ctx):
    from grmp_gb300 import _lib as L
    from grmp_gb300 import problems as P
    prob = P.poisson2d(8)
    sysd = P.DeviceSystem(ctx, prob, mixed=False)
    with pytest.raises(L.GrmpError) as ei:
        sysd.assemble_and_solve(G.GB300PCG(mode="fp64", reltol=1e-10, abstol=0.0, spmv_config=60404))
    assert ei.value.code == L.ERR_UNSUPPORTED
