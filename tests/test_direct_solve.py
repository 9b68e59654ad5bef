"""Single-problem direct solvers through grmp_solve: FP64 multifrontal
Cholesky with refinement ("direct") and FP32 multifrontal Cholesky as the
preconditioner of FP64 CG ("mixed_direct"), against the oracle's
sparse-direct FP64 solution (relative 2-norm error <= 1e-10)."""
import numpy as np
import pytest

from parity_helpers import oracle_system

pytestmark = pytest.mark.gpu


def _problems(G):
    from grmp_gb300 import problems as P
    return [P.poisson2d(24), P.poisson2d(20, order=1), P.elasticity2d(12, lam=1e3), P.poisson3d(5, order=2),
            P.poisson3d(7, order=1)]


@pytest.mark.parametrize("idx", range(5))
@pytest.mark.parametrize("mode", ["direct", "mixed_direct"])
def test_direct_solve_matches_oracle(G, O, ctx, idx, mode):
    from grmp_gb300 import problems as P
    prob = _problems(G)[idx]
    _, Apen, _, bpen = oracle_system(G, O, prob)
    uo = O.solve_direct(Apen, bpen)
    sysd = P.DeviceSystem(ctx, prob, mixed=False)
    st = sysd.assemble_and_solve(G.GB300PCG(mode=mode, reltol=1e-12, abstol=0.0, maxiter=200))
    u = sysd.x.entries
    err = np.linalg.norm(u - uo) / np.linalg.norm(uo)
    assert err <= 1e-10, (prob.name, err, st)
    assert st["iterations"] <= (4 if mode == "direct" else 60), st


def test_direct_solve_repeats_bitwise(G, ctx):
    """The factorisation is recomputed per call from the same values with
    fixed launch shapes: two solves give the same bits."""
    from grmp_gb300 import problems as P
    prob = P.elasticity2d(10, lam=1e3)
    sysd = P.DeviceSystem(ctx, prob, mixed=False)
    sysd.assemble_and_solve(G.GB300PCG(mode="mixed_direct", reltol=1e-12, abstol=0.0))
    u1 = sysd.x.entries
    sysd.assemble_and_solve(G.GB300PCG(mode="mixed_direct", reltol=1e-12, abstol=0.0))
    assert np.array_equal(u1, sysd.x.entries)


@pytest.mark.parametrize("mode", ["direct", "mixed_direct"])
def test_direct_solve_large_fronts(G, O, ctx, mode):
    """2D P2 elasticity on 96x96 squares (74k DoFs): the top fronts exceed
    1024 DoFs and are factored by the whole grid (cooperative launch).
    With lambda/mu = 1e3 this system's condition number is ~1e7, so two
    backward-stable FP64 solutions (ours, the oracle's SuperLU) can only agree
    to ~kappa*u = 1e-9: the tolerance here is 1e-8; the 1e-10 bar is held on
    the better-conditioned cases above.  Solved to the FP64 residual floor."""
    from grmp_gb300 import problems as P
    prob = P.elasticity2d(96, lam=1e3)
    _, Apen, _, bpen = oracle_system(G, O, prob)
    uo = O.solve_direct(Apen, bpen)
    sysd = P.DeviceSystem(ctx, prob, mixed=False)
    st = sysd.assemble_and_solve(G.GB300PCG(mode=mode, reltol=1e-14, abstol=0.0, maxiter=300))
    u = sysd.x.entries
    err = np.linalg.norm(u - uo) / np.linalg.norm(uo)
    assert err <= 1e-8, (err, st)
