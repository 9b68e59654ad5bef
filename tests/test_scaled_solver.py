"""The Jacobi-scaled mixed solver with the row state kept on chip
(spmv_config 64xxx / 65xxx / 66xxx) beyond the Poisson parity cases: a
starting guess, a vector (elasticity) pattern, a reaction term, and a matrix
imported from a penalised CSC (penalty rows eliminated before the FP32 copy
is scaled).  Tolerance: 1e-10 relative 2-norm error against the oracle's
sparse-direct FP64 solution, as in the other parity tests."""
import numpy as np
import pytest

from parity_helpers import oracle_system

pytestmark = pytest.mark.gpu

CFGS = [64404, 65208, 66404]


def _oracle(G, O, prob):
    _, Apen, _, bpen = oracle_system(G, O, prob)
    return O.solve_direct(Apen, bpen)


def _rel(u, uo):
    return np.linalg.norm(u - uo) / np.linalg.norm(uo)


@pytest.mark.parametrize("cfg", CFGS)
def test_starting_guess(G, O, ctx, cfg):
    from grmp_gb300 import problems as P
    prob = P.poisson3d(8, seed=4)
    uo = _oracle(G, O, prob)
    sysd = P.DeviceSystem(ctx, prob, mixed=True)
    G.assemble(sysd.A, prob.operators, G.FP64_FP32)
    sysd.b.fill(0.0)
    G.assemble(sysd.b, prob.rhs)
    G.apply_dirichlet(sysd.A, sysd.b, prob.fixed, None, G.DIRICHLET_ELIMINATE)
    rng = np.random.default_rng(5)
    sysd.x.upload(uo * (1.0 + 1e-3 * rng.standard_normal(uo.size)))
    st = G.GB300PCG(mode="mixed", reltol=1e-12, abstol=0.0, spmv_config=cfg, use_initial_guess=True).solve(
        sysd.A, sysd.b, sysd.x)
    assert st["spmv_config"] == cfg
    assert _rel(sysd.x.entries, uo) <= 1e-10


@pytest.mark.parametrize("cfg", CFGS)
def test_vector_pattern(G, O, ctx, cfg):
    """2D P2 elasticity (two components per node, Hooke with lambda = 10 so
    that Jacobi-PCG converges), clamped on the left edge."""
    from grmp_gb300 import problems as P
    prob = P.elasticity2d(10, seed=3, mu=1.0, lam=10.0)
    uo = _oracle(G, O, prob)
    sysd = P.DeviceSystem(ctx, prob, mixed=True)
    st = sysd.assemble_and_solve(G.GB300PCG(mode="mixed", reltol=1e-12, abstol=0.0, spmv_config=cfg))
    assert st["spmv_config"] == cfg
    assert _rel(sysd.x.entries, uo) <= 1e-10


@pytest.mark.parametrize("cfg", CFGS)
def test_reaction_term(G, O, ctx, cfg):
    """3D P1 Laplace + reaction (alpha = 5) on 6^3 Kuhn cubes, zero boundary values."""
    from grmp_gb300 import problems as P
    from grmp_gb300.fespace import FESpace, H1P1
    g = G.grid_unitcube_kuhn(6)
    FES = FESpace(H1P1(1), g)
    ops = [G.LaplaceOperator(1.0), G.ReactionOperator(5.0)]
    rhs = G.LinearForm(G.Identity, G.DataFunction.constant([1.0]))
    prob = P.LinearProblem("reaction", FES, ops, rhs, FES.boundary_dofs(), {})
    uo = _oracle(G, O, prob)
    sysd = P.DeviceSystem(ctx, prob, mixed=True)
    st = sysd.assemble_and_solve(G.GB300PCG(mode="mixed", reltol=1e-12, abstol=0.0, spmv_config=cfg))
    assert st["spmv_config"] == cfg
    assert _rel(sysd.x.entries, uo) <= 1e-10


@pytest.mark.parametrize("cfg", CFGS)
def test_imported_penalised_matrix(G, O, ctx, cfg):
    """LinearSolve's penalised SparseMatrixCSC (1-based, 1e60 rows) through
    the import: the penalty rows are eliminated before the FP32 copy is
    scaled, so nothing overflows and the scales stay O(1)."""
    from grmp_gb300 import problems as P
    prob = P.poisson3d(6, seed=2)
    _, Apen, _, bpen = oracle_system(G, O, prob)
    uo = O.solve_direct(Apen, bpen)
    C = Apen.tocsc()
    C.sort_indices()
    M = G.ImportedMatrix(ctx, (C.indptr.astype(np.int64) + 1, C.indices.astype(np.int64) + 1, C.data.copy()),
                         penalty_threshold=1e30, index_base=1)
    b = G.FEVector(ctx, prob.FES)
    b.upload(bpen)
    x = G.FEVector(ctx, prob.FES)
    st = G.GB300PCG(mode="mixed", reltol=1e-12, abstol=0.0, spmv_config=cfg).solve(M, b, x)
    assert st["spmv_config"] == cfg
    assert _rel(x.entries, uo) <= 1e-10
    M.free()
