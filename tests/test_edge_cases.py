"""Edge cases of the assembly + solve path: the smallest meshes (one triangle,
one tetrahedron), right-hand sides that are exactly zero, every DoF fixed,
a graded mesh whose cell areas span five orders of magnitude, a degenerate
(zero-area) cell, and empty meshes the C-ABI rejects before any launch.
Solutions are compared with the oracle's sparse-direct FP64 solution at
1e-10 relative 2-norm error, the bar of the other parity tests."""
import ctypes

import numpy as np
import pytest

from parity_helpers import oracle_system

pytestmark = pytest.mark.gpu


def _single_cell(G, dim):
    if dim == 2:
        coords = np.array([[0.0, 0.0], [1.0, 0.2], [0.3, 0.9]])
        cells = np.array([[0, 1, 2]])
    else:
        coords = np.array([[0.0, 0.0, 0.0], [1.0, 0.1, 0.0], [0.2, 0.8, 0.1], [0.1, 0.2, 0.7]])
        cells = np.array([[0, 1, 2, 3]])
    return G.SimplexMesh(coords, cells)


def _problem(G, g, order, operators, fixed=None):
    from grmp_gb300 import problems as P
    from grmp_gb300.fespace import FESpace, H1P1, H1P2
    FES = FESpace(H1P1(1) if order == 1 else H1P2(1, g.dim), g)
    rhs = G.LinearForm(G.Identity, G.DataFunction.constant([1.0]))
    fx = np.zeros(0, dtype=np.int32) if fixed is None else np.asarray(fixed, dtype=np.int32)
    return P.LinearProblem("edge", FES, operators, rhs, fx, {})


def _solve(G, ctx, prob, mode, cfg=0, reltol=1e-12):
    from grmp_gb300 import problems as P
    sysd = P.DeviceSystem(ctx, prob, mixed=mode == "mixed")
    st = sysd.assemble_and_solve(G.GB300PCG(mode=mode, reltol=reltol, abstol=0.0, spmv_config=cfg))
    return sysd, st


@pytest.mark.parametrize("dim,order", [(2, 1), (2, 2), (3, 1), (3, 2)])
@pytest.mark.parametrize("mode", ["fp64", "mixed"])
def test_single_cell_matches_oracle(G, O, ctx, dim, order, mode):
    """One simplex, Laplace + reaction (positive definite without boundary
    conditions), f = 1: 3 to 10 DoFs, so the mixed solve takes the
    one-cluster solver of the row-length heuristic."""
    g = _single_cell(G, dim)
    prob = _problem(G, g, order, [G.LaplaceOperator(1.0), G.ReactionOperator(2.0)])
    _, Apen, _, bpen = oracle_system(G, O, prob)
    uo = O.solve_direct(Apen, bpen)
    sysd, st = _solve(G, ctx, prob, mode, cfg=-1)
    if mode == "mixed":
        assert st["spmv_config"] >= 70000   # one cluster
    assert np.linalg.norm(sysd.x.entries - uo) <= 1e-10 * np.linalg.norm(uo)


@pytest.mark.parametrize("mode,cfg", [("fp64", 408), ("fp64", 70404), ("mixed", 10408), ("mixed", 60208),
                                      ("mixed", 66404), ("mixed", 70204), ("mixed", 80204)])
def test_zero_rhs_gives_zero_solution(G, ctx, mode, cfg):
    """b = 0 exactly: every solver form returns x = 0 with no iteration."""
    from grmp_gb300 import problems as P
    prob = P.poisson3d(3, seed=1)
    sysd = P.DeviceSystem(ctx, prob, mixed=mode == "mixed")
    G.assemble(sysd.A, prob.operators, G.FP64_FP32 if mode == "mixed" else G.FP64)
    sysd.b.fill(0.0)
    G.apply_dirichlet(sysd.A, sysd.b, prob.fixed, None, G.DIRICHLET_ELIMINATE)
    sysd.x.fill(7.0)
    st = G.GB300PCG(mode=mode, reltol=1e-12, abstol=0.0, spmv_config=cfg).solve(sysd.A, sysd.b, sysd.x)
    assert st["iterations"] == 0 and st["status"] == 0
    assert not np.any(sysd.x.entries)


@pytest.mark.parametrize("mode,cfg", [("fp64", 0), ("mixed", 0), ("mixed", 66404), ("mixed", 70204)])
def test_every_dof_fixed(G, ctx, mode, cfg):
    """All DoFs carry Dirichlet values: elimination leaves the identity and
    the solution is the prescribed values."""
    from grmp_gb300 import problems as P
    prob = P.poisson2d(6)
    sysd = P.DeviceSystem(ctx, prob, mixed=mode == "mixed")
    G.assemble(sysd.A, prob.operators, G.FP64_FP32 if mode == "mixed" else G.FP64)
    sysd.b.fill(0.0)
    G.assemble(sysd.b, prob.rhs)
    n = prob.FES.ndofs
    fixed = np.arange(n, dtype=np.int32)
    vals = np.random.default_rng(3).standard_normal(n)
    G.apply_dirichlet(sysd.A, sysd.b, fixed, vals, G.DIRICHLET_ELIMINATE)
    G.GB300PCG(mode=mode, reltol=1e-12, abstol=0.0, spmv_config=cfg).solve(sysd.A, sysd.b, sysd.x)
    assert np.max(np.abs(sysd.x.entries - vals)) <= 1e-12 * np.max(np.abs(vals))


@pytest.mark.parametrize("mode", ["fp64", "mixed"])
def test_graded_mesh_matches_oracle(G, O, ctx, mode):
    """Unit square 32 x 32 mapped by x -> x^3, y -> y^2: cell areas from about
    2e-8 to 3e-3 (five orders of magnitude), aspect ratios up to ~30, P2, zero
    boundary values; solved to relative residual 1e-13."""
    g0 = G.grid_unitsquare(32)
    c = g0.coords.copy()
    c[:, 0] = c[:, 0] ** 3
    c[:, 1] = c[:, 1] ** 2
    g = G.SimplexMesh(c, g0.cells)
    from grmp_gb300.fespace import FESpace, H1P2
    FES = FESpace(H1P2(1, 2), g)
    prob = _problem(G, g, 2, [G.LaplaceOperator(1.0)], fixed=FES.boundary_dofs())
    _, Apen, _, bpen = oracle_system(G, O, prob)
    uo = O.solve_direct(Apen, bpen)
    sysd, _ = _solve(G, ctx, prob, mode, reltol=1e-13)
    assert np.linalg.norm(sysd.x.entries - uo) <= 1e-10 * np.linalg.norm(uo)


def test_degenerate_cell_fails_loudly(G, ctx):
    """A zero-area triangle (collinear vertices) makes the element map
    singular: the solve must report an error, not return numbers."""
    coords = np.array([[0.0, 0.0], [1.0, 0.0], [1.0, 1.0], [0.0, 1.0], [2.0, 0.0]])
    cells = np.array([[0, 1, 2], [0, 2, 3], [0, 1, 4]])   # the last one is degenerate
    g = G.SimplexMesh(coords, cells)
    prob = _problem(G, g, 1, [G.LaplaceOperator(1.0), G.ReactionOperator(1.0)])
    for mode in ("fp64", "mixed"):
        with pytest.raises(G.GrmpError):
            _solve(G, ctx, prob, mode, cfg=-1)


@pytest.mark.parametrize("nverts,ncells", [(0, 1), (3, 0)])
def test_empty_mesh_rejected(G, ctx, nverts, ncells):
    coords = np.zeros((max(nverts, 1), 2))
    cells = np.zeros((max(ncells, 1), 3), dtype=np.int32)
    h = ctypes.c_void_p()
    rc = ctx.lib.grmp_mesh_upload(ctx.h, 2, nverts, coords.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), ncells,
                                  cells.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)), ctypes.byref(h))
    assert rc == 1 and not h.value
