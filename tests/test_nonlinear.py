"""NonlinearForm Newton terms and the Newton loop (src/assemblypatterns/
nonlinearform.jl:44-240, src/solvers.jl:519-566).

CPU: the oracle's Newton terms are pinned three ways -- with beta = 0 the
diffusion kernel is LaplaceOperator, so DG(u) is the oracle's (pinned)
Laplace matrix and DG(u) u - G(u) vanishes; the Jacobian agrees with central
differences of G(u) = DG(u) u - (DG(u) u - G(u)) for every kernel; and the
Newton loop of the nonlinear Poisson problem of
examples/Example205_NonlinearPoisson2D.jl converges quadratically.
GPU: the device's Newton terms against the oracle's per entry, BiCGStab
against a sparse LU, and the device Newton loop against the oracle's.
"""
import numpy as np
import pytest


def _space(G, dim, order, ncomp=1, n=None):
    from grmp_gb300 import fespace as F
    g = (G.grid_unitsquare(n or 6) if dim == 2 else G.grid_unitcube_kuhn(n or 3))
    ft = F.H1P1(ncomp) if order == 1 else F.H1P2(ncomp, dim)
    return g, F.FESpace(ft, g)


def _oracle_terms(O, g, S, u, kind, kappa=1.0, beta=1.0, bonus=2):
    fe = 1 if S.FEType.kind == 1 else 2
    M = O.Matrix(S.ndofs)
    b = np.zeros(S.ndofs)
    O.nl_assemble(M, b, g.coords, g.cells, fe, S.FEType.ncomponents, S.celldofs, u, kind, 1.0, kappa, beta, bonus)
    return M.csr(), b


def _G(O, g, S, u, kind, **kw):
    """G(u) = DG(u) u - (DG(u) u - G(u))."""
    A, b = _oracle_terms(O, g, S, u, kind, **kw)
    return A @ u - b, A


@pytest.mark.parametrize("dim,order", [(2, 1), (2, 2), (3, 2)])
def test_oracle_nl_diffusion_linear_limit_is_laplace(G, O, dim, order):
    g, S = _space(G, dim, order)
    rng = np.random.default_rng(1)
    u = rng.standard_normal(S.ndofs)
    A, b = _oracle_terms(O, g, S, u, O.NL_DIFFUSION, kappa=2.5, beta=0.0, bonus=0)
    M = O.Matrix(S.ndofs)
    M.add_bilinear(g.coords, g.cells, order, 1, S.celldofs, O.OP_GRADIENT, True, 2.5)
    L = M.csr()
    scale = np.max(np.abs(L.data))
    assert np.max(np.abs((A - L).toarray())) <= 1e-14 * scale
    assert np.max(np.abs(b)) <= 1e-13 * scale * np.max(np.abs(u))


@pytest.mark.parametrize("kind,dim,order,ncomp", [(1, 2, 2, 1), (1, 3, 1, 1), (2, 2, 1, 1), (2, 2, 2, 1),
                                                  (3, 2, 2, 2), (3, 3, 1, 3)])
def test_oracle_nl_jacobian_matches_finite_differences(G, O, kind, dim, order, ncomp):
    g, S = _space(G, dim, order, ncomp, n=4 if dim == 2 else 2)
    rng = np.random.default_rng(2)
    u = rng.standard_normal(S.ndofs) * 0.5
    d = rng.standard_normal(S.ndofs)
    eps = 1e-5
    Gp, _ = _G(O, g, S, u + eps * d, kind)
    Gm, _ = _G(O, g, S, u - eps * d, kind)
    _, A = _G(O, g, S, u, kind)
    Ad = A @ d
    fd = (Gp - Gm) / (2 * eps)
    assert np.linalg.norm(fd - Ad) <= 1e-7 * np.linalg.norm(Ad)


def test_oracle_newton_converges_quadratically(G, O):
    """-div((1 + u^2) grad u) = f, f = 10, zero boundary values (the
    nonlinear diffusion of examples/Example205_NonlinearPoisson2D.jl:114)."""
    g, S = _space(G, 2, 2, n=8)
    u, its = O.newton_nonlinear_poisson(g.coords, g.cells, 2, S.celldofs, S.ndofs, [(0, 10.0, 0, 0, 0)],
                                        S.boundary_dofs(), maxit=20, tol=1e-13)
    ch = [np.linalg.norm(its[k + 1] - its[k]) for k in range(len(its) - 1)]
    assert len(its) <= 10 and ch[-1] <= 1e-12 * np.linalg.norm(u)
    # quadratic: the change roughly squares from step to step once small
    small = [c for c in ch if c < 1e-2]
    for a, b in zip(small, small[1:]):
        if b > 1e-13:
            assert b <= 10 * a * a, ch


# ----------------------------------------------------------------------- GPU

@pytest.mark.gpu
@pytest.mark.parametrize("kind,dim,order,ncomp", [(1, 2, 1, 1), (1, 2, 2, 1), (1, 3, 2, 1), (2, 2, 2, 1),
                                                  (2, 3, 1, 1), (3, 2, 2, 2), (3, 3, 1, 3), (3, 3, 2, 3)])
def test_nl_terms_match_oracle(G, O, ctx, kind, dim, order, ncomp):
    """DG(u) and DG(u) u - G(u) on the device against the oracle, per entry
    to 1e-12 of the largest entry (entries of the structural pattern that
    the oracle drops as exact zeros must be zero to the same bound)."""
    g, S = _space(G, dim, order, ncomp, n=5 if dim == 2 else 2)
    rng = np.random.default_rng(3)
    uh = rng.standard_normal(S.ndofs) * 0.7
    A = G.FEMatrix(ctx, S, [G.StructuralCoupling()])
    b = G.FEVector(ctx, S)
    u = G.FEVector(ctx, S)
    u.upload(uh)
    b.fill(0.0)
    form = G.NonlinearForm({1: "diffusion", 2: "grad_diffusion", 3: "convection"}[kind], kappa=1.3, beta=0.8,
                           bonus_quadorder=2)
    G.assemble_nonlinear(A, b, u, form, G.FP64, add=False)
    Ad = A.download(G.FP64).toarray()
    Ao, bo = _oracle_terms(O, g, S, uh, kind, kappa=1.3, beta=0.8, bonus=2)
    Ao = Ao.toarray()
    assert np.max(np.abs(Ad - Ao)) <= 1e-12 * np.max(np.abs(Ao))
    assert np.max(np.abs(b.entries - bo)) <= 1e-12 * np.max(np.abs(bo))


@pytest.mark.gpu
def test_bicgstab_solves_newton_system(G, O, ctx):
    import scipy.sparse.linalg as spla
    g, S = _space(G, 2, 2, n=24)
    rng = np.random.default_rng(4)
    A = G.FEMatrix(ctx, S, [G.LaplaceOperator(1.0), G.StructuralCoupling()])
    b, u, x = G.FEVector(ctx, S), G.FEVector(ctx, S), G.FEVector(ctx, S)
    u.upload(rng.standard_normal(S.ndofs))
    G.assemble(A, [G.LaplaceOperator(1.0), G.StructuralCoupling()], G.FP64)
    b.upload(rng.standard_normal(S.ndofs))
    G.assemble_nonlinear(A, b, u, G.NonlinearForm("diffusion", kappa=1.0, beta=1.0), G.FP64, add=True)
    G.apply_dirichlet(A, b, S.boundary_dofs(), None, G.DIRICHLET_ELIMINATE)
    st = G.GB300PCG(mode="bicgstab", reltol=1e-13, abstol=0.0).solve(A, b, x)
    M = A.download(G.FP64).tocsc()
    assert abs(M - M.T).max() > 1e-3          # really non-symmetric
    xr = spla.spsolve(M, b.entries)
    assert np.linalg.norm(x.entries - xr) <= 1e-10 * np.linalg.norm(xr), st


@pytest.mark.gpu
@pytest.mark.parametrize("dim,order", [(2, 2), (3, 1)])
def test_solve_nonlinear_matches_oracle_newton(G, O, ctx, dim, order):
    g, S = _space(G, dim, order, n=16 if dim == 2 else 6)
    fixed = S.boundary_dofs()
    lf = G.LinearForm(G.Identity, G.DataFunction.constant([10.0]))
    form = G.NonlinearForm("diffusion", kappa=1.0, beta=1.0, bonus_quadorder=2)
    ud, stats = G.solve_nonlinear(ctx, S, [], form, lf, fixed, maxiterations=20, target_change=1e-13)
    uo, its = O.newton_nonlinear_poisson(g.coords, g.cells, order, S.celldofs, S.ndofs, [(0, 10.0, 0, 0, 0)], fixed,
                                         maxit=20, tol=1e-13)
    assert abs(len(stats) - len(its)) <= 1
    assert np.linalg.norm(ud - uo) <= 1e-10 * np.linalg.norm(uo)


@pytest.mark.gpu
def test_nl_refuses_pattern_without_structural_coupling(G, ctx):
    g, S = _space(G, 2, 1, n=6)
    A = G.FEMatrix(ctx, S, [G.LaplaceOperator(1.0)])   # drops the right-angle couplings
    b, u = G.FEVector(ctx, S), G.FEVector(ctx, S)
    u.upload(np.random.default_rng(5).standard_normal(S.ndofs))
    b.fill(0.0)
    G.assemble(A, [G.LaplaceOperator(1.0)], G.FP64)
    with pytest.raises(G.GrmpError):
        G.assemble_nonlinear(A, b, u, G.NonlinearForm("diffusion"), G.FP64, add=True)
