"""Pins of the CPU oracle against the reference's own known-answer tests.

The reference (Julia) cannot run here; its test suite (test/runtests.jl)
asserts exactness properties that survive a change of mesh numbering.  These
tests re-implement them against the oracle:

* quadrature exactness, runtests.jl:81-137 (same polynomials, same orders);
* polynomial reproduction of the elements by L2 / H1 best approximation,
  runtests.jl:170-510 (H1P1, H1P2 scalar and vector, 2D and 3D), here as the
  discrete solve of the Poisson / mass / elasticity problems with a
  polynomial exact solution of the element's order;
* the config-1 drop-exact-zero nnz count (395,265) and DoF count (66,049)
  computed independently when the workloads were specified;
* exact reference-element matrices (tests/golden/p2_reference_matrices.json,
  generated symbolically by tests/golden/make_golden.py).
"""
import json
import math
import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


# --------------------------------------------------------------------- quadrature
def _integrate(O, g, order, func):
    x, w, _ = O.qrule(g.dim, order)
    X = g.coords[g.cells]                         # (nc, d+1, d)
    A = np.transpose(X[:, 1:, :] - X[:, :1, :], (0, 2, 1))   # columns x_j - x_0
    vol = np.abs(np.linalg.det(A)) / math.factorial(g.dim)
    pts = X[:, None, 0, :] + np.einsum("ckj,qj->cqk", A, x[:, :g.dim])
    vals = func(pts)                              # (nc, nq, ncomp)
    return np.einsum("c,q,cqk->k", vol, w, vals)


@pytest.mark.parametrize("order", list(range(1, 21)))
def test_quadrature_triangle_exact(G, O, order):
    """runtests.jl:81-137 on Triangle2D up to order 20 (midpoint, edge
    midpoint and Stroud rules; the symmetric rules at orders 8 and 12-14)."""
    g = G.grid_unitsquare(2)
    p = order

    def f(x):
        return np.stack([x[..., 0] ** p + 2 * x[..., 1] ** p + 1, 3 * x[..., 0] ** p - x[..., 1] ** p - 1], axis=-1)

    val = _integrate(O, g, order, f)
    exact = np.array([3 / (p + 1) + 1, 2 / (p + 1) - 1])
    assert np.allclose(val, exact, rtol=1e-13, atol=1e-13)


@pytest.mark.parametrize("order", list(range(1, 9)))
def test_quadrature_tetrahedron_exact(G, O, order):
    """runtests.jl:81-137 on Tetrahedron3D (hard-coded rules, orders 1-4;
    the symmetric order-8 rule for 5-8)."""
    g = G.grid_unitcube_kuhn(2)
    p = order

    def f(x):
        return np.stack([2 * x[..., 2] ** p - x[..., 1] ** p - 1, x[..., 0] ** p + 2 * x[..., 1] ** p + 1,
                         3 * x[..., 0] ** p - x[..., 1] ** p - 1], axis=-1)

    val = _integrate(O, g, order, f)
    exact = np.array([1 / (p + 1) - 1, 3 / (p + 1) + 1, 2 / (p + 1) - 1])
    # the reference's order-4 tet weights are 16-digit decimals
    assert np.allclose(val, exact, rtol=1e-12, atol=1e-12)


@pytest.mark.parametrize("dim,order,npts", [(2, 8, 16), (2, 12, 46), (2, 13, 46), (2, 14, 46), (3, 5, 46),
                                            (3, 8, 46), (3, 11, 46)])
def test_symmetric_rules(G, O, dim, order, npts):
    """The symmetric rules of src/quadrature.jl:332-499: point counts, points
    inside the reference simplex, weights summing to one (to the digits the
    reference tabulates), and the rule above order 8 on tetrahedra being the
    order-8 rule (the reference warns and takes it)."""
    x, w, exact = O.qrule(dim, order)
    assert exact and x.shape[0] == npts
    assert np.all(x[:, :dim] > 0) and np.all(x[:, :dim].sum(axis=1) < 1)
    assert abs(w.sum() - 1.0) < 1e-4
    if dim == 3 and order > 8:
        x8, w8, _ = O.qrule(3, 8)
        assert np.array_equal(x, x8) and np.array_equal(w, w8)


# --------------------------------------------------------------------- bases
@pytest.mark.parametrize("dim", [2, 3])
def test_p2_basis_partition_of_unity(O, dim):
    x, w, _ = O.qrule(dim, 4)
    vals, der = O.basis_tables(2, dim, x[:, :dim])
    assert np.allclose(vals.sum(axis=1), 1.0, atol=1e-15)
    assert np.allclose(der.sum(axis=1), 0.0, atol=1e-14)


# --------------------------------------------------------------------- golden element matrices
def test_golden_reference_element_matrices(O):
    """Exact rational P1/P2 stiffness and mass matrices of the reference
    simplices (sympy), against the oracle's FP64 assembly on one cell."""
    gold = json.load(open(os.path.join(HERE, "golden", "p2_reference_matrices.json")))
    for key, ent in gold.items():
        dim, fe, kind = ent["dim"], ent["fe"], ent["kind"]
        coords = np.vstack([np.zeros(dim), np.eye(dim)])
        cells = np.arange(dim + 1, dtype=np.int32)[None, :]
        nb = np.array(ent["matrix"]).shape[0]
        cd = np.arange(nb, dtype=np.int32)[None, :]
        M = O.Matrix(nb)
        op = O.OP_GRADIENT if kind == "stiffness" else O.OP_IDENTITY
        M.add_bilinear(coords, cells, fe, 1, cd, op, True, 1.0)
        A = M.csr().toarray()
        ref = np.array(ent["matrix"], dtype=np.float64)
        assert np.allclose(A, ref, rtol=1e-14, atol=1e-15), key


# --------------------------------------------------------------------- counts
def test_config1_counts(G, O):
    """DoFs 66,049; structural nnz 755,713; drop-exact-zero nnz 395,265."""
    g = G.grid_unitsquare(128)
    cd, nd, _ = O.celldofs(2, 1, 2, g.nverts, g.cells)
    assert nd == 66049
    FES = G.FESpace(G.H1P2(1, 2), g)
    assert FES.ndofs == nd and np.array_equal(FES.celldofs, cd)
    rows = np.repeat(cd, cd.shape[1], axis=1).ravel()
    cols = np.tile(cd, (1, cd.shape[1])).ravel()
    assert np.unique(rows.astype(np.int64) * nd + cols).size == 755713
    A = O.Matrix(nd)
    A.add_bilinear(g.coords, g.cells, 2, 1, cd, O.OP_GRADIENT, True, 1e-3)
    assert A.csr().nnz == 395265


@pytest.mark.parametrize("fe,dim,ncomp", [(1, 2, 1), (2, 2, 1), (2, 2, 2), (1, 3, 1), (2, 3, 1)])
def test_dofmap_matches_library_host_mirror(G, O, fe, dim, ncomp):
    g = G.grid_unitsquare(3) if dim == 2 else G.grid_unitcube_kuhn(2)
    cd, nd, _ = O.celldofs(fe, ncomp, dim, g.nverts, g.cells)
    T = G.H1P1(ncomp) if fe == 1 else G.H1P2(ncomp, dim)
    FES = G.FESpace(T, g)
    assert FES.ndofs == nd
    assert np.array_equal(FES.celldofs, cd)


# --------------------------------------------------------------------- exactness solves
def _poly_eval(terms, ncomp, x):
    out = np.zeros((x.shape[0], ncomp))
    for c, coef, e1, e2, e3 in terms:
        v = coef * x[:, 0] ** e1 * x[:, 1] ** e2
        if x.shape[1] > 2:
            v = v * x[:, 2] ** e3
        out[:, int(c)] += v
    return out


def _dof_points(G, FES):
    """Coordinates of the Lagrange nodes of H1P1 / H1P2 DoFs (component 0)."""
    g = FES.xgrid
    pts = [g.coords]
    if FES.FEType.kind == G.FE_H1P2:
        en = g.faces()[0] if g.dim == 2 else g.edges()[0]
        pts.append(g.coords[en].mean(axis=1))
    return np.concatenate(pts)


@pytest.mark.parametrize("dim,fe", [(2, 1), (2, 2), (3, 1), (3, 2)])
def test_poisson_reproduces_polynomial(G, O, dim, fe):
    """H1 best approximation / Poisson exactness (runtests.jl:170-510):
    u = x^2 + 2y^2 (+ 3z^2) is in P2 (u = x + 2y (+3z) for P1); with
    -div(grad u) = f and u on the boundary (penalty 1e60) the discrete
    solution is u at every DoF."""
    g = G.grid_unitsquare(4) if dim == 2 else G.grid_unitcube_kuhn(2)
    T = G.H1P1(1) if fe == 1 else G.H1P2(1, dim)
    FES = G.FESpace(T, g)
    p = 2 if fe == 2 else 1
    terms = [(0, 1.0, p, 0, 0), (0, 2.0, 0, p, 0)] + ([(0, 3.0, 0, 0, p)] if dim == 3 else [])
    lap = (2.0 + 4.0 + (6.0 if dim == 3 else 0.0)) if p == 2 else 0.0   # Laplacian of u
    A = O.Matrix(FES.ndofs)
    A.add_bilinear(g.coords, g.cells, fe, 1, FES.celldofs, O.OP_GRADIENT, True, 1.0)
    b = np.zeros(FES.ndofs)
    O.assemble_linear(b, g.coords, g.cells, fe, 1, FES.celldofs, O.RHS_CONST, [-lap])
    fixed = FES.boundary_dofs()
    pts = _dof_points(G, FES)
    uex = _poly_eval(terms, 1, pts)[:, 0]
    A.penalize(fixed)
    bb = O.penalized_rhs(b, fixed, uex[fixed])
    u = O.solve_direct(A.csr(), bb)
    assert np.max(np.abs(u - uex)) < 1e-11


@pytest.mark.parametrize("dim,fe", [(2, 1), (2, 2), (3, 2)])
def test_l2_bestapprox_reproduces_polynomial(G, O, dim, fe):
    """L2 best approximation (mass matrix + LinearForm with a polynomial f)
    reproduces f of the element's order (runtests.jl:170-510)."""
    g = G.grid_unitsquare(3) if dim == 2 else G.grid_unitcube_kuhn(2)
    T = G.H1P1(1) if fe == 1 else G.H1P2(1, dim)
    FES = G.FESpace(T, g)
    p = fe
    terms = [(0, 1.0, p, 0, 0), (0, 2.0, 0, p, 0), (0, 1.0, 0, 0, 0)] + ([(0, -1.0, 0, 0, p)] if dim == 3 else [])
    A = O.Matrix(FES.ndofs)
    A.add_bilinear(g.coords, g.cells, fe, 1, FES.celldofs, O.OP_IDENTITY, True, 1.0)
    b = np.zeros(FES.ndofs)
    O.assemble_linear(b, g.coords, g.cells, fe, 1, FES.celldofs, O.RHS_POLY, np.array(terms, dtype=float),
                      bonus_quadorder=p)
    u = O.solve_direct(A.csr(), b)
    uex = _poly_eval(terms, 1, _dof_points(G, FES))[:, 0]
    assert np.max(np.abs(u - uex)) < 1e-12


def test_elasticity_reproduces_quadratic_displacement(G, O):
    """HookStiffnessOperator2D on H1P2{2,2}: a quadratic displacement with
    its constant body force -div C eps(u) is reproduced exactly."""
    mu, lam = 1.0, 7.0
    g = G.grid_unitsquare(4)
    FES = G.FESpace(G.H1P2(2, 2), g)
    # u1 = x^2 + xy, u2 = y^2 - 2 x^2
    # eps11 = 2x + y, eps22 = 2y, 2 eps12 = x - 4x = -3x  (du1/dy + du2/dx = x - 4x)
    # sigma = 2 mu eps + lam tr(eps) I ; f = -div sigma
    # d/dx sigma11 = 2mu*2 + lam*2 ; d/dy sigma12 = mu*0 ; f1 = -(4mu + 2lam + 0)
    # sigma22 = (lam+2mu)*2y + lam*(2x+y): d/dy sigma22 = 2(lam+2mu) + lam ; d/dx sigma12 = -3mu
    f1 = -(4 * mu + 2 * lam)
    f2 = -(-3 * mu + 2 * (lam + 2 * mu) + lam)
    terms = [(0, 1.0, 2, 0, 0), (0, 1.0, 1, 1, 0), (1, 1.0, 0, 2, 0), (1, -2.0, 2, 0, 0)]
    A = O.Matrix(FES.ndofs)
    A.add_bilinear(g.coords, g.cells, 2, 2, FES.celldofs, O.OP_SYMGRAD, False, 1.0, action=O.ACT_HOOKE2D, mu=mu,
                   lam=lam)
    b = np.zeros(FES.ndofs)
    O.assemble_linear(b, g.coords, g.cells, 2, 2, FES.celldofs, O.RHS_CONST, [f1, f2])
    fixed = FES.boundary_dofs()
    pts = _dof_points(G, FES)
    uex = _poly_eval(terms, 2, pts)
    uex = np.concatenate([uex[:, 0], uex[:, 1]])
    A.penalize(fixed)
    u = O.solve_direct(A.csr(), O.penalized_rhs(b, fixed, uex[fixed]))
    assert np.max(np.abs(u - uex)) < 1e-10


def test_oracle_cg_matches_direct(G, O):
    g = G.grid_unitcube_kuhn(3)
    FES = G.FESpace(G.H1P2(1, 3), g)
    rng = np.random.default_rng(1)
    kappa = np.exp(rng.standard_normal(g.ncells))
    A = O.Matrix(FES.ndofs)
    A.add_bilinear(g.coords, g.cells, 2, 1, FES.celldofs, O.OP_GRADIENT, True, 1.0, action=O.ACT_CELLSCALE,
                   cellcoef=kappa)
    b = np.zeros(FES.ndofs)
    O.assemble_linear(b, g.coords, g.cells, 2, 1, FES.celldofs, O.RHS_FOURIER, [1.0, 1, 2, 3, -0.5, 2, 2, 1])
    fixed = FES.boundary_dofs()
    A.penalize(fixed)
    bb = O.penalized_rhs(b, fixed)
    M = A.csr()
    u1 = O.solve_direct(M, bb)
    u2, it, rr = O.solve_cg(M, bb, 1e-14)
    assert rr < 1e-13
    assert np.linalg.norm(u1 - u2) / np.linalg.norm(u1) < 1e-10
