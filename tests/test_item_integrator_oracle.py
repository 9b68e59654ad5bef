"""The oracle's ItemIntegrator (L2ErrorIntegrator / L2NormIntegrator /
L2DifferenceIntegrator of src/assemblypatterns/itemintegrator.jl) pinned
against the reference's own exactness tests (test/runtests.jl:170-330:
interpolating exact_function{2,3}D(order) into an element of that order gives
L2 and H1 errors at rounding level) and against closed-form integrals."""
import numpy as np
import pytest

from item_helpers import exact_eval, exact_gradient_terms, exact_terms

RHS_POLY = 3
OP_IDENTITY, OP_GRADIENT = 0, 1


def _space(G, dim, n, fe, ncomp):
    from grmp_gb300 import fespace as F
    g = G.grid_unitsquare(n) if dim == 2 else G.grid_unitcube_kuhn(n)
    ft = F.H1P1(ncomp) if fe == 1 else F.H1P2(ncomp, dim)
    return g, F.FESpace(ft, g)


@pytest.mark.parametrize("dim,fe,order", [(2, 1, 1), (2, 2, 1), (2, 2, 2), (3, 1, 1), (3, 2, 2)])
def test_interpolation_exact_errors(G, O, dim, fe, order):
    g, FES = _space(G, dim, 4 if dim == 2 else 2, fe, dim)
    u = G.interpolate(FES, lambda x: exact_eval(dim, order, x))
    _, l2 = O.item_l2error(g.coords, g.cells, fe, dim, FES.celldofs, u, OP_IDENTITY, RHS_POLY,
                           exact_terms(dim, order), quadorder=order)
    _, h1 = O.item_l2error(g.coords, g.cells, fe, dim, FES.celldofs, u, OP_GRADIENT, RHS_POLY,
                           exact_gradient_terms(dim, order), quadorder=max(0, order - 1))
    assert np.sqrt(l2) < 1e-13, l2
    assert np.sqrt(h1) < 1e-12, h1


def test_interpolation_error_of_a_cubic_is_not_zero(G, O):
    g, FES = _space(G, 2, 4, 2, 2)
    u = G.interpolate(FES, lambda x: exact_eval(2, 3, x))
    _, l2 = O.item_l2error(g.coords, g.cells, 2, 2, FES.celldofs, u, OP_IDENTITY, RHS_POLY, exact_terms(2, 3),
                           quadorder=3)
    assert np.sqrt(l2) > 1e-4


def test_closed_form_norms(G, O):
    # u = x on the unit square: int u^2 = 1/3, int |grad u|^2 = 1; u - v with v = 0 gives the same
    g, FES = _space(G, 2, 5, 1, 1)
    u = G.interpolate(FES, lambda x: x[:, 0])
    cellv, tot = O.item_l2error(g.coords, g.cells, 1, 1, FES.celldofs, u, OP_IDENTITY, quadorder=2)
    assert abs(tot - 1.0 / 3.0) < 1e-14
    assert abs(cellv.sum() - tot) < 1e-14
    _, tg = O.item_l2error(g.coords, g.cells, 1, 1, FES.celldofs, u, OP_GRADIENT, quadorder=2)
    assert abs(tg - 1.0) < 1e-14
    _, td = O.item_l2error(g.coords, g.cells, 1, 1, FES.celldofs, u, OP_IDENTITY, quadorder=2,
                           v=np.zeros_like(u))
    assert td == tot
    # factor: (f - factor*u) with f = 0 and factor 2 gives 4/3
    _, t2 = O.item_l2error(g.coords, g.cells, 1, 1, FES.celldofs, u, OP_IDENTITY, RHS_POLY,
                           np.array([[0, 0.0, 0, 0, 0]]), factor=2.0, quadorder=2)
    assert abs(t2 - 4.0 / 3.0) < 1e-14


def _br_linear(G, dim, seed=0):
    """A linear vector field on a BR space: vertex values, zero bubbles, with
    its polynomial records and those of its (constant) gradient."""
    from grmp_gb300 import fespace as F
    g = G.grid_unitsquare(4) if dim == 2 else G.grid_unitcube_kuhn(2)
    S = F.FESpace(F.H1BR(dim), g)
    rng = np.random.default_rng(seed)
    M, c0 = rng.standard_normal((dim, dim)), rng.standard_normal(dim)
    vals = g.coords @ M.T + c0
    u = np.concatenate([vals.T.ravel(), np.zeros(g.faces()[0].shape[0])])
    terms = []
    for c in range(dim):
        terms.append((c, c0[c], 0, 0, 0))
        for j in range(dim):
            e = [0, 0, 0]
            e[j] = 1
            terms.append((c, M[c, j], *e))
    gterms = [(c * dim + j, M[c, j], 0, 0, 0) for c in range(dim) for j in range(dim)]
    return g, S, u, np.array(terms), np.array(gterms)


@pytest.mark.parametrize("dim", [2, 3])
def test_br_linear_fields_are_exact(G, O, dim):
    """H1BR{d} holds the linear vector fields (its P1 part): L2 and H1 errors
    of such a field against its own formula vanish -- the reference's
    interpolation test for H1BR{2} / H1BR{3} with expected order 1
    (test/runtests.jl:186-223, 224-260: for a linear function the
    interpolant is its vertex values with zero bubble coefficients)."""
    g, S, u, terms, gterms = _br_linear(G, dim)
    _, l2 = O.item_l2error_br(g, S.celldofs, u, OP_IDENTITY, RHS_POLY, terms, quadorder=2)
    _, h1 = O.item_l2error_br(g, S.celldofs, u, OP_GRADIENT, RHS_POLY, gterms, quadorder=0)
    assert np.sqrt(l2) < 1e-14 and np.sqrt(h1) < 1e-13


@pytest.mark.parametrize("dim", [2, 3])
def test_br_bubble_norm_closed_form(G, O, dim):
    """One face bubble with coefficient 1: ||phi_F||^2 = c (|T1| + |T2|) with
    c = 36 * 2 * 2!2!/6! = 2/5 in 2D (6 l_a l_b, src/fedefs/h1v_br.jl:117-130)
    and 3600 * 6 * 2!2!2!/9! = 10/21 in 3D (60 l_a l_b l_c, :221-233); the
    unit normal does not change the norm."""
    from grmp_gb300 import fespace as F
    g = G.grid_unitsquare(3) if dim == 2 else G.grid_unitcube_kuhn(2)
    S = F.FESpace(F.H1BR(dim), g)
    fn, cf = g.faces()
    cnt = np.bincount(cf.ravel(), minlength=fn.shape[0])
    face = int(np.nonzero(cnt == 2)[0][0])
    u = np.zeros(S.ndofs)
    u[dim * g.nverts + face] = 1.0
    cells = np.nonzero((cf == face).any(axis=1))[0]
    c = 2.0 / 5.0 if dim == 2 else 10.0 / 21.0
    _, n2 = O.item_l2error_br(g, S.celldofs, u, OP_IDENTITY, quadorder=2 if dim == 2 else 3)
    assert abs(n2 - c * g.cell_volumes()[cells].sum()) < 1e-15
