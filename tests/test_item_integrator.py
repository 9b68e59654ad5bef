"""Device ItemIntegrator (grmp_item_l2error) against the oracle.

* the reference's exactness pins (test/runtests.jl:170-330): interpolants of
  exact_function{2,3}D(order) have L2 and H1 errors at rounding level;
* parity with the oracle on random discrete functions: per-cell values within
  1e-12 of the largest cell value, totals within 1e-13 relative (the device
  sums cells in a fixed tree order, the reference in one running sum);
* L2NormIntegrator and L2DifferenceIntegrator; repeat runs bit-identical;
* unsupported elements and mismatched data are refused.
"""
import numpy as np
import pytest

from item_helpers import exact_eval, exact_gradient_terms, exact_terms

pytestmark = pytest.mark.gpu

RHS_POLY, RHS_FOURIER = 3, 2


def _space(G, dim, n, fe, ncomp):
    from grmp_gb300 import fespace as F
    g = G.grid_unitsquare(n) if dim == 2 else G.grid_unitcube_kuhn(n)
    ft = F.H1P1(ncomp) if fe == 1 else F.H1P2(ncomp, dim)
    return g, F.FESpace(ft, g)


def _vec(G, ctx, FES, values):
    v = G.FEVector(ctx, FES)
    v.upload(values)
    return v


@pytest.mark.parametrize("dim,fe,order", [(2, 1, 1), (2, 2, 2), (3, 1, 1), (3, 2, 2)])
def test_interpolation_exact_errors(G, ctx, dim, fe, order):
    g, FES = _space(G, dim, 6 if dim == 2 else 3, fe, dim)
    u = _vec(G, ctx, FES, G.interpolate(FES, lambda x: exact_eval(dim, order, x)))
    l2 = G.L2ErrorIntegrator(G.DataFunction.polynomial(exact_terms(dim, order), dim), G.Identity,
                             quadorder=order).evaluate(u)
    h1 = G.L2ErrorIntegrator(G.DataFunction.polynomial(exact_gradient_terms(dim, order), dim * dim), G.Gradient,
                             quadorder=max(0, order - 1)).evaluate(u)
    assert np.sqrt(l2) < 1e-13, l2
    assert np.sqrt(h1) < 1e-12, h1


CASES = [
    # dim, fe, ncomp, op, data kind
    (2, 2, 1, "Identity", "fourier"),
    (2, 2, 1, "Gradient", "poly"),
    (2, 1, 2, "Identity", "poly"),
    (3, 2, 1, "Identity", "fourier"),
    (3, 2, 3, "Gradient", "poly"),
    (3, 1, 1, "Gradient", None),
]


@pytest.mark.parametrize("case", CASES)
def test_parity_with_oracle(G, O, ctx, case):
    dim, fe, nc, opname, kind = case
    g, FES = _space(G, dim, 8 if dim == 2 else 4, fe, nc)
    rng = np.random.default_rng(11)
    uvals = rng.standard_normal(FES.ndofs)
    u = _vec(G, ctx, FES, uvals)
    op = G.Identity if opname == "Identity" else G.Gradient
    rdim = nc * (dim if opname == "Gradient" else 1)
    if kind == "fourier":
        amps = rng.standard_normal(4)
        ks = rng.integers(1, 4, size=(4, dim)).astype(float)
        data = G.DataFunction.fourier(amps, ks, bonus_quadorder=1)
    elif kind == "poly":
        terms = [(c, rng.standard_normal(), *rng.integers(0, 3, size=3)) for c in range(rdim) for _ in range(2)]
        data = G.DataFunction.polynomial(terms, rdim, bonus_quadorder=1)
    else:
        data = None
    if data is not None:
        integ = G.L2ErrorIntegrator(data, op, factor=0.75)
    else:
        integ = G.L2NormIntegrator(op, quadorder=2)
    cells = integ.evaluate_cells(u)
    tot = integ.evaluate(u)
    order_bonus = 2 * data.bonus_quadorder if data is not None else 2
    oc, ot = O.item_l2error(g.coords, g.cells, fe, nc, FES.celldofs, uvals, 0 if opname == "Identity" else 1,
                            data.kind if data is not None else -1, data.params if data is not None else None,
                            factor=0.75 if data is not None else 1.0, quadorder=order_bonus)
    assert np.max(np.abs(cells - oc)) <= 1e-12 * np.max(np.abs(oc))
    assert abs(tot - ot) <= 1e-13 * abs(ot)
    assert abs(cells.sum() - tot) <= 1e-13 * abs(ot)
    assert integ.evaluate(u) == tot   # bit-identical repeat


def test_difference_integrator(G, O, ctx):
    g, FES = _space(G, 3, 3, 2, 1)
    rng = np.random.default_rng(5)
    a, b = rng.standard_normal(FES.ndofs), rng.standard_normal(FES.ndofs)
    ua, ub = _vec(G, ctx, FES, a), _vec(G, ctx, FES, b)
    for opname, op in (("Identity", 0), ("Gradient", 1)):
        integ = G.L2DifferenceIntegrator(getattr(G, opname))
        t = integ.evaluate(ua, ub)
        _, ot = O.item_l2error(g.coords, g.cells, 2, 1, FES.celldofs, a, op, quadorder=2, v=b)
        assert abs(t - ot) <= 1e-13 * abs(ot)
        # ||a - b|| equals the norm of the difference vector
        ud = _vec(G, ctx, FES, a - b)
        tn = G.L2NormIntegrator(getattr(G, opname)).evaluate(ud)
        assert abs(t - tn) <= 1e-12 * abs(tn)


@pytest.mark.parametrize("dim,opname,kind", [(2, "Identity", "poly"), (2, "Gradient", None), (3, "Identity", None),
                                             (3, "Gradient", "poly"), (2, "Gradient", "poly")])
def test_br_parity_with_oracle(G, O, ctx, dim, opname, kind):
    """Bernardi-Raugel functions (vertex parts and face bubbles times the face
    normals) through the device integrator against the oracle."""
    from grmp_gb300 import fespace as F
    g = G.grid_unitsquare(6) if dim == 2 else G.grid_unitcube_kuhn(3)
    FES = F.FESpace(F.H1BR(dim), g)
    rng = np.random.default_rng(21 + dim)
    uvals = rng.standard_normal(FES.ndofs)
    u = _vec(G, ctx, FES, uvals)
    op = G.Identity if opname == "Identity" else G.Gradient
    rdim = dim * (dim if opname == "Gradient" else 1)
    if kind == "poly":
        terms = [(c, rng.standard_normal(), *rng.integers(0, 3, size=3)) for c in range(rdim) for _ in range(2)]
        data = G.DataFunction.polynomial(terms, rdim, bonus_quadorder=1)
        integ = G.L2ErrorIntegrator(data, op, factor=0.5)
        oc, ot = O.item_l2error_br(g, FES.celldofs, uvals, 0 if opname == "Identity" else 1, data.kind, data.params,
                                   factor=0.5, quadorder=2 * data.bonus_quadorder)
    else:
        integ = G.L2NormIntegrator(op, quadorder=2)
        oc, ot = O.item_l2error_br(g, FES.celldofs, uvals, 0 if opname == "Identity" else 1, quadorder=2)
    cells = integ.evaluate_cells(u)
    tot = integ.evaluate(u)
    assert np.max(np.abs(cells - oc)) <= 1e-12 * np.max(np.abs(oc))
    assert abs(tot - ot) <= 1e-13 * abs(ot)
    # difference of two BR functions equals the norm of their difference
    w = rng.standard_normal(FES.ndofs)
    td = G.L2DifferenceIntegrator(op).evaluate(u, _vec(G, ctx, FES, w))
    tn = G.L2NormIntegrator(op).evaluate(_vec(G, ctx, FES, uvals - w))
    assert abs(td - tn) <= 1e-12 * abs(tn)


def test_refusals(G, ctx):
    from grmp_gb300 import fespace as F
    from grmp_gb300 import _lib as L
    g = G.grid_unitsquare(4)
    FES = F.FESpace(F.L2P0(1), g)
    u = _vec(G, ctx, FES, np.zeros(FES.ndofs))
    with pytest.raises(G.GrmpError) as ei:
        G.L2NormIntegrator(G.Identity).evaluate(u)
    assert ei.value.code == L.ERR_UNSUPPORTED
    _, FES2 = _space(G, 2, 4, 2, 1)
    u2 = _vec(G, ctx, FES2, np.zeros(FES2.ndofs))
    bad = G.DataFunction.constant([1.0, 2.0])   # two components for a scalar Identity
    with pytest.raises(G.GrmpError) as ei:
        G.L2ErrorIntegrator(bad, G.Identity).evaluate(u2)
    assert ei.value.code == L.ERR_INVALID_ARG
