"""H1P2B{2,2} with the RT1 / BDM2 reconstruction test operators (2D).

CPU: the oracle's restatement of the reconstruction coefficients
(src/reconstructions.jl:43-330, :405-469) is pinned by the reference's own
p-robust catalogue entries (test/runtests.jl:684-723): [H1P2B{2,2}, broken
P1, HDIVRT1{2}] reproduces a linear velocity and [.., HDIVBDM2{2}] a
quadratic one with a cubic pressure, measured on the reconstructed velocity
as the reference does; the reconstruction of a P2 interpolant is exact for
fields in the target space, and RT1 is not exact for a quadratic velocity
(the catalogue's expected order 1).  GPU: the reconstructed right-hand side
against the oracle, per entry, on structured and shuffled meshes.
"""
import numpy as np
import pytest


def _exact(k):
    return lambda X: np.stack([X[:, 1] ** k + 1, X[:, 0] ** k - 1], axis=1)   # noqa: E731


def _velocity_terms(k):
    return np.array([(0, 1.0, 0, k, 0), (0, 1.0, 0, 0, 0), (1, 1.0, k, 0, 0), (1, -1.0, 0, 0, 0)])


def _force_terms(k):
    """f = -Laplace u + grad p, p = x^3 + y^3 - 1/2 (exact_functions_stokes2D)."""
    t = [(0, 3.0, 2, 0, 0), (1, 3.0, 0, 2, 0)]
    if k >= 2:
        t += [(0, -k * (k - 1.0), 0, k - 2, 0), (1, -k * (k - 1.0), k - 2, 0, 0)]
    return np.array(t)


@pytest.mark.parametrize("recon,k", [(3, 0), (3, 1), (4, 1), (4, 2)])
def test_oracle_p2b_p_robust_exact_velocity(G, O, recon, k):
    g = G.grid_unitsquare(4)
    ub = O.p2b_interpolant(g, _exact(k))
    u, p = O.p2b_stokes(g, 1.0, _force_terms(k), recon, ub, bonus_quadorder=2)
    err = O.p2b_recon_l2error(g, u, _velocity_terms(k), recon, order=6)
    assert err < 1e-12, err


def test_oracle_p2b_rt1_not_exact_for_quadratic_velocity(G, O):
    g = G.grid_unitsquare(4)
    ub = O.p2b_interpolant(g, _exact(2))
    u, p = O.p2b_stokes(g, 1.0, _force_terms(2), 3, ub, bonus_quadorder=2)
    assert O.p2b_recon_l2error(g, u, _velocity_terms(2), 3, order=6) > 1e-6


@pytest.mark.parametrize("recon,k", [(3, 1), (4, 2)])
def test_oracle_p2b_reconstruction_reproduces_target_fields(G, O, recon, k):
    """R of the P2 interpolant of a field in the target space is the field."""
    g = G.grid_unitsquare(5)
    ub = O.p2b_interpolant(g, _exact(k))
    assert O.p2b_recon_l2error(g, ub, _velocity_terms(k), recon, order=6) < 1e-13


@pytest.mark.parametrize("recon", [3, 4])
def test_oracle_p2b_reconstruction_keeps_cell_means(G, O, recon):
    """int_T R v = int_T v for every P2B function v (node functions 0, face
    functions |T|/3, the bubble |T|): the interior coefficients restore the
    cell integrals (for BDM2 as two of its three moment conditions)."""
    g = G.grid_unitsquare(3)
    C = O.p2b_coefficients(g, recon)
    x, w, _ = O.qrule(2, 4)
    vol = g.cell_volumes()
    fn, cf = g.faces()
    nrm, fv, sg = g.face_geometry()
    for cell in range(g.ncells):
        X = g.coords[g.cells[cell]]
        A = (X[1:] - X[0]).T
        det = np.linalg.det(A)
        s = sg[cell].astype(float)
        nr = 12 if recon == 4 else 8
        coef = np.ones(nr)
        if recon == 4:
            coef[0:9:3] = s
            coef[2:9:3] = s
        else:
            coef[0:6:2] = s
        ints = np.zeros((nr, 2))
        for q in range(len(w)):
            xi, eta = x[q, 0], x[q, 1]
            basis = _ref_basis(recon, xi, eta)
            ints += w[q] * vol[cell] * (basis @ A.T) * (coef / det)[:, None]
        got = C[cell, :, :nr] @ ints                   # (14, 2)
        want = np.zeros((14, 2))
        for c in range(2):
            want[7 * c + 3: 7 * c + 6, c] = vol[cell] / 3
            want[7 * c + 6, c] = vol[cell]
        assert np.max(np.abs(got - want)) < 1e-14 * max(1.0, vol[cell] * 100), (cell, got - want)


def _ref_basis(recon, x, y):
    if recon == 3:
        o = np.zeros((8, 2))
        o[0] = (x, y - 1)
        o[2] = (x, y)
        o[4] = (x - 1, y)
        o[1] = -12 * (0.5 - x - y) * o[0]
        o[3] = -(12 * (x - 0.5)) * o[2]
        o[5] = -(12 * (y - 0.5)) * o[4]
        o[6] = 12 * y * o[0]
        o[7] = 12 * x * o[4]
        return o
    lam = 1 - x - y
    o = np.zeros((12, 2))
    o[0] = (x, y - 1)
    o[3] = (x, y)
    o[6] = (x - 1, y)
    o[1] = (6 * x, 6 - 12 * x - 6 * y)
    o[4] = (-6 * x, 6 * y)
    o[7] = (6 * (x - 1) + 12 * y, -6 * y)
    o[2] = -15 * ((lam - 0.5) * o[1] + o[0])
    o[5] = -15 * ((x - 0.5) * o[4] + o[3])
    o[8] = -15 * ((y - 0.5) * o[7] + o[6])
    o[9] = y * o[1]
    o[10] = lam * o[4]
    o[11] = x * o[7]
    return o


def test_host_p2b_dofmap_matches_oracle(G, O):
    g = G.grid_unitsquare(4)
    S = G.FESpace(G.H1P2B(2, 2), g)
    cd, nd = O.p2b_celldofs(g)
    assert S.ndofs == nd and np.array_equal(S.celldofs, cd)


@pytest.mark.gpu
@pytest.mark.parametrize("recon", [3, 4])
@pytest.mark.parametrize("grid", ["square8", "square6_shuffled"])
def test_p2b_rhs_matches_oracle(G, O, ctx, recon, grid):
    """(f, R v) on the device against the oracle, per entry to 1e-12 of the
    vector's largest entry, for a cubic-plus-quadratic force."""
    from grmp_gb300 import api
    g = G.grid_unitsquare(8) if grid == "square8" else _shuffled(G, 6)
    S = G.FESpace(G.H1P2B(2, 2), g)
    terms = np.array([(0, 3.0, 2, 0, 0), (1, 3.0, 0, 2, 0), (0, -2.0, 0, 0, 0), (1, 1.5, 1, 1, 0),
                      (0, 0.7, 3, 0, 0)])
    op = api.ReconstructionIdentityRT1 if recon == 3 else api.ReconstructionIdentityBDM2
    lf = G.LinearForm(op, G.DataFunction.polynomial(terms, 2, bonus_quadorder=2))
    b = G.FEVector(ctx, S)
    b.fill(0.0)
    G.assemble(b, lf)
    bo = O.p2b_rhs(g, terms, recon, bonus_quadorder=2)
    assert np.max(np.abs(b.entries - bo)) <= 1e-12 * np.max(np.abs(bo))


@pytest.mark.gpu
def test_p2b_refusals(G, ctx):
    from grmp_gb300 import api
    g = G.grid_unitsquare(3)
    S = G.FESpace(G.H1P2B(2, 2), g)
    b = G.FEVector(ctx, S)
    lf = G.LinearForm(api.ReconstructionIdentity, G.DataFunction.polynomial(np.array([(0, 1.0, 0, 0, 0)]), 2))
    with pytest.raises(G.GrmpError):
        G.assemble(b, lf)                              # RT0 is the BR target, not P2B's
    with pytest.raises(G.GrmpError):
        G.FEMatrix(ctx, S, [G.LaplaceOperator(1.0)])   # bilinear forms on H1P2B are not built


def _shuffled(G, n):
    """The unit square mesh with cells listed in a random order and each
    cell's vertices rotated (orientation kept)."""
    g = G.grid_unitsquare(n)
    rng = np.random.default_rng(4)
    cells = g.cells[rng.permutation(g.ncells)]
    rot = rng.integers(0, 3, size=cells.shape[0])
    cells = np.stack([np.roll(c, r) for c, r in zip(cells, rot)])
    return G.SimplexMesh(g.coords, cells)
