"""Interior-face terms with Jump(Gradient) (update_dii4op!,
src/assemblypatterns.jl:103-153): the gradient-jump stabilisation
BilinearForm([Jump(Gradient), Jump(Gradient)], |F|^p action; AT = ON_IFACES)
of examples/Example203_ReactionConvectionDiffusion2D.jl:89-92 and the jump
ItemIntegrator of examples/Example210_PoissonLshapeAdaptive2D.jl:58-75.

CPU: the oracle's face terms vanish on globally smooth fields (linear for P1,
quadratic for P2: no gradient jumps), are symmetric positive semidefinite,
and give the hand-computed values on two triangles.  GPU: the device face
matrix, the per-face jump integrals and a stabilised solve against the oracle.
"""
import numpy as np
import pytest


def _space(G, dim, order, n):
    from grmp_gb300 import fespace as F
    g = G.grid_unitsquare(n) if dim == 2 else G.grid_unitcube_kuhn(n)
    return g, F.FESpace(F.H1P1(1) if order == 1 else F.H1P2(1, dim), g)


def _oracle_face_matrix(O, g, S, order, factor=1.0, power=2.0, bonus=0, laplace=0.0):
    M = O.Matrix(S.ndofs)
    if laplace:
        M.add_bilinear(g.coords, g.cells, order, 1, S.celldofs, O.OP_GRADIENT, True, laplace)
    O.face_jumpgrad(M, g, order, S.celldofs, factor, power, bonus)
    return M.csr()


def _poly(S, order, rng):
    """DoF vector of a random global polynomial of the element's degree."""
    from grmp_gb300 import fespace as F
    d = S.xgrid.dim
    c = rng.standard_normal(10)

    def f(X):
        x, y = X[:, 0], X[:, 1]
        z = X[:, 2] if d == 3 else 0 * x
        v = c[0] + c[1] * x + c[2] * y + c[3] * z
        if order == 2:
            v = v + c[4] * x * x + c[5] * x * y + c[6] * y * y + c[7] * z * z + c[8] * x * z + c[9] * y * z
        return v
    return F.interpolate(S, f)


@pytest.mark.parametrize("dim,order", [(2, 1), (2, 2), (3, 1), (3, 2)])
def test_oracle_face_matrix_vanishes_on_smooth_fields(G, O, dim, order):
    g, S = _space(G, dim, order, 4 if dim == 2 else 2)
    A = _oracle_face_matrix(O, g, S, order)
    u = _poly(S, order, np.random.default_rng(1))
    Ad = A.toarray()
    assert np.max(np.abs(Ad - Ad.T)) <= 1e-14 * np.max(np.abs(Ad))
    assert np.linalg.eigvalsh(Ad).min() >= -1e-12 * np.max(np.abs(Ad))
    assert np.max(np.abs(A @ u)) <= 1e-12 * np.max(np.abs(Ad)) * np.max(np.abs(u))
    jumps = O.face_jumps(g, order, S.celldofs, u, kind=0)
    assert np.max(np.abs(jumps)) <= 1e-24


def _two_triangles(G):
    coords = np.array([[0.0, 0.0], [1.0, 0.0], [1.0, 1.0], [0.0, 1.0]])
    cells = np.array([[0, 1, 2], [0, 2, 3]])
    return G.SimplexMesh(coords, cells)


def test_oracle_face_terms_on_two_triangles(G, O):
    """u = hat function of vertex (0, 1): zero on the lower triangle, y - x on
    the upper one; across the diagonal [grad u] = (1, -1), |F| = sqrt 2,
    ([grad u].n)^2 = |[grad u]|^2 = 2: the estimator is |F| |F| 2 = 4 and the
    face matrix entry of that vertex is |F| |F|^2 2 = 4 sqrt 2."""
    from grmp_gb300 import fespace as F
    g = _two_triangles(G)
    S = F.FESpace(F.H1P1(1), g)
    u = np.array([0.0, 0.0, 0.0, 1.0])
    eta = O.face_jumps(g, 1, S.celldofs, u, kind=1, power=1.0)
    assert abs(eta.sum() - 4.0) <= 1e-14
    A = _oracle_face_matrix(O, g, S, 1).toarray()
    assert abs(A[3, 3] - 4 * np.sqrt(2)) <= 1e-13


@pytest.mark.gpu
@pytest.mark.parametrize("dim,order", [(2, 1), (2, 2), (3, 1), (3, 2)])
def test_face_matrix_matches_oracle(G, O, ctx, dim, order):
    g, S = _space(G, dim, order, 6 if dim == 2 else 3)
    ops = [G.LaplaceOperator(1.0),
           G.BilinearForm([G.Jump(G.Gradient), G.Jump(G.Gradient)], G.FaceVolumePower(2.0), AT=G.ON_IFACES,
                          factor=0.3)]
    A = G.FEMatrix(ctx, S, ops)
    G.assemble(A, ops, G.FP64)
    Ad = A.download(G.FP64)
    Ao = _oracle_face_matrix(O, g, S, order, factor=0.3, power=2.0, laplace=1.0)
    scale = np.max(np.abs(Ao.data))
    assert np.max(np.abs((Ad - Ao).toarray())) <= 1e-12 * scale
    # the pattern holds the oracle's nonzeros
    Ao.data[:] = 1.0
    Ad.data[:] = 1.0
    assert (Ao - Ao.multiply(Ad)).nnz == 0


@pytest.mark.gpu
@pytest.mark.parametrize("dim,order", [(2, 1), (2, 2), (3, 2)])
def test_face_jump_integrator_matches_oracle(G, O, ctx, dim, order):
    g, S = _space(G, dim, order, 7 if dim == 2 else 3)
    rng = np.random.default_rng(2)
    uh = rng.standard_normal(S.ndofs)
    u = G.FEVector(ctx, S)
    u.upload(uh)
    for normal in (True, False):
        ig = G.FaceJumpIntegrator(normal=normal, power=1.0, factor=1.0, bonus_quadorder=order - 1)
        dev = ig.evaluate_faces(u)
        ref = O.face_jumps(g, order, S.celldofs, uh, kind=1 if normal else 0, power=1.0, bonus_quadorder=order - 1)
        assert np.max(np.abs(dev - ref)) <= 1e-12 * np.max(np.abs(ref))
        assert abs(ig.last_total - ref.sum()) <= 1e-12 * ref.sum()


@pytest.mark.gpu
def test_face_jumps_two_triangles(G, ctx):
    from grmp_gb300 import fespace as F
    g = _two_triangles(G)
    S = F.FESpace(F.H1P1(1), g)
    u = G.FEVector(ctx, S)
    u.upload(np.array([0.0, 0.0, 0.0, 1.0]))
    assert abs(G.FaceJumpIntegrator(normal=True, power=1.0).evaluate(u) - 4.0) <= 1e-13


@pytest.mark.gpu
def test_stabilised_solve_matches_oracle(G, O, ctx):
    """-Laplace u = 1 with the gradient-jump term (tau = 0.1, |F|^2), zero
    boundary values, P2 on a 12 x 12 mesh: the device FP64 PCG solution against
    the oracle's sparse-direct solution."""
    g, S = _space(G, 2, 2, 12)
    ops = [G.LaplaceOperator(1.0),
           G.BilinearForm([G.Jump(G.Gradient), G.Jump(G.Gradient)], G.FaceVolumePower(2.0), AT=G.ON_IFACES,
                          factor=0.1)]
    A = G.FEMatrix(ctx, S, ops)
    G.assemble(A, ops, G.FP64)
    b = G.FEVector(ctx, S)
    b.fill(0.0)
    G.assemble(b, G.LinearForm(G.Identity, G.DataFunction.constant([1.0])))
    bh = b.entries.copy()
    fixed = S.boundary_dofs()
    G.apply_dirichlet(A, b, fixed, None, G.DIRICHLET_ELIMINATE)
    x = G.FEVector(ctx, S)
    G.GB300PCG(mode="fp64", reltol=1e-14, abstol=0.0).solve(A, b, x)
    Ao = _oracle_face_matrix(O, g, S, 2, factor=0.1, power=2.0, laplace=1.0).tolil()
    for d in fixed:
        Ao.rows[d] = [d]
        Ao.data[d] = [1e60]
    bo = bh.copy()
    bo[fixed] = 0.0
    uo = O.solve_direct(Ao.tocsr(), bo)
    assert np.linalg.norm(x.entries - uo) <= 1e-10 * np.linalg.norm(uo)
