"""Bernardi-Raugel / P0 Stokes with the RT0 reconstruction (batched iterated penalty).

CPU: the oracle reproduces the reference's pressure-robustness known answer
(examples/Example222_PressureRobustness2D.jl:189-211, runtests.jl:684-723):
a pure gradient force gives a zero discrete velocity with the reconstructed
right-hand side.  GPU: pattern / matrix / rhs parity of the H1BR assembly,
solution parity of the batched solver against the oracle's iterated penalty
with sparse-direct solves, and bit-identical results alone and in a batch.
"""
import numpy as np
import pytest

from parity_helpers import stokes_tolerance


def _poly_terms(rng):
    from grmp_gb300 import stokes as S
    return S.grad_plus_curl_terms(S.cubic_coefficients(rng), S.cubic_coefficients(rng))


@pytest.mark.parametrize("recon", [1, 2])   # BR->RT0, BR->BDM1
def test_oracle_hydrostatic_velocity_is_zero(G, O, recon):
    """f = grad(phi), phi = x^3 + y^3 - xy: the gradient-robust scheme gives
    u_h = 0 and p_h = (cell means of phi) up to a constant
    (examples/Example222_PressureRobustness2D.jl:189-211)."""
    g = G.grid_unitsquare(6)
    phi = {(3, 0): 1.0, (0, 3): 1.0, (1, 1): -1.0}
    from grmp_gb300 import stokes as S
    terms = S.grad_plus_curl_terms(phi, {})
    for nu in (1.0, 1e-3):
        u, p, _ = O.stokes_iterated_penalty(g, nu, 1e4, terms, sweeps=10, recon=recon)
        assert np.max(np.abs(u)) < 1e-12, nu
        # cell means of phi (order-6 rule is exact for cubics)
        x, w, _ = O.qrule(2, 6)
        X = g.coords[g.cells]
        A = np.transpose(X[:, 1:, :] - X[:, :1, :], (0, 2, 1))
        pts = X[:, None, 0, :] + np.einsum("ckj,qj->cqk", A, x[:, :2])
        ph = pts[..., 0] ** 3 + pts[..., 1] ** 3 - pts[..., 0] * pts[..., 1]
        mean_phi = ph @ w
        target = mean_phi - np.dot(g.cell_volumes(), mean_phi) / g.cell_volumes().sum()
        assert np.max(np.abs(p - target)) < 1e-9 * np.max(np.abs(target)), nu


def br_linear_interpolant(g, field):
    """BR DoF vector of a linear vector field: vertex values per component
    (component-major), zero face bubbles (a linear field is its own P1 part)."""
    vals = field(g.coords)                      # (nverts, dim)
    nf = g.faces()[0].shape[0]
    return np.concatenate([vals.T.ravel(), np.zeros(nf)])


@pytest.mark.parametrize("recon,velocity", [(1, "const"), (2, "const"), (2, "linear")])
def test_oracle_p_robust_exact_velocity(G, O, recon, velocity):
    """The reference's p-robust Stokes test (test/runtests.jl:684-723,
    exact_functions_stokes2D): velocity (y^k + 1, x^k - 1) of order k = 0
    (BR + RT0, BR + BDM1) or 1 (BR + BDM1), pressure x^3 + y^3 - 1/2,
    f = grad p, boundary data the exact velocity.  The discrete velocity is
    exact (the reference checks its L2 error < 6e-12)."""
    g = G.grid_unitsquare(4)
    k = 0 if velocity == "const" else 1
    exact = lambda X: np.stack([X[:, 1] ** k + 1, X[:, 0] ** k - 1], axis=1)   # noqa: E731
    terms = np.array([(0, 3.0, 2, 0, 0), (1, 3.0, 0, 2, 0)])
    ub = br_linear_interpolant(g, exact)
    u, p, fixed = O.stokes_iterated_penalty(g, 1.0, 1e4, terms, sweeps=8, recon=recon, bonus_quadorder=2,
                                            u_boundary=ub)
    assert np.max(np.abs(u - ub)) < 1e-10


@pytest.mark.parametrize("recon", [1, 2])   # BR->RT0, BR->BDM1
def test_oracle_br_rhs_of_gradient_is_in_range_of_divergence(G, O, recon):
    """(grad phi, R v) = -(pi_0 phi, div v) for v vanishing on the boundary:
    the reconstructed load of a gradient is annihilated by div-free
    velocities -- the identity behind pressure robustness."""
    g = G.grid_unitsquare(4)
    from grmp_gb300 import stokes as S
    phi = {(2, 1): 1.0, (0, 2): -2.0}
    M, bf, fixed, cd, args = O.br_stokes_system(g, 1.0, 0.0, S.grad_plus_curl_terms(phi, {}), recon=recon)
    x, w, _ = O.qrule(2, 6)
    X = g.coords[g.cells]
    A = np.transpose(X[:, 1:, :] - X[:, :1, :], (0, 2, 1))
    pts = X[:, None, 0, :] + np.einsum("ckj,qj->cqk", A, x[:, :2])
    ph = pts[..., 0] ** 2 * pts[..., 1] - 2 * pts[..., 1] ** 2
    _, bp = O.br_div(g, args, p=ph @ w)
    free = np.setdiff1d(np.arange(bf.size), fixed)
    assert np.max(np.abs(bf[free] + bp[free])) < 1e-13 * max(1.0, np.max(np.abs(bf)))


def _small_batch(G, sizes, nus, seed=3):
    from grmp_gb300 import stokes as S
    return S.make_batch(sizes=np.array(sizes), nus=np.array(nus), seed=seed)


@pytest.mark.gpu
@pytest.mark.parametrize("recon", ["RT0", "BDM1"])
def test_br_assembly_parity(G, O, ctx, recon):
    from grmp_gb300 import stokes as S
    prob = _small_batch(G, [7], [0.3])
    sysd = S.StokesBatchSystem(ctx, prob, mixed=True, reconstruction=recon)
    g = prob.mesh.parts[0]
    M, bf, fixed, cd, args = O.br_stokes_system(g, prob.nus[0], prob.lam, prob.terms[0],
                                                recon=2 if recon == "BDM1" else 1)
    A0 = M.csr()
    rp, ci = sysd.A.pattern()
    assert np.array_equal(rp, A0.indptr) and np.array_equal(ci, A0.indices)
    api = __import__("grmp_gb300").api
    api.assemble(sysd.A, sysd.ops, G.FP64)
    Ag = sysd.A.download(G.FP64)
    o = A0.data
    rm = np.repeat(np.maximum.reduceat(np.abs(o), A0.indptr[:-1]), np.diff(A0.indptr))
    assert np.max(np.abs(Ag.data - o) / np.maximum(np.abs(o), 1e-3 * rm)) <= 1e-12
    sysd.assemble()
    b = sysd.bf.entries
    free = np.setdiff1d(np.arange(bf.size), fixed)
    assert np.max(np.abs(b[free] - bf[free])) <= 1e-12 * np.max(np.abs(bf))


@pytest.mark.gpu
@pytest.mark.parametrize("mode", ["fp64", "mixed", "direct"])
def test_batch_matches_oracle(G, O, ctx, mode):
    """Iterated-penalty result against the oracle's sparse-direct sweeps, per
    problem within max(1e-10, 10 cond eps) (stokes_tolerance: the condition
    number of each problem's velocity system is computed and stated).  The
    FP32 inner solve (mixed) only resolves moderate lambda/nu: with lambda =
    1e4 and nu = 0.05 its PCG needs ~1e5 iterations, so the mixed case uses
    nu >= 0.2."""
    from grmp_gb300 import stokes as S
    sizes, nus = [5, 9, 6], ([1.0, 0.2, 0.5] if mode == "mixed" else [1.0, 0.2, 0.05])
    prob = _small_batch(G, sizes, nus)
    sysd = S.StokesBatchSystem(ctx, prob, mixed=(mode == "mixed"), direct=(mode == "direct"))
    sysd.assemble()
    st = sysd.solve(sweeps=8, reltol=1e-12 if mode == "mixed" else 1e-13)
    u, p = sysd.velocity(), sysd.pressure()
    for k, g in enumerate(prob.mesh.parts):
        uo, po, _ = O.stokes_iterated_penalty(g, nus[k], prob.lam, prob.terms[k], sweeps=8)
        r0, r1 = prob.V.row_offsets[k], prob.V.row_offsets[k + 1]
        c0, c1 = prob.mesh.cell_offsets[k], prob.mesh.cell_offsets[k + 1]
        eu = np.linalg.norm(u[r0:r1] - uo) / np.linalg.norm(uo)
        ep = np.linalg.norm(p[c0:c1] - po) / np.linalg.norm(po)
        tol, cond = stokes_tolerance(O, g, nus[k], prob.lam, 1)
        assert eu <= tol and ep <= tol, (k, eu, ep, tol, cond, st)


@pytest.mark.gpu
def test_batch_mixed_direct_matches_oracle(G, O, ctx):
    """FP32 factor per problem preconditioning FP64 CG, with the FP64 factor
    as the fallback, against the oracle's sparse-direct sweeps over nu from 1
    down to 1e-4.  Problems whose CG reaches the tolerance meet the same
    bound as the FP64 direct mode; a problem solved to the FP64 floor of its
    conditioning (accepted, as in the FP64 mode, by a normwise backward error
    <= 1e-13) is held to the conditioning bound 10 cond eps itself (measured
    2.4e-8 at cond 2.1e9, within that bound of 4.6e-6)."""
    from grmp_gb300 import stokes as S
    sizes, nus = [5, 9, 6, 8], [1.0, 0.05, 1e-3, 1e-4]
    prob = _small_batch(G, sizes, nus, seed=7)
    sysd = S.StokesBatchSystem(ctx, prob, solver="mixed_direct")
    sysd.assemble()
    st = sysd.solve(sweeps=8, reltol=1e-13)
    assert 0 <= st["fp64_fallbacks"] <= len(sizes)
    u, p = sysd.velocity(), sysd.pressure()
    for k, g in enumerate(prob.mesh.parts):
        uo, po, _ = O.stokes_iterated_penalty(g, nus[k], prob.lam, prob.terms[k], sweeps=8)
        r0, r1 = prob.V.row_offsets[k], prob.V.row_offsets[k + 1]
        c0, c1 = prob.mesh.cell_offsets[k], prob.mesh.cell_offsets[k + 1]
        eu = np.linalg.norm(u[r0:r1] - uo) / np.linalg.norm(uo)
        ep = np.linalg.norm(p[c0:c1] - po) / np.linalg.norm(po)
        tol, cond = stokes_tolerance(O, g, nus[k], prob.lam, 1, cap=None if nus[k] < 1e-3 else 1e-8)
        assert eu <= tol and ep <= tol, (k, eu, ep, tol, cond, st)


@pytest.mark.gpu
def test_batch_bdm1_matches_oracle(G, O, ctx):
    """Direct batch with the BR -> BDM1 reconstructed right-hand side."""
    from grmp_gb300 import stokes as S
    sizes, nus = [6, 8], [1.0, 1e-3]
    prob = _small_batch(G, sizes, nus, seed=5)
    sysd = S.StokesBatchSystem(ctx, prob, direct=True, reconstruction="BDM1")
    sysd.assemble()
    st = sysd.solve(sweeps=8, reltol=1e-13)
    u, p = sysd.velocity(), sysd.pressure()
    for k, g in enumerate(prob.mesh.parts):
        uo, po, _ = O.stokes_iterated_penalty(g, nus[k], prob.lam, prob.terms[k], sweeps=8, recon=2)
        r0, r1 = prob.V.row_offsets[k], prob.V.row_offsets[k + 1]
        c0, c1 = prob.mesh.cell_offsets[k], prob.mesh.cell_offsets[k + 1]
        eu = np.linalg.norm(u[r0:r1] - uo) / np.linalg.norm(uo)
        ep = np.linalg.norm(p[c0:c1] - po) / np.linalg.norm(po)
        tol, cond = stokes_tolerance(O, g, nus[k], prob.lam, 2)
        assert eu <= tol and ep <= tol, (k, eu, ep, tol, cond, st)


@pytest.mark.gpu
@pytest.mark.parametrize("mode", ["mixed", "direct", "mixed_direct"])
def test_batch_result_same_alone_and_in_the_mix(G, ctx, mode):
    """Each problem is owned by one thread block: its bits do not depend on
    the other problems of the batch."""
    from grmp_gb300 import stokes as S
    sizes, nus = [6, 12, 4, 9], [1.0, 1e-2, 0.3, 1e-3]
    big = _small_batch(G, sizes, nus, seed=11)
    sb = S.StokesBatchSystem(ctx, big, solver=mode)
    sb.assemble()
    sb.solve(sweeps=5, reltol=1e-10)
    u, p = sb.velocity(), sb.pressure()
    k = 1
    alone = S.make_batch(sizes=np.array([sizes[k]]), nus=np.array([nus[k]]), seed=11)
    alone.terms = big.terms[k:k + 1].copy()
    sa = S.StokesBatchSystem(ctx, alone, solver=mode)
    sa.assemble()
    sa.solve(sweeps=5, reltol=1e-10)
    r0, r1 = big.V.row_offsets[k], big.V.row_offsets[k + 1]
    c0, c1 = big.mesh.cell_offsets[k], big.mesh.cell_offsets[k + 1]
    assert np.array_equal(sa.velocity(), u[r0:r1])
    assert np.array_equal(sa.pressure(), p[c0:c1])


@pytest.mark.parametrize("dim", [2, 3])
def test_oracle_divergence_coupling_recast(G, O, dim):
    """The reference's recast test (test/test_operators.jl:15-82) on the
    velocity-pressure coupling of the iterated penalty: on one cell, u = x
    (div u = dim) and p = 0.75 give (div u, p) = dim * 0.75 * |T| both as the
    cell mean of div u and as the assembled linear form (p, div v) applied to
    u (the matrix-vector consistency of the recast)."""
    from grmp_gb300 import mesh as M
    if dim == 2:
        g = M.SimplexMesh(np.array([[-1.0, 0.0], [1.0, 0.0], [0.0, 1.0]]), np.array([[0, 1, 2]], dtype=np.int32))
    else:
        g = M.SimplexMesh(np.array([[0.0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1]]),
                          np.array([[0, 1, 2, 3]], dtype=np.int32))
    _, _, _, cd, args = O.br_stokes_system(g, 1.0, 0.0, np.zeros((1, 5)), bonus_quadorder=0)
    nf = g.faces()[0].shape[0]
    u = np.concatenate([g.coords.T.ravel(), np.zeros(nf)])   # u = x: vertex values, no bubbles
    vol = g.cell_volumes()[0]
    divu, _ = O.br_div(g, args, u=u)
    assert abs(divu[0] * 0.75 * vol - dim * 0.75 * vol) < 1e-14
    _, bp = O.br_div(g, args, p=np.array([0.75]))
    assert abs(bp @ u - dim * 0.75 * vol) < 1e-14
    if dim == 2:
        assert abs(bp @ u - 1.5) < 1e-14      # the reference's expected value on its triangle
