"""Shared test helper: the oracle's system (matrix, right-hand side,
penalised form) for a problem given as FE space + operators + rhs + fixed
DoFs (problems.LinearProblem, serve.ServeRequest)."""
import numpy as np


def oracle_system(G, O, prob, penalty=True):
    """Oracle matrix (penalised) and rhs for a problems.LinearProblem."""
    FES = prob.FES
    g = FES.xgrid
    fe = 1 if FES.FEType.kind == G.FE_H1P1 else 2
    nc = FES.FEType.ncomponents
    M = O.Matrix(FES.ndofs)
    for op in prob.operators:
        if op.op_kind == 1:
            act = O.ACT_CELLSCALE if op.cell_coef is not None else O.ACT_NONE
            M.add_bilinear(g.coords, g.cells, fe, nc, FES.celldofs, O.OP_GRADIENT, op.symmetric, op.factor, act,
                           op.cell_coef, bonus_quadorder=op.bonus_quadorder)
        elif op.op_kind == 2:
            act = O.ACT_CELLSCALE if op.cell_coef is not None else O.ACT_NONE
            M.add_bilinear(g.coords, g.cells, fe, nc, FES.celldofs, O.OP_IDENTITY, op.symmetric, op.factor, act,
                           op.cell_coef, bonus_quadorder=op.bonus_quadorder)
        elif op.op_kind == 3:
            act = O.ACT_HOOKE2D if g.dim == 2 else O.ACT_HOOKE3D
            M.add_bilinear(g.coords, g.cells, fe, nc, FES.celldofs, O.OP_SYMGRAD, op.symmetric, op.factor, act,
                           mu=op.params[0], lam=op.params[1])
    A0 = M.csr()
    b = np.zeros(FES.ndofs)
    f = prob.rhs.f
    O.assemble_linear(b, g.coords, g.cells, fe, nc, FES.celldofs, f.kind, f.params, prob.rhs.factor,
                      f.bonus_quadorder)
    if penalty:
        M.penalize(prob.fixed)
    return A0, M.csr(), b, O.penalized_rhs(b, prob.fixed)


def stokes_tolerance(O, g, nu, lam, recon=1, cap=1e-8):
    """Relative-error bound for one problem of a batched iterated-penalty
    result against the oracle's sparse-direct sweeps: 1e-10, or 10 * cond *
    eps where the velocity matrix's condition number makes that larger, but
    never looser than 1e-8 (met in practice even at cond ~ 2e8).  The
    penalty lam makes the velocity system ill-conditioned (cond ~ lam / nu /
    h^2: its smallest eigenvalues belong to divergence-free fields, scaled by
    nu, its largest to the penalty); both solutions carry rounding errors of
    cond * eps, so no tighter agreement is meaningful.  cond is computed here
    (2-norm, dense, free DoFs) and returned with the bound; cap=None gives
    the plain conditioning bound."""
    import numpy as np
    M, _, fixed, _, _ = O.br_stokes_system(g, nu, lam, np.zeros((1, 5)), recon=recon)
    A = M.csr().toarray()
    free = np.setdiff1d(np.arange(A.shape[0]), fixed)
    cond = float(np.linalg.cond(A[np.ix_(free, free)]))
    b = 10.0 * cond * np.finfo(float).eps
    return max(1e-10, b if cap is None else min(cap, b)), cond
