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
