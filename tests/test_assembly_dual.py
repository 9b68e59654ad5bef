"""One-pass assembly of both precisions (GRMP_FP64_FP32): the FP64 and the
FP32 values equal, bit for bit, those of separate FP64 and FP32 assemblies
(each precision is computed in its own arithmetic from its own factors), for
scalar and vector elements, per-cell coefficients, mass terms and Hooke."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _problems(G):
    from grmp_gb300 import problems as P
    from grmp_gb300 import api
    from grmp_gb300 import fespace as F
    out = [P.poisson3d(4, seed=2), P.poisson2d(10), P.poisson3d(3, seed=5, order=1), P.elasticity2d(6, seed=1)]
    g = G.grid_unitsquare(7)
    FES = F.FESpace(F.H1P2(1, 2), g)
    rng = np.random.default_rng(4)
    ops = [api.LaplaceOperator(0.5), api.ReactionOperator(api.CellCoefficient(rng.uniform(0.0, 10.0, g.ncells)))]
    out.append(P.LinearProblem("reaction", FES, ops, None, FES.boundary_dofs(), {}))
    return out


@pytest.mark.parametrize("idx", range(5))
def test_dual_precision_assembly_matches_separate_passes(G, ctx, idx):
    prob = _problems(G)[idx]
    A = G.FEMatrix(ctx, prob.FES, prob.operators)
    G.assemble(A, prob.operators, G.FP64)
    G.assemble(A, prob.operators, G.FP32)
    a64, a32 = A.download(G.FP64), A.download(G.FP32)
    B = G.FEMatrix(ctx, prob.FES, prob.operators)
    G.assemble(B, prob.operators, G.FP64_FP32)
    b64, b32 = B.download(G.FP64), B.download(G.FP32)
    assert np.array_equal(a64.indptr, b64.indptr) and np.array_equal(a64.indices, b64.indices)
    assert np.array_equal(a64.data, b64.data)
    assert np.array_equal(a32.data, b32.data)
