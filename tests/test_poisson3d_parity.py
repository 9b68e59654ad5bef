"""Parity of the 3D P2 Poisson path at sizes well above the small-mesh tests,
through the SpMV configurations the benchmark's solves use.

The benchmark problem (64^3 Kuhn cubes, lognormal kappa, Fourier rhs) at
16^3 (35,937 DoFs) is compared with the oracle's sparse-direct FP64 solution
(SuperLU standing in for UMFPACK), and at 24^3 (117,649 DoFs) with the
oracle's refined FP64 solution (Jacobi-CG + iterative refinement with
double-double residuals, itself pinned against SuperLU in
test_oracle_reference.py).  Each GPU solve -- plain FP64 Jacobi-PCG and the
mixed FP32-inner / FP64-outer solver, in the row-loop (10408, 408),
staged-window (20204, 20408) and two-run 16-bit column (604xx, 60208,
60802; 64208 / 64404 / 65208 / 65404 / 66404 on the Jacobi-scaled copy
with the row state in shared memory) SpMV forms the autotuner picks among on the 64^3 matrix -- must be
within 1e-10 relative 2-norm error.  The FP64 matrix is
also checked against the oracle's per nonzero (1e-12 relative, floored at
1e-3 of the row maximum).
"""
import numpy as np
import pytest

from parity_helpers import oracle_system

pytestmark = pytest.mark.gpu

CONFIGS = [("fp64", 408), ("fp64", 208), ("mixed", 10408), ("mixed", 10404), ("mixed", 20204), ("mixed", 20408),
           ("mixed", 60404), ("mixed", 60208), ("mixed", 60802), ("mixed", 60408), ("mixed", 64208),
           ("mixed", 64404), ("mixed", 65208), ("mixed", 65404),
           ("mixed", 66404)]


def _reference(G, O, n):
    from grmp_gb300 import problems as P
    prob = P.poisson3d(n, seed=0)
    A0, Apen, b0, bpen = oracle_system(G, O, prob)
    if n <= 16:
        uo = O.solve_direct(Apen, bpen)
        how = "superlu"
    else:
        x0, _, _ = O.solve_cg(Apen, bpen, 1e-11)
        uo, info = O.solve_refined(Apen, bpen, inner_reltol=1e-6, x0=x0)
        assert info["last_correction"] <= 4.5e-16
        how = "refined"
    return prob, A0, uo, how


@pytest.fixture(scope="module", params=[16, 24])
def case(request, G, O, ctx):
    from grmp_gb300 import problems as P
    prob, A0, uo, how = _reference(G, O, request.param)
    sysd = P.DeviceSystem(ctx, prob, mixed=True)
    G.assemble(sysd.A, prob.operators, G.FP64)
    Ag = sysd.A.download(G.FP64)
    assert np.array_equal(Ag.indptr, A0.indptr) and np.array_equal(Ag.indices, A0.indices)
    rowmax = np.maximum.reduceat(np.abs(A0.data), A0.indptr[:-1])
    rm = np.repeat(rowmax, np.diff(A0.indptr))
    verr = np.abs(Ag.data - A0.data) / np.maximum(np.abs(A0.data), 1e-3 * rm)
    assert verr.max() <= 1e-12, verr.max()
    return request.param, sysd, uo, how


@pytest.mark.parametrize("mode,cfg", CONFIGS)
def test_solution_parity_bench_configs(G, case, mode, cfg):
    n, sysd, uo, how = case
    st = sysd.assemble_and_solve(G.GB300PCG(mode=mode, reltol=1e-11, abstol=0.0, spmv_config=cfg))
    assert st["spmv_config"] == cfg
    u = sysd.x.entries
    err = np.linalg.norm(u - uo) / np.linalg.norm(uo)
    assert err <= 1e-10, (n, how, mode, cfg, err, st)
