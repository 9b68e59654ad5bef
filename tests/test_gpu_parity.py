"""GPU parity of the CUDA path (through the C-ABI) against the CPU oracle.

Tolerances:
* sparsity pattern: bit-exact (rowptr and column indices equal);
* FP64 matrix values: per nonzero |a - o| <= 1e-12 * max(|o|, 1e-3 * max|o_row|)
  (1e-12 relative per nonzero; the floor covers entries that are sums of
  cancelling cell contributions, whose relative error is undefined);
* FP32 matrix values: row-scaled, |a - o| <= 2e-6 * max|o_row| (FP32 element
  matrices round each cell contribution; cancelling contributions make a
  per-entry relative bound meaningless at FP32);
* FP64 right-hand side: max |b - o| <= 1e-12 * max |o|;
* solutions: ||u - u_oracle||_2 / ||u_oracle||_2 <= 1e-10 for the FP64 and
  the mixed-precision solver, u_oracle from the sparse-direct FP64 solve of
  the reference's penalised system.
"""
import numpy as np
import pytest

from parity_helpers import oracle_system

pytestmark = pytest.mark.gpu


def check_values(Ag, Ao, tol, rowscaled=False):
    assert np.array_equal(Ag.indptr, Ao.indptr)
    assert np.array_equal(Ag.indices, Ao.indices)
    o = Ao.data
    rowmax = np.maximum.reduceat(np.abs(o), Ao.indptr[:-1])
    rm = np.repeat(rowmax, np.diff(Ao.indptr))
    scale = rm if rowscaled else np.maximum(np.abs(o), 1e-3 * rm)
    err = np.abs(Ag.data - o) / scale
    assert err.max() <= tol, f"max scaled error {err.max():.3e}"
    return err.max()


def small_problems(G):
    from grmp_gb300 import problems as P
    return [P.poisson2d(8), P.poisson2d(6, order=1), P.poisson3d(3, seed=3), P.poisson3d(3, seed=4, order=1),
            P.elasticity2d(6, seed=5)]


@pytest.mark.parametrize("idx", range(5))
def test_pattern_and_values_parity(G, O, ctx, idx):
    prob = small_problems(G)[idx]
    A0, Apen, b0, _ = oracle_system(G, O, prob)
    A = G.FEMatrix(ctx, prob.FES, prob.operators)
    rp, ci = A.pattern()
    assert np.array_equal(rp, A0.indptr), "row pointers differ"
    assert np.array_equal(ci, A0.indices), "column indices differ"
    G.assemble(A, prob.operators, G.FP64)
    check_values(A.download(G.FP64), A0, 1e-12)
    G.assemble(A, prob.operators, G.FP32)
    check_values(A.download(G.FP32), A0, 2e-6, rowscaled=True)
    b = G.FEVector(ctx, prob.FES)
    G.assemble(b, prob.rhs)
    bg = b.entries
    assert np.max(np.abs(bg - b0)) <= 1e-12 * np.max(np.abs(b0))


def test_config1_pattern_full_size(G, O, ctx):
    """128x128 P2 Laplace: the drop-exact-zero pattern has 395,265 nonzeros,
    identical to the oracle's."""
    from grmp_gb300 import problems as P
    prob = P.poisson2d(128)
    A0, _, _, _ = oracle_system(G, O, prob)
    A = G.FEMatrix(ctx, prob.FES, prob.operators)
    assert A.nnz == 395265
    rp, ci = A.pattern()
    assert np.array_equal(rp, A0.indptr) and np.array_equal(ci, A0.indices)


def test_assembly_is_bitwise_reproducible(G, ctx):
    from grmp_gb300 import problems as P
    prob = P.poisson3d(6, seed=7)
    A = G.FEMatrix(ctx, prob.FES, prob.operators)
    G.assemble(A, prob.operators, G.FP64)
    v1 = A.download(G.FP64).data.copy()
    G.assemble(A, prob.operators, G.FP64)
    v2 = A.download(G.FP64).data
    assert np.array_equal(v1.view(np.uint64), v2.view(np.uint64))


def test_penalty_dirichlet_matches_reference_form(G, O, ctx):
    from grmp_gb300 import problems as P
    prob = P.poisson2d(8)
    _, Apen, _, bpen = oracle_system(G, O, prob)
    A = G.FEMatrix(ctx, prob.FES, prob.operators)
    G.assemble(A, prob.operators, G.FP64)
    b = G.FEVector(ctx, prob.FES)
    G.assemble(b, prob.rhs)
    G.apply_dirichlet(A, b, prob.fixed, None, G.DIRICHLET_PENALTY, 1e60)
    check_values(A.download(G.FP64), Apen, 1e-12)
    assert np.max(np.abs(b.entries - bpen)) <= 1e-12 * np.max(np.abs(bpen))


@pytest.mark.parametrize("idx", range(5))
@pytest.mark.parametrize("mode", ["fp64", "mixed"])
def test_solve_parity(G, O, ctx, idx, mode):
    from grmp_gb300 import problems as P
    prob = small_problems(G)[idx]
    _, Apen, _, bpen = oracle_system(G, O, prob)
    uo = O.solve_direct(Apen, bpen)
    sysd = P.DeviceSystem(ctx, prob, mixed=(mode == "mixed"))
    st = sysd.assemble_and_solve(G.GB300PCG(mode=mode, reltol=1e-11, abstol=0.0))
    u = sysd.x.entries
    err = np.linalg.norm(u - uo) / np.linalg.norm(uo)
    assert err <= 1e-10, (err, st)


def test_solve_penalty_form_fp64(G, O, ctx):
    """The reference's own system (penalty 1e60) solved by FP64 PCG."""
    from grmp_gb300 import problems as P
    prob = P.poisson2d(16)
    _, Apen, _, bpen = oracle_system(G, O, prob)
    uo = O.solve_direct(Apen, bpen)
    sysd = P.DeviceSystem(ctx, prob, mixed=False)
    sysd.assemble_and_solve(G.GB300PCG(mode="fp64", reltol=1e-11, abstol=0.0), dirichlet=G.DIRICHLET_PENALTY)
    u = sysd.x.entries
    assert np.linalg.norm(u - uo) / np.linalg.norm(uo) <= 1e-10


@pytest.mark.parametrize("mode", ["fp64", "mixed"])
def test_config1_full_size_solve(G, O, ctx, mode):
    from grmp_gb300 import problems as P
    prob = P.poisson2d(128)
    _, Apen, _, bpen = oracle_system(G, O, prob)
    uo = O.solve_direct(Apen, bpen)
    sysd = P.DeviceSystem(ctx, prob, mixed=(mode == "mixed"))
    st = sysd.assemble_and_solve(G.GB300PCG(mode=mode, reltol=1e-11, abstol=0.0))
    u = sysd.x.entries
    err = np.linalg.norm(u - uo) / np.linalg.norm(uo)
    assert err <= 1e-10, (err, st)


def test_not_converged_is_reported(G, ctx):
    from grmp_gb300 import problems as P
    prob = P.poisson2d(16)
    sysd = P.DeviceSystem(ctx, prob, mixed=False)
    s = G.GB300PCG(mode="fp64", reltol=1e-14, abstol=0.0, maxiter=3)
    st = None
    with pytest.raises(G.GrmpError) as ei:
        st = sysd.assemble_and_solve(s)
    assert ei.value.code == 4
    assert s.last_stats["iterations"] == 3


def test_budget_rejects_oversized_request(G):
    from grmp_gb300 import problems as P
    c = G.GB300Context(0, hbm_budget_bytes=1 << 20)
    try:
        prob = P.poisson3d(8)
        with pytest.raises(G.GrmpError) as ei:
            G.FEMatrix(c, prob.FES, prob.operators)
        assert ei.value.code == 6
    finally:
        c.close()


def test_invalid_input_rejected_before_launch(G, ctx):
    import ctypes
    lib = ctx.lib
    h = ctypes.c_void_p()
    coords = np.zeros((3, 2))
    cells = np.array([[0, 1, 5]], dtype=np.int32)    # vertex 5 does not exist
    rc = lib.grmp_mesh_upload(ctx.h, 2, 3, coords.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), 1,
                              cells.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)), ctypes.byref(h))
    assert rc == 1
