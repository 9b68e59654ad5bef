"""The solve seam: a matrix handed over as compressed sparse columns, as
solve_direct! hands LinearSolve its SparseMatrixCSC{Float64,Int64} with the
Dirichlet rows penalised by 1e60 (src/solvers.jl:89-101, :640-661), and its
values replaced with the pattern kept (the fixpoint loops' cache.A = A,
:906-911).  The oracle's own penalised matrix and right-hand side go through
grmp_matrix_from_csc (1-based, as from Julia) and grmp_solve in every mode;
solutions are compared with the oracle's sparse-direct FP64 solve of the same
penalised system at <= 1e-10 relative 2-norm error (the eliminated form the
library solves differs from the penalised one by O(1e-60))."""
import ctypes

import numpy as np
import pytest

from parity_helpers import oracle_system

pytestmark = pytest.mark.gpu

MODES = ["fp64", "mixed", "direct", "mixed_direct"]


def _csc1(A):
    C = A.tocsc()
    C.sort_indices()
    return (C.indptr.astype(np.int64) + 1, C.indices.astype(np.int64) + 1, C.data.copy())


def _solve(G, ctx, FES, M, b, mode):
    bv = G.FEVector(ctx, FES)
    bv.upload(b)
    x = G.FEVector(ctx, FES)
    st = G.GB300PCG(mode=mode, reltol=1e-12, abstol=0.0, maxiter=100000).solve(M, bv, x)
    return x.entries, st


@pytest.fixture(scope="module")
def pen(G, O):
    from grmp_gb300 import problems as P
    prob = P.poisson3d(5, seed=2)
    _, Apen, _, bpen = oracle_system(G, O, prob)
    return prob, Apen, bpen, O.solve_direct(Apen, bpen)


@pytest.mark.parametrize("symmetric", [1, 0])
@pytest.mark.parametrize("mode", MODES)
def test_penalised_csc_matches_oracle(G, ctx, pen, mode, symmetric):
    prob, Apen, bpen, uo = pen
    M = G.ImportedMatrix(ctx, _csc1(Apen), symmetric=bool(symmetric), penalty_threshold=1e30, index_base=1)
    assert M.penalty_rows() == prob.fixed.size
    u, st = _solve(G, ctx, prob.FES, M, bpen, mode)
    assert np.linalg.norm(u - uo) / np.linalg.norm(uo) <= 1e-10, (mode, st)
    M.free()


def test_inhomogeneous_penalty_data(G, O, ctx, pen):
    """b_d = 1e60 * g_d on the penalty rows: the solution takes g there."""
    prob, Apen, bpen, _ = pen
    g = np.sin(np.arange(prob.fixed.size))
    b = bpen.copy()
    b[prob.fixed] = 1e60 * g
    uo = O.solve_direct(Apen, b)
    M = G.ImportedMatrix(ctx, _csc1(Apen), penalty_threshold=1e30, index_base=1)
    for mode in ("fp64", "mixed"):
        u, _ = _solve(G, ctx, prob.FES, M, b, mode)
        assert np.linalg.norm(u - uo) / np.linalg.norm(uo) <= 1e-10
        assert np.max(np.abs(u[prob.fixed] - g)) <= 1e-12


def test_update_values_keeps_pattern(G, O, ctx, pen):
    """cache.A = A': new values, same pattern -- the next solve uses them."""
    from grmp_gb300 import problems as P
    prob, Apen, bpen, _ = pen
    prob2 = P.poisson3d(5, seed=9)   # same mesh, other kappa
    _, Apen2, _, bpen2 = oracle_system(G, O, prob2)
    # both on the union of their drop-zero patterns (explicit zeros stored),
    # as a caller reusing one pattern across fixpoint steps holds them
    U = (abs(Apen) + abs(Apen2)).tocsc()
    U.sort_indices()
    U.data[:] = 0.0

    rows = U.indices
    cols = np.repeat(np.arange(U.shape[1]), np.diff(U.indptr))

    def on_union(A):
        B = U.copy()
        B.data = np.asarray(A.tocsr()[rows, cols]).ravel()
        return B

    M = G.ImportedMatrix(ctx, _csc1(on_union(Apen)), penalty_threshold=1e30, index_base=1)
    _solve(G, ctx, prob.FES, M, bpen, "mixed")
    M.update_values(_csc1(on_union(Apen2))[2])
    uo2 = O.solve_direct(Apen2, bpen2)
    for mode in ("mixed", "direct"):
        u, _ = _solve(G, ctx, prob.FES, M, bpen2, mode)
        assert np.linalg.norm(u - uo2) / np.linalg.norm(uo2) <= 1e-10


def test_unpenalised_import_equals_assembled(G, ctx):
    """Without penalty rows the imported matrix is the assembled one: an
    FP64 solve through it equals the assembled handle's bit for bit."""
    from grmp_gb300 import problems as P
    prob = P.poisson2d(12)
    sysd = P.DeviceSystem(ctx, prob, mixed=False)
    st0 = sysd.assemble_and_solve(G.GB300PCG(mode="fp64", reltol=1e-12, abstol=0.0, spmv_config=404))
    x0 = sysd.x.entries
    A = sysd.A.download(G.FP64)
    M = G.ImportedMatrix(ctx, A, symmetric=True, penalty_threshold=0.0)
    assert M.penalty_rows() == 0
    x = G.FEVector(ctx, prob.FES)
    st = G.GB300PCG(mode="fp64", reltol=1e-12, abstol=0.0, spmv_config=404).solve(M, sysd.b, x)
    assert st["iterations"] == st0["iterations"]
    assert np.array_equal(x.entries, x0)


def test_import_rejects_bad_input(G, ctx):
    from grmp_gb300 import _lib as L
    lib = ctx.lib
    h = ctypes.c_void_p()
    p64 = lambda a: a.ctypes.data_as(ctypes.POINTER(ctypes.c_int64))  # noqa: E731
    pd = lambda a: a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))  # noqa: E731
    colptr = np.array([1, 3, 4], dtype=np.int64)
    v = np.ones(3)
    unsorted = np.array([2, 1, 2], dtype=np.int64)
    assert lib.grmp_matrix_from_csc(ctx.h, 2, p64(colptr), p64(unsorted), pd(v), 1, 1, 0.0, ctypes.byref(h)) == \
        L.ERR_INVALID_ARG
    assert b"strictly increasing" in lib.grmp_last_error(ctx.h)
    outside = np.array([1, 3, 2], dtype=np.int64)
    assert lib.grmp_matrix_from_csc(ctx.h, 2, p64(colptr), p64(outside), pd(v), 1, 1, 0.0, ctypes.byref(h)) == \
        L.ERR_INVALID_ARG
    base0 = np.array([0, 2, 3], dtype=np.int64)
    assert lib.grmp_matrix_from_csc(ctx.h, 2, p64(base0), p64(unsorted), pd(v), 1, 1, 0.0, ctypes.byref(h)) == \
        L.ERR_INVALID_ARG
    # an imported matrix has no assembly space
    good = np.array([1, 2, 1, 2], dtype=np.int64)
    cp = np.array([1, 3, 5], dtype=np.int64)
    vals = np.array([2.0, -1.0, -1.0, 2.0])
    assert lib.grmp_matrix_from_csc(ctx.h, 2, p64(cp), p64(good), pd(vals), 1, 1, 0.0, ctypes.byref(h)) == 0
    t = (L.BilinearTerm * 1)()
    t[0].op_kind = L.OP_LAPLACE
    t[0].factor = 1.0
    assert lib.grmp_assemble_bilinear(h, 1, t, L.FP64) == L.ERR_INVALID_ARG
    assert lib.grmp_matrix_destroy(h) == 0
