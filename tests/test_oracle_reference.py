"""The oracle's large-problem FP64 reference and its threaded assembly (CPU).

bench.py measures the error of the GPU solutions at the full 3D size against
the oracle's own solution, which there cannot come from a sparse-direct
factorisation: FP64 Jacobi-CG corrected by iterative refinement with
double-double residuals.  These tests pin that reference against SuperLU on a
system the direct solver handles, and check that the threaded oracle
assembly (rows split over OpenMP threads) equals the one-thread loop bit for
bit.
"""
import json
import os
import subprocess
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _assemble(O, prob):
    FES = prob.FES
    g = FES.xgrid
    op = prob.operators[0]
    M = O.Matrix(FES.ndofs)
    M.add_bilinear(g.coords, g.cells, 2, 1, FES.celldofs, O.OP_GRADIENT, op.symmetric, op.factor,
                   O.ACT_CELLSCALE, op.cell_coef)
    b = np.zeros(FES.ndofs)
    f = prob.rhs.f
    O.assemble_linear(b, g.coords, g.cells, 2, 1, FES.celldofs, f.kind, f.params, prob.rhs.factor,
                      f.bonus_quadorder)
    M.penalize(prob.fixed)
    return M.csr(), O.penalized_rhs(b, prob.fixed)


def test_refined_cg_matches_superlu_3d_p2(G, O):
    from grmp_gb300 import problems as P
    prob = P.poisson3d(10, seed=3)   # 9,261 DoFs, lognormal kappa
    A, b = _assemble(O, prob)
    xd = O.solve_direct(A, b)
    x0, it, _ = O.solve_cg(A, b, 1e-11)
    xr, info = O.solve_refined(A, b, inner_reltol=1e-6, x0=x0)
    assert info["last_correction"] <= 4.5e-16 and info["relres"] <= 1e-14
    err = np.linalg.norm(xr - xd) / np.linalg.norm(xd)
    assert err <= 1e-13, err                       # both at FP64 rounding level
    # the refinement improves on the plain CG solve it starts from
    assert np.linalg.norm(xr - xd) < np.linalg.norm(x0 - xd)


def test_resid_dd_exact_on_integer_system(O):
    """Residuals that cancel exactly are found exactly (double-double sums)."""
    import scipy.sparse as sp
    A = sp.csr_matrix(np.array([[1e16, 1.0, -1e16], [1.0, 2.0, 0.0], [0.0, 0.0, 3.0]]))
    x = np.array([1.0, 1.0, 1.0])
    b = np.array([1.0, 3.0, 3.0])
    assert np.array_equal(O.resid_dd(A, x, b), np.zeros(3))


def _dump(threads: int, path: str):
    code = ("import sys, numpy as np; sys.path.insert(0, %r); sys.path.insert(0, %r);"
            "import conftest; import oracle as O; from test_oracle_reference import _assemble;"
            "from grmp_gb300 import problems as P; A, b = _assemble(O, P.poisson3d(7, seed=1));"
            "np.save(%r, np.concatenate([A.indptr.astype(float), A.indices.astype(float), A.data, b]))"
            % (os.path.join(ROOT, "oracle"), os.path.join(ROOT, "tests"), path))
    env = dict(os.environ, OMP_NUM_THREADS=str(threads))
    r = subprocess.run([sys.executable, "-c", code], env=env, capture_output=True, text=True, cwd=ROOT,
                       timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    return np.load(path)


def test_threaded_assembly_bitwise_equals_one_thread(tmp_path):
    a = _dump(1, str(tmp_path / "t1.npy"))
    b = _dump(5, str(tmp_path / "t5.npy"))
    assert a.shape == b.shape and np.array_equal(a, b)


def test_reference_arm_runs_the_full_workload():
    """With the sample size equal to the workload's, the reference arm says
    so (same_config) and its CPU baseline is the whole problem."""
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--workload",
                          "poisson3d", "--n", "6", "--cpu-n", "6", "--steps", "2", "--warmup", "3"],
                         capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert out.returncode == 0, out.stderr[-2000:]
    line = json.loads(out.stdout.strip().splitlines()[-1])
    assert line["config"]["same_config"] is True
    assert line["config"]["ndofs"] == 13 ** 3
    assert line["steps"] == 2 and line["warmup"] == 3   # warm-up as requested, up to three
