"""Staged SpMV configurations of the mixed solver: the FP32 (column, value)
pairs re-laid out in 32 KB row windows and streamed through a ring of
shared-memory stages by bulk async copies.

* every staged configuration solves to the oracle's sparse-direct FP64
  solution within 1e-10 (relative 2-norm), on a 3D P2 problem with more
  windows than blocks and on a 2D problem with fewer windows than blocks
  (blocks without windows; blocks whose window count is below the stage
  count, so the ring holds the same window twice);
* few blocks (many windows per block) give the same tolerance;
* a repeated solve is bit-identical;
* FP64 solves refuse the staged configurations (GRMP_ERR_UNSUPPORTED).
"""
import numpy as np
import pytest

from parity_helpers import oracle_system

pytestmark = pytest.mark.gpu

STAGED = [20204, 20408, 20804, 30408, 30804]


def _solve(G, ctx, prob, cfg, grid=0):
    from grmp_gb300 import problems as P
    sysd = P.DeviceSystem(ctx, prob, mixed=True)
    s = G.GB300PCG(mode="mixed", reltol=1e-11, abstol=0.0, spmv_config=cfg, grid_blocks=grid)
    st = sysd.assemble_and_solve(s)
    return sysd.x.entries.copy(), st


@pytest.fixture(scope="module")
def p3d(G, O):
    from grmp_gb300 import problems as P
    prob = P.poisson3d(16, seed=3)
    _, Apen, _, bpen = oracle_system(G, O, prob)
    return prob, O.solve_direct(Apen, bpen)


@pytest.fixture(scope="module")
def p2d(G, O):
    from grmp_gb300 import problems as P
    prob = P.poisson2d(24)
    _, Apen, _, bpen = oracle_system(G, O, prob)
    return prob, O.solve_direct(Apen, bpen)


@pytest.mark.parametrize("cfg", STAGED)
def test_staged_3d_matches_oracle(G, ctx, p3d, cfg):
    prob, uo = p3d
    u, st = _solve(G, ctx, prob, cfg)
    assert st["spmv_config"] == cfg
    err = np.linalg.norm(u - uo) / np.linalg.norm(uo)
    assert err <= 1e-10, (err, st)


@pytest.mark.parametrize("cfg", STAGED)
def test_staged_2d_fewer_windows_than_blocks(G, ctx, p2d, cfg):
    prob, uo = p2d
    u, st = _solve(G, ctx, prob, cfg)
    err = np.linalg.norm(u - uo) / np.linalg.norm(uo)
    assert err <= 1e-10, (err, st)


@pytest.mark.parametrize("grid", [1, 5])
def test_staged_many_windows_per_block(G, ctx, p3d, grid):
    prob, uo = p3d
    u, st = _solve(G, ctx, prob, 20408, grid=grid)
    assert st["grid_blocks"] == grid
    err = np.linalg.norm(u - uo) / np.linalg.norm(uo)
    assert err <= 1e-10, (err, st)


def test_staged_repeatable(G, ctx, p3d):
    prob, _ = p3d
    u1, s1 = _solve(G, ctx, prob, 30408)
    u2, s2 = _solve(G, ctx, prob, 30408)
    assert s1["iterations"] == s2["iterations"]
    assert np.array_equal(u1, u2)


def test_fp64_refuses_staged(G, ctx):
    from grmp_gb300 import problems as P
    prob = P.poisson2d(8)
    sysd = P.DeviceSystem(ctx, prob, mixed=False)
    with pytest.raises(G.GrmpError) as ei:
        sysd.assemble_and_solve(G.GB300PCG(mode="fp64", reltol=1e-11, abstol=0.0, spmv_config=20408))
    from grmp_gb300 import _lib as L
    assert ei.value.code == L.ERR_UNSUPPORTED
