"""Problem set-ups of the benchmark configurations and a solve_direct!-style driver.

Synthetic, seeded inputs with the shapes the benchmark names (no dataset is
involved):

* poisson2d: unit square n x n (n=128: 32,768 triangles), H1P2{1,2},
  LaplaceOperator(1e-3), f = 1, homogeneous Dirichlet on regions 1-4.
* poisson3d: unit cube n^3 Kuhn (n=64: 1,572,864 tets), H1P2{1,3},
  per-cell kappa = exp(N(0,1)) as BilinearForm([Gradient, Gradient],
  Action(kappa[cell] * input; "I")), f = sum_{m=1..8} a_m sin(pi k_m . x) with
  a_m ~ N(0,1), k_m in {1..4}^3, homogeneous Dirichlet on all faces.
* elasticity2d: unit square n x n (n=256), H1P2{2,2},
  HookStiffnessOperator2D(mu=1, lambda=1e3), per-cell body force ~ N(0,1)^2,
  homogeneous Dirichlet on the left edge (region 4), traction-free elsewhere.
"""
from __future__ import annotations

import time
from dataclasses import dataclass, field

import numpy as np

from . import api
from . import _lib as L
from .fespace import FESpace, H1P1, H1P2
from .mesh import grid_unitsquare, grid_unitcube_kuhn


@dataclass
class LinearProblem:
    name: str
    FES: FESpace
    operators: list
    rhs: api.LinearFormOp
    fixed: np.ndarray
    meta: dict = field(default_factory=dict)


def poisson2d(n: int = 128, kappa: float = 1e-3, order: int = 2) -> LinearProblem:
    g = grid_unitsquare(n)
    FES = FESpace(H1P2(1, 2) if order == 2 else H1P1(1), g)
    ops = [api.LaplaceOperator(kappa)]
    rhs = api.LinearForm(api.Identity, api.DataFunction.constant([1.0]))
    fixed = FES.boundary_dofs([1, 2, 3, 4])
    return LinearProblem(f"poisson2d_P{order}_{n}", FES, ops, rhs, fixed, {"dim": 2, "n": n, "kappa": kappa})


def fourier_modes(rng: np.random.Generator, dim: int, nmodes: int = 8):
    amp = rng.standard_normal(nmodes)
    k = rng.integers(1, 5, size=(nmodes, dim)).astype(np.float64)
    return amp, k


def poisson3d(n: int = 64, seed: int = 0, order: int = 2, sigma: float = 1.0) -> LinearProblem:
    rng = np.random.default_rng(seed)
    g = grid_unitcube_kuhn(n)
    FES = FESpace(H1P2(1, 3) if order == 2 else H1P1(1), g)
    kappa = np.exp(sigma * rng.standard_normal(g.ncells))
    ops = [api.BilinearForm([api.Gradient, api.Gradient], api.CellCoefficient(kappa),
                            APT=api.APT_SymmetricBilinearForm)]
    amp, k = fourier_modes(rng, 3)
    rhs = api.LinearForm(api.Identity, api.DataFunction.fourier(amp, k))
    fixed = FES.boundary_dofs()
    return LinearProblem(f"poisson3d_P{order}_{n}", FES, ops, rhs, fixed,
                         {"dim": 3, "n": n, "seed": seed, "kappa": kappa, "amp": amp, "k": k})


def elasticity2d(n: int = 256, seed: int = 0, mu: float = 1.0, lam: float = 1e3) -> LinearProblem:
    rng = np.random.default_rng(seed)
    g = grid_unitsquare(n)
    FES = FESpace(H1P2(2, 2), g)
    ops = [api.HookStiffnessOperator2D(mu, lam)]
    force = rng.standard_normal((g.ncells, 2))
    rhs = api.LinearForm(api.Identity, api.DataFunction.cellwise(force))
    fixed = FES.boundary_dofs([4])
    return LinearProblem(f"elasticity2d_P2_{n}", FES, ops, rhs, fixed,
                         {"dim": 2, "n": n, "seed": seed, "mu": mu, "lambda": lam, "force": force})


class DeviceSystem:
    """Pattern + vectors of one LinearProblem on a context (built once)."""

    def __init__(self, ctx: api.GB300Context, prob: LinearProblem, mixed: bool):
        self.ctx = ctx
        self.prob = prob
        self.mixed = mixed
        self.A = api.FEMatrix(ctx, prob.FES, prob.operators)
        self.b = api.FEVector(ctx, prob.FES)
        self.x = api.FEVector(ctx, prob.FES)

    def assemble_and_solve(self, solver: api.GB300PCG, dirichlet: int = L.DIRICHLET_ELIMINATE) -> dict:
        """assembly (FP64, plus FP32 for the mixed mode) + Dirichlet + solve."""
        t0 = time.perf_counter()
        api.assemble(self.A, self.prob.operators, L.FP64_FP32 if self.mixed else L.FP64)
        self.b.fill(0.0)
        api.assemble(self.b, self.prob.rhs)
        api.apply_dirichlet(self.A, self.b, self.prob.fixed, None, dirichlet)
        t1 = time.perf_counter()
        st = solver.solve(self.A, self.b, self.x)
        t2 = time.perf_counter()
        st = dict(st)
        st["assembly_s"] = t1 - t0
        st["solve_wall_s"] = t2 - t1
        return st
