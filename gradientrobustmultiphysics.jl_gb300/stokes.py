"""Batched gradient-robust Stokes: Bernardi-Raugel / P0 with the BR->RT0
reconstruction in the right-hand side, solved by the iterated penalty method.

Reference: examples/Example221_StokesIterated2D.jl:52-108 (iterated penalty,
subiterations [[1],[2]]), examples/Example222_PressureRobustness2D.jl:73-81
(LinearForm(ReconstructionIdentity{HDIVRT0{2}}, f)), src/solvers.jl:1018+.

Many independent problems are packed into one block-diagonal system: each
problem keeps its own DoF numbering (BR pattern "N1f1": component-1 nodes,
component-2 nodes, faces, src/fedefs/h1v_br.jl:33) shifted by the DoFs of the
problems before it, so every problem owns a contiguous row range; its cells
(= P0 pressure DoFs) are contiguous too.
"""
from __future__ import annotations

import ctypes
import time
from dataclasses import dataclass, field

import numpy as np

from . import _lib as L
from . import api
from .fespace import FESpace, H1BR, FE_H1BR
from .mesh import SimplexMesh, grid_unitcube_kuhn, grid_unitsquare


class BatchedMesh(SimplexMesh):
    """Disjoint union of meshes of one dimension with the faces of each part
    kept (face numbering, normals and signs are those of the part)."""

    def __init__(self, parts):
        coords, cells, cfaces, normals, fvols, signs = [], [], [], [], [], []
        voff = foff = 0
        self.cell_offsets = [0]
        self.vert_offsets = [0]
        self.face_offsets = [0]
        for g in parts:
            fn, cf = g.faces()
            nr, fv, sg = g.face_geometry()
            coords.append(g.coords)
            cells.append(g.cells.astype(np.int64) + voff)
            cfaces.append(cf.astype(np.int64) + foff)
            normals.append(nr)
            fvols.append(fv)
            signs.append(sg)
            voff += g.nverts
            foff += fn.shape[0]
            self.cell_offsets.append(self.cell_offsets[-1] + g.ncells)
            self.vert_offsets.append(voff)
            self.face_offsets.append(foff)
        super().__init__(np.concatenate(coords), np.concatenate(cells).astype(np.int32), name=f"batch{len(parts)}")
        self.parts = list(parts)
        self._faces = (np.zeros((foff, self.dim), dtype=np.int32), np.concatenate(cfaces).astype(np.int32))
        self._facegeo = (np.concatenate(normals), np.concatenate(fvols), np.concatenate(signs))

    def faces(self):
        return self._faces

    def face_geometry(self):
        return self._facegeo


class BatchedBRSpace(FESpace):
    """H1BR{d} over a BatchedMesh with per-problem contiguous DoF blocks."""

    def __init__(self, bmesh: BatchedMesh):
        self.FEType = H1BR(bmesh.dim)
        self.xgrid = bmesh
        self.name = f"H1BR{{{bmesh.dim}}} batch"
        cds, fixed = [], []
        self.row_offsets = [0]
        off = 0
        for g in bmesh.parts:
            S = FESpace(H1BR(bmesh.dim), g)
            cds.append(S.celldofs.astype(np.int64) + off)
            fixed.append(S.boundary_dofs().astype(np.int64) + off)
            off += S.ndofs
            self.row_offsets.append(off)
        self.celldofs = np.ascontiguousarray(np.concatenate(cds).astype(np.int32))
        self.ndofs = off
        self.coffset = 0
        self._fixed = np.concatenate(fixed).astype(np.int32)

    def boundary_dofs(self, regions=None):
        return self._fixed


def cubic_coefficients(rng: np.random.Generator):
    """Coefficients a_ij of a cubic polynomial sum_{i+j<=3} a_ij x^i y^j."""
    return {(i, j): rng.standard_normal() for i in range(4) for j in range(4) if i + j <= 3}


def grad_plus_curl_terms(phi: dict, psi: dict):
    """Polynomial records (component, coef, e1, e2, 0) of
    f = grad(phi) + curl(psi), curl psi = (d psi/dy, -d psi/dx); degree <= 2.
    Always 12 records (the 6 monomials of degree <= 2 per component)."""
    acc = {}

    def add(c, coef, i, j):
        acc[(c, i, j)] = acc.get((c, i, j), 0.0) + coef

    for (i, j), a in phi.items():
        if i > 0:
            add(0, i * a, i - 1, j)
        if j > 0:
            add(1, j * a, i, j - 1)
    for (i, j), b in psi.items():
        if j > 0:
            add(0, j * b, i, j - 1)
        if i > 0:
            add(1, -i * b, i - 1, j)
    out = []
    for c in (0, 1):
        for i in range(3):
            for j in range(3 - i):
                out.append((c, acc.get((c, i, j), 0.0), i, j, 0))
    return np.array(out, dtype=np.float64)


def cubic_coefficients_3d(rng: np.random.Generator):
    """Coefficients a_ijk of a cubic sum_{i+j+k<=3} a_ijk x^i y^j z^k."""
    return {(i, j, k): rng.standard_normal() for i in range(4) for j in range(4) for k in range(4) if i + j + k <= 3}


def grad_plus_curl_terms_3d(phi: dict, psi):
    """Polynomial records (component, coef, e1, e2, e3) of
    f = grad(phi) + curl(psi) for a cubic phi and a cubic vector psi
    (curl psi = (d2 psi3 - d3 psi2, d3 psi1 - d1 psi3, d1 psi2 - d2 psi1));
    degree <= 2.  Always 30 records (the 10 monomials of degree <= 2 per
    component)."""
    acc = {}

    def add(c, coef, e):
        acc[(c, e)] = acc.get((c, e), 0.0) + coef

    def deriv(poly, j):
        for e, a in poly.items():
            if e[j] > 0:
                ee = list(e)
                ee[j] -= 1
                yield tuple(ee), e[j] * a

    for c in range(3):
        for e, a in deriv(phi, c):
            add(c, a, e)
    # (component, psi index, derivative direction, sign) of the curl
    for c, m, j, sg in ((0, 2, 1, 1), (0, 1, 2, -1), (1, 0, 2, 1), (1, 2, 0, -1), (2, 1, 0, 1), (2, 0, 1, -1)):
        for e, a in deriv(psi[m], j):
            add(c, sg * a, e)
    out = []
    for c in range(3):
        for i in range(3):
            for j in range(3 - i):
                for k in range(3 - i - j):
                    out.append((c, acc.get((c, (i, j, k)), 0.0), i, j, k))
    return np.array(out, dtype=np.float64)


@dataclass
class StokesBatchProblem:
    sizes: np.ndarray
    nus: np.ndarray
    terms: np.ndarray           # [nprob][12][5]
    mesh: BatchedMesh
    V: BatchedBRSpace
    lam: float = 1e4
    meta: dict = field(default_factory=dict)

    @property
    def nproblems(self) -> int:
        return len(self.sizes)

    @property
    def dim(self) -> int:
        return self.mesh.dim


def make_batch(nproblems: int = 2048, nmin: int = 8, nmax: int = 96, seed: int = 0, lam: float = 1e4,
               sizes=None, nus=None, dim: int = 2) -> StokesBatchProblem:
    """Seeded batch: n log-uniform in [nmin, nmax] (2D: n x n squares, 2 n^2
    triangles; 3D: n^3 cubes, 6 n^3 Kuhn tetrahedra), nu log-uniform in
    [1e-4, 1], f = grad(cubic) + curl(cubic)."""
    if dim not in (2, 3):
        raise ValueError("dim must be 2 or 3")
    rng = np.random.default_rng(seed)
    if sizes is None:
        sizes = np.rint(np.exp(rng.uniform(np.log(nmin), np.log(nmax), nproblems))).astype(int)
    if nus is None:
        nus = np.exp(rng.uniform(np.log(1e-4), np.log(1.0), len(sizes)))
    if dim == 2:
        terms = np.stack([grad_plus_curl_terms(cubic_coefficients(rng), cubic_coefficients(rng)) for _ in sizes])
    else:
        terms = np.stack([grad_plus_curl_terms_3d(cubic_coefficients_3d(rng),
                                                  [cubic_coefficients_3d(rng) for _ in range(3)]) for _ in sizes])
    cache = {}
    parts = []
    for n in sizes:
        if n not in cache:
            cache[n] = grid_unitsquare(int(n)) if dim == 2 else grid_unitcube_kuhn(int(n))
        parts.append(cache[n])
    bm = BatchedMesh(parts)
    V = BatchedBRSpace(bm)
    return StokesBatchProblem(np.asarray(sizes), np.asarray(nus), terms, bm, V, lam)


def velocity_operators(prob: StokesBatchProblem):
    """nu (grad u, grad v) [LaplaceOperator, symmetric] with nu per cell, and
    lambda (div R u, div R v) [BilinearForm([ReconstructionDivergence]^2),
    APT_BilinearForm]."""
    cellnu = np.repeat(prob.nus, np.diff(prob.mesh.cell_offsets))
    lap = api.Operator(L.OP_LAPLACE, True, 1.0, cell_coef=cellnu, name="nu (grad u, grad v)")
    pen = api.Operator(L.OP_RDIVRDIV, False, prob.lam, name="lambda (div R u, div R v)")
    return [lap, pen]


class StokesBatchSystem:
    """Device-resident batched system: pattern, assembly, reconstructed rhs."""

    def __init__(self, ctx: api.GB300Context, prob: StokesBatchProblem, mixed: bool = True,
                 split_penalty: bool = True, direct: bool = False, reconstruction: str = "RT0",
                 solver: str = ""):
        """mixed: FP32 inner solves inside FP64 refinement.  split_penalty
        (mixed only): the FP32 matrix holds the viscous term alone and the
        inner operator applies the penalty per cell in factored form.
        direct: FP64 multifrontal Cholesky per problem (the reference's
        sparse-direct sweep solves), factored once for all sweeps.
        solver (overrides mixed / direct): "fp64" or "mixed" (block PCG),
        "direct", or "mixed_direct" (an FP32 factor per problem
        preconditioning FP64 CG, with the FP64 factor as the per-problem
        fallback).
        reconstruction: "RT0" or "BDM1", the H(div) space of the
        right-hand side's ReconstructionIdentity test operator."""
        if reconstruction not in ("RT0", "BDM1"):
            raise ValueError("reconstruction must be RT0 or BDM1")
        self.reconstruction = reconstruction
        self.ctx = ctx
        self.prob = prob
        if solver:
            if solver not in ("fp64", "mixed", "direct", "mixed_direct"):
                raise ValueError(f"solver {solver}")
            direct = solver in ("direct", "mixed_direct")
            mixed = solver == "mixed"
        self.mixed_direct = solver == "mixed_direct"
        self.direct = bool(direct)
        mixed = mixed and not self.direct
        self.mixed = mixed
        self.split_penalty = bool(split_penalty and mixed)
        self.ops = velocity_operators(prob)
        t0 = time.perf_counter()
        self.A = api.FEMatrix(ctx, prob.V, self.ops)
        self.bf = api.FEVector(ctx, prob.V)
        self.u = api.FEVector(ctx, prob.V)
        self.p = _RawVector(ctx, prob.mesh.ncells)
        self.setup_s = time.perf_counter() - t0

    def assemble(self):
        api.assemble(self.A, self.ops, L.FP64)
        if self.mixed:
            api.assemble(self.A, self.ops[:1] if self.split_penalty else self.ops, L.FP32)
        self.bf.fill(0.0)
        r = L.Rhs()
        r.kind = L.RHS_POLY
        r.ncomponents = self.prob.dim
        par = np.ascontiguousarray(self.prob.terms, dtype=np.float64).ravel()
        grp = np.ascontiguousarray(np.repeat(np.arange(self.prob.nproblems, dtype=np.int32),
                                             np.diff(self.prob.mesh.cell_offsets)))
        self._keep = (par, grp)
        r.params = par.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
        r.nparams = par.size
        r.factor = 1.0
        r.bonus_quadorder = 2
        r.test_operator = 2 if self.reconstruction == "BDM1" else 1
        r.cell_group = grp.ctypes.data_as(ctypes.POINTER(ctypes.c_int32))
        r.ngroups = self.prob.nproblems
        sh = self.ctx.space(self.prob.V)
        self.ctx.check(self.ctx.lib.grmp_assemble_linear(sh, ctypes.byref(r), self.bf.h))
        api.apply_dirichlet(self.A, self.bf, self.prob.V.boundary_dofs(), None, L.DIRICHLET_ELIMINATE)

    def solve(self, sweeps: int = 6, reltol: float = 1e-11, maxiter: int = 200000, sweep_tol: float = 0.0,
              inner_reltol: float = 0.1, block_threads: int = 0, raise_on_error: bool = True):
        P = L.StokesBatchParams()
        ro = np.ascontiguousarray(self.prob.V.row_offsets, dtype=np.int32)
        co = np.ascontiguousarray(self.prob.mesh.cell_offsets, dtype=np.int32)
        P.nproblems = self.prob.nproblems
        P.row_offsets = ro.ctypes.data_as(ctypes.POINTER(ctypes.c_int32))
        P.cell_offsets = co.ctypes.data_as(ctypes.POINTER(ctypes.c_int32))
        P.lam = self.prob.lam
        P.sweeps = sweeps
        P.sweep_tol = sweep_tol
        P.mode = (L.SOLVE_MIXED_DIRECT if self.mixed_direct else
                  L.SOLVE_DIRECT if self.direct else (L.SOLVE_MIXED if self.mixed else L.SOLVE_FP64))
        P.reltol = reltol
        P.inner_reltol = inner_reltol
        P.maxiter = maxiter
        P.block_threads = block_threads
        P.split_penalty = 1 if self.split_penalty else 0
        st = L.StokesBatchStats()
        its = np.zeros(self.prob.nproblems, dtype=np.int32)
        rc = self.ctx.lib.grmp_stokes_batch_solve(self.A.h, self.bf.h, self.u.h, self.p.h, ctypes.byref(P),
                                                  its.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)),
                                                  ctypes.byref(st))
        out = {"rc": rc, "status": st.status, "max_iterations": st.max_iterations,
               "total_iterations": st.total_iterations, "max_sweeps": st.max_sweeps,
               "failed": st.failed_problems, "max_relres": st.max_relres, "solve_ms": st.solve_ms,
               "fp64_fallbacks": st.fp64_fallbacks, "iterations": its}
        if raise_on_error:
            self.ctx.check(rc)
        return out

    def velocity(self) -> np.ndarray:
        return self.u.entries

    def pressure(self) -> np.ndarray:
        return self.p.entries


class _RawVector:
    """A device vector of given length (the P0 pressure of all cells)."""

    def __init__(self, ctx, n: int):
        self.ctx = ctx
        self.n = n
        self.h = ctypes.c_void_p()
        ctx.check(ctx.lib.grmp_vector_create(ctx.h, n, ctypes.byref(self.h)))

    @property
    def entries(self) -> np.ndarray:
        out = np.empty(self.n)
        self.ctx.check(self.ctx.lib.grmp_vector_download(self.h, out.ctypes.data_as(ctypes.POINTER(ctypes.c_double))))
        return out
