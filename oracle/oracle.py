"""Python harness of the CPU oracle -- TEST INFRASTRUCTURE ONLY.

Imported by tests/, by __graft_entry__.smoke() and by bench.py's CPU-baseline
leg.  The product never imports this module.

It wraps ``grmp_oracle.c`` (a restatement of GradientRobustMultiPhysics.jl's
assembly, see that file's header), restates the DoF-map construction of
``init_dofmap_from_pattern!`` (src/dofmaps.jl:201-330) independently of the
library's own, and performs the reference's FP64 solve: penalised system
(src/solvers.jl:640-652) and a sparse-direct factorisation.  The reference's
default is UMFPACK via LinearSolve.jl (src/solvers.jl:55); scipy's SuperLU is
the sparse-direct solver available here and stands in for it.  For systems
too large for a direct factorisation the FP64 CG of grmp_oracle.c is used with
a stated tolerance.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
SO = os.path.join(BUILD, "libgrmp_oracle.so")

FE_P1, FE_P2, FE_BR, FE_RT0, FE_BDM1, FE_P0 = 1, 2, 3, 4, 5, 6
OP_IDENTITY, OP_GRADIENT, OP_SYMGRAD, OP_DIVERGENCE = 0, 1, 2, 3
ACT_NONE, ACT_CELLSCALE, ACT_HOOKE2D, ACT_HOOKE3D = 0, 1, 2, 3
RHS_CONST, RHS_CELL, RHS_FOURIER, RHS_POLY = 0, 1, 2, 3


def build(force: bool = False) -> str:
    """Compile grmp_oracle.c (no FMA contraction, OpenMP for the CG)."""
    src = os.path.join(HERE, "grmp_oracle.c")
    os.makedirs(BUILD, exist_ok=True)
    if force or not os.path.exists(SO) or os.path.getmtime(SO) < os.path.getmtime(src):
        cmd = ["gcc", "-O2", "-std=c11", "-D_GNU_SOURCE", "-fPIC", "-shared", "-ffp-contract=off",
               "-fno-fast-math", "-fopenmp", src, "-o", SO, "-lm"]
        subprocess.check_call(cmd)
    return SO


_lib = None


def lib():
    global _lib
    if _lib is None:
        _lib = ctypes.CDLL(build())
        L = _lib
        dp = ctypes.POINTER(ctypes.c_double)
        ip = ctypes.POINTER(ctypes.c_int)
        llp = ctypes.POINTER(ctypes.c_longlong)
        L.oracle_qrule.argtypes = [ctypes.c_int, ctypes.c_int, dp, dp]
        L.oracle_qrule.restype = ctypes.c_int
        L.oracle_basis_tables.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, dp, dp, dp]
        L.oracle_basis_tables.restype = ctypes.c_int
        L.oracle_mat_new.argtypes = [ctypes.c_int]
        L.oracle_mat_new.restype = ctypes.c_void_p
        L.oracle_mat_free.argtypes = [ctypes.c_void_p]
        L.oracle_mat_nnz.argtypes = [ctypes.c_void_p]
        L.oracle_mat_nnz.restype = ctypes.c_longlong
        L.oracle_mat_csr.argtypes = [ctypes.c_void_p, llp, ip, dp]
        L.oracle_mat_penalize.argtypes = [ctypes.c_void_p, ctypes.c_int, ip, ctypes.c_double]
        L.oracle_assemble_bilinear.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, dp, ctypes.c_int, ip,
                                               ctypes.c_int, ctypes.c_int, ip, ctypes.c_int, ctypes.c_int,
                                               ctypes.c_double, ctypes.c_int, dp, ctypes.c_double, ctypes.c_double,
                                               ctypes.c_int]
        L.oracle_assemble_bilinear.restype = ctypes.c_int
        L.oracle_assemble_linear.argtypes = [dp, ctypes.c_int, ctypes.c_int, dp, ctypes.c_int, ip, ctypes.c_int,
                                             ctypes.c_int, ip, ctypes.c_int, dp, ctypes.c_int, ctypes.c_double,
                                             ctypes.c_int]
        L.oracle_assemble_linear.restype = ctypes.c_int
        L.oracle_item_l2error.argtypes = [dp, dp, ctypes.c_int, ctypes.c_int, dp, ctypes.c_int, ip, ctypes.c_int,
                                          ctypes.c_int, ip, dp, dp, ctypes.c_int, ctypes.c_int, dp, ctypes.c_int,
                                          ctypes.c_double, ctypes.c_int]
        L.oracle_item_l2error.restype = ctypes.c_int
        L.oracle_item_l2error_br.argtypes = [dp, dp, ctypes.c_int, ctypes.c_int, dp, ip, ip, dp, ip, dp, dp,
                                             ctypes.c_int, ctypes.c_int, dp, ctypes.c_int, ctypes.c_double,
                                             ctypes.c_int]
        L.oracle_item_l2error_br.restype = ctypes.c_int
        L.oracle_cg.argtypes = [ctypes.c_int, llp, ip, dp, dp, dp, ctypes.c_double, ctypes.c_int, dp]
        L.oracle_cg.restype = ctypes.c_int
        L.oracle_set_threads.argtypes = [ctypes.c_int]
        L.oracle_set_threads.restype = None
        L.oracle_resid_dd.argtypes = [ctypes.c_int, llp, ip, dp, dp, dp, dp]
        L.oracle_resid_dd.restype = None
        sp = ctypes.POINTER(ctypes.c_byte)
        brm = [ctypes.c_int, dp, ip, ip, dp, dp, sp, ip]
        L.oracle_br_assemble.argtypes = [ctypes.c_void_p] + brm + [ctypes.c_double, dp, ctypes.c_double]
        L.oracle_br_assemble.restype = ctypes.c_int
        L.oracle_br_rhs.argtypes = [dp] + brm + [dp, ctypes.c_int, ctypes.c_double, ctypes.c_int]
        L.oracle_br_rhs.restype = ctypes.c_int
        L.oracle_br_rhs_recon.argtypes = [dp] + brm + [dp, ctypes.c_int, ctypes.c_double, ctypes.c_int, ctypes.c_int]
        L.oracle_br_rhs_recon.restype = ctypes.c_int
        L.oracle_br_div.argtypes = brm + [dp, dp, dp, dp]
        L.oracle_br3_assemble.argtypes = [ctypes.c_void_p] + brm + [ctypes.c_double, dp, ctypes.c_double]
        L.oracle_br3_assemble.restype = ctypes.c_int
        L.oracle_br3_rhs.argtypes = [dp] + brm + [dp, ctypes.c_int, ctypes.c_double, ctypes.c_int]
        L.oracle_br3_rhs.restype = ctypes.c_int
        L.oracle_br3_div.argtypes = brm + [dp, dp, dp, dp]
        L.oracle_br3_rhs_recon.argtypes = [dp] + brm + [dp, ctypes.c_int, ctypes.c_double, ctypes.c_int, ctypes.c_int]
        L.oracle_br3_rhs_recon.restype = ctypes.c_int
        L.oracle_br3_bdm1_moments.argtypes = [dp, dp, ctypes.c_int, ctypes.c_int, ctypes.c_int, dp]
        L.oracle_br3_recon_l2error.argtypes = brm + [dp, dp, ctypes.c_int, ctypes.c_int, ctypes.c_int]
        L.oracle_br3_recon_l2error.restype = ctypes.c_double
        brm_nocd = brm[:-1]
        L.oracle_p2b_coeffs.argtypes = brm_nocd + [ctypes.c_int, dp]
        L.oracle_p2b_coeffs.restype = None
        L.oracle_p2b_rhs_recon.argtypes = [dp] + brm + [dp, ctypes.c_int, ctypes.c_double, ctypes.c_int, ctypes.c_int]
        L.oracle_p2b_rhs_recon.restype = ctypes.c_int
        L.oracle_p2b_stokes.argtypes = [ctypes.c_void_p, ctypes.c_int, dp, ip, ip, ctypes.c_double, dp]
        L.oracle_p2b_stokes.restype = ctypes.c_int
        L.oracle_p2b_recon_l2error.argtypes = brm + [dp, dp, ctypes.c_int, ctypes.c_int, ctypes.c_int]
        L.oracle_p2b_recon_l2error.restype = ctypes.c_double
        L.oracle_nl_assemble.argtypes = [ctypes.c_void_p, dp, ctypes.c_int, dp, ctypes.c_int, ip, ctypes.c_int,
                                         ctypes.c_int, ip, dp, ctypes.c_int, ctypes.c_double, ctypes.c_double,
                                         ctypes.c_double, ctypes.c_int]
        L.oracle_nl_assemble.restype = ctypes.c_int
        L.oracle_face_jumpgrad.argtypes = [ctypes.c_void_p, ctypes.c_int, dp, ctypes.c_int, ip, ip, ctypes.c_int,
                                           ctypes.c_int, ip, ctypes.c_double, ctypes.c_double, ctypes.c_int]
        L.oracle_face_jumpgrad.restype = ctypes.c_int
        L.oracle_face_jumps.argtypes = [ctypes.c_int, dp, ctypes.c_int, ip, ip, ctypes.c_int, dp, dp, ctypes.c_int,
                                        ip, dp, ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.c_int, dp]
        L.oracle_face_jumps.restype = ctypes.c_int
    return _lib


def _dp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _ip(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_int))


def _llp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_longlong))


# --------------------------------------------------------------------------
# quadrature and bases
# --------------------------------------------------------------------------

def qrule(dim: int, order: int):
    """(xref (n, 3), w (n,), exact_reference_rule: bool)."""
    x = np.zeros(3 * 128)
    w = np.zeros(128)
    n = lib().oracle_qrule(dim, order, _dp(x), _dp(w))
    if n == 0:
        raise ValueError(f"no quadrature rule dim={dim} order={order}")
    return x[: 3 * abs(n)].reshape(-1, 3).copy(), w[: abs(n)].copy(), n > 0


def basis_tables(fe: int, dim: int, xref: np.ndarray):
    nq = xref.shape[0]
    nb = (dim + 1) if fe == FE_P1 else (6 if dim == 2 else 10)
    vals = np.zeros(nq * nb)
    der = np.zeros(nq * nb * dim)
    x3 = np.zeros((nq, 3))
    x3[:, : xref.shape[1]] = xref
    x = np.ascontiguousarray(x3, dtype=np.float64).ravel()
    lib().oracle_basis_tables(fe, dim, nq, _dp(x), _dp(vals), _dp(der))
    return vals.reshape(nq, nb), der.reshape(nq, nb, dim)


# --------------------------------------------------------------------------
# DoF maps, restated from src/dofmaps.jl:201-330 (patterns N1, N1F1, N1E1)
# --------------------------------------------------------------------------

def _enumerate_entities(cells: np.ndarray, local: np.ndarray):
    loc = np.sort(cells[:, local], axis=2).reshape(-1, local.shape[1])
    uniq, inv = np.unique(loc, axis=0, return_inverse=True)
    return uniq, inv.reshape(cells.shape[0], local.shape[0])


def celldofs(fe: int, ncomp: int, dim: int, nverts: int, cells: np.ndarray):
    """(celldofs (ncells, ldofs) int32, ndofs, coffset) for H1P1 / H1P2."""
    if fe == FE_P1:
        coffset = nverts
        items = [cells]
    else:
        if dim == 2:
            local = np.array([[0, 1], [1, 2], [2, 0]])
        else:
            local = np.array([[0, 1], [0, 2], [0, 3], [1, 2], [1, 3], [2, 3]])
        ents, cent = _enumerate_entities(cells, local)
        coffset = nverts + ents.shape[0]
        items = [cells, cent + nverts]
    cols = []
    for c in range(ncomp):
        for it in items:
            cols.append(it.astype(np.int64) + c * coffset)
    return np.concatenate(cols, axis=1).astype(np.int32), coffset * ncomp, coffset


# --------------------------------------------------------------------------
# assembly
# --------------------------------------------------------------------------

class Matrix:
    """Sparse accumulator with the reference's accumulation order and the
    drop-exact-zero rule of _addnz."""

    def __init__(self, n: int):
        self.n = n
        self.h = lib().oracle_mat_new(n)

    def __del__(self):
        if getattr(self, "h", None):
            lib().oracle_mat_free(self.h)
            self.h = None

    def add_bilinear(self, coords, cells, fe, ncomp, cdofs, op, symmetric, factor=1.0, action=ACT_NONE,
                     cellcoef=None, mu=0.0, lam=0.0, bonus_quadorder=0):
        coords = np.ascontiguousarray(coords, dtype=np.float64)
        cells = np.ascontiguousarray(cells, dtype=np.int32)
        cdofs = np.ascontiguousarray(cdofs, dtype=np.int32)
        dim = coords.shape[1]
        cc = np.ascontiguousarray(cellcoef if cellcoef is not None else np.zeros(1), dtype=np.float64)
        nq = lib().oracle_assemble_bilinear(self.h, dim, coords.shape[0], _dp(coords), cells.shape[0], _ip(cells),
                                            fe, ncomp, _ip(cdofs), op, int(symmetric), float(factor), action,
                                            _dp(cc), float(mu), float(lam), int(bonus_quadorder))
        if nq < 0:
            raise RuntimeError("oracle bilinear assembly failed")
        return nq

    def penalize(self, fixed, penalty=1e60):
        f = np.ascontiguousarray(fixed, dtype=np.int32)
        lib().oracle_mat_penalize(self.h, f.shape[0], _ip(f), float(penalty))

    def csr(self):
        import scipy.sparse as sp
        nnz = lib().oracle_mat_nnz(self.h)
        rp = np.zeros(self.n + 1, dtype=np.int64)
        ci = np.zeros(nnz, dtype=np.int32)
        v = np.zeros(nnz)
        lib().oracle_mat_csr(self.h, _llp(rp), _ip(ci), _dp(v))
        return sp.csr_matrix((v, ci, rp), shape=(self.n, self.n))


def assemble_linear(b, coords, cells, fe, ncomp, cdofs, rhs_kind, params, factor=1.0, bonus_quadorder=0):
    coords = np.ascontiguousarray(coords, dtype=np.float64)
    cells = np.ascontiguousarray(cells, dtype=np.int32)
    cdofs = np.ascontiguousarray(cdofs, dtype=np.int32)
    par = np.ascontiguousarray(params, dtype=np.float64).ravel()
    if par.size == 0:
        par = np.zeros(1)
    assert b.dtype == np.float64 and b.flags.c_contiguous
    nq = lib().oracle_assemble_linear(_dp(b), coords.shape[1], coords.shape[0], _dp(coords), cells.shape[0],
                                      _ip(cells), fe, ncomp, _ip(cdofs), rhs_kind, _dp(par), par.size,
                                      float(factor), int(bonus_quadorder))
    if nq < 0:
        raise RuntimeError("oracle linear assembly failed")
    return b


# --------------------------------------------------------------------------
# ItemIntegrator (src/assemblypatterns/itemintegrator.jl)
# --------------------------------------------------------------------------

OP_IDENTITY, OP_GRADIENT = 0, 1


def item_l2error(coords, cells, fe, ncomp, cdofs, u, op=OP_IDENTITY, data_kind=-1, params=None, factor=1.0,
                 quadorder=0, v=None):
    """L2ErrorIntegrator / L2NormIntegrator (data_kind -1) / L2DifferenceIntegrator (v given) over all
    cells; returns (per-cell values, total), the total summed in the reference's order."""
    coords = np.ascontiguousarray(coords, dtype=np.float64)
    cells = np.ascontiguousarray(cells, dtype=np.int32)
    cdofs = np.ascontiguousarray(cdofs, dtype=np.int32)
    u = np.ascontiguousarray(u, dtype=np.float64)
    par = np.zeros(1) if params is None else np.ascontiguousarray(params, dtype=np.float64).ravel()
    if par.size == 0:
        par = np.zeros(1)
    cellv = np.zeros(cells.shape[0])
    total = np.zeros(1)
    vp = None
    if v is not None:
        v = np.ascontiguousarray(v, dtype=np.float64)
        vp = _dp(v)
    nq = lib().oracle_item_l2error(_dp(cellv), _dp(total), coords.shape[1], coords.shape[0], _dp(coords),
                                   cells.shape[0], _ip(cells), fe, ncomp, _ip(cdofs), _dp(u), vp, op, data_kind,
                                   _dp(par), par.size, float(factor), int(quadorder))
    if nq < 0:
        raise RuntimeError("oracle item integrator failed")
    return cellv, float(total[0])


def item_l2error_br(g, cdofs, u, op=OP_IDENTITY, data_kind=-1, params=None, factor=1.0, quadorder=0, v=None):
    """The same integrators on an H1BR{dim} function over the mesh g (its
    faces and face normals as the host mesh module numbers them)."""
    fn, cf = g.faces()
    nrm, _, _ = g.face_geometry()
    coords = np.ascontiguousarray(g.coords, dtype=np.float64)
    cells = np.ascontiguousarray(g.cells, dtype=np.int32)
    cf = np.ascontiguousarray(cf, dtype=np.int32)
    nrm = np.ascontiguousarray(nrm, dtype=np.float64)
    cdofs = np.ascontiguousarray(cdofs, dtype=np.int32)
    u = np.ascontiguousarray(u, dtype=np.float64)
    par = np.zeros(1) if params is None else np.ascontiguousarray(params, dtype=np.float64).ravel()
    if par.size == 0:
        par = np.zeros(1)
    cellv = np.zeros(g.ncells)
    total = np.zeros(1)
    vp = None
    if v is not None:
        v = np.ascontiguousarray(v, dtype=np.float64)
        vp = _dp(v)
    nq = lib().oracle_item_l2error_br(_dp(cellv), _dp(total), g.dim, g.ncells, _dp(coords), _ip(cells), _ip(cf),
                                      _dp(nrm), _ip(cdofs), _dp(u), vp, op, data_kind, _dp(par), par.size,
                                      float(factor), int(quadorder))
    if nq < 0:
        raise RuntimeError("oracle BR item integrator failed")
    return cellv, float(total[0])


# --------------------------------------------------------------------------
# solve (src/solvers.jl:622-686)
# --------------------------------------------------------------------------

def penalized_rhs(b, fixed, values=None, penalty=1e60):
    b = b.copy()
    if values is None:
        b[fixed] = 0.0
    else:
        b[fixed] = penalty * values
    return b


def solve_direct(A, b):
    """FP64 sparse-direct solve (SuperLU standing in for UMFPACK)."""
    import scipy.sparse.linalg as spla
    return spla.spsolve(A.tocsc(), b)


def set_threads(n: int):
    """Threads of the oracle's OpenMP regions (n <= 0: all processors)."""
    lib().oracle_set_threads(int(n))


def solve_cg(A, b, reltol=1e-14, maxit=100000):
    """FP64 Jacobi-CG of grmp_oracle.c (OpenMP); returns (x, iters, relres)."""
    A = A.tocsr()
    n = A.shape[0]
    rp = np.ascontiguousarray(A.indptr, dtype=np.int64)
    ci = np.ascontiguousarray(A.indices, dtype=np.int32)
    v = np.ascontiguousarray(A.data, dtype=np.float64)
    bb = np.ascontiguousarray(b, dtype=np.float64)
    x = np.zeros(n)
    rr = ctypes.c_double(0)
    it = lib().oracle_cg(n, _llp(rp), _ip(ci), _dp(v), _dp(bb), _dp(x), reltol, maxit, ctypes.byref(rr))
    return x, it, rr.value


def resid_dd(A, x, b):
    """b - A x with every row sum carried in double-double (grmp_oracle.c
    oracle_resid_dd), rounded once to FP64."""
    A = A.tocsr()
    rp = np.ascontiguousarray(A.indptr, dtype=np.int64)
    ci = np.ascontiguousarray(A.indices, dtype=np.int32)
    v = np.ascontiguousarray(A.data, dtype=np.float64)
    xx = np.ascontiguousarray(x, dtype=np.float64)
    bb = np.ascontiguousarray(b, dtype=np.float64)
    r = np.empty(A.shape[0])
    lib().oracle_resid_dd(A.shape[0], _llp(rp), _ip(ci), _dp(v), _dp(xx), _dp(bb), _dp(r))
    return r


def solve_refined(A, b, inner_reltol=1e-10, max_refine=8, maxit=200000, x0=None):
    """FP64 solution of A x = b accurate to about the FP64 rounding of x, for
    systems too large for a sparse-direct factorisation here: iterative
    refinement whose residual is computed in double-double (resid_dd) and
    whose corrections come from the FP64 Jacobi-CG of grmp_oracle.c, until a
    correction is below 2 ulp of the solution norm.  With an extra-precise
    residual the limiting accuracy does not grow with the condition number
    (it needs only cond(A) * inner_reltol < 1).  x0: a starting solution
    (e.g. an FP64 CG solve of the same system).  Returns (x, info) with
    info = {"refinements", "cg_iterations", "last_correction", "relres"};
    last_correction is ||dx|| / ||x|| of the final step, an estimate of the
    remaining relative error."""
    A = A.tocsr()
    b = np.ascontiguousarray(b, dtype=np.float64)
    x = np.zeros(A.shape[0]) if x0 is None else np.array(x0, dtype=np.float64)
    bn = max(np.linalg.norm(b), 1e-300)
    its, corr, k = [], 1.0, 0
    for k in range(1, max_refine + 1):
        r = resid_dd(A, x, b)
        d, it, _ = solve_cg(A, r, inner_reltol, maxit)
        its.append(it)
        x = x + d
        corr = float(np.linalg.norm(d) / max(np.linalg.norm(x), 1e-300))
        if corr <= 4.5e-16:
            break
    relres = float(np.linalg.norm(resid_dd(A, x, b)) / bn)
    return x, {"refinements": k, "cg_iterations": its, "last_correction": corr, "relres": relres}


if __name__ == "__main__":  # pragma: no cover - manual build helper
    print(build(force="--force" in sys.argv))


# --------------------------------------------------------------------------
# Bernardi-Raugel / P0 Stokes with the RT0 reconstruction (2D)
# --------------------------------------------------------------------------

def br_celldofs(nverts: int, cells: np.ndarray, cell_faces: np.ndarray):
    """H1BR{d} cell DoFs, pattern "N1f1" (src/fedefs/h1v_br.jl:33) restated
    from src/dofmaps.jl:201-330: the nodes of each component, then faces."""
    nf = int(cell_faces.max()) + 1
    dim = cells.shape[1] - 1
    cd = np.concatenate([cells + c * nverts for c in range(dim)] + [cell_faces + dim * nverts], axis=1).astype(np.int32)
    return np.ascontiguousarray(cd), dim * nverts + nf


def _br_args(g, cd):
    fn, cf = g.faces()
    nrm, fv, sg = g.face_geometry()
    arrs = [np.ascontiguousarray(g.coords, dtype=np.float64), np.ascontiguousarray(g.cells, dtype=np.int32),
            np.ascontiguousarray(cf, dtype=np.int32), np.ascontiguousarray(nrm, dtype=np.float64),
            np.ascontiguousarray(fv, dtype=np.float64), np.ascontiguousarray(sg, dtype=np.int8),
            np.ascontiguousarray(cd, dtype=np.int32)]
    ptrs = [g.ncells, _dp(arrs[0]), _ip(arrs[1]), _ip(arrs[2]), _dp(arrs[3]), _dp(arrs[4]),
            arrs[5].ctypes.data_as(ctypes.POINTER(ctypes.c_byte)), _ip(arrs[6])]
    return arrs, ptrs


RECON_RT0, RECON_BDM1 = 1, 2


def br_stokes_system(g, nu: float, lam: float, terms, bonus_quadorder: int = 2, recon: int = RECON_RT0):
    # (2D: H1BR{2} with RT0 or BDM1; 3D: H1BR{3} with RT0 or BDM1)
    """(A (penalised), bf, fixed, celldofs) of the velocity update system:
    nu (grad u, grad v) + lam (div R u, div R v) = (f, R_rhs v), R_rhs the
    BR->RT0 (recon 1) or BR->BDM1 (recon 2) reconstruction (the penalty uses
    the RT0 divergence: the BDM1 functions beyond RT0 carry no flux, so the
    divergence of either reconstruction is the same cell constant)."""
    fn, cf = g.faces()
    cd, nd = br_celldofs(g.nverts, g.cells, cf)
    arrs, ptrs = _br_args(g, cd)
    M = Matrix(nd)
    bf = np.zeros(nd)
    par = np.ascontiguousarray(terms, dtype=np.float64).ravel()
    if g.dim == 3:
        lib().oracle_br3_assemble(M.h, *ptrs, float(nu), None, float(lam))
        if lib().oracle_br3_rhs_recon(_dp(bf), *ptrs, _dp(par), par.size, 1.0, int(bonus_quadorder), int(recon)) < 0:
            raise RuntimeError("oracle: no tetrahedral rule of that order")
    else:
        lib().oracle_br_assemble(M.h, *ptrs, float(nu), None, float(lam))
        lib().oracle_br_rhs_recon(_dp(bf), *ptrs, _dp(par), par.size, 1.0, int(bonus_quadorder), int(recon))
    # homogeneous Dirichlet on all boundary faces: nodes (every component) and face bubbles
    bf_ids = np.nonzero(np.bincount(cf.ravel(), minlength=fn.shape[0]) == 1)[0]
    bnodes = np.unique(fn[bf_ids].ravel())
    fixed = np.unique(np.concatenate([bnodes + c * g.nverts for c in range(g.dim)] +
                                     [bf_ids + g.dim * g.nverts])).astype(np.int32)
    return M, bf, fixed, cd, (arrs, ptrs)


def br3_recon_l2error(g, u, terms, recon: int = RECON_BDM1, order: int = 4) -> float:
    """L2 error ||R u - f|| of an H1BR{3} function's reconstruction (RT0 or
    BDM1) against polynomial data f (terms (component, coef, e1, e2, e3))."""
    fn, cf = g.faces()
    cd, nd = br_celldofs(g.nverts, g.cells, cf)
    _, ptrs = _br_args(g, cd)
    par = np.ascontiguousarray(terms, dtype=np.float64).ravel()
    uu = np.ascontiguousarray(u, dtype=np.float64)
    e2 = lib().oracle_br3_recon_l2error(*ptrs, _dp(uu), _dp(par), par.size, int(recon), int(order))
    if e2 < 0:
        raise RuntimeError("oracle: no tetrahedral rule of that order")
    return float(np.sqrt(e2))


def br_div(g, cd_args, u=None, p=None):
    """(cell averages of div u, int p div phi as a vector)."""
    arrs, ptrs = cd_args
    nc = g.ncells
    nd = int(arrs[6].max()) + 1
    divu = np.zeros(nc) if u is not None else None
    b = np.zeros(nd) if p is not None else None
    uu = np.ascontiguousarray(u, dtype=np.float64) if u is not None else None
    pp = np.ascontiguousarray(p, dtype=np.float64) if p is not None else None
    fn = lib().oracle_br3_div if arrs[1].shape[1] == 4 else lib().oracle_br_div
    fn(*ptrs, _dp(uu) if uu is not None else None, _dp(pp) if pp is not None else None,
       _dp(divu) if divu is not None else None, _dp(b) if b is not None else None)
    return divu, b


def stokes_iterated_penalty(g, nu: float, lam: float, terms, sweeps: int = 6, recon: int = RECON_RT0,
                            bonus_quadorder: int = 2, u_boundary=None):
    """Iterated penalty (examples/Example221_StokesIterated2D.jl:61-95, no
    convection): sparse-direct velocity solves of the penalised system,
    P0 pressure update p <- p - lam * avg(div u), zero mean.  u_boundary:
    optional full-length vector whose entries at the boundary DoFs are the
    Dirichlet values, imposed in the reference's penalty form (A[d,d] = 1e60,
    b[d] = 1e60 u_D, src/solvers.jl:640-652); None = homogeneous."""
    import scipy.sparse.linalg as spla
    M, bf, fixed, cd, args = br_stokes_system(g, nu, lam, terms, bonus_quadorder=bonus_quadorder, recon=recon)
    M.penalize(fixed)
    A = M.csr().tocsc()
    lu = spla.splu(A)
    vol = g.cell_volumes()
    p = np.zeros(g.ncells)
    u = None
    for _ in range(sweeps):
        _, bp = br_div(g, args, p=p)
        b = bf + bp
        b[fixed] = 0.0 if u_boundary is None else 1e60 * np.asarray(u_boundary, dtype=np.float64)[fixed]
        u = lu.solve(b)
        divu, _ = br_div(g, args, u=u)
        p = p - lam * divu
        p -= np.dot(vol, p) / vol.sum()
    return u, p, fixed


# --------------------------------------------------------------------------
# H1P2B{2,2} with the RT1 / BDM2 reconstructions (2D)
# --------------------------------------------------------------------------

RECON_RT1, RECON_BDM2 = 3, 4


def p2b_celldofs(g):
    """H1P2B{2,2} cell DoFs, pattern "N1F1I1" per component
    (src/fedefs/h1_p2b.jl:33), components blocked as in src/dofmaps.jl:201-330:
    nodes, faces, then the cell of component 1, then those of component 2."""
    fn, cf = g.faces()
    nf = fn.shape[0]
    nd1 = g.nverts + nf + g.ncells
    one = np.concatenate([g.cells, cf + g.nverts, (np.arange(g.ncells) + g.nverts + nf)[:, None]], axis=1)
    cd = np.concatenate([one, one + nd1], axis=1).astype(np.int32)
    return np.ascontiguousarray(cd), 2 * nd1


def p2b_coefficients(g, recon: int = RECON_RT1):
    """Reconstruction coefficients [ncells][14][12] (columns past 8 zero for RT1)."""
    fn, cf = g.faces()
    cd, _ = p2b_celldofs(g)
    _, ptrs = _br_args(g, cd)
    out = np.zeros((g.ncells, 14, 12))
    lib().oracle_p2b_coeffs(*ptrs[:-1], int(recon), _dp(out))
    return out


def p2b_rhs(g, terms, recon: int = RECON_RT1, bonus_quadorder: int = 0, factor: float = 1.0):
    """(f, R v) over H1P2B{2,2} with R = RT1 (recon 3) or BDM2 (recon 4)."""
    cd, nd = p2b_celldofs(g)
    _, ptrs = _br_args(g, cd)
    b = np.zeros(nd)
    par = np.ascontiguousarray(terms, dtype=np.float64).ravel()
    if lib().oracle_p2b_rhs_recon(_dp(b), *ptrs, _dp(par), par.size, float(factor), int(bonus_quadorder),
                                  int(recon)) < 0:
        raise RuntimeError("oracle: no triangle rule of that order")
    return b


def p2b_recon_l2error(g, u, terms, recon: int = RECON_RT1, order: int = 6) -> float:
    """||R u - f||_L2 of an H1P2B{2,2} vector against polynomial data."""
    cd, _ = p2b_celldofs(g)
    _, ptrs = _br_args(g, cd)
    par = np.ascontiguousarray(terms, dtype=np.float64).ravel()
    uu = np.ascontiguousarray(u, dtype=np.float64)
    e2 = lib().oracle_p2b_recon_l2error(*ptrs, _dp(uu), _dp(par), par.size, int(recon), int(order))
    if e2 < 0:
        raise RuntimeError("oracle: no triangle rule of that order")
    return float(np.sqrt(max(e2, 0.0)))


def p2b_stokes(g, nu: float, terms, recon: int, u_boundary, bonus_quadorder: int = 0):
    """Stokes with H1P2B{2,2} velocity and broken P1 pressure (the
    reference's p-robust catalogue entries, test/runtests.jl:684-723):
    nu (grad u, grad v) - (p, div v) = (f, R v), (q, div u) = 0, mean(p) = 0,
    velocity Dirichlet data u_boundary on every boundary DoF (nodes and edge
    midpoints of boundary faces); sparse LU of the saddle-point matrix.
    Returns (u, p)."""
    import scipy.sparse as sp
    import scipy.sparse.linalg as spla
    cd, nd = p2b_celldofs(g)
    M = Matrix(nd)
    Bloc = np.zeros((g.ncells, 3, 14))
    lib().oracle_p2b_stokes(M.h, g.ncells, _dp(np.ascontiguousarray(g.coords, dtype=np.float64)),
                            _ip(np.ascontiguousarray(g.cells, dtype=np.int32)), _ip(cd), float(nu), _dp(Bloc))
    A = M.csr()
    npres = 3 * g.ncells
    rows = np.repeat(np.arange(npres), 14)
    cols = np.tile(cd, (1, 3)).reshape(g.ncells, 3, 14).reshape(-1)
    B = sp.csr_matrix((Bloc.reshape(-1), (rows, cols)), shape=(npres, nd))
    vol = g.cell_volumes()
    mean = sp.csr_matrix(np.repeat(vol / 3.0, 3)[None, :])       # int of each barycentric function
    K = sp.bmat([[A, -B.T, None], [-B, None, mean.T], [None, mean, None]], format="csr")
    rhs = np.concatenate([p2b_rhs(g, terms, recon, bonus_quadorder), np.zeros(npres + 1)])
    fn, cf = g.faces()
    bfaces = np.nonzero(np.bincount(cf.ravel(), minlength=fn.shape[0]) == 1)[0]
    bnodes = np.unique(fn[bfaces].ravel())
    nd1 = nd // 2
    fixed = np.unique(np.concatenate([bnodes + c * nd1 for c in range(2)] +
                                     [bfaces + g.nverts + c * nd1 for c in range(2)]))
    ub = np.asarray(u_boundary, dtype=np.float64)
    free = np.setdiff1d(np.arange(K.shape[0]), fixed)
    x = np.zeros(K.shape[0])
    x[fixed] = ub[fixed]
    rr = rhs - K @ x
    Kff = K[free][:, free].tocsc()
    x[free] = spla.splu(Kff).solve(rr[free])
    return x[:nd], x[nd:nd + npres]


def p2b_interpolant(g, field):
    """P2B DoF vector of a vector field with values at the vertices and edge
    midpoints (its P2 Lagrange interpolant) and zero bubbles; exact for
    quadratic fields up to the bubble part."""
    fn, cf = g.faces()
    nd1 = g.nverts + fn.shape[0] + g.ncells
    vv = field(g.coords)
    mid = field(0.5 * (g.coords[fn[:, 0]] + g.coords[fn[:, 1]]))
    u = np.zeros(2 * nd1)
    for c in range(2):
        u[c * nd1: c * nd1 + g.nverts] = vv[:, c]
        u[c * nd1 + g.nverts: c * nd1 + g.nverts + fn.shape[0]] = mid[:, c]
    return u


# --------------------------------------------------------------------------
# NonlinearForm Newton terms and the Newton loop (src/solvers.jl:519-566)
# --------------------------------------------------------------------------

NL_DIFFUSION, NL_GRAD_DIFFUSION, NL_CONVECTION = 1, 2, 3


def nl_assemble(M, b, coords, cells, fe, ncomp, cdofs, u, kind, factor=1.0, kappa=1.0, beta=1.0,
                bonus_quadorder=0):
    """Adds DG(u) into the accumulator M and DG(u) u - G(u) into b."""
    dim = coords.shape[1]
    uu = np.ascontiguousarray(u, dtype=np.float64)
    nq = lib().oracle_nl_assemble(M.h, _dp(b), dim, _dp(np.ascontiguousarray(coords, dtype=np.float64)),
                                  cells.shape[0], _ip(np.ascontiguousarray(cells, dtype=np.int32)), int(fe), int(ncomp),
                                  _ip(np.ascontiguousarray(cdofs, dtype=np.int32)), _dp(uu), int(kind), float(factor),
                                  float(kappa), float(beta), int(bonus_quadorder))
    if nq < 0:
        raise RuntimeError("oracle: no rule of that order")
    return b


def newton_nonlinear_poisson(coords, cells, fe, cdofs, nd, f_terms, fixed, kind=NL_DIFFUSION, kappa=1.0, beta=1.0,
                             bonus_quadorder=2, rhs_bonus=0, maxit=20, tol=1e-12, u0=None):
    """Newton iteration of G(u) = (f, v) with homogeneous Dirichlet DoFs
    `fixed`: each step assembles DG(u), DG(u) u - G(u) + (f, v), imposes the
    Dirichlet DoFs in the reference's penalty form and solves with a sparse
    LU (the reference's default linear solver); stops when the update's
    norm drops below tol times the iterate's.  Returns (u, iterates)."""
    import scipy.sparse.linalg as spla
    dim = coords.shape[1]
    f = np.zeros(nd)
    assemble_linear(f, coords, cells, fe, 1, cdofs, RHS_POLY, np.asarray(f_terms, dtype=np.float64).ravel(), 1.0,
                    rhs_bonus)
    u = np.zeros(nd) if u0 is None else np.array(u0, dtype=np.float64)
    its = []
    for _ in range(maxit):
        M = Matrix(nd)
        b = f.copy()
        nl_assemble(M, b, coords, cells, fe, 1, cdofs, u, kind, 1.0, kappa, beta, bonus_quadorder)
        M.penalize(fixed)
        A = M.csr().tocsc()
        b[fixed] = 0.0
        un = spla.spsolve(A, b)
        its.append(un)
        done = np.linalg.norm(un - u) <= tol * max(np.linalg.norm(un), 1e-300)
        u = un
        if done:
            break
    return u, its


# --------------------------------------------------------------------------
# Interior-face terms with Jump(Gradient)
# --------------------------------------------------------------------------

def face_jumpgrad(M, g, fe, cdofs, factor=1.0, power=2.0, bonus_quadorder=0):
    """Adds factor |F| |F|^power int_F [grad u].[grad v] over interior faces to M."""
    fn, cf = g.faces()
    nq = lib().oracle_face_jumpgrad(M.h, g.dim, _dp(np.ascontiguousarray(g.coords, dtype=np.float64)), g.ncells,
                                    _ip(np.ascontiguousarray(g.cells, dtype=np.int32)),
                                    _ip(np.ascontiguousarray(cf, dtype=np.int32)), fn.shape[0], int(fe),
                                    _ip(np.ascontiguousarray(cdofs, dtype=np.int32)), float(factor), float(power),
                                    int(bonus_quadorder))
    if nq < 0:
        raise RuntimeError("oracle: no face rule of that order")


def face_jumps(g, fe, cdofs, u, kind=1, power=1.0, factor=1.0, bonus_quadorder=0):
    """Per-face values of the Jump(Gradient) ItemIntegrator (0 on boundary faces)."""
    fn, cf = g.faces()
    nrm, fv, sg = g.face_geometry()
    out = np.zeros(fn.shape[0])
    nq = lib().oracle_face_jumps(g.dim, _dp(np.ascontiguousarray(g.coords, dtype=np.float64)), g.ncells,
                                 _ip(np.ascontiguousarray(g.cells, dtype=np.int32)),
                                 _ip(np.ascontiguousarray(cf, dtype=np.int32)), fn.shape[0],
                                 _dp(np.ascontiguousarray(nrm, dtype=np.float64)),
                                 _dp(np.ascontiguousarray(fv, dtype=np.float64)), int(fe),
                                 _ip(np.ascontiguousarray(cdofs, dtype=np.int32)),
                                 _dp(np.ascontiguousarray(u, dtype=np.float64)), int(kind), float(power), float(factor),
                                 int(bonus_quadorder), _dp(out))
    if nq < 0:
        raise RuntimeError("oracle: no face rule of that order")
    return out
