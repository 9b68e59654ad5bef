"""Host-side mirror of the reference's assembly / solve interface over the C-ABI.

Names and argument meanings follow GradientRobustMultiPhysics.jl:
``LaplaceOperator(kappa)`` (src/pdeoperators.jl:154-169),
``ReactionOperator(alpha)`` (:176-203), ``HookStiffnessOperator2D(mu, lambda)``
(:256-273), ``BilinearForm([Gradient, Gradient], action)`` (:355-396),
``LinearForm(Identity, f)`` (:659-755), ``FEMatrix`` / ``FEVector``
(src/fematrix.jl, src/fevector.jl), ``assemble!`` (src/assemblypatterns/
bilinearform.jl:92, linearform.jl:47) and ``solve!`` with a ``linsolver``
(src/solvers.jl:55, :622-686).  Every compute call goes through
libgrmp_gpu.so; nothing here computes on the CPU.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass, field
from typing import Optional, Sequence

import numpy as np

from . import _lib as L
from .fespace import FESpace, FE_H1BR, FE_H1P2B
from .mesh import SimplexMesh

# operator tags of src/functionoperators.jl
Identity = "Identity"
Gradient = "Gradient"
SymmetricGradient = "SymmetricGradient"
Divergence = "Divergence"
ReconstructionIdentity = "ReconstructionIdentity"          # ReconstructionIdentity{HDIVRT0{d}}
ReconstructionIdentityBDM1 = "ReconstructionIdentity{HDIVBDM1}"   # ReconstructionIdentity{HDIVBDM1{d}}
ReconstructionIdentityRT1 = "ReconstructionIdentity{HDIVRT1}"     # ReconstructionIdentity{HDIVRT1{2}} (H1P2B)
ReconstructionIdentityBDM2 = "ReconstructionIdentity{HDIVBDM2}"   # ReconstructionIdentity{HDIVBDM2{2}} (H1P2B)
ReconstructionDivergence = "ReconstructionDivergence"


def Jump(op: str) -> str:
    """Jump(op) of src/functionoperators.jl:187: op|T1 - op|T2 across a face."""
    return f"Jump({op})"


# assembly types (src/assemblypatterns.jl)
ON_CELLS = "ON_CELLS"
ON_IFACES = "ON_IFACES"

APT_BilinearForm = "APT_BilinearForm"
APT_SymmetricBilinearForm = "APT_SymmetricBilinearForm"


def _dp(a: np.ndarray):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _ip(a: np.ndarray):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_int32))


# ----------------------------------------------------------------------- context
class GB300Context:
    """One GPU, one CUDA stream, an HBM budget.  Owns every device handle."""

    def __init__(self, device: int = 0, hbm_budget_bytes: int = 0):
        self.lib = L.load()
        h = ctypes.c_void_p()
        rc = self.lib.grmp_create_context(device, hbm_budget_bytes, ctypes.byref(h))
        if rc != L.OK:
            raise L.GrmpError(rc, "could not create a context (is a CUDA device visible?)")
        self.h = h
        self._meshes = {}
        self._spaces = {}

    def check(self, rc: int):
        L.check(rc, self.h)

    @property
    def stream(self) -> int:
        s = ctypes.c_void_p()
        self.check(self.lib.grmp_context_stream(self.h, ctypes.byref(s)))
        return s.value or 0

    def synchronize(self):
        self.check(self.lib.grmp_synchronize(self.h))

    def memory_in_use(self) -> int:
        v = ctypes.c_size_t()
        self.check(self.lib.grmp_context_memory(self.h, ctypes.byref(v)))
        return v.value

    # -- handles ------------------------------------------------------------
    def mesh(self, grid: SimplexMesh, with_faces: bool = False):
        # entries keep a strong reference to the grid so that its id() cannot
        # be reused by another object while the device copy exists
        key = id(grid)
        ent = self._meshes.get(key)
        if ent is not None and ent["grid"] is not grid:
            ent = None
        if ent is None:
            h = ctypes.c_void_p()
            coords = np.ascontiguousarray(grid.coords, dtype=np.float64)
            cells = np.ascontiguousarray(grid.cells, dtype=np.int32)
            self.check(self.lib.grmp_mesh_upload(self.h, grid.dim, grid.nverts, _dp(coords), grid.ncells, _ip(cells),
                                                 ctypes.byref(h)))
            ent = {"h": h, "grid": grid, "faces": False}
            self._meshes[key] = ent
        if with_faces and not ent["faces"]:
            fnodes, cfaces = grid.faces()
            normals, vols, signs = grid.face_geometry()
            cf = np.ascontiguousarray(cfaces, dtype=np.int32)
            nr = np.ascontiguousarray(normals, dtype=np.float64)
            fv = np.ascontiguousarray(vols, dtype=np.float64)
            sg = np.ascontiguousarray(signs, dtype=np.int8)
            self.check(self.lib.grmp_mesh_set_faces(ent["h"], fnodes.shape[0], _ip(cf), _dp(nr), _dp(fv),
                                                    sg.ctypes.data_as(ctypes.POINTER(ctypes.c_int8))))
            ent["faces"] = True
        return ent["h"]

    def space(self, FES: FESpace):
        key = id(FES)
        ent = self._spaces.get(key)
        if ent is None or ent[0] is not FES:
            mh = self.mesh(FES.xgrid, with_faces=(FES.FEType.kind in (FE_H1BR, FE_H1P2B)))
            h = ctypes.c_void_p()
            cd = np.ascontiguousarray(FES.celldofs, dtype=np.int32)
            self.check(self.lib.grmp_space_create(mh, FES.FEType.kind, FES.FEType.ncomponents, _ip(cd), FES.ndofs,
                                                  ctypes.byref(h)))
            ent = (FES, h)
            self._spaces[key] = ent
        return ent[1]

    def space_on_device(self, fetype, grid: SimplexMesh, download: bool = True) -> FESpace:
        """FESpace{FEType}(xgrid) with the dofmap built on the device
        (grmp_space_create_on_device; H1P1 / H1P2).  The returned FESpace is
        registered with this context (its device handle is reused by every
        call); with download=True its host CellDofs are filled in too."""
        mh = self.mesh(grid)
        h = ctypes.c_void_p()
        nd = ctypes.c_int32()
        self.check(self.lib.grmp_space_create_on_device(mh, fetype.kind, fetype.ncomponents, ctypes.byref(h),
                                                        ctypes.byref(nd)))
        FES = FESpace.__new__(FESpace)
        FES.FEType = fetype
        FES.xgrid = grid
        FES.name = repr(fetype)
        FES.ndofs = nd.value
        nv = grid.nverts
        FES.coffset = nv if fetype.kind == FE_H1BR else nd.value // fetype.ncomponents
        ld = ctypes.c_int()
        self.check(self.lib.grmp_space_ndofs4cell(h, ctypes.byref(ld)))
        if download:
            cd = np.empty((grid.ncells, ld.value), dtype=np.int32)
            self.check(self.lib.grmp_space_celldofs(h, _ip(cd)))
            FES.celldofs = cd
        self._spaces[id(FES)] = (FES, h)
        return FES

    def mesh_faces(self, grid: SimplexMesh, build: bool = True):
        """(cell_faces, face_normals, face_volumes, cell_face_signs) of the
        mesh on the device; build=True computes them there first
        (grmp_mesh_build_faces), as SimplexMesh.faces / face_geometry do on
        the host."""
        mh = self.mesh(grid)
        if build:
            self.check(self.lib.grmp_mesh_build_faces(mh))
        nf = ctypes.c_int32()
        self.check(self.lib.grmp_mesh_faces(mh, ctypes.byref(nf), None, None, None, None))
        cf = np.empty((grid.ncells, grid.dim + 1), dtype=np.int32)
        nr = np.empty((nf.value, grid.dim))
        fv = np.empty(nf.value)
        sg = np.empty((grid.ncells, grid.dim + 1), dtype=np.int8)
        self.check(self.lib.grmp_mesh_faces(mh, ctypes.byref(nf), _ip(cf), _dp(nr), _dp(fv),
                                            sg.ctypes.data_as(ctypes.POINTER(ctypes.c_int8))))
        return cf, nr, fv, sg

    def boundary_dofs(self, FES: FESpace) -> np.ndarray:
        """DoFs on all boundary faces, computed on the device
        (grmp_space_boundary_dofs); equal to FES.boundary_dofs()."""
        h = self.space(FES)
        n = ctypes.c_int32()
        self.check(self.lib.grmp_space_boundary_dofs(h, 0, None, ctypes.byref(n)))
        out = np.empty(max(1, n.value), dtype=np.int32)
        self.check(self.lib.grmp_space_boundary_dofs(h, out.size, _ip(out), ctypes.byref(n)))
        return out[:n.value]

    def release(self, FES: FESpace):
        """Free the device copy of a space (its mesh stays resident)."""
        ent = self._spaces.pop(id(FES), None)
        if ent is not None:
            self.lib.grmp_space_destroy(ent[1])

    def close(self):
        if getattr(self, "h", None):
            for _, h in self._spaces.values():
                self.lib.grmp_space_destroy(h)
            for ent in self._meshes.values():
                self.lib.grmp_mesh_destroy(ent["h"])
            self.lib.grmp_destroy_context(self.h)
            self.h = None
            self._spaces.clear()
            self._meshes.clear()

    def __del__(self):  # pragma: no cover
        try:
            self.close()
        except Exception:
            pass


# ----------------------------------------------------------------------- operators
@dataclass
class Operator:
    """One bilinear-form term (a PDEOperator with an APT)."""
    op_kind: int
    symmetric: bool
    factor: float = 1.0
    cell_coef: Optional[np.ndarray] = None
    params: tuple = (0.0, 0.0, 0.0, 0.0)
    bonus_quadorder: int = 0
    name: str = ""

    def term(self) -> L.BilinearTerm:
        t = L.BilinearTerm()
        t.op_kind = self.op_kind
        t.symmetric = 1 if self.symmetric else 0
        t.factor = float(self.factor)
        if self.cell_coef is not None:
            self._cc = np.ascontiguousarray(self.cell_coef, dtype=np.float64)
            t.cell_coef = _dp(self._cc)
        else:
            t.cell_coef = ctypes.POINTER(ctypes.c_double)()
        for i, v in enumerate(self.params[:4]):
            t.param[i] = float(v)
        t.bonus_quadorder = int(self.bonus_quadorder)
        return t


@dataclass
class FaceVolumePower:
    """The item-dependent action input .* |F|^power of a face form
    (Action((result, input, item) -> result .= input .* xFaceVolumes[item]^power),
    examples/Example203_ReactionConvectionDiffusion2D.jl:89-91)."""
    power: float = 2.0


@dataclass
class CellCoefficient:
    """An Action with "I" dependency: result = coef[cell] * input
    (the reference's Action(kernel, [d, d]; dependencies = "I"))."""
    values: np.ndarray
    bonus_quadorder: int = 0


def LaplaceOperator(kappa: float = 1.0, *, name: str = "auto") -> Operator:
    """a(u,v) = kappa (grad u, grad v), APT_SymmetricBilinearForm."""
    return Operator(L.OP_LAPLACE, True, float(kappa), name=name)


def ReactionOperator(alpha=1.0, *, name: str = "auto") -> Operator:
    """a(u,v) = (alpha u, v).  A number gives APT_SymmetricBilinearForm with
    factor alpha; a CellCoefficient gives the Action form (APT_BilinearForm),
    as in src/pdeoperators.jl:186-202."""
    if isinstance(alpha, CellCoefficient):
        return Operator(L.OP_MASS, False, 1.0, cell_coef=alpha.values, bonus_quadorder=alpha.bonus_quadorder,
                        name=name)
    return Operator(L.OP_MASS, True, float(alpha), name=name)


def HookStiffnessOperator2D(mu: float, lam: float, *, name: str = "auto") -> Operator:
    """a(u,v) = (C eps(u), eps(v)) with SymmetricGradient{1}, APT_BilinearForm."""
    return Operator(L.OP_HOOKE, False, 1.0, params=(mu, lam, 0.0, 0.0), name=name)


def HookStiffnessOperator3D(mu: float, lam: float, *, name: str = "auto") -> Operator:
    return Operator(L.OP_HOOKE, False, 1.0, params=(mu, lam, 0.0, 0.0), name=name)


def StructuralCoupling() -> Operator:
    """Pattern-only term that couples every local pair of a cell: include it
    in an FEMatrix's operators when a NonlinearForm's Jacobian is assembled
    into it (the Jacobian fills every local pair); it adds nothing to
    assembled values."""
    return Operator(L.OP_STRUCTURAL, False, 1.0, name="structural coupling")


def BilinearForm(operators: Sequence[str], action=None, *, APT: str = APT_BilinearForm, factor: float = 1.0,
                 AT: str = ON_CELLS, bonus_quadorder: int = 0, name: str = "auto") -> Operator:
    """BilinearForm([op, op], action) for the operator pairs on the hot path;
    AT = ON_IFACES with [Jump(Gradient), Jump(Gradient)] and a FaceVolumePower
    action (or none: power 0) is the interior-face gradient-jump form."""
    ops = tuple(operators)
    if AT == ON_IFACES:
        if ops != (Jump(Gradient), Jump(Gradient)):
            raise ValueError(f"face form {ops} is not on the GPU path")
        if action is not None and not isinstance(action, FaceVolumePower):
            raise ValueError("face forms take a FaceVolumePower action")
        power = action.power if action is not None else 0.0
        return Operator(L.OP_JUMPGRAD, True, factor, params=(power, 0.0, 0.0, 0.0), bonus_quadorder=bonus_quadorder,
                        name=name)
    if AT != ON_CELLS:
        raise ValueError(f"assembly type {AT} is not on the GPU path")
    sym = APT == APT_SymmetricBilinearForm
    cc = action.values if isinstance(action, CellCoefficient) else None
    bonus = action.bonus_quadorder if isinstance(action, CellCoefficient) else 0
    if action is not None and not isinstance(action, CellCoefficient):
        raise ValueError("supported actions: CellCoefficient")
    if ops == (Gradient, Gradient):
        return Operator(L.OP_LAPLACE, sym, factor, cell_coef=cc, bonus_quadorder=bonus, name=name)
    if ops == (Identity, Identity):
        return Operator(L.OP_MASS, sym, factor, cell_coef=cc, bonus_quadorder=bonus, name=name)
    if ops == (ReconstructionDivergence, ReconstructionDivergence):
        return Operator(L.OP_RDIVRDIV, sym, factor, cell_coef=cc, bonus_quadorder=bonus, name=name)
    raise ValueError(f"BilinearForm{ops} is not on the GPU path")


# ----------------------------------------------------------------------- data functions
@dataclass
class DataFunction:
    """Right-hand side data of the kinds the library evaluates on device."""
    kind: int
    ncomponents: int
    params: np.ndarray
    bonus_quadorder: int = 0

    @staticmethod
    def constant(values, bonus_quadorder: int = 0) -> "DataFunction":
        v = np.atleast_1d(np.asarray(values, dtype=np.float64))
        return DataFunction(L.RHS_CONST, v.size, v, bonus_quadorder)

    @staticmethod
    def cellwise(values: np.ndarray, bonus_quadorder: int = 0) -> "DataFunction":
        v = np.asarray(values, dtype=np.float64)
        nc = 1 if v.ndim == 1 else v.shape[1]
        return DataFunction(L.RHS_CELL, nc, v.reshape(-1), bonus_quadorder)

    @staticmethod
    def fourier(amplitudes, wavevectors, bonus_quadorder: int = 0) -> "DataFunction":
        a = np.asarray(amplitudes, dtype=np.float64).reshape(-1, 1)
        k = np.asarray(wavevectors, dtype=np.float64)
        return DataFunction(L.RHS_FOURIER, 1, np.concatenate([a, k], axis=1).reshape(-1), bonus_quadorder)

    @staticmethod
    def polynomial(terms, ncomponents: int, bonus_quadorder: int = 0) -> "DataFunction":
        """terms: iterable of (component, coefficient, e1, e2, e3)."""
        t = np.asarray(terms, dtype=np.float64).reshape(-1, 5)
        return DataFunction(L.RHS_POLY, ncomponents, t.reshape(-1), bonus_quadorder)


@dataclass
class LinearFormOp:
    test_operator: str
    f: DataFunction
    factor: float = 1.0

    def rhs(self) -> L.Rhs:
        r = L.Rhs()
        r.kind = self.f.kind
        r.ncomponents = self.f.ncomponents
        self._p = np.ascontiguousarray(self.f.params, dtype=np.float64)
        r.params = _dp(self._p)
        r.nparams = self._p.size
        r.factor = float(self.factor)
        r.bonus_quadorder = int(self.f.bonus_quadorder)
        r.test_operator = {ReconstructionIdentity: 1, ReconstructionIdentityBDM1: 2, ReconstructionIdentityRT1: 3,
                           ReconstructionIdentityBDM2: 4}.get(self.test_operator, 0)
        return r


def LinearForm(operator: str, f: DataFunction, *, factor: float = 1.0) -> LinearFormOp:
    return LinearFormOp(operator, f, factor)


# ----------------------------------------------------------------------- containers
class FEVector:
    """Device-resident FP64 vector over an FESpace (FEVector, src/fevector.jl)."""

    def __init__(self, ctx: GB300Context, FES: FESpace, name: str = ""):
        self.ctx = ctx
        self.FES = FES
        self.name = name
        self.h = ctypes.c_void_p()
        ctx.check(ctx.lib.grmp_vector_create(ctx.h, FES.ndofs, ctypes.byref(self.h)))

    @property
    def n(self) -> int:
        return self.FES.ndofs

    @property
    def entries(self) -> np.ndarray:
        out = np.empty(self.n, dtype=np.float64)
        self.ctx.check(self.ctx.lib.grmp_vector_download(self.h, _dp(out)))
        return out

    def upload(self, values: np.ndarray):
        v = np.ascontiguousarray(values, dtype=np.float64)
        assert v.size == self.n
        self.ctx.check(self.ctx.lib.grmp_vector_upload(self.h, _dp(v)))

    def fill(self, value: float = 0.0):
        self.ctx.check(self.ctx.lib.grmp_vector_fill(self.h, float(value)))

    def free(self):
        if self.h:
            self.ctx.lib.grmp_vector_destroy(self.h)
            self.h = None

    def __del__(self):  # pragma: no cover
        try:
            if self.ctx.h:
                self.free()
        except Exception:
            pass


def _terms(ops: Sequence[Operator]):
    arr = (L.BilinearTerm * len(ops))()
    for i, o in enumerate(ops):
        arr[i] = o.term()
    return arr


class FEMatrix:
    """Device CSR matrix over FES x FES whose sparsity pattern is the union of
    the nonzero local contributions of `operators` (drop-exact-zero rule of
    _addnz).  Built once; values assembled with assemble()."""

    def __init__(self, ctx: GB300Context, FES: FESpace, operators: Sequence[Operator], name: str = ""):
        self.ctx = ctx
        self.FES = FES
        self.operators = list(operators)
        self.name = name
        sh = ctx.space(FES)
        if any(o.op_kind == L.OP_JUMPGRAD for o in self.operators):
            ctx.mesh(FES.xgrid, with_faces=True)   # face terms need the mesh's faces
        self.h = ctypes.c_void_p()
        ctx.check(ctx.lib.grmp_pattern_build(sh, len(self.operators), _terms(self.operators), ctypes.byref(self.h)))

    def info(self):
        n = ctypes.c_int32()
        nnz = ctypes.c_int64()
        mx = ctypes.c_int32()
        self.ctx.check(self.ctx.lib.grmp_matrix_info(self.h, ctypes.byref(n), ctypes.byref(nnz), ctypes.byref(mx)))
        return n.value, nnz.value, mx.value

    @property
    def nnz(self) -> int:
        return self.info()[1]

    def pattern(self):
        n, nnz, _ = self.info()
        rp = np.empty(n + 1, dtype=np.int64)
        ci = np.empty(nnz, dtype=np.int32)
        self.ctx.check(self.ctx.lib.grmp_matrix_download(self.h, L.FP64, rp.ctypes.data_as(
            ctypes.POINTER(ctypes.c_int64)), _ip(ci), ctypes.POINTER(ctypes.c_double)()))
        return rp, ci

    def download(self, precision: int = L.FP64):
        import scipy.sparse as sp
        n, nnz, _ = self.info()
        rp = np.empty(n + 1, dtype=np.int64)
        ci = np.empty(nnz, dtype=np.int32)
        v = np.empty(nnz, dtype=np.float64)
        self.ctx.check(self.ctx.lib.grmp_matrix_download(self.h, precision, rp.ctypes.data_as(
            ctypes.POINTER(ctypes.c_int64)), _ip(ci), _dp(v)))
        return sp.csr_matrix((v, ci, rp), shape=(n, n))

    def free(self):
        if self.h:
            self.ctx.lib.grmp_matrix_destroy(self.h)
            self.h = None

    def __del__(self):  # pragma: no cover
        try:
            if self.ctx.h:
                self.free()
        except Exception:
            pass


class ImportedMatrix:
    """A matrix handed over as compressed sparse columns -- what LinearSolve
    receives from solve_direct! (SparseMatrixCSC{Float64,Int64},
    src/solvers.jl:89-101) -- imported with grmp_matrix_from_csc.  `A` is a
    scipy sparse matrix (converted to CSC) or a (colptr, rowval, nzval) triple
    with the given index base.  Rows with a diagonal >= penalty_threshold are
    the reference's penalised Dirichlet rows (eliminated for the solvers,
    grmp_solve maps b accordingly).  Solved with GB300PCG like an FEMatrix."""

    def __init__(self, ctx: GB300Context, A, symmetric: bool = True, penalty_threshold: float = 1e30,
                 index_base: int = 0):
        self.ctx = ctx
        if isinstance(A, tuple):
            colptr, rowval, nzval = A
        else:
            C = A.tocsc()
            C.sort_indices()
            colptr, rowval, nzval = C.indptr + index_base, C.indices + index_base, C.data
        self.colptr = np.ascontiguousarray(colptr, dtype=np.int64)
        rowval = np.ascontiguousarray(rowval, dtype=np.int64)
        nzval = np.ascontiguousarray(nzval, dtype=np.float64)
        self.n = self.colptr.size - 1
        self.h = ctypes.c_void_p()
        ctx.check(ctx.lib.grmp_matrix_from_csc(
            ctx.h, self.n, self.colptr.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)),
            rowval.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)), _dp(nzval), index_base, int(symmetric),
            float(penalty_threshold), ctypes.byref(self.h)))

    def update_values(self, nzval):
        """cache.A = A with the same pattern (values in the import's CSC order)."""
        v = np.ascontiguousarray(nzval, dtype=np.float64)
        self.ctx.check(self.ctx.lib.grmp_matrix_update_values(self.h, _dp(v)))

    def penalty_rows(self) -> int:
        c = ctypes.c_int32()
        self.ctx.check(self.ctx.lib.grmp_matrix_penalty_rows(self.h, ctypes.byref(c)))
        return c.value

    def free(self):
        if self.h:
            self.ctx.lib.grmp_matrix_destroy(self.h)
            self.h = None

    def __del__(self):  # pragma: no cover
        try:
            if self.ctx.h:
                self.free()
        except Exception:
            pass


def assemble(target, operators, precision: int = L.FP64):
    """assemble!(A, operators) / assemble!(b, LinearForm): device assembly.

    For an FEMatrix the values of the given precision are overwritten with the
    sum of `operators` (a list of Operator).  For an FEVector the LinearForm is
    added to the vector's current entries."""
    if isinstance(target, FEMatrix):
        ops = list(operators) if isinstance(operators, (list, tuple)) else [operators]
        target.ctx.check(target.ctx.lib.grmp_assemble_bilinear(target.h, len(ops), _terms(ops), precision))
        return target
    if isinstance(target, FEVector):
        lf = operators
        r = lf.rhs()
        sh = target.ctx.space(target.FES)
        target.ctx.check(target.ctx.lib.grmp_assemble_linear(sh, ctypes.byref(r), target.h))
        return target
    raise TypeError("assemble target must be an FEMatrix or FEVector")


# ----------------------------------------------------------------------- nonlinear forms
@dataclass
class NonlinearForm:
    """NonlinearForm(test, [operators of the iterate], kernel) for the closed
    set of kernels the device has (src/pdeoperators.jl:590-636):
    "diffusion" ((kappa + beta u^2) grad u, grad v) -- Example205's first
    form with kappa = beta = 1; "grad_diffusion" ((kappa + |grad u|^2) grad u,
    grad v) -- Example205's second form; "convection" ((u . grad) u, v) on a
    vector space -- the Navier-Stokes convection term.  Newton is the only
    linearisation, as in the reference (newton = true)."""
    kind: str = "diffusion"
    kappa: float = 1.0
    beta: float = 1.0
    factor: float = 1.0
    bonus_quadorder: int = 0

    def term(self) -> L.NonlinearTerm:
        t = L.NonlinearTerm()
        t.kind = {"diffusion": L.NL_DIFFUSION, "grad_diffusion": L.NL_GRAD_DIFFUSION,
                  "convection": L.NL_CONVECTION}[self.kind]
        t.factor = float(self.factor)
        t.param[0] = float(self.kappa)
        t.param[1] = float(self.beta)
        t.bonus_quadorder = int(self.bonus_quadorder)
        return t


def assemble_nonlinear(A: "FEMatrix", b: "FEVector", u: "FEVector", form: NonlinearForm, precision: int = L.FP64,
                       add: bool = True):
    """The Newton terms of `form` at the iterate u: DG(u) into A and
    DG(u) u - G(u) into b (added to the current values, or overwriting them
    with add=False) -- grmp_assemble_nonlinear."""
    t = form.term()
    A.ctx.check(A.ctx.lib.grmp_assemble_nonlinear(A.h, b.h, u.h, ctypes.byref(t), precision, 1 if add else 0))


def solve_nonlinear(ctx: "GB300Context", FES, operators, form: NonlinearForm, rhs, fixed, *, maxiterations: int = 20,
                    target_change: float = 1e-12, reltol: float = 1e-13, u0=None):
    """The Newton loop of solve! for a problem with linear `operators`, one
    NonlinearForm and a right-hand side, homogeneous Dirichlet DoFs `fixed`
    (src/solvers.jl:519-566, :887-990): per step the linear operators are
    assembled, the Newton terms added at the current iterate, the Dirichlet
    DoFs eliminated and the non-symmetric system solved by BiCGStab; stops when
    ||u_next - u|| <= target_change ||u_next||.  Returns (u, per-step stats)."""
    ops = list(operators)
    A = FEMatrix(ctx, FES, ops + [StructuralCoupling()])
    f = FEVector(ctx, FES)
    b = FEVector(ctx, FES)
    u = FEVector(ctx, FES)
    x = FEVector(ctx, FES)
    f.fill(0.0)
    if rhs is not None:
        assemble(f, rhs)
    fh = f.entries
    u.upload(np.zeros(FES.ndofs) if u0 is None else np.asarray(u0, dtype=np.float64))
    solver = GB300PCG(mode="bicgstab", reltol=reltol, abstol=0.0)
    stats = []
    fixed = np.ascontiguousarray(fixed, dtype=np.int32)
    try:
        for _ in range(maxiterations):
            assemble(A, ops + [StructuralCoupling()], L.FP64)
            b.upload(fh)
            assemble_nonlinear(A, b, u, form, L.FP64, add=True)
            apply_dirichlet(A, b, fixed, None, L.DIRICHLET_ELIMINATE)
            st = solver.solve(A, b, x)
            xn, un = x.entries, u.entries
            change = float(np.linalg.norm(xn - un) / max(np.linalg.norm(xn), 1e-300))
            st = dict(st, change=change)
            stats.append(st)
            u.upload(xn)
            if change <= target_change:
                break
        return u.entries, stats
    finally:
        for v in (A, f, b, u, x):
            v.free()


# ----------------------------------------------------------------------- face integrators
@dataclass
class FaceJumpIntegrator:
    """ItemIntegrator([Jump(Gradient)], action; AT = ON_IFACES): per interior
    face factor |F| |F|^power int_F g with g = ([grad u].n_F)^2 (normal=True,
    the jump part of the estimator of
    examples/Example210_PoissonLshapeAdaptive2D.jl:58-75, power 1) or
    |[grad u]|^2 -- grmp_item_face_jumps."""
    normal: bool = True
    power: float = 1.0
    factor: float = 1.0
    bonus_quadorder: int = 0

    def evaluate_faces(self, u: "FEVector") -> np.ndarray:
        ctx = u.ctx
        g = u.FES.xgrid
        ctx.mesh(g, with_faces=True)
        out = np.zeros(g.faces()[0].shape[0])
        tot = ctypes.c_double()
        ctx.check(ctx.lib.grmp_item_face_jumps(ctx.space(u.FES), u.h, 1 if self.normal else 0, float(self.power),
                                               float(self.factor), int(self.bonus_quadorder), _dp(out),
                                               ctypes.byref(tot)))
        self.last_total = tot.value
        return out

    def evaluate(self, u: "FEVector") -> float:
        self.evaluate_faces(u)
        return self.last_total


# ----------------------------------------------------------------------- item integrators
@dataclass
class ItemIntegrator:
    """L2ErrorIntegrator / L2NormIntegrator / L2DifferenceIntegrator of
    src/assemblypatterns/itemintegrator.jl (:40-158) over all cells;
    `evaluate` / `evaluate_cells` mirror evaluate (:314-330) / evaluate!
    (:173-300) and run on the device (grmp_item_l2error)."""
    operator: str
    data: Optional[DataFunction] = None
    factor: float = 1.0
    quadorder: int = -1          # -1: the reference's "auto"
    difference: bool = False

    def _call(self, u: FEVector, v: Optional[FEVector], cells: bool):
        if self.difference != (v is not None):
            raise ValueError("L2DifferenceIntegrator takes two FEVectors, the other integrators one")
        op = {Identity: L.ITEM_IDENTITY, Gradient: L.ITEM_GRADIENT}[self.operator]
        rp = None
        if self.data is not None:
            r = L.Rhs()
            r.kind = self.data.kind
            r.ncomponents = self.data.ncomponents
            par = np.ascontiguousarray(self.data.params, dtype=np.float64)
            r.params = _dp(par)
            r.nparams = par.size
            r.factor = 1.0
            r.bonus_quadorder = int(self.data.bonus_quadorder)
            rp = ctypes.byref(r)
        out = np.empty(u.FES.xgrid.ncells) if cells else None
        tot = ctypes.c_double(0.0)
        sh = u.ctx.space(u.FES)
        u.ctx.check(u.ctx.lib.grmp_item_l2error(sh, u.h, v.h if v is not None else None, op, rp, float(self.factor),
                                                int(self.quadorder), _dp(out) if cells else None,
                                                ctypes.byref(tot)))
        return out if cells else tot.value

    def evaluate(self, u: FEVector, v: Optional[FEVector] = None) -> float:
        """Sum over all cells (the squared error / norm / difference)."""
        return self._call(u, v, False)

    def evaluate_cells(self, u: FEVector, v: Optional[FEVector] = None) -> np.ndarray:
        """Per-cell values (evaluate! into a [1, ncells] array)."""
        return self._call(u, v, True)


def L2ErrorIntegrator(data: DataFunction, operator: str = Identity, *, quadorder="auto",
                      factor: float = 1.0) -> ItemIntegrator:
    return ItemIntegrator(operator, data, factor, -1 if quadorder == "auto" else int(quadorder))


def L2NormIntegrator(operator: str = Identity, *, quadorder: int = 2) -> ItemIntegrator:
    return ItemIntegrator(operator, None, 1.0, int(quadorder))


def L2DifferenceIntegrator(operator: str = Identity, *, quadorder: int = 2) -> ItemIntegrator:
    return ItemIntegrator(operator, None, 1.0, int(quadorder), difference=True)


def apply_dirichlet(A: FEMatrix, b: Optional[FEVector], fixed_dofs: np.ndarray, values=None,
                    mode: int = L.DIRICHLET_ELIMINATE, penalty: float = 1e60):
    """Dirichlet treatment of fixed DoFs: the reference's penalty form
    (fixed_penalty = 1e60, src/solvers.jl:640-652) or symmetric elimination."""
    f = np.ascontiguousarray(fixed_dofs, dtype=np.int32)
    vals = None if values is None else np.ascontiguousarray(values, dtype=np.float64)
    A.ctx.check(A.ctx.lib.grmp_apply_dirichlet(A.h, b.h if b is not None else None, f.size, _ip(f),
                                               _dp(vals) if vals is not None else ctypes.POINTER(ctypes.c_double)(),
                                               mode, float(penalty)))


@dataclass
class GB300PCG:
    """The linear solver handed to solve! as `linsolver` (the LinearSolve
    algorithm slot of default_solver_kwargs, src/solvers.jl:55).

    mode "fp64": Jacobi-PCG in FP64.  mode "mixed": FP32 Jacobi-PCG inside an
    FP64 refinement loop (FP64 residual b - A x and solution update).
    mode "direct": FP64 multifrontal Cholesky + residual refinement (the
    counterpart of the reference's sparse-direct default).  mode
    "mixed_direct": FP32 multifrontal Cholesky as the preconditioner of FP64
    conjugate gradients.  mode "bicgstab": FP64 Jacobi-preconditioned
    BiCGStab for non-symmetric matrices (Newton steps of a NonlinearForm)."""
    mode: str = "fp64"
    abstol: float = 1e-12
    reltol: float = 1e-12
    maxiter: int = 100000
    inner_reltol: float = 0.1
    max_outer: int = 1000
    spmv_config: int = 0
    grid_blocks: int = 0
    use_initial_guess: bool = False
    last_stats: dict = field(default_factory=dict)

    def params(self) -> L.SolveParams:
        p = L.SolveParams()
        p.abstol = self.abstol
        p.reltol = self.reltol
        p.maxiter = self.maxiter
        p.mode = {"fp64": L.SOLVE_FP64, "mixed": L.SOLVE_MIXED, "direct": L.SOLVE_DIRECT,
                  "mixed_direct": L.SOLVE_MIXED_DIRECT, "bicgstab": L.SOLVE_BICGSTAB}[self.mode]
        p.inner_reltol = self.inner_reltol
        p.max_outer = self.max_outer
        p.spmv_config = self.spmv_config
        p.grid_blocks = self.grid_blocks
        p.use_initial_guess = 1 if self.use_initial_guess else 0
        return p

    def solve(self, A: FEMatrix, b: FEVector, x: FEVector, raise_on_error: bool = True) -> dict:
        st = L.SolveStats()
        p = self.params()
        rc = A.ctx.lib.grmp_solve(A.h, b.h, x.h, ctypes.byref(p), ctypes.byref(st))
        self.last_stats = {"status": st.status, "iterations": st.iterations, "outer_iterations": st.outer_iterations,
                           "spmv_config": st.spmv_config, "grid_blocks": st.grid_blocks,
                           "final_relres": st.final_relres, "solve_ms": st.solve_ms, "rc": rc}
        if raise_on_error:
            A.ctx.check(rc)
        return self.last_stats


def spmv(A: FEMatrix, x: FEVector, y: FEVector, precision: int = L.FP64):
    A.ctx.check(A.ctx.lib.grmp_spmv(A.h, precision, x.h, y.h))
