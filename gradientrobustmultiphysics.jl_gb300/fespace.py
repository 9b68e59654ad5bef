"""Finite element spaces and their DoF maps (the reference's FESpace layer).

Element types mirror the reference's parametric types: ``H1P1(ncomponents)``
(src/fedefs/h1_p1.jl), ``H1P2(ncomponents, edim)`` (src/fedefs/h1_p2.jl),
``H1BR(edim)`` (src/fedefs/h1v_br.jl), ``L2P0(ncomponents)``
(src/fedefs/l2_p0.jl), ``HDIVRT0(edim)`` / ``HDIVBDM1(edim)`` as
reconstruction targets.

Global numbering follows ``init_dofmap_from_pattern!``
(src/dofmaps.jl:201-330): components are blocked with a per-component offset
``coffset`` (the number of DoFs of one component); within a component the
pattern order is nodes, then faces ("N1F1", 2D P2) or edges ("N1E1", 3D P2);
the BR face bubbles ("f1", not per component) follow all node DoFs.  Local
cell DoFs are component-major in the same pattern order, which is the row
order of the reference bases.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from .mesh import SimplexMesh, TRI_LOCAL_FACES, TET_LOCAL_EDGES, TET_LOCAL_FACES

# element kind codes shared with the C-ABI (include/grmp.h)
FE_H1P1 = 1
FE_H1P2 = 2
FE_H1BR = 3
FE_HDIVRT0 = 4
FE_HDIVBDM1 = 5
FE_L2P0 = 6
FE_H1P2B = 7
FE_HDIVRT1 = 8
FE_HDIVBDM2 = 9


@dataclass(frozen=True)
class FEType:
    kind: int
    ncomponents: int
    name: str

    def __repr__(self) -> str:
        return self.name


def H1P1(ncomponents: int = 1) -> FEType:
    return FEType(FE_H1P1, ncomponents, f"H1P1{{{ncomponents}}}")


def H1P2(ncomponents: int = 1, edim: int = 2) -> FEType:
    return FEType(FE_H1P2, ncomponents, f"H1P2{{{ncomponents},{edim}}}")


def H1BR(edim: int = 2) -> FEType:
    return FEType(FE_H1BR, edim, f"H1BR{{{edim}}}")


def H1P2B(ncomponents: int = 2, edim: int = 2) -> FEType:
    """P2 plus a cell bubble per component (src/fedefs/h1_p2b.jl; 2D vector
    fields, the reference's H1P2B{2,2})."""
    if ncomponents != 2 or edim != 2:
        raise ValueError("H1P2B is built for H1P2B{2,2}")
    return FEType(FE_H1P2B, ncomponents, f"H1P2B{{{ncomponents},{edim}}}")


def HDIVRT1(edim: int = 2) -> FEType:
    return FEType(FE_HDIVRT1, edim, f"HDIVRT1{{{edim}}}")


def HDIVBDM2(edim: int = 2) -> FEType:
    return FEType(FE_HDIVBDM2, edim, f"HDIVBDM2{{{edim}}}")


def L2P0(ncomponents: int = 1) -> FEType:
    return FEType(FE_L2P0, ncomponents, f"L2P0{{{ncomponents}}}")


def HDIVRT0(edim: int = 2) -> FEType:
    return FEType(FE_HDIVRT0, edim, f"HDIVRT0{{{edim}}}")


def HDIVBDM1(edim: int = 2) -> FEType:
    return FEType(FE_HDIVBDM1, edim, f"HDIVBDM1{{{edim}}}")


def polynomial_order(fe: FEType, dim: int) -> int:
    """get_polynomialorder for the element on a simplex of dimension dim."""
    if fe.kind == FE_H1P1:
        return 1
    if fe.kind == FE_H1P2:
        return 2
    if fe.kind == FE_H1BR:
        return 2 if dim == 2 else 3          # src/fedefs/h1v_br.jl:23-29
    if fe.kind == FE_L2P0:
        return 0
    if fe.kind == FE_HDIVRT0:
        return 1
    if fe.kind == FE_HDIVBDM1:
        return 1
    if fe.kind == FE_H1P2B:
        return 3                             # src/fedefs/h1_p2b.jl:24-26
    if fe.kind in (FE_HDIVRT1, FE_HDIVBDM2):
        return 2
    raise ValueError(fe)


class FESpace:
    """FESpace{FEType}(grid): holds the cell DoF map and boundary DoFs."""

    def __init__(self, fetype: FEType, grid: SimplexMesh, name: str = ""):
        self.FEType = fetype
        self.xgrid = grid
        self.name = name or repr(fetype)
        self._build()

    def _build(self):
        g = self.xgrid
        fe = self.FEType
        nn = g.nverts
        nc = fe.ncomponents
        if fe.kind == FE_H1P1:
            self.coffset = nn
            self.ndofs = nn * nc
            per = [g.cells.astype(np.int64) + c * nn for c in range(nc)]
            self.celldofs = np.concatenate(per, axis=1).astype(np.int32)
        elif fe.kind == FE_H1P2:
            if g.dim == 2:
                ent, cent = g.faces()[0].shape[0], g.faces()[1]
            else:
                ent, cent = g.edges()[0].shape[0], g.edges()[1]
            self.coffset = nn + ent
            self.ndofs = self.coffset * nc
            per = []
            for c in range(nc):
                off = c * self.coffset
                per.append(g.cells.astype(np.int64) + off)
                per.append(cent.astype(np.int64) + off + nn)
            self.celldofs = np.concatenate(per, axis=1).astype(np.int32)
        elif fe.kind == FE_H1BR:
            fnodes, cfaces = g.faces()
            self.coffset = nn
            self.ndofs = nn * nc + fnodes.shape[0]
            per = [g.cells.astype(np.int64) + c * nn for c in range(nc)]
            per.append(cfaces.astype(np.int64) + nc * nn)
            self.celldofs = np.concatenate(per, axis=1).astype(np.int32)
        elif fe.kind == FE_H1P2B:
            # "N1F1I1" per component: nodes, faces, then the cell bubble
            fnodes, cfaces = g.faces()
            self.coffset = nn + fnodes.shape[0] + g.ncells
            self.ndofs = self.coffset * nc
            per = []
            for c in range(nc):
                off = c * self.coffset
                per.append(g.cells.astype(np.int64) + off)
                per.append(cfaces.astype(np.int64) + off + nn)
                per.append((np.arange(g.ncells, dtype=np.int64) + off + nn + fnodes.shape[0])[:, None])
            self.celldofs = np.concatenate(per, axis=1).astype(np.int32)
        elif fe.kind == FE_L2P0:
            self.coffset = g.ncells
            self.ndofs = g.ncells * nc
            self.celldofs = np.stack([np.arange(g.ncells) + c * g.ncells for c in range(nc)], axis=1).astype(np.int32)
        elif fe.kind in (FE_HDIVRT0,):
            fnodes, cfaces = g.faces()
            self.coffset = fnodes.shape[0]
            self.ndofs = fnodes.shape[0]
            self.celldofs = cfaces.astype(np.int32)
        else:
            raise ValueError(f"unsupported element {fe}")
        self.celldofs = np.ascontiguousarray(self.celldofs)

    @property
    def ndofs4cell(self) -> int:
        return self.celldofs.shape[1]

    def boundary_dofs(self, regions=None) -> np.ndarray:
        """Sorted unique DoFs on boundary faces of the given regions (all if
        None): the BFaceDofs collection of the homogeneous-Dirichlet branch of
        boundarydata! (src/boundarydata.jl:200-260)."""
        g = self.xgrid
        fe = self.FEType
        bf, reg = g.boundary_faces()
        if regions is not None:
            bf = bf[np.isin(reg, np.asarray(regions))]
        fnodes = g.faces()[0][bf]                          # (nb, dim)
        nn = g.nverts
        out = []
        if fe.kind in (FE_H1P1, FE_H1P2, FE_H1BR, FE_H1P2B):
            for c in range(fe.ncomponents):
                out.append(fnodes.ravel().astype(np.int64) + c * self.coffset)
            if fe.kind in (FE_H1P2, FE_H1P2B):
                if g.dim == 2:
                    for c in range(fe.ncomponents):
                        out.append(bf.astype(np.int64) + nn + c * self.coffset)
                else:
                    # edges of the boundary faces
                    enodes = g.edges()[0]
                    key = enodes[:, 0].astype(np.int64) * (nn + 1) + enodes[:, 1]
                    order = np.argsort(key)
                    pairs = np.concatenate([fnodes[:, [0, 1]], fnodes[:, [0, 2]], fnodes[:, [1, 2]]])
                    pairs = np.sort(pairs, axis=1)
                    pk = pairs[:, 0].astype(np.int64) * (nn + 1) + pairs[:, 1]
                    eid = order[np.searchsorted(key[order], pk)]
                    for c in range(fe.ncomponents):
                        out.append(eid.astype(np.int64) + nn + c * self.coffset)
            if fe.kind == FE_H1BR:
                out.append(bf.astype(np.int64) + fe.ncomponents * nn)
        elif fe.kind == FE_L2P0:
            pass
        else:
            raise ValueError(fe)
        if not out:
            return np.zeros(0, dtype=np.int32)
        return np.unique(np.concatenate(out)).astype(np.int32)


# local P2 edge DoFs: the two local vertices of each edge, in the basis order of
# src/fedefs/h1_p2.jl (edge functions 4 lambda_a lambda_b)
_P2_EDGES = {2: [(0, 1), (1, 2), (2, 0)], 3: [(0, 1), (0, 2), (0, 3), (1, 2), (1, 3), (2, 3)]}


def interpolate(FES: FESpace, f, edge_points: int = 5) -> np.ndarray:
    """interpolate!(Target, FES, f) for H1P1 and H1P2 (scalar or vector) and
    H1BR (see _interpolate_br):
    vertex DoFs by point evaluation (point_evaluation!, src/fedefs/h1_p2.jl:
    47-59), P2 edge DoFs so that the interpolant keeps the mean of f on every
    edge (ensure_moments!, :61-71, :73-92), the mean taken with a Gauss rule of
    `edge_points` points.  Along an edge (a, b) the vertex functions integrate
    to |E|/6 and the edge function to 2|E|/3, so the edge DoF is
    3/2 mean_E(f) - (f(a) + f(b))/4.  f maps points (m, dim) to values
    (m, ncomponents) or (m,).  Host-side, like the reference's."""
    g = FES.xgrid
    fe = FES.FEType
    if fe.kind == FE_H1BR:
        return _interpolate_br(FES, f)
    if fe.kind not in (FE_H1P1, FE_H1P2):
        raise ValueError(f"interpolate: element {fe} not supported")
    dim, nc = g.dim, fe.ncomponents
    nv = dim + 1
    nb = nv if fe.kind == FE_H1P1 else (6 if dim == 2 else 10)

    def ev(x):
        y = np.asarray(f(x), dtype=np.float64)
        return y.reshape(x.shape[0], nc)

    X = g.coords[g.cells]                       # (ncells, dim+1, dim)
    out = np.zeros(FES.ndofs)
    cd = FES.celldofs
    vals_v = [ev(X[:, a, :]) for a in range(nv)]
    for c in range(nc):
        for a in range(nv):
            out[cd[:, c * nb + a]] = vals_v[a][:, c]
    if fe.kind == FE_H1P2:
        t, w = np.polynomial.legendre.leggauss(edge_points)
        t, w = 0.5 * (t + 1.0), 0.5 * w
        for e, (a, b) in enumerate(_P2_EDGES[dim]):
            mean = np.zeros((X.shape[0], nc))
            for tk, wk in zip(t, w):
                mean += wk * ev((1.0 - tk) * X[:, a, :] + tk * X[:, b, :])
            dofv = 1.5 * mean - 0.25 * (vals_v[a] + vals_v[b])
            for c in range(nc):
                out[cd[:, c * nb + nv + e]] = dofv[:, c]
    return out


def _interpolate_br(FES: FESpace, f) -> np.ndarray:
    """interpolate!(Target, FES, f) for H1BR{dim} (src/fedefs/h1v_br.jl:41-99):
    vertex DoFs of every component by point evaluation, then the bubble of
    face F set to (1/|F|) int_F (f - I_1 f) . n_F, with I_1 f the vertex
    interpolant (its face integral |F| times the mean of the face's vertex
    values) -- the bubbles have face mean 1, so the interpolant keeps every
    face's normal flux of f.  The face integrals use a rule exact for
    polynomials of degree 5 (Gauss on edges, Stroud's conical rule on
    triangles)."""
    g = FES.xgrid
    dim = g.dim
    fn, _ = g.faces()
    nrm, fvol, _ = g.face_geometry()
    nn = g.nverts

    def ev(x):
        return np.asarray(f(x), dtype=np.float64).reshape(x.shape[0], dim)

    out = np.zeros(FES.ndofs)
    vv = ev(g.coords)                                   # (nverts, dim)
    for c in range(dim):
        out[c * nn:(c + 1) * nn] = vv[:, c]
    P = g.coords[fn]                                    # (nfaces, dim, dim): the faces' vertices
    if dim == 2:
        t, w = np.polynomial.legendre.leggauss(3)
        t, w = 0.5 * (t + 1.0), 0.5 * w
        pts = [((1.0 - tk) * P[:, 0] + tk * P[:, 1], wk) for tk, wk in zip(t, w)]
    else:
        s1, w1 = np.polynomial.legendre.leggauss(3)
        s1, w1 = 0.5 * (s1 + 1.0), 0.5 * w1
        s2, w2 = _gauss_jacobi_10(3)
        pts = []
        for a, wa in zip(s1, w1):            # conical product: (s, r (1 - s)) on the unit triangle
            for b, wb in zip(s2, w2):
                x1, x2 = b, a * (1.0 - b)
                pts.append((P[:, 0] + x1 * (P[:, 1] - P[:, 0]) + x2 * (P[:, 2] - P[:, 0]), 2.0 * wa * wb))
    mean = np.zeros((fn.shape[0], dim))
    for x, wk in pts:
        mean += wk * ev(x)
    vmean = vv[fn].mean(axis=1)                         # mean of the vertex interpolant on the face
    out[dim * nn:] = np.einsum("fc,fc->f", mean - vmean, nrm)
    return out


def _gauss_jacobi_10(n: int):
    """n-point Gauss rule on [0, 1] for the weight (1 - s): nodes and weights
    (the collapsed direction of the conical triangle rule), from the
    eigenvalues of the Jacobi matrix of that weight."""
    # monic recurrence of the Jacobi polynomials P^(1,0) mapped to [0, 1]
    k = np.arange(n, dtype=np.float64)
    a, b = 1.0, 0.0
    alpha = (b * b - a * a) / ((2 * k + a + b) * (2 * k + a + b + 2))
    kk = np.arange(1, n, dtype=np.float64)
    beta = 4 * kk * (kk + a) * (kk + b) * (kk + a + b) / ((2 * kk + a + b) ** 2 * (2 * kk + a + b + 1) *
                                                          (2 * kk + a + b - 1))
    J = np.diag(alpha) + np.diag(np.sqrt(beta), 1) + np.diag(np.sqrt(beta), -1)
    x, V = np.linalg.eigh(J)
    w = 2.0 ** (a + b + 1) / (a + b + 1) * V[0] ** 2     # mu_0 = int_{-1}^{1} (1 - x) dx = 2
    return 0.5 * (x + 1.0), 0.25 * w                     # to [0, 1]: int_0^1 (1 - s) ds = 1/2
