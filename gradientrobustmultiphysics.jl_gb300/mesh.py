"""Structured simplex meshes and their topology.

This module plays the role ExtendableGrids.jl plays for the reference
(``grid_unitsquare``, ``uniform_refine``, ``FaceNodes``, ``CellFaces``,
``CellEdges``, ``FaceNormals``, ``CellFaceSigns``, ``BFaceRegions``).  That
package is not part of the reference tree, so the numbering and orientation
conventions below are this library's own and are stated here:

* 2D unit square, n x n squares.  Node (i, j) has index ``j*(n+1) + i`` and
  coordinates ``(i/n, j/n)``.  Square (i, j) is split along its (0,0)-(1,1)
  diagonal into ``(v00, v10, v11)`` and ``(v00, v11, v01)``; both are
  counter-clockwise.  Cell index ``2*(j*n + i) + t``.
* 3D unit cube, n^3 cubes, each split into the 6 Kuhn tetrahedra sharing the
  diagonal v000-v111: for each permutation (a, b, c) of the axes the tet is
  ``(v000, v000+e_a, v000+e_a+e_b, v111)``.  Permutations are taken in
  lexicographic order.  Cell index ``6*cube + p``.
* Local faces of a triangle (the reference's local_cellfacenodes for
  Triangle2D and the P2 / BR bases, src/fedefs/h1_p2.jl:134-146):
  face f joins local nodes (f, f+1 mod 3).
* Local edges of a tetrahedron (src/fedefs/h1_p2.jl:149-165 basis order):
  (0,1) (0,2) (0,3) (1,2) (1,3) (2,3).
* Local faces of a tetrahedron: (0,1,2) (0,1,3) (1,2,3) (0,2,3)
  (opposite nodes 3, 2, 0, 1).
* Global faces / edges are numbered by the lexicographic order of their
  sorted node tuples.
* Face normals: unit normals with a fixed global orientation -- the normal
  points out of the first cell (lowest cell index) that contains the face.
  ``cell_face_signs[c, f]`` is +1 when the global normal is the outward
  normal of cell c, else -1.
* Boundary regions, 2D: 1 = {y=0}, 2 = {x=1}, 3 = {y=1}, 4 = {x=0}.
  3D: 1 = {z=0}, 2 = {y=0}, 3 = {x=1}, 4 = {y=1}, 5 = {x=0}, 6 = {z=1}.
"""
from __future__ import annotations

import itertools

import numpy as np

TRI_LOCAL_FACES = np.array([[0, 1], [1, 2], [2, 0]], dtype=np.int64)
TET_LOCAL_EDGES = np.array([[0, 1], [0, 2], [0, 3], [1, 2], [1, 3], [2, 3]], dtype=np.int64)
TET_LOCAL_FACES = np.array([[0, 1, 2], [0, 1, 3], [1, 2, 3], [0, 2, 3]], dtype=np.int64)


class SimplexMesh:
    """A conforming triangle (dim=2) or tetrahedron (dim=3) mesh.

    ``coords`` is (nverts, dim) float64, ``cells`` (ncells, dim+1) int32.
    Topology arrays are built on first use and cached.
    """

    def __init__(self, coords: np.ndarray, cells: np.ndarray, name: str = "mesh"):
        self.coords = np.ascontiguousarray(coords, dtype=np.float64)
        self.cells = np.ascontiguousarray(cells, dtype=np.int32)
        self.dim = self.coords.shape[1]
        if self.cells.shape[1] != self.dim + 1:
            raise ValueError("cells must have dim+1 vertices")
        self.name = name
        self._cache: dict = {}

    # -- sizes -------------------------------------------------------------
    @property
    def nverts(self) -> int:
        return self.coords.shape[0]

    @property
    def ncells(self) -> int:
        return self.cells.shape[0]

    # -- topology ----------------------------------------------------------
    def _enumerate(self, local: np.ndarray, key: str):
        if key in self._cache:
            return self._cache[key]
        loc = self.cells[:, local]                   # (ncells, nloc, k)
        srt = np.sort(loc, axis=2).reshape(-1, local.shape[1])
        k = srt.shape[1]
        B = max(int(self.nverts), 2)
        if B ** k <= 2 ** 63:
            # lexicographic order of the sorted tuples = order of the int64 keys
            code = np.zeros(srt.shape[0], dtype=np.int64)
            for j in range(k):
                code = code * B + srt[:, j].astype(np.int64)
            _, first, inv = np.unique(code, return_index=True, return_inverse=True)
            uniq = srt[first]
        else:
            uniq, inv = np.unique(srt, axis=0, return_inverse=True)
        inv = inv.reshape(self.ncells, local.shape[0]).astype(np.int32)
        self._cache[key] = (uniq.astype(np.int32), inv)
        return self._cache[key]

    def edges(self):
        """(edge_nodes (nedges, 2), cell_edges (ncells, nlocal))."""
        if self.dim == 2:
            return self._enumerate(TRI_LOCAL_FACES, "edges")
        return self._enumerate(TET_LOCAL_EDGES, "edges")

    def faces(self):
        """(face_nodes (nfaces, dim), cell_faces (ncells, dim+1))."""
        if self.dim == 2:
            return self._enumerate(TRI_LOCAL_FACES, "edges")
        return self._enumerate(TET_LOCAL_FACES, "faces")

    @property
    def nfaces(self) -> int:
        return self.faces()[0].shape[0]

    @property
    def nedges(self) -> int:
        return self.edges()[0].shape[0]

    def cell_volumes(self) -> np.ndarray:
        X = self.coords[self.cells]                  # (nc, d+1, d)
        A = X[:, 1:, :] - X[:, :1, :]
        det = np.linalg.det(A)
        return np.abs(det) / (2.0 if self.dim == 2 else 6.0)

    def face_geometry(self):
        """(face_normals (nfaces, dim), face_volumes (nfaces,),
        cell_face_signs (ncells, dim+1) int8)."""
        if "facegeo" in self._cache:
            return self._cache["facegeo"]
        fnodes, cfaces = self.faces()
        nf = fnodes.shape[0]
        nloc = cfaces.shape[1]
        local = TRI_LOCAL_FACES if self.dim == 2 else TET_LOCAL_FACES
        X = self.coords
        cellc = X[self.cells].mean(axis=1)
        outward = np.zeros((self.ncells, nloc, self.dim))
        vols = np.zeros(nf)
        for f in range(nloc):
            P = X[self.cells[:, local[f]]]
            if self.dim == 2:
                t = P[:, 1] - P[:, 0]
                nrm = np.stack([t[:, 1], -t[:, 0]], axis=1)
            else:
                nrm = np.cross(P[:, 1] - P[:, 0], P[:, 2] - P[:, 0])
            ln = np.linalg.norm(nrm, axis=1)
            nrm = nrm / ln[:, None]
            out = np.sign(np.einsum("ij,ij->i", nrm, P.mean(axis=1) - cellc))
            outward[:, f] = nrm * out[:, None]
            vols[cfaces[:, f]] = ln if self.dim == 2 else 0.5 * ln
        gf = cfaces.ravel()
        cid = np.repeat(np.arange(self.ncells), nloc)
        order = np.lexsort((cid, gf))
        _, first = np.unique(gf[order], return_index=True)
        owner = order[first]                      # flat (cell, local) index of lowest cell
        normals = outward.reshape(-1, self.dim)[owner]
        dots = np.einsum("ij,ij->i", outward.reshape(-1, self.dim), normals[gf])
        signs = np.where(dots > 0, 1, -1).astype(np.int8).reshape(self.ncells, nloc)
        self._cache["facegeo"] = (normals, vols, signs)
        return self._cache["facegeo"]

    def boundary_faces(self):
        """(bface_ids (nbfaces,), bface_regions (nbfaces,)) -- faces owned by
        exactly one cell, with the region numbers of the module docstring."""
        if "bfaces" in self._cache:
            return self._cache["bfaces"]
        fnodes, cfaces = self.faces()
        cnt = np.bincount(cfaces.ravel(), minlength=fnodes.shape[0])
        bf = np.nonzero(cnt == 1)[0].astype(np.int32)
        mid = self.coords[fnodes[bf]].mean(axis=1)
        reg = np.zeros(bf.shape[0], dtype=np.int32)
        tol = 1e-12
        if self.dim == 2:
            reg[np.abs(mid[:, 1]) < tol] = 1
            reg[np.abs(mid[:, 0] - 1) < tol] = 2
            reg[np.abs(mid[:, 1] - 1) < tol] = 3
            reg[np.abs(mid[:, 0]) < tol] = 4
        else:
            reg[np.abs(mid[:, 2]) < tol] = 1
            reg[np.abs(mid[:, 1]) < tol] = 2
            reg[np.abs(mid[:, 0] - 1) < tol] = 3
            reg[np.abs(mid[:, 1] - 1) < tol] = 4
            reg[np.abs(mid[:, 0]) < tol] = 5
            reg[np.abs(mid[:, 2] - 1) < tol] = 6
        self._cache["bfaces"] = (bf, reg)
        return self._cache["bfaces"]


def grid_unitsquare(n: int) -> SimplexMesh:
    """Unit square, n x n squares each split into 2 triangles (2 n^2 cells)."""
    i, j = np.meshgrid(np.arange(n + 1), np.arange(n + 1), indexing="xy")
    coords = np.stack([i.ravel() / n, j.ravel() / n], axis=1)
    ii, jj = np.meshgrid(np.arange(n), np.arange(n), indexing="xy")
    ii = ii.ravel(); jj = jj.ravel()
    v00 = jj * (n + 1) + ii
    v10 = v00 + 1
    v01 = v00 + (n + 1)
    v11 = v01 + 1
    t1 = np.stack([v00, v10, v11], axis=1)
    t2 = np.stack([v00, v11, v01], axis=1)
    cells = np.stack([t1, t2], axis=1).reshape(-1, 3)
    return SimplexMesh(coords, cells, name=f"unitsquare{n}")


def grid_unitcube_kuhn(n: int) -> SimplexMesh:
    """Unit cube, n^3 cubes each split into 6 Kuhn tetrahedra (6 n^3 cells)."""
    g = np.arange(n + 1)
    k, j, i = np.meshgrid(g, g, g, indexing="ij")
    coords = np.stack([i.ravel() / n, j.ravel() / n, k.ravel() / n], axis=1)

    def vid(a, b, c):
        return (c * (n + 1) + b) * (n + 1) + a

    cc, bb, aa = np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing="ij")
    aa = aa.ravel(); bb = bb.ravel(); cc = cc.ravel()
    unit = np.eye(3, dtype=np.int64)
    tets = []
    for perm in itertools.permutations(range(3)):
        p0 = np.zeros(3, dtype=np.int64)
        p1 = unit[perm[0]]
        p2 = p1 + unit[perm[1]]
        p3 = np.ones(3, dtype=np.int64)
        tets.append(np.stack([vid(aa + p[0], bb + p[1], cc + p[2]) for p in (p0, p1, p2, p3)], axis=1))
    cells = np.stack(tets, axis=1).reshape(-1, 4)
    return SimplexMesh(coords, cells, name=f"unitcube{n}")
