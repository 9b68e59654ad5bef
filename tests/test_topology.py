"""Device-built topology and DoF maps (grmp_space_create_on_device,
grmp_space_boundary_dofs) against the host mesh module and FESpace: the
CellDofs of H1P1 / H1P2 spaces bit for bit (the dofmap of
src/dofmaps.jl:201-330 with the lexicographic entity numbering), the DoF
count, and the boundary DoFs (BFaceDofs of src/boundarydata.jl:200-260) of
H1P1 / H1P2 / H1BR spaces, on structured grids, on grids whose vertex and
cell numbering has been shuffled, and on a single cell; a device-built space
assembles and solves like the host-built one."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _shuffled(G, g, seed):
    """The same mesh with permuted vertex and cell numbers and rotated local
    vertex order (the entity numbering then differs from the structured one)."""
    rng = np.random.default_rng(seed)
    pv = rng.permutation(g.nverts)
    inv = np.empty_like(pv)
    inv[pv] = np.arange(g.nverts)
    coords = g.coords[pv]
    cells = inv[g.cells][rng.permutation(g.ncells)]
    cells = np.roll(cells, 1, axis=1)
    return type(g)(coords, cells.astype(np.int32), name="shuffled")


def _grids(G):
    one2 = type(G.grid_unitsquare(1))(np.array([[0.0, 0.0], [1.0, 0.0], [0.0, 1.0]]),
                                      np.array([[0, 1, 2]], dtype=np.int32), name="one triangle")
    one3 = type(one2)(np.array([[0.0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1]]), np.array([[0, 1, 2, 3]], dtype=np.int32),
                      name="one tetrahedron")
    return {
        "square7": G.grid_unitsquare(7),
        "cube3": G.grid_unitcube_kuhn(3),
        "square6_shuffled": _shuffled(G, G.grid_unitsquare(6), 1),
        "cube3_shuffled": _shuffled(G, G.grid_unitcube_kuhn(3), 2),
        "one_triangle": one2,
        "one_tetrahedron": one3,
    }


@pytest.mark.parametrize("grid", ["square7", "cube3", "square6_shuffled", "cube3_shuffled", "one_triangle",
                                  "one_tetrahedron"])
@pytest.mark.parametrize("fe,nc", [("P1", 1), ("P2", 1), ("P2", 3), ("P1", 2)])
def test_device_dofmap_equals_host(G, ctx, grid, fe, nc):
    from grmp_gb300 import fespace as F
    g = _grids(G)[grid]
    ft = F.H1P1(nc) if fe == "P1" else F.H1P2(nc, g.dim)
    host = F.FESpace(ft, g)
    dev = ctx.space_on_device(ft, g)
    assert dev.ndofs == host.ndofs
    assert np.array_equal(dev.celldofs, host.celldofs)
    assert np.array_equal(ctx.boundary_dofs(dev), host.boundary_dofs())
    assert np.array_equal(ctx.boundary_dofs(host), host.boundary_dofs())


@pytest.mark.parametrize("grid", ["square7", "cube3", "cube3_shuffled"])
def test_device_boundary_dofs_of_br_space(G, ctx, grid):
    from grmp_gb300 import fespace as F
    g = _grids(G)[grid]
    S = F.FESpace(F.H1BR(g.dim), g)
    assert np.array_equal(ctx.boundary_dofs(S), S.boundary_dofs())


def test_refusals(G, ctx):
    from grmp_gb300 import fespace as F
    from grmp_gb300 import _lib as L
    g = G.grid_unitsquare(3)
    with pytest.raises(G.GrmpError) as ei:
        ctx.space_on_device(F.H1BR(3), g)          # BR{3} on a 2D mesh
    assert ei.value.code == L.ERR_UNSUPPORTED
    with pytest.raises(G.GrmpError) as ei:
        ctx.space_on_device(F.L2P0(1), g)
    assert ei.value.code == L.ERR_UNSUPPORTED
    import ctypes
    S = F.FESpace(F.H1P2(1, 2), g)
    n = ctypes.c_int32()
    buf = np.zeros(3, dtype=np.int32)
    rc = ctx.lib.grmp_space_boundary_dofs(ctx.space(S), 3, buf.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)),
                                          ctypes.byref(n))
    assert rc == L.ERR_INVALID_ARG and n.value == S.boundary_dofs().size


def test_device_space_solves_like_host_space(G, ctx):
    """3D P2 Poisson on a device-built space: the same matrix and solution as
    on the host-built space (same DoF numbering)."""
    from grmp_gb300 import fespace as F
    from grmp_gb300 import problems as P
    prob = P.poisson3d(4, seed=3)
    dev = ctx.space_on_device(F.H1P2(1, 3), prob.FES.xgrid)
    out = []
    for FES in (prob.FES, dev):
        A = G.FEMatrix(ctx, FES, prob.operators)
        G.assemble(A, prob.operators, G.FP64)
        b = G.FEVector(ctx, FES)
        b.fill(0.0)
        G.assemble(b, prob.rhs)
        G.apply_dirichlet(A, b, ctx.boundary_dofs(FES), None, G.DIRICHLET_ELIMINATE)
        x = G.FEVector(ctx, FES)
        G.GB300PCG(mode="fp64", reltol=1e-13, abstol=0.0).solve(A, b, x)
        out.append((A.download(G.FP64), x.entries))
    assert np.array_equal(out[0][0].indptr, out[1][0].indptr)
    assert np.array_equal(out[0][0].indices, out[1][0].indices)
    assert np.array_equal(out[0][0].data, out[1][0].data)
    assert np.array_equal(out[0][1], out[1][1])


@pytest.mark.parametrize("grid", ["square7", "cube3", "square6_shuffled", "cube3_shuffled", "one_tetrahedron"])
def test_device_faces_equal_host(G, ctx, grid):
    """grmp_mesh_build_faces against SimplexMesh.faces / face_geometry:
    numbering and signs exact, normals and measures to rounding."""
    g = _grids(G)[grid]
    cf, nr, fv, sg = ctx.mesh_faces(g)
    hfn, hcf = g.faces()
    hnr, hfv, hsg = g.face_geometry()
    assert np.array_equal(cf, hcf)
    assert np.array_equal(sg, hsg)
    assert nr.shape == hnr.shape and np.max(np.abs(nr - hnr)) <= 1e-15
    assert np.max(np.abs(fv - hfv) / hfv) <= 1e-15


@pytest.mark.parametrize("grid", ["square7", "cube3_shuffled"])
def test_device_br_space_assembles_like_host(G, O, ctx, grid):
    """An H1BR{d} space built on the device (DoF map and face data) gives the
    host-built space's CellDofs and boundary DoFs, and the same penalised
    Stokes matrix and reconstructed load to rounding of the face normals."""
    from grmp_gb300 import fespace as F
    from grmp_gb300 import _lib as L
    from grmp_gb300 import api
    g = _grids(G)[grid]
    gd = type(g)(g.coords.copy(), g.cells.copy(), name="device copy")   # its own mesh handle
    host = F.FESpace(F.H1BR(g.dim), g)
    dev = ctx.space_on_device(F.H1BR(g.dim), gd)
    assert dev.ndofs == host.ndofs and np.array_equal(dev.celldofs, host.celldofs)
    assert np.array_equal(ctx.boundary_dofs(dev), host.boundary_dofs())
    ops = [api.Operator(L.OP_LAPLACE, True, 0.7), api.Operator(L.OP_RDIVRDIV, False, 50.0)]
    if g.dim == 2:
        terms = np.array([(0, 1.0, 1, 0, 0), (1, -2.0, 0, 2, 0), (0, 0.5, 0, 0, 0)])
    else:
        terms = np.array([(0, 1.0, 1, 0, 0), (1, -2.0, 0, 2, 0), (2, 0.5, 0, 1, 1)])
    out = []
    for FES in (host, dev):
        A = api.FEMatrix(ctx, FES, ops)
        api.assemble(A, ops, L.FP64)
        b = api.FEVector(ctx, FES)
        b.fill(0.0)
        api.assemble(b, api.LinearForm(api.ReconstructionIdentity, api.DataFunction.polynomial(terms, g.dim, 1)))
        out.append((A.download(L.FP64), b.entries))
    (Ah, bh), (Ad, bd) = out
    assert np.array_equal(Ah.indptr, Ad.indptr) and np.array_equal(Ah.indices, Ad.indices)
    assert np.max(np.abs(Ad.data - Ah.data)) <= 1e-13 * np.max(np.abs(Ah.data))
    assert np.max(np.abs(bd - bh)) <= 1e-13 * np.max(np.abs(bh))
