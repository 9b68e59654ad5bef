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
        ctx.space_on_device(F.H1BR(2), g)
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
