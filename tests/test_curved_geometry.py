"""Curved (high-order) 2D geometry on the CPU: the library's gmsh node order and Lagrange map (lattice indices,
product-formula basis) against the oracle's independent restatement (positions built ring by ring from the
corners, Vandermonde basis), through the geometry each side builds on the same curved meshes; and the MSH reader
keeping a 2D mesh's high-order nodes."""
import math

import numpy as np
import pytest

import subrosadg_gb300 as sdg
from oracle.orc import Oracle
from tests import cases


@pytest.mark.parametrize("q,split", [(2, 0.0), (3, 0.0), (4, 0.0), (5, 0.0), (2, 0.5), (3, 0.5), (4, 0.6)])
def test_curved_volume_points_match_oracle(q, split):
    mesh = sdg.Mesh.annulus(1.0, 2.0, 3, 9, geometry_order=q, split_fraction=split, seed=2)
    cfg = cases.config(q, sdg.HLLC)
    g = sdg.GpuSolver(mesh, cfg, device=-1)
    o = Oracle(mesh, cfg, faithful=False, precision="extended")
    np.testing.assert_allclose(g.volume_points(), o.volume_points(), rtol=0, atol=1e-14)
    # the geometry is curved: the volume points are not those of the straight-sided elements
    straight = sdg.Mesh(2, mesh.nodes, triangles=mesh.triangles, quadrangles=mesh.quadrangles, boundary=mesh.boundary,
                        boundary_physical=mesh.boundary_physical, physical_conditions=mesh.physical_conditions)
    assert np.abs(sdg.GpuSolver(straight, cfg, device=-1).volume_points() - g.volume_points()).max() > 1e-4


@pytest.mark.parametrize("q", [2, 3, 4])
def test_curved_boundary_points_lie_on_the_circles(q):
    """Boundary face points of the curved mesh lie on the boundary circles up to the order-q interpolation error
    of a circle (straight edges miss by h^2/8); the oracle places them at the same points."""
    mesh = sdg.Mesh.annulus(1.0, 2.0, 2, 16, geometry_order=q, boundary_conditions=(sdg.RIEMANN_FARFIELD,) * 2)
    g = sdg.GpuSolver(mesh, cases.config(q, sdg.HLLC), device=-1)
    pts, phys = g.boundary_points()
    r = np.hypot(pts[:, 0], pts[:, 1])
    target = np.where(np.repeat(phys, g.counts.face_point_count) == 1, 1.0, 2.0)
    miss = np.abs(r - target).max()
    h = 2 * math.pi / 16
    assert miss < 0.2 * (h ** 2 / 8) * (2.0 ** (2 - q))
    o = Oracle(mesh, cases.config(q, sdg.HLLC), faithful=False)
    po, _ = o.boundary_points()
    key = lambda a: np.lexsort(np.round(a[:, :2], 10).T)
    np.testing.assert_allclose(pts[key(pts)], po[key(po)], atol=1e-13)


def test_straight_mesh_given_at_high_order_is_unchanged():
    """A straight-sided mesh handed over with order-q geometry nodes (setOrder on straight elements) builds the
    straight geometry: the same volume points and adjacency as the first-order mesh."""
    base = sdg.Mesh.box_2d(0.0, 0.0, 1.0, 1.0, 4, 4, periodic=True, split_fraction=0.5, seed=4)
    ho = cases.with_geometry_nodes(base, 3)
    cfg = cases.config(3, sdg.ROE)
    a, b = sdg.GpuSolver(base, cfg, device=-1), sdg.GpuSolver(ho, cfg, device=-1)
    np.testing.assert_array_equal(a.volume_points(), b.volume_points())
    for x, y in zip(a.adjacency(), b.adjacency()):
        np.testing.assert_array_equal(x, y)


def test_curved_geometry_errors():
    mesh = sdg.Mesh.annulus(1.0, 2.0, 2, 6, geometry_order=3)
    bad = sdg.Mesh(2, mesh.nodes, quadrangles=mesh.quadrangles, boundary=mesh.boundary,
                   boundary_physical=mesh.boundary_physical, physical_conditions=mesh.physical_conditions,
                   geometry_order=3)  # no geometry nodes
    with pytest.raises(sdg.SdgError):
        sdg.GpuSolver(bad, cases.config(3, sdg.HLLC), device=-1)


def _write_msh(path, mesh):
    """The mesh as a gmsh MSH 4.1 ASCII file of order-q elements (types 10/36/37 quadrangles, 9/21/23
    triangles) with the two circles as physical curves."""
    q = mesh.geometry_order
    qtype = {2: 10, 3: 36, 4: 37, 5: 38}[q]
    ttype = {2: 9, 3: 21, 4: 23, 5: 25}[q]
    lines = ["$MeshFormat", "4.1 0 8", "$EndMeshFormat", "$Entities", "0 2 1 0",
             "1 0 0 0 0 0 0 1 1 0", "2 0 0 0 0 0 0 1 2 0", "1 0 0 0 0 0 0 0 0", "$EndEntities"]
    n = len(mesh.nodes)
    lines += ["$Nodes", f"1 {n} 1 {n}", f"2 1 0 {n}"] + [str(i + 1) for i in range(n)]
    lines += [f"{x:.17g} {y:.17g} {z:.17g}" for x, y, z in mesh.nodes] + ["$EndNodes"]
    blocks, tag = [], 1
    for phys in (1, 2):
        sel = mesh.boundary[mesh.boundary_physical == phys]
        rows = []
        for b in sel:
            rows.append(f"{tag} {b[0] + 1} {b[1] + 1}")
            tag += 1
        blocks.append((1, phys, 1, rows))
    for geo, t in ((mesh.triangle_geometry, ttype), (mesh.quadrangle_geometry, qtype)):
        if geo is None:
            continue
        rows = []
        for el in geo:
            rows.append(f"{tag} " + " ".join(str(v + 1) for v in el))
            tag += 1
        blocks.append((2, 1, t, rows))
    total = sum(len(b[3]) for b in blocks)
    lines += ["$Elements", f"{len(blocks)} {total} 1 {tag - 1}"]
    for d, ent, t, rows in blocks:
        lines.append(f"{d} {ent} {t} {len(rows)}")
        lines += rows
    lines.append("$EndElements")
    path.write_text("\n".join(lines) + "\n")


@pytest.mark.parametrize("q,split", [(2, 0.5), (3, 0.0), (4, 0.5)])
def test_msh_reader_keeps_high_order_nodes(tmp_path, q, split):
    mesh = sdg.Mesh.annulus(1.0, 2.0, 2, 8, geometry_order=q, split_fraction=split, seed=6)
    path = tmp_path / "curved.msh"
    _write_msh(path, mesh)
    back = sdg.Mesh.read_msh(path)
    back.set_boundary_condition(1, sdg.RIEMANN_FARFIELD)
    back.set_boundary_condition(2, sdg.RIEMANN_FARFIELD)
    assert back.geometry_order == q
    cfg = cases.config(q, sdg.HLLC)
    a, b = sdg.GpuSolver(mesh, cfg, device=-1), sdg.GpuSolver(back, cfg, device=-1)
    np.testing.assert_allclose(b.volume_points(), a.volume_points(), atol=1e-14)


# ---- curved hexahedra -------------------------------------------------------------------------------------

@pytest.mark.parametrize("q", [2, 3, 4, 5])
def test_curved_hexahedra_volume_points_match_oracle(q):
    """Order-q hexahedra (gmsh's hexahedron node order, library: lattice indices and products of 1D Lagrange
    polynomials; oracle: node positions built from the corners, edges, faces and interior, and 1D Vandermonde
    inverses) give the same volume points, which differ from those of the trilinear elements."""
    mesh, cfg = cases.curved_hex(cases.tgv_case(n=3, p=q), q)[:2]
    g = sdg.GpuSolver(mesh, cfg, device=-1)
    o = Oracle(mesh, cfg, faithful=False, precision="extended")
    np.testing.assert_allclose(g.volume_points(), o.volume_points(), rtol=0, atol=1e-13)
    trilinear = cases.warped(cases.tgv_case(n=3, p=q))[0]
    assert np.abs(sdg.GpuSolver(trilinear, cfg, device=-1).volume_points() - g.volume_points()).max() > 1e-2


def test_curved_hexahedra_boundary_points_match_oracle():
    mesh, cfg = cases.curved_hex(cases.hex_box_case(p=3), 3)[:2]
    g = sdg.GpuSolver(mesh, cfg, device=-1)
    o = Oracle(mesh, cfg, faithful=False)
    pg, _ = g.boundary_points()
    po, _ = o.boundary_points()
    key = lambda a: np.lexsort(np.round(a, 10).T)
    np.testing.assert_allclose(pg[key(pg)], po[key(po)], atol=1e-13)


def test_straight_hexahedra_given_at_high_order_are_unchanged():
    """Straight hexahedra handed over with order-q geometry nodes build the straight geometry bit for bit."""
    base = cases.hex_box_case(p=3)
    ho = cases.curved_hex(cases.hex_box_case(p=3), 3, amplitude=0.0)[0]
    cfg = base[1]
    a, b = sdg.GpuSolver(base[0], cfg, device=-1), sdg.GpuSolver(ho, cfg, device=-1)
    np.testing.assert_array_equal(a.volume_points(), b.volume_points())
    np.testing.assert_array_equal(a.boundary_points()[0], b.boundary_points()[0])


def test_curved_hexahedra_errors():
    mesh = cases.curved_hex(cases.hex_box_case(p=2), 2)[0]
    bad = sdg.Mesh(3, mesh.nodes, hexahedra=mesh.hexahedra, boundary=mesh.boundary,
                   boundary_physical=mesh.boundary_physical, physical_conditions=mesh.physical_conditions,
                   geometry_order=2)  # no geometry nodes
    with pytest.raises(sdg.SdgError):
        sdg.GpuSolver(bad, cases.config(2, sdg.HLLC), device=-1)
    tets = cases.tet_box_case(p=2)[0]
    tets.geometry_order = 2
    with pytest.raises(sdg.SdgError) as err:
        sdg.GpuSolver(tets, cases.config(2, sdg.HLLC), device=-1)
    assert err.value.code == 5  # SDG_ERR_UNSUPPORTED: curved tetrahedra are not built


def _write_msh_hex(path, mesh):
    """A hexahedral mesh as a gmsh MSH 4.1 ASCII file of order-q hexahedra (types 12/92/93/94) with its boundary
    quadrangles (type 3) on physical surfaces 1..n."""
    q = mesh.geometry_order
    htype = {2: 12, 3: 92, 4: 93, 5: 94}[q]
    groups = sorted(set(int(p) for p in mesh.boundary_physical))
    lines = ["$MeshFormat", "4.1 0 8", "$EndMeshFormat", "$Entities", f"0 0 {len(groups)} 1"]
    lines += [f"{g} 0 0 0 0 0 0 1 {g} 0" for g in groups] + ["1 0 0 0 0 0 0 0 0", "$EndEntities"]
    n = len(mesh.nodes)
    lines += ["$Nodes", f"1 {n} 1 {n}", f"3 1 0 {n}"] + [str(i + 1) for i in range(n)]
    lines += [f"{x:.17g} {y:.17g} {z:.17g}" for x, y, z in mesh.nodes] + ["$EndNodes"]
    blocks, tag = [], 1
    for g in groups:
        rows = []
        for b in mesh.boundary[mesh.boundary_physical == g]:
            rows.append(f"{tag} " + " ".join(str(v + 1) for v in b))
            tag += 1
        blocks.append((2, g, 3, rows))
    rows = []
    for el in mesh.hexahedron_geometry:
        rows.append(f"{tag} " + " ".join(str(v + 1) for v in el))
        tag += 1
    blocks.append((3, 1, htype, rows))
    total = sum(len(b[3]) for b in blocks)
    lines += ["$Elements", f"{len(blocks)} {total} 1 {tag - 1}"]
    for d, ent, t, rows in blocks:
        lines.append(f"{d} {ent} {t} {len(rows)}")
        lines += rows
    lines.append("$EndElements")
    path.write_text("\n".join(lines) + "\n")


@pytest.mark.parametrize("q", [2, 3, 4])
def test_msh_reader_keeps_hexahedron_high_order_nodes(tmp_path, q):
    mesh, cfg = cases.curved_hex(cases.hex_box_case(p=q), q)[:2]
    path = tmp_path / "curved_hex.msh"
    _write_msh_hex(path, mesh)
    back = sdg.Mesh.read_msh(path)
    for k in range(1, 7):
        back.set_boundary_condition(k, sdg.RIEMANN_FARFIELD)
    assert back.geometry_order == q
    np.testing.assert_array_equal(back.hexahedron_geometry, mesh.hexahedron_geometry)
    a, b = sdg.GpuSolver(mesh, cfg, device=-1), sdg.GpuSolver(back, cfg, device=-1)
    np.testing.assert_allclose(b.volume_points(), a.volume_points(), atol=1e-14)
