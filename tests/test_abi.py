"""CPU tests of the C ABI library: it loads, exports every symbol include/sdg_gpu.h declares, validates its
arguments, and its host-side mesh layer (adjacency, periodic pairing, geometry) is bit-exact with the oracle."""
import ctypes
import os
import re

import numpy as np
import pytest

import subrosadg_gb300 as sdg
from subrosadg_gb300 import _abi
from oracle.orc import Oracle
from tests import cases

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared_symbols():
    txt = open(os.path.join(ROOT, "include", "sdg_gpu.h")).read()
    return sorted(set(re.findall(r"^\s*(?:int|const char\*)\s+(sdg_\w+)\s*\(", txt, re.M)))


def test_library_exports_every_declared_symbol():
    lib = _abi.load()
    declared = _declared_symbols()
    assert len(declared) >= 20
    for name in declared:
        assert hasattr(lib, name), name
    assert set(declared) == set(_abi.SIGNATURES), set(declared) ^ set(_abi.SIGNATURES)


def test_invalid_arguments_are_rejected_without_a_gpu():
    lib = _abi.load()
    mesh = sdg.Mesh.box_2d(0, 0, 1, 1, 2, 2)
    m = mesh.struct()
    h = ctypes.c_void_p()
    bad = cases.config(9, sdg.HLLC)
    assert lib.sdg_create(ctypes.byref(m), ctypes.byref(bad), 0, ctypes.byref(h)) == 1
    assert b"order" in lib.sdg_last_error(None)
    bad = cases.config(2, 7)
    assert lib.sdg_create(ctypes.byref(m), ctypes.byref(bad), 0, ctypes.byref(h)) == 1
    assert lib.sdg_step(None, 1, 1e-3) == 1
    g = _abi.SdgGeneratedMesh()
    assert lib.sdg_mesh_generate_2d(0, 0, 1, 1, 0, 2, 0.0, 0.0, 0, 1, None, ctypes.byref(g)) == 1


def test_host_only_handle_refuses_state_calls():
    mesh = sdg.Mesh.box_2d(0, 0, 1, 1, 3, 3)
    s = sdg.GpuSolver(mesh, cases.config(2, sdg.HLLC), device=-1)
    with pytest.raises(sdg.SdgError) as e:
        s.stepSolver(1e-3)
    assert e.value.code == 8


@pytest.mark.parametrize("name,mesh_fn", [
    ("periodic-quad", lambda: sdg.Mesh.box_2d(-5, -5, 10, 10, 7, 5)),
    ("periodic-hex", lambda: sdg.Mesh.box_3d(0, 0, 0, 1, 2, 3, 3, 4, 3)),
    ("hybrid-jitter", lambda: sdg.Mesh.box_2d(0, 0, 1, 1, 9, 7, jitter=0.1, split_fraction=0.5, seed=9)),
    ("walls", lambda: sdg.Mesh.box_2d(0, 0, 2, 1, 6, 3, periodic=False, boundary_conditions=[4, 2, 4, 1])),
    ("walls-hex", lambda: sdg.Mesh.box_3d(0, 0, 0, 1, 1, 1, 2, 3, 2, periodic=False, boundary_conditions=[0, 1, 2, 3, 4, 5])),
    ("periodic-line", lambda: sdg.Mesh.line_1d(0, 2, 7)),
    ("farfield-line", lambda: sdg.Mesh.line_1d(-5, 10, 9, periodic=False, boundary_conditions=[0, 0])),
])
def test_adjacency_bit_exact_with_oracle(name, mesh_fn):
    mesh = mesh_fn()
    cfg = cases.config(2, sdg.HLLC)
    s = sdg.GpuSolver(mesh, cfg, device=-1)
    o = Oracle(mesh, cfg, faithful=False)
    a1, b1 = s.adjacency()
    a2, b2 = o.adjacency()
    assert np.array_equal(a1, a2)
    assert np.array_equal(b1, b2)
    # every element face appears exactly once as a side
    sides = set()
    for r in a1:
        sides.add((r[0], r[1], r[2])); sides.add((r[3], r[4], r[5]))
    for r in b1:
        sides.add((r[0], r[1], r[2]))
    nfaces = sum(n * k for n, k in ((0 if mesh.lines is None else len(mesh.lines), 2),
                                    (0 if mesh.triangles is None else len(mesh.triangles), 3),
                                    (0 if mesh.quadrangles is None else len(mesh.quadrangles), 4),
                                    (0 if mesh.hexahedra is None else len(mesh.hexahedra), 6)))
    assert len(sides) == nfaces
    np.testing.assert_allclose(s.volume_points(), o.volume_points(), atol=1e-13)
    bp1, ph1 = s.boundary_points()
    bp2, ph2 = o.boundary_points()
    assert bp1.shape == bp2.shape


def test_two_wide_periodic_mesh_is_rejected():
    # folding periodic nodes onto masters makes two distinct edges share a vertex set when a periodic
    # direction is only two elements wide; that mesh is rejected as a mesh error
    with pytest.raises(sdg.SdgError) as e:
        sdg.GpuSolver(sdg.Mesh.box_2d(0, 0, 1, 1, 2, 3), cases.config(2, sdg.HLLC), device=-1)
    assert e.value.code == 4


def test_periodic_pairing_counts():
    mesh = sdg.Mesh.box_3d(0, 0, 0, 1, 1, 1, 4, 4, 4)
    s = sdg.GpuSolver(mesh, cases.config(1, sdg.HLLC), device=-1)
    a, b = s.adjacency()
    assert len(a) == 3 * 64 and len(b) == 0
    rot = np.unique(a[:, 6])
    assert set(rot.tolist()) <= {0, 1, 2, 3}


def test_mesh_errors():
    # a boundary face without a boundary element (physical group missing)
    mesh = sdg.Mesh.box_2d(0, 0, 1, 1, 2, 2, periodic=False, boundary_conditions=[4, 4, 4, 4])
    mesh.boundary = mesh.boundary[:-1].copy()
    mesh.boundary_physical = mesh.boundary_physical[:-1].copy()
    with pytest.raises(sdg.SdgError) as e:
        sdg.GpuSolver(mesh, cases.config(2, sdg.HLLC), device=-1)
    assert e.value.code == 4
    # an inverted element
    mesh = sdg.Mesh.box_2d(0, 0, 1, 1, 3, 3)
    mesh.quadrangles[0] = mesh.quadrangles[0][::-1].copy()
    with pytest.raises(sdg.SdgError):
        sdg.GpuSolver(mesh, cases.config(2, sdg.HLLC), device=-1)


def test_msh_reader_roundtrip(tmp_path):
    """Write a small MSH 4.1 file (periodic 2D quads) and read it back through the library."""
    nx = ny = 2
    nodes = [(i / nx, j / ny) for j in range(ny + 1) for i in range(nx + 1)]
    quads = [(j * 3 + i + 1, j * 3 + i + 2, (j + 1) * 3 + i + 2, (j + 1) * 3 + i + 1) for j in range(ny) for i in range(nx)]
    lines = []
    for i in range(nx):
        lines.append((1, i + 1, i + 2))
        lines.append((3, 7 + i + 1, 7 + i))
    for j in range(ny):
        lines.append((2, j * 3 + 3, (j + 1) * 3 + 3))
        lines.append((4, (j + 1) * 3 + 1, j * 3 + 1))
    txt = ["$MeshFormat", "4.1 0 8", "$EndMeshFormat", "$Entities", "0 4 1 0"]
    for c in range(1, 5):
        txt.append(f"{c} 0 0 0 1 1 0 1 {c} 0")
    txt.append("1 0 0 0 1 1 0 1 5 0")
    txt += ["$EndEntities", "$Nodes", f"1 {len(nodes)} 1 {len(nodes)}", f"2 1 0 {len(nodes)}"]
    txt += [str(k + 1) for k in range(len(nodes))]
    txt += [f"{x} {y} 0" for x, y in nodes]
    txt += ["$EndNodes", "$Elements", f"5 {len(lines) + len(quads)} 1 {len(lines) + len(quads)}"]
    tag = 1
    for c in range(1, 5):
        mine = [l for l in lines if l[0] == c]
        txt.append(f"1 {c} 1 {len(mine)}")
        for l in mine:
            txt.append(f"{tag} {l[1]} {l[2]}"); tag += 1
    txt.append(f"2 1 3 {len(quads)}")
    for q in quads:
        txt.append(f"{tag} {' '.join(map(str, q))}"); tag += 1
    txt += ["$EndElements"]
    path = tmp_path / "box.msh"
    path.write_text("\n".join(txt) + "\n")
    m = sdg.Mesh.read_msh(path)
    assert m.dimension == 2 and len(m.quadrangles) == 4 and len(m.boundary) == 8
    assert len(m.physical_conditions) == 4
    for k in range(1, 5):
        m.set_boundary_condition(k, sdg.ADIABATIC_SLIP_WALL)
    s = sdg.GpuSolver(m, cases.config(2, sdg.HLLC), device=-1)
    a, b = s.adjacency()
    assert len(a) == 4 and len(b) == 8


def _msh_1d(tmp_path, n, groups):
    """MSH 4.1 file of [0, 1] in n lines (the 1D example drivers' transfinite curve); groups: the physical tag of
    each end point (equal tags: one group holding both)."""
    nodes = [i / n for i in range(n + 1)]
    txt = ["$MeshFormat", "4.1 0 8", "$EndMeshFormat", "$Entities", "2 1 0 0",
           f"1 0 0 0 1 {groups[0]}", f"2 1 0 0 1 {groups[1]}", "1 0 0 0 1 0 0 1 9 2 1 -2", "$EndEntities",
           "$Nodes", f"3 {n + 1} 1 {n + 1}", "0 1 0 1", "1", "0 0 0", "0 2 0 1", "2", "1 0 0",
           f"1 1 0 {n - 1}"]
    txt += [str(k + 3) for k in range(n - 1)]
    txt += [f"{x} 0 0" for x in nodes[1:-1]]
    txt += ["$EndNodes", "$Elements", f"3 {n + 2} 1 {n + 2}", "0 1 15 1", "1 1", "0 2 15 1", "2 2", f"1 1 1 {n}"]
    order = [1] + [k + 3 for k in range(n - 1)] + [2]
    for i in range(n):
        txt.append(f"{i + 3} {order[i]} {order[i + 1]}")
    txt += ["$EndElements"]
    path = tmp_path / "line.msh"
    path.write_text("\n".join(txt) + "\n")
    return sdg.Mesh.read_msh(path)


def test_msh_reader_1d_farfield_and_periodic(tmp_path):
    """1D meshes as the reference's 1D drivers write them: point physical groups; two farfield groups
    (sod_1d_ceuler.cpp:75-77), or one periodic group holding both end points (periodic_1d_ceuler.cpp:70),
    whose two points the reference joins into one interior face (Adjacency.cpp:185-211)."""
    m = _msh_1d(tmp_path, 6, (1, 2))
    assert m.dimension == 1 and len(m.lines) == 6 and len(m.boundary) == 2 and len(m.physical_conditions) == 2
    m.set_boundary_condition(1, sdg.RIEMANN_FARFIELD)
    m.set_boundary_condition(2, sdg.RIEMANN_FARFIELD)
    s = sdg.GpuSolver(m, cases.config(3, sdg.HLLC), device=-1)
    a, b = s.adjacency()
    assert len(a) == 5 and len(b) == 2
    assert b[:, 2].tolist() == [0, 1] and b[:, 3].tolist() == [1, 2]
    o = Oracle(m, cases.config(3, sdg.HLLC), faithful=False)
    a2, b2 = o.adjacency()
    assert np.array_equal(a, a2) and np.array_equal(b, b2)
    p = _msh_1d(tmp_path, 6, (1, 1))
    assert len(p.physical_conditions) == 1
    p.set_boundary_condition(1, sdg.PERIODIC)
    s = sdg.GpuSolver(p, cases.config(3, sdg.HLLC), device=-1)
    a, b = s.adjacency()
    assert len(a) == 6 and len(b) == 0
    # the joined face (type, element, face of each side, rotation): the first point element's parent (element 0,
    # its local face 0) on the left
    assert [sdg.LINE, 0, 0, sdg.LINE, 5, 1, 0] in a.tolist()
    o = Oracle(p, cases.config(3, sdg.HLLC), faithful=False)
    a2, b2 = o.adjacency()
    assert np.array_equal(a, a2)
    # the generated periodic line (a periodic node map) gives the same faces
    g = sdg.GpuSolver(sdg.Mesh.line_1d(0, 1, 6), cases.config(3, sdg.HLLC), device=-1)
    assert np.array_equal(g.adjacency()[0], a)
