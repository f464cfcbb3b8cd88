"""CPU tests of the tetrahedral path: the rules against exact moments and the reference's point counts, the
face-point pairing against the reference's Triangle permutation tables (read as text into the golden
fixture), the face vertex list, the adjacency of the host layer against the oracle's, and exact properties
of the oracle's discretisation on tetrahedra (free stream, conservation, convergence of an advected wave).

The rules are Keast's (volume) and Dunavant's (faces) restated from the published values, and for the P4
volume the Grundmann-Moeller rule s = 4 (70 points before merging the doubled centroid, exact to degree 9) in
place of gmsh's 43-point order-8 rule; gmsh, whose tables the reference calls, is not vendored, so the point
values are unpinned against it.  The P4 face rule's orbit order is pinned by the reference's P4 permutation."""
import json
import math
import os
import re

import numpy as np
import pytest

import subrosadg_gb300 as sdg
from oracle.orc import Oracle
from tests import cases

HERE = os.path.dirname(__file__)
RULES = os.path.join(HERE, "..", "subrosadg_gb300", "csrc", "tetrahedron_rules.h")


def _tables():
    with open(os.path.join(HERE, "golden", "reference_tables.json")) as f:
        return json.load(f)


def _array(text, name):
    m = re.search(r"%s\[\d+\] = \{([^}]*)\}" % name, text)
    return np.array([float(x) for x in m.group(1).split(",")])


def _rules():
    text = open(RULES).read()
    face = {d: (_array(text, f"kFaceTri{d}Xi"), _array(text, f"kFaceTri{d}Eta"), _array(text, f"kFaceTri{d}W"))
            for d in (3, 5, 7, 9, 11)}
    vol = {d: (_array(text, f"kTet{d}Xi"), _array(text, f"kTet{d}Eta"), _array(text, f"kTet{d}Zeta"),
               _array(text, f"kTet{d}W")) for d in (2, 4, 6, 8, 10)}
    return face, vol


def test_rules_integrate_their_degree_and_match_the_reference_counts():
    face, vol = _rules()
    counts = _tables()["quadrature_count"]
    for d, (x, y, w) in face.items():
        assert len(w) == counts["Triangle"][d]
        for a in range(d + 1):
            for b in range(d + 1 - a):
                exact = math.factorial(a) * math.factorial(b) / math.factorial(a + b + 2)
                assert abs((w * x ** a * y ** b).sum() - exact) < 1e-16
    for d, (x, y, z, w) in vol.items():
        # orders 8 and 10: Grundmann-Moeller s = 4 and 5 (69 points against the reference's 43; 126 points,
        # the reference's count, with the doubled centroid merged into 125), exact to degrees 9 and 11
        assert len(w) == {8: 69, 10: 125}.get(d, counts["Tetrahedron"][d])
        assert np.all(x >= 0) and np.all(y >= 0) and np.all(z >= 0) and np.all(x + y + z <= 1)
        top = {8: 9, 10: 11}.get(d, d)
        for a in range(top + 1):
            for b in range(top + 1 - a):
                for c in range(top + 1 - a - b):
                    exact = math.factorial(a) * math.factorial(b) * math.factorial(c) / math.factorial(a + b + c + 3)
                    # the Grundmann-Moeller weights alternate in sign: a little more cancellation in the sum
                    assert abs((w * x ** a * y ** b * z ** c).sum() - exact) < (2e-16 if d >= 8 else 1e-16)


@pytest.mark.parametrize("p", [1, 2, 3, 4, 5])
def test_face_point_pairing_matches_the_reference_tables(p):
    """A right face lists the shared vertices in the opposite orientation with the left face's first vertex
    at position r: left (xi, eta) is right r=0 (eta, xi), r=1 (1-xi-eta, eta), r=2 (xi, 1-xi-eta).  On the
    face rule's points this is the reference's permutation (SimulationControl.cpp:405-434)."""
    face, _ = _rules()
    x, y, _ = face[2 * p + 1]
    ref = _tables()["face_permutation"][f"Triangle/P{p}"]
    for r in range(3):
        X, Y = [(y, x), (1 - x - y, y), (x, 1 - x - y)][r]
        perm = [int(np.argmin((x - X[j]) ** 2 + (y - Y[j]) ** 2)) for j in range(len(x))]
        assert perm == ref[str(r)]


def test_face_vertex_list_and_outward_normals():
    """Tetrahedron faces (SimulationControl.cpp:195-200) and their outward orientation on the reference
    element: (v1 - v0) x (v2 - v0) of each listed face points away from the opposite vertex."""
    assert _tables()["face_vertices"]["Tetrahedron"] == [0, 2, 1, 0, 1, 3, 0, 3, 2, 3, 1, 2]
    ref = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1]], float)
    faces = np.array(_tables()["face_vertices"]["Tetrahedron"]).reshape(4, 3)
    for f in faces:
        n = np.cross(ref[f[1]] - ref[f[0]], ref[f[2]] - ref[f[0]])
        opposite = ref[[v for v in range(4) if v not in f][0]]
        assert np.dot(n, ref[f[0]] - opposite) > 0


@pytest.mark.parametrize("periodic", [True, False])
def test_adjacency_matches_the_oracle(periodic):
    """Host-layer adjacency (a handle with no GPU) equals the oracle's, bit for bit; shuffled vertex lists
    put shared faces at all three rotations."""
    mesh = cases.tet_mesh(3, periodic=periodic, conditions=None if periodic else [sdg.RIEMANN_FARFIELD] * 6)
    g = sdg.GpuSolver(mesh, cases.config(2, sdg.HLLC), device=-1)
    o = Oracle(mesh, cases.config(2, sdg.HLLC), faithful=False)
    gi, gb = g.adjacency()
    oi, ob = o.adjacency()
    assert np.array_equal(np.asarray(gi), np.asarray(oi)) and np.array_equal(np.asarray(gb), np.asarray(ob))
    assert set(np.asarray(gi)[:, 6]) == {0, 1, 2}
    assert g.counts.interior_face_count == (324 if periodic else 270)
    assert g.counts.boundary_face_count == (0 if periodic else 108)
    g.close()


def test_tetrahedra_of_orders_four_and_five_are_accepted():
    mesh = cases.tet_mesh(3)
    for p in (4, 5):
        g = sdg.GpuSolver(mesh, cases.config(p, sdg.HLLC), device=-1)
        assert g.counts.face_point_count == {4: 19, 5: 27}[p]
        g.close()


@pytest.mark.parametrize("p,flux", [(1, sdg.ROE), (2, sdg.HLLC), (3, sdg.LAX_FRIEDRICHS)])
def test_free_stream_preserved(p, flux):
    mesh = cases.tet_mesh(3, periodic=False, conditions=[sdg.RIEMANN_FARFIELD] * 6)
    o = Oracle(mesh, cases.config(p, flux), faithful=True)
    prim = np.tile([1.0, 0.3, 0.2, -0.1, 1.0 / cases.R_GAS], (o.volume_points_count, 1))
    o.initialize_primitive(prim)
    bpts, _ = o.boundary_points()
    o.set_boundary_primitive(np.repeat(prim[:1], len(bpts), 0))
    assert np.abs(o.residual_point()).max() < 1e-11


def test_conservation_on_a_periodic_box():
    """Telescoping face fluxes: the quadrature integral of every conserved variable stays constant."""
    mesh, cfg, prim, _, dt, _ = cases.tet_tgv_case(n=3, p=2, flux=sdg.ROE)
    o = Oracle(mesh, cfg, faithful=False)
    o.initialize_primitive(prim(o.volume_points()))
    host = sdg.GpuSolver(mesh, cfg, device=-1)  # w_q |J| of the same volume points, from the host layer
    jw = host.volume_weights()[:, None]
    host.close()
    before = (o.state_point() * jw).sum(0)
    o.step(dt, 10)
    after = (o.state_point() * jw).sum(0)
    np.testing.assert_allclose(after, before, rtol=1e-12, atol=1e-12 * np.abs(before).max())


def _wave_error(n, p):
    """Max density error at the volume points after t = 0.02 of rho = 1 + 0.1 sin(2 pi (x - t)),
    u = (1, 0.5, 0.25), p = 1 (an exact solution) on the periodic unit box of n^3 x 6 tetrahedra."""
    mesh = cases.tet_mesh(n)
    o = Oracle(mesh, cases.config(p, sdg.HLLC), faithful=False)
    x = o.volume_points()

    def prim(pts, t=0.0):
        rho = 1.0 + 0.1 * np.sin(2 * math.pi * (pts[:, 0] - t))
        one = np.ones_like(rho)
        return np.stack([rho, one, 0.5 * one, 0.25 * one, 1.0 / (rho * cases.R_GAS)], 1)

    o.initialize_primitive(prim(x))
    o.step(1e-3, 20)
    return np.abs(o.state_point()[:, 0] - prim(x, 0.02)[:, 0]).max()


def test_advected_density_wave_converges_with_order_and_mesh():
    e = [_wave_error(4, p) for p in (1, 2, 3)]
    assert e[0] > 2.5 * e[1] > 2.5 ** 2 * e[2], e
    assert _wave_error(3, 2) > 3.0 * _wave_error(6, 2)
