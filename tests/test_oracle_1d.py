"""CPU tests of the oracle's 1D path (DimensionEnum::D1, line meshes with point faces): the reference's own
tables read as text (line face vertices, point-face normals, line quadrature counts) and exact properties of
the discretisation (free stream, conservation on a periodic segment, the advected density wave)."""
import json
import os

import numpy as np
import pytest

import subrosadg_gb300 as sdg
from oracle.orc import Oracle
from tests import cases

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def _tables():
    with open(os.path.join(GOLDEN, "reference_tables.json")) as f:
        return json.load(f)


def test_line_tables_match_reference():
    """Line faces are its two vertices (SimulationControl.cpp:170-216); point faces face -1 at local face 0 and
    +1 at local face 1 (Geometry.cpp:102-112); the line rule of order 2P has P + 1 points
    (kLineQuadratureNumber, SimulationControl.cpp:268)."""
    t = _tables()
    assert t["face_vertices"]["Line"] == [0, 1]
    assert t["point_normals"] == {"0": -1.0, "1": 1.0}
    mesh = sdg.Mesh.line_1d(0.0, 1.0, 5, periodic=False, boundary_conditions=[sdg.RIEMANN_FARFIELD] * 2)
    for p in range(1, 6):
        o = Oracle(mesh, cases.config(p, sdg.HLLC), faithful=False)
        assert o.volume_points_count == o.elements * t["quadrature_count"]["Line"][2 * p]
        assert o.nfq == 1
        a, _ = o.adjacency()
        g = o.interior_face_geometry()
        for row, geo in zip(a, g):  # normal of each interior face from its left side's local face
            assert geo[0, 0] == t["point_normals"][str(row[2])]


@pytest.mark.parametrize("p,flux", [(1, sdg.ROE), (2, sdg.LAX_FRIEDRICHS), (3, sdg.HLLC), (5, sdg.CENTRAL)])
def test_free_stream_preserved(p, flux):
    mesh = sdg.Mesh.line_1d(-1.0, 3.0, 9, periodic=False, boundary_conditions=[sdg.RIEMANN_FARFIELD] * 2)
    o = Oracle(mesh, cases.config(p, flux), faithful=True)
    prim = cases.uniform_primitive(o.volume_points_count, 1)
    o.initialize_primitive(prim)
    bpts, _ = o.boundary_points()
    o.set_boundary_primitive(np.repeat(prim[:1], len(bpts), 0))
    assert np.abs(o.residual_point()).max() < 1e-12


def test_mass_momentum_energy_conserved_on_a_periodic_segment():
    """Telescoping point fluxes: the quadrature integral of every conserved variable is constant."""
    n, p = 12, 3
    mesh, cfg, prim, _, dt, _ = cases.density_wave_1d_case(n=n, p=p)
    o = Oracle(mesh, cfg, faithful=False)
    o.initialize_primitive(prim(o.volume_points()))
    # volume weights of the uniform segment [0, 2]: |J| w_q with |J| = h / 2, element after element
    _, w = np.polynomial.legendre.leggauss(p + 1)
    jw = np.tile(w * (2.0 / n) / 2.0, n)[:, None]
    before = (o.state_point() * jw).sum(0)
    o.step(dt, 20)
    after = (o.state_point() * jw).sum(0)
    np.testing.assert_allclose(after, before, rtol=1e-13)


@pytest.mark.parametrize("p", [1, 2, 3, 4, 5])
def test_density_wave_converges_to_the_advected_profile(p):
    """rho = 1 + 0.2 sin(pi (x - t)), u = 1, p = 1 is an exact solution; the error after t = 0.1 falls with
    the order (P = 1: ~1e-4 on 40 elements, P = 5: ~1e-12)."""
    mesh, cfg, prim, _, _, _ = cases.density_wave_1d_case(n=40, p=p)
    o = Oracle(mesh, cfg, faithful=False)
    x = o.volume_points()[:, 0]
    o.initialize_primitive(prim(o.volume_points()))
    dt, steps = 1e-4, 1000
    o.step(dt, steps)
    err = np.abs(o.state_point()[:, 0] - (1.0 + 0.2 * np.sin(np.pi * (x - dt * steps)))).max()
    bound = {1: 1e-3, 2: 2e-5, 3: 2e-7, 4: 2e-9, 5: 2e-11}[p]
    assert err < bound, err
