"""CPU tests of the oracle's artificial viscosity (the reference's shock capturing: Persson-Peraire density
sensor, node max, the artificial viscous flux of the volume gradient; SpatialDiscrete.cpp:37-250,528-842,
ViscousFlux.cpp:105-200) through analytic invariants."""
import math

import numpy as np
import pytest

import subrosadg_gb300 as sdg
from oracle.orc import Oracle
from tests import cases


def _oracle(case):
    mesh, cfg, prim, bprim, dt, steps = case
    o = Oracle(mesh, cfg, faithful=False, precision="double")
    o.initialize_primitive(prim(o.volume_points()))
    if o.boundary:
        bpts, phys = o.boundary_points()
        o.set_boundary_primitive(bprim(bpts, np.repeat(phys, o.nfq)))
    return o


def _uniform(dim):
    def prim(pts):
        out = np.zeros((len(pts), dim + 2))
        out[:, 0] = 1.0
        out[:, 1:1 + dim] = (0.3, -0.2, 0.1)[:dim]
        out[:, dim + 1] = 1.0 / cases.R_GAS
        return out
    return prim


@pytest.mark.parametrize("p", [1, 2, 4])
def test_av_free_stream(p):
    """Uniform flow: the volume gradient vanishes, so the artificial flux does for any eps (P1: eps = eps0 h/2)."""
    mesh = sdg.Mesh.box_2d(0.0, 0.0, 1.0, 1.0, 4, 4, periodic=True, jitter=0.1, split_fraction=0.5, seed=2)
    case = cases.with_av((mesh, cases.config(p, sdg.HLLC), _uniform(2), None, 1e-3, 1))
    o = _oracle(case)
    assert np.abs(o.residual_point()).max() <= 1e-11
    av = o.node_artificial_viscosity()
    assert (av > 0).any() if p == 1 else np.all(av == 0.0)


def test_av_p1_is_half_the_full_viscosity():
    """P1 takes the whole density as its high-order part: s = 0 = s0, the ramp's midpoint eps0 h/2
    (SpatialDiscrete.cpp:51-52,79-86); on a uniform 4x4 grid of the unit square h = 1/8 (inscribed circle)."""
    mesh = sdg.Mesh.box_2d(0.0, 0.0, 1.0, 1.0, 4, 4, periodic=True)
    case = cases.with_av((mesh, cases.config(1, sdg.HLLC), _uniform(2), None, 1e-3, 1), tolerance=0.5, factor=2.0)
    av = _oracle(case).node_artificial_viscosity()
    np.testing.assert_allclose(av, 2.0 * (1.0 / 8.0) / 1.0 / 2.0, rtol=1e-14)


def test_av_smooth_flow_is_untouched():
    """A smooth vortex: every element's sensor is far below s0 - kappa, eps = 0 and the residual is exactly
    the one without shock capturing."""
    base = cases.vortex_case(n=6, p=3, flux=sdg.ROE)
    r0 = _oracle(base).residual_point()
    o = _oracle(cases.with_av(cases.vortex_case(n=6, p=3, flux=sdg.ROE), tolerance=0.5))
    assert np.all(o.node_artificial_viscosity() == 0.0)
    np.testing.assert_allclose(o.residual_point(), r0, rtol=0, atol=1e-13 * np.abs(r0).max())


def test_av_shock_switches_on_and_is_bounded():
    case = cases.shock_tube_case(p=3, n=8)
    o = _oracle(case)
    av = o.node_artificial_viscosity()
    mesh = case[0]
    nodes_x = mesh.nodes[:, 0]
    hmax = 2 * (1 / 8) * (0.25 / 2) / (1 / 8 + 0.25 / 2) / 3.0  # eps0 h / P with h = 2A / perimeter
    assert av.max() > 0.0 and av.max() <= hmax * (1 + 1e-12)
    assert np.all(av[np.abs(nodes_x - 0.5) > 0.3] == 0.0)  # away from the jump the flow is smooth


def test_av_residual_is_affine_in_the_factor():
    """eps is linear in eps0 and the artificial flux is linear in eps: R(2 f) - 2 R(f) + R(0) = 0."""
    rs = [_oracle(cases.shock_tube_case(p=2, n=8, factor=f)).residual_point() for f in (0.0, 0.5, 1.0)]
    d = rs[2] - 2 * rs[1] + rs[0]
    assert np.abs(d).max() <= 1e-10 * np.abs(rs[2] - rs[0]).max()
    assert np.abs(rs[2] - rs[0]).max() > 1e-6  # the artificial flux is not round-off


def test_av_3d_hex_runs_and_switches_on():
    case = cases.shock_tube_case(p=2, n=8, dim=3)
    o = _oracle(case)
    assert o.node_artificial_viscosity().max() > 0
    o.step(case[4], 2)
    assert np.isfinite(o.state_point()).all()
