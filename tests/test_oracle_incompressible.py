"""CPU tests of the oracle's incompressible model (the reference's IncompresibleEuler / IncompresibleNS with the
weakly compressible equation of state, PhysicalModel.cpp:57-78, and the Boussinesq source, SourceTerm.cpp:29-58)
through analytic invariants of the discretisation."""
import numpy as np
import pytest

import subrosadg_gb300 as sdg
from oracle.orc import Oracle
from tests import cases


def _oracle(mesh, cfg, prim, bprim=None):
    o = Oracle(mesh, cfg, faithful=False, precision="double")
    o.initialize_primitive(prim(o.volume_points()))
    if o.boundary:
        bpts, phys = o.boundary_points()
        o.set_boundary_primitive(bprim(bpts, np.repeat(phys, o.nfq)))
    return o


def _uniform(dim, rho=1.0, vel=(0.3, -0.2, 0.1), t=1.0):
    def prim(pts):
        out = np.zeros((len(pts), dim + 2))
        out[:, 0] = rho
        out[:, 1:1 + dim] = vel[:dim]
        out[:, dim + 1] = t
        return out
    return prim


@pytest.mark.parametrize("flux", [sdg.CENTRAL, sdg.LAX_FRIEDRICHS, sdg.EXACT])
@pytest.mark.parametrize("viscous", [None, sdg.BR1, sdg.BR2])
def test_incompressible_free_stream_2d_hybrid(flux, viscous):
    mesh = sdg.Mesh.box_2d(0.0, 0.0, 1.0, 1.0, 4, 4, periodic=True, jitter=0.1, split_fraction=0.5, seed=2)
    cfg = cases.inc_config(3, flux, viscous, mu=1e-2, c0=10.0)
    r = _oracle(mesh, cfg, _uniform(2)).residual_point()
    assert np.abs(r).max() <= 1e-10, np.abs(r).max()  # flux terms are O(p (P+1)^2 / h) ~ 30


@pytest.mark.parametrize("flux", [sdg.LAX_FRIEDRICHS, sdg.EXACT])
def test_incompressible_free_stream_3d(flux):
    mesh = sdg.Mesh.box_3d(0, 0, 0, 1, 1, 1, 3, 3, 3, periodic=True)
    cfg = cases.inc_config(2, flux, sdg.BR2, mu=1e-2, c0=10.0)
    r = _oracle(mesh, cfg, _uniform(3)).residual_point()
    assert np.abs(r).max() <= 1e-10, np.abs(r).max()  # flux terms are O(p (P+1)^2 / h) ~ 30


@pytest.mark.parametrize("dim", [2, 3])
def test_boussinesq_at_rest_is_pure_buoyancy(dim):
    """A uniform fluid at rest in a periodic box: every flux cancels and du/dt is the source itself,
    rho beta (T - Tref) g on the last momentum component (g = 1, SourceTerm.cpp:31)."""
    rho, t, beta, tref = 1.2, 0.8, 0.7, 0.5
    if dim == 2:
        mesh = sdg.Mesh.box_2d(0.0, 0.0, 1.0, 1.0, 3, 3, periodic=True, jitter=0.1, split_fraction=0.5, seed=8)
    else:
        mesh = sdg.Mesh.box_3d(0, 0, 0, 1, 1, 1, 3, 3, 3, periodic=True)
    cfg = cases.inc_config(2, sdg.EXACT, sdg.BR2, mu=1e-2, c0=5.0, source=sdg.SOURCE_BOUSSINESQ, beta=beta, tref=tref)
    r = _oracle(mesh, cfg, _uniform(dim, rho=rho, vel=(0.0, 0.0, 0.0), t=t)).residual_point()
    want = np.zeros(dim + 2)
    want[dim] = rho * beta * (t - tref) * 1.0
    np.testing.assert_allclose(r, np.broadcast_to(want, r.shape), atol=1e-10)  # pressure terms O(c0^2 rho)


@pytest.mark.parametrize("flux,viscous", [(sdg.CENTRAL, None), (sdg.LAX_FRIEDRICHS, None),
                                          (sdg.LAX_FRIEDRICHS, sdg.BR2), (sdg.CENTRAL, sdg.BR1)])
def test_uniform_internal_energy_is_carried_by_mass(flux, viscous):
    """With e uniform, the rho e equation is e times the mass equation: the internal-energy flux is e rho u
    (ConvectiveFlux.cpp:45-56, no pressure work), the LF jump is e times the density jump, and grad T = 0 so the
    conduction flux vanishes (ViscousFlux.cpp:84-101)."""
    mesh, cfg, prim, _, _, _ = cases.taylor_vortex_case(n=4, p=3, flux=flux, viscous=viscous, mu=1e-2)
    t0 = 1.0
    r = _oracle(mesh, cfg, prim).residual_point()
    e = cfg.specific_heat_constant_volume * t0
    np.testing.assert_allclose(r[:, 3], e * r[:, 0], atol=1e-11 * np.abs(r[:, 0]).max())


def test_incompressible_dt_uses_reference_sound_speed():
    """dt = CFL h_min / ((|u| + c0) (P+1)^2) (TimeIntegration.cpp:119-125 with the EOS sound speed c0)."""
    c0 = 32.0
    mesh, cfg, prim, _, _, _ = cases.taylor_vortex_case(n=4, p=2, c0=c0)
    o = _oracle(mesh, cfg, prim)
    u = prim(o.volume_points())[:, 1:3]
    h = 1.0 / 4.0
    want = 0.2 * h / ((np.sqrt((u ** 2).sum(1)).max() + c0) * 9.0)
    # the oracle takes the speed at its own volume points of the projected state: within the projection error
    assert abs(o.delta_time(0.2) - want) <= 2e-3 * want


@pytest.mark.parametrize("equation,flux", [(sdg.INCOMPRESSIBLE_EULER, sdg.HLLC),
                                           (sdg.INCOMPRESSIBLE_NAVIER_STOKES, sdg.ROE), (sdg.EULER, sdg.EXACT)])
def test_flux_model_combinations_rejected(equation, flux):
    mesh = sdg.Mesh.box_2d(0.0, 0.0, 1.0, 1.0, 2, 2, periodic=True)
    cfg = sdg.make_config(2, equation=equation, convective_flux=flux,
                          viscous_flux=sdg.BR2 if equation == sdg.INCOMPRESSIBLE_NAVIER_STOKES else sdg.VISCOUS_NONE,
                          mu=1e-2, sound_speed=10.0, density=1.0)
    with pytest.raises(RuntimeError):
        Oracle(mesh, cfg, faithful=False)
