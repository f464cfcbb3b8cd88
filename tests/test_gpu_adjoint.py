"""GPU tests of the tangent-linear model and the discrete adjoint.

Pins, for the residual R(U) = du/dt and for SSP-RK trajectories (with checkpointing):
  - JVP against central finite differences of the forward residual (step h relative 1e-6: truncation
    ~h^2, round-off ~1e-16/h, so agreement ~1e-8; tolerance 1e-6 relative L2);
  - the dot-product identity <lam, JVP(dU)> = <VJP(lam), dU> (+ the viscosity terms) to 1e-11 relative,
    which holds to round-off because both are exact derivatives of the same discrete operator;
  - the adjoint gradient of the integrated kinetic energy with respect to U_0 (a seeded random direction)
    and to mu against central finite differences of the forward trajectory (h = 1e-6, tolerance 1e-6).
The symmetric analytic flows put face points exactly on the non-differentiable sets of the Riemann
solvers (bitwise-equal wave speeds in Lax-Friedrichs' max on the vortex's symmetry lines, S* = 0 in HLLC
on the Taylor-Green's symmetry planes), where the tangent takes the branch of the forward evaluation and
central differences average the two one-sided slopes; the initial states here carry a seeded smooth
perturbation that breaks the symmetry.
"""
import numpy as np
import pytest

import subrosadg_gb300 as sdg
from subrosadg_gb300 import _abi
from tests import cases

pytestmark = pytest.mark.gpu

VISCOUS = (sdg.NAVIER_STOKES, sdg.INCOMPRESSIBLE_NAVIER_STOKES)

CASES = {
    "euler-quad-p3-roe": lambda: cases.vortex_case(n=4, p=3, flux=sdg.ROE),
    "euler-quad-p2-lf": lambda: cases.vortex_case(n=4, p=2, flux=sdg.LAX_FRIEDRICHS),
    "euler-hex-p2-hllc": lambda: cases.tgv_case(n=3, p=2, flux=sdg.HLLC),
    "euler-tet-p2-hllc": lambda: cases.tet_tgv_case(n=3, p=2, flux=sdg.HLLC),
    "euler-tet-p3-roe": lambda: cases.tet_tgv_case(n=3, p=3, flux=sdg.ROE),
    "euler-tet-box-farfield-p2-roe": lambda: cases.tet_box_case(p=2, flux=sdg.ROE),
    "ns-tet-p2-br1-roe": lambda: cases.tet_tgv_case(n=3, p=2, flux=sdg.ROE, viscous=sdg.BR1, mu=0.02),
    "ns-tet-p2-br2-hllc": lambda: cases.tet_tgv_case(n=3, p=2, flux=sdg.HLLC, viscous=sdg.BR2, mu=0.02),
    "euler-hex-p3-central": lambda: cases.tgv_case(n=3, p=3, flux=sdg.CENTRAL),
    "ns-hex-p3-br1-roe": lambda: cases.tgv_case(n=3, p=3, flux=sdg.ROE, viscous=sdg.BR1, mu=0.02),
    "ns-quad-p4-br1-hllc": lambda: cases.vortex_case(n=3, p=4, flux=sdg.HLLC, viscous=sdg.BR1, mu=0.05),
    "ns-quad-p3-br1-sutherland-lf": lambda: _sutherland(cases.vortex_case(n=4, p=3, flux=sdg.LAX_FRIEDRICHS,
                                                                          viscous=sdg.BR1, mu=0.05)),
    # Euler with boundary faces (slip walls, velocity inflow, pressure outflow, Riemann farfield)
    "euler-channel-quad-p3-roe": lambda: cases.channel_case(p=3, flux=sdg.ROE, n=3),
    "euler-channel-farfield-quad-p2-hllc": lambda: cases.channel_case(p=2, flux=sdg.HLLC, n=3,
                                                                      conditions=(sdg.RIEMANN_FARFIELD,) * 4),
    "euler-box-walls-farfield-hex-p2-roe": lambda: _box3d(p=2, flux=sdg.ROE),
    # Navier-Stokes BR1 with walls (isothermal / adiabatic no-slip, slip), inflow, outflow, farfield
    "ns-channel-walls-quad-p3-br1-roe": lambda: cases.channel_case(
        p=3, flux=sdg.ROE, n=3, viscous=sdg.BR1, mu=0.01,
        conditions=(sdg.ISOTHERMAL_NONSLIP_WALL, sdg.PRESSURE_OUTFLOW, sdg.ADIABATIC_NONSLIP_WALL, sdg.VELOCITY_INFLOW)),
    "ns-channel-farfield-quad-p2-br1-hllc": lambda: cases.channel_case(
        p=2, flux=sdg.HLLC, n=3, viscous=sdg.BR1, mu=0.02,
        conditions=(sdg.ADIABATIC_SLIP_WALL, sdg.RIEMANN_FARFIELD, sdg.ADIABATIC_SLIP_WALL, sdg.RIEMANN_FARFIELD)),
    "ns-box-walls-hex-p2-br1-roe": lambda: _box3d(p=2, flux=sdg.ROE, viscous=True),
    # BR2 (the face gradients carry each face's own lift)
    "ns-hex-p2-br2-hllc": lambda: cases.tgv_case(n=3, p=2, flux=sdg.HLLC, viscous=sdg.BR2, mu=0.02),
    "ns-quad-p3-br2-roe": lambda: cases.vortex_case(n=4, p=3, flux=sdg.ROE, viscous=sdg.BR2, mu=0.05),
    "ns-channel-walls-quad-p3-br2-roe": lambda: cases.channel_case(
        p=3, flux=sdg.ROE, n=3, viscous=sdg.BR2, mu=0.01,
        conditions=(sdg.ISOTHERMAL_NONSLIP_WALL, sdg.PRESSURE_OUTFLOW, sdg.ADIABATIC_NONSLIP_WALL, sdg.VELOCITY_INFLOW)),
    # incompressible model (weakly compressible EOS; Central / Lax-Friedrichs / Exact), Boussinesq source
    "inc-euler-shearlayer-quad-p3-exact": lambda: cases.shear_layer_case(n=4, p=3, flux=sdg.EXACT, jitter=0.0,
                                                                         split=0.0),
    "inc-euler-shearlayer-quad-p2-central": lambda: cases.shear_layer_case(n=4, p=2, flux=sdg.CENTRAL, jitter=0.0,
                                                                           split=0.0),
    "inc-ns-taylorvortex-quad-p4-exact-br2": lambda: cases.taylor_vortex_case(n=4, p=4, mu=1e-2, c0=10.0, dt=1e-4),
    "inc-ns-taylorvortex-quad-p3-lf-br1": lambda: cases.taylor_vortex_case(n=4, p=3, flux=sdg.LAX_FRIEDRICHS,
                                                                           viscous=sdg.BR1, mu=1e-2, c0=10.0, dt=1e-4),
    "inc-euler-channel-farfield-quad-p2-exact": lambda: cases.inc_channel_case(p=2, n=3),
    "inc-ns-lidcavity-quad-p3-lf-br2": lambda: cases.cavity_case(p=3, n=4, mu=1e-2),
    "inc-ns-thermalcavity-quad-p3-exact-br1-boussinesq": lambda: cases.cavity_case(
        p=3, n=4, flux=sdg.EXACT, viscous=sdg.BR1, mu=1e-2, boussinesq=True),
    "inc-ns-lidcavity-hex-p2-lf-br2": lambda: cases.cavity_3d_case(p=2, n=3, flux=sdg.LAX_FRIEDRICHS,
                                                                    viscous=sdg.BR2, mu=1e-2),
    "inc-ns-thermalcavity-hex-p2-exact-br1-boussinesq": lambda: cases.cavity_3d_case(p=2, n=3, mu=1e-2,
                                                                                      boussinesq=True),
    # 1D (line meshes): periodic, farfield ends, walls; Euler, Navier-Stokes, incompressible
    "euler-line-p3-roe": lambda: cases.density_wave_1d_case(n=8, p=3, flux=sdg.ROE),
    "euler-line-farfield-p2-hllc": lambda: cases.sod_1d_case(n=9, p=2, av=False, smooth=0.15, dt=2e-4),
    "ns-line-p4-br1-roe": lambda: cases.density_wave_1d_case(n=6, p=4, flux=sdg.ROE, viscous=sdg.BR1, mu=0.02),
    "ns-line-walls-p3-br2-roe": lambda: _ns1d(cases.sod_1d_case(
        n=9, p=3, flux=sdg.ROE, av=False, smooth=0.15, dt=2e-4,
        conditions=(sdg.ISOTHERMAL_NONSLIP_WALL, sdg.ADIABATIC_NONSLIP_WALL)), sdg.BR2, 0.02),
    "inc-line-p3-exact": lambda: cases.inc_wave_1d_case(n=8),
    # dense (modal) blocks -- triangles, first-order and bilinear quadrangles -- and hybrid meshes with bilinear
    # tensor quadrangles: the Euler equations
    "euler-tri-p2-hllc": lambda: cases.kh_case(n=4, p=2, flux=sdg.HLLC, split=1.0),
    "euler-tri-p3-central": lambda: cases.kh_case(n=4, p=3, flux=sdg.CENTRAL, split=1.0),
    "euler-tri-p5-roe": lambda: cases.kh_case(n=3, p=5, flux=sdg.ROE, split=1.0, dt=5e-5),
    "euler-quad-p1-roe-dense": lambda: cases.vortex_case(n=4, p=1, flux=sdg.ROE),
    "euler-jitter-quad-p1-hllc-bilinear": lambda: cases.kh_case(n=4, p=1, flux=sdg.HLLC, split=0.0),
    "euler-hybrid-p3-lf-bilinear": lambda: cases.kh_case(n=4, p=3, flux=sdg.LAX_FRIEDRICHS, split=0.5),
    "euler-jitter-quad-p4-roe-bilinear": lambda: cases.kh_case(n=3, p=4, flux=sdg.ROE, split=0.0, dt=1e-4),
    "euler-channel-tri-p3-roe": lambda: cases.channel_case(p=3, flux=sdg.ROE, n=3, split=1.0),
    # (the Riemann farfield takes the tangential velocity and entropy of the ghost or of the interior by the sign of
    # u.n: a jump where u.n crosses 0, as on a farfield side parallel to the stream; farfield on the stream's ends)
    "euler-channel-hybrid-farfield-p2-hllc": lambda: cases.channel_case(
        p=2, flux=sdg.HLLC, n=3, split=0.5, jitter=0.1,
        conditions=(sdg.ADIABATIC_SLIP_WALL, sdg.RIEMANN_FARFIELD, sdg.ADIABATIC_SLIP_WALL, sdg.RIEMANN_FARFIELD)),
    "inc-euler-shearlayer-tri-p3-exact": lambda: cases.shear_layer_case(n=4, p=3, flux=sdg.EXACT, split=1.0),
    "inc-euler-thermalcavity-hybrid-p2-exact-boussinesq": lambda: cases.cavity_case(
        p=2, flux=sdg.EXACT, viscous=None, mu=0.0, n=4, split=0.5, boussinesq=True, c0=3.0,
        conditions=(sdg.ADIABATIC_SLIP_WALL,) * 4),
    # Navier-Stokes on affine dense blocks (triangles, first-order quadrangles) and affine hybrids
    "ns-tri-p2-br1-roe": lambda: cases.kh_case(n=4, p=2, flux=sdg.ROE, split=1.0, viscous=sdg.BR1, mu=2e-3),
    "ns-tri-p3-br2-hllc": lambda: cases.kh_case(n=4, p=3, flux=sdg.HLLC, split=1.0, viscous=sdg.BR2, mu=2e-3),
    "ns-quad-p1-br2-roe-dense": lambda: cases.vortex_case(n=4, p=1, flux=sdg.ROE, viscous=sdg.BR2, mu=0.05),
    "ns-hybrid-p3-br1-lf": lambda: cases.kh_case(n=4, p=3, flux=sdg.LAX_FRIEDRICHS, split=0.5, jitter=0.0,
                                                 viscous=sdg.BR1, mu=2e-3),
    "ns-channel-walls-tri-p2-br2-roe": lambda: cases.channel_case(
        p=2, flux=sdg.ROE, n=3, split=1.0, viscous=sdg.BR2, mu=0.01,
        conditions=(sdg.ISOTHERMAL_NONSLIP_WALL, sdg.PRESSURE_OUTFLOW, sdg.ADIABATIC_NONSLIP_WALL, sdg.VELOCITY_INFLOW)),
    # (Central: the rounding of a dense block's weakly compressible residual is too large for the small step the
    # Exact flux's upwind switch needs; Exact on triangles is in the shear-layer case)
    "inc-ns-lidcavity-tri-p2-central-br2": lambda: cases.cavity_case(p=2, n=4, flux=sdg.CENTRAL, mu=1e-2, split=1.0),
    # Navier-Stokes on bilinear (jittered) quadrangles, alone and in the hybrid Kelvin-Helmholtz mesh of the NS
    # workload (P4, BR2, LF)
    "ns-jitter-quad-p3-br2-roe-bilinear": lambda: cases.kh_case(n=4, p=3, flux=sdg.ROE, split=0.0, viscous=sdg.BR2,
                                                                mu=2e-3),
    "ns-jitter-quad-p2-br1-hllc-bilinear": lambda: cases.kh_case(n=4, p=2, flux=sdg.HLLC, split=0.0, viscous=sdg.BR1,
                                                                 mu=2e-3),
    "ns-hybrid-jitter-p4-br2-lf": lambda: cases.kh_case(n=4, p=4, flux=sdg.LAX_FRIEDRICHS, split=0.5, viscous=sdg.BR2,
                                                        mu=2e-3, dt=1e-4),
    "ns-jitter-quad-p1-br2-roe-bilinear": lambda: cases.kh_case(n=4, p=1, flux=sdg.ROE, split=0.0, viscous=sdg.BR2,
                                                                mu=2e-3),
    "ns-jitter-quad-p1-br1-hllc-bilinear": lambda: cases.kh_case(n=5, p=1, flux=sdg.HLLC, split=0.0, viscous=sdg.BR1,
                                                                 mu=2e-3),
    "ns-channel-walls-jitter-p3-br1-roe": lambda: cases.channel_case(
        p=3, flux=sdg.ROE, n=3, jitter=0.1, viscous=sdg.BR1, mu=0.01,
        conditions=(sdg.ISOTHERMAL_NONSLIP_WALL, sdg.PRESSURE_OUTFLOW, sdg.ADIABATIC_NONSLIP_WALL, sdg.VELOCITY_INFLOW)),
    # per-face-point geometry: hexahedra that are not parallelepipeds (trilinear, and curved of geometry order 2),
    # curved quadrangles
    "euler-warped-hex-p2-hllc": lambda: cases.warped(cases.tgv_case(n=3, p=2, flux=sdg.HLLC)),
    "ns-warped-hex-p2-br1-roe": lambda: cases.warped(cases.tgv_case(n=3, p=2, flux=sdg.ROE, viscous=sdg.BR1,
                                                                    mu=0.02)),
    "ns-warped-hex-box-p2-br1-hllc": lambda: cases.warped(_box3d(p=2, flux=sdg.HLLC, viscous=True)),
    "ns-curved-hex-p2-q2-br2-lf": lambda: cases.curved_hex(cases.tgv_case(n=3, p=2, flux=sdg.LAX_FRIEDRICHS,
                                                                          viscous=sdg.BR2, mu=0.02), 2),
    "euler-curved-annulus-quad-p3-roe": lambda: cases.annulus_case(p=3, flux=sdg.ROE),
    # (walls on both circles: the outer farfield's branch switch where u.n crosses 0 on the circle would be
    # straddled by the difference quotient)
    "ns-curved-annulus-quad-p2-br1-hllc": lambda: cases.annulus_case(
        p=2, flux=sdg.HLLC, viscous=sdg.BR1, mu=0.01,
        conditions=(sdg.ADIABATIC_NONSLIP_WALL, sdg.ADIABATIC_SLIP_WALL)),
    "euler-curved-annulus-tri-p2-hllc": lambda: cases.annulus_case(p=2, flux=sdg.HLLC, split=1.0),
    "ns-curved-annulus-hybrid-p2-br2-roe": lambda: cases.annulus_case(
        p=2, flux=sdg.ROE, viscous=sdg.BR2, mu=0.01, split=0.5,
        conditions=(sdg.ADIABATIC_NONSLIP_WALL, sdg.ADIABATIC_SLIP_WALL)),
    "ns-curved-annulus-tri-p3-br1-hllc": lambda: cases.annulus_case(
        p=3, flux=sdg.HLLC, viscous=sdg.BR1, mu=0.01, split=1.0,
        conditions=(sdg.ISOTHERMAL_NONSLIP_WALL, sdg.ADIABATIC_SLIP_WALL)),
    "ns-curved-annulus-quad-p3-br2-roe": lambda: cases.annulus_case(
        p=3, flux=sdg.ROE, viscous=sdg.BR2, mu=0.01,
        conditions=(sdg.ISOTHERMAL_NONSLIP_WALL, sdg.ADIABATIC_SLIP_WALL)),
}


def _ns1d(case, viscous, mu):
    mesh, cfg, ic, bc, dt, steps = case
    return (mesh, cases.ns_config(cfg.polynomial_order, cfg.convective_flux, viscous, mu), ic, bc, dt, steps)


def _force_group(s):
    """A wall group and a force direction of the case's dimension."""
    return {1: (1, [1.0]), 2: (1, [0.3, -1.0]), 3: (3, [0.2, -1.0, 0.4])}[s.counts.dimension]


def _box3d(p=2, flux=sdg.ROE, n=3, viscous=False):
    """3D compressible box [0,2]x[0,1]x[0,1]: farfield in x; slip walls on y and z (Navier-Stokes: an isothermal
    no-slip y- wall, adiabatic no-slip elsewhere)."""
    walls = ([sdg.ISOTHERMAL_NONSLIP_WALL] + [sdg.ADIABATIC_NONSLIP_WALL] * 3 if viscous
             else [sdg.ADIABATIC_SLIP_WALL] * 4)
    mesh = sdg.Mesh.box_3d(0, 0, 0, 2.0, 1.0, 1.0, 2 * n, n, n, periodic=False,
                           boundary_conditions=[sdg.RIEMANN_FARFIELD, sdg.RIEMANN_FARFIELD] + walls)
    cfg = cases.ns_config(p, flux, sdg.BR1, 0.02) if viscous else cases.config(p, flux)

    def ic(pts):
        x, y, z = pts[:, 0], pts[:, 1], pts[:, 2]
        rho = 1.0 + 0.1 * np.sin(np.pi * x) * np.sin(np.pi * y)
        out = np.zeros((len(pts), 5))
        out[:, 0] = rho
        out[:, 1] = 0.4 + 0.05 * np.cos(np.pi * z)
        out[:, 2] = 0.05 * np.sin(np.pi * x)
        out[:, 3] = 0.03 * np.sin(np.pi * y)
        out[:, 4] = (1.0 + 0.05 * np.cos(np.pi * x)) / (rho * cases.R_GAS)
        return out

    def bc(pts, phys):
        out = np.zeros((len(pts), 5))
        out[:, 0] = 1.0
        out[:, 1] = 0.4
        out[:, 4] = 1.0 / cases.R_GAS
        return out

    return (mesh, cfg, ic, bc, 5e-4, 3)


def _sutherland(case):
    case[1].transport_model = sdg.TRANSPORT_SUTHERLAND
    return case


def smooth_perturbation(pts, nv, seed=11, amplitude=0.02):
    """Seeded sum of low-order sine modes per primitive variable (relative amplitude)."""
    rng = np.random.default_rng(seed)
    out = np.zeros((len(pts), nv))
    for v in range(nv):
        for _ in range(3):
            k = rng.integers(1, 3, size=3) * 2 * np.pi / 10.0
            out[:, v] += rng.uniform(-1, 1) * np.sin(pts @ k + rng.uniform(0, 2 * np.pi))
    return amplitude * out


def make(name):
    mesh, cfg, prim, bprim, dt, steps = CASES[name]()
    s = sdg.GpuSolver(mesh, cfg, device=0)
    pts = s.volume_points()
    p0 = prim(pts)
    s.initialize_primitive(p0 * (1.0 + smooth_perturbation(pts, p0.shape[1])))
    if s.counts.boundary_face_count:
        bpts, phys = s.boundary_points()
        s.set_boundary_primitive(bprim(bpts, np.repeat(phys, s.counts.face_point_count)))
    return s, dt


def direction(u, seed, floor=1e-3):
    """Seeded perturbation scaled per variable by the state's own magnitude (at least `floor`)."""
    rng = np.random.default_rng(seed)
    scale = np.abs(u).mean(0) + floor
    return rng.standard_normal(u.shape) * scale


def rel(a, b):
    return float(np.linalg.norm(np.ravel(a - b)) / max(np.linalg.norm(np.ravel(b)), 1e-300))


@pytest.mark.parametrize("name", list(CASES))
def test_jvp_residual_matches_central_differences(name):
    s, _ = make(name)
    u = s.state_point()
    d = direction(u, 1)
    jvp = s.jvp_residual(d)
    # Lax-Friedrichs' max(|u.n| + c) switches sides at face points where the two are within ~h of each
    # other, and the Exact flux takes its upwind side from the sign of u* (exactly 0 where the initial
    # state's normal velocity vanishes at a face point); the difference quotient straddles the switch there
    # (an error that shrinks with h), so its step is smaller
    flux = s.config.convective_flux
    h, tol = {sdg.LAX_FRIEDRICHS: (1e-8, 1e-5), sdg.EXACT: (1e-7, 1e-6)}.get(flux, (1e-6, 1e-6))
    s.set_state_point(u + h * d)
    rp = s.residual_point()
    s.set_state_point(u - h * d)
    rm = s.residual_point()
    s.set_state_point(u)
    fd = (rp - rm) / (2 * h)
    assert rel(jvp, fd) < tol, rel(jvp, fd)


@pytest.mark.parametrize("name", list(CASES))
def test_vjp_is_the_transpose_of_jvp(name):
    s, _ = make(name)
    u = s.state_point()
    d = direction(u, 2)
    lam = np.random.default_rng(3).standard_normal(u.shape)
    jvp = s.jvp_residual(d)
    vjp, mubar = s.vjp_residual(lam)
    lhs, rhs = float(np.sum(lam * jvp)), float(np.sum(vjp * d))
    assert abs(lhs - rhs) <= 1e-11 * max(abs(lhs), abs(rhs)), (lhs, rhs)
    if s.config.equation in VISCOUS:
        dmu = s.jvp_residual(np.zeros_like(u), viscosity_tangent=1.0)
        lm = float(np.sum(lam * dmu))
        assert abs(lm - mubar) <= 1e-11 * max(abs(lm), 1e-300), (lm, mubar)
        # and against differences in mu
        mu = s.config.dynamic_viscosity
        hm = 1e-6 * mu
        s.set_viscosity(mu + hm)
        rp = s.residual_point()
        s.set_viscosity(mu - hm)
        rm = s.residual_point()
        s.set_viscosity(mu)
        assert rel(dmu, (rp - rm) / (2 * hm)) < 1e-6


@pytest.mark.parametrize("name", ["euler-quad-p3-roe", "euler-hex-p2-hllc", "euler-tet-p2-hllc", "ns-tet-p2-br2-hllc", "ns-hex-p3-br1-roe",
                                  "inc-ns-taylorvortex-quad-p4-exact-br2", "inc-ns-thermalcavity-hex-p2-exact-br1-boussinesq",
                                  "ns-line-p4-br1-roe", "euler-hybrid-p3-lf-bilinear", "euler-tri-p5-roe",
                                  "ns-hybrid-p3-br1-lf", "ns-tri-p3-br2-hllc", "ns-hybrid-jitter-p4-br2-lf",
                                  "ns-jitter-quad-p1-br2-roe-bilinear",
                                  "ns-quad-p4-br1-hllc", "ns-hex-p2-br2-hllc", "ns-channel-walls-quad-p3-br2-roe",
                                  "ns-warped-hex-p2-br1-roe", "ns-curved-hex-p2-q2-br2-lf",
                                  "ns-curved-annulus-hybrid-p2-br2-roe"])
def test_trajectory_dot_product_with_checkpointing(name):
    steps, interval = 5, 2
    a, dt = make(name)
    b, _ = make(name)
    u0 = a.state_point()
    d0 = direction(u0, 4)
    dmu = 0.3 if a.config.equation in VISCOUS else 0.0
    dN = a.jvp_steps(dt, steps, d0, viscosity_tangent=dmu)
    uN_tlm = a.state_point()
    lamN = np.random.default_rng(5).standard_normal(u0.shape)
    lam0, mubar = b.adjoint_steps(dt, steps, lamN, checkpoint_interval=interval)
    uN_adj = b.state_point()
    # both leave the handle at U_N, equal to a plain forward run
    c, _ = make(name)
    c.stepSolver(dt, steps)
    assert np.array_equal(uN_tlm, c.state_point())
    assert np.array_equal(uN_adj, c.state_point())
    lhs = float(np.sum(lamN * dN))
    rhs = float(np.sum(lam0 * d0)) + mubar * dmu
    assert abs(lhs - rhs) <= 1e-11 * max(abs(lhs), abs(rhs)), (lhs, rhs)


def test_checkpoint_interval_does_not_change_the_adjoint():
    lams = []
    for interval in (1, 3, 7):
        s, dt = make("ns-hex-p3-br1-roe")
        lamN = np.random.default_rng(6).standard_normal(s.state_point().shape)
        lam0, mubar = s.adjoint_steps(dt, 6, lamN, checkpoint_interval=interval)
        lams.append((lam0, mubar))
    for lam0, mubar in lams[1:]:
        assert np.array_equal(lam0, lams[0][0])
        assert mubar == lams[0][1]


@pytest.mark.parametrize("name", ["ns-hex-p3-br1-roe", "euler-hybrid-p3-lf-bilinear", "ns-tet-p2-br2-hllc"])
def test_trajectory_store_gives_the_checkpointed_adjoint(name):
    """Keeping every stage input on the forward sweep (no segment recompute) gives the checkpoint scheme's
    gradient bit for bit, in the one-call and in the recorded form, and leaves the same final state."""
    a, dt = make(name)
    b, _ = make(name)
    lamN = np.random.default_rng(12).standard_normal(a.state_point().shape)
    lam_a, mu_a = a.adjoint_steps(dt, 7, lamN, checkpoint_interval=3)
    b.set_adjoint_trajectory_store(True)
    lam_b, mu_b = b.adjoint_steps(dt, 7, lamN, checkpoint_interval=3)
    assert np.array_equal(b.state_point(), a.state_point())
    assert np.array_equal(lam_a, lam_b) and mu_a == mu_b
    c, _ = make(name)
    c.set_adjoint_trajectory_store(True)
    c.forward_steps(dt, 7, checkpoint_interval=3)
    lam_c, mu_c = c.adjoint_recorded(lamN)
    assert np.array_equal(lam_a, lam_c) and mu_a == mu_c
    held = c.adjoint_memory()
    assert held >= (7 * 3 + 4) * c.counts.degree_of_freedom_count * 8


# HLLC and Lax-Friedrichs switch branches (PVRS pressure against each side's pressure, the larger wave
# speed) at many face points of a low-Mach trajectory, where difference quotients straddle the switches;
# the trajectory checks use the smooth fluxes (cfg: Roe + BR1 is the adjoint workload)
@pytest.mark.parametrize("name", ["euler-hex-p3-central", "ns-hex-p3-br1-roe", "euler-quad-p3-roe",
                                  "inc-ns-taylorvortex-quad-p4-exact-br2", "inc-euler-shearlayer-quad-p2-central",
                                  "ns-line-walls-p3-br2-roe", "euler-tri-p3-central", "ns-tri-p2-br1-roe",
                                  "ns-jitter-quad-p3-br2-roe-bilinear", "ns-warped-hex-p2-br1-roe",
                                  "euler-curved-annulus-quad-p3-roe"])
def test_kinetic_energy_gradient_matches_finite_differences(name):
    steps, interval = 6, 3
    s, dt = make(name)
    u0 = s.state_point()
    w = s.volume_weights()
    d0 = direction(u0, 7)

    def J(u, mu=None):
        if mu is not None:
            s.set_viscosity(mu)
        s.set_state_point(u)
        s.stepSolver(dt, steps)
        return s.kinetic_energy(weights=w)[0]

    mu0 = s.config.dynamic_viscosity
    J0 = J(u0)
    _, lamN = s.kinetic_energy(weights=w)
    s.set_state_point(u0)
    lam0, mubar = s.adjoint_steps(dt, steps, lamN, checkpoint_interval=interval)
    h = 1e-6
    fd = (J(u0 + h * d0) - J(u0 - h * d0)) / (2 * h)
    ad = float(np.sum(lam0 * d0))
    assert abs(fd - ad) <= 1e-6 * max(abs(fd), abs(ad)), (fd, ad, J0)
    if s.config.equation in VISCOUS:
        hm = 1e-6 * mu0
        fdm = (J(u0, mu0 + hm) - J(u0, mu0 - hm)) / (2 * hm)
        s.set_viscosity(mu0)
        assert abs(fdm - mubar) <= 1e-6 * max(abs(fdm), abs(mubar)), (fdm, mubar)


def test_torch_autograd_binding():
    import torch

    from subrosadg_gb300 import autograd as sa
    s, dt = make("ns-hex-p3-br1-roe")
    u0 = torch.from_numpy(s.state_point()).requires_grad_(True)
    mu = torch.tensor(s.config.dynamic_viscosity, dtype=torch.float64, requires_grad=True)
    uN = sa.trajectory(s, u0, mu, steps=4, dt=dt, checkpoint_interval=2)
    J = sa.kinetic_energy(s, uN)
    J.backward()
    # the same gradient through the C ABI directly
    t, _ = make("ns-hex-p3-br1-roe")
    t.stepSolver(dt, 4)
    _, lamN = t.kinetic_energy()
    t2, _ = make("ns-hex-p3-br1-roe")
    lam0, mubar = t2.adjoint_steps(dt, 4, lamN, checkpoint_interval=2)
    assert np.allclose(u0.grad.numpy(), lam0, rtol=1e-12, atol=1e-14 * np.abs(lam0).max())
    assert abs(float(mu.grad) - mubar) <= 1e-10 * abs(mubar)


def test_derivatives_refuse_unsupported_configurations():
    mesh, cfg, ic, bc, _, _ = cases.shock_tube_case(p=2, n=8)  # artificial viscosity is not differentiated
    walls = sdg.GpuSolver(mesh, cfg, device=0)
    walls.initialize_primitive(ic(walls.volume_points()))
    with pytest.raises(sdg.SdgError) as e:
        walls.vjp_residual(np.zeros((walls.counts.volume_point_count, 4)))
    assert e.value.code == _abi.SDG_ERR_UNSUPPORTED
    mesh, cfg, ic, _, _, _ = cases.tet_tgv_case(n=3, p=4, flux=sdg.ROE)  # tetrahedra P4: no derivative kernels
    tet = sdg.GpuSolver(mesh, cfg, device=0)
    tet.initialize_primitive(ic(tet.volume_points()))
    with pytest.raises(sdg.SdgError) as e:
        tet.vjp_residual(np.zeros((tet.counts.volume_point_count, 5)))
    assert e.value.code == _abi.SDG_ERR_UNSUPPORTED


def test_recorded_trajectory_adjoint_equals_the_one_call_adjoint():
    a, dt = make("ns-hex-p3-br1-roe")
    b, _ = make("ns-hex-p3-br1-roe")
    lamN = np.random.default_rng(8).standard_normal(a.state_point().shape)
    lam_a, mu_a = a.adjoint_steps(dt, 5, lamN, checkpoint_interval=2)
    b.forward_steps(dt, 5, checkpoint_interval=2)
    assert np.array_equal(b.state_point(), a.state_point())
    lam_b, mu_b = b.adjoint_recorded(lamN)
    assert np.array_equal(lam_a, lam_b) and mu_a == mu_b
    # any state change in between invalidates the recorded trajectory
    b.forward_steps(dt, 2, checkpoint_interval=2)
    b.stepSolver(dt, 1)
    with pytest.raises(sdg.SdgError) as e:
        b.adjoint_recorded(lamN)
    assert e.value.code == _abi.SDG_ERR_STATE


# ---- surface force and boundary (freestream) gradients (Euler) -------------------------------------------

def test_surface_force_of_a_fluid_at_rest_is_the_pressure_times_the_area():
    """Uniform fluid at rest at p0 in a closed slip box [0,2]x[0,1]: the bottom wall (group 1, outward normal
    -y) carries (0, -2 p0), the right wall (group 2) (p0, 0)."""
    mesh = sdg.Mesh.box_2d(0.0, 0.0, 2.0, 1.0, 4, 2, periodic=False, boundary_conditions=[sdg.ADIABATIC_SLIP_WALL] * 4)
    s = sdg.GpuSolver(mesh, cases.config(3, sdg.HLLC), device=0)
    p0 = 1.7
    prim = np.zeros((s.counts.volume_point_count, 4))
    prim[:, 0] = 1.2
    prim[:, 3] = p0 / (1.2 * cases.R_GAS)
    s.initialize_primitive(prim)
    bpts, _ = s.boundary_points()
    s.set_boundary_primitive(np.repeat(prim[:1], len(bpts), 0))
    np.testing.assert_allclose(s.surface_force(1), [0.0, -2.0 * p0], rtol=1e-14, atol=1e-14)
    np.testing.assert_allclose(s.surface_force(2), [p0, 0.0], rtol=1e-14, atol=1e-14)


@pytest.mark.parametrize("name", ["euler-channel-quad-p3-roe", "euler-box-walls-farfield-hex-p2-roe",
                                  "ns-channel-walls-quad-p3-br1-roe", "ns-box-walls-hex-p2-br1-roe",
                                  "inc-ns-thermalcavity-quad-p3-exact-br1-boussinesq", "inc-ns-lidcavity-hex-p2-lf-br2",
                                  "ns-line-walls-p3-br2-roe", "euler-channel-tri-p3-roe",
                                  "euler-channel-hybrid-farfield-p2-hllc", "ns-channel-walls-tri-p2-br2-roe",
                                  "ns-warped-hex-box-p2-br1-hllc", "ns-curved-annulus-tri-p3-br1-hllc"])
def test_surface_force_cotangent_matches_central_differences(name):
    s, _ = make(name)
    group, e = _force_group(s)
    u = s.state_point()
    cot = s.surface_force_cotangent(group, e)
    d = direction(u, 5)
    h = 1e-6
    s.set_state_point(u + h * d)
    jp = float(np.dot(s.surface_force(group), e))
    s.set_state_point(u - h * d)
    jm = float(np.dot(s.surface_force(group), e))
    s.set_state_point(u)
    fd = (jp - jm) / (2 * h)
    assert abs(float(np.sum(cot * d)) - fd) <= 1e-7 * abs(fd), (float(np.sum(cot * d)), fd)


@pytest.mark.parametrize("name", ["euler-channel-quad-p3-roe", "euler-channel-farfield-quad-p2-hllc",
                                  "euler-box-walls-farfield-hex-p2-roe", "ns-channel-walls-quad-p3-br1-roe",
                                  "ns-channel-farfield-quad-p2-br1-hllc", "ns-box-walls-hex-p2-br1-roe",
                                  "ns-channel-walls-quad-p3-br2-roe", "inc-euler-channel-farfield-quad-p2-exact",
                                  "inc-ns-lidcavity-quad-p3-lf-br2", "inc-ns-thermalcavity-quad-p3-exact-br1-boussinesq",
                                  "inc-ns-thermalcavity-hex-p2-exact-br1-boussinesq", "euler-line-farfield-p2-hllc",
                                  "ns-line-walls-p3-br2-roe", "euler-channel-tri-p3-roe",
                                  "euler-channel-hybrid-farfield-p2-hllc", "ns-channel-walls-tri-p2-br2-roe",
                                  "inc-ns-lidcavity-tri-p2-central-br2", "ns-channel-walls-jitter-p3-br1-roe"])
def test_force_gradient_through_a_trajectory(name):
    """J = e . force on a wall after N steps: dJ/dU_0 in a seeded direction and dJ/d(boundary primitives) in a
    seeded direction of every boundary point's (rho, u, T), against central differences of the trajectory."""
    s, dt = make(name)
    group, e = _force_group(s)
    steps = 6
    u0 = s.state_point()
    bpts, phys = s.boundary_points()
    g0 = CASES[name]()[3](bpts, np.repeat(phys, s.counts.face_point_count))

    def J(u, g):
        s.set_state_point(u)
        s.set_boundary_primitive(g)
        s.stepSolver(dt, steps)
        return float(np.dot(s.surface_force(group), e))

    s.set_state_point(u0)
    s.set_boundary_primitive(g0)
    s.forward_steps(dt, steps, 2)
    cot = s.surface_force_cotangent(group, e)
    gu, gmu = s.adjoint_recorded(cot)
    gg = s.adjoint_boundary_cotangent()
    # the weakly compressible pressure c0^2 (rho - rho0) scales the density's rounding by c0^2, so the
    # difference quotients of the incompressible cases take larger steps (round-off ~ 1e-14 / h) and a ghost
    # direction whose zero velocities (walls at rest) are perturbed at 0.1
    inc = s.config.equation in (sdg.INCOMPRESSIBLE_EULER, sdg.INCOMPRESSIBLE_NAVIER_STOKES)
    du = direction(u0, 7)
    dg = direction(g0, 8, floor=0.1 if inc else 1e-3)
    h = 1e-5 if inc else 1e-6
    fd_u = (J(u0 + h * du, g0) - J(u0 - h * du, g0)) / (2 * h)
    fd_g = (J(u0, g0 + h * dg) - J(u0, g0 - h * dg)) / (2 * h)
    assert abs(float(np.sum(gu * du)) - fd_u) <= 1e-6 * abs(fd_u), (float(np.sum(gu * du)), fd_u)
    assert abs(float(np.sum(gg * dg)) - fd_g) <= 1e-6 * abs(fd_g), (float(np.sum(gg * dg)), fd_g)
    if s.config.equation in VISCOUS:
        # and the viscosity: the adjoint gives the trajectory's part, the force's own (tau is linear in mu)
        # is its value at U_N with the state held
        mu = s.config.dynamic_viscosity
        hm = (1e-4 if inc else 1e-6) * mu
        s.set_state_point(u0)
        s.set_boundary_primitive(g0)
        s.stepSolver(dt, steps)
        s.set_viscosity(mu + hm)
        fp = float(np.dot(s.surface_force(group), e))
        s.set_viscosity(mu - hm)
        fm = float(np.dot(s.surface_force(group), e))
        direct = (fp - fm) / (2 * hm)
        s.set_viscosity(mu + hm)
        jp = J(u0, g0)
        s.set_viscosity(mu - hm)
        jm = J(u0, g0)
        s.set_viscosity(mu)
        fd_mu = (jp - jm) / (2 * hm)
        assert abs(gmu + direct - fd_mu) <= 1e-6 * abs(fd_mu), (gmu, direct, fd_mu)
