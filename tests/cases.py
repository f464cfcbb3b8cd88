"""Seeded synthetic test cases: the benchmark workloads (re-exported from subrosadg_gb300.workloads) plus the
boundary-condition, incompressible, artificial-viscosity and 1D cases of the parity tests.

Each *_case returns (mesh, config, initial primitive function of the volume points, boundary primitive
function or None, dt, steps).  Thermodynamics follow the example drivers: cp = 2.5, cv = 25/14 (R = 1/1.4),
gamma = 1.4 (examples/periodic_2d_ceuler.cpp:51).
"""
from __future__ import annotations

import math

import numpy as np

import subrosadg_gb300 as sdg
from subrosadg_gb300.workloads import (CP, CV, GAMMA, R_GAS, batch_instances, config, curved_hex,  # noqa: F401
                                       hex_lattice, kh_case, kh_primitive, ns_config, tet_mesh, tet_tgv_case, tgv_case,
                                       tgv_primitive, uniform_primitive, vortex_case, vortex_primitive, warped)


def tet_box_case(p=2, flux=sdg.HLLC, conditions=(sdg.RIEMANN_FARFIELD,) * 6, n=3, dt=5e-4, steps=3, viscous=None,
                 mu=0.01):
    """Non-periodic tetrahedral unit box, groups x-, x+, y-, y+, z-, z+: a smooth perturbation of a uniform
    stream at u = (0.4, 0.1, -0.1), the same stream as the boundary state (inflow at x-, outflow at x+)."""
    mesh = tet_mesh(n, 1.0, periodic=False, conditions=conditions)

    def ic(pts):
        x, y, z = pts[:, 0], pts[:, 1], pts[:, 2]
        rho = 1.0 + 0.1 * np.sin(math.pi * x) * np.sin(math.pi * y) * np.sin(math.pi * z)
        u = 0.4 + 0.05 * np.cos(math.pi * y)
        v = 0.1 + 0.05 * np.sin(math.pi * z)
        w = -0.1 + 0.05 * np.sin(math.pi * x)
        pr = 1.0 + 0.05 * np.cos(math.pi * x) * np.cos(math.pi * z)
        return np.stack([rho, u, v, w, pr / (rho * R_GAS)], 1)

    def bc(pts, phys):
        out = np.zeros((len(pts), 5))
        out[:, 0] = 1.0
        out[:, 1], out[:, 2], out[:, 3] = 0.4, 0.1, -0.1
        out[:, 4] = 1.0 / R_GAS
        return out

    cfg = config(p, flux) if viscous is None else ns_config(p, flux, viscous, mu)
    return (mesh, cfg, ic, bc, dt, steps)


def hex_box_case(p=2, flux=sdg.HLLC, conditions=(sdg.RIEMANN_FARFIELD,) * 6, n=3, **kw):
    """tet_box_case's flow, states and groups on n^3 hexahedra of the same unit box."""
    _, cfg, ic, bc, dt, steps = tet_box_case(p=p, flux=flux, conditions=conditions, n=n, **kw)
    mesh = sdg.Mesh.box_3d(0, 0, 0, 1, 1, 1, n, n, n, periodic=False, boundary_conditions=list(conditions))
    return (mesh, cfg, ic, bc, dt, steps)


def channel_case(p=2, flux=sdg.HLLC, conditions=(sdg.ADIABATIC_SLIP_WALL, sdg.PRESSURE_OUTFLOW,
                                                  sdg.ADIABATIC_SLIP_WALL, sdg.VELOCITY_INFLOW),
                 n=6, dt=5e-4, steps=3, jitter=0.0, split=0.0, viscous=None, mu=0.0,
                 transport=sdg.TRANSPORT_CONSTANT):
    """Non-periodic box with boundary groups bottom/right/top/left (all six BC kinds testable)."""
    mesh = sdg.Mesh.box_2d(0.0, 0.0, 2.0, 1.0, 2 * n, n, periodic=False, jitter=jitter, split_fraction=split,
                           seed=5, boundary_conditions=list(conditions))
    cfg = config(p, flux) if viscous is None else ns_config(p, flux, viscous, mu, transport=transport)

    def ic(pts):
        x, y = pts[:, 0], pts[:, 1]
        rho = 1.0 + 0.1 * np.sin(math.pi * x) * np.sin(math.pi * y)
        u = 0.4 + 0.05 * np.cos(math.pi * y)
        v = 0.05 * np.sin(math.pi * x)
        p = 1.0 + 0.05 * np.cos(math.pi * x)
        return np.stack([rho, u, v, p / (rho * R_GAS)], 1)

    def bc(pts, phys):
        n_ = len(pts)
        out = np.zeros((n_, 4))
        out[:, 0] = 1.0
        out[:, 1] = np.where(phys == 4, 0.4, 0.0)
        out[:, 2] = 0.0
        out[:, 3] = np.where(phys == 1, 1.2, 1.0) / R_GAS  # a warmer bottom wall (isothermal case)
        return out

    return (mesh, cfg, ic, bc, dt, steps)


# ---- 1D (DimensionEnum::D1, line meshes): the reference's 1D drivers ------------------------------------------

def density_wave_1d_case(n=40, p=3, flux=sdg.HLLC, dt=1e-4, steps=5, viscous=None, mu=0.0):
    """Periodic density wave on [0, 2] (examples/periodic_1d_ceuler.cpp:31-38, 63-77): rho = 1 + 0.2 sin(pi x),
    u = 1, T = 1.4 / rho (p = 1); Navier-Stokes with `viscous`."""
    mesh = sdg.Mesh.line_1d(0.0, 2.0, n, periodic=True)
    cfg = config(p, flux) if viscous is None else ns_config(p, flux, viscous, mu)

    def ic(pts):
        rho = 1.0 + 0.2 * np.sin(math.pi * pts[:, 0])
        return np.stack([rho, np.ones_like(rho), 1.4 / rho], 1)

    return (mesh, cfg, ic, None, dt, steps)


def sod_1d_case(n=100, p=3, flux=sdg.HLLC, tolerance=0.5, factor=1.0, dt=2e-6, steps=4,
                conditions=(sdg.RIEMANN_FARFIELD, sdg.RIEMANN_FARFIELD), av=True, smooth=0.0):
    """Sod's tube with a left stream on [0, 1] (examples/sod_1d_ceuler.cpp:28-50, 56-82): (rho, u, T) =
    (1, 0.75, 1.4) | (0.125, 0, 1.12) at x = 0.5, farfield ends holding the two states, artificial viscosity.
    With the driver's 100 elements the jump lies on an element boundary, where the sensor sees constant
    elements (no artificial viscosity until the jump has spread into them).  Inside an element a sharp jump's
    interpolant overshoots to negative end-point traces at P >= 2 (the reference's own projection does the
    same); `smooth` > 0 spreads it as a tanh of that width instead."""
    mesh = sdg.Mesh.line_1d(0.0, 1.0, n, periodic=False, boundary_conditions=list(conditions))
    left, right = np.array([1.0, 0.75, 1.4]), np.array([0.125, 0.0, 0.8 * 1.4])

    def ic(pts):
        if smooth > 0:
            t = 0.5 * (1.0 + np.tanh((pts[:, 0] - 0.5) / smooth))[:, None]
            return left * (1.0 - t) + right * t
        return np.where((pts[:, 0] <= 0.5)[:, None], left, right)

    def bc(pts, phys):
        return np.where((phys == 1)[:, None], left, right)

    case = (mesh, config(p, flux), ic, bc, dt, steps)
    return with_av(case, tolerance, factor) if av else case


def shu_osher_1d_case(n=100, p=3, flux=sdg.HLLC, tolerance=3.0, factor=1.0, dt=2e-5, steps=4, smooth=0.0):
    """Shu-Osher shock / entropy-wave interaction on [-5, 5] (examples/shuosher_1d_ceuler.cpp:28-52, 58-84):
    (3.857143, 2.629369, 3.750342) for x <= -4, else rho = 1 + 0.2 sin 5x, u = 0, T = 1.4 / rho."""
    mesh = sdg.Mesh.line_1d(-5.0, 10.0, n, periodic=False, boundary_conditions=[sdg.RIEMANN_FARFIELD] * 2)
    post = np.array([3.857143, 2.629369, 3.750342])
    far = np.array([1.0 + 0.2 * math.sin(25.0), 0.0, 1.4 / (1.0 + 0.2 * math.sin(25.0))])

    def ic(pts):
        x = pts[:, 0]
        rho = 1.0 + 0.2 * np.sin(5.0 * x)
        wave = np.stack([rho, np.zeros_like(x), 1.4 / rho], 1)
        if smooth > 0:
            t = 0.5 * (1.0 + np.tanh((x + 4.0) / smooth))[:, None]
            return post * (1.0 - t) + wave * t
        return np.where((x <= -4.0)[:, None], post, wave)

    def bc(pts, phys):
        return np.where((phys == 1)[:, None], post, far)

    return with_av((mesh, config(p, flux), ic, bc, dt, steps), tolerance, factor)


def inc_wave_1d_case(n=20, p=3, flux=sdg.EXACT, viscous=None, mu=0.0, c0=3.0, dt=1e-4, steps=4):
    """Weakly compressible acoustic / entropy wave on the periodic segment [0, 1].  The momentum residual
    c0^2 d(rho)/dx moves by ~ulp(rho) (P+1)^2 / h relative to c0^2 drho k under one ulp of rounding of the state:
    a 2 % density wave keeps that FP64 floor near 1e-13 (a 0.2 % wave puts it at ~1e-12)."""
    mesh = sdg.Mesh.line_1d(0.0, 1.0, n, periodic=True)
    cfg = inc_config(p, flux, viscous, mu, c0)

    def ic(pts):
        x = pts[:, 0]
        return np.stack([1.0 + 0.02 * np.sin(2 * math.pi * x), 0.3 + 0.05 * np.cos(2 * math.pi * x),
                         1.0 + 0.1 * np.sin(4 * math.pi * x)], 1)

    return (mesh, cfg, ic, None, dt, steps)


# ---- incompressible model (weakly compressible EOS p = c0^2 (rho - rho0) + 0.01 rho0 c0^2, cp = cv = 1) ----------
# Workload shapes follow the reference's incompressible example drivers (examples/taylorvortex_2d_incns.cpp,
# lidcavity_2d_incns.cpp, thermalcavity_2d_incns.cpp, shearlayer_2d_inceuler.cpp): rho0 = 1, cp = cv = 1,
# Pr = 0.71; primitive temperature T = e / cv.

def inc_config(p, flux, viscous=None, mu=0.0, c0=10.0, rho0=1.0, source=sdg.SOURCE_NONE, beta=0.0, tref=0.0,
               transport=sdg.TRANSPORT_CONSTANT):
    eq = sdg.INCOMPRESSIBLE_EULER if viscous is None else sdg.INCOMPRESSIBLE_NAVIER_STOKES
    return sdg.make_config(p, equation=eq, convective_flux=flux,
                           viscous_flux=sdg.VISCOUS_NONE if viscous is None else viscous, cp=1.0, cv=1.0, gamma=GAMMA,
                           mu=mu, transport=transport, sound_speed=c0, density=rho0, source=source,
                           thermal_expansion=beta, reference_temperature=tref)


def taylor_vortex_case(n=6, p=4, flux=sdg.EXACT, viscous=sdg.BR2, mu=1e-3, c0=32.0, dt=2e-5, steps=3,
                       jitter=0.0, split=0.0):
    """Incompressible Taylor vortex on the periodic unit square (examples/taylorvortex_2d_incns.cpp:31-44):
    rho = 0.99 + (cos 4 pi x + cos 4 pi y) / (4 c0^2), u = sin 2 pi x cos 2 pi y, v = -cos 2 pi x sin 2 pi y, T = 1."""
    mesh = sdg.Mesh.box_2d(0.0, 0.0, 1.0, 1.0, n, n, periodic=True, jitter=jitter, split_fraction=split, seed=3)
    cfg = inc_config(p, flux, viscous, mu, c0)

    def ic(pts):
        x, y = pts[:, 0], pts[:, 1]
        rho = (np.cos(4 * math.pi * x) + np.cos(4 * math.pi * y)) / 4.0 / c0 ** 2 + 0.99
        u = np.sin(2 * math.pi * x) * np.cos(2 * math.pi * y)
        v = -np.cos(2 * math.pi * x) * np.sin(2 * math.pi * y)
        return np.stack([rho, u, v, np.ones_like(x)], 1)

    return (mesh, cfg, ic, None, dt, steps)


def shear_layer_case(n=6, p=3, flux=sdg.LAX_FRIEDRICHS, c0=10.0, dt=1e-4, steps=3, jitter=0.1, split=0.5,
                     viscous=None, mu=0.0):
    """Incompressible double shear layer on the periodic unit square (shearlayer_2d_inceuler.cpp shape):
    u = tanh(80 (y - 1/4)) or tanh(80 (3/4 - y)), v = 0.05 sin(2 pi x), rho = 1, T = 1 + 0.1 sin(2 pi y)."""
    mesh = sdg.Mesh.box_2d(0.0, 0.0, 1.0, 1.0, n, n, periodic=True, jitter=jitter, split_fraction=split, seed=9)
    cfg = inc_config(p, flux, viscous, mu, c0)

    def ic(pts):
        x, y = pts[:, 0], pts[:, 1]
        u = np.where(y <= 0.5, np.tanh(30.0 * (y - 0.25)), np.tanh(30.0 * (0.75 - y)))
        v = 0.05 * np.sin(2 * math.pi * x)
        rho = np.ones_like(x) + 0.002 * np.cos(2 * math.pi * x)
        return np.stack([rho, u, v, 1.0 + 0.1 * np.sin(2 * math.pi * y)], 1)

    return (mesh, cfg, ic, None, dt, steps)


def cavity_case(p=3, flux=sdg.LAX_FRIEDRICHS, viscous=sdg.BR2, mu=2e-3, c0=10.0, n=5, dt=2e-4, steps=3,
                jitter=0.0, split=0.0, conditions=None, boussinesq=False, lid=1.0):
    """Lid-driven (lidcavity_2d_incns.cpp) or differentially heated (thermalcavity_2d_incns.cpp, Boussinesq
    beta = 1, Tref = 0.5) unit cavity; groups bottom/right/top/left.  The lid case moves the top wall at `lid`;
    the thermal case holds the right wall at T = 0 and the left at T = 1."""
    if conditions is None:
        conditions = ((sdg.ADIABATIC_NONSLIP_WALL, sdg.ISOTHERMAL_NONSLIP_WALL, sdg.ADIABATIC_NONSLIP_WALL,
                       sdg.ISOTHERMAL_NONSLIP_WALL) if boussinesq else (sdg.ADIABATIC_NONSLIP_WALL,) * 4)
    mesh = sdg.Mesh.box_2d(0.0, 0.0, 1.0, 1.0, n, n, periodic=False, jitter=jitter, split_fraction=split, seed=4,
                           boundary_conditions=list(conditions))
    cfg = inc_config(p, flux, viscous, mu, c0, source=sdg.SOURCE_BOUSSINESQ if boussinesq else sdg.SOURCE_NONE,
                     beta=1.0 if boussinesq else 0.0, tref=0.5 if boussinesq else 0.0)

    def ic(pts):
        x, y = pts[:, 0], pts[:, 1]
        rho = 1.0 + 0.003 * np.sin(math.pi * x) * np.sin(math.pi * y)
        u = 0.1 * np.sin(math.pi * x) * np.sin(2 * math.pi * y)
        v = -0.1 * np.sin(2 * math.pi * x) * np.sin(math.pi * y)
        t = 0.5 + 0.3 * (0.5 - x) + 0.05 * np.sin(math.pi * y)
        return np.stack([rho, u, v, t], 1)

    def bc(pts, phys):
        out = np.zeros((len(pts), 4))
        out[:, 0] = 1.0
        out[:, 1] = np.where(phys == 3, 0.0 if boussinesq else lid, 0.0)
        out[:, 3] = np.where(phys == 4, 1.0, np.where(phys == 2, 0.0, 0.5))
        return out

    return (mesh, cfg, ic, bc, dt, steps)


def inc_channel_case(p=2, flux=sdg.EXACT, viscous=None, mu=0.0, c0=10.0, n=4, dt=2e-4, steps=3, split=0.0,
                     conditions=(sdg.ADIABATIC_SLIP_WALL, sdg.RIEMANN_FARFIELD, sdg.ADIABATIC_SLIP_WALL,
                                 sdg.RIEMANN_FARFIELD)):
    """Incompressible flow through [0,2]x[0,1] at u = 0.4 with farfield / inflow / outflow groups
    (the cylinder and aerofoil drivers' boundary set)."""
    mesh = sdg.Mesh.box_2d(0.0, 0.0, 2.0, 1.0, 2 * n, n, periodic=False, split_fraction=split, seed=6,
                           boundary_conditions=list(conditions))
    cfg = inc_config(p, flux, viscous, mu, c0)

    def ic(pts):
        x, y = pts[:, 0], pts[:, 1]
        rho = 1.0 + 0.004 * np.sin(math.pi * x) * np.sin(math.pi * y)
        u = 0.4 + 0.05 * np.cos(math.pi * y)
        v = 0.05 * np.sin(math.pi * x)
        return np.stack([rho, u, v, 1.0 + 0.05 * np.cos(math.pi * x)], 1)

    def bc(pts, phys):
        out = np.zeros((len(pts), 4))
        out[:, 0] = np.where(phys == 2, 0.999, 1.0)
        out[:, 1] = 0.4
        out[:, 3] = 1.0
        return out

    return (mesh, cfg, ic, bc, dt, steps)


def cavity_3d_case(p=2, flux=sdg.EXACT, viscous=sdg.BR1, mu=2e-3, c0=10.0, n=3, dt=2e-4, steps=3, boussinesq=False,
                   tets=False):
    """3D cavity on hexahedra (lidcavity_3d_incns.cpp / thermalcavity_3d_incns.cpp shapes); groups
    x-, x+, y-, y+, z-, z+.  Lid: the z+ wall moves at u = 1.  Thermal: x- at T = 1, x+ at T = 0, buoyancy
    on w."""
    conds = ([sdg.ISOTHERMAL_NONSLIP_WALL, sdg.ISOTHERMAL_NONSLIP_WALL] + [sdg.ADIABATIC_NONSLIP_WALL] * 4
             if boussinesq else [sdg.ADIABATIC_NONSLIP_WALL] * 6)
    mesh = (tet_mesh(n, 1.0, periodic=False, conditions=conds) if tets else
            sdg.Mesh.box_3d(0, 0, 0, 1, 1, 1, n, n, n, periodic=False, boundary_conditions=conds))
    cfg = inc_config(p, flux, viscous, mu, c0, source=sdg.SOURCE_BOUSSINESQ if boussinesq else sdg.SOURCE_NONE,
                     beta=1.0 if boussinesq else 0.0, tref=0.5 if boussinesq else 0.0)

    def ic(pts):
        x, y, z = pts[:, 0], pts[:, 1], pts[:, 2]
        rho = 1.0 + 0.003 * np.sin(math.pi * x) * np.sin(math.pi * y) * np.sin(math.pi * z)
        u = 0.1 * np.sin(math.pi * x) * np.sin(2 * math.pi * z)
        v = 0.05 * np.sin(math.pi * y) * np.sin(math.pi * x)
        w = -0.1 * np.sin(2 * math.pi * x) * np.sin(math.pi * z)
        t = 0.5 + 0.3 * (0.5 - x) + 0.05 * np.sin(math.pi * z)
        return np.stack([rho, u, v, w, t], 1)

    def bc(pts, phys):
        out = np.zeros((len(pts), 5))
        out[:, 0] = 1.0
        out[:, 1] = np.where(phys == 6, 0.0 if boussinesq else 1.0, 0.0)
        out[:, 4] = np.where(phys == 1, 1.0, np.where(phys == 2, 0.0, 0.5))
        return out

    return (mesh, cfg, ic, bc, dt, steps)


# ---- artificial viscosity (shock capturing, System::setArtificialViscosity) -------------------------------
# The reference's shock drivers (examples/sodshock/explosion/sedovblast/khinstability_2d_ceuler.cpp) run
# compressible Euler with setArtificialViscosity(kappa[, factor]).

def with_av(case, tolerance=1.0, factor=1.0):
    """The same case with artificial viscosity switched on."""
    mesh, cfg, ic, bc, dt, steps = case
    cfg.shock_capturing = sdg.ARTIFICIAL_VISCOSITY
    cfg.empirical_tolerance = tolerance
    cfg.artificial_viscosity_factor = factor
    return (mesh, cfg, ic, bc, dt, steps)


def shock_tube_case(p=3, flux=sdg.HLLC, n=8, dt=2e-4, steps=3, split=0.0, jitter=0.0, dim=2, tolerance=1.0,
                    factor=1.0, tets=False, width=0.02):
    """Sod's shock tube (rho, p) = (1, 1) | (0.125, 0.1) at x = 0.5 in a slip-walled box [0,1] x [0,1/4]
    (x [0,1/4] in 3D; `tets`: tetrahedra), smoothed over `width` (a few % of the length) so the projected state
    stays positive."""
    if dim == 3 and tets:
        mesh = sdg.Mesh.box_3d_tetrahedra(0, 0, 0, 1.0, 0.25, 0.25, n, max(2, n // 4), max(2, n // 4), periodic=False,
                                          boundary_conditions=[sdg.ADIABATIC_SLIP_WALL] * 6)
    elif dim == 2:
        mesh = sdg.Mesh.box_2d(0.0, 0.0, 1.0, 0.25, n, max(2, n // 4), periodic=False, jitter=jitter,
                               split_fraction=split, seed=12, boundary_conditions=[sdg.ADIABATIC_SLIP_WALL] * 4)
    else:
        mesh = sdg.Mesh.box_3d(0, 0, 0, 1.0, 0.25, 0.25, n, max(2, n // 4), max(2, n // 4), periodic=False,
                               boundary_conditions=[sdg.ADIABATIC_SLIP_WALL] * 6)
    cfg = config(p, flux)

    def ic(pts):
        x = pts[:, 0]
        t = 0.5 * (1.0 + np.tanh((x - 0.5) / width))
        rho = 1.0 + (0.125 - 1.0) * t
        pr = 1.0 + (0.1 - 1.0) * t
        out = np.zeros((len(pts), dim + 2))
        out[:, 0] = rho
        out[:, 1] = 0.05 * np.sin(math.pi * pts[:, 1] * 4)
        out[:, 2] = 0.03 * np.sin(4 * math.pi * x)  # small transverse velocities: no variable is identically 0
        if dim == 3:
            out[:, 3] = 0.03 * np.sin(4 * math.pi * x + 1.0) * np.cos(4 * math.pi * pts[:, 2])
        out[:, dim + 1] = pr / (rho * R_GAS)
        return out

    def bc(pts, phys):
        out = np.zeros((len(pts), dim + 2))
        out[:, 0] = 1.0
        out[:, dim + 1] = 1.0 / R_GAS
        return out

    return with_av((mesh, cfg, ic, bc, dt, steps), tolerance, factor)


def golden_cases():
    return {
        "vortex2d_quad_p3_roe": lambda: vortex_case(n=6, p=3, flux=sdg.ROE, steps=4),
        "tgv3d_hex_p3_hllc": lambda: tgv_case(n=3, p=3, flux=sdg.HLLC, steps=3),
        "kh2d_hybrid_p4_lf": lambda: kh_case(n=6, p=4, flux=sdg.LAX_FRIEDRICHS, steps=3),
        "channel2d_quad_p2_hllc_bc": lambda: channel_case(p=2, flux=sdg.HLLC, n=4, steps=3),
        "farfield2d_tri_p3_roe_bc": lambda: channel_case(p=3, flux=sdg.ROE, n=4, steps=3, split=1.0,
                                                         conditions=(sdg.RIEMANN_FARFIELD,) * 4),
        "ns_kh2d_hybrid_p3_br2_lf": lambda: kh_case(n=5, p=3, steps=2, viscous=sdg.BR2, mu=2e-3),
        "ns_channel2d_walls_p2_br1_hllc": lambda: channel_case(
            p=2, flux=sdg.HLLC, n=4, steps=2, viscous=sdg.BR1, mu=0.01,
            conditions=(sdg.ISOTHERMAL_NONSLIP_WALL, sdg.PRESSURE_OUTFLOW, sdg.ADIABATIC_NONSLIP_WALL,
                        sdg.VELOCITY_INFLOW)),
        "inc_taylorvortex2d_p3_exact_br2": lambda: taylor_vortex_case(n=4, p=3, mu=1e-2, steps=2),
        "inc_thermalcavity2d_p2_exact_br2_boussinesq": lambda: cavity_case(p=2, flux=sdg.EXACT, mu=1e-2,
                                                                          boussinesq=True, c0=3.0, n=4, steps=2),
        "av_shocktube2d_hybrid_p3_hllc": lambda: shock_tube_case(p=3, n=8, split=0.5, steps=2),
        "wave1d_line_p3_hllc": lambda: density_wave_1d_case(n=10, p=3, steps=3),
        "av_sod1d_line_p3_hllc": lambda: sod_1d_case(n=19, p=3, steps=3),
    }


def transformed(case, matrix):
    """The same case on the mesh mapped by the linear map `matrix` (a rotation or shear keeps elements affine,
    with off-diagonal metric terms): nodes x' = A x, initial state evaluated at A^-1 x' (periodic on the mapped
    lattice)."""
    mesh, cfg, prim, bprim, dt, steps = case
    a = np.asarray(matrix, np.float64)
    d = mesh.dimension
    full = np.eye(3)
    full[:d, :d] = a
    mesh.nodes = np.ascontiguousarray(mesh.nodes @ full.T)
    inv = np.linalg.inv(full)
    return (mesh, cfg, lambda pts: prim(np.ascontiguousarray(pts @ inv.T)), bprim, dt, steps)


def rotation_2d(degrees):
    t = math.radians(degrees)
    return [[math.cos(t), -math.sin(t)], [math.sin(t), math.cos(t)]]


SHEAR_3D = [[1.0, 0.3, 0.0], [0.0, 1.0, 0.2], [0.1, 0.0, 1.0]]


# ---- curved (high-order) 2D geometry ------------------------------------------------------------------------

def annulus_case(p=3, q=None, flux=sdg.HLLC, nr=3, ntheta=10, split=0.0, steps=3, dt=2e-4, viscous=None, mu=0.0,
                 conditions=(sdg.ADIABATIC_SLIP_WALL, sdg.RIEMANN_FARFIELD), seed=5):
    """Flow in the curved annulus 1 <= r <= 2 (nodes of the order-q geometry on the exact circles): a slip wall
    (or a no-slip wall with `viscous`) at the inner circle, farfield at the outer one, a smooth perturbed stream
    inside; q defaults to the polynomial order, as the reference's drivers set it (setOrder(P))."""
    mesh = sdg.Mesh.annulus(1.0, 2.0, nr, ntheta, geometry_order=q or p, split_fraction=split, seed=seed,
                            boundary_conditions=conditions)
    cfg = config(p, flux) if viscous is None else ns_config(p, flux, viscous, mu)

    def ic(pts):
        x, y = pts[:, 0], pts[:, 1]
        rho = 1.0 + 0.1 * np.sin(x) * np.cos(y)
        u = 0.3 + 0.05 * np.cos(y)
        v = 0.05 * np.sin(x)
        pr = 1.0 + 0.05 * np.cos(x + y)
        return np.stack([rho, u, v, pr / (rho * R_GAS)], 1)

    def bc(pts, phys):
        out = np.zeros((len(pts), 4))
        out[:, 0] = 1.0
        out[:, 1] = 0.3
        out[:, 3] = 1.0 / R_GAS
        return out

    return (mesh, cfg, ic, bc, dt, steps)


def with_geometry_nodes(mesh, q):
    """The same straight-sided 2D mesh given as an order-q mesh: geometry nodes on the straight element maps
    (a gmsh mesh of straight elements after setOrder(q))."""
    from subrosadg_gb300.solver import Mesh
    index = {}
    for i, x in enumerate(mesh.nodes):
        index.setdefault((round(x[0], 12), round(x[1], 12)), i)
    new = list(mesh.nodes)

    def node_at(x):
        key = (round(x[0], 12), round(x[1], 12))
        if key not in index:
            index[key] = len(new)
            new.append(np.array([x[0], x[1], 0.0]))
        return index[key]

    def lattice(kind):
        out, r, o = [], q, 0
        if kind == "quad":
            while r >= 0:
                if r == 0:
                    out.append((o, o))
                    break
                a, b = o, o + r
                out += [(a, a), (b, a), (b, b), (a, b)]
                out += [(a + k, a) for k in range(1, r)] + [(b, a + k) for k in range(1, r)]
                out += [(b - k, b) for k in range(1, r)] + [(a, b - k) for k in range(1, r)]
                r, o = r - 2, o + 1
            return [(-1 + 2 * i / q, -1 + 2 * j / q) for i, j in out]
        while r >= 0:
            if r == 0:
                out.append((o, o))
                break
            out += [(o, o), (o + r, o), (o, o + r)]
            out += [(o + k, o) for k in range(1, r)] + [(o + r - k, o + k) for k in range(1, r)]
            out += [(o, o + r - k) for k in range(1, r)]
            r, o = r - 3, o + 1
        return [(i / q, j / q) for i, j in out]

    def geo(elems, kind):
        if elems is None:
            return None
        rows = []
        for el in elems:
            v = mesh.nodes[el]
            row = []
            for X, Y in lattice(kind):
                if kind == "quad":
                    sh = [0.25 * (1 - X) * (1 - Y), 0.25 * (1 + X) * (1 - Y), 0.25 * (1 + X) * (1 + Y),
                          0.25 * (1 - X) * (1 + Y)]
                else:
                    sh = [1 - X - Y, X, Y]
                row.append(node_at(sum(s * v[k] for k, s in enumerate(sh))))
            rows.append(row)
        return np.array(rows, np.int32)

    tg, qg = geo(mesh.triangles, "tri"), geo(mesh.quadrangles, "quad")
    master = None
    if mesh.periodic_master is not None:
        master = np.concatenate([mesh.periodic_master, np.arange(len(mesh.nodes), len(new), dtype=np.int32)])
    return Mesh(2, np.array(new), triangles=mesh.triangles, quadrangles=mesh.quadrangles, boundary=mesh.boundary,
                boundary_physical=mesh.boundary_physical, physical_conditions=mesh.physical_conditions,
                periodic_master=master, geometry_order=q, triangle_geometry=tg, quadrangle_geometry=qg)
