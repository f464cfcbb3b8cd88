"""Seeded synthetic workloads of the benchmark configurations (analytic flows; no dataset is involved).

  vortex2d : periodic isentropic vortex (strength 5, rho=1, u=(1,1), p=1) on [-5,5]^2, quads, Roe, dt 1e-3
  tgv3d    : Taylor-Green vortex, Mach 0.1, periodic [0,2pi]^3, hexahedra (HLLC; Navier-Stokes BR1 Roe at Re 1600)
  kh2d     : Kelvin-Helmholtz shear layer on [0,1]^2 (rho 1/2 bands, u=+-0.5, seeded 1e-2 sinusoidal v),
             jittered quads with a seeded half split into triangles, LF (Navier-Stokes BR2 at Re 1e4)
  batched  : independent Kelvin-Helmholtz instances of seeded size, order, element kind, Mach and Reynolds number
  tet3d    : Taylor-Green vortex on periodic tetrahedra
Thermodynamics follow the example drivers: cp = 2.5, cv = 25/14 (R = 1/1.4), gamma = 1.4
(examples/periodic_2d_ceuler.cpp:51), so the primitive temperature is T = p / (rho R).  The vortex follows
examples/periodic_2d_ceuler.cpp, the Kelvin-Helmholtz pressure examples/khinstability_2d_ceuler.cpp:33-40.
Each *_case returns (mesh, config, initial primitive function of the volume points, boundary primitive
function or None, dt, steps).
"""
from __future__ import annotations

import math

import numpy as np

from . import _abi as sdg
from .solver import Mesh, make_config

GAMMA = 1.4
CP, CV = 2.5, 25.0 / 14.0
R_GAS = CP - CV


def vortex_primitive(x, y, beta=5.0, gamma=GAMMA, period=10.0):
    # nearest periodic image of the vortex centre at the origin
    x = (x + period / 2) % period - period / 2
    y = (y + period / 2) % period - period / 2
    r2 = x * x + y * y
    du = beta / (2 * math.pi) * np.exp(0.5 * (1 - r2))
    u = 1.0 - du * y
    v = 1.0 + du * x
    t = 1.0 - (gamma - 1) * beta ** 2 / (8 * gamma * math.pi ** 2) * np.exp(1 - r2)
    rho = t ** (1.0 / (gamma - 1))
    p = rho ** gamma
    return np.stack([rho, u, v, p / (rho * R_GAS)], 1)


def tgv_primitive(x, y, z, mach=0.1, gamma=GAMMA):
    p0 = 1.0 / (gamma * mach ** 2)
    u = np.sin(x) * np.cos(y) * np.cos(z)
    v = -np.cos(x) * np.sin(y) * np.cos(z)
    w = np.zeros_like(x)
    p = p0 + (np.cos(2 * x) + np.cos(2 * y)) * (np.cos(2 * z) + 2.0) / 16.0
    rho = p / p0  # isothermal start, T0 = p0 / (rho0 R)
    return np.stack([rho, u, v, w, p / (rho * R_GAS)], 1)


def kh_primitive(x, y, seed=7, pressure=2.5):
    rng = np.random.default_rng(seed)
    k = int(rng.integers(1, 4))
    phase = float(rng.uniform(0, 2 * math.pi))
    band = (y >= 0.25) & (y <= 0.75)
    rho = np.where(band, 2.0, 1.0)
    u = np.where(band, 0.5, -0.5)
    v = 1e-2 * np.sin(2 * math.pi * k * x + phase)
    p = np.full_like(x, pressure)  # 2.5: examples/khinstability_2d_ceuler.cpp:33-40
    return np.stack([rho, u, v, p / (rho * R_GAS)], 1)


def uniform_primitive(n, dim, rho=1.0, vel=(0.3, -0.2, 0.1), p=1.0):
    out = np.zeros((n, dim + 2))
    out[:, 0] = rho
    out[:, 1:1 + dim] = vel[:dim]
    out[:, dim + 1] = p / (rho * R_GAS)
    return out


def config(p, flux, equation=sdg.EULER, viscous=sdg.VISCOUS_NONE, mu=0.0, prandtl=0.71, rk=sdg.SSPRK3):
    return make_config(p, equation=equation, convective_flux=flux, viscous_flux=viscous, time_integration=rk,
                           cp=CP, cv=CV, gamma=GAMMA, mu=mu, prandtl=prandtl)


def ns_config(p, flux, viscous, mu, prandtl=0.71, transport=sdg.TRANSPORT_CONSTANT):
    """Compressible Navier-Stokes with BR1/BR2 (the reference fixes Pr = 0.71, PhysicalModel.cpp:91)."""
    c = config(p, flux, equation=sdg.NAVIER_STOKES, viscous=viscous, mu=mu, prandtl=prandtl)
    c.transport_model = transport
    return c


def vortex_case(n=8, p=3, flux=sdg.ROE, dt=1e-3, steps=4, viscous=None, mu=0.0):
    mesh = Mesh.box_2d(-5.0, -5.0, 10.0, 10.0, n, n, periodic=True)
    cfg = config(p, flux) if viscous is None else ns_config(p, flux, viscous, mu)
    return (mesh, cfg, lambda pts: vortex_primitive(pts[:, 0], pts[:, 1]), None, dt, steps)


def tgv_case(n=3, p=3, flux=sdg.HLLC, dt=None, steps=3, viscous=None, mu=1.0 / 1600.0):
    """Taylor-Green vortex; with `viscous` the Navier-Stokes case at Re = 1/mu (1600 by default)."""
    mesh = Mesh.box_3d(0, 0, 0, 2 * math.pi, 2 * math.pi, 2 * math.pi, n, n, n, periodic=True)
    if dt is None:
        # CFL 0.2 with minEdge = 2 pi / n and max(|u|+c) ~ 1 + 1/Mach (TimeIntegration.cpp:119-125)
        dt = 0.2 * (2 * math.pi / n) / ((1.0 + 1.0 / 0.1 + 0.05) * (p + 1) ** 2)
    cfg = config(p, flux) if viscous is None else ns_config(p, flux, viscous, mu)
    return (mesh, cfg, lambda pts: tgv_primitive(pts[:, 0], pts[:, 1], pts[:, 2]), None, dt, steps)


# Even permutations of a tetrahedron's vertex list (orientation kept): shuffling each element's list this way
# makes shared faces meet at all three rotations.
_EVEN_TET = np.array([(0, 1, 2, 3), (0, 2, 3, 1), (0, 3, 1, 2), (1, 0, 3, 2), (1, 2, 0, 3), (1, 3, 2, 0),
                      (2, 0, 1, 3), (2, 1, 3, 0), (2, 3, 0, 1), (3, 0, 2, 1), (3, 1, 0, 2), (3, 2, 1, 0)])


def tet_mesh(n=3, length=1.0, periodic=True, conditions=None, seed=7):
    """Structured tetrahedral box [0, length]^3 (six tetrahedra per cube), vertex lists shuffled (seeded)."""
    mesh = Mesh.box_3d_tetrahedra(0, 0, 0, length, length, length, n, n, n, periodic=periodic,
                                      boundary_conditions=None if periodic else list(conditions))
    pick = np.random.default_rng(seed).integers(0, len(_EVEN_TET), len(mesh.tetrahedra))
    mesh.tetrahedra = np.ascontiguousarray(mesh.tetrahedra[np.arange(len(pick))[:, None], _EVEN_TET[pick]])
    return mesh


def tet_tgv_case(n=3, p=2, flux=sdg.HLLC, steps=3, mach=0.3, viscous=None, mu=0.02):
    """Taylor-Green vortex on periodic tetrahedra of [0, 2 pi]^3 (Mach 0.3 for a nonlinear flux); with
    `viscous` the Navier-Stokes case at Re = 1/mu."""
    mesh = tet_mesh(n, 2 * math.pi)
    dt = 0.2 * (2 * math.pi / n) / ((1.0 + 1.0 / mach) * (p + 1) ** 2)
    cfg = config(p, flux) if viscous is None else ns_config(p, flux, viscous, mu)
    return (mesh, cfg, lambda pts: tgv_primitive(pts[:, 0], pts[:, 1], pts[:, 2], mach=mach), None, dt,
            steps)


def _warp(x, lo, span, amplitude):
    s = np.sin(2.0 * math.pi * (x - lo) / span)
    d = amplitude * span / (2.0 * math.pi) * np.stack([s[:, 1] * s[:, 2], s[:, 2] * s[:, 0], s[:, 0] * s[:, 1]], 1)
    return np.ascontiguousarray(x + d)


def warped(case, amplitude=0.08):
    """The same case on a smoothly deformed 3D mesh: node x moves by amplitude L/(2 pi) times
    (sin k y sin k z, sin k z sin k x, sin k x sin k y), k = 2 pi / L per direction over the mesh's bounding box.
    The deformation is periodic over the box (opposite faces of a periodic box stay translates of each other)
    and leaves no hexahedron a parallelepiped: the elements are general trilinear maps, their faces bilinear
    (neither planar nor of constant |J_f|) -- the mapped hexahedra of the reference's 3D drivers
    (examples/sphere_3d_cns.cpp, examples/protuberance_3d_ceuler.cpp) at geometry order 1."""
    mesh, cfg, ic, bc, dt, steps = case
    lo, hi = mesh.nodes.min(0), mesh.nodes.max(0)
    mesh.nodes = _warp(mesh.nodes, lo, hi - lo, amplitude)
    return (mesh, cfg, ic, bc, dt, steps)


_HEX_CORNERS = [(-1, -1, -1), (1, -1, -1), (1, 1, -1), (-1, 1, -1), (-1, -1, 1), (1, -1, 1), (1, 1, 1), (-1, 1, 1)]
_HEX_EDGES = [(0, 1), (0, 3), (0, 4), (1, 2), (1, 5), (2, 3), (2, 6), (3, 7), (4, 5), (4, 7), (5, 6), (6, 7)]
_HEX_FACES = [(0, 3, 2, 1), (0, 1, 5, 4), (0, 4, 7, 3), (1, 2, 6, 5), (2, 3, 7, 6), (4, 5, 6, 7)]
_HEX_NEIGHBOURS = [(1, 3, 4), (0, 2, 5), (1, 3, 6), (0, 2, 7), (0, 5, 7), (1, 4, 6), (2, 5, 7), (3, 4, 6)]


def _quad_nodes(c, r):
    """gmsh's order-r quadrangle nodes on four corner points c (3D): corners, edge interiors in edge direction,
    then the inner quadrangle of order r - 2 one lattice step inside, recursively."""
    out = []
    while r >= 0:
        if r == 0:
            out.append(sum(c) / 4.0)
            break
        out += list(c)
        for k in range(4):
            out += [c[k] + (c[(k + 1) % 4] - c[k]) * i / r for i in range(1, r)]
        if r < 2:
            break
        c = [c[k] + (c[(k + 1) % 4] - c[k]) / r + (c[(k - 1) % 4] - c[k]) / r for k in range(4)]
        r -= 2
    return out


def hex_lattice(q):
    """Reference points of gmsh's order-q hexahedron in its node order: the 8 corners, the edge interiors
    (gmsh's edge table, in edge direction), each face's interior as an order q-2 quadrangle whose corners follow
    the face's vertex list (gmsh's face table), then the interior as an order q-2 hexahedron, recursively."""
    c = [np.array(p, dtype=float) for p in _HEX_CORNERS]
    out, r = [], q
    while r >= 0:
        if r == 0:
            out.append(sum(c) / 8.0)
            break
        out += c
        for a, b in _HEX_EDGES:
            out += [c[a] + (c[b] - c[a]) * i / r for i in range(1, r)]
        if r < 2:
            break
        for f in _HEX_FACES:
            fc = [c[f[k]] + (c[f[(k + 1) % 4]] - c[f[k]]) / r + (c[f[(k - 1) % 4]] - c[f[k]]) / r for k in range(4)]
            out += _quad_nodes(fc, r - 2)
        c = [c[k] + sum((c[m] - c[k]) / r for m in _HEX_NEIGHBOURS[k]) for k in range(8)]
        r -= 2
    return np.array(out)


def curved_hex(case, q, amplitude=0.08):
    """The same case on curved hexahedra of geometry order q: each element's gmsh-ordered order-q nodes are
    placed by its trilinear map and then moved, with the vertices, by the `warped` deformation, so every face is
    a curved surface (the order-q elements of the reference's 3D drivers after setOrder(P), e.g.
    examples/sphere_3d_cns.cpp:379).  Interior nodes are per element; the corners are the mesh vertices."""
    mesh, cfg, ic, bc, dt, steps = case
    x = mesh.nodes
    lo, hi = x.min(0), x.max(0)
    lat = hex_lattice(q)
    sx = np.stack([(1 + sgn * lat[:, d]) / 2 for d in range(3) for sgn in (-1, 1)], 1)  # [(1-X)/2, (1+X)/2, ...]
    shape = np.stack([sx[:, 0 + (c[0] > 0)] * sx[:, 2 + (c[1] > 0)] * sx[:, 4 + (c[2] > 0)] for c in _HEX_CORNERS], 1)
    hexes = mesh.hexahedra
    pts = np.einsum("qk,ekd->eqd", shape, x[hexes])[:, 8:, :]
    ne, extra = len(hexes), len(lat) - 8
    ids = len(x) + np.arange(ne * extra, dtype=np.int32).reshape(ne, extra)
    nodes = _warp(np.concatenate([x, pts.reshape(-1, 3)]), lo, hi - lo, amplitude)
    periodic = None
    if mesh.periodic_master is not None:
        periodic = np.concatenate([mesh.periodic_master, ids.reshape(-1)])
    out = Mesh(3, nodes, hexahedra=hexes, boundary=mesh.boundary, boundary_physical=mesh.boundary_physical,
                   physical_conditions=mesh.physical_conditions, periodic_master=periodic, geometry_order=q,
                   hexahedron_geometry=np.concatenate([hexes, ids], 1))
    return (out, cfg, ic, bc, dt, steps)


def curved_wall_case(n=32, p=3, q=3, flux=sdg.HLLC, viscous=sdg.BR2, re=200.0, amplitude=0.08, steps=3):
    """Navier-Stokes along a curved no-slip wall, the shape of examples/sphere_3d_cns.cpp (P3, HLLC, BR2, curved
    hexahedra of geometry order 3 after setOrder(3), a Riemann farfield and an adiabatic no-slip wall, the stream
    rho = 1.4, v = 0.2, T = 1 (Mach 0.2) and mu = 1.4 * 0.2 / Re with Re = 200): the unit box of n^3 curved
    hexahedra of geometry order q (curved_hex of the warped box), the wall at z = 0 (group 5) and the farfield on
    the other five sides.  The initial state is the stream with a smooth density perturbation."""
    conds = [sdg.RIEMANN_FARFIELD] * 4 + [sdg.ADIABATIC_NONSLIP_WALL, sdg.RIEMANN_FARFIELD]
    mesh = Mesh.box_3d(0, 0, 0, 1, 1, 1, n, n, n, periodic=False, boundary_conditions=conds)
    cfg = ns_config(p, flux, viscous, 1.4 * 0.2 / re)

    def ic(pts):
        x, y, z = pts[:, 0], pts[:, 1], pts[:, 2]
        out = np.zeros((len(pts), 5))
        out[:, 0] = 1.4 * (1.0 + 0.02 * np.sin(2 * math.pi * x) * np.sin(2 * math.pi * y) * np.sin(math.pi * z))
        out[:, 2] = 0.2
        out[:, 4] = 1.4 / out[:, 0]  # p = rho R T = 1 with R = 1/1.4
        return out

    def bc(pts, phys):
        out = np.zeros((len(pts), 5))
        out[:, 0] = 1.4
        out[:, 2] = np.where(phys == 5, 0.0, 0.2)
        out[:, 4] = 1.0
        return out

    dt = 0.2 * (1.0 / n) / ((0.2 + 1.0) * (p + 1) ** 2)
    return curved_hex((mesh, cfg, ic, bc, dt, steps), q, amplitude)


def kh_case(n=8, p=4, flux=sdg.LAX_FRIEDRICHS, dt=2e-4, steps=3, jitter=0.1, split=0.5, seed=11, viscous=None,
            mu=1e-4):
    """Kelvin-Helmholtz; with `viscous` the Navier-Stokes case at Re = 1/mu (1e4 by default)."""
    mesh = Mesh.box_2d(0.0, 0.0, 1.0, 1.0, n, n, periodic=True, jitter=jitter, split_fraction=split, seed=seed)
    cfg = config(p, flux) if viscous is None else ns_config(p, flux, viscous, mu)
    return (mesh, cfg, lambda pts: kh_primitive(pts[:, 0], pts[:, 1]), None, dt, steps)


def batch_instances(count=256, seed=2024, min_elements=500, max_elements=50000, orders=(1, 2, 3, 4, 5)):
    """The batched workload: `count` independent 2D Kelvin-Helmholtz solves on [0,1]^2 (periodic), element
    counts log-uniform in [min_elements, max_elements], P uniform in `orders`, jittered (10% of h) quads or
    the hybrid with a 50% triangle split, Mach of the shear speed uniform in [0.1, 0.8] (p = rho c^2 / gamma
    with c = 0.5 / Mach in the light band), Re = 1 / mu log-uniform in [1e2, 1e4], Euler or Navier-Stokes
    (BR2) with equal odds, Lax-Friedrichs flux, SSP-RK3.  Returns a list of (mesh, cfg, primitive) and the
    parameter records."""
    rng = np.random.default_rng(seed)
    out, params = [], []
    for i in range(count):
        target = math.exp(rng.uniform(math.log(min_elements), math.log(max_elements)))
        p = int(rng.choice(orders))
        hybrid = bool(rng.random() < 0.5)
        mach = float(rng.uniform(0.1, 0.8))
        re = float(math.exp(rng.uniform(math.log(1e2), math.log(1e4))))
        ns = bool(rng.random() < 0.5)
        split = 0.5 if hybrid else 0.0
        n = max(3, int(round(math.sqrt(target / (1.0 + split)))))
        mesh = Mesh.box_2d(0.0, 0.0, 1.0, 1.0, n, n, periodic=True, jitter=0.1, split_fraction=split,
                               seed=seed * 1000 + i)
        cfg = ns_config(p, sdg.LAX_FRIEDRICHS, sdg.BR2, 1.0 / re) if ns else config(p, sdg.LAX_FRIEDRICHS)
        pressure = 0.25 / (GAMMA * mach * mach)
        out.append((mesh, cfg, (lambda pr, sd: (lambda pts: kh_primitive(pts[:, 0], pts[:, 1], seed=sd, pressure=pr)))(
            pressure, seed + i)))
        params.append({"n": n, "order": p, "hybrid": hybrid, "mach": mach, "reynolds": re, "navier_stokes": ns})
    return out, params
