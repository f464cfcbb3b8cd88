"""GPU parity: the CUDA path (through the C ABI) against the oracle on the same meshes and initial states.

The truth is the oracle built in extended precision (long double): the reference's algorithm evaluated to
~1e-18 on the same double inputs.  Tolerances (the GPU path computes in FP64 throughout):
  * initial state (least-squares projection)          relative L2 <= 1e-13
  * one-stage residual du/dt at the volume points      relative L2 <= 1e-12, or -- where FP64 round-off of
    the problem itself is above that, i.e. the reference's own FP64 arithmetic (the faithful double oracle)
    misses 1e-12 -- at least 10x closer to the truth than the reference's FP64 arithmetic
  * state after N steps, per conserved variable        relative L2 <= 1e-10
  * relative error of the last step (basis-dependent)  relative     <= 1e-9
  * CFL time step                                      relative     <= 1e-13
The GPU path uses a nodal Gauss-collocation basis on quadrangles/hexahedra and the oracle the reference's
modal basis; both represent the same DG solution, so states and rates are compared at the volume points.
"""
import math

import numpy as np
import pytest

import subrosadg_gb300 as sdg
from oracle.orc import Oracle
from tests import cases

pytestmark = pytest.mark.gpu


def rel_l2(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def per_var(a, b):
    return [rel_l2(a[:, v], b[:, v]) if np.linalg.norm(b[:, v]) > 0 else float(np.abs(a[:, v]).max())
            for v in range(b.shape[1])]


def pair(case, precision="extended"):
    """GPU solver and oracle on the same mesh, configuration, initial and boundary states.  The default
    oracle is the extended-precision build: the exact answer of the discrete scheme to ~1e-18."""
    mesh, cfg, prim, bprim, dt, steps = case
    g = sdg.GpuSolver(mesh, cfg)
    o = Oracle(mesh, cfg, faithful=False, precision=precision)
    pts = g.volume_points()
    np.testing.assert_allclose(pts, o.volume_points(), atol=1e-12)
    p0 = prim(pts)
    g.initialize_primitive(p0)
    o.initialize_primitive(p0)
    if g.counts.boundary_face_count:
        # each side enumerates its boundary faces in its own order: evaluate the ghost state at each
        # side's own boundary points
        nfq = g.counts.face_point_count
        bpts, phys = g.boundary_points()
        g.set_boundary_primitive(bprim(bpts, np.repeat(phys, nfq)))
        bpo, pho = o.boundary_points()
        o.set_boundary_primitive(bprim(bpo, np.repeat(pho, nfq)))
    return g, o, dt, steps


CASES = {
    "vortex-quad-p3-roe": lambda: cases.vortex_case(n=6, p=3, flux=sdg.ROE, steps=5),
    "vortex-quad-p2-hllc": lambda: cases.vortex_case(n=6, p=2, flux=sdg.HLLC, steps=5),
    "vortex-quad-p4-lf": lambda: cases.vortex_case(n=5, p=4, flux=sdg.LAX_FRIEDRICHS, steps=5),
    "vortex-quad-p5-central": lambda: cases.vortex_case(n=4, p=5, flux=sdg.CENTRAL, steps=3),
    "vortex-quad-p1-roe-dense": lambda: cases.vortex_case(n=8, p=1, flux=sdg.ROE, steps=5),
    "tgv-hex-p1-hllc": lambda: cases.tgv_case(n=4, p=1, flux=sdg.HLLC, steps=4),
    "tgv-hex-p2-roe": lambda: cases.tgv_case(n=3, p=2, flux=sdg.ROE, steps=4),
    "tgv-hex-p3-hllc": lambda: cases.tgv_case(n=3, p=3, flux=sdg.HLLC, steps=4),
    "tgv-hex-p3-lf": lambda: cases.tgv_case(n=3, p=3, flux=sdg.LAX_FRIEDRICHS, steps=3),
    "tgv-hex-p4-hllc": lambda: cases.tgv_case(n=3, p=4, flux=sdg.HLLC, steps=2),
    "tgv-hex-p5-roe": lambda: cases.tgv_case(n=3, p=5, flux=sdg.ROE, steps=2),
    # curved (high-order) geometry: the annulus 1 <= r <= 2 with its order-q nodes on the circles, slip wall inside,
    # farfield outside (order q = P as the reference's drivers set it, and one case with q below P)
    "curved-annulus-quad-p2-hllc": lambda: cases.annulus_case(p=2),
    "curved-annulus-quad-p3-roe": lambda: cases.annulus_case(p=3, flux=sdg.ROE),
    "curved-annulus-quad-p4-lf": lambda: cases.annulus_case(p=4, flux=sdg.LAX_FRIEDRICHS, nr=2, ntheta=8),
    "curved-annulus-quad-p5-hllc": lambda: cases.annulus_case(p=5, nr=2, ntheta=8, steps=2),
    "curved-annulus-quad-p3-geometry-q2": lambda: cases.annulus_case(p=3, q=2),
    "curved-annulus-hybrid-p3-hllc": lambda: cases.annulus_case(p=3, split=0.5),
    "curved-annulus-tri-p2-roe": lambda: cases.annulus_case(p=2, flux=sdg.ROE, split=1.0),
    "curved-annulus-tri-p4-lf": lambda: cases.annulus_case(p=4, flux=sdg.LAX_FRIEDRICHS, split=1.0, nr=2, ntheta=8),
    "ns-curved-annulus-quad-p3-br2-hllc": lambda: cases.annulus_case(
        p=3, viscous=sdg.BR2, mu=0.01, conditions=(sdg.ISOTHERMAL_NONSLIP_WALL, sdg.RIEMANN_FARFIELD)),
    "ns-curved-annulus-hybrid-p2-br1-lf": lambda: cases.annulus_case(
        p=2, flux=sdg.LAX_FRIEDRICHS, split=0.5, viscous=sdg.BR1, mu=0.01,
        conditions=(sdg.ADIABATIC_NONSLIP_WALL, sdg.RIEMANN_FARFIELD)),
    "ns-curved-annulus-tri-p3-br2-roe": lambda: cases.annulus_case(
        p=3, flux=sdg.ROE, split=1.0, viscous=sdg.BR2, mu=0.01, nr=2, ntheta=8,
        conditions=(sdg.ISOTHERMAL_NONSLIP_WALL, sdg.PRESSURE_OUTFLOW)),
    # affine elements with off-diagonal metric terms (the structured boxes above take the diagonal-metric path)
    "tgv-hex-p3-sheared-hllc": lambda: cases.transformed(cases.tgv_case(n=3, p=3, flux=sdg.HLLC), cases.SHEAR_3D),
    "tgv-hex-p2-sheared-roe": lambda: cases.transformed(cases.tgv_case(n=4, p=2, flux=sdg.ROE), cases.SHEAR_3D),
    "vortex-quad-p3-rotated-roe": lambda: cases.transformed(cases.vortex_case(n=6, p=3, flux=sdg.ROE),
                                                            cases.rotation_2d(30.0)),
    "ns-tgv-hex-p3-sheared-br1-roe": lambda: cases.transformed(
        cases.tgv_case(n=3, p=3, flux=sdg.ROE, steps=2, viscous=sdg.BR1, mu=0.02), cases.SHEAR_3D),
    "ns-vortex-quad-p2-rotated-br2-hllc": lambda: cases.transformed(
        cases.vortex_case(n=5, p=2, flux=sdg.HLLC, steps=3, viscous=sdg.BR2, mu=0.05), cases.rotation_2d(20.0)),
    # tetrahedra (dense modal blocks in 3D; shuffled vertex lists: shared faces at all three rotations)
    "tet-tgv-p1-hllc": lambda: cases.tet_tgv_case(n=3, p=1, flux=sdg.HLLC, steps=4),
    "tet-tgv-p2-roe": lambda: cases.tet_tgv_case(n=3, p=2, flux=sdg.ROE, steps=3),
    "tet-tgv-p3-lf": lambda: cases.tet_tgv_case(n=3, p=3, flux=sdg.LAX_FRIEDRICHS, steps=3),
    "tet-tgv-p3-central": lambda: cases.tet_tgv_case(n=3, p=3, flux=sdg.CENTRAL, steps=2),
    "tet-farfield-p2-hllc": lambda: cases.tet_box_case(p=2, flux=sdg.HLLC),
    "tet-slip-inflow-outflow-p3-roe": lambda: cases.tet_box_case(
        p=3, flux=sdg.ROE, conditions=(sdg.VELOCITY_INFLOW, sdg.PRESSURE_OUTFLOW) + (sdg.ADIABATIC_SLIP_WALL,) * 4),
    "ns-tet-tgv-p2-br1-roe": lambda: cases.tet_tgv_case(n=3, p=2, flux=sdg.ROE, viscous=sdg.BR1, mu=0.02),
    "ns-tet-tgv-p3-br2-hllc": lambda: cases.tet_tgv_case(n=3, p=3, flux=sdg.HLLC, steps=2, viscous=sdg.BR2, mu=0.02),
    "ns-tet-walls-p2-br2-lf": lambda: cases.tet_box_case(
        p=2, flux=sdg.LAX_FRIEDRICHS, viscous=sdg.BR2, mu=0.01,
        conditions=(sdg.VELOCITY_INFLOW, sdg.PRESSURE_OUTFLOW, sdg.ISOTHERMAL_NONSLIP_WALL,
                    sdg.ADIABATIC_NONSLIP_WALL, sdg.RIEMANN_FARFIELD, sdg.ADIABATIC_SLIP_WALL)),
    "ns-tet-box-p1-br1-hllc": lambda: cases.tet_box_case(p=1, flux=sdg.HLLC, viscous=sdg.BR1, mu=0.01),
    # hexahedra that are not parallelepipeds (trilinear maps of a smoothly warped box: the metric |J| dxi/dx and
    # 1/|J| per node, normals and |J_f| per face point of the bilinear faces)
    "warped-hex-tgv-p1-hllc": lambda: cases.warped(cases.tgv_case(n=4, p=1, flux=sdg.HLLC, steps=3)),
    "warped-hex-tgv-p3-hllc": lambda: cases.warped(cases.tgv_case(n=3, p=3, flux=sdg.HLLC, steps=2)),
    "warped-hex-tgv-p5-roe": lambda: cases.warped(cases.tgv_case(n=3, p=5, flux=sdg.ROE, steps=2)),
    "warped-hex-farfield-p2-lf": lambda: cases.warped(cases.hex_box_case(p=2, flux=sdg.LAX_FRIEDRICHS)),
    "warped-hex-slip-inflow-outflow-p4-roe": lambda: cases.warped(cases.hex_box_case(
        p=4, flux=sdg.ROE, steps=2,
        conditions=(sdg.VELOCITY_INFLOW, sdg.PRESSURE_OUTFLOW) + (sdg.ADIABATIC_SLIP_WALL,) * 4)),
    "ns-warped-hex-tgv-p2-br1-roe": lambda: cases.warped(cases.tgv_case(n=3, p=2, flux=sdg.ROE, viscous=sdg.BR1,
                                                                        mu=0.02)),
    "ns-warped-hex-walls-p3-br2-lf": lambda: cases.warped(cases.hex_box_case(
        p=3, flux=sdg.LAX_FRIEDRICHS, viscous=sdg.BR2, mu=0.01, steps=2,
        conditions=(sdg.VELOCITY_INFLOW, sdg.PRESSURE_OUTFLOW, sdg.ISOTHERMAL_NONSLIP_WALL,
                    sdg.ADIABATIC_NONSLIP_WALL, sdg.RIEMANN_FARFIELD, sdg.ADIABATIC_SLIP_WALL))),
    "ns-warped-hex-walls-p5-br1-hllc": lambda: cases.warped(cases.hex_box_case(
        p=5, flux=sdg.HLLC, viscous=sdg.BR1, mu=0.01, steps=2,
        conditions=(sdg.VELOCITY_INFLOW, sdg.PRESSURE_OUTFLOW, sdg.ISOTHERMAL_NONSLIP_WALL,
                    sdg.ADIABATIC_NONSLIP_WALL, sdg.RIEMANN_FARFIELD, sdg.ADIABATIC_SLIP_WALL))),
    "inc-warped-lidcavity-hex-p3-exact-br2": lambda: cases.warped(cases.cavity_3d_case(p=3, viscous=sdg.BR2, mu=1e-2,
                                                                                       steps=2)),
    "av-warped-shocktube-hex-p3-hllc": lambda: cases.warped(cases.shock_tube_case(p=3, dim=3, n=6, steps=2),
                                                            amplitude=0.04),
    # curved hexahedra: order-q geometry nodes (gmsh's hexahedron node order) on a warped box; the per-node metric
    # and the per-face-point normals and |J_f| of the order-q map
    "curved-hex-tgv-p2-q2-hllc": lambda: cases.curved_hex(cases.tgv_case(n=3, p=2, flux=sdg.HLLC, steps=2), 2),
    "curved-hex-tgv-p3-q3-roe": lambda: cases.curved_hex(cases.tgv_case(n=3, p=3, flux=sdg.ROE, steps=2), 3),
    "curved-hex-tgv-p4-q2-lf": lambda: cases.curved_hex(cases.tgv_case(n=3, p=4, flux=sdg.LAX_FRIEDRICHS, steps=2), 2),
    "curved-hex-tgv-p5-q5-hllc": lambda: cases.curved_hex(cases.tgv_case(n=3, p=5, flux=sdg.HLLC, steps=2), 5),
    "curved-hex-farfield-p3-q3-hllc": lambda: cases.curved_hex(cases.hex_box_case(p=3, flux=sdg.HLLC, steps=2), 3),
    "ns-curved-hex-tgv-p2-q2-br1-roe": lambda: cases.curved_hex(cases.tgv_case(n=3, p=2, flux=sdg.ROE,
                                                                               viscous=sdg.BR1, mu=0.02), 2),
    "ns-curved-hex-walls-p3-q3-br2-lf": lambda: cases.curved_hex(cases.hex_box_case(
        p=3, flux=sdg.LAX_FRIEDRICHS, viscous=sdg.BR2, mu=0.01, steps=2,
        conditions=(sdg.VELOCITY_INFLOW, sdg.PRESSURE_OUTFLOW, sdg.ISOTHERMAL_NONSLIP_WALL,
                    sdg.ADIABATIC_NONSLIP_WALL, sdg.RIEMANN_FARFIELD, sdg.ADIABATIC_SLIP_WALL)), 3),
    "ns-curved-hex-walls-p4-q4-br1-hllc": lambda: cases.curved_hex(cases.hex_box_case(
        p=4, flux=sdg.HLLC, viscous=sdg.BR1, mu=0.01, steps=2,
        conditions=(sdg.VELOCITY_INFLOW, sdg.PRESSURE_OUTFLOW, sdg.ISOTHERMAL_NONSLIP_WALL,
                    sdg.ADIABATIC_NONSLIP_WALL, sdg.RIEMANN_FARFIELD, sdg.ADIABATIC_SLIP_WALL)), 4),
    "inc-curved-lidcavity-hex-p3-q3-exact-br2": lambda: cases.curved_hex(
        cases.cavity_3d_case(p=3, viscous=sdg.BR2, mu=1e-2, steps=2), 3),
    "av-curved-shocktube-hex-p3-q3-hllc": lambda: cases.curved_hex(cases.shock_tube_case(p=3, dim=3, n=6, steps=2),
                                                                   3, amplitude=0.04),
    # tetrahedra P4 (35 modes, the 69-point Grundmann-Moeller volume rule, 19-point Dunavant faces)
    "tet-tgv-p4-hllc": lambda: cases.tet_tgv_case(n=3, p=4, flux=sdg.HLLC, steps=2),
    "tet-tgv-p4-roe": lambda: cases.tet_tgv_case(n=3, p=4, flux=sdg.ROE, steps=2),
    "ns-tet-tgv-p4-br2-lf": lambda: cases.tet_tgv_case(n=3, p=4, flux=sdg.LAX_FRIEDRICHS, steps=2, viscous=sdg.BR2,
                                                       mu=0.02),
    "ns-tet-walls-p4-br1-hllc": lambda: cases.tet_box_case(
        p=4, flux=sdg.HLLC, viscous=sdg.BR1, mu=0.01, steps=2,
        conditions=(sdg.VELOCITY_INFLOW, sdg.PRESSURE_OUTFLOW, sdg.ISOTHERMAL_NONSLIP_WALL,
                    sdg.ADIABATIC_NONSLIP_WALL, sdg.RIEMANN_FARFIELD, sdg.ADIABATIC_SLIP_WALL)),
    "inc-lidcavity-tet-p4-exact-br2": lambda: cases.cavity_3d_case(p=4, viscous=sdg.BR2, mu=1e-2, steps=2, tets=True),
    "av-shocktube-tet-p4-hllc": lambda: cases.shock_tube_case(p=4, dim=3, n=6, steps=2, tets=True),
    # tetrahedra P5 (56 modes, the 125-point Grundmann-Moeller rule, 27-point faces with an orbit outside the
    # face; the stage kernel reads its 377 KB of operator tables from global memory)
    "tet-tgv-p5-hllc": lambda: cases.tet_tgv_case(n=3, p=5, flux=sdg.HLLC, steps=2),
    "ns-tet-tgv-p5-br1-roe": lambda: cases.tet_tgv_case(n=3, p=5, flux=sdg.ROE, steps=2, viscous=sdg.BR1, mu=0.02),
    "ns-tet-walls-p5-br2-lf": lambda: cases.tet_box_case(
        p=5, flux=sdg.LAX_FRIEDRICHS, viscous=sdg.BR2, mu=0.01, steps=2,
        conditions=(sdg.VELOCITY_INFLOW, sdg.PRESSURE_OUTFLOW, sdg.ISOTHERMAL_NONSLIP_WALL,
                    sdg.ADIABATIC_NONSLIP_WALL, sdg.RIEMANN_FARFIELD, sdg.ADIABATIC_SLIP_WALL)),
    "inc-thermalcavity-tet-p5-exact-br1-boussinesq": lambda: cases.cavity_3d_case(
        p=5, mu=1e-2, boussinesq=True, c0=3.0, steps=2, tets=True),
    # (P5 on this mesh needs the jump spread over 6 % of the length: with 2 % the projected state goes
    # negative and the oracle diverges too)
    "av-shocktube-tet-p5-roe": lambda: cases.shock_tube_case(p=5, flux=sdg.ROE, dim=3, n=6, steps=2, tets=True,
                                                             width=0.06),
    "inc-euler-cavity-tet-p2-exact": lambda: cases.cavity_3d_case(p=2, viscous=None, mu=0.0, tets=True),
    "inc-lidcavity-tet-p2-exact-br1": lambda: cases.cavity_3d_case(p=2, mu=1e-2, tets=True),
    "inc-thermalcavity-tet-p3-lf-br2-boussinesq": lambda: cases.cavity_3d_case(
        p=3, flux=sdg.LAX_FRIEDRICHS, viscous=sdg.BR2, mu=1e-2, boussinesq=True, c0=3.0, steps=2, tets=True),
    "av-shocktube-tet-p2-hllc": lambda: cases.shock_tube_case(p=2, dim=3, n=8, tets=True),
    "av-shocktube-tet-p3-roe": lambda: cases.shock_tube_case(p=3, flux=sdg.ROE, dim=3, n=6, steps=2, tets=True),
    "kh-hybrid-p4-lf": lambda: cases.kh_case(n=6, p=4, flux=sdg.LAX_FRIEDRICHS, steps=4),
    "kh-jitter-quad-p3-hllc": lambda: cases.kh_case(n=6, p=3, flux=sdg.HLLC, split=0.0, steps=4),
    "kh-jitter-quad-p1-roe": lambda: cases.kh_case(n=6, p=1, flux=sdg.ROE, split=0.0, steps=4),
    "kh-tri-p1-lf": lambda: cases.kh_case(n=6, p=1, flux=sdg.LAX_FRIEDRICHS, split=1.0, steps=4),
    "kh-tri-p2-hllc": lambda: cases.kh_case(n=6, p=2, flux=sdg.HLLC, split=1.0, steps=4),
    "kh-tri-p3-roe": lambda: cases.kh_case(n=5, p=3, flux=sdg.ROE, split=1.0, steps=3),
    "kh-tri-p5-lf": lambda: cases.kh_case(n=4, p=5, flux=sdg.LAX_FRIEDRICHS, split=1.0, steps=2),
    "channel-slip-inflow-outflow": lambda: cases.channel_case(p=2, flux=sdg.HLLC, n=4, steps=4),
    "channel-farfield-tri": lambda: cases.channel_case(p=3, flux=sdg.ROE, n=4, steps=3, split=1.0,
                                                       conditions=(sdg.RIEMANN_FARFIELD,) * 4),
    "channel-walls-hybrid": lambda: cases.channel_case(p=3, flux=sdg.LAX_FRIEDRICHS, n=4, steps=3, split=0.5, jitter=0.1,
                                                       conditions=(sdg.ISOTHERMAL_NONSLIP_WALL, sdg.ADIABATIC_NONSLIP_WALL,
                                                                   sdg.ADIABATIC_SLIP_WALL, sdg.VELOCITY_INFLOW)),
    # Navier-Stokes (BR1 / BR2); viscosities large enough that the viscous terms are not round-off
    "ns-vortex-quad-p2-br1-roe": lambda: cases.vortex_case(n=5, p=2, flux=sdg.ROE, steps=4, viscous=sdg.BR1, mu=0.05),
    "ns-vortex-quad-p3-br2-hllc": lambda: cases.vortex_case(n=5, p=3, flux=sdg.HLLC, steps=4, viscous=sdg.BR2, mu=0.05),
    "ns-kh-jitter-quad-p4-br2-lf": lambda: cases.kh_case(n=5, p=4, flux=sdg.LAX_FRIEDRICHS, split=0.0, steps=3,
                                                         viscous=sdg.BR2, mu=2e-3),
    "ns-kh-jitter-quad-p2-br1-lf": lambda: cases.kh_case(n=6, p=2, flux=sdg.LAX_FRIEDRICHS, split=0.0, steps=3,
                                                         viscous=sdg.BR1, mu=2e-3),
    "ns-tgv-hex-p3-br1-roe": lambda: cases.tgv_case(n=3, p=3, flux=sdg.ROE, steps=3, viscous=sdg.BR1, mu=0.02),
    "ns-tgv-hex-p2-br2-hllc": lambda: cases.tgv_case(n=3, p=2, flux=sdg.HLLC, steps=3, viscous=sdg.BR2, mu=0.02),
    "ns-channel-walls-quad-p2-br2": lambda: cases.channel_case(p=2, flux=sdg.HLLC, n=4, steps=3, viscous=sdg.BR2, mu=0.01,
                                                               conditions=(sdg.ISOTHERMAL_NONSLIP_WALL, sdg.PRESSURE_OUTFLOW,
                                                                           sdg.ADIABATIC_NONSLIP_WALL, sdg.VELOCITY_INFLOW)),
    "ns-channel-farfield-slip-quad-p3-br1-sutherland": lambda: cases.channel_case(
        p=3, flux=sdg.ROE, n=4, steps=3, viscous=sdg.BR1, mu=0.01, transport=sdg.TRANSPORT_SUTHERLAND,
        conditions=(sdg.ADIABATIC_SLIP_WALL, sdg.RIEMANN_FARFIELD, sdg.ADIABATIC_SLIP_WALL, sdg.RIEMANN_FARFIELD)),
    # Navier-Stokes on dense (modal) blocks: triangles, P1 quadrangles, and the hybrid BR2 Kelvin-Helmholtz workload
    "ns-kh-hybrid-p4-br2-lf": lambda: cases.kh_case(n=6, p=4, flux=sdg.LAX_FRIEDRICHS, steps=3, viscous=sdg.BR2,
                                                    mu=2e-3),
    "ns-kh-tri-p3-br1-roe": lambda: cases.kh_case(n=5, p=3, flux=sdg.ROE, split=1.0, steps=3, viscous=sdg.BR1, mu=2e-3),
    "ns-kh-tri-p2-br2-hllc": lambda: cases.kh_case(n=5, p=2, flux=sdg.HLLC, split=1.0, steps=3, viscous=sdg.BR2,
                                                   mu=2e-3),
    "ns-vortex-quad-p1-br2-roe": lambda: cases.vortex_case(n=6, p=1, flux=sdg.ROE, steps=4, viscous=sdg.BR2, mu=0.05),
    "ns-kh-jitter-quad-p1-br1-lf": lambda: cases.kh_case(n=6, p=1, flux=sdg.LAX_FRIEDRICHS, split=0.0, steps=3,
                                                         viscous=sdg.BR1, mu=2e-3),
    "ns-channel-walls-hybrid-p3-br2": lambda: cases.channel_case(
        p=3, flux=sdg.LAX_FRIEDRICHS, n=4, steps=3, split=0.5, jitter=0.1, viscous=sdg.BR2, mu=0.01,
        conditions=(sdg.ISOTHERMAL_NONSLIP_WALL, sdg.ADIABATIC_NONSLIP_WALL, sdg.ADIABATIC_SLIP_WALL,
                    sdg.VELOCITY_INFLOW)),
    "ns-tri-p5-br2-hllc": lambda: cases.kh_case(n=4, p=5, flux=sdg.HLLC, split=1.0, steps=2, viscous=sdg.BR2, mu=2e-3),
    # incompressible model (weakly compressible EOS; Exact / LF / Central fluxes; Boussinesq source)
    "inc-taylorvortex-quad-p4-exact-br2": lambda: cases.taylor_vortex_case(n=5, p=4, mu=1e-2),
    "inc-taylorvortex-hybrid-p3-exact-br1": lambda: cases.taylor_vortex_case(n=5, p=3, viscous=sdg.BR1, mu=1e-2,
                                                                            jitter=0.1, split=0.5),
    "inc-taylorvortex-quad-p1-exact-br2-dense": lambda: cases.taylor_vortex_case(n=6, p=1, mu=1e-2),
    "inc-shearlayer-hybrid-p3-lf": lambda: cases.shear_layer_case(n=6, p=3),
    "inc-shearlayer-tri-p2-central": lambda: cases.shear_layer_case(n=6, p=2, flux=sdg.CENTRAL, split=1.0),
    "inc-shearlayer-quad-p5-exact": lambda: cases.shear_layer_case(n=4, p=5, flux=sdg.EXACT, split=0.0, steps=2),
    "inc-lidcavity-quad-p3-lf-br2": lambda: cases.cavity_case(p=3, mu=1e-2),
    "inc-thermalcavity-quad-p2-exact-br2-boussinesq": lambda: cases.cavity_case(p=2, flux=sdg.EXACT, mu=1e-2,
                                                                                boussinesq=True, c0=3.0),
    "inc-thermalcavity-hybrid-p3-exact-br1-boussinesq": lambda: cases.cavity_case(
        p=3, flux=sdg.EXACT, viscous=sdg.BR1, mu=1e-2, boussinesq=True, c0=3.0, jitter=0.1, split=0.5),
    "inc-channel-farfield-quad-p2-exact": lambda: cases.inc_channel_case(p=2),
    "inc-channel-inflow-outflow-tri-p3-lf": lambda: cases.inc_channel_case(
        p=3, flux=sdg.LAX_FRIEDRICHS, split=1.0,
        conditions=(sdg.ADIABATIC_SLIP_WALL, sdg.PRESSURE_OUTFLOW, sdg.ADIABATIC_SLIP_WALL, sdg.VELOCITY_INFLOW)),
    "inc-ns-channel-walls-quad-p3-exact-br2": lambda: cases.inc_channel_case(
        p=3, viscous=sdg.BR2, mu=1e-2,
        conditions=(sdg.ISOTHERMAL_NONSLIP_WALL, sdg.RIEMANN_FARFIELD, sdg.ADIABATIC_NONSLIP_WALL, sdg.VELOCITY_INFLOW)),
    "inc-lidcavity-hex-p2-exact-br1": lambda: cases.cavity_3d_case(p=2, mu=1e-2),
    "inc-thermalcavity-hex-p3-lf-br2-boussinesq": lambda: cases.cavity_3d_case(
        p=3, flux=sdg.LAX_FRIEDRICHS, viscous=sdg.BR2, mu=1e-2, boussinesq=True, c0=3.0),
    "inc-euler-cavity-hex-p3-exact": lambda: cases.cavity_3d_case(p=3, viscous=None, mu=0.0),
    # artificial viscosity (shock capturing): Sod tubes in slip-walled boxes and the Kelvin-Helmholtz bands
    "av-shocktube-quad-p3-hllc": lambda: cases.shock_tube_case(p=3, n=8),
    "av-shocktube-hybrid-p2-lf": lambda: cases.shock_tube_case(p=2, flux=sdg.LAX_FRIEDRICHS, split=0.5, jitter=0.1),
    "av-shocktube-tri-p4-roe": lambda: cases.shock_tube_case(p=4, flux=sdg.ROE, split=1.0, n=6),
    "av-shocktube-quad-p1-hllc-dense": lambda: cases.shock_tube_case(p=1, n=8),
    "av-shocktube-jitter-quad-p4-roe": lambda: cases.shock_tube_case(p=4, flux=sdg.ROE, jitter=0.1, n=6),
    "av-shocktube-hex-p2-hllc": lambda: cases.shock_tube_case(p=2, dim=3, n=8),
    "av-shocktube-hex-p4-roe": lambda: cases.shock_tube_case(p=4, flux=sdg.ROE, dim=3, n=6, steps=2),
    "av-kh-hybrid-p4-lf": lambda: cases.with_av(cases.kh_case(n=6, p=4, steps=3), tolerance=1.0),
    "av-kh-jitter-quad-p5-hllc": lambda: cases.with_av(cases.kh_case(n=4, p=5, flux=sdg.HLLC, split=0.0, steps=2),
                                                       tolerance=2.0, factor=0.5),
    # 1D (line meshes, point faces): the periodic density wave, Sod and Shu-Osher with artificial viscosity,
    # Navier-Stokes and the incompressible model
    "line-wave-p1-roe": lambda: cases.density_wave_1d_case(p=1, flux=sdg.ROE),
    "line-wave-p2-lf": lambda: cases.density_wave_1d_case(p=2, flux=sdg.LAX_FRIEDRICHS),
    "line-wave-p3-hllc": lambda: cases.density_wave_1d_case(p=3),
    "line-wave-p4-central": lambda: cases.density_wave_1d_case(n=20, p=4, flux=sdg.CENTRAL),
    "line-wave-p5-roe": lambda: cases.density_wave_1d_case(n=20, p=5, flux=sdg.ROE, dt=5e-5),
    "line-sod-walls-p3-roe": lambda: cases.sod_1d_case(n=40, p=3, flux=sdg.ROE, av=False, dt=1e-5,
                                                       conditions=(sdg.ADIABATIC_SLIP_WALL, sdg.ADIABATIC_SLIP_WALL)),
    "line-sod-inflow-outflow-p2-hllc": lambda: cases.sod_1d_case(n=40, p=2, av=False, dt=1e-5,
                                                                 conditions=(sdg.VELOCITY_INFLOW, sdg.PRESSURE_OUTFLOW)),
    "ns-line-wave-p3-br1-hllc": lambda: cases.density_wave_1d_case(n=20, p=3, viscous=sdg.BR1, mu=0.01),
    "ns-line-wave-p4-br2-roe": lambda: cases.density_wave_1d_case(n=20, p=4, flux=sdg.ROE, viscous=sdg.BR2, mu=0.01,
                                                                  dt=5e-5),
    "ns-line-sod-walls-p2-br2-lf": lambda: _ns(cases.sod_1d_case(
        n=40, p=2, flux=sdg.LAX_FRIEDRICHS, av=False, dt=1e-5,
        conditions=(sdg.ISOTHERMAL_NONSLIP_WALL, sdg.ADIABATIC_NONSLIP_WALL)), sdg.BR2, 0.01),
    # (odd element counts put the jumps inside elements, where the sensor sees them)
    "av-sod-line-p3-hllc": lambda: cases.sod_1d_case(n=99, p=3),
    "av-sod-line-p4-roe": lambda: cases.sod_1d_case(n=99, p=4, flux=sdg.ROE),
    "av-sod-line-p1-lf": lambda: cases.sod_1d_case(n=99, p=1, flux=sdg.LAX_FRIEDRICHS),
    "av-shuosher-line-p3-hllc": lambda: cases.shu_osher_1d_case(n=99, smooth=0.04, dt=5e-6),
    "av-shuosher-line-p5-roe": lambda: cases.shu_osher_1d_case(n=99, p=5, flux=sdg.ROE, smooth=0.04, dt=5e-6),
    "av-shuosher-line-p2-lf": lambda: cases.shu_osher_1d_case(n=99, p=2, flux=sdg.LAX_FRIEDRICHS, smooth=0.04,
                                                              dt=5e-6),
    "inc-line-wave-p3-exact": lambda: cases.inc_wave_1d_case(),
    "inc-ns-line-wave-p4-lf-br2": lambda: cases.inc_wave_1d_case(p=4, flux=sdg.LAX_FRIEDRICHS, viscous=sdg.BR2, mu=0.01,
                                                                 dt=5e-5),
}


def _ns(case, viscous, mu):
    """The same case as Navier-Stokes with `viscous` and viscosity mu."""
    mesh, cfg, ic, bc, dt, steps = case
    return (mesh, cases.ns_config(cfg.polynomial_order, cfg.convective_flux, viscous, mu), ic, bc, dt, steps)


def reference_arithmetic_residual(case):
    """Residual of the reference's own FP64 arithmetic (double oracle, plain inverses) on the same input."""
    mesh, cfg, prim, bprim, dt, steps = case
    o = Oracle(mesh, cfg, faithful=True, precision="double")
    o.initialize_primitive(prim(o.volume_points()))
    if o.boundary:
        bpo, pho = o.boundary_points()
        o.set_boundary_primitive(bprim(bpo, np.repeat(pho, o.nfq)))
    return o.residual_point()


@pytest.mark.parametrize("name", list(CASES))
def test_parity(name):
    g, o, dt, steps = pair(CASES[name]())
    # initial state
    s0g, s0o = g.state_point(), o.state_point()
    assert rel_l2(s0g, s0o) <= 1e-13, rel_l2(s0g, s0o)
    if g.config.shock_capturing:  # the artificial viscosity field of the initial state
        ag, ao = g.node_artificial_viscosity(), o.node_artificial_viscosity()
        assert ao.max() > 0.0
        np.testing.assert_allclose(ag, ao, rtol=1e-9, atol=1e-13 * ao.max())
    # one residual evaluation
    rg, ro = g.residual_point(), o.residual_point()
    err = rel_l2(rg, ro)
    if err > 1e-12:
        ref_err = rel_l2(reference_arithmetic_residual(CASES[name]()), ro)
        print(f"{name}: GPU residual error {err:.2e}, reference FP64 arithmetic error {ref_err:.2e}")
        if not (ref_err > 1e-12 and err <= 0.1 * ref_err):
            # diagnostic: the truth at the GPU's own state separates projection error from residual arithmetic
            o.set_state_point(g.state_point())
            own = rel_l2(rg, o.residual_point())
            raise AssertionError(f"residual {err:.3e} (reference arithmetic {ref_err:.3e}, at the GPU's own state "
                                 f"{own:.3e}) per variable {per_var(rg, ro)}")
    # time step
    dtg, dto = g.calculateDeltaTime(0.2), o.delta_time(0.2)
    assert abs(dtg - dto) <= 1e-13 * dto
    # N steps
    for _ in range(steps):
        eg = g.stepSolver(dt).copy()
        o.step(dt)
    sg, so = g.state_point(), o.state_point()
    pv = per_var(sg, so)
    assert max(pv) <= 1e-10, pv
    np.testing.assert_allclose(eg, o.relative_error(), rtol=1e-9, atol=1e-15)


def test_tgv_config_dt_matches_reference_formula():
    """cfg: TGV dt from CFL 0.2 (TimeIntegration.cpp:119-125) on the GPU equals the oracle's."""
    g, o, _, _ = pair(cases.tgv_case(n=4, p=3))
    assert abs(g.calculateDeltaTime(0.2) - o.delta_time(0.2)) <= 1e-13 * o.delta_time(0.2)


def test_free_stream_preserved_on_gpu():
    mesh = sdg.Mesh.box_2d(0, 0, 1, 1, 5, 5, jitter=0.15, split_fraction=0.5, seed=3)
    g = sdg.GpuSolver(mesh, cases.config(4, sdg.ROE))
    g.initialize_primitive(cases.uniform_primitive(g.counts.volume_point_count, 2))
    assert np.abs(g.residual_point()).max() < 1e-9
    mesh = sdg.Mesh.box_3d(0, 0, 0, 1, 1, 1, 3, 3, 3)
    g = sdg.GpuSolver(mesh, cases.config(3, sdg.HLLC))
    g.initialize_primitive(cases.uniform_primitive(g.counts.volume_point_count, 3))
    assert np.abs(g.residual_point()).max() < 1e-10


def test_deterministic():
    """No atomics on the data path: two identical runs are bit-identical."""
    out = []
    for _ in range(2):
        g, o, dt, steps = pair(cases.tgv_case(n=3, p=3, steps=3))
        g.stepSolver(dt, 3)
        out.append((g.state_point(), g.relative_error()))
    assert np.array_equal(out[0][0], out[1][0]) and np.array_equal(out[0][1], out[1][1])


def test_nan_state_is_reported_by_relative_error():
    """The reference's only failure detection: all relative errors NaN (SystemControl.cpp:185-191)."""
    g, o, dt, _ = pair(cases.vortex_case(n=4, p=2))
    s = g.state_point()
    s[:, 0] = np.nan
    g.set_state_point(s)
    err = g.stepSolver(dt)
    assert np.isnan(err).all()


@pytest.mark.parametrize("case", [lambda: cases.vortex_case(n=4, p=3), lambda: cases.density_wave_1d_case(n=6, p=4)],
                         ids=["quad-p3", "line-p4"])
def test_modal_state_roundtrip_and_layout(case):
    g, o, dt, _ = pair(case())
    m = g.state_modal()
    mo = o.state_modal()
    # same modal basis and layout as the oracle (reference layout: column-major (d+2) x Nb per element)
    assert rel_l2(m, mo) <= 1e-12
    g.set_state_modal(m)
    assert rel_l2(g.state_point(), o.state_point()) <= 1e-13


def test_launch_count_and_shape():
    g, o, dt, _ = pair(cases.tgv_case(n=3, p=3))
    n0 = g.launch_count()
    g.stepSolver(dt)
    # per SSP-RK3 stage: 1 face kernel + 1 element kernel; plus 1 reduction per step
    assert g.launch_count() - n0 == 3 * 2 + 1


@pytest.mark.parametrize("q", [2, 3, 4])
def test_curved_wall_force_of_a_uniform_state_vanishes(q):
    """The pressure force on the closed curved inner wall of a uniform state is zero to round-off: the face
    quadrature integrates n|J_f| of the order-q edges exactly and the edges close (the reference's View force,
    VariableConvertor.cpp:883-906)."""
    mesh = sdg.Mesh.annulus(1.0, 2.0, 2, 10, geometry_order=q, split_fraction=0.4, seed=1,
                            boundary_conditions=(sdg.ADIABATIC_SLIP_WALL, sdg.RIEMANN_FARFIELD))
    g = sdg.GpuSolver(mesh, cases.config(q, sdg.HLLC))
    g.initialize_primitive(cases.uniform_primitive(g.counts.volume_point_count, 2, vel=(0.0, 0.0)))
    f = g.surface_force(1)
    assert np.abs(f).max() < 1e-12, f


@pytest.mark.parametrize("q", [1, 2, 3])
def test_warped_hexahedra_wall_force_of_a_uniform_state_vanishes(q):
    """Per-point face geometry of bilinear (q = 1) and order-q hexahedron faces: the pressure force of a uniform
    state on the closed (warped) boundary of a box is zero to round-off, since the face rule integrates the
    faces' n|J_f| exactly and the boundary closes."""
    case = cases.hex_box_case(p=q + 1, conditions=(sdg.ADIABATIC_SLIP_WALL,) * 6)
    mesh = (cases.warped(case) if q == 1 else cases.curved_hex(case, q))[0]
    g = sdg.GpuSolver(mesh, cases.config(q + 1, sdg.HLLC))
    g.initialize_primitive(cases.uniform_primitive(g.counts.volume_point_count, 3, vel=(0.0, 0.0, 0.0)))
    f = sum(g.surface_force(k) for k in range(1, 7))
    assert np.abs(f).max() < 1e-12, f
