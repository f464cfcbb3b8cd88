"""GPU parity at the benchmark configurations' stated sizes (the workloads bench.py times), through the C ABI.

  vortex2d  40x40 quadrangles P3, Roe, dt 1e-3: the one-stage residual and the state after all 200 SSP-RK3
            steps (long-horizon round-off growth)
  tgv3d     64^3 hexahedra P3, HLLC, dt from CFL 0.2: one-stage residual, dt, three steps
  kh2d-ns   256^2 quadrangles jittered by 10% of h with a seeded half split into triangles (98,k elements), P4,
            Navier-Stokes BR2, Lax-Friedrichs, Re 1e4, Pr 0.71 (the reference's fixed value): residual, three steps
  tgv3d-ns  32^3 hexahedra P3, Navier-Stokes BR1, Roe, Re 1600, Mach 0.1: residual, three steps

Tolerances (the path computes in FP64): one-stage residual du/dt relative L2 <= 1e-12; state per conserved
variable relative L2 <= 1e-10; relative error of the last step <= 1e-9; dt <= 1e-13.  These meshes are too
large for the long-double oracle on every host (on aarch64 long double is a software binary128), so the truth
is the double-precision oracle in its parity mode (M^-1 products and projections refined by one residual
correction), whose own round-off on these problems is measured here against the long-double build on the
small 40x40 vortex and stays at the 1e-14 level.  The element-to-oracle comparison is at the volume points
(the GPU path stores nodal values, the oracle the reference's modal coefficients).
"""
import math

import numpy as np
import pytest

import subrosadg_gb300 as sdg
from oracle.orc import Oracle
from subrosadg_gb300 import workloads as wl

pytestmark = pytest.mark.gpu


def rel_l2(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def per_var(a, b):
    return [rel_l2(a[:, v], b[:, v]) for v in range(b.shape[1])]


def _pair(mesh, cfg, prim, precision="double"):
    g = sdg.GpuSolver(mesh, cfg)
    o = Oracle(mesh, cfg, faithful=False, precision=precision)
    pts = g.volume_points()
    np.testing.assert_allclose(pts, o.volume_points(), atol=1e-12)
    p0 = prim(pts)
    g.initialize_primitive(p0)
    o.initialize_primitive(p0)
    return g, o


def _check(g, o, dt, steps, residual_tol=1e-12):
    rg, ro = g.residual_point(), o.residual_point()
    err = rel_l2(rg, ro)
    assert err <= residual_tol, (err, per_var(rg, ro))
    for _ in range(steps):
        eg = g.stepSolver(dt).copy()
    o.step(dt, steps)
    pv = per_var(g.state_point(), o.state_point())
    assert max(pv) <= 1e-10, pv
    np.testing.assert_allclose(eg, o.relative_error(), rtol=1e-9, atol=1e-15)
    return err, pv


def test_vortex2d_40x40_p3_roe_200_steps():
    """The isentropic vortex at its stated size and horizon: 1,600 quadrangles P3 (102,400 DOF), Roe,
    dt 1e-3, 200 steps (t = 0.2)."""
    mesh, cfg, prim, _, dt, _ = wl.vortex_case(n=40, p=3, flux=sdg.ROE)
    g, o = _pair(mesh, cfg, prim)
    # the double oracle's own round-off, against the long-double truth, on this mesh
    x = Oracle(mesh, cfg, faithful=False, precision="extended")
    x.initialize_primitive(prim(x.volume_points()))
    truth = x.residual_point()
    assert rel_l2(o.residual_point(), truth) <= 1e-13
    assert rel_l2(g.residual_point(), truth) <= 1e-12
    err, pv = _check(g, o, dt, 200)
    print(f"vortex2d 40x40 P3 Roe: residual {err:.2e}, state after 200 steps per variable {pv}")


def test_tgv3d_64cubed_p3_hllc():
    """The headline workload: 262,144 hexahedra P3 (83,886,080 DOF), HLLC, dt from CFL 0.2."""
    mesh, cfg, prim, _, _, _ = wl.tgv_case(n=64, p=3, flux=sdg.HLLC)
    g, o = _pair(mesh, cfg, prim)
    dtg, dto = g.calculateDeltaTime(0.2), o.delta_time(0.2)
    assert abs(dtg - dto) <= 1e-13 * dto
    err, pv = _check(g, o, dtg, 3)
    print(f"tgv3d 64^3 P3 HLLC: residual {err:.2e}, state after 3 steps per variable {pv}")


def test_kh2d_ns_br2_256squared_hybrid_p4_lf():
    """The Navier-Stokes workload: 256^2 jittered quadrangles, a seeded half split into triangles, P4, BR2,
    Lax-Friedrichs, Re 1e4, Pr 0.71."""
    mesh = sdg.Mesh.box_2d(0.0, 0.0, 1.0, 1.0, 256, 256, periodic=True, jitter=0.1, split_fraction=0.5, seed=11)
    cfg = wl.ns_config(4, sdg.LAX_FRIEDRICHS, sdg.BR2, 1e-4, prandtl=0.71)
    g, o = _pair(mesh, cfg, lambda pts: wl.kh_primitive(pts[:, 0], pts[:, 1]))
    assert g.counts.block_count == 2
    dtg, dto = g.calculateDeltaTime(0.2), o.delta_time(0.2)
    assert abs(dtg - dto) <= 1e-13 * dto
    err, pv = _check(g, o, dtg, 3)
    print(f"kh2d NS BR2 256^2 hybrid P4 LF: residual {err:.2e}, state after 3 steps per variable {pv}")


def test_tgv3d_ns_br1_32cubed_p3_roe():
    """The adjoint workload's forward scheme: 32^3 hexahedra P3, Navier-Stokes BR1, Roe, Re 1600, Mach 0.1."""
    mesh, cfg, prim, _, _, _ = wl.tgv_case(n=32, p=3, flux=sdg.ROE, viscous=sdg.BR1, mu=1.0 / 1600.0)
    g, o = _pair(mesh, cfg, prim)
    dtg, dto = g.calculateDeltaTime(0.2), o.delta_time(0.2)
    assert abs(dtg - dto) <= 1e-13 * dto
    err, pv = _check(g, o, dtg, 3)
    print(f"tgv3d NS BR1 32^3 P3 Roe: residual {err:.2e}, state after 3 steps per variable {pv}")


def test_tgv3d_64cubed_graph_replay_equals_plain_launches():
    """The bench times CUDA-graph replays of the step: they give the plain-launch state bit for bit at 64^3."""
    mesh, cfg, prim, _, _, _ = wl.tgv_case(n=64, p=3, flux=sdg.HLLC)
    out = []
    for graph in (0, 1):
        g = sdg.GpuSolver(mesh, cfg)
        g.initialize_primitive(prim(g.volume_points()))
        g.lib.sdg_set_graph(g.h, graph)
        dt = g.calculateDeltaTime(0.2)
        g.stepSolver(dt, 2)
        out.append(g.state_point())
        g.close()
    assert np.array_equal(out[0], out[1])
