"""GPU parity at the benchmark configurations' stated sizes (the workloads bench.py times), through the C ABI.

  vortex2d  40x40 quadrangles P3, Roe, dt 1e-3: the one-stage residual and the state after all 200 SSP-RK3
            steps (long-horizon round-off growth)
  tgv3d     64^3 hexahedra P3, HLLC, dt from CFL 0.2: one-stage residual, dt, three steps
  kh2d-ns   256^2 quadrangles jittered by 10% of h with a seeded half split into triangles, P4, Navier-Stokes
            BR2, Lax-Friedrichs, Re 1e4, Pr 0.71 (the reference's fixed value): residual, dt, three steps
  tgv3d-ns  32^3 hexahedra P3, Navier-Stokes BR1, Roe, Re 1600, Mach 0.1: residual, dt, three steps

Tolerances (the path computes in FP64):
  * one-stage residual du/dt, relative L2 against the truth <= 1e-12, or -- where the reference's own FP64
    arithmetic misses the truth by more than that -- at least 10x closer to the truth than that arithmetic.
    The truth is the long-double oracle; on these meshes it runs in its element-sample mode (the residual of a
    seeded sample of elements, which equals the full evaluation there: a residual depends only on an element and
    its face neighbours), and the reference's FP64 arithmetic is the faithful double oracle on the same sample.
    At Mach 0.1 the residual is a small difference of O(p0) fluxes, so this problem's own conditioning puts the
    reference's FP64 residual 1e-9..1e-8 away from the truth at these sizes;
  * state after N steps per conserved variable, L2 difference against the double oracle <= 1e-10 of the
    variable's scale (its own norm; for a momentum component the momentum's norm), over the whole mesh;
  * relative error of the last step <= 1e-9; dt <= 1e-13.
States and residuals are compared at the volume points (the GPU path stores nodal values, the oracle the
reference's modal coefficients).
"""
import numpy as np
import pytest

import subrosadg_gb300 as sdg
from oracle.orc import Oracle
from subrosadg_gb300 import workloads as wl

pytestmark = pytest.mark.gpu

SAMPLE = 256  # sampled elements of the residual truth


def rel_l2(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def per_var(a, b):
    return [rel_l2(a[:, v], b[:, v]) for v in range(b.shape[1])]


def per_var_scaled(a, b):
    """Per conserved variable, the L2 difference over the variable's natural scale: its own norm, and for the
    momentum components the norm of the whole momentum (a component that is zero in the initial state, as the
    Taylor-Green vortex's rho w, carries only round-off of the momentum's size)."""
    d = b.shape[1] - 2
    mom = np.linalg.norm(b[:, 1:1 + d])
    out = []
    for v in range(b.shape[1]):
        scale = max(np.linalg.norm(b[:, v]), mom if 1 <= v <= d else 0.0, 1e-300)
        out.append(float(np.linalg.norm(a[:, v] - b[:, v]) / scale))
    return out


def sample_rows(g, sample):
    """Volume-point rows of the sampled elements (global element indices in block order)."""
    c = g.counts
    rows, off, first = [], 0, 0
    for b in range(c.block_count):
        ne, nq = c.block_element_count[b], c.block_volume_point_count[b]
        sel = sample[(sample >= first) & (sample < first + ne)] - first
        rows.append((off + sel[:, None] * nq + np.arange(nq)[None, :]).ravel())
        off += ne * nq
        first += ne
    return np.concatenate(rows)


def check_residual(mesh, cfg, g, p0, seed):
    """GPU residual on a seeded element sample against the long-double truth and the reference arithmetic."""
    sample = np.sort(np.random.default_rng(seed).choice(g.counts.element_count, SAMPLE, replace=False))
    rows = sample_rows(g, sample)
    rg = g.residual_point()[rows]
    truth = Oracle(mesh, cfg, faithful=False, precision="extended", sample=sample)
    truth.initialize_primitive(p0)
    rt = truth.residual_point()[rows]
    del truth
    ref = Oracle(mesh, cfg, faithful=True, precision="double", sample=sample)
    ref.initialize_primitive(p0)
    rr = ref.residual_point()[rows]
    del ref
    err, ref_err = rel_l2(rg, rt), rel_l2(rr, rt)
    assert err <= 1e-12 or (ref_err > 1e-12 and err <= 0.1 * ref_err), (err, ref_err, per_var(rg, rt))
    return err, ref_err


def run(mesh, cfg, prim, steps, dt=None, seed=0):
    g = sdg.GpuSolver(mesh, cfg)
    p0 = prim(g.volume_points())
    g.initialize_primitive(p0)
    err, ref_err = check_residual(mesh, cfg, g, p0, seed)
    o = Oracle(mesh, cfg, faithful=False, precision="double")
    o.initialize_primitive(p0)
    if dt is None:
        dtg, dto = g.calculateDeltaTime(0.2), o.delta_time(0.2)
        assert abs(dtg - dto) <= 1e-13 * dto
        dt = dtg
    for _ in range(steps):
        eg = g.stepSolver(dt).copy()
    o.step(dt, steps)
    pv = per_var_scaled(g.state_point(), o.state_point())
    assert max(pv) <= 1e-10, pv
    np.testing.assert_allclose(eg, o.relative_error(), rtol=1e-9, atol=1e-15)
    return err, ref_err, pv


def test_vortex2d_40x40_p3_roe_200_steps():
    """The isentropic vortex at its stated size and horizon: 1,600 quadrangles P3 (102,400 DOF), Roe,
    dt 1e-3, 200 steps (t = 0.2)."""
    mesh, cfg, prim, _, dt, _ = wl.vortex_case(n=40, p=3, flux=sdg.ROE)
    err, ref_err, pv = run(mesh, cfg, prim, 200, dt=dt, seed=1)
    print(f"vortex2d 40^2 P3 Roe: residual {err:.2e} (reference arithmetic {ref_err:.2e}), "
          f"state after 200 steps per variable {pv}")


def test_tgv3d_64cubed_p3_hllc():
    """The headline workload: 262,144 hexahedra P3 (83,886,080 DOF), HLLC, dt from CFL 0.2."""
    mesh, cfg, prim, _, _, _ = wl.tgv_case(n=64, p=3, flux=sdg.HLLC)
    err, ref_err, pv = run(mesh, cfg, prim, 3, seed=2)
    print(f"tgv3d 64^3 P3 HLLC: residual {err:.2e} (reference arithmetic {ref_err:.2e}), "
          f"state after 3 steps per variable {pv}")


def test_kh2d_ns_br2_256squared_hybrid_p4_lf():
    """The Navier-Stokes workload: 256^2 jittered quadrangles, a seeded half split into triangles, P4, BR2,
    Lax-Friedrichs, Re 1e4, Pr 0.71."""
    mesh = sdg.Mesh.box_2d(0.0, 0.0, 1.0, 1.0, 256, 256, periodic=True, jitter=0.1, split_fraction=0.5, seed=11)
    cfg = wl.ns_config(4, sdg.LAX_FRIEDRICHS, sdg.BR2, 1e-4, prandtl=0.71)
    err, ref_err, pv = run(mesh, cfg, lambda pts: wl.kh_primitive(pts[:, 0], pts[:, 1]), 3, seed=3)
    print(f"kh2d NS BR2 256^2 hybrid P4 LF: residual {err:.2e} (reference arithmetic {ref_err:.2e}), "
          f"state after 3 steps per variable {pv}")


def test_tgv3d_ns_br1_32cubed_p3_roe():
    """The adjoint workload's forward scheme: 32^3 hexahedra P3, Navier-Stokes BR1, Roe, Re 1600, Mach 0.1."""
    mesh, cfg, prim, _, _, _ = wl.tgv_case(n=32, p=3, flux=sdg.ROE, viscous=sdg.BR1, mu=1.0 / 1600.0)
    err, ref_err, pv = run(mesh, cfg, prim, 3, seed=4)
    print(f"tgv3d NS BR1 32^3 P3 Roe: residual {err:.2e} (reference arithmetic {ref_err:.2e}), "
          f"state after 3 steps per variable {pv}")


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
