"""GPU tests of the execution modes: CUDA-graph replay, autotuned tiles, batched persistent launches.

Every mode runs the same per-element and per-point arithmetic as the plain one-instance launches, so the
states they produce must be identical bit for bit (tiles only regroup elements into CTAs; the batch only
regroups CTAs into launches).  The relative-error sums depend on the tile grouping, so they are compared
bit for bit where the tiles agree and to 1e-12 where they do not.  Parity of the one-instance path with the
oracle is covered by test_gpu_parity.py.
"""
import numpy as np
import pytest

import subrosadg_gb300 as sdg
from tests import cases

pytestmark = pytest.mark.gpu


def make(case):
    mesh, cfg, prim, bprim, dt, steps = case
    s = sdg.GpuSolver(mesh, cfg, device=0)
    s.initialize_primitive(prim(s.volume_points()))
    if bprim is not None:
        pts, phys = s.boundary_points()
        nfq = s.counts.face_point_count
        s.set_boundary_primitive(bprim(pts, np.repeat(phys, nfq)))
    return s, dt, steps


MIXED = {
    "euler-quad-p3-roe": lambda: cases.vortex_case(n=5, p=3, flux=sdg.ROE),
    "euler-hybrid-p4-lf": lambda: cases.kh_case(n=5, p=4),
    "ns-quad-p2-br2": lambda: cases.vortex_case(n=4, p=2, flux=sdg.HLLC, viscous=sdg.BR2, mu=0.05),
    "ns-tri-p1-br1": lambda: cases.kh_case(n=5, p=1, split=1.0, flux=sdg.ROE, viscous=sdg.BR1, mu=2e-3),
    "euler-quad-p1-jitter": lambda: cases.kh_case(n=6, p=1, split=0.0, jitter=0.1),
    "euler-hex-p2-hllc": lambda: cases.tgv_case(n=3, p=2),
    "ns-hex-p3-br1-roe": lambda: cases.tgv_case(n=3, p=3, flux=sdg.ROE, viscous=sdg.BR1, mu=0.02),
    "euler-channel-walls-hybrid": lambda: cases.channel_case(p=3, flux=sdg.LAX_FRIEDRICHS, n=4, split=0.5,
                                                             jitter=0.1),
    "ns-channel-walls-p2": lambda: cases.channel_case(p=2, flux=sdg.HLLC, n=4, viscous=sdg.BR2, mu=0.01,
                                                      conditions=(sdg.ISOTHERMAL_NONSLIP_WALL, sdg.PRESSURE_OUTFLOW,
                                                                  sdg.ADIABATIC_NONSLIP_WALL, sdg.VELOCITY_INFLOW)),
    "euler-warped-hex-p3-hllc": lambda: cases.warped(cases.tgv_case(n=3, p=3)),
    "ns-curved-hex-p2-q2-br2": lambda: cases.curved_hex(cases.tgv_case(n=3, p=2, flux=sdg.LAX_FRIEDRICHS,
                                                                        viscous=sdg.BR2, mu=0.02), 2),
    "euler-line-p3-hllc": lambda: cases.density_wave_1d_case(n=20, p=3),
    "euler-tet-p2-roe": lambda: cases.tet_tgv_case(n=3, p=2, flux=sdg.ROE),
    "euler-tet-box-p3-hllc": lambda: cases.tet_box_case(p=3, flux=sdg.HLLC),
    "ns-tet-p2-br2-lf": lambda: cases.tet_tgv_case(n=3, p=2, flux=sdg.LAX_FRIEDRICHS, viscous=sdg.BR2, mu=0.02),
    # artificial viscosity: the per-step sensor passes run as batched levels before stage 0
    "av-shocktube-hybrid-p2-lf": lambda: cases.shock_tube_case(p=2, flux=sdg.LAX_FRIEDRICHS, split=0.5, jitter=0.1),
    "av-sod-line-p3-hllc": lambda: cases.sod_1d_case(n=99, p=3),
    "av-shocktube-tet-p2-hllc": lambda: cases.shock_tube_case(p=2, dim=3, n=8, tets=True),
    "ns-line-walls-p2-br2": lambda: _ns(cases.sod_1d_case(n=30, p=2, av=False, smooth=0.05, dt=1e-5,
                                                          conditions=(sdg.ISOTHERMAL_NONSLIP_WALL, sdg.RIEMANN_FARFIELD)),
                                        sdg.BR2, 0.01),
}


def _ns(case, viscous, mu):
    mesh, cfg, prim, bprim, dt, steps = case
    return (mesh, cases.ns_config(cfg.polynomial_order, cfg.convective_flux, viscous, mu), prim, bprim, dt, steps)


@pytest.mark.parametrize("name", ["euler-hybrid-p4-lf", "ns-hex-p3-br1-roe", "ns-tri-p1-br1", "ns-line-walls-p2-br2"])
def test_graph_replay_equals_plain_launches(name):
    a, dt, steps = make(MIXED[name]())
    b, _, _ = make(MIXED[name]())
    b.set_graph(False)
    ra = a.stepSolver(dt, steps).copy()
    rb = b.stepSolver(dt, steps).copy()
    assert np.array_equal(a.state_point(), b.state_point())
    assert np.array_equal(ra, rb)
    assert a.launch_count() == b.launch_count()


@pytest.mark.parametrize("name", ["euler-hybrid-p4-lf", "ns-hex-p3-br1-roe", "euler-hex-p2-hllc", "ns-quad-p2-br2"])
def test_autotuned_tiles_give_the_same_state(name):
    a, dt, steps = make(MIXED[name]())
    b, _, _ = make(MIXED[name]())
    before = [b.tile(k) for k in range(b.counts.block_count)]
    tuned = b.autotune(retime=True)
    assert len(tuned) == len(before)
    assert np.array_equal(a.state_point(), b.state_point())  # tuning does not touch the state
    ra = a.stepSolver(dt, steps).copy()
    rb = b.stepSolver(dt, steps).copy()
    assert np.array_equal(a.state_point(), b.state_point())
    assert np.allclose(ra, rb, rtol=1e-12, atol=0.0)


def test_explicit_tiles_give_the_same_state():
    a, dt, steps = make(MIXED["euler-hybrid-p4-lf"]())
    b, _, _ = make(MIXED["euler-hybrid-p4-lf"]())
    b.set_tile(0, 3, 64, 2, 128)   # triangles P4: dense block, 3 elements per CTA on 64 threads
    b.set_tile(1, 1, 0, 1, 0)      # quadrangles P4: tensor block, one element per CTA
    a.stepSolver(dt, steps)
    b.stepSolver(dt, steps)
    assert np.array_equal(a.state_point(), b.state_point())


def _twins(names):
    batch = [make(MIXED[n]()) for n in names]
    alone = [make(MIXED[n]()) for n in names]
    return batch, alone


@pytest.mark.parametrize("persist", [0, 2])
def test_batch_equals_each_instance_alone(persist):
    names = list(MIXED)
    batch, alone = _twins(names)
    b = sdg.Batch([s for s, _, _ in batch])
    b.set_persistence(persist)
    b.set_delta_time([dt for _, dt, _ in batch])
    c = b.counts()
    assert c["instance_count"] == len(names)
    assert c["launches_per_step"] < c["sequential_launches_per_step"]
    b.step(3)
    for (s, dt, _), (t, _, _), n in zip(batch, alone, names):
        rt = t.stepSolver(dt, 3).copy()
        assert np.array_equal(s.state_point(), t.state_point()), n
        assert np.array_equal(s.relative_error(), rt), n
    b.close()


def test_batch_sequential_mode_equals_batched_mode():
    names = ["euler-quad-p3-roe", "ns-tri-p1-br1", "euler-hex-p2-hllc"]
    first, second = _twins(names)
    b1 = sdg.Batch([s for s, _, _ in first])
    b2 = sdg.Batch([s for s, _, _ in second])
    dts = [dt for _, dt, _ in first]
    b1.set_delta_time(dts)
    b2.set_delta_time(dts)
    b1.step(2)
    b2.step_sequential_async(2)
    b2.synchronize()
    for (s, _, _), (t, _, _) in zip(first, second):
        assert np.array_equal(s.state_point(), t.state_point())
    b1.close()
    b2.close()


def test_batch_autotune_restores_states_and_keeps_results():
    names = ["euler-hybrid-p4-lf", "ns-quad-p2-br2", "euler-hex-p2-hllc", "euler-quad-p3-roe"]
    batch, alone = _twins(names)
    b = sdg.Batch([s for s, _, _ in batch])
    b.set_delta_time([dt for _, dt, _ in batch])
    start = [s.state_point() for s, _, _ in batch]
    b.autotune(retime=True)
    for (s, _, _), u0 in zip(batch, start):
        assert np.array_equal(s.state_point(), u0)
    b.step(2)
    for (s, dt, _), (t, _, _) in zip(batch, alone):
        t.stepSolver(dt, 2)
        assert np.array_equal(s.state_point(), t.state_point())
    b.close()


def test_batch_new_delta_time_without_recapture():
    names = ["euler-quad-p3-roe", "ns-quad-p2-br2"]
    batch, alone = _twins(names)
    b = sdg.Batch([s for s, _, _ in batch])
    dts = np.array([dt for _, dt, _ in batch])
    b.set_delta_time(dts)
    b.step(1)
    b.set_delta_time(dts * 0.5)
    b.step(1)
    for (s, dt, _), (t, _, _) in zip(batch, alone):
        t.stepSolver(dt, 1)
        t.stepSolver(dt * 0.5, 1)
        assert np.array_equal(s.state_point(), t.state_point())
    b.close()
