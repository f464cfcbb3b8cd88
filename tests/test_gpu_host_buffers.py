"""Pinned host buffers: sdg_set_state_point / sdg_get_state_point read and write page-locked host memory in
place (kernels over the CPU-GPU link); pageable buffers go through a staging copy.  Both paths run the same
arithmetic, so the states and point values they produce are bit-identical."""
import numpy as np
import pytest

import subrosadg_gb300 as sdg
from tests import cases

pytestmark = pytest.mark.gpu


def _pinned(n):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch.empty(n, dtype=torch.float64, pin_memory=True).numpy()


@pytest.mark.parametrize("name,case", [
    ("hex-p3", lambda: cases.tgv_case(n=4, p=3)),
    ("hybrid-p4", lambda: cases.kh_case(n=6, p=4)),
    ("tet-p2", lambda: cases.tet_tgv_case(n=3, p=2)),
    ("line-p3", lambda: cases.sod_1d_case(n=9, p=3)),
])
def test_pinned_and_pageable_buffers_agree(name, case):
    mesh, cfg, prim, _, dt, _ = case()
    s = sdg.GpuSolver(mesh, cfg)
    s.initialize_primitive(prim(s.volume_points()))
    s.stepSolver(dt, 1)
    nv = s.counts.conserved_variable_count
    u = s.state_point()                      # pageable download
    pin = _pinned(u.size).reshape(u.shape)
    s.state_point(pin)                       # pinned download
    np.testing.assert_array_equal(pin, u)
    modal = s.state_modal()
    rng = np.random.default_rng(3)
    v = u * (1.0 + 1e-3 * rng.standard_normal(u.shape))
    s.set_state_point(v)                     # pageable upload
    a = s.state_modal()
    pin[...] = v
    s.set_state_point(pin)                   # pinned upload
    np.testing.assert_array_equal(s.state_modal(), a)
    assert not np.array_equal(a, modal)
    out = _pinned(u.size).reshape(-1, nv)
    s.state_point(out)
    np.testing.assert_array_equal(out, s.state_point())


@pytest.mark.parametrize("name,case", [
    ("hex-p3", lambda: cases.tgv_case(n=4, p=3)),
    ("hybrid-p4", lambda: cases.kh_case(n=6, p=4)),
    ("tet-p2", lambda: cases.tet_tgv_case(n=3, p=2)),
    ("line-p3", lambda: cases.sod_1d_case(n=9, p=3)),
    ("ns-hex-p2", lambda: cases.tgv_case(n=3, p=2, viscous=sdg.BR1)),
])
def test_step_state_point_matches_step_then_download(name, case):
    """sdg_step_state_point: the last stage of tensor blocks writes the new state into a pinned buffer
    itself; the state, the point values and the relative error are those of sdg_step + sdg_get_state_point,
    bit for bit, for pinned and pageable buffers, with the step graph re-captured between the two forms."""
    mesh, cfg, prim, _, dt, _ = case()
    a = sdg.GpuSolver(mesh, cfg)
    b = sdg.GpuSolver(mesh, cfg)
    for s in (a, b):
        s.initialize_primitive(prim(s.volume_points()))
    nv = a.counts.conserved_variable_count
    pin = _pinned(a.counts.volume_point_count * nv).reshape(-1, nv)
    for step in range(3):
        err_a = a.stepSolver(dt).copy()
        u_a = a.state_point()
        if step == 1:
            u_b, err_b = b.step_state_point(dt)          # pageable: converted and copied after the step
            u_b = u_b.copy()
        else:
            pin[...] = np.nan
            u_b, err_b = b.step_state_point(dt, pin)     # pinned: written by the last stage
        np.testing.assert_array_equal(u_b, u_a)
        np.testing.assert_array_equal(err_b, err_a)
        np.testing.assert_array_equal(b.state_modal(), a.state_modal())
    b.stepSolver(dt)                                     # back to the plain step graph
    a.stepSolver(dt)
    np.testing.assert_array_equal(b.state_modal(), a.state_modal())


@pytest.mark.parametrize("name,case", [
    ("hex-p3", lambda: cases.tgv_case(n=4, p=3)),
    ("hybrid-p4", lambda: cases.kh_case(n=6, p=4)),
    ("tet-p2", lambda: cases.tet_tgv_case(n=3, p=2)),
    ("ns-hex-p2", lambda: cases.tgv_case(n=3, p=2, viscous=sdg.BR1)),
])
def test_step_state_point_from_matches_set_step_get(name, case):
    """sdg_step_state_point_from[_async]: host state in, one step, host state out.  Every call equals
    sdg_set_state_point + sdg_step + sdg_get_state_point bit for bit, for pinned and pageable buffers, and a chain
    of asynchronous calls (each call's input transfer overlapping the previous call's step) gives each call's
    own result in its own output buffer."""
    mesh, cfg, prim, _, dt, _ = case()
    a = sdg.GpuSolver(mesh, cfg)
    b = sdg.GpuSolver(mesh, cfg)
    a.initialize_primitive(prim(a.volume_points()))
    nv = a.counts.conserved_variable_count
    u0 = a.state_point()
    rng = np.random.default_rng(5)
    inputs = [u0 * (1.0 + 1e-3 * rng.standard_normal(u0.shape)) for _ in range(3)]
    expected, errs = [], []
    for u in inputs:
        a.set_state_point(u)
        errs.append(a.stepSolver(dt).copy())
        expected.append(a.state_point())
    # synchronous, pageable and pinned
    out, err = b.step_state_point_from(dt, inputs[0])
    np.testing.assert_array_equal(out, expected[0])
    np.testing.assert_array_equal(err, errs[0])
    pin_in = [_pinned(u.size).reshape(u.shape) for u in inputs]
    pin_out = [_pinned(u.size).reshape(-1, nv) for u in inputs]
    for pi, u in zip(pin_in, inputs):
        pi[...] = u
    out, err = b.step_state_point_from(dt, pin_in[1], pin_out[1])
    np.testing.assert_array_equal(pin_out[1], expected[1])
    np.testing.assert_array_equal(err, errs[1])
    # asynchronous chain
    for po in pin_out:
        po[...] = np.nan
    for pi, po in zip(pin_in, pin_out):
        b.step_state_point_from(dt, pi, po, asynchronous=True)
    b.synchronize()
    for po, e in zip(pin_out, expected):
        np.testing.assert_array_equal(po, e)
    np.testing.assert_array_equal(b.relative_error(), errs[-1])
    np.testing.assert_array_equal(b.state_modal(), a.state_modal())
