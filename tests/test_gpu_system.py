"""GPU test of the System driver's outputs (src/Utils/SystemControl.cpp:159-195): raw-binary files every
io_interval steps and at step 0, error.txt with the reference's header and one line per step
(View/CommandLine.cpp:70-150), and the LastStep / SpecificFile restarts.  The driver is the reference's
sod_1d_ceuler.cpp (100 lines, P3, HLLC, artificial viscosity 0.5, farfield ends) with a fixed time step."""
import os

import numpy as np
import pytest

import subrosadg_gb300 as sdg

pytestmark = pytest.mark.gpu

LEFT, RIGHT = np.array([1.0, 0.75, 1.4]), np.array([0.125, 0.0, 0.8 * 1.4])


def sod_system(out, start=0, end=10, kind=sdg.INITIAL_FUNCTION):
    system = sdg.System(1, 3, sdg.EULER, sdg.HLLC, initial_condition_kind=kind)
    system.setMesh(sdg.Mesh.line_1d(0.0, 1.0, 100, periodic=False, boundary_conditions=[0, 0]))
    system.addBoundaryCondition(sdg.RIEMANN_FARFIELD, 1)
    system.addBoundaryCondition(sdg.RIEMANN_FARFIELD, 2)
    system.setThermodynamicModel(2.5, 25.0 / 14.0)
    system.setArtificialViscosity(0.5)
    system.setTimeIntegration(0.001, (start, end))
    system.setDeltaTime(2e-6)
    system.setViewConfig(out, "sod_1d_ceuler", 5)
    system.initial_condition = lambda x: np.where((x[:, 0] <= 0.5)[:, None], LEFT, RIGHT)
    system.boundary_condition = lambda x, phys: np.where((phys == 1)[:, None], LEFT, RIGHT)
    system.synchronize()
    return system


def test_outputs_and_last_step_restart(tmp_path):
    a = sod_system(tmp_path)
    history = a.solve()
    raw = tmp_path / "raw"
    assert sorted(os.listdir(raw)) == [f"sod_1d_ceuler_{i}.zst" for i in (0, 10, 5)]
    lines = (tmp_path / "error.txt").read_text().splitlines()
    assert lines[0] == "|{:^13}|{:^13}|{:^13}|{:^13}|".format("Time", "rho", "rho*u", "rho*E")
    assert len(lines) == 2 + 10
    for (t, err), line in zip(history, lines[2:]):
        fields = [float(x) for x in line.strip("|").split("|")]
        np.testing.assert_allclose(fields, [t, *err], rtol=1e-5)
    final = a.solver.state_point()
    # LastStep: continue from raw/sod_1d_ceuler_5.zst; error.txt keeps its first 5 + 2 lines
    b = sod_system(tmp_path, start=5, end=10, kind=sdg.INITIAL_LAST_STEP)
    b.solve()
    relines = (tmp_path / "error.txt").read_text().splitlines()
    assert relines[:7] == lines[:7] and len(relines) == 12
    np.testing.assert_allclose(b.solver.state_point(), final, rtol=1e-12, atol=1e-14)
    # SpecificFile: the state of the step-10 file
    c = sod_system(tmp_path / "again", start=0, end=0)
    c.addInitialCondition(raw / "sod_1d_ceuler_10.zst")
    c.solve()
    np.testing.assert_allclose(c.solver.state_point(), final, rtol=1e-13, atol=1e-15)


def test_time_varying_inflow_matches_oracle():
    """BoundaryTimeEnum::TimeVarying (src/Solver/TimeIntegration.cpp:333-335, BoundaryCondition.cpp:29-74): the
    System re-evaluates the ghost states at the start of every step at time iteration_ * dt (iteration_ is 0
    before the first step), here a pulsating velocity inflow into a slip-walled channel with an outflow; the
    oracle steps with the same per-step ghost states."""
    from oracle.orc import Oracle
    from tests import cases
    conditions = (sdg.ADIABATIC_SLIP_WALL, sdg.PRESSURE_OUTFLOW, sdg.ADIABATIC_SLIP_WALL, sdg.VELOCITY_INFLOW)
    mesh, cfg, ic, _, dt, _ = cases.channel_case(p=2, flux=sdg.HLLC, n=4, conditions=conditions)
    steps = 12

    def bc(x, t, phys):
        out = np.zeros((len(x), 4))
        out[:, 0] = 1.0
        out[:, 1] = np.where(phys == 4, 0.4 * (1.0 + 0.5 * np.sin(300.0 * t)) * (1.0 + 0.2 * x[:, 1]), 0.0)
        out[:, 3] = 1.0 / cases.R_GAS
        return out

    system = sdg.System(2, 2, sdg.EULER, sdg.HLLC, boundary_time=sdg.BOUNDARY_TIME_VARYING)
    system.setMesh(mesh)
    system.setThermodynamicModel(cases.CP, cases.CV)
    system.setTimeIntegration(1.0, (0, steps))
    system.setDeltaTime(dt)
    system.initial_condition = lambda x: ic(x)
    system.boundary_condition = bc
    system.synchronize()
    system.solve()
    got = system.solver.state_point()

    o = Oracle(mesh, cfg, faithful=False)
    o.initialize_primitive(ic(o.volume_points()))
    bpts, phys = o.boundary_points()
    phys = np.repeat(phys, o.nfq)
    for i in range(1, steps + 1):
        o.set_boundary_primitive(bc(bpts, (i - 1) * dt, phys))
        o.step(dt)
    ref = o.state_point()
    pv = [np.linalg.norm(got[:, v] - ref[:, v]) / np.linalg.norm(ref[:, v]) for v in range(4)]
    assert max(pv) <= 1e-10, pv
    # the ghost states did change: a steady run at the time-0 inflow ends elsewhere
    s = sdg.System(2, 2, sdg.EULER, sdg.HLLC)
    s.setMesh(mesh)
    s.setThermodynamicModel(cases.CP, cases.CV)
    s.setTimeIntegration(1.0, (0, steps))
    s.setDeltaTime(dt)
    s.initial_condition = lambda x: ic(x)
    s.boundary_condition = lambda x, phys: bc(x, 0.0, phys)
    s.synchronize()
    s.solve()
    assert np.linalg.norm(s.solver.state_point() - ref) > 1e-6 * np.linalg.norm(ref)
