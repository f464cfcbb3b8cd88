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
