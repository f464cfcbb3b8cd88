"""The compiled C++23 caller of the C ABI: subrosadg_gb300/cpp/periodic_2d_ceuler.cpp (the reference's example
examples/periodic_2d_ceuler.cpp written against the C++ mirror of System<SC> / Solver<SC> in
subrosadg_gb300/cpp/gpu_solver.hpp), built by build().  The host-only run needs no GPU; the GPU run is compared
with the oracle on the same mesh and initial state."""
import math
import os
import subprocess

import numpy as np
import pytest

import subrosadg_gb300 as sdg
from subrosadg_gb300 import build as lib_build
from subrosadg_gb300 import workloads as wl

DRIVER = os.path.join(lib_build.LIBDIR, "sdg_periodic_2d_ceuler")


def _example_case():
    mesh = sdg.Mesh.box_2d(0.0, 0.0, 2.0, 2.0, 10, 10, periodic=True)
    cfg = wl.config(3, sdg.HLLC)

    def ic(pts):
        s = np.sin(math.pi * (pts[:, 0] + pts[:, 1]))
        return np.stack([1.0 + 0.2 * s, np.full_like(s, 0.7), np.full_like(s, 0.3), 1.4 / (1.0 + 0.2 * s)], 1)
    return mesh, cfg, ic


def test_cpp_driver_host_only(tmp_path):
    out = subprocess.run([DRIVER, "3", str(tmp_path), "--host-only"], capture_output=True, text=True, check=True)
    mesh, cfg, _ = _example_case()
    g = sdg.GpuSolver(mesh, cfg, device=-1)
    c = g.counts
    assert out.stdout.split() == ["elements", str(c.element_count), "interior_faces", str(c.interior_face_count),
                                  "boundary_faces", str(c.boundary_face_count), "volume_points",
                                  str(c.volume_point_count), "dof", str(c.degree_of_freedom_count)]


@pytest.mark.gpu
def test_cpp_driver_matches_oracle(tmp_path):
    from oracle.orc import Oracle
    steps = 40
    out = subprocess.run([DRIVER, str(steps), str(tmp_path), "20"], capture_output=True, text=True, check=True)
    mesh, cfg, ic = _example_case()
    o = Oracle(mesh, cfg, faithful=False)
    o.initialize_primitive(ic(o.volume_points()))
    o.step(1e-3, steps)
    ref = o.state_point()
    got = np.fromfile(tmp_path / "state.f64", dtype=np.float64).reshape(ref.shape)
    for v in range(4):
        assert np.linalg.norm(got[:, v] - ref[:, v]) <= 1e-10 * np.linalg.norm(ref[:, v]), v
    rel = [float(x) for x in out.stdout.split()[3:]]
    np.testing.assert_allclose(rel, o.relative_error(), rtol=1e-9, atol=1e-15)
    lines = (tmp_path / "error.txt").read_text().splitlines()
    assert lines[0] == "|    Time     |     rho     |    rho*u    |    rho*v    |    rho*E    |"
    assert len(lines) == 2 + steps
    assert float(lines[-1].split("|")[1]) == pytest.approx(steps * 1e-3)
    assert sorted(os.listdir(tmp_path / "raw")) == [f"periodic_2d_ceuler_{i}.zst" for i in (0, 20, 40)]
