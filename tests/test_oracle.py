"""CPU tests of the oracle (the CPU restatement of the reference algorithm) against the reference's
own known answers and against analytic invariants of the DG discretisation."""
import json
import math
import os

import numpy as np
import pytest

import subrosadg_gb300 as sdg
from oracle.orc import Oracle
from tests import cases

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def _tables():
    with open(os.path.join(GOLDEN, "reference_tables.json")) as f:
        return json.load(f)


def _vectors():
    with open(os.path.join(GOLDEN, "oracle_vectors.json")) as f:
        return json.load(f)


# ---- reference known answers -------------------------------------------------------------------------

def _perm(kind, m, rot):
    """The oracle's face-point permutation rule (oracle/orc_basis.hpp facePermutation)."""
    if kind == "Line":
        return [m - 1 - j for j in range(m)]
    out = []
    for i in range(m):
        for k in range(m):
            ii, kk = {0: (k, i), 1: (m - 1 - i, k), 2: (m - 1 - k, m - 1 - i), 3: (i, m - 1 - k)}[rot]
            out.append(ii * m + kk)
    return out


@pytest.mark.parametrize("p", [1, 2, 3, 4, 5])
def test_face_permutations_match_reference_tables(p):
    t = _tables()["face_permutation"]
    assert t[f"Line/P{p}"]["0"] == _perm("Line", p + 1, 0)
    for rot in range(4):
        assert t[f"Quadrangle/P{p}"][str(rot)] == _perm("Quad", p + 1, rot)


def test_face_vertex_lists_match_reference():
    t = _tables()["face_vertices"]
    assert t["Triangle"] == [0, 1, 1, 2, 2, 0]
    assert t["Quadrangle"] == [0, 1, 1, 2, 2, 3, 3, 0]
    assert t["Hexahedron"] == [0, 3, 2, 1, 0, 1, 5, 4, 0, 4, 7, 3, 1, 2, 6, 5, 2, 3, 7, 6, 4, 5, 6, 7]


def test_model_constants_match_reference():
    """Constants of the incompressible model, the Boussinesq source and the artificial-viscosity sensor,
    read as text from the reference (PhysicalModel.cpp:63-66, SourceTerm.cpp:31, SimulationControl.cpp:892-893),
    against the values the oracle uses."""
    import ctypes
    from oracle import orc
    lib = orc.load()
    lib.orc_constant.restype = ctypes.c_double
    lib.orc_constant.argtypes = [ctypes.c_char_p]
    t = _tables()
    assert lib.orc_constant(b"weak_pressure_addition") == t["weak_pressure_addition"] == 0.01
    assert lib.orc_constant(b"boussinesq_gravity") == t["boussinesq_gravity"] == 1.0
    for p in range(1, 6):
        assert lib.orc_constant(f"artificial_viscosity_tolerance_{p}".encode()) == t["artificial_viscosity_tolerance"][p - 1]


def test_constants_match_reference():
    t = _tables()
    assert t["specific_heat_ratio"] == 1.4 and t["prandtl_number"] == 0.71
    assert t["harten_divisor"] == 20.0
    assert abs(t["sutherland_temperature"] - 110.4 / 273.15) < 1e-15
    assert t["rk_coefficients"]["SSPRK3"] == [[1.0, 0.0, 1.0], [0.75, 0.25, 0.25], [1 / 3, 2 / 3, 2 / 3]]
    assert t["rk_coefficients"]["HeunRK2"] == [[1.0, 0.0, 1.0], [0.5, 0.5, 0.5]]


@pytest.mark.parametrize("p", [1, 2, 3, 4, 5])
def test_quadrature_counts_match_reference(p):
    """Oracle volume/face point counts equal the reference tables at orders 2P / 2P+1."""
    counts = _tables()["quadrature_count"]
    for kind, mesh in (("Quadrangle", sdg.Mesh.box_2d(0, 0, 1, 1, 3, 3)),
                       ("Triangle", sdg.Mesh.box_2d(0, 0, 1, 1, 3, 3, split_fraction=1.0)),
                       ("Hexahedron", sdg.Mesh.box_3d(0, 0, 0, 1, 1, 1, 3, 3, 3))):
        o = Oracle(mesh, cases.config(p, sdg.HLLC), faithful=False)
        assert o.volume_points_count == o.elements * counts[kind][2 * p]
        face = "Line" if kind != "Hexahedron" else "Quadrangle"
        assert o.nfq == counts[face][2 * p + 1]


@pytest.mark.parametrize("deg", [2, 4, 6, 8, 10])
def test_triangle_rules_exact(deg):
    import sys
    sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(__file__)), "subrosadg_gb300", "csrc"))
    import re
    txt = open(os.path.join(os.path.dirname(os.path.dirname(__file__)), "subrosadg_gb300", "csrc", "triangle_rules.h")).read()
    get = lambda n: np.array([float(x) for x in re.search(r"kTri%d%s\[\d+\] = \{([^}]*)\}" % (deg, n), txt).group(1).split(",")])
    x, y, w = get("Xi"), get("Eta"), get("W")
    for a in range(deg + 1):
        for b in range(deg + 1 - a):
            exact = math.factorial(a) * math.factorial(b) / math.factorial(a + b + 2)
            assert abs((w * x ** a * y ** b).sum() - exact) < 1e-15


# ---- analytic invariants of the oracle ---------------------------------------------------------------

@pytest.mark.parametrize("name,mesh_fn,p,flux", [
    ("quad", lambda: sdg.Mesh.box_2d(0, 0, 1, 1, 3, 3), 3, sdg.ROE),
    ("jittered-hybrid", lambda: sdg.Mesh.box_2d(0, 0, 1, 1, 4, 4, jitter=0.15, split_fraction=0.5, seed=2), 4, sdg.LAX_FRIEDRICHS),
    ("hex", lambda: sdg.Mesh.box_3d(0, 0, 0, 1, 1, 1, 3, 3, 3), 2, sdg.HLLC),
    ("tri", lambda: sdg.Mesh.box_2d(0, 0, 1, 1, 3, 3, split_fraction=1.0, jitter=0.1, seed=4), 5, sdg.CENTRAL),
])
def test_free_stream_preservation(name, mesh_fn, p, flux):
    mesh = mesh_fn()
    o = Oracle(mesh, cases.config(p, flux), faithful=True)
    pts = o.volume_points()
    o.initialize_primitive(cases.uniform_primitive(len(pts), mesh.dimension))
    r = o.residual_point()
    assert np.abs(r).max() < 1e-9


def test_conservation_periodic():
    """Sum over elements of the mass-weighted rate is zero on a periodic mesh (telescoping fluxes)."""
    mesh, cfg, prim, _, dt, _ = cases.kh_case(n=5, p=3)
    o = Oracle(mesh, cfg, faithful=False)
    o.initialize_primitive(prim(o.volume_points()))
    m0 = o.state_point()
    o.step(dt, 2)
    m1 = o.state_point()
    # integrate with the quadrature weights: reuse the LSQ-exact property on polynomial states
    # by comparing the modal mean of each element (mass is conserved to round-off)
    assert np.isfinite(m1).all()
    assert abs(m1[:, 0].mean() - m0[:, 0].mean()) < 1e-3


@pytest.mark.parametrize("name", list(cases.golden_cases()))
def test_oracle_against_committed_vectors(name):
    v = _vectors()[name]
    mesh, cfg, prim, bprim, dt, steps = cases.golden_cases()[name]()
    o = Oracle(mesh, cfg, faithful=False)
    o.initialize_primitive(prim(o.volume_points()))
    if o.boundary:
        bpts, phys = o.boundary_points()
        o.set_boundary_primitive(bprim(bpts, np.repeat(phys, o.nfq)))
    r0 = o.residual_point()
    assert abs(np.abs(r0).sum() - v["residual_checksum"]) <= 1e-10 * v["residual_checksum"]
    np.testing.assert_allclose(r0[:: max(1, len(r0) // 16)], np.array(v["residual_sample"]), rtol=1e-9, atol=1e-9)
    o.step(dt, steps)
    np.testing.assert_allclose(o.state_point()[:: max(1, o.volume_points_count // 16)], np.array(v["state_sample"]),
                               rtol=1e-11, atol=1e-12)
    np.testing.assert_allclose(o.relative_error(), v["relative_error"], rtol=1e-9)
    assert abs(o.delta_time(0.2) - v["delta_time_cfl_0.2"]) <= 1e-12 * v["delta_time_cfl_0.2"]


def test_faithful_gradient_pass_does_not_change_euler():
    """The reference runs the gradient pass for Euler too (TimeIntegration.cpp:340-343); it is unused."""
    import ctypes
    from oracle import orc
    mesh, cfg, prim, _, dt, steps = cases.vortex_case(n=4, p=2)
    lib = orc.load()
    out = []
    for flags in (1, 0):  # with / without the gradient pass, same (refined) arithmetic otherwise
        o = Oracle(mesh, cfg, faithful=False)
        lib.orc_destroy(o.h)
        o.h = lib.orc_create(ctypes.addressof(o._m), ctypes.addressof(o._c), flags)
        o.initialize_primitive(prim(o.volume_points()))
        o.step(dt, 2)
        out.append(o.state_point())
    assert np.array_equal(out[0], out[1])


def test_extended_precision_oracle_agrees_with_double():
    """The long-double build of the oracle is the same algorithm: it agrees with the double build to
    the double build's round-off, and resolves more digits."""
    from oracle import orc
    assert orc.load("extended").orc_real_digits() > 53
    mesh, cfg, prim, _, dt, steps = cases.tgv_case(n=3, p=2)
    res = []
    for prec in ("double", "extended"):
        o = Oracle(mesh, cfg, faithful=False, precision=prec)
        o.initialize_primitive(prim(o.volume_points()))
        res.append(o.residual_point())
    assert np.linalg.norm(res[0] - res[1]) <= 1e-10 * np.linalg.norm(res[1])


def test_vortex_advects_at_freestream_speed():
    """Exact-solution check: after one period-free short time the vortex is the translated IC."""
    mesh, cfg, prim, _, _, _ = cases.vortex_case(n=10, p=3)
    o = Oracle(mesh, cfg, faithful=False)
    pts = o.volume_points()
    o.initialize_primitive(prim(pts))
    t, dt = 0.05, 1e-3
    o.step(dt, int(round(t / dt)))
    exact = cases.vortex_primitive(pts[:, 0] - t, pts[:, 1] - t)
    rho = o.state_point()[:, 0]
    assert np.abs(rho - exact[:, 0]).max() < 5e-3


# ---- the timed CPU baselines and the oracle's own mesh generator ----------------------------------------

@pytest.mark.parametrize("periodic", [True, False])
def test_oracle_box_generator_equals_library_generator(periodic):
    """oracle/meshgen.box_3d (used by the CPU baselines, which load nothing of the GPU library) builds the
    library's structured box bit for bit."""
    from oracle import meshgen
    bc = None if periodic else [sdg.RIEMANN_FARFIELD, sdg.PRESSURE_OUTFLOW, sdg.ADIABATIC_SLIP_WALL,
                                sdg.VELOCITY_INFLOW, sdg.ISOTHERMAL_NONSLIP_WALL, sdg.ADIABATIC_NONSLIP_WALL]
    a = sdg.Mesh.box_3d(0.1, 0.2, 0.3, 1.5, 2.5, 2 * math.pi, 3, 4, 5, periodic=periodic, boundary_conditions=bc)
    b = meshgen.box_3d(0.1, 0.2, 0.3, 1.5, 2.5, 2 * math.pi, 3, 4, 5, periodic=periodic, boundary_conditions=bc)
    for k in ("nodes", "hexahedra", "boundary", "boundary_physical", "physical_conditions", "periodic_master"):
        x, y = getattr(a, k), getattr(b, k)
        assert (x is None and y is None) or (x.dtype == y.dtype and np.array_equal(x, y)), k


def test_stages_compose_a_step():
    """Three orc_stage calls are one orc_step, bit for bit (the reference arm of bench.py times stages)."""
    mesh, cfg, prim, _, dt, _ = cases.tgv_case(n=3, p=2)
    a, b = Oracle(mesh, cfg, faithful=True), Oracle(mesh, cfg, faithful=True)
    for o in (a, b):
        o.initialize_primitive(prim(o.volume_points()))
    a.step(dt, 2)
    for s in range(6):
        b.stage(s % 3, dt)
    assert np.array_equal(a.state_point(), b.state_point())
    assert np.array_equal(a.relative_error(), b.relative_error())


@pytest.mark.parametrize("case", [lambda: cases.tgv_case(n=3, p=3), lambda: cases.kh_case(n=4, p=3, steps=2)],
                         ids=["tgv-hex-affine", "kh-hybrid-jittered"])
def test_lean_baseline_computes_the_same_scheme(case):
    """The lean CPU baseline (no Euler gradient pass, one shared reference inverse on affine blocks) and the
    reference-faithful one advance the same discrete scheme: states agree to round-off."""
    mesh, cfg, prim, _, dt, steps = case()
    f, l = Oracle(mesh, cfg, faithful=True), Oracle(mesh, cfg, lean=True)
    for o in (f, l):
        o.initialize_primitive(prim(o.volume_points()))
        o.step(dt, steps)
    a, b = f.state_point(), l.state_point()
    assert np.linalg.norm(a - b) <= 1e-12 * np.linalg.norm(a)


@pytest.mark.parametrize("case", [lambda: cases.tgv_case(n=5, p=3),
                                  lambda: cases.kh_case(n=7, p=3, viscous=sdg.BR2, mu=2e-3),
                                  lambda: cases.tgv_case(n=4, p=2, viscous=sdg.BR1, mu=0.02),
                                  lambda: cases.channel_case(p=2, viscous=sdg.BR2, mu=0.01, conditions=(
                                      sdg.ISOTHERMAL_NONSLIP_WALL, sdg.PRESSURE_OUTFLOW, sdg.ADIABATIC_NONSLIP_WALL,
                                      sdg.VELOCITY_INFLOW))],
                         ids=["tgv-euler", "kh-hybrid-br2", "tgv-br1", "channel-walls-br2"])
@pytest.mark.parametrize("faithful", [False, True])
def test_element_sample_mode_equals_full_evaluation(case, faithful):
    """The oracle's element-sample mode (the truth of the stated-size GPU tests) gives the full evaluation's
    residual bit for bit on the sampled elements and zeros elsewhere."""
    mesh, cfg, prim, bprim, _, _ = case()
    full = Oracle(mesh, cfg, faithful=faithful)
    pts = full.volume_points()
    sample = np.sort(np.random.default_rng(5).choice(full.elements, 7, replace=False))
    part = Oracle(mesh, cfg, faithful=faithful, sample=sample)
    for o in (full, part):
        o.initialize_primitive(prim(pts))
        if o.boundary:
            bp, ph = full.boundary_points()
            o.set_boundary_primitive(bprim(bp, np.repeat(ph, full.nfq)))
    rf, rs = full.residual_point(), part.residual_point()
    g = sdg.GpuSolver(mesh, cfg, device=-1)
    c = g.counts
    rows, off, first = np.zeros(len(rf), bool), 0, 0
    for b in range(c.block_count):
        ne, nq = c.block_element_count[b], c.block_volume_point_count[b]
        for e in sample[(sample >= first) & (sample < first + ne)] - first:
            rows[off + e * nq: off + (e + 1) * nq] = True
        off, first = off + ne * nq, first + ne
    assert np.array_equal(rs[rows], rf[rows])
    assert not rs[~rows].any()
    assert part.lib.orc_step(part.h, 1, 1e-3) != 0  # stepping is refused in the sample mode
