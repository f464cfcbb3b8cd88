"""GPU tests of the raw-binary solution files (the reference's writeRawBinary and its LastStep / SpecificFile
restarts, src/View/RawBinary.cpp:42-191, src/Solver/InitialCondition.cpp:40-80).

The file is decoded here independently of the library (libzstd through ctypes): header = ZSTD_compressBound of
the payload, payload = per element the column-major (d+2) x Nb modal coefficients (Navier-Stokes: then the
(d+2)*d x Nb gradient coefficients), per boundary face its parent's coefficients, one zero per mesh node.
"""
import ctypes
import ctypes.util

import numpy as np
import pytest

import subrosadg_gb300 as sdg
from tests import cases

pytestmark = pytest.mark.gpu


def _zstd():
    name = ctypes.util.find_library("zstd") or "libzstd.so.1"
    try:
        z = ctypes.CDLL(name)
    except OSError:
        pytest.skip("libzstd is not available")
    z.ZSTD_compressBound.restype = ctypes.c_size_t
    z.ZSTD_compressBound.argtypes = [ctypes.c_size_t]
    z.ZSTD_decompress.restype = ctypes.c_size_t
    z.ZSTD_decompress.argtypes = [ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p, ctypes.c_size_t]
    z.ZSTD_isError.restype = ctypes.c_uint
    z.ZSTD_isError.argtypes = [ctypes.c_size_t]
    return z


def decode(path):
    z = _zstd()
    data = open(path, "rb").read()
    header = int.from_bytes(data[:8], "little")
    frame = data[8:]
    out = ctypes.create_string_buffer(header)
    got = z.ZSTD_decompress(out, header, frame, len(frame))
    assert not z.ZSTD_isError(got)
    assert header == z.ZSTD_compressBound(got)
    return np.frombuffer(out.raw[:got], dtype=np.float64)


def make(case):
    mesh, cfg, prim, bprim, dt, _ = case
    s = sdg.GpuSolver(mesh, cfg, device=0)
    s.initialize_primitive(prim(s.volume_points()))
    if bprim is not None:
        pts, phys = s.boundary_points()
        s.set_boundary_primitive(bprim(pts, np.repeat(phys, s.counts.face_point_count)))
    return s, dt, mesh


@pytest.mark.parametrize("name,case", [
    ("euler-hybrid-p3", lambda: cases.kh_case(n=4, p=3, steps=1)),
    ("ns-hex-p2-br1", lambda: cases.tgv_case(n=3, p=2, viscous=sdg.BR1, mu=0.02)),
    ("ns-channel-walls-p2-br2", lambda: cases.channel_case(p=2, n=3, viscous=sdg.BR2, mu=0.01,
                                                           conditions=(sdg.ISOTHERMAL_NONSLIP_WALL, sdg.PRESSURE_OUTFLOW,
                                                                       sdg.ADIABATIC_SLIP_WALL, sdg.VELOCITY_INFLOW))),
    ("euler-line-p3-farfield", lambda: cases.sod_1d_case(n=9, p=3, av=False)),
    ("ns-line-p2-br1", lambda: cases.density_wave_1d_case(n=8, p=2, viscous=sdg.BR1, mu=0.01)),
    ("euler-tet-p3", lambda: cases.tet_tgv_case(n=3, p=3)),
    ("ns-tet-walls-p2-br2", lambda: cases.tet_box_case(p=2, viscous=sdg.BR2, mu=0.01,
                                                      conditions=(sdg.ADIABATIC_NONSLIP_WALL,) * 6)),
])
def test_raw_binary_layout(tmp_path, name, case):
    s, dt, mesh = make(case())
    s.stepSolver(dt, 2)
    path = tmp_path / "state.zst"
    s.writeRawBinary(path)
    payload = decode(path)
    c = s.counts
    nv, d = c.conserved_variable_count, c.dimension
    ns = s.config.equation == sdg.NAVIER_STOKES
    modal = s.state_modal()
    per = lambda nb: nv * nb * (1 + (d if ns else 0))
    pos, moff, parents = 0, 0, []
    for k in range(c.block_count):
        nb, ne = c.block_basis_count[k], c.block_element_count[k]
        for e in range(ne):
            np.testing.assert_array_equal(payload[pos:pos + nv * nb], modal[moff + e * nv * nb: moff + (e + 1) * nv * nb])
            pos += per(nb)
        moff += ne * nv * nb
    # boundary faces: one parent record each; then one zero per mesh node
    nb_face = c.boundary_face_count
    tail = payload[pos:]
    assert len(tail) >= nb_face * per(min(c.block_basis_count[k] for k in range(c.block_count)))
    assert np.all(payload[-len(mesh.nodes):] == 0.0)


def test_raw_binary_last_step_restart(tmp_path):
    s, dt, _ = make(cases.tgv_case(n=3, p=3, viscous=sdg.BR1, mu=0.02))
    s.stepSolver(dt, 2)
    u = s.state_point()
    path = tmp_path / "last.zst"
    s.writeRawBinary(path)
    s.stepSolver(dt, 3)
    s.read_raw_binary(path)
    np.testing.assert_allclose(s.state_point(), u, rtol=1e-14, atol=1e-14 * np.abs(u).max())


def test_raw_binary_specific_file_from_lower_order(tmp_path):
    lo, dt, _ = make(cases.kh_case(n=4, p=2, split=0.0, jitter=0.0))
    lo.stepSolver(dt, 1)
    path = tmp_path / "p2.zst"
    lo.writeRawBinary(path)
    hi, _, _ = make(cases.kh_case(n=4, p=3, split=0.0, jitter=0.0))
    hi.read_raw_binary(path, lower_order=True)
    m_lo, m_hi = lo.state_modal().reshape(-1, 9 * 4), hi.state_modal().reshape(-1, 16 * 4)
    # leading Nb(P-1) columns copied, the rest zero (InitialCondition.cpp:58-80)
    np.testing.assert_allclose(m_hi[:, :36], m_lo, rtol=1e-13, atol=1e-13)
    assert np.all(np.abs(m_hi[:, 36:]) < 1e-13)


def test_raw_binary_carries_the_node_artificial_viscosity(tmp_path):
    """With shock capturing the file's trailing node block is the node artificial viscosity of the state
    (RawBinary.cpp:185-190 writes node_artificial_viscosity_)."""
    s, dt, mesh = make(cases.shock_tube_case(p=3, n=8))
    s.stepSolver(dt, 1)
    path = tmp_path / "av.zst"
    s.writeRawBinary(path)
    payload = decode(path)
    av = s.node_artificial_viscosity()
    assert av.max() > 0
    np.testing.assert_array_equal(payload[-len(mesh.nodes):], av)


@pytest.mark.parametrize("name,case", [
    ("euler-channel-hybrid-p3", lambda: cases.channel_case(p=3, n=3, split=0.5, jitter=0.1)),
    ("euler-tet-box-p2", lambda: cases.tet_box_case(p=2)),
])
def test_raw_binary_boundary_block_in_callers_order(tmp_path, name, case):
    """The boundary block follows the caller's boundary-face order (the reference's adjacency order,
    src/View/RawBinary.cpp:120-154) given by sdg_set_boundary_face_order: record k is the modal state of the
    parent of the caller's k-th boundary face."""
    s, dt, mesh = make(case())
    s.stepSolver(dt, 1)
    c = s.counts
    _, bnd = s.adjacency()  # (type, element, face, physical, condition) per boundary face
    order = bnd[np.random.default_rng(9).permutation(len(bnd))][:, :3]
    s.set_boundary_face_order(order)
    path = tmp_path / "ordered.zst"
    s.writeRawBinary(path)
    payload = decode(path)
    nv = c.conserved_variable_count
    modal = s.state_modal()
    block_of = {c.block_element_type[k]: k for k in range(c.block_count)}
    first, moff = {}, 0
    pos = 0
    for k in range(c.block_count):
        first[k] = moff
        moff += c.block_element_count[k] * nv * c.block_basis_count[k]
    pos = moff  # Euler: the element block is the modal state itself
    for t, e, _ in order:
        k = block_of[t]
        nb = c.block_basis_count[k]
        np.testing.assert_array_equal(payload[pos:pos + nv * nb], modal[first[k] + e * nv * nb: first[k] + (e + 1) * nv * nb])
        pos += nv * nb
    assert pos == len(payload) - len(mesh.nodes)
    # an order that lists a face twice is refused
    bad = order.copy()
    bad[1] = bad[0]
    with pytest.raises(sdg.SdgError):
        s.set_boundary_face_order(bad)


def _records(payload, counts, order_parents):
    """Split a Navier-Stokes payload into the element gradient records (block order) and the boundary
    gradient records (file order); order_parents lists the block of each boundary record."""
    nv, d = counts.conserved_variable_count, counts.dimension
    nr = nv * d
    pos, elem = 0, []
    for k in range(counts.block_count):
        nb = counts.block_basis_count[k]
        for _ in range(counts.block_element_count[k]):
            elem.append(payload[pos + nv * nb: pos + nv * nb + nr * nb])
            pos += nv * nb + nr * nb
    bnd = []
    for k in order_parents:
        nb = counts.block_basis_count[k]
        bnd.append(payload[pos + nv * nb: pos + nv * nb + nr * nb])
        pos += nv * nb + nr * nb
    return np.concatenate(elem), np.concatenate(bnd) if bnd else np.zeros(0)


GRADIENT_CASES = {
    "channel-quad-p2-br2-walls": lambda: cases.channel_case(
        p=2, n=3, viscous=sdg.BR2, mu=0.01,
        conditions=(sdg.ISOTHERMAL_NONSLIP_WALL, sdg.PRESSURE_OUTFLOW, sdg.ADIABATIC_SLIP_WALL, sdg.VELOCITY_INFLOW)),
    "channel-hybrid-p3-br2-walls": lambda: cases.channel_case(
        p=3, n=3, split=0.5, jitter=0.1, viscous=sdg.BR2, mu=0.01,
        conditions=(sdg.ADIABATIC_NONSLIP_WALL, sdg.RIEMANN_FARFIELD, sdg.ISOTHERMAL_NONSLIP_WALL, sdg.VELOCITY_INFLOW)),
    "channel-bilinear-p1-br2-walls": lambda: cases.channel_case(
        p=1, n=3, jitter=0.1, viscous=sdg.BR2, mu=0.01,
        conditions=(sdg.ADIABATIC_NONSLIP_WALL, sdg.PRESSURE_OUTFLOW, sdg.ADIABATIC_SLIP_WALL, sdg.VELOCITY_INFLOW)),
    "channel-quad-p2-br1-walls": lambda: cases.channel_case(
        p=2, n=3, viscous=sdg.BR1, mu=0.01,
        conditions=(sdg.ISOTHERMAL_NONSLIP_WALL, sdg.PRESSURE_OUTFLOW, sdg.ADIABATIC_SLIP_WALL, sdg.VELOCITY_INFLOW)),
    "annulus-curved-hybrid-p3-br2": lambda: cases.annulus_case(
        p=3, split=0.5, viscous=sdg.BR2, mu=0.01, nr=2, ntheta=8,
        conditions=(sdg.ISOTHERMAL_NONSLIP_WALL, sdg.RIEMANN_FARFIELD)),
    "cavity-hex-p2-br2-inc": lambda: cases.cavity_3d_case(p=2, viscous=sdg.BR2, mu=1e-2),
    "tet-box-p2-br2-walls": lambda: cases.tet_box_case(
        p=2, viscous=sdg.BR2, mu=0.01,
        conditions=(sdg.VELOCITY_INFLOW, sdg.PRESSURE_OUTFLOW, sdg.ISOTHERMAL_NONSLIP_WALL,
                    sdg.ADIABATIC_NONSLIP_WALL, sdg.RIEMANN_FARFIELD, sdg.ADIABATIC_SLIP_WALL)),
}


@pytest.mark.parametrize("name", sorted(GRADIENT_CASES))
def test_raw_binary_gradient_records_match_the_oracle(tmp_path, name):
    """Navier-Stokes gradient records of the file against the oracle's (RawBinary.cpp:75-112): per element the
    gradient coefficients of the last stage input; per boundary face its parent's -- BR1 the element gradient,
    BR2 the volume gradient plus the lift of that face only. Boundary records follow the oracle's sorted order."""
    from oracle.orc import Oracle
    mesh, cfg, prim, bprim, dt, steps = GRADIENT_CASES[name]()
    g = sdg.GpuSolver(mesh, cfg)
    o = Oracle(mesh, cfg, faithful=False, precision="extended")
    p0 = prim(g.volume_points())
    g.initialize_primitive(p0)
    o.initialize_primitive(p0)
    nfq = g.counts.face_point_count
    bpts, phys = g.boundary_points()
    g.set_boundary_primitive(bprim(bpts, np.repeat(phys, nfq)))
    bpo, pho = o.boundary_points()
    o.set_boundary_primitive(bprim(bpo, np.repeat(pho, nfq)))
    g.stepSolver(dt, 2)
    o.step(dt, 2)
    c = g.counts
    _, bnd = g.adjacency()  # sorted (type, element, face, physical, condition): the oracle's boundary order
    g.set_boundary_face_order(bnd[:, :3])
    path = tmp_path / "ns.zst"
    g.writeRawBinary(path)
    block_of = {c.block_element_type[k]: k for k in range(c.block_count)}
    parents = [block_of[t] for t in bnd[:, 0]]
    elem, brec = _records(decode(path), c, parents)
    nr = c.conserved_variable_count * c.dimension
    o_elem, o_bnd = o.raw_gradient(len(elem), sum(nr * c.block_basis_count[k] for k in parents))
    scale = np.abs(o_elem).max()
    assert np.abs(elem - o_elem).max() <= 1e-10 * scale
    assert np.abs(brec - o_bnd).max() <= 1e-10 * scale
    # BR2: a boundary record is not its parent's element record (the other faces' lifts are left out)
    first, off = {}, 0
    for k in range(c.block_count):
        first[k] = off
        off += c.block_element_count[k] * nr * c.block_basis_count[k]
    parent_rec = np.concatenate([o_elem[first[k] + e * nr * c.block_basis_count[k]:
                                        first[k] + (e + 1) * nr * c.block_basis_count[k]]
                                 for k, e in zip(parents, bnd[:, 1])])
    gap = np.abs(parent_rec - o_bnd).max()
    assert (gap > 1e-6 * scale) if cfg.viscous_flux == sdg.BR2 else (gap <= 1e-14 * scale)
