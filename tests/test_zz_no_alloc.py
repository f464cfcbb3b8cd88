"""The allocation-free time-step entry point (sdg_delta_time_noalloc).

Callers that cannot call cudaMalloc -- a framework whose memory pool forbids raw device allocations, a
real-time loop that must not allocate, a host that only records into a stream it was handed -- get the
CFL time step from device arrays they already own.  This checks, through the C ABI, that it returns the
same dt as the allocating entry point sdg_calculate_delta_time (relative 1e-13, the dt tolerance of the
parity tests), on two calls in a row, for the ideal gas in 1D, 2D and 3D, for the incompressible models'
constant sound speed, and on a hybrid mesh with one call per element block; and that it rejects a size
beyond its static scratch and a point count that is not a whole number of elements.  It lives in a file of
its own that pytest collects last.
"""
import ctypes

import numpy as np
import pytest

import subrosadg_gb300 as sdg
from subrosadg_gb300 import _abi
from tests import cases

pytestmark = pytest.mark.gpu

EDGES = {2: [(0, 1)], 3: [(0, 1), (1, 2), (2, 0)], 4: [(0, 1), (1, 2), (2, 3), (3, 0)],
         8: [(0, 1), (1, 2), (2, 3), (3, 0), (4, 5), (5, 6), (6, 7), (7, 4), (0, 4), (1, 5), (2, 6), (3, 7)]}


def min_edges(nodes, elems):
    out = np.full(len(elems), np.inf)
    for a, b in EDGES[elems.shape[1]]:
        out = np.minimum(out, np.linalg.norm(nodes[elems[:, a]] - nodes[elems[:, b]], axis=1))
    return out


CASES = {
    "tgv-hex-p3": lambda: cases.tgv_case(n=4, p=3),
    "jittered-quad-p2": lambda: cases.kh_case(n=5, p=2, split=0.0, jitter=0.15),
    "hybrid-tri-quad-p3": lambda: cases.kh_case(n=5, p=3, split=0.5, jitter=0.1),
    "line-p4": lambda: cases.density_wave_1d_case(n=12, p=4),
    "incompressible-quad-p3": lambda: cases.taylor_vortex_case(n=4, p=3, mu=1e-2),
}


@pytest.mark.parametrize("name", list(CASES))
def test_noalloc_delta_time_matches_allocating_entry_point(name):
    import torch

    mesh, cfg, prim, _, _, _ = CASES[name]()
    g = sdg.GpuSolver(mesh, cfg, device=0)
    g.initialize_primitive(prim(g.volume_points()))
    expect = g.calculateDeltaTime(0.2)
    c = g.counts
    blocks = {sdg.LINE: mesh.lines, sdg.TRIANGLE: mesh.triangles, sdg.QUADRANGLE: mesh.quadrangles,
              sdg.HEXAHEDRON: mesh.hexahedra}
    state = g.state_point()
    lib = _abi.load()
    stream = torch.cuda.current_stream(0)
    c0 = cfg.reference_sound_speed if cfg.equation in (sdg.INCOMPRESSIBLE_EULER, sdg.INCOMPRESSIBLE_NAVIER_STOKES) \
        else 0.0
    out = torch.zeros(c.block_count, dtype=torch.float64, device="cuda:0")
    for _ in range(2):  # the static scratch keeps the previous call's contents
        out.fill_(-1.0)
        first = 0
        keep = []
        for b in range(c.block_count):  # one call per element block
            nq, ne = c.block_volume_point_count[b], c.block_element_count[b]
            pts = torch.from_numpy(state[first:first + ne * nq]).to("cuda:0").contiguous()
            edge = torch.from_numpy(min_edges(mesh.nodes, blocks[c.block_element_type[b]])).to("cuda:0")
            keep += [pts, edge]
            rc = lib.sdg_delta_time_noalloc(pts.data_ptr(), edge.data_ptr(), ne * nq, nq, c.dimension,
                                            cfg.polynomial_order, cfg.specific_heat_ratio, c0, 0.2,
                                            out.data_ptr() + 8 * b, ctypes.c_void_p(stream.cuda_stream))
            assert rc == 0, lib.sdg_last_error(None)
            first += ne * nq
        stream.synchronize()
        got = float(out.min().item())
        assert abs(got - expect) <= 1e-13 * expect, (got, expect)


def test_noalloc_rejects_sizes_beyond_its_scratch():
    import torch

    lib = _abi.load()
    buf = torch.zeros(8, dtype=torch.float64, device="cuda:0")
    too_many = 131072 * 256 + 1
    rc = lib.sdg_delta_time_noalloc(buf.data_ptr(), buf.data_ptr(), too_many, 1, 3, 3, 1.4, 0.0, 0.2,
                                    buf.data_ptr(), None)
    assert rc == 1
    assert b"exceed the maximum" in lib.sdg_last_error(None)
    # 10 points are not a whole number of 4-point elements: rejected before anything is read
    rc = lib.sdg_delta_time_noalloc(buf.data_ptr(), buf.data_ptr(), 10, 4, 2, 1, 1.4, 0.0, 0.2, buf.data_ptr(), None)
    assert rc == 1
    assert b"multiple of points_per_element" in lib.sdg_last_error(None)
