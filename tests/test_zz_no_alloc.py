"""The allocation-free time-step entry point (sdg_delta_time_noalloc).

Callers that cannot call cudaMalloc -- a framework whose memory pool forbids raw device allocations, a
real-time loop that must not allocate, a host that only records into a stream it was handed -- get the
CFL time step from device arrays they already own.  This checks, through the C ABI, that it returns the
same dt as the allocating entry point sdg_calculate_delta_time (relative 1e-13, the dt tolerance of the
parity tests), on two calls in a row, and that it rejects a size beyond its static scratch.  It lives in
a file of its own that pytest collects last.
"""
import ctypes

import numpy as np
import pytest

import subrosadg_gb300 as sdg
from subrosadg_gb300 import _abi
from tests import cases

pytestmark = pytest.mark.gpu

EDGES = {4: [(0, 1), (1, 2), (2, 3), (3, 0)],
         8: [(0, 1), (1, 2), (2, 3), (3, 0), (4, 5), (5, 6), (6, 7), (7, 4), (0, 4), (1, 5), (2, 6), (3, 7)]}


def min_edges(nodes, elems):
    out = np.full(len(elems), np.inf)
    for a, b in EDGES[elems.shape[1]]:
        out = np.minimum(out, np.linalg.norm(nodes[elems[:, a]] - nodes[elems[:, b]], axis=1))
    return out


@pytest.mark.parametrize("case", ["tgv-hex-p3", "jittered-quad-p2"])
def test_noalloc_delta_time_matches_allocating_entry_point(case):
    import torch

    if case == "tgv-hex-p3":
        mesh, cfg, prim, _, _, _ = cases.tgv_case(n=4, p=3)
        elems, dim, p = mesh.hexahedra, 3, 3
    else:
        mesh, cfg, prim, _, _, _ = cases.kh_case(n=5, p=2, split=0.0, jitter=0.15)
        elems, dim, p = mesh.quadrangles, 2, 2
    g = sdg.GpuSolver(mesh, cfg, device=0)
    g.initialize_primitive(prim(g.volume_points()))
    expect = g.calculateDeltaTime(0.2)
    nq = g.counts.block_volume_point_count[0]
    state = torch.from_numpy(g.state_point()).to("cuda:0").contiguous()
    edge = torch.from_numpy(min_edges(mesh.nodes, elems)).to("cuda:0").contiguous()
    out = torch.zeros(1, dtype=torch.float64, device="cuda:0")
    lib = _abi.load()
    stream = torch.cuda.current_stream(0)
    for _ in range(2):  # the static scratch keeps the previous call's contents
        out.fill_(-1.0)
        rc = lib.sdg_delta_time_noalloc(state.data_ptr(), edge.data_ptr(), state.shape[0], nq, dim, p, 1.4, 0.2,
                                        out.data_ptr(), ctypes.c_void_p(stream.cuda_stream))
        assert rc == 0, lib.sdg_last_error(None)
        stream.synchronize()
        got = float(out.item())
        assert abs(got - expect) <= 1e-13 * expect, (got, expect)


def test_noalloc_rejects_sizes_beyond_its_scratch():
    import torch

    lib = _abi.load()
    buf = torch.zeros(8, dtype=torch.float64, device="cuda:0")
    too_many = 131072 * 256 + 1
    rc = lib.sdg_delta_time_noalloc(buf.data_ptr(), buf.data_ptr(), too_many, 1, 3, 3, 1.4, 0.2, buf.data_ptr(), None)
    assert rc == 1
    assert b"exceed the maximum" in lib.sdg_last_error(None)
