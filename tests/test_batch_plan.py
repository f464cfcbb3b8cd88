"""CPU tests of the batch planner and the tile interface (host-only handles: no GPU needed).

A batch groups every instance's per-stage launches by (dependency level, kernel variant, tile); these tests
pin the resulting launch counts against a count made by hand from the launch structure of one step:

  Euler stage:         [level 2] interior (+ boundary) face flux  [level 3] one stage kernel per block
  Navier-Stokes stage: [level 0] trace exchange (+ boundary)  [level 1] one gradient kernel per block
                       [level 2] viscous face flux (+ boundary)  [level 3] one stage kernel per block
  after the last stage: one relative-error reduction.
"""
import ctypes

import pytest

import subrosadg_gb300 as sdg
from subrosadg_gb300 import _abi
from tests import cases


def host(mesh, cfg):
    return sdg.GpuSolver(mesh, cfg, device=-1)


def test_batch_groups_identical_variants_into_one_launch():
    quads = [host(sdg.Mesh.box_2d(0, 0, 1, 1, n, n), cases.config(3, sdg.ROE)) for n in (3, 5, 8)]
    b = sdg.Batch(quads)
    c = b.counts()
    # one face launch + one stage launch per stage, one reduction: 3 * 2 + 1, whatever the instance count
    assert c["instance_count"] == 3
    assert c["launches_per_step"] == 7
    assert c["sequential_launches_per_step"] == 3 * 7
    assert c["stage_count"] == 3
    assert c["element_count"] == 9 + 25 + 64
    # work items: face chunks of 256 points + stage tiles per stage (3 stages), one item per instance reduction
    tiles = 0
    faces = 0
    for s, n in zip(quads, (3, 5, 8)):
        epb = s.tile(0)[0]
        tiles += -(-n * n // epb)
        faces += -(-(2 * n * n * 4) // 256)
    assert c["work_items_per_step"] == 3 * (tiles + faces) + 3
    b.close()


def test_batch_mixed_euler_and_navier_stokes_plan():
    e1 = host(sdg.Mesh.box_2d(0, 0, 1, 1, 4, 4), cases.config(3, sdg.LAX_FRIEDRICHS))
    e2 = host(sdg.Mesh.box_2d(0, 0, 1, 1, 6, 6), cases.config(3, sdg.LAX_FRIEDRICHS))
    ns = host(sdg.Mesh.box_2d(0, 0, 1, 1, 6, 6, jitter=0.1, split_fraction=0.5, seed=3),
              cases.ns_config(2, sdg.LAX_FRIEDRICHS, sdg.BR2, 1e-3))
    assert ns.counts.block_count == 2
    b = sdg.Batch([e1, e2, ns])
    c = b.counts()
    # per stage: L0 exchange (1) + L1 gradients tri/quad (2) + L2 Euler face + NS face (2) + L3 stage
    # kernels quad P3 / tri P2 / quad P2 (3) = 8; three stages and one reduction launch
    assert c["launches_per_step"] == 3 * 8 + 1
    # alone: Euler 3 * 2 + 1 each; NS 3 * (1 + 2 + 1 + 2) + 1
    assert c["sequential_launches_per_step"] == 2 * 7 + 19
    b.close()


def test_batch_rejects_bad_instance_lists():
    lib = _abi.load()
    s = host(sdg.Mesh.box_2d(0, 0, 1, 1, 3, 3), cases.config(2, sdg.HLLC))
    out = ctypes.c_void_p()
    arr = (ctypes.c_void_p * 2)(s.h, s.h)
    assert lib.sdg_batch_create(arr, 2, ctypes.byref(out)) == _abi.SDG_ERR_INVALID_ARGUMENT
    assert lib.sdg_batch_create(arr, 0, ctypes.byref(out)) == _abi.SDG_ERR_INVALID_ARGUMENT
    b = sdg.Batch([s])
    with pytest.raises(sdg.SdgError) as e:
        b.step()
    assert e.value.code == _abi.SDG_ERR_STATE  # host-only instances only plan
    b.close()


def test_tiles_are_validated():
    hexes = host(sdg.Mesh.box_3d(0, 0, 0, 1, 1, 1, 3, 3, 3), cases.config(3, sdg.HLLC))
    epb, threads, gepb, gthreads = hexes.tile(0)
    assert epb == 4 and threads == 256  # 64 nodes per hexahedron, 256 threads
    hexes.set_tile(0, 2, 0, 1, 0)       # one thread per node: threads follow the tile
    assert hexes.tile(0)[:2] == (2, 128)
    with pytest.raises(sdg.SdgError):
        hexes.set_tile(0, 9, 0, 1, 0)   # 9 * 64 threads > 512
    tri = host(sdg.Mesh.box_2d(0, 0, 1, 1, 3, 3, split_fraction=1.0, seed=1), cases.config(4, sdg.ROE))
    tri.set_tile(0, 32, 128, 8, 256)
    assert tri.tile(0) == (32, 128, 8, 256)
    with pytest.raises(sdg.SdgError):
        tri.set_tile(0, 8, 100, 8, 256)  # not a whole number of warps
    with pytest.raises(sdg.SdgError):
        tri.set_tile(0, 1024, 256, 8, 256)  # shared memory beyond the opt-in limit
