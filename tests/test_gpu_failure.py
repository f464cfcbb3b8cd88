"""Failure detection of the bounded device waits, made to run out without faulting anything.

The tensor stage kernels stage each element tile with TMA bulk copies that complete on an mbarrier and wait
for it a bounded number of rounds.  sdg_set_wait_check declares bytes beyond what the copies carry, with a
short limit: the copies all land, the wait can only end by its limit, the kernel flags the timeout, withdraws
the extra bytes, waits (bounded) for its own copies and returns.  The call must report SDG_ERR_TIMEOUT and the
context must stay usable: a new handle then steps and matches the oracle.  Nothing here faults, traps or waits
without a bound.
"""
import numpy as np
import pytest

import subrosadg_gb300 as sdg
from oracle.orc import Oracle
from subrosadg_gb300 import _abi
from subrosadg_gb300 import workloads as wl

pytestmark = pytest.mark.gpu

SDG_ERR_TIMEOUT = 7


def _normal_step_matches_oracle(mesh, cfg, prim, dt):
    g = sdg.GpuSolver(mesh, cfg)
    o = Oracle(mesh, cfg, faithful=False)
    p0 = prim(g.volume_points())
    g.initialize_primitive(p0)
    o.initialize_primitive(p0)
    g.stepSolver(dt, 2)
    o.step(dt, 2)
    a, b = g.state_point(), o.state_point()
    assert np.linalg.norm(a - b) <= 1e-10 * np.linalg.norm(b)


@pytest.mark.parametrize("graph", [1, 0], ids=["graph", "plain-launches"])
def test_bounded_wait_runs_out_and_is_reported(graph):
    mesh, cfg, prim, _, dt, _ = wl.tgv_case(n=3, p=3, flux=sdg.HLLC)
    g = sdg.GpuSolver(mesh, cfg)
    g.initialize_primitive(prim(g.volume_points()))
    lib = g.lib
    assert lib.sdg_set_graph(g.h, graph) == 0
    assert lib.sdg_set_wait_check(g.h, 4096, 16) == 0
    rc = lib.sdg_step(g.h, 1, dt)
    assert rc == SDG_ERR_TIMEOUT, (rc, lib.sdg_last_error(g.h))
    assert b"timed out" in lib.sdg_last_error(g.h)
    # the timeout is sticky on this handle (its state is no longer a step's result)
    assert lib.sdg_step(g.h, 1, dt) == SDG_ERR_TIMEOUT
    g.close()
    _normal_step_matches_oracle(mesh, cfg, prim, dt)


def test_bounded_wait_runs_out_in_a_batch():
    """The batched persistent kernel leaves its work list at the timed-out tile and the batch step reports it."""
    cases = [wl.tgv_case(n=3, p=2), wl.vortex_case(n=6, p=3)]
    solvers = []
    for mesh, cfg, prim, _, dt, _ in cases:
        g = sdg.GpuSolver(mesh, cfg)
        g.initialize_primitive(prim(g.volume_points()))
        solvers.append(g)
    assert _abi.load().sdg_set_wait_check(solvers[0].h, 4096, 16) == 0
    b = sdg.Batch(solvers)
    b.set_delta_time([c[4] for c in cases])
    with pytest.raises(sdg.SdgError) as err:
        b.step(1)
    assert err.value.code == SDG_ERR_TIMEOUT
    b.close()
    for g in solvers:
        g.close()
    mesh, cfg, prim, _, dt, _ = cases[1]
    _normal_step_matches_oracle(mesh, cfg, prim, dt)


def test_wait_check_arguments():
    mesh, cfg, prim, _, dt, _ = wl.tgv_case(n=3, p=1)
    g = sdg.GpuSolver(mesh, cfg)
    assert g.lib.sdg_set_wait_check(g.h, 0, 65537) == 1
    assert g.lib.sdg_set_wait_check(None, 0, 0) == 1
    assert g.lib.sdg_set_wait_check(g.h, 0, 0) == 0
